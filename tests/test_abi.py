"""CPU checks of the C ABI: librsx.so loads and exports every entry point the
public headers declare; calls that need no GPU report their errors cleanly."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(rsx_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def librsx():
    from resaxs_gb300 import _lib
    return _lib.lib()


def test_headers_declare_entry_points():
    names = declared_symbols()
    assert "rsx_debye_calc" in names and "rsx_calc_saxs_curve" in names
    assert len(names) >= 20


def test_every_declared_symbol_is_exported(librsx):
    missing = [n for n in declared_symbols() if not hasattr(librsx, n)]
    assert not missing, missing


def test_python_binding_covers_header(librsx):
    from resaxs_gb300 import _lib
    bound = set(_lib.exported_symbols())
    missing = [n for n in declared_symbols() if n not in bound]
    assert not missing, missing


def test_version_string(librsx):
    from resaxs_gb300 import _lib
    v = _lib.lib().rsx_version().decode()
    assert v.startswith("1.") and "sm_103a" in v


def test_null_and_invalid_arguments_without_gpu(librsx):
    from resaxs_gb300 import _lib
    L = _lib.lib()
    # null handle -> ALG_NOT_INITIALIZED (resaxs.hpp:215), no GPU touched
    assert L.rsx_debye_commit(None) == _lib.RSX_ALG_NOT_INITIALIZED
    assert L.rsx_debye_set_factors(None, np.zeros(1, np.float32), 1) == _lib.RSX_ALG_NOT_INITIALIZED
    h = ctypes.c_void_p()
    q = np.zeros(4, np.float32)
    st = L.rsx_debye_create(q, 0, np.zeros(4, np.float32), 1, 10, None, ctypes.byref(h))
    assert st == _lib.RSX_INVALID_ARG
    assert "positive" in _lib.last_error()


def test_create_without_gpu_fails_loudly(librsx):
    """No CPU fallback: on a machine without a GB300 the handle cannot be created."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from resaxs_gb300 import _lib
    from resaxs_gb300.saxs import Debye
    with pytest.raises(_lib.ResaxsError) as e:
        Debye(np.linspace(0, 0.5, 8), np.ones((8, 2)), 10)
    assert e.value.code in (_lib.RSX_INVALID_DEVICE, _lib.RSX_PROGRAM_NOT_LOADED)


def test_missing_library_raises(monkeypatch, tmp_path):
    from resaxs_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "librsx.so"))
    with pytest.raises(_lib.LibraryNotBuilt):
        _lib.lib()


@pytest.mark.parametrize("n,types,max_items", [(1500, 5, 7), (1500, 5, 16384), (0, 3, 10),
                                               (1, 2, 1), (5000, 8, 100), (300, 21, 3)])
def test_layout_covers_every_block_pair_once(librsx, n, types, max_items):
    """Host logic of the work decomposition (no GPU): type-uniform block tiles,
    each block pair (bi <= bj) in exactly one item, bounded item count."""
    from resaxs_gb300 import _lib
    from resaxs_gb300 import workloads as W
    rng = np.random.default_rng(n + types)
    bodies = W.pack_bodies(rng.normal(size=(n, 3)), rng.integers(0, types, n))
    nb, ni, na, good = (ctypes.c_int() for _ in range(4))
    _lib.check(_lib.lib().rsx_debug_layout(bodies.reshape(-1), n, types, max_items, 1216,
                                           ctypes.byref(nb), ctypes.byref(ni), ctypes.byref(na),
                                           ctypes.byref(good)))
    assert good.value == 1
    assert nb.value >= (n + 127) // 128
    if n:
        # at most one item per (I-block, remaining type run) once the cap bites
        assert ni.value <= max(max_items, nb.value * types)


def test_wide_slab_plan_covers_every_q(librsx):
    """The slab plan of the wide kernels: main slabs plus one remainder slab
    cover [0, n_q) exactly, every kernel width exists (16..128 in steps of 16)
    and a 64-q plan (the incremental kernel's) never needs a remainder slab
    wider than 112 q."""
    from resaxs_gb300 import _lib
    out = np.zeros(5, np.int32)
    mains = {64: (64,), 128: (64, 112, 128), 192: (64, 112, 128, 192)}
    for q_slab in (64, 128, 192):
        for n_q in range(1, 700):
            _lib.check(librsx.rsx_debug_wide_plan(n_q, q_slab, out))
            main, full, k0, tail_len, tail_w = (int(x) for x in out)
            assert main in mains[q_slab], (n_q, out)
            assert k0 == full * main and k0 + tail_len == n_q, (n_q, out)
            if tail_len:
                assert tail_w % 16 == 0 and tail_len <= tail_w <= 128, (n_q, out)
                if q_slab == 64:
                    assert tail_w <= 112, (n_q, out)
            else:
                assert tail_w == 0
    # the measured costs pick the 192-q slabs for the configurations' grids
    for n_q in (201, 256, 512):
        _lib.check(librsx.rsx_debug_wide_plan(n_q, 192, out))
        assert int(out[0]) == 192, (n_q, out)
    assert librsx.rsx_debug_wide_plan(0, 128, out) == _lib.RSX_INVALID_ARG
    assert librsx.rsx_debug_wide_plan(10, 32, out) == _lib.RSX_INVALID_ARG


def test_chain_plan_covers_every_q(librsx):
    """The chain plan of the uniform forward: full chains of 384 q from q 0,
    then one rest chain of up to two 192-q slabs and a tail of 8 q (for a
    remainder of 1..8 q) or of 16..176 q (a multiple of 16) that covers
    [rest_k0, n_q) with less than 16 q to spare (less than 8 for a tail of 8)."""
    from resaxs_gb300 import _lib
    out = np.zeros(5, np.int32)
    for n_q in range(1, 2500):
        _lib.check(librsx.rsx_debug_chain_plan(n_q, out))
        full, k0, main, tail, rest = (int(x) for x in out)
        assert k0 == 384 * full and k0 <= n_q, (n_q, out)
        assert rest == (k0 < n_q), (n_q, out)
        if rest:
            covered = 192 * main + tail
            assert (tail == 8 or tail % 16 == 0) and 0 <= tail <= 176 and 0 <= main <= 2, (n_q, out)
            assert n_q - k0 <= covered < n_q - k0 + (8 if tail == 8 else 16), (n_q, out)
            assert (tail == 8) == (0 < (n_q - k0) % 192 <= 8), (n_q, out)
    assert librsx.rsx_debug_chain_plan(0, out) == _lib.RSX_INVALID_ARG


def test_theta_level_thresholds(librsx):
    """The small-angle level that picks the kernel instantiations: 2 up to
    |dq| * diagonal * 1.0001 = 0.7, 1 up to 1.4, else 0; never above 0 for a
    non-uniform grid or a non-finite extent."""
    lv = librsx.rsx_debug_theta_level
    dq = 0.0025
    for diag, want in ((0.0, 2), (100.0, 2), (279.9, 2), (280.1, 1), (400.0, 1), (559.9, 1),
                       (560.1, 0), (900.0, 0)):
        assert lv(1, dq, diag) == want, (diag, want)
        assert lv(1, -dq, diag) == want, (diag, want)
        assert lv(0, dq, diag) == 0
    assert lv(1, dq, float("inf")) == 0
    assert lv(1, dq, float("nan")) == 0
    assert lv(1, dq, -1.0) == 0


def test_autotune_cache_file_keeps_only_valid_slabs(tmp_path):
    """The q-slab cache file named by RSX_AUTOTUNE_CACHE is read once per
    process; lines whose value is not a q-slab size rsx_debye_create accepts
    are ignored.  Run in a fresh process so the file is loaded there."""
    import subprocess
    import sys
    cache = tmp_path / "slabs.txt"
    cache.write_text("dev|forward|14|201|5|1|0 128\n"
                     "dev|forward|10|101|5|1|0 48\n"
                     "dev|forward|11|101|5|1|0 -16\n"
                     "dev|forward|12|101|5|1|0 32x\n"
                     "no_value_line\n"
                     "dev|forward|13|64|2|0|1 16\n")
    code = (
        "import ctypes\n"
        "from resaxs_gb300 import _lib\n"
        "L = _lib.lib()\n"
        "for k in ['dev|forward|14|201|5|1|0', 'dev|forward|10|101|5|1|0',\n"
        "          'dev|forward|11|101|5|1|0', 'dev|forward|12|101|5|1|0',\n"
        "          'dev|forward|13|64|2|0|1', 'missing']:\n"
        "    v = ctypes.c_int(0)\n"
        "    print(L.rsx_debug_autotune_lookup(k.encode(), ctypes.byref(v)), v.value)\n")
    env = dict(os.environ, RSX_AUTOTUNE_CACHE=str(cache))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                       cwd=ROOT, env=env, timeout=120)
    assert r.returncode == 0, r.stderr
    rows = [tuple(map(int, line.split())) for line in r.stdout.split("\n") if line.strip()]
    assert rows == [(1, 128), (0, 0), (0, 0), (0, 0), (1, 16), (0, 0)]
