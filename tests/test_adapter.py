"""The header-only C++ adapter include/rsx/saxs_algorithm.hpp, compiled the way
a C++ caller of resaxslib's algorithm interface would compile it
(saxs_algorithm.hpp:118-244, rsasa_algorithm.hpp:42-61) and driven by
tests/adapter_check.cpp.

On the CPU: the header compiles against librsx, and the interface's error
paths raise rsx::error with the reference's codes (resaxs.hpp:212-220),
including initialize() without a CUDA device (no CPU path).  On the GPU: the
curves of calc_curve / recalc_curve / commit / revert, with and without the
implicit-water term (given rsasa, and the adapter's own SASA of the bodies
as the reference computes it) and across a second initialize(), against the
FP64 oracle, and calc_rsasa against the strict-FP32 oracle counts."""
import os
import subprocess

import numpy as np
import pytest

from resaxs_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOL = 1e-5


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))


@pytest.fixture(scope="module")
def adapter_exe(tmp_path_factory):
    from resaxs_gb300 import _lib
    lib_path = _lib.lib()._name
    exe = str(tmp_path_factory.mktemp("adapter") / "adapter_check")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "adapter_check.cpp"),
           "-o", exe, lib_path, f"-Wl,-rpath,{os.path.dirname(lib_path)}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_adapter_error_paths_without_gpu(adapter_exe):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: initialize() would succeed")
    r = subprocess.run([adapter_exe, "nogpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr


@pytest.mark.gpu
def test_adapter_curves_and_rsasa(adapter_exe, oracle_lib, tmp_path):
    w = W.make_config(2, seed=31, n_override=1500)
    n, n_q, n_t = w.n, len(w.q), w.ff.shape[1]
    rng = np.random.default_rng(7)
    water_index = n_t - 1
    start, length = 200, 40
    rsasa = rng.uniform(0.0, 1.0, n).astype(np.float32)
    radius_of_type = rng.uniform(1.2, 1.9, n_t).astype(np.float32)
    inp, outp = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        f.write(np.array([n, n_q, n_t, water_index, start, length], np.int32).tobytes())
        for a in (w.q, w.ff, w.bodies, rsasa, radius_of_type):
            f.write(np.ascontiguousarray(a, np.float32).tobytes())
    r = subprocess.run([adapter_exe, "gpu", str(inp), str(outp)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(outp, np.float32)
    assert raw.size == 8 * n_q + 4 * n
    curves = raw[:8 * n_q].reshape(8, n_q)
    got_rsasa, water_rsasa, water_rsasa_moved, typed_rsasa = raw[8 * n_q:].reshape(4, n)

    moved, moved2 = w.bodies.copy(), w.bodies.copy()
    moved[start:start + length, 0] += np.float32(0.3)
    moved2[start:start + length, 0] += np.float32(0.6)
    ref0 = oracle_lib.debye_f64(w.q, w.bodies, w.ff)
    ref1 = oracle_lib.debye_f64(w.q, moved, w.ff)
    ref2 = oracle_lib.debye_f64(w.q, moved2, w.ff)
    ref_w = oracle_lib.debye_f64(w.q, w.bodies, w.ff, rsasa=rsasa, water_weight=0.7,
                                 water_index=water_index)
    assert rel(curves[0], ref0) < TOL
    assert rel(curves[1], ref1) < TOL
    assert rel(curves[2], ref2) < TOL
    assert rel(curves[3], ref2) < TOL
    assert rel(curves[4], ref_w) < TOL
    # the water term reaches the handle made by the second initialize()
    assert rel(curves[5], ref_w) < TOL
    assert rel(ref_w, ref0) > 1e-3

    dots = oracle_lib.fibonacci_unit_dots(960)
    types = w.bodies.view(np.uint32)[:, 3]
    counts = oracle_lib.sasa_counts(w.bodies, radius_of_type[types], dots, 1.4)
    want = counts.astype(np.float32) / np.float32(960)
    assert np.array_equal(got_rsasa, want)

    # the water term's own SASA: the reference's OpenCL dot map (the
    # create_dodeca_icosa_dots sphere of each atomic radius, probe 1.8 A,
    # saxs_alg_cl_gpu_pt_wf.cpp:82-96, rsasa_cl_gpu_alg.cpp:60-89)
    from resaxs_gb300 import _lib
    from resaxs_gb300.sasa import reference_dot_map
    atomic_radii = np.zeros(16, np.float32)
    _lib.check(_lib.lib().rsx_ff_radii(atomic_radii))
    ico = reference_dot_map(atomic_radii, "dodeca_icosa", 1.8)
    for bodies, got, curve in ((w.bodies, water_rsasa, curves[6]),
                               (moved, water_rsasa_moved, curves[7])):
        c = oracle_lib.sasa_counts_typed(bodies, atomic_radii, ico, 1.8)
        rs = c.astype(np.float32) / np.float32(32)
        assert np.array_equal(got, rs)
        ref = oracle_lib.debye_f64(w.q, bodies, w.ff, rsasa=rs, water_weight=0.7,
                                   water_index=water_index)
        assert rel(curve, ref) < TOL
    assert rel(curves[6], ref_w) > 1e-4
    # the reference CPU algorithm's dot sets through rsasa_gpu::initialize
    lat = reference_dot_map(atomic_radii, "latitude", 1.4, 5.0)
    c = oracle_lib.sasa_counts_typed(w.bodies, atomic_radii, lat, 1.4)
    n_dots = np.isfinite(lat[:, :, 0]).sum(axis=1)[types].astype(np.float32)
    assert np.array_equal(typed_rsasa, c.astype(np.float32) / n_dots)
