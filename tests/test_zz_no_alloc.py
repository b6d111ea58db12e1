"""The allocation-free entry point, rsx_calc_saxs_curve_device_noalloc.

It exists for callers that cannot allocate device memory themselves (a host
framework that owns every device allocation through its own pool, or a stream
driven by a scheduler that must see no allocator calls): they pass device
buffers for the inputs and the curve, and the pair kernel's working memory is
a static device array inside librsx.  This file is collected last so that a
run stopping at the first failure has run every other test before it.

The test owns its device buffers (allocated here through torch, outside the
entry point) and checks two calls in a row -- the array keeps the previous
call's contents -- against the FP64 oracle and the existing entry point,
rsx_calc_saxs_curve_status, within the 1e-5 relative tolerance of the other
parity tests; then a problem large enough that the pair sums of one work item
cover several J blocks (the array would not hold one sum per block pair)."""
import ctypes

import numpy as np
import pytest

from resaxs_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-5


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))


def _existing_entry(q, bodies, ff):
    from resaxs_gb300 import _lib
    out = np.zeros(len(q), np.float32)
    _lib.check(_lib.lib().rsx_calc_saxs_curve_status(q, len(q), bodies.reshape(-1), len(bodies),
                                                     ff.reshape(-1), ff.shape[1], out))
    return out


def _noalloc_entry(torch, q, bodies, ff):
    from resaxs_gb300 import _lib
    dev = torch.device("cuda", 0)
    d_q = torch.from_numpy(np.ascontiguousarray(q, np.float32)).to(dev)
    d_b = torch.from_numpy(np.ascontiguousarray(bodies, np.float32)).to(dev)
    d_f = torch.from_numpy(np.ascontiguousarray(ff, np.float32)).to(dev)
    d_o = torch.full((len(q),), float("nan"), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize(dev)
    st = _lib.lib().rsx_calc_saxs_curve_device_noalloc(
        d_q.data_ptr(), len(q), d_b.data_ptr(), len(bodies), d_f.data_ptr(), ff.shape[1],
        d_o.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
    _lib.check(st)
    return d_o.cpu().numpy()


def test_noalloc_matches_oracle_and_existing_entry_twice(oracle_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    first = W.make_config(1, seed=41, n_override=1500)
    second = W.make_config(4, seed=42, n_override=900)      # other q grid, 8 types
    for w in (first, second):
        got = _noalloc_entry(torch, w.q, w.bodies, w.ff)
        assert np.all(np.isfinite(got))
        assert rel(got, oracle_lib.debye_f64(w.q, w.bodies, w.ff)) < TOL
        assert rel(got, _existing_entry(w.q, w.bodies, w.ff)) < TOL


SCRATCH_DOUBLES = 1048544   # the array's room for partial sums


def test_noalloc_several_j_blocks_per_item(oracle_lib):
    """20,000 bodies and 201 q: one partial sum per block pair would need
    157 * 158 / 2 * 201 doubles, more than the array holds, so each work item
    sums a run of J blocks.  Checked against the existing entry on every q and
    the FP64 oracle on every 8th q."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    w = W.make_config(2, seed=44)
    nb = (w.n + 127) // 128
    assert nb * (nb + 1) // 2 * len(w.q) > SCRATCH_DOUBLES     # the J runs are needed
    assert nb * len(w.q) <= SCRATCH_DOUBLES                    # and the call is accepted
    got = _noalloc_entry(torch, w.q, w.bodies, w.ff)
    assert rel(got, _existing_entry(w.q, w.bodies, w.ff)) < TOL
    sel = np.arange(0, len(w.q), 8)
    q64 = w.q.astype(np.float64)
    dq = (q64[-1] - q64[0]) / (len(q64) - 1)
    ref = oracle_lib.debye_f64_uniform(q64[0], 8 * dq, len(sel), w.bodies, w.ff[sel])
    assert rel(got[sel], ref) < TOL


def test_noalloc_rejects_oversize_and_bad_types():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from resaxs_gb300 import _lib
    L = _lib.lib()
    dev = torch.device("cuda", 0)
    d = torch.zeros(16, device=dev)
    # ceil(n/128) * n_q beyond the static array: rejected before any launch
    st = L.rsx_calc_saxs_curve_device_noalloc(d.data_ptr(), 1 << 20, d.data_ptr(), 1 << 20,
                                              d.data_ptr(), 1, d.data_ptr(), None)
    assert st == _lib.RSX_INVALID_ARG and "static scratch" in _lib.last_error()
    w = W.make_config(1, seed=43, n_override=200)
    bad = w.bodies.copy()
    bad.view(np.uint32)[7, 3] = 99
    with pytest.raises(_lib.ResaxsError) as e:
        _noalloc_entry(torch, w.q, bad, w.ff)
    assert e.value.code == _lib.RSX_INVALID_ARG
    # the array's error word is cleared on the next call
    got = _noalloc_entry(torch, w.q, w.bodies, w.ff)
    assert rel(got, _existing_entry(w.q, w.bodies, w.ff)) < TOL
