"""Precision at the full 200,000-body configuration: FP32 kernel with FP64
cross-block reduction against the FP64 oracle on 8 q values (a uniform sub-grid
of the 512-point grid on [0, 1]).  Bound: 1e-5 relative per q."""
import numpy as np
import pytest

from resaxs_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_config4_per_q_error():
    from oracle import oracle
    from resaxs_gb300.saxs import Debye
    w = W.make_config(4, seed=0)
    with Debye(w.q, w.ff, w.n) as d:
        d.calc(w.bodies)
        out = d.curve_f64()
    step = 64
    sel = np.arange(0, len(w.q), step)
    q64 = w.q.astype(np.float64)
    dq = (q64[-1] - q64[0]) / (len(q64) - 1)
    ref = oracle.debye_f64_uniform(q64[0], step * dq, len(sel), w.bodies, w.ff[sel])
    err = np.abs(out[sel] - ref) / np.abs(ref)
    print("config4 q:", [round(float(x), 4) for x in w.q[sel]])
    print("config4 per-q relative error:", [f"{x:.2e}" for x in err])
    assert err.max() < 1e-5
