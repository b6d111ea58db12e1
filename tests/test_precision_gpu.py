"""Precision at the full 200,000-body configuration: FP32 kernel with FP64
cross-block reduction against the FP64 oracle on 15 of the 512 q values (the
FP32 grid values themselves).  The forward runs the q past q = 0 as a chain
over q 1..384 (two 192-q slabs on one seed per pair, the second resuming
from shared memory) and a 128-q slab over q 385..511; the samples take q = 0
(from the type counts), the first slab and its end (191, 192), the second
slab from 8 q after the resume, the chain's far end (383, 384: 192 paired
steps after the seed) and the reseeded slab up to q = 1.0.  Bound: 1e-5
relative per q."""
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
    sel = np.array([0, 100, 191, 192, 200, 255, 256, 300, 383, 384, 420, 448, 480, 500, 511])
    ref = oracle.debye_f64(w.q[sel].astype(np.float64), w.bodies, w.ff[sel])
    err = np.abs(out[sel] - ref) / np.abs(ref)
    print("config4 q:", [round(float(x), 4) for x in w.q[sel]])
    print("config4 per-q relative error:", [f"{x:.2e}" for x in err])
    assert err.max() < 1e-5
