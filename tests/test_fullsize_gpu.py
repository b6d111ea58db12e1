"""Parity at the full sizes of the adjoint and batching configurations.

* N = 50,000 bodies, 256 q on [0, 0.6] (the chi^2 configuration): the
  gradient rows of 64 seeded bodies against FP64 oracle rows, and FP64 central
  differences (h = 1e-4 A) along 64 seeded coordinates, for the tabulated
  adjoint and the per-pair*q one.  Only the moved body's pairs enter either
  check, which keeps them to seconds on the host.
* 256 members with N ~ U[1,000, 30,000], 201 q: every member's batched curve
  against a single-structure forward, and four members (the largest among
  them) against the FP64 oracle on every 25th q, with their chi^2 gradient
  rows against FP64 oracle rows.
"""
import numpy as np
import pytest

from resaxs_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))


def grad_err(g, ref):
    g = np.asarray(g, np.float64)
    ref = np.asarray(ref, np.float64)
    return (np.linalg.norm(g - ref) / np.linalg.norm(ref),
            np.max(np.abs(g - ref)) / np.max(np.abs(ref)))


@pytest.fixture(scope="module")
def config3():
    w = W.make_config(3, seed=0)
    rng = np.random.default_rng(3)
    target = w.bodies.copy()
    target[:, :3] += rng.normal(0, 1.0, (w.n, 3)).astype(np.float32)
    return w, target


@pytest.mark.parametrize("tables", [True, False])
def test_config3_gradient_rows_and_finite_differences(config3, oracle_lib, tables):
    from resaxs_gb300.saxs import Debye
    w, target_bodies = config3
    with Debye(w.q, w.ff, w.n, pair_tables=tables) as d:
        target = d.calc(target_bodies)
        sigma = (0.01 * target).astype(np.float32)
        d.calc(w.bodies)
        iq = d.curve_f64()
        # dchi^2/dI(q) at this point (sigma_q = 0.01 I_t), as the loss weights
        lam = (2.0 * (iq - target) / sigma.astype(np.float64) ** 2).astype(np.float32)
        g = np.asarray(d.backward(lam, f64=True), np.float64)
    lam64 = lam.astype(np.float64)
    rng = np.random.default_rng(64)
    rows = rng.choice(w.n, 64, replace=False)
    ref = oracle_lib.debye_grad_rows_f64(w.q, lam64, w.bodies, w.ff, rows)
    e_norm, e_max = grad_err(g[rows], ref)
    assert e_norm < 2e-5 and e_max < 1e-4, (tables, e_norm, e_max)
    coords = [(int(i), int(k % 3)) for k, i in enumerate(rows)]
    fd = oracle_lib.debye_fd_f64(w.q, lam64, w.bodies, w.ff, coords, h=1e-4)
    got = np.array([g[i, a] for i, a in coords])
    scale = np.max(np.abs(ref))
    assert np.all(np.abs(fd - got) <= 1e-4 * np.abs(fd) + 2e-5 * scale), \
        np.max(np.abs(fd - got) / (1e-4 * np.abs(fd) + 2e-5 * scale))


@pytest.fixture(scope="module")
def config5():
    return W.batch_members(n_members=256, seed=0)


def test_config5_full_batch(config5, oracle_lib):
    from resaxs_gb300.batch import DebyeBatch
    from resaxs_gb300.saxs import Debye
    q, ff, members = config5
    sizes = np.array([len(m) for m in members])
    assert sizes.max() > 25000 and len(members) == 256
    with DebyeBatch(q, ff, list(sizes)) as b:
        out = b.forward(members)
        t = (out * np.float32(1.01)).astype(np.float32)
        sigma = (0.01 * t + 1e-3).astype(np.float32)
        b.set_targets(t, sigma)
        out2, chi2, grad = b.forward_chi2_backward(members)
    assert np.array_equal(out, out2)
    # every member against the single-structure forward (oracle-pinned)
    for m, body in enumerate(members):
        with Debye(q, ff, len(body)) as d:
            d.calc(body)
            single = d.curve_f64()
        assert rel(out[m], single) < 1e-5, m
    # four members against the FP64 oracle, with their chi^2 gradient rows
    rng = np.random.default_rng(5)
    picks = [int(np.argmax(sizes)), int(np.argmin(sizes))] + \
        [int(x) for x in rng.choice(len(members), 2, replace=False)]
    offsets = np.concatenate([[0], np.cumsum(sizes)])
    sel = np.arange(0, len(q), 25)
    for m in picks:
        body = members[m]
        ref = oracle_lib.debye_f64(q[sel].astype(np.float64), body, ff[sel])
        assert rel(out[m][sel], ref) < 1e-5, m
        lam = 2.0 * (out[m].astype(np.float64) - t[m]) / sigma[m].astype(np.float64) ** 2
        assert abs(chi2[m] - np.sum(((out[m].astype(np.float64) - t[m]) / sigma[m]) ** 2)) \
            <= 1e-4 * chi2[m]
        rows = rng.choice(len(body), 32, replace=False)
        ref_g = oracle_lib.debye_grad_rows_f64(q, lam, body, ff, rows)
        e_norm, e_max = grad_err(grad[offsets[m] + rows], ref_g)
        assert e_norm < 1e-4 and e_max < 5e-4, (m, e_norm, e_max)
