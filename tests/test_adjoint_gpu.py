"""GPU tests of the adjoint kernel: dL/dx from dL/dI(q) in one pair pass,
checked against the FP64 analytic gradient and FP64 central finite
differences (through a torch.autograd wrapper), and chi^2 gradients."""
import numpy as np
import pytest

from resaxs_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    from resaxs_gb300 import saxs
    return saxs


def grad_err(g, ref):
    g = np.asarray(g, np.float64)
    ref = np.asarray(ref, np.float64)
    return np.linalg.norm(g - ref) / np.linalg.norm(ref), np.max(np.abs(g - ref)) / np.max(np.abs(ref))


@pytest.mark.parametrize("tables", [True, False])
@pytest.mark.parametrize("idx,n", [(1, 600), (3, 500), (4, 300)])
def test_backward_vs_fp64_gradient(S, oracle_lib, idx, n, tables):
    """Both adjoints: the tabulated pair functions (default) and the
    recurrence evaluated per pair*q (pair_tables=False)."""
    w = W.make_config(idx, seed=31, n_override=n)
    rng = np.random.default_rng(idx)
    lam = rng.normal(size=len(w.q)).astype(np.float32)
    with S.Debye(w.q, w.ff, w.n, pair_tables=tables) as d:
        d.calc(w.bodies)
        g = d.backward(lam, f64=True)
    ref = oracle_lib.debye_grad_f64(w.q, lam.astype(np.float64), w.bodies, w.ff)
    e_norm, e_max = grad_err(g, ref)
    assert e_norm < 2e-5 and e_max < 1e-4, (e_norm, e_max)


@pytest.mark.parametrize("tables", [True, False])
@pytest.mark.parametrize("diag", [150.0, 400.0, 700.0, 1500.0])
def test_backward_on_every_small_theta_level(S, oracle_lib, diag, tables):
    """dq = 0.6/255: the adjoint's reduction-free half-angle seeds hold up to
    a box diagonal of 595 A; beyond 668 A the far body's pairs have
    theta > pi/2 and take the rotation form.  One body of a compact structure
    is placed so that the diagonal is `diag`; the gradient must match the
    FP64 analytic gradient in every case."""
    w = W.make_config(3, seed=35, n_override=500)
    b = w.bodies.copy()
    lo = b[1:, :3].min(0)
    hi = b[1:, :3].max(0)
    rest = float(np.sum((hi[1:] - lo[1:]) ** 2))
    b[0, 0] = np.float32(lo[0] + np.sqrt(diag * diag - rest))
    b[0, 1:3] = lo[1:]
    rng = np.random.default_rng(int(diag))
    lam = rng.normal(size=len(w.q)).astype(np.float32)
    with S.Debye(w.q, w.ff, w.n, pair_tables=tables) as d:
        d.calc(b)
        g = d.backward(lam, f64=True)
    ref = oracle_lib.debye_grad_f64(w.q, lam.astype(np.float64), b, w.ff)
    e_norm, e_max = grad_err(g, ref)
    assert e_norm < 2e-5 and e_max < 1e-4, (e_norm, e_max)


@pytest.mark.parametrize("tables", [True, False])
@pytest.mark.parametrize("ww", [0.6, -1.2])
def test_backward_uniform_q_and_water(S, oracle_lib, tables, ww):
    """Water on a uniform grid: the tables hold one entry per rsasa
    combination (1, rs_i, rs_j, rs_i rs_j); without them the rotation form
    with per-pair water factors runs."""
    w = W.make_config(3, seed=34, n_override=500)
    rng = np.random.default_rng(6)
    lam = rng.normal(size=len(w.q)).astype(np.float32)
    rs = rng.uniform(0, 1, w.n).astype(np.float32)
    with S.Debye(w.q, w.ff, w.n, pair_tables=tables) as d:
        d.set_water(ww, 3, rs)
        d.calc(w.bodies)
        g = d.backward(lam, f64=True)
    ref = oracle_lib.debye_grad_f64(w.q, lam.astype(np.float64), w.bodies, w.ff, rsasa=rs,
                                    water_weight=ww, water_index=3)
    e_norm, e_max = grad_err(g, ref)
    assert e_norm < 2e-5 and e_max < 1e-4, (e_norm, e_max)


@pytest.mark.parametrize("tables", [True, False])
def test_backward_general_q_and_water(S, oracle_lib, tables):
    w = W.make_config(1, seed=32, n_override=400)
    rng = np.random.default_rng(5)
    q = np.sort(rng.uniform(0, 0.5, 29)).astype(np.float32)
    ff = W.exp_form_factors(q, W.Z5, rng.uniform(0.5, 2.0, 5))
    lam = rng.normal(size=len(q)).astype(np.float32)
    rs = rng.uniform(0, 1, w.n).astype(np.float32)
    with S.Debye(q, ff, w.n, pair_tables=tables) as d:
        d.set_water(0.6, 3, rs)
        d.calc(w.bodies)
        g = d.backward(lam, f64=True)
    ref = oracle_lib.debye_grad_f64(q, lam.astype(np.float64), w.bodies, ff, rsasa=rs,
                                    water_weight=0.6, water_index=3)
    e_norm, e_max = grad_err(g, ref)
    assert e_norm < 2e-5 and e_max < 1e-4, (e_norm, e_max)


@pytest.mark.parametrize("tables", [True, False])
@pytest.mark.parametrize("uniform", [True, False])
def test_backward_edge_cases(S, oracle_lib, tables, uniform):
    """One body (no pair: a zero gradient), two bodies, and a coincident
    pair beside a third body (the coincident pair adds nothing: d sinc/dr
    vanishes at r = 0 and so does the direction), on a uniform and a
    non-uniform q grid."""
    rng = np.random.default_rng(9)
    if uniform:
        q = np.linspace(0, 0.5, 33).astype(np.float32)
    else:
        q = np.sort(rng.uniform(0, 0.5, 33)).astype(np.float32)
        q[0] = 0.0
    ff = W.exp_form_factors(q, (6, 8), (1.0, 0.5))
    lam = rng.normal(size=len(q)).astype(np.float32)
    cases = [
        W.pack_bodies(np.array([[1.0, 2.0, 3.0]]), np.array([1])),
        W.pack_bodies(np.array([[1.0, 2.0, 3.0], [4.5, -2.0, 7.25]]), np.array([0, 1])),
        W.pack_bodies(np.array([[1.0, 2.0, 3.0], [1.0, 2.0, 3.0], [-3.0, 0.5, 2.0]]),
                      np.array([0, 1, 1])),
    ]
    for bodies in cases:
        with S.Debye(q, ff, len(bodies), pair_tables=tables) as d:
            d.calc(bodies)
            g = np.asarray(d.backward(lam, f64=True), np.float64)
        assert g.shape == (len(bodies), 3) and np.all(np.isfinite(g))
        if len(bodies) == 1:
            assert np.all(g == 0)
            continue
        ref = oracle_lib.debye_grad_f64(q, lam.astype(np.float64), bodies, ff)
        e_norm, e_max = grad_err(g, ref)
        assert e_norm < 2e-5 and e_max < 1e-4, (len(bodies), e_norm, e_max)


def test_autograd_wrapper_vs_finite_differences(S, oracle_lib):
    """64 seeded coordinates, FP64 central differences with h = 1e-4 A (the
    represented FP32 step is used as the divisor)."""
    torch = pytest.importorskip("torch")
    from tests.torch_debye import debye_curve
    w = W.make_config(3, seed=33, n_override=300)
    types = W.body_types(w.bodies)
    rng = np.random.default_rng(7)
    lam = rng.normal(size=len(w.q))
    xyz = torch.tensor(w.bodies[:, :3].copy(), requires_grad=True)
    with S.Debye(w.q, w.ff, w.n) as d:
        iq = debye_curve(xyz, d, types)
        loss = (iq.double() * torch.tensor(lam)).sum()
        loss.backward()
    g = xyz.grad.numpy().astype(np.float64)
    coords = [(int(i), int(c)) for i, c in zip(rng.integers(0, w.n, 64), rng.integers(0, 3, 64))]
    scale = np.abs(g).max()
    q64 = w.q.astype(np.float64)
    for i, c in coords:
        bp = w.bodies.copy()
        bm = w.bodies.copy()
        bp[i, c] = np.float32(bp[i, c] + 1e-4)
        bm[i, c] = np.float32(bm[i, c] - 1e-4)
        step = float(bp[i, c]) - float(bm[i, c])
        fd = (lam @ oracle_lib.debye_f64(q64, bp, w.ff) - lam @ oracle_lib.debye_f64(q64, bm, w.ff)) / step
        assert abs(fd - g[i, c]) <= 1e-3 * abs(fd) + 2e-5 * scale, (i, c, fd, g[i, c])


def test_chi2_backward(S, oracle_lib):
    """chi^2 against a target from a displaced copy, sigma_q = 0.01 I_t."""
    w = W.make_config(3, seed=34, n_override=400)
    rng = np.random.default_rng(8)
    target_b = w.bodies.copy()
    target_b[:, :3] += rng.normal(0, 1.0, (w.n, 3)).astype(np.float32)
    it = oracle_lib.debye_f64(w.q, target_b, w.ff).astype(np.float32)
    sigma = (0.01 * it).astype(np.float32)
    with S.Debye(w.q, w.ff, w.n) as d:
        d.calc(w.bodies)
        chi2, g = d.chi2_backward(it, sigma)
    iq = oracle_lib.debye_f64(w.q, w.bodies, w.ff)
    lam = 2 * (iq - it.astype(np.float64)) / sigma.astype(np.float64) ** 2
    ref_chi2 = np.sum(((iq - it) / sigma.astype(np.float64)) ** 2)
    assert abs(chi2 - ref_chi2) / ref_chi2 < 1e-4
    ref = oracle_lib.debye_grad_f64(w.q, lam, w.bodies, w.ff)
    e_norm, e_max = grad_err(g, ref)
    assert e_norm < 1e-4 and e_max < 5e-4, (e_norm, e_max)


def test_backward_before_calc_is_an_error(S):
    from resaxs_gb300 import _lib
    w = W.make_config(1, seed=35, n_override=50)
    with S.Debye(w.q, w.ff, w.n) as d:
        with pytest.raises(_lib.ResaxsError) as e:
            d.backward(np.ones(len(w.q), np.float32))
        assert e.value.code == _lib.RSX_NO_INITIAL_CALC
