"""Seeded randomized sweep over the paths of one Debye handle, each case
checked against the FP64 oracle: the forward (1e-5 relative per q), the
adjoint (gradient norm and max error), and one incremental step.

Each case draws its own body count, structure (compact chain or a uniform
box from a few to several hundred Angstroms), type count (with unused
columns), q grid (uniform from zero, uniform from q_min > 0, or sorted
random), q_slab, implicit water (weight, column, rsasa) and whether the
tabulated / gridded forms run.  So the slab plans, the small-theta levels,
the gridded forward below and past its node cap, the table adjoint and the
recurrence adjoint all meet inputs no hand-written case pins.  A second
sweep does the same for batched ensembles (members of uneven sizes, empty
ones included): the forward and the chi^2 gradient of every member."""
import numpy as np
import pytest

from resaxs_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-5
N_CASES = 96
N_BATCH_CASES = 24


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))


def grad_err(g, ref):
    g = np.asarray(g, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = max(np.linalg.norm(ref), 1e-300)
    return np.linalg.norm(g - ref) / scale, np.max(np.abs(g - ref)) / max(np.max(np.abs(ref)), 1e-300)


def draw_grid(rng, n_types):
    q_max = float(rng.uniform(0.1, 1.2))
    n_q = int(rng.integers(1, 300))
    grid = rng.choice(["uniform", "offset", "random"], p=[0.5, 0.25, 0.25])
    if grid == "uniform":
        q = W.q_grid(n_q, q_max)
    elif grid == "offset":
        q = W.q_grid(n_q, q_max, q_min=float(rng.uniform(0.01, 0.5 * q_max)))
    else:
        q = np.sort(rng.uniform(0, q_max, n_q)).astype(np.float32)
    Z = rng.choice([1, 6, 7, 8, 15, 16, 26, 30], size=n_types)
    return q, W.exp_form_factors(q, Z, rng.uniform(0.3, 2.5, n_types)), str(grid)


def draw_case(seed):
    rng = np.random.default_rng(1000 + seed)
    n = int(np.exp(rng.uniform(np.log(2), np.log(2500))))
    n_types = int(rng.integers(1, 9))
    used = int(rng.integers(1, n_types + 1))
    p = rng.dirichlet(np.ones(used))
    types = rng.choice(used, size=n, p=p)
    if rng.uniform() < 0.5:
        xyz = W.make_config(1, seed=seed, n_override=max(n, 2)).bodies[:n, :3].astype(np.float64)
        kind = "chain"
    else:
        size = float(np.exp(rng.uniform(np.log(3.0), np.log(600.0))))
        xyz = rng.uniform(-size / 2, size / 2, (n, 3))
        kind = "box %.0f A" % size
    bodies = W.pack_bodies(xyz, types)
    q, ff, grid = draw_grid(rng, n_types)
    n_q, q_max = len(q), float(q[-1])
    water = None
    if rng.uniform() < 0.35:
        water = (float(rng.uniform(-2.0, 4.0)), int(rng.integers(0, n_types)),
                 rng.uniform(0, 1, n).astype(np.float32))
    q_slab = int(rng.choice([0, 0, 8, 16, 32, 64, 128]))
    tables = bool(rng.uniform() < 0.7)
    k = int(rng.integers(1, max(2, n // 4) + 1))
    return dict(rng=rng, n=n, bodies=bodies, q=q, ff=ff, water=water, q_slab=q_slab,
                tables=tables, k=min(k, n), desc="%s n=%d T=%d/%d %s n_q=%d q_max=%.2f water=%s "
                "q_slab=%d tables=%s" % (kind, n, used, n_types, grid, n_q, q_max,
                                          water is not None, q_slab, tables))


@pytest.mark.parametrize("seed", range(N_CASES))
def test_sweep_forward_adjoint_recalc(oracle_lib, seed):
    from resaxs_gb300.saxs import Debye
    c = draw_case(seed)
    rng, n, q, ff, bodies = c["rng"], c["n"], c["q"], c["ff"], c["bodies"]
    kw = {}
    if c["water"] is not None:
        ww, wi, rs = c["water"]
        kw = dict(rsasa=rs, water_weight=ww, water_index=wi)
    lam = rng.normal(size=len(q)).astype(np.float32)
    idx = rng.choice(n, size=c["k"], replace=False).astype(np.uint32)
    moved = bodies[idx].copy()
    moved[:, :3] += rng.normal(0, 0.7, (c["k"], 3)).astype(np.float32)
    after = bodies.copy()
    after[idx] = moved
    with Debye(q, ff, n, q_slab=c["q_slab"], pair_tables=c["tables"]) as d:
        if c["water"] is not None:
            d.set_water(ww, wi, rs)
        d.calc(bodies)
        out64 = d.curve_f64()
        g = np.asarray(d.backward(lam, f64=True), np.float64)
        d.recalc_indices(moved, idx)
        rec64 = d.curve_f64()
    ref = oracle_lib.debye_f64(q, bodies, ff, **kw)
    e = rel(out64, ref)
    assert e < TOL, ("forward", c["desc"], e)
    gref = oracle_lib.debye_grad_f64(q, lam.astype(np.float64), bodies, ff, **kw)
    if n == 1 or not np.any(gref):
        assert np.all(g == 0), c["desc"]
    else:
        e_norm, e_max = grad_err(g, gref)
        assert e_norm < 2e-5 and e_max < 1e-4, ("adjoint", c["desc"], e_norm, e_max)
    e = rel(rec64, oracle_lib.debye_f64(q, after, ff, **kw))
    assert e < TOL, ("recalc", c["desc"], e)


@pytest.mark.parametrize("seed", range(N_BATCH_CASES))
def test_sweep_batch_forward_chi2_gradient(oracle_lib, seed):
    from resaxs_gb300.batch import DebyeBatch
    rng = np.random.default_rng(5000 + seed)
    n_types = int(rng.integers(1, 9))
    q, ff, grid = draw_grid(rng, n_types)
    members = []
    for m in range(int(rng.integers(1, 11))):
        n = 0 if rng.uniform() < 0.1 else int(np.exp(rng.uniform(0, np.log(900))))
        if rng.uniform() < 0.5 and n >= 2:
            xyz = W.make_config(1, seed=100 * seed + m, n_override=n).bodies[:, :3].astype(np.float64)
        else:
            size = float(np.exp(rng.uniform(np.log(3.0), np.log(400.0))))
            xyz = rng.uniform(-size / 2, size / 2, (n, 3))
        members.append(W.pack_bodies(xyz.reshape(n, 3), rng.integers(0, n_types, n)))
    tables = bool(rng.uniform() < 0.7)
    q_slab = int(rng.choice([0, 0, 8, 16, 32, 64, 128]))
    desc = "members=%s %s n_q=%d q_max=%.2f tables=%s q_slab=%d" % (
        [len(m) for m in members], grid, len(q), float(q[-1]), tables, q_slab)
    targets, sigmas = [], []
    for m in members:
        tb = m.copy()
        tb[:, :3] += rng.normal(0, 1.0, (len(m), 3)).astype(np.float32)
        it = oracle_lib.debye_f64(q, tb, ff).astype(np.float32) if len(m) else np.ones(len(q), np.float32)
        targets.append(it)
        sigmas.append(np.maximum(0.01 * it, 1e-3).astype(np.float32))
    with DebyeBatch(q, ff, [len(m) for m in members], q_slab=q_slab, pair_tables=tables) as b:
        out = b.forward(members)
        b.set_targets(np.stack(targets), np.stack(sigmas))
        out2, chi2, grad = b.forward_chi2_backward(members)
    assert np.array_equal(out, out2), desc
    off = 0
    for i, m in enumerate(members):
        if len(m) == 0:
            ref_chi2 = np.sum((1.0 / sigmas[i].astype(np.float64)) ** 2)
            assert np.all(out[i] == 0) and abs(chi2[i] - ref_chi2) <= 1e-6 * ref_chi2, desc
            continue
        iq = oracle_lib.debye_f64(q, m, ff)
        assert rel(out[i], iq) < TOL, ("forward", i, desc)
        s64 = sigmas[i].astype(np.float64)
        lam = 2 * (iq - targets[i]) / s64 ** 2
        g_ref = oracle_lib.debye_grad_f64(q, lam, m, ff)
        g = grad[off:off + len(m)].astype(np.float64)
        if np.any(g_ref):
            e = np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref)
            assert e < 1e-4, ("gradient", i, desc, e)
        else:
            assert np.all(g == 0), ("gradient", i, desc)
        off += len(m)
