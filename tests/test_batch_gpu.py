"""Batched ensembles: one graph-captured persistent pass over members with
uneven body counts must give each member's curve (and chi^2 gradient) as the
FP64 oracle does for that member alone."""
import numpy as np
import pytest

from resaxs_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-5


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))


@pytest.fixture(scope="module")
def ensemble():
    q, ff, members = W.batch_members(n_members=10, seed=3, n_lo=40, n_hi=1500)
    members[3] = members[3][:1]          # a one-body member
    members[7] = members[7][:0]          # an empty member
    return q, ff, members


def test_batch_forward_vs_oracle(oracle_lib, ensemble):
    from resaxs_gb300.batch import DebyeBatch
    q, ff, members = ensemble
    with DebyeBatch(q, ff, [len(m) for m in members]) as b:
        out = b.forward(members)
        again = b.forward(members)     # graph replay
        cfg = b.config()
    assert cfg["persistent_ctas"] >= 152
    assert np.array_equal(out, again)
    for m, body in enumerate(members):
        if len(body) == 0:
            assert np.all(out[m] == 0)
            continue
        assert rel(out[m], oracle_lib.debye_f64(q, body, ff)) < TOL, m


def test_batch_spread_member_switches_kernels(oracle_lib, ensemble):
    """Stretching one member 600 A wide takes the whole pass off the
    small-theta kernels (signed far-pair steps, reduced seeds, graph captured
    again); compacting it brings them back.  Every curve must follow."""
    from resaxs_gb300.batch import DebyeBatch
    q, ff, members = ensemble
    spread = [m.copy() for m in members]
    spread[5][:, :3] *= np.float32(8.0)
    with DebyeBatch(q, ff, [len(m) for m in members]) as b:
        for ms in (members, spread, members):
            out = b.forward(ms)
            for m, body in enumerate(ms):
                if len(body) > 0:
                    assert rel(out[m], oracle_lib.debye_f64(q, body, ff)) < TOL, m


def test_batch_new_positions_and_types(oracle_lib, ensemble):
    from resaxs_gb300.batch import DebyeBatch
    q, ff, members = ensemble
    rng = np.random.default_rng(1)
    with DebyeBatch(q, ff, [len(m) for m in members]) as b:
        b.forward(members)
        moved = [m.copy() for m in members]
        for m in moved:
            m[:, :3] += rng.normal(0, 0.7, (len(m), 3)).astype(np.float32)
        out = b.forward(moved)                          # same types: graph reused
        for i in (0, 5, 9):
            assert rel(out[i], oracle_lib.debye_f64(q, moved[i], ff)) < TOL
        retyped = [m.copy() for m in moved]
        t = W.body_types(retyped[0])
        retyped[0].view(np.uint32)[:, 3] = (t + 1) % 5   # new layout, new graph
        out = b.forward(retyped)
        assert rel(out[0], oracle_lib.debye_f64(q, retyped[0], ff)) < TOL
        assert rel(out[9], oracle_lib.debye_f64(q, retyped[9], ff)) < TOL


def test_batch_matches_single_structure_handles(ensemble):
    from resaxs_gb300.batch import DebyeBatch
    from resaxs_gb300.saxs import Debye
    q, ff, members = ensemble
    with DebyeBatch(q, ff, [len(m) for m in members], autotune=True) as b:
        out = b.forward(members)
    for m in (0, 4, 8):
        with Debye(q, ff, len(members[m])) as d:
            assert rel(out[m], d.calc(members[m])) < 2e-6


@pytest.mark.parametrize("tables", [True, False])
def test_batch_chi2_gradients(oracle_lib, tables):
    from resaxs_gb300.batch import DebyeBatch
    q, ff, members = W.batch_members(n_members=4, seed=8, n_lo=100, n_hi=400)
    rng = np.random.default_rng(2)
    targets, sigmas = [], []
    for m in members:
        tb = m.copy()
        tb[:, :3] += rng.normal(0, 1.0, (len(m), 3)).astype(np.float32)
        it = oracle_lib.debye_f64(q, tb, ff).astype(np.float32)
        targets.append(it)
        sigmas.append((0.01 * it).astype(np.float32))
    with DebyeBatch(q, ff, [len(m) for m in members], pair_tables=tables) as b:
        b.set_targets(np.stack(targets), np.stack(sigmas))
        out, chi2, grad = b.forward_chi2_backward(members)
    off = 0
    for i, m in enumerate(members):
        iq = oracle_lib.debye_f64(q, m, ff)
        s = sigmas[i].astype(np.float64)
        ref_chi2 = np.sum(((iq - targets[i]) / s) ** 2)
        assert abs(chi2[i] - ref_chi2) / ref_chi2 < 1e-4
        lam = 2 * (iq - targets[i]) / s ** 2
        g_ref = oracle_lib.debye_grad_f64(q, lam, m, ff)
        g = grad[off:off + len(m)].astype(np.float64)
        assert np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref) < 1e-4
        off += len(m)


def test_batch_adjoint_tables_follow_the_extent(oracle_lib):
    """The batched adjoint reads per-member pair-function tables whose node
    count is fixed in the captured graph and whose step each pass sends to
    the device.  Stretching one member 8x needs more nodes (new capacity, new
    graph); compacting it again replays that graph with a smaller step.  The
    chi^2 gradients (targets: displaced copies, sigma = 1 % of the target, so
    that dL/dI is insensitive to the curves' rounding) must match the FP64
    gradient on every pass."""
    from resaxs_gb300.batch import DebyeBatch
    q, ff, members = W.batch_members(n_members=3, seed=9, n_lo=150, n_hi=300)
    stretched = [m.copy() for m in members]
    stretched[1][:, :3] *= np.float32(8.0)
    rng = np.random.default_rng(3)
    with DebyeBatch(q, ff, [len(m) for m in members]) as b:
        for ms in (members, stretched, members):
            tgt, sig = [], []
            for m in ms:
                tb = m.copy()
                tb[:, :3] += rng.normal(0, 1.0, (len(m), 3)).astype(np.float32)
                it = oracle_lib.debye_f64(q, tb, ff).astype(np.float32)
                tgt.append(it)
                sig.append((0.01 * it).astype(np.float32))
            b.set_targets(np.stack(tgt), np.stack(sig))
            _, _, grad = b.forward_chi2_backward(ms)
            off = 0
            for i, m in enumerate(ms):
                iq = oracle_lib.debye_f64(q, m, ff)
                s = sig[i].astype(np.float64)
                lam = 2 * (iq - tgt[i]) / s ** 2
                g_ref = oracle_lib.debye_grad_f64(q, lam, m, ff)
                g = grad[off:off + len(m)].astype(np.float64)
                assert np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref) < 1e-4, i
                off += len(m)


def test_batch_errors():
    from resaxs_gb300 import _lib
    from resaxs_gb300.batch import DebyeBatch
    q = W.q_grid(16, 0.5)
    ff = np.ones((16, 2), np.float32)
    with DebyeBatch(q, ff, [3, 2]) as b:
        with pytest.raises(_lib.ResaxsError) as e:
            b.forward_chi2_backward(np.zeros((5, 4), np.float32))
        assert e.value.code == _lib.RSX_ARGS_NOT_SET
        bad = W.pack_bodies(np.zeros((5, 3)), np.array([0, 1, 2, 0, 1]))
        with pytest.raises(_lib.ResaxsError) as e:
            b.forward(bad)
        assert e.value.code == _lib.RSX_INVALID_ARG
        # short host arrays are refused before the C calls read from them
        good = W.pack_bodies(np.arange(15, dtype=np.float32).reshape(5, 3),
                             np.array([0, 1, 0, 1, 0]))
        for call in (lambda: b.forward(good[:4]),
                     lambda: b.set_targets(np.ones((1, 16), np.float32),
                                           np.ones((2, 16), np.float32))):
            with pytest.raises(_lib.ResaxsError) as e:
                call()
            assert e.value.code == _lib.RSX_INVALID_ARG
        assert np.all(np.isfinite(b.forward(good)))


@pytest.mark.parametrize("q_slab,pairs", [(128, 4), (192, 2), (192, 4)])
def test_batch_tile_shapes(oracle_lib, ensemble, q_slab, pairs):
    """Every tile shape the batch tuner chooses from gives the oracle's curves."""
    from resaxs_gb300.batch import DebyeBatch
    q, ff, members = ensemble
    with DebyeBatch(q, ff, [len(m) for m in members], q_slab=q_slab,
                    pairs_per_step=pairs) as b:
        out = b.forward(members)
    for m, body in enumerate(members):
        if len(body) > 0:
            assert rel(out[m], oracle_lib.debye_f64(q, body, ff)) < TOL, m


def test_batch_autotuned_tile_shape(oracle_lib, ensemble):
    from resaxs_gb300.batch import DebyeBatch
    q, ff, members = ensemble
    with DebyeBatch(q, ff, [len(m) for m in members], autotune=True) as b:
        out = b.forward(members)
        cfg = b.config()
    assert cfg["q_slab"] in (32, 64, 128, 192)
    for m, body in enumerate(members):
        if len(body) > 0:
            assert rel(out[m], oracle_lib.debye_f64(q, body, ff)) < TOL, m


@pytest.mark.parametrize("q_slab,general,ww", [(0, False, 0.8), (16, False, -1.5), (32, False, 2.0),
                                               (64, False, 0.8), (128, False, 3.0),
                                               (192, False, 0.8), (0, True, 0.8), (8, True, -1.5)])
def test_batch_water(oracle_lib, ensemble, q_slab, general, ww):
    """The implicit water term in the batched forward (f~_i = f_t + w rsasa_i
    f_w): every member against the FP64 oracle with its own rsasa; new rsasa at
    the same weight reaches the next replay; weight 0 gives the dry curves."""
    from resaxs_gb300.batch import DebyeBatch
    q, ff, members = ensemble
    sizes = [len(m) for m in members]
    rng = np.random.default_rng(q_slab + 7 * general)
    rs = rng.uniform(0, 1, sum(sizes)).astype(np.float32)
    rs2 = rng.uniform(0, 1, sum(sizes)).astype(np.float32)
    off = np.concatenate([[0], np.cumsum(sizes)])
    with DebyeBatch(q, ff, sizes, q_slab=q_slab, force_general_q=general) as b:
        dry = b.forward(members)
        for r in (rs, rs2):
            b.set_water(ww, 4, r)
            out = b.forward(members)
            for m, body in enumerate(members):
                if len(body) == 0:
                    assert np.all(out[m] == 0)
                    continue
                ref = oracle_lib.debye_f64(q, body, ff, rsasa=r[off[m]:off[m + 1]],
                                           water_weight=ww, water_index=4)
                assert rel(out[m], ref) < TOL, (m, rel(out[m], ref))
        b.set_water(0.0, 4)
        assert np.array_equal(b.forward(members), dry)


def test_batch_water_autotuned_and_factors(oracle_lib, ensemble):
    """A tuned handle with water, then a new factor table (as an expansion
    factor changes it) under the same water weight."""
    from resaxs_gb300.batch import DebyeBatch
    q, ff, members = ensemble
    sizes = [len(m) for m in members]
    rs = np.random.default_rng(11).uniform(0, 1, sum(sizes)).astype(np.float32)
    off = np.concatenate([[0], np.cumsum(sizes)])
    ff2 = (ff * np.float32(1.07)).astype(np.float32)
    with DebyeBatch(q, ff, sizes, autotune=True) as b:
        b.set_water(1.3, 2, rs)
        for table in (ff, ff2):
            b.set_factors(table)
            out = b.forward(members)
            assert b.config()["q_slab"] in (32, 64, 128)
            for m, body in enumerate(members):
                if len(body) > 0:
                    ref = oracle_lib.debye_f64(q, body, table, rsasa=rs[off[m]:off[m + 1]],
                                               water_weight=1.3, water_index=2)
                    assert rel(out[m], ref) < TOL, m


def test_batch_water_errors(ensemble):
    from resaxs_gb300 import _lib
    from resaxs_gb300.batch import DebyeBatch
    q, ff, members = ensemble
    sizes = [len(m) for m in members]
    with DebyeBatch(q, ff, sizes) as b:
        for call in (lambda: b.set_water(0.5, 1),                       # no rsasa yet
                     lambda: b.set_water(0.5, 5, np.zeros(sum(sizes))),   # column 5 of 5
                     lambda: b.set_water(np.inf, 1, np.zeros(sum(sizes))),
                     lambda: b.set_water(0.5, 1, np.zeros(sum(sizes) - 1)),
                     lambda: b.set_factors(ff[:, :4])):
            with pytest.raises(_lib.ResaxsError) as e:
                call()
            assert e.value.code == _lib.RSX_INVALID_ARG
        b.set_water(0.5, 1, np.zeros(sum(sizes), np.float32))
        b.set_targets(np.ones((len(sizes), len(q)), np.float32),
                      np.ones((len(sizes), len(q)), np.float32))
        with pytest.raises(_lib.ResaxsError) as e:
            b.forward_chi2_backward(members)
        assert e.value.code == _lib.RSX_NOT_SUPPORTED
        b.set_water(0.0, 1)
        _, chi2, _ = b.forward_chi2_backward(members)
        assert np.all(np.isfinite(chi2))


@pytest.mark.parametrize("q_min,n_q", [(0.01, 201), (0.01, 200), (0.0, 193)])
def test_batch_chain_grids(oracle_lib, ensemble, q_min, n_q):
    """The chained batch pass on grids that do not start at q = 0 (every q
    takes pair work: 201 q as 192 + 16, 200 q as 192 + 8) and on 193 q from
    q = 0 (the 192 q past it: one 192-q slab, no tail)."""
    from resaxs_gb300.batch import DebyeBatch
    _, _, members = ensemble
    q = W.q_grid(n_q, 0.5, q_min)
    ff = W.exp_form_factors(q, W.Z5, np.random.default_rng(n_q).uniform(0.5, 2.0, 5))
    with DebyeBatch(q, ff, [len(m) for m in members], q_slab=192, pairs_per_step=2) as b:
        out = b.forward(members)
    for m, body in enumerate(members):
        if len(body) > 0:
            assert rel(out[m], oracle_lib.debye_f64(q, body, ff)) < TOL, m
