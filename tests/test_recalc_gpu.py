"""GPU tests of the incremental recalculation (delta of the moved pairs with
FP64 running totals) and of commit / revert, against full FP64 recomputes."""
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
def S():
    from resaxs_gb300 import saxs
    return saxs


@pytest.mark.parametrize("q_slab,n_q,q_min", [(0, 201, 0.0), (32, 201, 0.0), (16, 201, 0.0),
                                               (128, 101, 0.0), (128, 256, 0.0), (64, 150, 0.0),
                                               (64, 40, 0.0), (0, 113, 0.0), (0, 384, 0.0),
                                               (0, 450, 0.0), (0, 97, 0.0), (0, 201, 0.01),
                                               (0, 200, 0.01)])
def test_recalc_indices_matches_full_recompute(S, oracle_lib, q_slab, n_q, q_min):
    """Config-2 style moves (k random bodies, Gaussian sigma 0.5 A) at a size the
    oracle recomputes quickly; every step is checked.  The slab sizes and q
    counts cover the wide delta chains (a grid from q = 0 runs on the q past
    it: 201 q as 112 + 88, 384 q as 224 and 112 + 48, 450 q as two 224-q
    chains and a 16-q slab; from q = 0.01, 201 q as 112 + 96 and 200 q as
    112 + 88) and the 16 / 32-q kernel."""
    w = W.make_config(2, seed=21, n_override=1200)
    q = W.q_grid(n_q, 0.5, q_min)
    ff = W.exp_form_factors(q, W.Z5, np.random.default_rng(n_q).uniform(0.5, 2.0, 5))
    rng = np.random.default_rng(1)
    bodies = w.bodies.copy()
    with S.Debye(q, ff, w.n, q_slab=q_slab) as d:
        d.calc(bodies)
        for step in range(4):
            idx = rng.choice(w.n, size=50, replace=False).astype(np.uint32)
            moved = bodies[idx].copy()
            moved[:, :3] += rng.normal(0, 0.5, (50, 3)).astype(np.float32)
            out = d.recalc_indices(moved, idx)
            bodies[idx] = moved
            ref = oracle_lib.debye_f64(q, bodies, ff)
            assert rel(d.curve_f64(), ref) < TOL, step
            assert rel(out, ref) < TOL


def test_recalc_far_pairs(S, oracle_lib):
    """A free random-walk chain on a coarse grid: many pairs step angles past
    pi/2 (signed far-pair steps in the wide delta kernel); moves far beyond
    the current extent must also be followed."""
    w = W.make_config(1, seed=23, n_override=1500)
    q = W.q_grid(101, 0.8)
    ff = W.exp_form_factors(q, W.Z5, np.random.default_rng(4).uniform(0.5, 2.0, 5))
    rng = np.random.default_rng(5)
    bodies = w.bodies.copy()
    with S.Debye(q, ff, w.n) as d:
        d.calc(bodies)
        for step in range(3):
            idx = rng.choice(w.n, size=40, replace=False).astype(np.uint32)
            moved = bodies[idx].copy()
            moved[:, :3] += rng.normal(0, 40.0 if step == 1 else 0.5, (40, 3)).astype(np.float32)
            d.recalc_indices(moved, idx)
            bodies[idx] = moved
            assert rel(d.curve_f64(), oracle_lib.debye_f64(q, bodies, ff)) < TOL, step


def test_recalc_range_matches_full_recompute(S, oracle_lib):
    """The reference's contiguous-range API (saxs_algorithm.hpp:172)."""
    w = W.make_config(1, seed=22, n_override=900)
    rng = np.random.default_rng(2)
    bodies = w.bodies.copy()
    with S.Debye(w.q, w.ff, w.n) as d:
        d.calc(bodies)
        for start, length in [(0, 30), (500, 77), (870, 30), (123, 1)]:
            bodies[start:start + length, :3] += rng.normal(0, 1.0, (length, 3)).astype(np.float32)
            out = d.recalc_range(bodies, start, length)
            assert rel(out, oracle_lib.debye_f64(w.q, bodies, w.ff)) < TOL


def test_recalc_zero_length_and_large_move_fallback(S, oracle_lib):
    w = W.make_config(1, seed=23, n_override=400)
    with S.Debye(w.q, w.ff, w.n) as d:
        a = d.calc(w.bodies)
        b = d.recalc_range(w.bodies, 10, 0)
        assert np.array_equal(a, b)
        moved = w.bodies.copy()
        moved[:, :3] *= np.float32(1.01)
        out = d.recalc_range(moved, 0, w.n)   # everything moved: full recompute
        assert rel(out, oracle_lib.debye_f64(w.q, moved, w.ff)) < TOL


def test_many_steps_do_not_drift(S):
    """1,000 small moves on 3,000 bodies: the FP64 running curve equals a fresh
    full calculation of the final structure."""
    w = W.make_config(2, seed=24, n_override=3000)
    rng = np.random.default_rng(3)
    bodies = w.bodies.copy()
    with S.Debye(w.q, w.ff, w.n) as d:
        d.calc(bodies)
        for _ in range(1000):
            idx = rng.choice(w.n, size=20, replace=False).astype(np.uint32)
            moved = bodies[idx].copy()
            moved[:, :3] += rng.normal(0, 0.5, (20, 3)).astype(np.float32)
            d.recalc_indices(moved, idx)
            bodies[idx] = moved
        running = d.curve_f64()
    with S.Debye(w.q, w.ff, w.n) as d2:
        d2.calc(bodies)
        fresh = d2.curve_f64()
    assert rel(running, fresh) < TOL


def test_commit_revert(S, oracle_lib):
    """commit() checkpoints, revert() restores (saxs_alg_cl_gpu_pt_wf.cpp:592-620);
    revert before any commit is a no-op (:607-608)."""
    w = W.make_config(1, seed=25, n_override=600)
    rng = np.random.default_rng(4)
    b0 = w.bodies.copy()
    with S.Debye(w.q, w.ff, w.n) as d:
        c0 = d.calc(b0)
        b1 = b0.copy()
        b1[10:40, :3] += rng.normal(0, 1, (30, 3)).astype(np.float32)
        c1 = d.recalc_range(b1, 10, 30)
        d.revert()                                  # no checkpoint yet: no-op
        assert np.array_equal(d.curve_f64().astype(np.float32), c1)
        d.commit()                                  # checkpoint = b1
        b2 = b1.copy()
        b2[100:150, :3] += rng.normal(0, 1, (50, 3)).astype(np.float32)
        d.recalc_range(b2, 100, 50)
        d.revert()                                  # back to b1
        assert rel(d.curve_f64(), oracle_lib.debye_f64(w.q, b1, w.ff)) < TOL
        # continuing from the reverted state uses the reverted positions
        b3 = b1.copy()
        b3[300:310, :3] += np.float32(0.7)
        out = d.recalc_range(b3, 300, 10)
        assert rel(out, oracle_lib.debye_f64(w.q, b3, w.ff)) < TOL
        assert not np.array_equal(c0, out)


def test_recalc_errors(S):
    from resaxs_gb300 import _lib
    w = W.make_config(1, seed=26, n_override=100)
    with S.Debye(w.q, w.ff, w.n) as d:
        with pytest.raises(_lib.ResaxsError) as e:
            d.recalc_range(w.bodies, 0, 5)
        assert e.value.code == _lib.RSX_NO_INITIAL_CALC
        with pytest.raises(_lib.ResaxsError) as e:
            d.commit()
        assert e.value.code == _lib.RSX_NO_INITIAL_CALC
        d.calc(w.bodies)
        with pytest.raises(_lib.ResaxsError) as e:
            d.recalc_range(w.bodies, 90, 20)
        assert e.value.code == _lib.RSX_INVALID_ARG
        with pytest.raises(_lib.ResaxsError) as e:
            d.recalc_indices(w.bodies[:2], [3, 3])
        assert e.value.code == _lib.RSX_INVALID_ARG
        bad = w.bodies[:1].copy()
        bad.view(np.uint32)[0, 3] = (W.body_types(w.bodies)[5] + 1) % 5
        with pytest.raises(_lib.ResaxsError) as e:
            d.recalc_indices(bad, [5])
        assert e.value.code == _lib.RSX_INVALID_ARG


def test_dirty_factors_force_full_recompute(S, oracle_lib):
    w = W.make_config(1, seed=27, n_override=500)
    with S.Debye(w.q, w.ff, w.n) as d:
        d.calc(w.bodies)
        ff2 = (w.ff * np.float32(1.1)).astype(np.float32)
        d.set_factors(ff2)
        b = w.bodies.copy()
        b[0:5, :3] += np.float32(0.3)
        out = d.recalc_range(b, 0, 5)
        assert rel(out, oracle_lib.debye_f64(w.q, b, ff2)) < TOL


def test_saxs_algorithm_mirror(S, oracle_lib):
    """The i_saxs-style interface: params, initialize, calc_curve, recalc_curve."""
    w = W.make_config(1, seed=28, n_override=400)
    alg = S.SaxsAlgorithm()
    p = alg.access_params()
    p.initialize(w.q, w.bodies, factors=w.ff)
    p.get_implicit_water_params().set_water_weight(0)
    alg.initialize()
    out = []
    alg.calc_curve(w.bodies, out)
    assert rel(out, oracle_lib.debye_f64(w.q, w.bodies, w.ff)) < TOL
    b = w.bodies.copy()
    b[50:60, :3] += np.float32(1.0)
    alg.recalc_curve(b, 50, 10, out)
    assert rel(out, oracle_lib.debye_f64(w.q, b, w.ff)) < TOL
    alg.commit()
    alg.revert()


def test_saxs_algorithm_mirror_water_computes_its_own_rsasa(S, oracle_lib):
    """With a non-zero water weight the i_saxs mirror recomputes rsasa from the
    bodies on each update, as the reference's GPU algorithm does (its own
    dodeca-icosa dot map, probe 1.8 A, atomic radii by type); given rsasa
    values are kept only with no_rsasa_recalc set."""
    from resaxs_gb300 import _lib
    from resaxs_gb300.sasa import reference_dot_map
    w = W.make_config(2, seed=29, n_override=600)
    radii = np.zeros(16, np.float32)
    _lib.check(_lib.lib().rsx_ff_radii(radii))
    ico = reference_dot_map(radii, "dodeca_icosa", 1.8)
    widx = w.ff.shape[1] - 1

    def expect(bodies, rs):
        return oracle_lib.debye_f64(w.q, bodies, w.ff, rsasa=rs, water_weight=1.5,
                                    water_index=widx)

    alg = S.SaxsAlgorithm()
    p = alg.access_params()
    p.initialize(w.q, w.bodies, factors=w.ff)
    p.get_ff_params().set_water_ff_index(widx)
    p.get_implicit_water_params().set_water_weight(1.5)
    alg.initialize()
    out = alg.calc_curve(w.bodies)
    rs = (oracle_lib.sasa_counts_typed(w.bodies, radii, ico, 1.8).astype(np.float32)
          / np.float32(32))
    assert np.array_equal(p.get_implicit_water_params().rsasa, rs)
    assert rel(out, expect(w.bodies, rs)) < TOL
    b = w.bodies.copy()
    b[100:130, :3] += np.float32(2.0)
    out = alg.recalc_curve(b, 100, 30)
    rs_b = (oracle_lib.sasa_counts_typed(b, radii, ico, 1.8).astype(np.float32)
            / np.float32(32))
    assert rel(out, expect(b, rs_b)) < TOL
    given = np.random.default_rng(3).uniform(0, 1, w.n).astype(np.float32)
    water = p.get_implicit_water_params()
    water.no_rsasa_recalc = True
    water.access_rsasa()
    water.rsasa = given
    out = alg.calc_curve(b)
    assert rel(out, expect(b, given)) < TOL
