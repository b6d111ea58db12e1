"""GPU parity tests of the Debye forward path against the FP64 oracle and the
reference's golden vectors.  Tolerance: 1e-5 relative per q (FP32 kernel vs
FP64 oracle on the same FP32 inputs)."""
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
def saxs():
    from resaxs_gb300 import saxs as S
    return S


def gpu_curve(S, q, ff, bodies, **kw):
    with S.Debye(q, ff, len(bodies), **kw) as d:
        out = d.calc(bodies)
        return out, d.curve_f64(), d.config()


@pytest.mark.parametrize("idx,n", [(1, 2000), (2, 2500), (3, 1500), (4, 1200)])
def test_forward_configs_vs_oracle(saxs, oracle_lib, idx, n):
    w = W.make_config(idx, seed=11, n_override=n)
    out, out64, cfg = gpu_curve(saxs, w.q, w.ff, w.bodies)
    ref = oracle_lib.debye_f64(w.q, w.bodies, w.ff)
    assert cfg["uniform_q"]
    assert rel(out64, ref) < TOL
    assert rel(out, ref) < TOL


@pytest.mark.parametrize("q_slab", [8, 16, 32, 64, 128, 192])
def test_forward_slab_sizes(saxs, oracle_lib, q_slab):
    w = W.make_config(1, seed=12, n_override=700)
    _, out64, cfg = gpu_curve(saxs, w.q, w.ff, w.bodies, q_slab=q_slab)
    assert cfg["q_slab"] == q_slab
    assert rel(out64, oracle_lib.debye_f64(w.q, w.bodies, w.ff)) < TOL


@pytest.mark.parametrize("q_slab", [64, 128, 192])
@pytest.mark.parametrize("n_q", [5, 16, 33, 47, 64, 65, 80, 100, 111, 112, 113, 130, 192, 193,
                                 201, 240, 300, 384, 400])
def test_wide_slab_tails(saxs, oracle_lib, q_slab, n_q):
    # every tail width of the wide uniform path (16..112 after full slabs)
    rng = np.random.default_rng(n_q)
    w = W.make_config(2, seed=19, n_override=300)
    q = W.q_grid(n_q, 0.5)
    ff = W.exp_form_factors(q, W.Z5, rng.uniform(0.5, 2.0, 5))
    _, out64, cfg = gpu_curve(saxs, q, ff, w.bodies, q_slab=q_slab)
    assert cfg["uniform_q"] or n_q < 3
    assert rel(out64, oracle_lib.debye_f64(q, w.bodies, ff)) < TOL


def test_seed_paths_both_sides_of_the_small_theta_bound(saxs, oracle_lib):
    """A compact structure lets every seed skip the range reduction of
    theta/2 (dq * extent <= 1.4); moving two bodies 900 A away switches that
    off for the whole launch.  Both must match the oracle, and the compact
    structure's pairs must give the same sums either way."""
    w = W.make_config(2, seed=31, n_override=900)
    far = w.bodies.copy()
    far[:2, 0] += np.float32(900.0)
    for bodies in (w.bodies, far):
        _, out64, _ = gpu_curve(saxs, w.q, w.ff, bodies)
        assert rel(out64, oracle_lib.debye_f64(w.q, bodies, w.ff)) < TOL


@pytest.mark.parametrize("diag,level", [(150.0, 2), (279.0, 2), (281.0, 1), (400.0, 1),
                                        (559.0, 1), (561.0, 0), (900.0, 0)])
def test_forward_on_every_small_theta_level(saxs, oracle_lib, diag, level):
    """The forward picks its instantiation from the bounding box: plain
    paired steps with reduction-free seeds (|theta| < pi/4 for every pair),
    or the signed steps with range-reduced seeds.  One body of a compact
    structure is placed so that the box diagonal lands on each side of both
    thresholds (dq = 0.0025: 280 and 560 A); every case must match the
    oracle, including the pairs of the far body."""
    from resaxs_gb300 import _lib
    w = W.make_config(2, seed=37, n_override=800)
    b = w.bodies.copy()
    lo = b[1:, :3].min(0)
    hi = b[1:, :3].max(0)
    # body 0 on the far side of the box's x extent so that the diagonal is `diag`
    rest = float(np.sum((hi[1:] - lo[1:]) ** 2))
    b[0, 0] = np.float32(lo[0] + np.sqrt(diag * diag - rest))
    b[0, 1:3] = lo[1:]
    ext = b[:, :3].max(0).astype(np.float64) - b[:, :3].min(0).astype(np.float64)
    dq = float(w.q[1] - w.q[0])
    assert _lib.lib().rsx_debug_theta_level(1, dq, float(np.sqrt(np.sum(ext ** 2)))) == level
    _, out64, cfg = gpu_curve(saxs, w.q, w.ff, b)
    assert cfg["uniform_q"]
    assert rel(out64, oracle_lib.debye_f64(w.q, b, w.ff)) < TOL


def test_forward_general_q_path(saxs, oracle_lib):
    w = W.make_config(2, seed=13, n_override=800)
    rng = np.random.default_rng(3)
    q = np.sort(rng.uniform(0.0, 0.5, 37)).astype(np.float32)
    ff = W.exp_form_factors(q, W.Z5, rng.uniform(0.5, 2.0, 5))
    _, out64, cfg = gpu_curve(saxs, q, ff, w.bodies)
    assert not cfg["uniform_q"]
    assert rel(out64, oracle_lib.debye_f64(q, w.bodies, ff)) < TOL
    # forcing the general path on a uniform grid gives the same curve
    _, a, _ = gpu_curve(saxs, w.q, w.ff, w.bodies, force_general_q=True)
    _, b, _ = gpu_curve(saxs, w.q, w.ff, w.bodies)
    assert rel(a, b) < TOL


def test_golden_test1888(saxs, golden_1888):
    """The reference's own fixture: 1888 bodies, 21 types, q = 0..0.75."""
    g = golden_1888
    out, out64, _ = gpu_curve(saxs, g["q"], g["ff"], g["bodies"])
    assert rel(out64, g["iq_ref_dd"]) < TOL   # compiled reference host_debye<double,double>
    assert rel(out, g["iq"]) < 5e-5           # Iq_vec.txt pins ~4.3e-5
    assert abs(out64[0] - g["iq_ref_dd"][0]) / g["iq_ref_dd"][0] < 1e-9


@pytest.mark.parametrize("case", ["cfg1_n300", "cfg2_n400", "cfg4_n250"])
def test_golden_synthetic(saxs, golden_synth, case):
    s = golden_synth
    _, out64, _ = gpu_curve(saxs, s[case + "_q"], s[case + "_ff"], s[case + "_bodies"])
    assert rel(out64, s[case + "_iq_ref_dd"]) < TOL


def test_function_pointer_abi(saxs, golden_synth):
    s = golden_synth
    out = saxs.calc_saxs_curve(s["cfg1_n300_q"], s["cfg1_n300_bodies"], s["cfg1_n300_ff"])
    assert rel(out, s["cfg1_n300_iq_ref_dd"]) < TOL


def test_water_term(saxs, oracle_lib):
    w = W.make_config(1, seed=14, n_override=600)
    rng = np.random.default_rng(4)
    rs = rng.uniform(0, 1, w.n).astype(np.float32)
    with saxs.Debye(w.q, w.ff, w.n) as d:
        d.set_water(0.8, 2, rs)
        out64 = (d.calc(w.bodies), d.curve_f64())[1]
    ref = oracle_lib.debye_f64(w.q, w.bodies, w.ff, rsasa=rs, water_weight=0.8, water_index=2)
    assert rel(out64, ref) < TOL


@pytest.mark.parametrize("q_slab,n_q,ww", [(0, 201, 0.8), (64, 201, -1.5), (128, 101, 3.0),
                                           (128, 47, 0.8), (64, 130, 2.0)])
def test_water_term_wide_slabs(saxs, oracle_lib, q_slab, n_q, ww):
    """The implicit water term on uniform grids runs in the wide slabs (the
    per-(j, q) coefficient f_t + w rsasa f_w folded into the paired steps):
    compact structure (unsigned steps), several slab plans and tail widths,
    negative and large water weights; FP64 oracle."""
    w = W.make_config(2, seed=16, n_override=900)
    rng = np.random.default_rng(n_q)
    q = W.q_grid(n_q, 0.5)
    ff = W.exp_form_factors(q, W.Z5, rng.uniform(0.5, 2.0, 5))
    rs = rng.uniform(0, 1, w.n).astype(np.float32)
    with saxs.Debye(q, ff, w.n, q_slab=q_slab) as d:
        d.set_water(ww, 4, rs)
        d.calc(w.bodies)
        out64 = d.curve_f64()
        assert d.config()["uniform_q"]
    ref = oracle_lib.debye_f64(q, w.bodies, ff, rsasa=rs, water_weight=ww, water_index=4)
    assert rel(out64, ref) < TOL


@pytest.mark.parametrize("tables", [True, False])
@pytest.mark.parametrize("ww,n", [(0.0, 1500), (0.7, 1500), (-1.5, 900), (3.0, 600)])
def test_nonuniform_grid_gridded_forward(saxs, oracle_lib, ww, n, tables):
    """Non-uniform q grids run through the gridded pair-distance
    distribution (Hermite deposits on an r grid with q_max h <= 0.05, the
    sums over q evaluated on the nodes), with and without water; FP64 oracle
    at the grid's own q values."""
    w = W.make_config(2, seed=17, n_override=n)
    rng = np.random.default_rng(n)
    q = np.sort(rng.uniform(0, 0.6, 77)).astype(np.float32)
    q[0] = 0.0
    ff = W.exp_form_factors(q, W.Z5, rng.uniform(0.5, 2.0, 5))
    rs = rng.uniform(0, 1, w.n).astype(np.float32)
    with saxs.Debye(q, ff, w.n, pair_tables=tables) as d:
        if ww != 0.0:
            d.set_water(ww, 4, rs)
        d.calc(w.bodies)
        out64 = d.curve_f64()
        assert not d.config()["uniform_q"]
    kw = dict(rsasa=rs, water_weight=ww, water_index=4) if ww != 0.0 else {}
    assert rel(out64, oracle_lib.debye_f64(q, w.bodies, ff, **kw)) < TOL


def test_small_item_cap_forces_chunking(saxs, oracle_lib):
    w = W.make_config(2, seed=15, n_override=1500)
    _, _, cfg1 = gpu_curve(saxs, w.q, w.ff, w.bodies)
    _, out64, cfg = gpu_curve(saxs, w.q, w.ff, w.bodies, max_items=7)
    assert cfg["n_items"] < cfg1["n_items"]   # J runs grouped several blocks per item
    assert rel(out64, oracle_lib.debye_f64(w.q, w.bodies, w.ff)) < TOL


# ---- edge cases ------------------------------------------------------------

def test_zero_and_one_body(saxs):
    q = W.q_grid(20, 0.5)
    ff = W.exp_form_factors(q, (6, 8), (1.0, 0.5))
    out, _, _ = gpu_curve(saxs, q, ff, np.zeros((0, 4), np.float32))
    assert np.all(out == 0)
    one = W.pack_bodies(np.array([[1.0, 2.0, 3.0]]), np.array([1]))
    out, out64, _ = gpu_curve(saxs, q, ff, one)
    assert np.allclose(out64, ff[:, 1].astype(np.float64) ** 2, rtol=1e-12)


def test_coincident_bodies_give_sinc_one(saxs):
    """Distinct bodies at one position: sinc(0) = 1 (the reference's device
    kernel maps the 0/0 case to 1, gpu_saxs_pt_wf.cl:55)."""
    q = W.q_grid(33, 0.5)
    ff = W.exp_form_factors(q, (6, 8), (1.0, 0.5))
    b = W.pack_bodies(np.array([[1.0, 2.0, 3.0], [1.0, 2.0, 3.0]]), np.array([0, 1]))
    _, out64, _ = gpu_curve(saxs, q, ff, b)
    expect = (ff[:, 0].astype(np.float64) + ff[:, 1]) ** 2
    assert rel(out64, expect) < 1e-6


def test_nonuniform_grid_edge_cases(saxs, oracle_lib):
    """The gridded forward of non-uniform grids at its edges: no body, one
    body, two coincident bodies (sinc(0) = 1, node 0), two bodies, and a
    structure wide enough that its node count is past the shared-memory cap
    (the direct-sine kernel then runs)."""
    rng = np.random.default_rng(4)
    q = np.sort(rng.uniform(0, 0.5, 29)).astype(np.float32)
    q[0] = 0.0
    ff = W.exp_form_factors(q, (6, 8), (1.0, 0.5))
    out, _, cfg = gpu_curve(saxs, q, ff, np.zeros((0, 4), np.float32))
    assert not cfg["uniform_q"] and np.all(out == 0)
    one = W.pack_bodies(np.array([[1.0, 2.0, 3.0]]), np.array([1]))
    _, out64, _ = gpu_curve(saxs, q, ff, one)
    assert np.allclose(out64, ff[:, 1].astype(np.float64) ** 2, rtol=1e-12)
    same = W.pack_bodies(np.array([[1.0, 2.0, 3.0], [1.0, 2.0, 3.0]]), np.array([0, 1]))
    _, out64, _ = gpu_curve(saxs, q, ff, same)
    assert rel(out64, (ff[:, 0].astype(np.float64) + ff[:, 1]) ** 2) < 1e-6
    two = W.pack_bodies(np.array([[1.0, 2.0, 3.0], [4.5, -2.0, 7.25]]), np.array([0, 1]))
    _, out64, _ = gpu_curve(saxs, q, ff, two)
    assert rel(out64, oracle_lib.debye_f64(q, two, ff)) < TOL
    wide = W.pack_bodies(rng.uniform(-2500, 2500, (300, 3)), rng.integers(0, 2, 300))
    _, out64, _ = gpu_curve(saxs, q, ff, wide)
    assert rel(out64, oracle_lib.debye_f64(q, wide, ff)) < TOL


def test_q_zero_is_sum_squared(saxs):
    w = W.make_config(1, seed=16, n_override=500)
    _, out64, _ = gpu_curve(saxs, w.q, w.ff, w.bodies)
    f0 = w.ff[0, W.body_types(w.bodies)].astype(np.float64)
    assert abs(out64[0] - f0.sum() ** 2) / f0.sum() ** 2 < 1e-12


def test_single_q_and_empty_type(saxs, oracle_lib):
    w = W.make_config(1, seed=17, n_override=300)
    q = np.array([0.21], np.float32)
    ff = np.concatenate([w.ff[[42]], np.full((1, 3), 9.0, np.float32)], axis=1)  # types 5..7 unused
    _, out64, _ = gpu_curve(saxs, q, ff, w.bodies)
    assert rel(out64, oracle_lib.debye_f64(q, w.bodies, ff)) < TOL


def test_invalid_type_rejected(saxs):
    from resaxs_gb300 import _lib
    q = W.q_grid(8, 0.5)
    ff = np.ones((8, 2), np.float32)
    b = W.pack_bodies(np.zeros((3, 3)), np.array([0, 1, 2]))
    with saxs.Debye(q, ff, 3) as d:
        with pytest.raises(_lib.ResaxsError) as e:
            d.calc(b)
        assert e.value.code == _lib.RSX_INVALID_ARG


def test_short_host_arrays_rejected_before_the_call(saxs):
    """The Python handles check array sizes before handing pointers to the C
    calls, which read a fixed count from each; the handle stays usable."""
    from resaxs_gb300 import _lib
    q = W.q_grid(8, 0.5)
    ff = np.ones((8, 2), np.float32)
    b = W.pack_bodies(np.arange(12, dtype=np.float32).reshape(4, 3), np.array([0, 1, 0, 1]))
    with saxs.Debye(q, ff, 4) as d:
        for call in (lambda: d.calc(b[:3]), lambda: d.set_factors(ff[:7]),
                     lambda: d.set_water(0.5, 1, np.zeros(3, np.float32)),
                     lambda: d.recalc_indices(b[:1], np.array([0, 1], np.uint32)),
                     lambda: d.backward(np.ones(7, np.float32))):
            with pytest.raises(_lib.ResaxsError) as e:
                call()
            assert e.value.code == _lib.RSX_INVALID_ARG
        d.calc(b)
        with pytest.raises(_lib.ResaxsError) as e:
            d.recalc_range(b[:2], 1, 3)
        assert e.value.code == _lib.RSX_INVALID_ARG
        assert np.all(np.isfinite(d.calc(b)))


def test_permutation_and_translation_invariance_full_size(saxs):
    """Size-independent properties at the full 20,000-body size."""
    w = W.make_config(2, seed=0)
    rng = np.random.default_rng(9)
    perm = rng.permutation(w.n)
    shifted = w.bodies.copy()
    shifted[:, :3] += np.float32(3.25)   # rounding of the shifted FP32 positions stays < 1e-5
    _, a, _ = gpu_curve(saxs, w.q, w.ff, w.bodies)
    _, b, _ = gpu_curve(saxs, w.q, w.ff, w.bodies[perm])
    _, c, _ = gpu_curve(saxs, w.q, w.ff, shifted)
    assert rel(b, a) < 2e-6
    assert rel(c, a) < 1e-5


def test_full_size_config2_q_subset_vs_oracle(saxs, oracle_lib):
    """Full 20,000 bodies against the FP64 oracle on every 8th q (26 of the
    201; a uniform sub-grid, evaluated with the oracle's FP64 recurrence
    form)."""
    w = W.make_config(2, seed=0)
    _, out64, _ = gpu_curve(saxs, w.q, w.ff, w.bodies)
    sel = np.arange(0, len(w.q), 8)
    assert len(sel) >= 25
    q64 = w.q.astype(np.float64)
    dq = (q64[-1] - q64[0]) / (len(q64) - 1)
    ref = oracle_lib.debye_f64_uniform(q64[0], 8 * dq, len(sel), w.bodies, w.ff[sel])
    assert rel(out64[sel], ref) < TOL


@pytest.mark.parametrize("q_slab,n_q", [(128, 300), (192, 512), (192, 450)])
def test_four_pairs_per_step(saxs, oracle_lib, q_slab, n_q):
    """The second tile dimension: four pairs stepped together in the wide
    main slabs (128 q and more); the tail slab keeps two."""
    rng = np.random.default_rng(n_q)
    w = W.make_config(4, seed=23, n_override=700)
    q = W.q_grid(n_q, 1.0)
    ff = W.exp_form_factors(q, W.Z8, rng.uniform(0.3, 2.5, 8))
    with saxs.Debye(q, ff, w.n, q_slab=q_slab, pairs_per_step=4) as d:
        d.calc(w.bodies)
        out64 = d.curve_f64()
        cfg = d.config()
    assert cfg["pairs_per_step"] == 4 and cfg["q_slab"] == q_slab
    assert rel(out64, oracle_lib.debye_f64(q, w.bodies, ff)) < TOL
    # a spread structure takes the signed instantiation
    b = w.bodies.copy()
    b[0, :3] += np.float32(500.0)
    with saxs.Debye(q, ff, w.n, q_slab=q_slab, pairs_per_step=4) as d:
        d.calc(b)
        out64 = d.curve_f64()
    assert rel(out64, oracle_lib.debye_f64(q, b, ff)) < TOL


def test_tile_shape_options_rejected(saxs):
    from resaxs_gb300 import _lib
    w = W.make_config(1, seed=5, n_override=50)
    with pytest.raises(_lib.ResaxsError):
        saxs.Debye(w.q, w.ff, w.n, pairs_per_step=3)


def test_autotuned_slab(saxs, oracle_lib):
    from resaxs_gb300 import _lib
    _lib.lib().rsx_autotune_clear()
    w = W.make_config(2, seed=18, n_override=3000)
    _, out64, cfg = gpu_curve(saxs, w.q, w.ff, w.bodies, autotune=True)
    assert cfg["q_slab"] in (16, 32, 64, 128, 192)
    assert cfg["pairs_per_step"] in (2, 4)
    assert rel(out64, oracle_lib.debye_f64(w.q, w.bodies, w.ff)) < TOL
    _, again, cfg2 = gpu_curve(saxs, w.q, w.ff, w.bodies, autotune=True)   # cached choice
    assert cfg2["q_slab"] == cfg["q_slab"]
    assert rel(again, out64) < 1e-12


@pytest.mark.parametrize("n_q,q_max,spread,q_min", [(190, 0.5, 1.0, 0.0), (577, 0.5, 1.0, 0.0),
                                                    (700, 2.0, 8.0, 0.0), (1200, 0.6, 1.0, 0.0),
                                                    (201, 0.5, 1.0, 0.0), (201, 0.5, 1.0, 0.01),
                                                    (200, 0.5, 8.0, 0.01), (578, 0.5, 1.0, 0.01)])
def test_chained_forward_plans(saxs, oracle_lib, n_q, q_max, spread, q_min):
    """The chained forward (one seed per pair and chain of up to two 192-q
    slabs; it runs when the work items fill 4 waves, >= 8 per SM: 9,000
    bodies give ~2,700).  A grid from q = 0 runs on the q past it: 190 q as
    one 192-q slab, a full 384-q chain and a 192-q rest chain (577 q), a
    spread structure whose far pairs take the signed steps (700 q to 2.0/A:
    384, then 192 + 128), three full chains with a 48-q rest slab on the
    second stream (1,200 q), one 192 + 8 chain (201 q).  From q = 0.01: 192 +
    16 (201 q), 192 + 8 with signed steps (200 q), 384 and 192 + 8 (578 q).
    FP64 oracle on the chains' first, boundary and last q and every 23rd."""
    w = W.make_config(2, seed=21, n_override=9000)
    bodies = w.bodies.copy()
    bodies[:, :3] *= np.float32(spread)
    rng = np.random.default_rng(n_q)
    q = W.q_grid(n_q, q_max, q_min)
    ff = W.exp_form_factors(q, W.Z5, rng.uniform(0.5, 2.0, 5))
    with saxs.Debye(q, ff, len(bodies)) as d:
        d.calc(bodies)
        out64 = d.curve_f64()
        assert d.config()["n_items"] >= 8 * 152
    edges = [k + d for c in range(0, n_q, 384) for k in (c, c + 191, c + 192, c + 383)
             for d in (0, 1)]
    sel = np.array(sorted({k for k in edges + list(range(0, n_q, 23)) + [n_q - 1] if k < n_q}))
    ref = oracle_lib.debye_f64(q[sel], bodies, ff[sel])
    assert rel(out64[sel], ref) < TOL, rel(out64[sel], ref)
