"""CPU tests of the oracle itself: it must reproduce the reference's own known
answers before the GPU path is checked against it."""
import numpy as np
import pytest

from resaxs_gb300 import workloads as W


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))


def test_test1888_golden_file(oracle_lib, golden_1888):
    """test_resaxs/test1888.Iq_vec.txt pins I(q) to ~5e-5 (the file was made by
    another code; the reference's own host_debye differs from it by 4.3e-5)."""
    g = golden_1888
    o = oracle_lib.debye_f64(g["q"], g["bodies"], g["ff"])
    assert rel(o, g["iq"]) < 5e-5
    assert abs(o[0] - g["iq"][0]) / g["iq"][0] < 1e-8  # q = 0 is exact


def test_test1888_matches_compiled_reference(oracle_lib, golden_1888):
    g = golden_1888
    o = oracle_lib.debye_f64(g["q"], g["bodies"], g["ff"])
    assert rel(o, g["iq_ref_dd"]) < 1e-12          # host_debye<double,double>
    assert rel(o, g["iq_ref_df"]) < 2e-7           # host_debye<double,float> (FP32 output)


@pytest.mark.parametrize("case", ["cfg1_n300", "cfg2_n400", "cfg4_n250"])
def test_synthetic_matches_compiled_reference(oracle_lib, golden_synth, case):
    s = golden_synth
    o = oracle_lib.debye_f64(s[case + "_q"], s[case + "_bodies"], s[case + "_ff"])
    assert rel(o, s[case + "_iq_ref_dd"]) < 1e-12


@pytest.mark.parametrize("case", ["cfg1_n300", "cfg2_n400", "cfg4_n250"])
def test_refport_bitexact(oracle_lib, golden_synth, case):
    """The CPU-baseline port equals the compiled reference host_debye<double,float>
    bit for bit on x86 (same operation order)."""
    import platform
    s = golden_synth
    p, _ = oracle_lib.refport_host_debye(s[case + "_q"], s[case + "_bodies"], s[case + "_ff"])
    if platform.machine() == "x86_64":
        assert np.array_equal(p, s[case + "_iq_ref_df"])
    else:
        assert rel(p, s[case + "_iq_ref_df"]) < 1e-6
    p2, _ = oracle_lib.refport_host_debye(s[case + "_q"], s[case + "_bodies"], s[case + "_ff"],
                                          threads=3)
    assert np.array_equal(p, p2)


def test_uniform_oracle_matches_direct(oracle_lib):
    w = W.make_config(2, seed=3, n_override=300)
    q = w.q.astype(np.float64)
    exact_q = q[0] + (q[-1] - q[0]) / (len(q) - 1) * np.arange(len(q))
    d = oracle_lib.debye_f64(exact_q, w.bodies, w.ff)
    u = oracle_lib.debye_f64_uniform(exact_q[0], exact_q[1] - exact_q[0], len(q), w.bodies, w.ff)
    assert rel(u, d) < 1e-11


def test_oracle_water_term(oracle_lib):
    """f = F + rsasa * F_w * w (gpu_saxs_pt_wf.cl:130-138): with rsasa = 1 for
    every body and weight w, the curve equals one with factors F + w F_w."""
    w = W.make_config(1, seed=1, n_override=120)
    ww, widx = 0.7, 2
    rs = np.ones(w.n, np.float32)
    a = oracle_lib.debye_f64(w.q, w.bodies, w.ff, rsasa=rs, water_weight=ww, water_index=widx)
    ff2 = (w.ff.astype(np.float64) + ww * w.ff[:, [widx]].astype(np.float64)).astype(np.float32)
    b = oracle_lib.debye_f64(w.q, w.bodies, ff2)
    assert rel(a, b) < 1e-6


def test_oracle_gradient_finite_differences(oracle_lib):
    w = W.make_config(1, seed=2, n_override=60)
    q = w.q.astype(np.float64)
    rng = np.random.default_rng(0)
    lam = rng.normal(size=len(q))
    g = oracle_lib.debye_grad_f64(q, lam, w.bodies, w.ff)
    h = 1e-3
    for (i, c) in [(0, 0), (7, 1), (33, 2), (59, 0)]:
        bp = w.bodies.copy()
        bm = w.bodies.copy()
        bp[i, c] += h
        bm[i, c] -= h
        # positions are float32: use the actually represented step
        step = float(bp[i, c]) - float(bm[i, c])
        lp = lam @ oracle_lib.debye_f64(q, bp, w.ff)
        lm = lam @ oracle_lib.debye_f64(q, bm, w.ff)
        fd = (lp - lm) / step
        assert abs(fd - g[i, c]) <= 2e-3 * max(1.0, abs(g[i, c])) + 1e-6 * np.abs(g).max()


def test_sasa_cells_equal_brute_force(oracle_lib):
    rng = np.random.default_rng(5)
    xyz = W.confined_chain(400, rng, 14.0)
    atoms = W.pack_bodies(xyz, np.zeros(400, np.uint32))
    radii = rng.uniform(1.2, 1.9, 400).astype(np.float32)
    dots = oracle_lib.fibonacci_unit_dots(64)
    a = oracle_lib.sasa_counts(atoms, radii, dots, 1.4, use_cells=False)
    b = oracle_lib.sasa_counts(atoms, radii, dots, 1.4, use_cells=True)
    assert np.array_equal(a, b)
    assert 0 < a.sum() < 400 * 64


def test_sasa_isolated_atoms_fully_exposed(oracle_lib):
    xyz = np.array([[0, 0, 0], [50, 0, 0], [0, 80, 0]], np.float32)
    atoms = W.pack_bodies(xyz, np.zeros(3, np.uint32))
    radii = np.full(3, 1.5, np.float32)
    dots = oracle_lib.fibonacci_unit_dots(960)
    assert np.array_equal(oracle_lib.sasa_counts(atoms, radii, dots, 1.4), [960, 960, 960])


def test_fibonacci_dots_on_unit_sphere(oracle_lib):
    d = oracle_lib.fibonacci_unit_dots(960).astype(np.float64)
    assert d.shape == (960, 3)
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)
    # reference formula: z = i/n for i in [-(n-1), n]
    n = 480
    assert np.allclose(d[:, 2], np.arange(-(n - 1), n + 1) / n, atol=1e-7)
