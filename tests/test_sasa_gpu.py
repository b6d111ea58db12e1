"""Dot-sphere SASA: GPU counts must equal the strict-FP32 oracle and the
reference's own CPU SASA bit for bit."""
import numpy as np
import pytest

from conftest import sasa_dot_map
from resaxs_gb300 import workloads as W


def test_fibonacci_dots_match_oracle_bitwise(oracle_lib):
    """Host-side generator (no GPU): same FP32 bits as the oracle's restatement
    of create_fibonacci_dots (rsasa_algorithm.cpp:96-116)."""
    from resaxs_gb300 import sasa
    for n in (2, 64, 960, 4096):
        a = sasa.fibonacci_dots(n)
        b = oracle_lib.fibonacci_unit_dots(n)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), n


def test_dodeca_icosa_dots_are_unit_vectors():
    from resaxs_gb300 import sasa
    d = sasa.dodeca_icosa_dots().astype(np.float64)
    assert d.shape == (32, 3)
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=2e-6)
    assert len({tuple(np.round(x, 5)) for x in d}) == 32


def test_invalid_dot_counts_rejected():
    from resaxs_gb300 import _lib, sasa
    with pytest.raises(_lib.ResaxsError):
        sasa.fibonacci_dots(7)


gpu = pytest.mark.gpu


def _case(n, seed, compact=True):
    rng = np.random.default_rng(seed)
    if compact:
        xyz = W.confined_chain(n, rng, 25.0 * (n / 20000) ** (1 / 3) * 1.29)
    else:
        xyz = W.random_walk_chain(n, rng)
    atoms = W.pack_bodies(xyz, np.zeros(n, np.uint32))
    radii = rng.uniform(1.2, 1.9, n).astype(np.float32)
    return atoms, radii


@gpu
def test_full_config2_counts_bitexact(oracle_lib):
    """Config 2: 20,000 atoms, 960 Fibonacci dots, radii U[1.2,1.9], probe 1.4."""
    from resaxs_gb300.sasa import DotSphereSasa
    w = W.make_config(2, seed=0)
    radii = np.random.default_rng(0).uniform(1.2, 1.9, w.n).astype(np.float32)
    dots = oracle_lib.fibonacci_unit_dots(960)
    with DotSphereSasa(w.n, n_dots=960, probe=1.4) as s:
        got = s.counts(w.bodies, radii)
        tests, ms = s.stats()
    ref = oracle_lib.sasa_counts(w.bodies, radii, dots, 1.4)
    assert np.array_equal(got, ref), int(np.sum(got != ref))
    assert tests > 0 and ms > 0


@gpu
@pytest.mark.parametrize("n,n_dots,probe,compact", [(2000, 960, 1.4, False),
                                                    (3000, 100, 1.4, True),
                                                    (1500, 4096, 1.8, False),
                                                    (700, 2, 0.0, True)])
def test_counts_bitexact_variants(oracle_lib, n, n_dots, probe, compact):
    from resaxs_gb300.sasa import DotSphereSasa
    atoms, radii = _case(n, n + n_dots, compact)
    dots = oracle_lib.fibonacci_unit_dots(n_dots)
    with DotSphereSasa(n, n_dots=n_dots, probe=probe) as s:
        got = s.counts(atoms, radii)
    assert np.array_equal(got, oracle_lib.sasa_counts(atoms, radii, dots, probe))


@gpu
def test_dodeca_icosa_set_and_rsasa(oracle_lib):
    from resaxs_gb300 import sasa
    atoms, radii = _case(1200, 5, False)
    dots = sasa.dodeca_icosa_dots()
    with sasa.DotSphereSasa(1200, probe=1.8, unit_dots=dots) as s:
        got = s.counts(atoms, radii)
        rs = s.rsasa(atoms, radii)
    ref = oracle_lib.sasa_counts(atoms, radii, dots, 1.8)
    assert np.array_equal(got, ref)
    assert np.array_equal(rs, (ref / np.float32(32)).astype(np.float32))


@gpu
def test_isolated_large_coordinates_and_duplicates(oracle_lib):
    """Far-apart atoms at large coordinates (self-occlusion rounding as the
    reference's test has it), exact duplicates, a zero radius."""
    from resaxs_gb300.sasa import DotSphereSasa
    xyz = np.array([[0, 0, 0], [1000.5, -2000.25, 300.0], [5e4, 5e4, 5e4], [3.0, 0, 0],
                    [3.0, 0, 0], [0, 7.0, 0]], np.float32)
    atoms = W.pack_bodies(xyz, np.zeros(len(xyz), np.uint32))
    radii = np.array([1.5, 1.9, 1.2, 1.6, 1.6, 0.0], np.float32)
    dots = oracle_lib.fibonacci_unit_dots(960)
    with DotSphereSasa(len(xyz), n_dots=960, probe=1.4) as s:
        got = s.counts(atoms, radii)
    ref = oracle_lib.sasa_counts(atoms, radii, dots, 1.4, use_cells=False)
    assert np.array_equal(got, ref)


@gpu
def test_rsasa_algorithm_mirror(oracle_lib):
    from resaxs_gb300 import _lib
    from resaxs_gb300.sasa import RsasaAlgorithm
    rng = np.random.default_rng(3)
    n = 900
    xyz = W.random_walk_chain(n, rng)
    types = rng.integers(0, 3, n)
    atoms = W.pack_bodies(xyz, types)
    radius_of_type = np.array([1.7, 1.55, 1.52], np.float32)
    alg = RsasaAlgorithm()
    with pytest.raises(_lib.ResaxsError):
        alg.recalc_rsasa(atoms)
    alg.initialize(n, radius_of_type, probe_radius=1.4, n_dots=256)
    out = np.zeros(n, np.float32)
    alg.calc_rsasa(atoms, out)
    ref = oracle_lib.sasa_counts(atoms, radius_of_type[types], oracle_lib.fibonacci_unit_dots(256), 1.4)
    assert np.array_equal(out, (ref / np.float32(256)).astype(np.float32))
    again = alg.recalc_rsasa(atoms)
    assert np.array_equal(again, out)


@gpu
def test_bad_inputs_rejected():
    from resaxs_gb300 import _lib
    from resaxs_gb300.sasa import DotSphereSasa
    atoms = W.pack_bodies(np.zeros((3, 3)), np.zeros(3, np.uint32))
    with DotSphereSasa(3, n_dots=32) as s:
        with pytest.raises(_lib.ResaxsError) as e:
            s.counts(atoms, np.array([1.0, -1.0, 1.0], np.float32))
        assert e.value.code == _lib.RSX_INVALID_ARG
        bad = atoms.copy()
        bad[1, 0] = np.nan
        with pytest.raises(_lib.ResaxsError):
            s.counts(bad, np.ones(3, np.float32))
    with pytest.raises(_lib.ResaxsError):
        DotSphereSasa(3, unit_dots=np.zeros((4097, 3), np.float32))
    # short host arrays are refused before the C call reads n values from them
    with DotSphereSasa(3, n_dots=32) as s:
        for args in ((atoms[:2], np.ones(3, np.float32)), (atoms, np.ones(2, np.float32))):
            with pytest.raises(_lib.ResaxsError) as e:
                s.rsasa(*args)
            assert e.value.code == _lib.RSX_INVALID_ARG
        assert s.counts(atoms, np.ones(3, np.float32)).shape == (3,)


# ---- the reference's own dot layout (typed handles) -----------------------------


def _types(atoms):
    return np.ascontiguousarray(atoms, np.float32).view(np.uint32)[:, 3]


@gpu
@pytest.mark.parametrize("name", ["a", "b", "c"])
def test_typed_counts_equal_reference_cpu_sasa(golden_sasa, name):
    """The reference's per-type latitude dot sets (create_dots, 5 dots/A^2,
    probe 1.4) through rsx_sasa_create_typed: counts and rsasa equal those of
    the reference's compiled rsasa_cpu_alg<float,float>::calc_rsasa."""
    from resaxs_gb300.sasa import TypedDotSphereSasa
    g = golden_sasa
    atoms = g[f"{name}_atoms"]
    n_dots = np.diff(g["dots_latitude_start"])[_types(atoms)]
    ref = g[f"{name}_rsasa_ref"]
    with TypedDotSphereSasa(len(atoms), sasa_dot_map(g, "latitude"), g["radii"],
                            float(g["probe"])) as s:
        got = s.counts(atoms)
        rs = s.rsasa(atoms)
        tests, ms = s.stats()
    assert np.array_equal(got.astype(np.int64), np.rint(ref * n_dots).astype(np.int64)), \
        int(np.sum(got != np.rint(ref * n_dots)))
    assert np.array_equal(rs.view(np.uint32), ref.view(np.uint32))
    assert tests > 0 and ms > 0


@gpu
@pytest.mark.parametrize("kind", ["dodeca_icosa", "fibonacci", "32", "dodecahedron"])
def test_typed_reference_dot_maps_match_oracle(oracle_lib, golden_sasa, kind):
    """The reference's other generators, including the OpenCL algorithm's
    dodeca-icosa map (32 dots per type, probe 1.8), on all 16 types."""
    from resaxs_gb300.sasa import TypedDotSphereSasa
    g = golden_sasa
    atoms = g["b_atoms"]
    dm = sasa_dot_map(g, kind)
    probe = float(g[f"dots_{kind}_probe"])
    with TypedDotSphereSasa(len(atoms), dm, g["radii"], probe) as s:
        got = s.counts(atoms)
    ref = oracle_lib.sasa_counts_typed(atoms, g["radii"], dm, probe)
    assert np.array_equal(got, ref), int(np.sum(got != ref))


@gpu
def test_typed_and_unit_forms_agree(golden_sasa):
    """Fibonacci dots: the reference's pre-scaled per-type set and the unit
    set scaled in the kernel give the same counts."""
    from resaxs_gb300.sasa import DotSphereSasa, TypedDotSphereSasa, fibonacci_dots
    g = golden_sasa
    atoms = g["a_atoms"]
    radii = g["radii"][_types(atoms)]
    with TypedDotSphereSasa(len(atoms), sasa_dot_map(g, "fibonacci"), g["radii"],
                            float(g["probe"])) as s:
        typed = s.counts(atoms)
    with DotSphereSasa(len(atoms), probe=float(g["probe"]), unit_dots=fibonacci_dots(64)) as s:
        unit = s.counts(atoms, radii)
    assert np.array_equal(typed, unit)


@gpu
def test_typed_edge_cases(oracle_lib, golden_sasa):
    """One atom; duplicates; a type whose dot set is all padding; atoms at
    large coordinates; a dot map whose padding sits between dots."""
    from resaxs_gb300.sasa import TypedDotSphereSasa
    g = golden_sasa
    dm = sasa_dot_map(g, "latitude")
    dm[5, :] = -np.inf                       # type 5: no dots
    dm[3, ::7] = np.nan                       # padding inside type 3's set
    xyz = np.array([[0, 0, 0], [2.5, 0, 0], [2.5, 0, 0], [1e4, -3e4, 5e3], [1e4 + 3.1, -3e4, 5e3],
                    [0, 0, 3.0], [-2.0, 1.0, 0.5]], np.float32)
    atoms = W.pack_bodies(xyz, np.array([0, 3, 3, 2, 3, 5, 11], np.uint32))
    for sub in (atoms[:1], atoms):
        with TypedDotSphereSasa(len(sub), dm, g["radii"], 1.4) as s:
            got = s.counts(sub)
            rs = s.rsasa(sub)
        ref = oracle_lib.sasa_counts_typed(sub, g["radii"], dm, 1.4)
        assert np.array_equal(got, ref)
        n_dots = np.isfinite(dm[:, :, 0]).sum(axis=1)[_types(sub)]
        with np.errstate(invalid="ignore", divide="ignore"):
            want = got.astype(np.float32) / n_dots.astype(np.float32)
        assert np.array_equal(np.isnan(rs), np.isnan(want))
        assert np.array_equal(rs[~np.isnan(rs)], want[~np.isnan(want)])


@gpu
def test_typed_bad_inputs(golden_sasa):
    from resaxs_gb300 import _lib
    from resaxs_gb300.sasa import TypedDotSphereSasa
    g = golden_sasa
    dm = sasa_dot_map(g, "dodeca_icosa")
    atoms = W.pack_bodies(np.zeros((2, 3), np.float32), np.array([0, 16], np.uint32))
    with TypedDotSphereSasa(2, dm, g["radii"], 1.8) as s:
        with pytest.raises(_lib.ResaxsError) as e:
            s.counts(atoms)                   # type 16 is outside the 16-type map
        assert e.value.code == _lib.RSX_INVALID_ARG
        status = _lib.lib().rsx_sasa_counts(s._h, atoms.reshape(-1), np.ones(2, np.float32),
                                            np.zeros(2, np.uint32))
        assert status == _lib.RSX_INVALID_ARG  # unit-form call on a typed handle
    with pytest.raises(_lib.ResaxsError):
        TypedDotSphereSasa(2, dm, -g["radii"], 1.8)


@gpu
@pytest.mark.parametrize("name", ["a", "c"])
def test_rsasa_mirror_reproduces_reference_cpu_algorithm(golden_sasa, name):
    """i_rsasa mirror initialized like the reference's rsasa_cpu_alg
    (dot_spheres_params(5 dots/A^2, probe 1.4), the create_dots sphere of each
    atomic radius): calc_rsasa and recalc_rsasa give the reference's rsasa bit
    for bit."""
    from resaxs_gb300.sasa import RsasaAlgorithm
    g = golden_sasa
    atoms = g[f"{name}_atoms"]
    alg = RsasaAlgorithm()
    alg.initialize(len(atoms), dot_density=float(g["density"]), probe_radius=float(g["probe"]),
                   dot_kind="latitude")
    out = np.zeros(len(atoms), np.float32)
    alg.calc_rsasa(atoms, out)
    assert np.array_equal(out.view(np.uint32), g[f"{name}_rsasa_ref"].view(np.uint32))
    again = alg.recalc_rsasa(atoms)
    assert np.array_equal(again, out)
