"""Dot-sphere SASA: GPU counts must equal the strict-FP32 oracle bit for bit."""
import numpy as np
import pytest

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
