"""CPU pins of the SASA oracle to the reference itself (no GPU).

The fixtures in tests/golden/sasa_ref.npz come from the reference's own
dot generators and its CPU SASA (rsasa_cpu_alg<float,float>::calc_rsasa),
compiled from its sources by oracle/build_ref.sh (tests/golden/make_golden.py).
The strict-FP32 restatement used as the GPU checker must reproduce them before
any GPU count is compared with it."""
import numpy as np
import pytest

from conftest import sasa_dot_map, sasa_dot_sets

STRUCTS = ("a", "b", "c")


def _dots_per_atom(golden, atoms, kind="latitude"):
    sizes = np.diff(golden[f"dots_{kind}_start"])
    return sizes[np.ascontiguousarray(atoms).view(np.uint32)[:, 3]]


@pytest.mark.parametrize("name", STRUCTS)
def test_typed_restatement_equals_reference_cpu_sasa(oracle_lib, golden_sasa, name):
    """Exact counts of the restatement (pre-scaled per-type dots, every
    candidate within reach) equal the reference's rsasa x dots, bit for bit."""
    g = golden_sasa
    atoms = g[f"{name}_atoms"]
    cnt = oracle_lib.sasa_counts_typed(atoms, g["radii"], sasa_dot_map(g, "latitude"),
                                       float(g["probe"]))
    n_dots = _dots_per_atom(g, atoms)
    ref = g[f"{name}_rsasa_ref"]
    assert np.array_equal(np.rint(ref * n_dots).astype(np.int64), cnt.astype(np.int64))
    # and the reference's rsasa is that count over the type's dot count, in FP32
    assert np.array_equal((cnt.astype(np.float32) / n_dots.astype(np.float32)).view(np.uint32),
                          ref.view(np.uint32))
    assert 0 < cnt.sum() < n_dots.sum()


@pytest.mark.parametrize("name", STRUCTS)
def test_cpu_port_bitexact_with_reference(oracle_lib, golden_sasa, name):
    """The port of rsasa_cpu_alg (voxel grid and all) used as the SASA CPU
    baseline reproduces the reference's rsasa bit for bit."""
    g = golden_sasa
    atoms = g[f"{name}_atoms"]
    got = oracle_lib.refport_rsasa_typed(atoms, g["radii"], sasa_dot_sets(g, "latitude"),
                                         float(g["probe"]), threads=3)
    assert np.array_equal(got.view(np.uint32), g[f"{name}_rsasa_ref"].view(np.uint32))


def test_unit_and_typed_forms_agree(oracle_lib, golden_sasa):
    """Fibonacci dots: the reference's pre-scaled set equals unit dots x
    (r + P) in FP32, so the unit and typed restatements give the same counts."""
    g = golden_sasa
    atoms = g["a_atoms"]
    types = atoms.view(np.uint32)[:, 3]
    radii = g["radii"][types]
    unit = oracle_lib.fibonacci_unit_dots(64)
    c_unit = oracle_lib.sasa_counts(atoms, radii, unit, float(g["probe"]))
    c_typed = oracle_lib.sasa_counts_typed(atoms, g["radii"], sasa_dot_map(g, "fibonacci"),
                                           float(g["probe"]))
    assert np.array_equal(c_unit, c_typed)
    c_port = oracle_lib.refport_rsasa_unit(atoms, radii, unit, float(g["probe"]), threads=2)
    assert np.array_equal(c_port, c_unit)


def test_fibonacci_unit_dots_scale_to_reference_set(oracle_lib, golden_sasa):
    """create_fibonacci_dots(r) (n = 32) is fl(unit x fl(r + P)) component by
    component, for every type radius."""
    g = golden_sasa
    unit = oracle_lib.fibonacci_unit_dots(64)
    P = np.float32(g["dots_fibonacci_probe"])
    for t, ref in enumerate(sasa_dot_sets(g, "fibonacci")):
        ext = np.float32(g["radii"][t]) + P
        assert np.array_equal((unit * ext).astype(np.float32).view(np.uint32),
                              ref[:, :3].view(np.uint32)), t
        assert np.all(ref[:, 3] == g["radii"][t])


def test_library_dot_generators_match_reference(golden_sasa):
    """Host-side generators of librsx (no GPU): the Fibonacci set scales to the
    reference's bit for bit; the dodeca-icosa unit directions scale to the
    reference's set within 2 ulp (the reference multiplies by the radius
    before the golden-ratio factors)."""
    from resaxs_gb300 import sasa
    g = golden_sasa
    fib = sasa.fibonacci_dots(64)
    di = sasa.dodeca_icosa_dots()
    for t in range(len(g["radii"])):
        ext = np.float32(g["radii"][t]) + np.float32(g["dots_fibonacci_probe"])
        ref = sasa_dot_sets(g, "fibonacci")[t][:, :3]
        assert np.array_equal((fib * ext).astype(np.float32).view(np.uint32), ref.view(np.uint32))
        ext = np.float32(g["radii"][t]) + np.float32(g["dots_dodeca_icosa_probe"])
        ref = sasa_dot_sets(g, "dodeca_icosa")[t][:, :3]
        scaled = (di * ext).astype(np.float32)
        assert np.max(np.abs(scaled - ref)) <= 2 * np.spacing(np.float32(ext))


def test_reference_dot_sets_shapes(golden_sasa):
    g = golden_sasa
    for kind, n in (("fibonacci", 64), ("dodeca_icosa", 32), ("32", None),
                    ("dodecahedron", 20)):
        for t, d in enumerate(sasa_dot_sets(g, kind)):
            if n is not None:
                assert len(d) == n, (kind, t)
            r = np.linalg.norm(d[:, :3].astype(np.float64), axis=1)
            ext = float(g["radii"][t]) + float(g[f"dots_{kind}_probe"])
            assert np.allclose(r, ext, rtol=1e-5), (kind, t)
    sizes = np.diff(g["dots_latitude_start"])
    assert np.all(sizes > 20) and np.all(np.diff(sizes[np.argsort(g["radii"])]) >= 0)


@pytest.mark.parametrize("kind", ["latitude", "32", "fibonacci", "dodecahedron", "dodeca_icosa"])
def test_library_sphere_dots_bitexact_with_reference(golden_sasa, kind):
    """rsx_sasa_sphere_dots (host code, no GPU) gives the reference
    generators' dots bit for bit for every type radius."""
    from resaxs_gb300 import sasa
    g = golden_sasa
    probe = float(g[f"dots_{kind}_probe"])
    for t, ref in enumerate(sasa_dot_sets(g, kind)):
        got = sasa.sphere_dots(kind, float(g["radii"][t]), probe, float(g["density"]))
        assert got.shape == ref.shape, (kind, t)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (kind, t)


def test_library_sphere_dots_rejects_bad_input():
    from resaxs_gb300 import _lib, sasa
    with pytest.raises(_lib.ResaxsError):
        sasa.sphere_dots("latitude", 1.5, 1.4, -1.0)
    with pytest.raises(_lib.ResaxsError):
        sasa.sphere_dots("fibonacci", float("nan"), 1.4)
    big = sasa.sphere_dots("latitude", 1.9, 1.4, 50.0)   # grows the output buffer
    assert len(big) > 1000
