"""Regenerates the golden fixtures in this folder from the reference tree.

Run in a container that has the reference sources:

    python tests/golden/make_golden.py <reference_root>

Outputs (committed, so that tests on machines without the reference tree
can use them):

* ``test1888.npz`` -- the reference's own known-answer fixture
  (test_resaxs/test1888.{pos_matrix,ff_db,q_vec,Iq_vec}.txt: 1888 bodies,
  21 factor types, 51 q) parsed the way test_resaxs/SAXSTest.cpp:68-156 parses
  it (values read as float), plus the outputs of the reference's compiled
  host_debye (oracle/_ref) on it: ``iq_ref_df`` = host_debye<double,float>,
  ``iq_ref_dd`` = host_debye<double,double>.
* ``synthetic_ref.npz`` -- small seeded synthetic cases and the outputs of the
  compiled reference host_debye<double,float> and <double,double> on them.
* ``ff_ref.npz`` -- form-factor tables and radii of the reference's
  atomic_form_factors (resaxslib/include/ff_coef.hpp) for q = 0..0.75 (500
  points) and three (expansion factor, mean radius) pairs.
* ``synthetic_a.pdb``, ``synthetic_nonl.pdb`` and ``pdb_ref.npz`` -- two
  synthetic PDB files (resaxs_gb300.workloads.write_synthetic_pdb: waters,
  alternate locations, hydrogens, unknown and blank elements, short and
  over-long lines; the second ends in an ATOM line with no newline) and the
  bodies the reference's own parse_pdb<float>::all_models_as_complex_atoms
  (resaxslib/src/parse_pdb.cpp, compiled into oracle/_ref) reads from them.

* ``sasa_ref.npz`` -- the reference's dot-sphere SASA: the 16 atom-type radii
  of atomic_form_factors::calc_radii, the dot sets its dot_spheres_params
  generators make for each type radius (create_dots at 5 dots/A^2 and probe
  1.4 A -- the CPU algorithm's set; create_dodeca_icosa_dots at probe 1.8 A --
  the OpenCL algorithm's set; create_fibonacci_dots, create_32_dots and
  create_dodecahedron_dots at 1.4 A), and the rsasa of the reference's own
  rsasa_cpu_alg<float,float>::calc_rsasa (rsasa_cpu_alg.cpp, compiled into
  oracle/_ref) on three seeded structures: ``a`` uses only the types whose
  radius is <= 1.5 A (there the reference's max_radius neighbour prune is
  exact), ``b`` all 16 types, ``c`` a free (spread) chain.

``python tests/golden/make_golden.py <reference_root> --only pdb`` (or
``--only sasa``) rewrites only those fixtures.
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from resaxs_gb300 import workloads as W  # noqa: E402


def parse_test1888(ref_root):
    base = os.path.join(ref_root, "test_resaxs", "test1888")
    q = np.array(open(base + ".q_vec.txt").read().split(), dtype=np.float32)
    rows = re.findall(r"\[([^\[\]]*)\]", open(base + ".ff_db.txt").read())
    ff = np.array([[float(v) for v in r.split(",")] for r in rows], dtype=np.float32)
    pos = open(base + ".pos_matrix.txt").read().split()
    arr = np.array(pos, dtype=np.float64).reshape(-1, 4)
    bodies = W.pack_bodies(arr[:, :3].astype(np.float32), arr[:, 3].astype(np.uint32))
    iq = np.array(open(base + ".Iq_vec.txt").read().split(), dtype=np.float64).reshape(-1, 2)
    return q, ff, bodies, iq[:, 1].astype(np.float32)


def ref_df(q, bodies, ff):
    out = np.zeros(len(q), np.float32)
    oracle.ref_lib().ref_host_debye_df(np.ascontiguousarray(q, np.float32), len(q),
                                       bodies.reshape(-1), len(bodies),
                                       np.ascontiguousarray(ff).reshape(-1), ff.shape[1], out)
    return out


def ref_dd(q, bodies, ff):
    b64 = np.zeros((len(bodies), 4), np.float64)
    b64[:, :3] = bodies[:, :3]
    b64.view(np.uint64)[:, 3] = W.body_types(bodies).astype(np.uint64)
    out = np.zeros(len(q), np.float64)
    oracle.ref_lib().ref_host_debye_dd(np.ascontiguousarray(q, np.float64), len(q),
                                       b64.reshape(-1), len(bodies),
                                       np.ascontiguousarray(ff, np.float64).reshape(-1),
                                       ff.shape[1], out)
    return out


def ref_parse_pdb(path):
    import ctypes
    L = oracle.ref_lib()
    f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
    L.ref_parse_pdb.argtypes = [ctypes.c_char_p, f32p, ctypes.c_int, i32p, ctypes.c_int]
    out = np.zeros((100000, 4), np.float32)
    sizes = np.zeros(64, np.int32)
    k = L.ref_parse_pdb(path.encode(), out.reshape(-1), len(out), sizes, len(sizes))
    if k < 0:
        raise RuntimeError(f"reference parse of {path} failed: {k}")
    return out[: sizes[:k].sum()].copy(), sizes[:k].copy()


def make_pdb_fixtures():
    a = os.path.join(HERE, "synthetic_a.pdb")
    W.write_synthetic_pdb(a, n_residues=40, n_models=3, seed=3)
    b = os.path.join(HERE, "synthetic_nonl.pdb")
    W.write_synthetic_pdb(b, n_residues=12, n_models=1, seed=5)
    lines = open(b).read().split("\n")
    atom = [ln for ln in lines if ln.startswith("ATOM")]
    body = [ln for ln in lines if not ln.startswith(("ENDMDL", "END "))
            and ln.strip() != "END" and ln != ""]
    with open(b, "w") as f:  # last record an ATOM line with no newline
        f.write("\n".join(body + [atom[0]]))
    fa, sa = ref_parse_pdb(a)
    fb, sb = ref_parse_pdb(b)
    np.savez_compressed(os.path.join(HERE, "pdb_ref.npz"), a_bodies=fa, a_sizes=sa,
                        nonl_bodies=fb, nonl_sizes=sb)


SASA_DENSITY = 5.0
SASA_PROBE = 1.4
SASA_TYPES_EXACT = (0, 2, 3, 4, 6, 10, 11)   # calc_radii <= 1.5 A


def sasa_structure(name):
    """The seeded structures of sasa_ref.npz: (atoms float4 with type bits)."""
    import math
    if name == "a":
        n, rng, pool = 3000, np.random.default_rng(31), SASA_TYPES_EXACT
        xyz = W.confined_chain(n, rng, 25.0 * (n / 20000) ** (1 / 3) * math.sqrt(5 / 3))
    elif name == "b":
        n, rng, pool = 2000, np.random.default_rng(32), tuple(range(16))
        xyz = W.confined_chain(n, rng, 25.0 * (n / 20000) ** (1 / 3) * math.sqrt(5 / 3))
    else:
        n, rng, pool = 1500, np.random.default_rng(33), SASA_TYPES_EXACT
        xyz = W.random_walk_chain(n, rng) + np.array([250.0, -40.0, 1000.0])
    types = rng.choice(np.array(pool), n).astype(np.uint32)
    return W.pack_bodies(xyz, types)


def make_sasa_fixtures():
    radii = np.load(os.path.join(HERE, "ff_ref.npz"))["radii"]
    out = {"radii": radii, "density": np.float32(SASA_DENSITY), "probe": np.float32(SASA_PROBE)}
    for kind, probe in (("latitude", SASA_PROBE), ("dodeca_icosa", 1.8), ("fibonacci", SASA_PROBE),
                        ("32", SASA_PROBE), ("dodecahedron", SASA_PROBE)):
        sets = [oracle.ref_sasa_dots(kind, r, SASA_DENSITY, probe) for r in radii]
        out[f"dots_{kind}"] = np.concatenate(sets)
        out[f"dots_{kind}_start"] = np.concatenate([[0], np.cumsum([len(d) for d in sets])]
                                                  ).astype(np.int32)
        out[f"dots_{kind}_probe"] = np.float32(probe)
    for name in ("a", "b", "c"):
        atoms = sasa_structure(name)
        out[f"{name}_atoms"] = atoms
        out[f"{name}_rsasa_ref"] = oracle.ref_rsasa_cpu(atoms, SASA_DENSITY, SASA_PROBE)
    np.savez_compressed(os.path.join(HERE, "sasa_ref.npz"), **out)


def main(ref_root=None, only=None):
    ref_root = ref_root or os.environ.get("RESAXS_REFERENCE_ROOT")
    oracle.build()
    if oracle.build_ref(ref_root) is None:
        raise SystemExit(f"reference tree not found at {ref_root!r}")
    if only in (None, "sasa"):
        make_sasa_fixtures()
    if only == "sasa":
        return
    make_pdb_fixtures()
    if only == "pdb":
        return
    q, ff, bodies, iq = parse_test1888(ref_root)
    np.savez_compressed(os.path.join(HERE, "test1888.npz"), q=q, ff=ff, bodies=bodies, iq=iq,
                        iq_ref_df=ref_df(q, bodies, ff), iq_ref_dd=ref_dd(q, bodies, ff))
    cases = {}
    for name, idx, n in (("cfg1_n300", 1, 300), ("cfg2_n400", 2, 400), ("cfg4_n250", 4, 250)):
        w = W.make_config(idx, seed=7, n_override=n)
        cases[name + "_q"] = w.q
        cases[name + "_ff"] = w.ff
        cases[name + "_bodies"] = w.bodies
        cases[name + "_iq_ref_df"] = ref_df(w.q, w.bodies, w.ff)
        cases[name + "_iq_ref_dd"] = ref_dd(w.q, w.bodies, w.ff)
    np.savez_compressed(os.path.join(HERE, "synthetic_ref.npz"), **cases)
    # form-factor tables of the reference (ff_coef.hpp) for the CLI's q grid
    L = oracle.ref_lib()
    import ctypes
    f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    L.ref_ff_generate.argtypes = [f32p, ctypes.c_int, ctypes.c_float, ctypes.c_float, f32p]
    L.ref_ff_radii.argtypes = [f32p]
    qq = np.linspace(0.0, 0.75, 500).astype(np.float32)
    ff_cases = {"q": qq}
    for name, c, rm in (("c100", 1.0, 1.6), ("c103", 1.03, 1.65), ("c095", 0.95, 1.5)):
        out = np.zeros(len(qq) * 16, np.float32)
        L.ref_ff_generate(qq, len(qq), ctypes.c_float(rm), ctypes.c_float(c), out)
        ff_cases[name] = out.reshape(len(qq), 16)
        ff_cases[name + "_args"] = np.array([c, rm], np.float32)
    radii = np.zeros(16, np.float32)
    L.ref_ff_radii(radii)
    ff_cases["radii"] = radii
    np.savez_compressed(os.path.join(HERE, "ff_ref.npz"), **ff_cases)
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--only")]
    only = None
    if "--only" in sys.argv:
        only = sys.argv[sys.argv.index("--only") + 1]
        args = [a for a in args if a != only]
    main(*args, only=only)
