"""The calc_saxs command line (resaxs_gb300/cli/calc_saxs.cpp) and the PDB
reader behind it.

CPU: the reader against the bodies the reference's own parse_pdb reads from
the same files (tests/golden/pdb_ref.npz), and the CLI's argument and file
errors (calc_saxs/main.cpp:176-318), which stop before any GPU work.
GPU: the written curve against the FP64 oracle for fixed parameters, and the
parameter fit recovering known scale / water weight / expansion factor."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def _read_pdb(path):
    from resaxs_gb300 import _lib
    L = _lib.lib()
    nm, nb = ctypes.c_int(), ctypes.c_int()
    _lib.check(L.rsx_pdb_count(path.encode(), ctypes.byref(nm), ctypes.byref(nb)))
    out = np.zeros((max(nb.value, 1), 4), np.float32)
    sizes = np.zeros(max(nm.value, 1), np.int32)
    _lib.check(L.rsx_pdb_read(path.encode(), 0, out.reshape(-1), nb.value, sizes, nm.value))
    return out[: nb.value], sizes[: nm.value]


@pytest.fixture(scope="module")
def cli():
    from resaxs_gb300 import build as B
    exe = os.path.join(B.BIN_DIR, "calc_saxs")
    if not os.path.exists(exe) or os.path.getmtime(exe) < os.path.getmtime(B.LIB):
        exe = B.build_cli()
    return exe


def _run(exe, args, cwd):
    return subprocess.run([exe] + args, cwd=cwd, capture_output=True, text=True, timeout=600)


# ------------------------------------------------------------------ CPU ---

@pytest.mark.parametrize("name", ["a", "nonl"])
def test_pdb_reader_matches_reference_parser(name):
    path = os.path.join(GOLD, "synthetic_a.pdb" if name == "a" else "synthetic_nonl.pdb")
    ref = np.load(os.path.join(GOLD, "pdb_ref.npz"))
    bodies, sizes = _read_pdb(path)
    np.testing.assert_array_equal(sizes, ref[name + "_sizes"])
    # bit-exact: coordinates and the type bits in .w
    np.testing.assert_array_equal(bodies.view(np.uint32), ref[name + "_bodies"].view(np.uint32))


def test_pdb_reader_types_and_skips():
    from resaxs_gb300 import workloads as W
    bodies, sizes = _read_pdb(os.path.join(GOLD, "synthetic_a.pdb"))
    t = W.body_types(bodies)
    assert len(sizes) == 3 and len(set(sizes.tolist())) == 1
    assert not np.any(t == 0)  # hydrogens never become bodies
    assert not np.any(t == 14)  # nor waters (OH2 is the implicit water group)
    assert np.all(t < 16)
    # complex groups are present (CH, CH2, CH3, NH, ...)
    assert {7, 8, 9, 10} <= set(t.tolist())


def test_pdb_missing_file_code():
    from resaxs_gb300 import _lib
    L = _lib.lib()
    nm, nb = ctypes.c_int(), ctypes.c_int()
    assert L.rsx_pdb_count(b"/nonexistent/x.pdb", ctypes.byref(nm),
                           ctypes.byref(nb)) == _lib.RSX_PDB_FILE_NOT_FOUND
    assert "file not found" in _lib.last_error()


def test_cli_requires_outfile_and_inputs(cli, tmp_path):
    r = _run(cli, [os.path.join(GOLD, "synthetic_a.pdb")], tmp_path)
    assert r.returncode == 1 and "PARSE ERROR" in r.stderr and "outfile" in r.stderr
    r = _run(cli, ["-o", "out.dat"], tmp_path)
    assert r.returncode == 1 and "pdb_files" in r.stderr
    r = _run(cli, ["-v", "loud", "-o", "o", "x.pdb"], tmp_path)
    assert r.returncode == 1 and "quiet|normal|details|debug" in r.stderr


def test_cli_range_checks(cli, tmp_path):
    # ranges outside [-2,4] / [0.95,1.05] are argument errors
    r = _run(cli, ["-w", "[-3,1]", "-f", "p", "-o", "o", "x.pdb"], tmp_path)
    assert r.returncode == 1 and "valid range" in r.stderr
    r = _run(cli, ["-e", "1.2", "-f", "p", "-o", "o", "x.pdb"], tmp_path)
    assert r.returncode == 1 and "valid range" in r.stderr
    # a range without an experimental profile: message, exit status 0
    r = _run(cli, ["-w", "[0,1]", "-o", "o", "x.pdb"], tmp_path)
    assert r.returncode == 0 and "without an experimental profile" in r.stderr
    assert not os.path.exists(tmp_path / "o")


def test_cli_missing_profile_and_pdb(cli, tmp_path):
    # the profile is read first (calc_saxs/main.cpp:262-266): -1101
    r = _run(cli, ["-o", "o", os.path.join(GOLD, "synthetic_a.pdb")], tmp_path)
    assert r.returncode == 255 and "(-1101)" in r.stderr
    prof = tmp_path / "p.dat"
    prof.write_text("# q I err\n0.01 100 1\n0.02 90 1\n")
    r = _run(cli, ["-f", str(prof), "-o", "o", str(tmp_path / "missing.pdb")], tmp_path)
    assert r.returncode == 255 and "(-1100)" in r.stderr


# ------------------------------------------------------------------ GPU ---

def _write_profile(path, q, iq, err=None):
    with open(path, "w") as f:
        f.write("# synthetic profile\n")
        for k in range(len(q)):
            if err is None:
                f.write(f"{q[k]:.6f} {iq[k]:.9g}\n")
            else:
                f.write(f"{q[k]:.6f} {iq[k]:.9g} {err[k]:.9g}\n")


def _read_output(path):
    lines = open(path).read().splitlines()
    head = lines[0]
    vals = np.array([[float(x) for x in ln.split()] for ln in lines[1:]])
    params = {}
    for part in head.lstrip("# ").split(","):
        k, v = part.split(":")
        params[k.strip()] = float(v)
    return params, vals[:, 0], vals[:, 1]


def _oracle_curve(oracle_lib, q, models, ef, ww, rsasa=None):
    from resaxs_gb300 import _lib
    L = _lib.lib()
    q = np.ascontiguousarray(q, np.float32)
    rm = ctypes.c_float()
    _lib.check(L.rsx_ff_avg_radius(models[0].reshape(-1), len(models[0]), ctypes.byref(rm)))
    ff = np.zeros((len(q), 16), np.float32)
    _lib.check(L.rsx_ff_atomic_table(q, len(q), rm.value, ef, ff.reshape(-1)))
    tot = np.zeros(len(q))
    for m, b in enumerate(models):
        tot += oracle_lib.debye_f64(q, b, ff, rsasa=None if rsasa is None else rsasa[m],
                                    water_weight=ww, water_index=14)
    return tot / len(models)


def _oracle_rsasa(oracle_lib, models):
    """rsasa of each model as the CLI computes it: the reference GPU
    algorithm's dot map (create_dodeca_icosa_dots per atomic radius, probe
    1.8 A, 32 dots per type)."""
    from resaxs_gb300 import _lib
    from resaxs_gb300.sasa import reference_dot_map
    L = _lib.lib()
    radii16 = np.zeros(16, np.float32)
    _lib.check(L.rsx_ff_radii(radii16))
    ico = reference_dot_map(radii16, "dodeca_icosa", 1.8)
    out = []
    for b in models:
        cnt = oracle_lib.sasa_counts_typed(b, radii16, ico, 1.8)
        out.append((cnt.astype(np.float32) / np.float32(32)))
    return out


@pytest.mark.gpu
def test_cli_fixed_parameters_curve(cli, tmp_path, oracle_lib):
    pdb = os.path.join(GOLD, "synthetic_a.pdb")
    bodies, sizes = _read_pdb(pdb)
    models = np.split(bodies, np.cumsum(sizes)[:-1])
    q = np.linspace(0.0, 0.5, 101).astype(np.float32)
    ref = 2.5 * _oracle_curve(oracle_lib, q, models, 1.0, 0.0)
    prof = tmp_path / "p.dat"
    _write_profile(prof, q, ref * 1.01)
    r = _run(cli, ["-s", "2.5", "-w", "0", "-e", "1", "-f", str(prof), "-o", "out.dat", pdb],
             tmp_path)
    assert r.returncode == 0, r.stderr
    assert "bodies generated" in r.stdout
    params, qq, iq = _read_output(tmp_path / "out.dat")
    assert params["scale"] == 2.5 and params["water weight"] == 0
    assert params["expansion factor"] == 1
    np.testing.assert_allclose(qq, np.round(q.astype(np.float64), 6), atol=1e-6)
    # 1e-5 relative, plus the 6 decimals the output format keeps
    np.testing.assert_allclose(iq, ref, rtol=1e-5, atol=1e-6)


@pytest.mark.gpu
def test_cli_fixed_water_and_expansion(cli, tmp_path, oracle_lib):
    """Fixed water weight and expansion factor: the ensemble average (one
    batched pass over the models) with the oracle's rsasa on the reference
    dot map."""
    pdb = os.path.join(GOLD, "synthetic_a.pdb")
    bodies, sizes = _read_pdb(pdb)
    models = np.split(bodies, np.cumsum(sizes)[:-1])
    assert len(models) > 1
    q = np.linspace(0.0, 0.5, 101).astype(np.float32)
    rsasa = _oracle_rsasa(oracle_lib, models)
    ref = 1.5 * _oracle_curve(oracle_lib, q, models, 1.03, 1.2, rsasa)
    prof = tmp_path / "p.dat"
    _write_profile(prof, q, ref)
    r = _run(cli, ["-s", "1.5", "-w", "1.2", "-e", "1.03", "-f", str(prof), "-o", "out.dat",
                   pdb], tmp_path)
    assert r.returncode == 0, r.stderr
    params, qq, iq = _read_output(tmp_path / "out.dat")
    assert params["water weight"] == pytest.approx(1.2) and params["expansion factor"] == \
        pytest.approx(1.03)
    np.testing.assert_allclose(iq, ref, rtol=1e-5, atol=1e-6)


@pytest.mark.gpu
def test_cli_fit_recovers_parameters(cli, tmp_path, oracle_lib):
    pdb = os.path.join(GOLD, "synthetic_a.pdb")
    bodies, sizes = _read_pdb(pdb)
    models = np.split(bodies, np.cumsum(sizes)[:-1])
    q = np.linspace(0.005, 0.5, 100).astype(np.float32)
    rsasa = _oracle_rsasa(oracle_lib, models)
    true_scale, true_ww, true_ef = 3.0, 0.8, 1.02
    target = true_scale * _oracle_curve(oracle_lib, q, models, true_ef, true_ww, rsasa)
    prof = tmp_path / "p.dat"
    _write_profile(prof, q, target, err=0.01 * target)
    r = _run(cli, ["-v", "details", "-w", "[-2,4]", "-e", "[0.95,1.05]", "-f", str(prof),
                   "-o", "out.dat", pdb], tmp_path)
    assert r.returncode == 0, r.stderr
    params, qq, iq = _read_output(tmp_path / "out.dat")
    assert abs(params["expansion factor"] - true_ef) < 2e-3, params
    assert abs(params["water weight"] - true_ww) < 0.05, params
    assert abs(params["scale"] / true_scale - 1) < 1e-2, params
    assert params["Chi"] < 0.5, params
    np.testing.assert_allclose(iq, target, rtol=2e-2)


@pytest.mark.gpu
def test_cli_self_test_flag(cli, tmp_path, oracle_lib):
    pdb = os.path.join(GOLD, "synthetic_a.pdb")
    q = np.linspace(0.0, 0.5, 51).astype(np.float32)
    prof = tmp_path / "p.dat"
    _write_profile(prof, q, np.ones_like(q))
    r = _run(cli, ["-t", "-s", "1", "-o", "out.dat", "-f", str(prof), pdb], tmp_path)
    assert r.returncode == 0, r.stderr
    chisq = float(r.stdout.split("Chi square:")[1].split()[0])
    # the written curve is the average of 3 models; -t compares it with the
    # first model alone, as the reference's verify_result does
    assert np.isfinite(chisq) and chisq >= 0


def test_pdb_reader_survives_damaged_files(tmp_path):
    """Seeded damage to a PDB file (cut, overwritten, repeated, dropped lines,
    random bytes, stray MODEL/ENDMDL/END records): the reader returns a status
    and never crashes, and rsx_pdb_read fills exactly the bodies rsx_pdb_count
    announced.  Runs in a child process so that a crash fails only this test."""
    import subprocess
    import sys
    code = r'''
import ctypes, sys
import numpy as np
from resaxs_gb300 import _lib
L = _lib.lib()
src = open(sys.argv[1], "rb").read().split(b"\n")
rng = np.random.default_rng(11)
for it in range(150):
    lines = list(src)
    for _ in range(int(rng.integers(1, 40))):
        i = int(rng.integers(0, len(lines)))
        op, ln = int(rng.integers(0, 6)), lines[i]
        if op == 0 and ln:
            lines[i] = ln[: int(rng.integers(0, len(ln) + 1))]
        elif op == 1 and ln:
            j = int(rng.integers(0, len(ln)))
            lines[i] = ln[:j] + bytes([int(rng.integers(0, 256))]) + ln[j + 1:]
        elif op == 2:
            lines.insert(i, rng.integers(0, 256, int(rng.integers(0, 200))).astype(np.uint8).tobytes())
        elif op == 3:
            lines.insert(i, [b"MODEL     9", b"ENDMDL", b"END", b"TER", b"ATOM", b"HETATM"][int(rng.integers(0, 6))])
        elif op == 4:
            del lines[i]
        else:
            lines[i] = ln * int(rng.integers(2, 6))
    path = sys.argv[2] + "/f%d.pdb" % it
    open(path, "wb").write(b"\n".join(lines))
    nm, nb = ctypes.c_int(), ctypes.c_int()
    if L.rsx_pdb_count(path.encode(), ctypes.byref(nm), ctypes.byref(nb)) != 0:
        continue
    out = np.zeros((max(nb.value, 1), 4), np.float32)
    sizes = np.zeros(max(nm.value, 1), np.int32)
    st = L.rsx_pdb_read(path.encode(), 0, out.reshape(-1), nb.value, sizes, nm.value)
    assert st != 0 or sizes[: nm.value].sum() == nb.value, path
print("ok")
'''
    r = subprocess.run([sys.executable, "-c", code, os.path.join(GOLD, "synthetic_a.pdb"),
                        str(tmp_path)], capture_output=True, text=True,
                       cwd=ROOT, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr[-2000:]
