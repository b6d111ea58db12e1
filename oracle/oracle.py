"""ctypes loader for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module.  The product library (``resaxs_gb300``) never does.

``liboracle.so`` is the C restatement in this folder (debye_oracle.c,
sasa_oracle.c); ``_ref/libref_host_debye.so`` holds the reference's own CPU
code (host_debye, the PDB reader, the dot generators and the CPU SASA),
compiled by ``build_ref.sh`` from the reference tree where it exists.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_host_debye.so")

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def build(cc: str = "gcc") -> str:
    """Compile liboracle.so from the C restatement (seconds)."""
    objs = []
    for src, extra in (("debye_oracle.c", ["-O3", "-fno-math-errno"]),
                       ("sasa_oracle.c", ["-ffp-contract=off"]),
                       ("rsasa_cpu_port.c", ["-ffp-contract=off"])):
        obj = os.path.join(HERE, src.replace(".c", ".o"))
        subprocess.check_call([cc, "-O2", "-fPIC", "-std=c11", "-D_GNU_SOURCE", *extra,
                               "-c", os.path.join(HERE, src), "-o", obj])
        objs.append(obj)
    subprocess.check_call([cc, "-shared", *objs, "-o", LIB_PATH, "-lm", "-lpthread"])
    for o in objs:
        os.remove(o)
    return LIB_PATH


def build_ref(reference_root: str) -> str | None:
    """Compile the reference's CPU sources into _ref/ when ``reference_root``
    holds the reference tree (None otherwise)."""
    if not reference_root or not os.path.isfile(
            os.path.join(reference_root, "resaxslib", "src", "host_debye.cpp")):
        return None
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), reference_root])
    return REF_PATH


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        i, d, vp = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
        L.orc_debye_f64.argtypes = [_f64p, i, _f32p, i, _f32p, i, vp, d, i, _f64p, i]
        L.orc_debye_f64_libm.argtypes = [_f64p, i, _f32p, i, _f32p, i, vp, d, i, _f64p, i]
        L.orc_sin_probe.argtypes = [d]
        L.orc_sin_probe.restype = d
        L.orc_debye_f64_uniform.argtypes = [d, d, i, _f32p, i, _f32p, i, _f64p, i]
        L.orc_debye_grad_f64.argtypes = [_f64p, i, _f64p, _f32p, i, _f32p, i, vp, d, i, _f64p, i]
        L.orc_debye_grad_rows_f64.argtypes = [_f64p, i, _f64p, _f32p, i, _f32p, i, _i32p, i,
                                              _f64p, i]
        L.orc_debye_fd_f64.argtypes = [_f64p, i, _f64p, _f32p, i, _f32p, i, _i32p, _i32p,
                                       _f32p, _f32p, i, _f64p, i]
        L.orc_refport_host_debye.argtypes = [_f32p, i, _f32p, i, _f32p, i, _f32p]
        L.orc_refport_host_debye_mt.argtypes = [_f32p, i, _f32p, i, _f32p, i, _f32p, i]
        L.orc_refport_host_debye_mt.restype = d
        L.orc_refport_host_debye_rows.argtypes = [_f32p, i, _f32p, i, _f32p, i, _i32p, i,
                                                  _f64p, i]
        L.orc_refport_host_debye_rows.restype = i
        L.orc_sasa_counts.argtypes = [_f32p, _f32p, i, _f32p, i, ctypes.c_float, _u32p, i, i]
        L.orc_fibonacci_unit_dots.argtypes = [i, _f32p]
        f = ctypes.c_float
        L.orc_sasa_counts_typed.argtypes = [_f32p, i, _f32p, i, _f32p, i, f, _u32p, i]
        L.orc_sasa_counts_typed.restype = i
        L.orc_refport_rsasa_typed.argtypes = [_f32p, i, _f32p, i, _f32p, _i32p, f, _f32p, i]
        L.orc_refport_rsasa_typed.restype = i
        L.orc_refport_rsasa_unit.argtypes = [_f32p, i, _f32p, _f32p, i, f, _u32p, i]
        L.orc_refport_rsasa_unit.restype = i
        _lib = L
    return _lib


def ref_lib():
    """The compiled reference host_debye, or None when it was not built."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        L = ctypes.CDLL(REF_PATH)
        i = ctypes.c_int
        L.ref_host_debye_df.argtypes = [_f32p, i, _f32p, i, _f32p, i, _f32p]
        L.ref_host_debye_ff.argtypes = [_f32p, i, _f32p, i, _f32p, i, _f32p]
        L.ref_host_debye_dd.argtypes = [_f64p, i, _f64p, i, _f64p, i, _f64p]
        if hasattr(L, "ref_sasa_dots"):
            f = ctypes.c_float
            L.ref_sasa_dots.argtypes = [i, f, f, f, _f32p, i]
            L.ref_sasa_dots.restype = i
            L.ref_rsasa_cpu.argtypes = [_f32p, i, f, f, _f32p]
            L.ref_rsasa_cpu.restype = i
        _ref = L
    return _ref


SASA_DOT_KINDS = {"latitude": 0, "32": 1, "fibonacci": 2, "dodecahedron": 3, "dodeca_icosa": 4}


def ref_sasa_dots(kind: str, radius: float, dot_density: float, probe: float) -> np.ndarray:
    """The reference's dot sphere of one type ((n, 4) float32: x, y, z and the
    radius in w), from the compiled dot_spheres_params generators."""
    L = ref_lib()
    if L is None or not hasattr(L, "ref_sasa_dots"):
        raise RuntimeError("the compiled reference (oracle/_ref) is not available")
    out = np.zeros((8192, 4), np.float32)
    n = L.ref_sasa_dots(SASA_DOT_KINDS[kind], float(radius), float(dot_density), float(probe),
                        out, len(out))
    if n < 0:
        raise ValueError(f"ref_sasa_dots failed ({n})")
    return out[:n].copy()


def ref_rsasa_cpu(atoms, dot_density: float, probe: float) -> np.ndarray:
    """The reference's CPU SASA (rsasa_cpu_alg<float,float>::calc_rsasa):
    rsasa per atom of float4 bodies with type bits in .w."""
    L = ref_lib()
    if L is None or not hasattr(L, "ref_rsasa_cpu"):
        raise RuntimeError("the compiled reference (oracle/_ref) is not available")
    atoms = _c(atoms, np.float32)
    out = np.zeros(len(atoms), np.float32)
    rc = L.ref_rsasa_cpu(atoms.reshape(-1), len(atoms), float(dot_density), float(probe), out)
    if rc != 0:
        raise ValueError(f"ref_rsasa_cpu failed ({rc})")
    return out


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def debye_f64(q, bodies, ff, rsasa=None, water_weight=0.0, water_index=0, threads=0):
    """FP64 I(q) of float4 bodies (N,4 float32 with uint type bits in column 3)."""
    q = _c(q, np.float64)
    bodies = _c(bodies, np.float32)
    ff = _c(ff, np.float32)
    n_q, n_f = ff.shape
    out = np.zeros(len(q), np.float64)
    rs = None
    if rsasa is not None:
        rs_arr = _c(rsasa, np.float32)
        rs = rs_arr.ctypes.data
    lib().orc_debye_f64(q, len(q), bodies.reshape(-1), len(bodies), ff.reshape(-1), n_f,
                        rs, float(water_weight), int(water_index), out, int(threads))
    return out


def debye_f64_libm(q, bodies, ff, threads=0):
    q = _c(q, np.float64)
    bodies = _c(bodies, np.float32)
    ff = _c(ff, np.float32)
    out = np.zeros(len(q), np.float64)
    lib().orc_debye_f64_libm(q, len(q), bodies.reshape(-1), len(bodies), ff.reshape(-1),
                             ff.shape[1], None, 0.0, 0, out, int(threads))
    return out


def debye_f64_uniform(q0, dq, n_q, bodies, ff, threads=0):
    bodies = _c(bodies, np.float32)
    ff = _c(ff, np.float32)
    out = np.zeros(n_q, np.float64)
    lib().orc_debye_f64_uniform(float(q0), float(dq), int(n_q), bodies.reshape(-1), len(bodies),
                                ff.reshape(-1), ff.shape[1], out, int(threads))
    return out


def debye_grad_f64(q, w_q, bodies, ff, rsasa=None, water_weight=0.0, water_index=0, threads=0):
    q = _c(q, np.float64)
    w_q = _c(w_q, np.float64)
    bodies = _c(bodies, np.float32)
    ff = _c(ff, np.float32)
    grad = np.zeros((len(bodies), 3), np.float64)
    rs = None
    if rsasa is not None:
        rs_arr = _c(rsasa, np.float32)
        rs = rs_arr.ctypes.data
    lib().orc_debye_grad_f64(q, len(q), w_q, bodies.reshape(-1), len(bodies), ff.reshape(-1),
                             ff.shape[1], rs, float(water_weight), int(water_index),
                             grad.reshape(-1), int(threads))
    return grad


def debye_grad_rows_f64(q, w_q, bodies, ff, rows, threads=0):
    """FP64 gradient rows of L = sum_q w_q I(q) for the bodies ``rows``."""
    q = _c(q, np.float64)
    w_q = _c(w_q, np.float64)
    bodies = _c(bodies, np.float32)
    ff = _c(ff, np.float32)
    rows = _c(rows, np.int32)
    grad = np.zeros((len(rows), 3), np.float64)
    lib().orc_debye_grad_rows_f64(q, len(q), w_q, bodies.reshape(-1), len(bodies), ff.reshape(-1),
                                  ff.shape[1], rows, len(rows), grad.reshape(-1), int(threads))
    return grad


def debye_fd_f64(q, w_q, bodies, ff, coords, h=1e-4, threads=0):
    """FP64 central differences of L = sum_q w_q I(q) along the (body, axis)
    pairs ``coords``, with the FP32-represented steps x +/- h as divisor."""
    q = _c(q, np.float64)
    w_q = _c(w_q, np.float64)
    bodies = _c(bodies, np.float32)
    ff = _c(ff, np.float32)
    atom = _c([c[0] for c in coords], np.int32)
    axis = _c([c[1] for c in coords], np.int32)
    x = bodies[atom, axis].astype(np.float64)
    plus = _c(x + h, np.float32)
    minus = _c(x - h, np.float32)
    out = np.zeros(len(coords), np.float64)
    lib().orc_debye_fd_f64(q, len(q), w_q, bodies.reshape(-1), len(bodies), ff.reshape(-1),
                           ff.shape[1], atom, axis, plus, minus, len(coords), out, int(threads))
    return out


def refport_host_debye(q, bodies, ff, threads=1):
    """Port of host_debye<double,float,cl_float4>; returns (I(q) float32, t_matrix_s)."""
    q = _c(q, np.float32)
    bodies = _c(bodies, np.float32)
    ff = _c(ff, np.float32)
    out = np.zeros(len(q), np.float32)
    if threads == 1:
        lib().orc_refport_host_debye(q, len(q), bodies.reshape(-1), len(bodies), ff.reshape(-1),
                                     ff.shape[1], out)
        return out, None
    t = lib().orc_refport_host_debye_mt(q, len(q), bodies.reshape(-1), len(bodies),
                                        ff.reshape(-1), ff.shape[1], out, int(threads))
    return out, t


def refport_host_debye_rows(q, bodies, ff, rows, threads=0):
    """host_debye<double,float> port over the rows ``rows`` of the lower
    triangle only: returns the FP64 partial sum per q (see rsx_oracle.h)."""
    q = _c(q, np.float32)
    bodies = _c(bodies, np.float32)
    ff = _c(ff, np.float32)
    rows = _c(rows, np.int32)
    out = np.zeros(len(q), np.float64)
    rc = lib().orc_refport_host_debye_rows(q, len(q), bodies.reshape(-1), len(bodies),
                                           ff.reshape(-1), ff.shape[1], rows, len(rows), out,
                                           int(threads))
    if rc != 0:
        raise ValueError(f"orc_refport_host_debye_rows failed ({rc})")
    return out


def sasa_counts(atoms, radii, unit_dots, probe, use_cells=True, threads=0):
    atoms = _c(atoms, np.float32)
    radii = _c(radii, np.float32)
    unit_dots = _c(unit_dots, np.float32)
    counts = np.zeros(len(atoms), np.uint32)
    lib().orc_sasa_counts(atoms.reshape(-1), radii, len(atoms), unit_dots.reshape(-1),
                          len(unit_dots), ctypes.c_float(probe), counts, int(bool(use_cells)),
                          int(threads))
    return counts


def sasa_counts_typed(atoms, type_radii, dot_map, probe, threads=0):
    """Exact counts with pre-scaled per-type dots (dot_map: (n_types, stride,
    4) float32, non-finite x = padding); see rsx_oracle.h."""
    atoms = _c(atoms, np.float32)
    type_radii = _c(type_radii, np.float32)
    dot_map = _c(dot_map, np.float32)
    n_types, stride = dot_map.shape[0], dot_map.shape[1]
    counts = np.zeros(len(atoms), np.uint32)
    rc = lib().orc_sasa_counts_typed(atoms.reshape(-1), len(atoms), type_radii, n_types,
                                     dot_map.reshape(-1), stride, ctypes.c_float(probe), counts,
                                     int(threads))
    if rc != 0:
        raise ValueError(f"orc_sasa_counts_typed failed ({rc})")
    return counts


def refport_rsasa_typed(atoms, type_radii, dot_sets, probe, threads=0):
    """Port of the reference CPU SASA with per-type dot sets (a list of (n_t,
    4) arrays, one per type): rsasa per atom."""
    atoms = _c(atoms, np.float32)
    type_radii = _c(type_radii, np.float32)
    start = np.zeros(len(dot_sets) + 1, np.int32)
    start[1:] = np.cumsum([len(d) for d in dot_sets])
    dots = _c(np.concatenate([np.asarray(d, np.float32).reshape(-1, 4) for d in dot_sets]),
              np.float32)
    out = np.zeros(len(atoms), np.float32)
    rc = lib().orc_refport_rsasa_typed(atoms.reshape(-1), len(atoms), type_radii, len(dot_sets),
                                       dots.reshape(-1), start, ctypes.c_float(probe), out,
                                       int(threads))
    if rc != 0:
        raise ValueError(f"orc_refport_rsasa_typed failed ({rc})")
    return out


def refport_rsasa_unit(atoms, radii, unit_dots, probe, threads=0):
    """Port of the reference CPU SASA with per-atom radii and unit dots scaled
    by r_i + P: accessible-dot counts per atom."""
    atoms = _c(atoms, np.float32)
    radii = _c(radii, np.float32)
    unit_dots = _c(unit_dots, np.float32)
    counts = np.zeros(len(atoms), np.uint32)
    rc = lib().orc_refport_rsasa_unit(atoms.reshape(-1), len(atoms), radii,
                                      unit_dots.reshape(-1), len(unit_dots),
                                      ctypes.c_float(probe), counts, int(threads))
    if rc != 0:
        raise ValueError(f"orc_refport_rsasa_unit failed ({rc})")
    return counts


def fibonacci_unit_dots(n_dots):
    out = np.zeros((n_dots, 3), np.float32)
    lib().orc_fibonacci_unit_dots(int(n_dots), out)
    return out
