"""Dot-sphere SASA through librsx: ``DotSphereSasa`` owns an ``rsx_sasa``
handle with one unit dot set and per-atom radii; ``TypedDotSphereSasa`` owns
one with the reference's per-type pre-scaled dot map and per-type radii
(resaxslib/src/rsasa_cl_gpu_alg.cpp:59-89); ``RsasaAlgorithm`` mirrors
resaxslib's ``i_rsasa`` interface (resaxslib/include/rsasa_algorithm.hpp:42-61)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import ResaxsError, check, lib

__all__ = ["DotSphereSasa", "TypedDotSphereSasa", "RsasaAlgorithm", "fibonacci_dots",
           "dodeca_icosa_dots", "dot_map_from_sets", "sphere_dots", "reference_dot_map"]


def fibonacci_dots(n_dots: int) -> np.ndarray:
    out = np.zeros((n_dots, 3), np.float32)
    check(lib().rsx_sasa_fibonacci_dots(int(n_dots), out.reshape(-1)))
    return out


DOT_KINDS = {"latitude": 0, "32": 1, "fibonacci": 2, "dodecahedron": 3, "dodeca_icosa": 4}


def sphere_dots(kind: str, radius: float, probe: float, dot_density: float = 0.0) -> np.ndarray:
    """The reference's dot sphere for one radius ((n, 4) float32: x, y, z on
    the sphere of radius + probe, w = radius): dot_spheres_params::create_*."""
    cap = 8192
    while True:
        out = np.zeros((cap, 4), np.float32)
        n = ctypes.c_int()
        st = lib().rsx_sasa_sphere_dots(DOT_KINDS[kind], ctypes.c_float(radius),
                                        ctypes.c_float(dot_density), ctypes.c_float(probe),
                                        out.reshape(-1), cap, ctypes.byref(n))
        if st == 0:
            return out[: n.value].copy()
        if n.value > cap:
            cap = n.value
            continue
        check(st)


def reference_dot_map(type_radii, kind: str, probe: float, dot_density: float = 0.0) -> np.ndarray:
    """Per-type pre-scaled dot map ((n_types, stride, 4), -inf padding) built
    the way the reference builds dots_map_ (rsasa_cl_gpu_alg.cpp:60-89) or
    its per-type sets (rsasa_cpu_alg.cpp:46-61)."""
    return dot_map_from_sets([sphere_dots(kind, float(r), probe, dot_density)
                              for r in np.asarray(type_radii, np.float32)])


def dodeca_icosa_dots() -> np.ndarray:
    out = np.zeros((32, 3), np.float32)
    check(lib().rsx_sasa_dodeca_icosa_dots(out.reshape(-1)))
    return out


class DotSphereSasa:
    """Accessible-dot counts of every atom for a fixed unit dot set and probe."""

    def __init__(self, n_atoms: int, n_dots: int = 960, probe: float = 1.4, unit_dots=None,
                 device: int = -1):
        if unit_dots is None:
            unit_dots = fibonacci_dots(n_dots)
        self.unit = np.ascontiguousarray(unit_dots, np.float32)
        if self.unit.ndim != 2 or self.unit.shape[1] != 3:
            raise ResaxsError(_lib.RSX_INVALID_ARG, "unit dots must be [n_dots][3]")
        self.n = int(n_atoms)
        self.n_dots = len(self.unit)
        self.probe = float(probe)
        h = ctypes.c_void_p()
        check(lib().rsx_sasa_create(self.n, self.unit.reshape(-1), self.n_dots,
                                    ctypes.c_float(self.probe), int(device), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().rsx_sasa_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _inputs(self, atoms, radii):
        # the C calls read n atoms of 4 floats and n radii
        atoms = np.ascontiguousarray(atoms, np.float32).reshape(-1)
        radii = np.ascontiguousarray(radii, np.float32).reshape(-1)
        if atoms.size < 4 * self.n or radii.size < self.n:
            raise ResaxsError(_lib.RSX_INVALID_ARG, f"need {self.n} atoms and {self.n} radii")
        return atoms, radii

    def counts(self, atoms, radii) -> np.ndarray:
        atoms, radii = self._inputs(atoms, radii)
        out = np.zeros(self.n, np.uint32)
        check(lib().rsx_sasa_counts(self._h, atoms, radii, out))
        return out

    def rsasa(self, atoms, radii) -> np.ndarray:
        atoms, radii = self._inputs(atoms, radii)
        out = np.zeros(self.n, np.float32)
        check(lib().rsx_sasa_calc(self._h, atoms, radii, out))
        return out

    def stats(self):
        t = ctypes.c_ulonglong()
        ms = ctypes.c_float()
        check(lib().rsx_sasa_stats(self._h, ctypes.byref(t), ctypes.byref(ms)))
        return int(t.value), float(ms.value)


def dot_map_from_sets(dot_sets) -> np.ndarray:
    """Per-type dot sets (a list of (n_t, 3 or 4) arrays) as one (n_types,
    stride, 4) map padded with -inf dots, the layout of the reference's
    dots_map_ (rsasa_cl_gpu_alg.cpp:72-86)."""
    sets = [np.asarray(d, np.float32).reshape(len(d), -1) for d in dot_sets]
    stride = max([len(d) for d in sets] + [1])
    m = np.full((len(sets), stride, 4), -np.inf, np.float32)
    for t, d in enumerate(sets):
        m[t, :len(d), :3] = d[:, :3]
        m[t, :len(d), 3] = 0.0
    return m


class TypedDotSphereSasa:
    """Accessible-dot counts with the reference's own dot layout: pre-scaled
    dots per atom type (``dot_map``: (n_types, stride, 4), a dot whose x is not
    finite is padding) and one radius per type; atoms carry their type in
    column 3."""

    def __init__(self, n_atoms: int, dot_map, type_radii, probe: float, device: int = -1):
        self.map = np.ascontiguousarray(dot_map, np.float32)
        if self.map.ndim != 3 or self.map.shape[2] != 4:
            raise ResaxsError(_lib.RSX_INVALID_ARG, "dot map must be [n_types][stride][4]")
        self.type_radii = np.ascontiguousarray(type_radii, np.float32).reshape(-1)
        if len(self.type_radii) < self.map.shape[0]:
            raise ResaxsError(_lib.RSX_INVALID_ARG, "need one radius per type")
        self.n = int(n_atoms)
        self.probe = float(probe)
        h = ctypes.c_void_p()
        check(lib().rsx_sasa_create_typed(self.n, self.map.reshape(-1), self.map.shape[0],
                                          self.map.shape[1], self.type_radii,
                                          ctypes.c_float(self.probe), int(device),
                                          ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().rsx_sasa_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _atoms(self, atoms):
        atoms = np.ascontiguousarray(atoms, np.float32).reshape(-1)
        if atoms.size < 4 * self.n:
            raise ResaxsError(_lib.RSX_INVALID_ARG, f"need {self.n} atoms")
        return atoms

    def counts(self, atoms) -> np.ndarray:
        out = np.zeros(self.n, np.uint32)
        check(lib().rsx_sasa_counts_typed(self._h, self._atoms(atoms), out))
        return out

    def rsasa(self, atoms) -> np.ndarray:
        out = np.zeros(self.n, np.float32)
        check(lib().rsx_sasa_calc_typed(self._h, self._atoms(atoms), out))
        return out

    def stats(self):
        t = ctypes.c_ulonglong()
        ms = ctypes.c_float()
        check(lib().rsx_sasa_stats(self._h, ctypes.byref(t), ctypes.byref(ms)))
        return int(t.value), float(ms.value)


class RsasaAlgorithm:
    """Mirror of ``i_rsasa<float>``: ``initialize(params)`` then
    ``calc_rsasa(atoms, rsasa)`` / ``recalc_rsasa(atoms, rsasa)``.

    ``initialize(n_atoms, dot_density=..., probe_radius=...)`` uses the
    reference's own per-type dot spheres for the 16 atomic radii
    (``dot_kind="dodeca_icosa"``: rsasa_cl_gpu's map, rsasa_cl_gpu_alg.cpp:60-89;
    ``"latitude"``: rsasa_cpu_alg's create_dots sets, rsasa_cpu_alg.cpp:46-61).
    With ``radius_of_type`` it uses one unit dot set (``unit_dots`` or
    ``n_dots`` Fibonacci dots) and a radius per body type instead."""

    def __init__(self):
        self._s = None
        self._typed = False
        self._computing = False

    def initialize(self, n_atoms: int, radius_of_type=None, probe_radius: float = 1.4,
                   unit_dots=None, n_dots: int = 960, device: int = -1,
                   dot_density: float = 0.0, dot_kind: str = "dodeca_icosa"):
        if self._s is not None:
            self._s.close()
        self._s = None
        self._computing = False
        if radius_of_type is None:
            radii = np.zeros(16, np.float32)
            check(lib().rsx_ff_radii(radii))
            self._s = TypedDotSphereSasa(n_atoms, reference_dot_map(radii, dot_kind, probe_radius,
                                                                    dot_density),
                                         radii, probe_radius, device=device)
            self._typed = True
        else:
            self.radius_of_type = np.asarray(radius_of_type, np.float32)
            self._s = DotSphereSasa(n_atoms, n_dots=n_dots, probe=probe_radius,
                                    unit_dots=unit_dots, device=device)
            self._typed = False

    def _radii(self, atoms):
        types = np.ascontiguousarray(atoms, np.float32).view(np.uint32)[:, 3]
        if types.size and types.max() >= len(self.radius_of_type):
            raise ResaxsError(_lib.RSX_INVALID_ARG, "atom type without a radius")
        return self.radius_of_type[types]

    def calc_rsasa(self, atoms, rsasa=None):
        if self._s is None:
            raise ResaxsError(_lib.RSX_ARGS_NOT_SET, "initialize() was not called")
        if rsasa is not None and len(rsasa) < len(atoms):
            raise ResaxsError(_lib.RSX_INVALID_ARG, "rsasa vector too small")
        if self._typed:
            res = self._s.rsasa(atoms)
        else:
            res = self._s.rsasa(atoms, self._radii(atoms))
        self._computing = True
        if rsasa is not None:
            rsasa[: len(res)] = res
            return rsasa
        return res

    def recalc_rsasa(self, atoms, rsasa=None):
        if not self._computing:
            raise ResaxsError(_lib.RSX_NO_INITIAL_CALC, "recalc_rsasa() before calc_rsasa()")
        return self.calc_rsasa(atoms, rsasa)
