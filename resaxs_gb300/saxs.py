"""Python side of the Debye path: a thin owner of an ``rsx_debye`` handle
(``Debye``) and a mirror of resaxslib's algorithm interface
(``SaxsAlgorithm`` ~ ``resaxs::algorithm::i_saxs<float>``,
resaxslib/include/saxs_algorithm.hpp:118-183), raising ``ResaxsError`` with the
reference's error codes (resaxslib/include/resaxs.hpp:212-220).

Bodies are ``(N, 4) float32`` arrays in the reference layout (x, y, z, uint32
type bits in column 3).  All arithmetic runs in librsx on the GPU.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import DebyeOptions, ResaxsError, check, lib

__all__ = ["Debye", "SaxsAlgorithm", "SaxsParams", "calc_saxs_curve", "ResaxsError"]


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None and a.shape != shape:
        a = a.reshape(shape)
    return a


def calc_saxs_curve(q, bodies, factors) -> np.ndarray:
    """The C-style entry ``CalcSaxsCurveFn`` (resaxslib/include/host_debye.hpp:30)."""
    q = _f32(q)
    bodies = _f32(bodies)
    factors = _f32(factors)
    out = np.zeros(len(q), np.float32)
    check(lib().rsx_calc_saxs_curve_status(q, len(q), bodies.reshape(-1), len(bodies),
                                           factors.reshape(-1), factors.shape[-1], out))
    return out


class Debye:
    """Owner of one ``rsx_debye`` handle (one device, one stream)."""

    def __init__(self, q, factors, n_bodies: int, *, device: int = -1, q_slab: int = 0,
                 max_items: int = 0, force_general_q: bool = False, timing: bool = False,
                 autotune: bool = False, pair_tables: bool = True, pairs_per_step: int = 0):
        self.q = _f32(q)
        factors = _f32(factors)
        if factors.ndim != 2 or factors.shape[0] != len(self.q):
            raise ResaxsError(_lib.RSX_INVALID_ARG, "factor table must be [n_q][n_factors]")
        self.n_q = len(self.q)
        self.n_factors = factors.shape[1]
        self.n = int(n_bodies)
        opts = DebyeOptions()
        lib().rsx_debye_default_options(ctypes.byref(opts))
        opts.device = device
        opts.q_slab = q_slab
        opts.max_items = max_items
        opts.force_general_q = int(force_general_q)
        opts.timing = int(timing)
        opts.autotune = int(autotune)
        opts.no_pair_tables = int(not pair_tables)
        opts.pairs_per_step = int(pairs_per_step)
        h = ctypes.c_void_p()
        check(lib().rsx_debye_create(self.q, self.n_q, factors.reshape(-1), self.n_factors,
                                     self.n, ctypes.byref(opts), ctypes.byref(h)))
        self._h = h

    # lifetime ------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().rsx_debye_destroy(self._h)
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

    @property
    def handle(self):
        return self._h

    # parameters ----------------------------------------------------------
    def set_factors(self, factors):
        factors = _f32(factors)
        # the C call reads n_q rows of n_factors values
        if factors.ndim != 2 or factors.shape[0] != self.n_q:
            raise ResaxsError(_lib.RSX_INVALID_ARG, "factor table must be [n_q][n_factors]")
        check(lib().rsx_debye_set_factors(self._h, factors.reshape(-1), factors.shape[-1]))

    def set_water(self, weight: float, water_index: int, rsasa=None):
        ptr = None
        if rsasa is not None:
            keep = _f32(rsasa).reshape(-1)
            # the C call reads one value per body
            if keep.size != self.n:
                raise ResaxsError(_lib.RSX_INVALID_ARG, "rsasa needs one value per body")
            self._rsasa_keep = keep
            ptr = self._rsasa_keep.ctypes.data
        check(lib().rsx_debye_set_water(self._h, float(weight), int(water_index), ptr))

    # computation ---------------------------------------------------------
    def _need(self, a, count: int, what: str):
        # the C calls read `count` floats from the pointer they are given
        if a.size < count:
            raise ResaxsError(_lib.RSX_INVALID_ARG, f"{what}: need {count} values, got {a.size}")
        return a

    def calc(self, bodies) -> np.ndarray:
        bodies = self._need(_f32(bodies), 4 * self.n, "bodies")
        out = np.zeros(self.n_q, np.float32)
        check(lib().rsx_debye_calc(self._h, bodies.reshape(-1), out))
        return out

    def calc_shard(self, bodies, shard: int, n_shards: int) -> np.ndarray:
        """This shard's additive FP64 contribution to I(q) (rsx_debye_calc_shard);
        the sum over shards 0..n_shards-1 is the full curve."""
        bodies = self._need(_f32(bodies), 4 * self.n, "bodies")
        out = np.zeros(self.n_q, np.float64)
        check(lib().rsx_debye_calc_shard(self._h, bodies.reshape(-1), int(shard), int(n_shards),
                                         out))
        return out

    def recalc_range(self, bodies, start: int, length: int) -> np.ndarray:
        bodies = self._need(_f32(bodies), 4 * min(int(start) + int(length), self.n),
                            "bodies vector too small in recalc_range")
        out = np.zeros(self.n_q, np.float32)
        check(lib().rsx_debye_recalc_range(self._h, bodies.reshape(-1), int(start), int(length),
                                           out))
        return out

    def recalc_indices(self, moved, idx) -> np.ndarray:
        idx = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1)
        moved = self._need(_f32(moved), 4 * len(idx), "moved bodies")
        out = np.zeros(self.n_q, np.float32)
        check(lib().rsx_debye_recalc_indices(self._h, moved.reshape(-1), idx, len(idx), out))
        return out

    def commit(self):
        check(lib().rsx_debye_commit(self._h))

    def revert(self):
        check(lib().rsx_debye_revert(self._h))

    def curve_f64(self) -> np.ndarray:
        out = np.zeros(self.n_q, np.float64)
        check(lib().rsx_debye_curve_f64(self._h, out))
        return out

    def forward_resident(self):
        check(lib().rsx_debye_forward_resident(self._h))

    def sync(self):
        check(lib().rsx_debye_sync(self._h))

    def timing(self):
        k = ctypes.c_float()
        c = ctypes.c_float()
        check(lib().rsx_debye_timing(self._h, ctypes.byref(k), ctypes.byref(c)))
        return k.value, c.value

    def backward(self, dl_diq, f64: bool = False) -> np.ndarray:
        lam = self._need(_f32(dl_diq).reshape(-1), self.n_q, "dL/dI")
        if f64:
            g = np.zeros((self.n, 3), np.float64)
            check(lib().rsx_debye_backward_f64(self._h, lam, g.reshape(-1)))
        else:
            g = np.zeros((self.n, 3), np.float32)
            check(lib().rsx_debye_backward(self._h, lam, g.reshape(-1)))
        return g

    def chi2_backward(self, target, sigma, want_grad: bool = True):
        target = self._need(_f32(target).reshape(-1), self.n_q, "target curve")
        sigma = self._need(_f32(sigma).reshape(-1), self.n_q, "sigma")
        c2 = ctypes.c_double()
        g = np.zeros((self.n, 3), np.float32) if want_grad else None
        check(lib().rsx_debye_chi2_backward(self._h, target, sigma, ctypes.byref(c2),
                                            g.ctypes.data if want_grad else None))
        return c2.value, g

    def config(self):
        qs, ni, un, pp = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().rsx_debye_config(self._h, ctypes.byref(qs), ctypes.byref(ni), ctypes.byref(un)))
        check(lib().rsx_debye_tile_shape(self._h, None, ctypes.byref(pp)))
        return {"q_slab": qs.value, "n_items": ni.value, "uniform_q": bool(un.value),
                "pairs_per_step": pp.value}


# ---------------------------------------------------------------------------
# reference-interface mirror
# ---------------------------------------------------------------------------

class _Dirty:
    """params_base (resaxslib/include/re_algorithm.hpp:66-89)."""

    def __init__(self):
        self._dirty = False

    def is_dirty(self):
        return self._dirty

    def clear_dirty(self):
        self._dirty = False

    def set_dirty(self):
        self._dirty = True


class FormFactorParams(_Dirty):
    """form_factor_params (saxs_algorithm.hpp:79-109)."""

    def __init__(self):
        super().__init__()
        self.factors = None          # [n_q][n_factors] float32
        self.water_ff_index = -1
        self.expansion_factor = 1.0

    def access_factors(self):
        self.set_dirty()
        return self.factors

    def set_water_ff_index(self, index: int):
        if self.water_ff_index != index:
            self.water_ff_index = int(index)
            self.set_dirty()

    def set_factors(self, factors):
        self.factors = _f32(factors)
        self.set_dirty()


class ImplicitWaterParams(_Dirty):
    """implicit_water_params (saxs_algorithm.hpp:55-77)."""

    def __init__(self):
        super().__init__()
        self.water_weight = 0.0
        self.no_rsasa_recalc = False
        self.rsasa = None

    def set_water_weight(self, weight: float):
        if self.water_weight != weight:
            self.water_weight = float(weight)
            self.set_dirty()

    def access_rsasa(self):
        self.set_dirty()
        return self.rsasa


class SaxsParams(_Dirty):
    """saxs_params (saxs_algorithm.hpp:118-138)."""

    def __init__(self):
        super().__init__()
        self.qq = None
        self.n_bodies = 0
        self.device = -1
        self.workgroup_size = 64
        self._ff = FormFactorParams()
        self._water = ImplicitWaterParams()

    def initialize(self, qq, bodies, devices=None, workgroup_size: int = 64, factors=None):
        self.qq = _f32(qq)
        self.n_bodies = len(bodies)
        self.device = -1 if not devices else int(devices[0])
        self.workgroup_size = int(workgroup_size)
        if factors is not None:
            self._ff.set_factors(factors)
        self.set_dirty()

    def get_ff_params(self):
        return self._ff

    def get_implicit_water_params(self):
        return self._water


class SaxsAlgorithm:
    """Mirror of ``i_saxs<float>`` over librsx.  Use::

        alg = SaxsAlgorithm()
        p = alg.access_params()
        p.initialize(q, bodies, factors=table)
        p.get_implicit_water_params().set_water_weight(0)
        alg.initialize()
        out = []
        alg.calc_curve(bodies, out)
        alg.recalc_curve(bodies, start, length, out)
        alg.commit(); alg.revert()
    """

    def __init__(self, **debye_kwargs):
        self._params = SaxsParams()
        self._d = None
        self._sasa = None
        self._kw = debye_kwargs
        self._computing = False

    def access_params(self) -> SaxsParams:
        return self._params

    def initialize(self):
        p = self._params
        if p.qq is None:
            raise ResaxsError(_lib.RSX_ARGS_NOT_SET, "saxs_params.initialize() was not called")
        ff = p.get_ff_params().factors
        if ff is None:
            raise ResaxsError(_lib.RSX_ARGS_NOT_SET, "no form-factor table set")
        if self._d is not None:
            self._d.close()
        if self._sasa is not None:
            self._sasa.close()
            self._sasa = None
        self._d = Debye(p.qq, ff, p.n_bodies, device=p.device, **self._kw)
        p.get_ff_params().clear_dirty()
        self._computing = False

    def _push_params(self, water_always: bool = False):
        p = self._params
        ff = p.get_ff_params()
        w = p.get_implicit_water_params()
        if ff.is_dirty():
            self._d.set_factors(ff.factors)
            ff.clear_dirty()
        if w.is_dirty() or water_always:
            idx = ff.water_ff_index if ff.water_ff_index >= 0 else 0
            self._d.set_water(w.water_weight, idx, w.rsasa)
            w.clear_dirty()

    def _update_rsasa(self, bodies, moved: bool):
        """The water term's rsasa as the reference's GPU algorithm keeps it
        (saxs_alg_cl_gpu_pt_wf.cpp:82-96, 333-401): with a non-zero water weight
        every update of the bodies recomputes rsasa from all bodies with the
        reference's own OpenCL dot map (the create_dodeca_icosa_dots sphere of
        each of the 16 atomic radii, probe 1.8 A, rsasa_cl_gpu_alg.cpp:60-89),
        unless ``no_rsasa_recalc`` is set and rsasa values are present."""
        w = self._params.get_implicit_water_params()
        if w.water_weight == 0:
            return
        n = self._params.n_bodies
        present = w.rsasa is not None and len(w.rsasa) >= n
        if present and (w.no_rsasa_recalc or not moved):
            return
        from .sasa import TypedDotSphereSasa, reference_dot_map
        bodies = np.ascontiguousarray(bodies, np.float32).reshape(-1, 4)
        if len(bodies) < n:
            raise ResaxsError(_lib.RSX_INVALID_ARG, "the water term's SASA needs every body")
        types = bodies[:n].view(np.uint32)[:, 3]
        if types.size and types.max() >= 16:
            raise ResaxsError(_lib.RSX_INVALID_ARG,
                              "the water term's SASA needs an atomic type (0..15) on every body")
        if self._sasa is None:
            radii = np.zeros(16, np.float32)
            check(lib().rsx_ff_radii(radii))
            self._sasa = TypedDotSphereSasa(n, reference_dot_map(radii, "dodeca_icosa", 1.8),
                                            radii, 1.8, device=self._params.device)
        w.access_rsasa()
        w.rsasa = self._sasa.rsasa(bodies[:n])

    @staticmethod
    def _emit(out, values):
        if out is None:
            return values
        if isinstance(out, np.ndarray):
            out[: len(values)] = values
        else:
            out[:] = list(values)
        return out

    def calc_curve(self, bodies, out_iqq=None):
        if self._d is None:
            raise ResaxsError(_lib.RSX_ARGS_NOT_SET, "initialize() was not called")
        if len(bodies) != self._params.n_bodies:
            raise ResaxsError(_lib.RSX_INVALID_ARG,
                              "different number of bodies expected in calc_curve()")
        # a full calculation always takes the current water parameters, as the
        # reference's calc_curve sets the weight argument on every call
        # (saxs_alg_cl_gpu_pt_wf.cpp:433-438); this also carries them into a
        # handle made by a later initialize()
        self._update_rsasa(bodies, moved=True)
        self._push_params(water_always=True)
        res = self._d.calc(bodies)
        self._computing = True
        return self._emit(out_iqq, res)

    def recalc_curve(self, bodies, upd_start: int, upd_length: int, out_iqq=None):
        if self._d is None or not self._computing:
            raise ResaxsError(_lib.RSX_NO_INITIAL_CALC,
                              "recalc_curve() called before an initial call to calc_curve()")
        if len(bodies) < upd_start + upd_length:
            raise ResaxsError(_lib.RSX_INVALID_ARG, "bodies vector too small in recalc_curve()")
        self._update_rsasa(bodies, moved=upd_length > 0)
        self._push_params()
        res = self._d.recalc_range(bodies, upd_start, upd_length)
        return self._emit(out_iqq, res)

    def commit(self):
        if self._d is None or not self._computing:
            raise ResaxsError(_lib.RSX_NO_INITIAL_CALC,
                              "commit() called before an initial call to calc_curve()")
        self._d.commit()

    def revert(self):
        if self._d is None or not self._computing:
            raise ResaxsError(_lib.RSX_NO_INITIAL_CALC,
                              "revert() called before an initial call to calc_curve()")
        self._d.revert()

    @property
    def debye(self) -> Debye:
        return self._d
