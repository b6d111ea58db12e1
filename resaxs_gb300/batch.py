"""Batched ensembles through librsx: ``DebyeBatch`` owns an ``rsx_batch``
handle (members share q and the factor table; each pass is one CUDA graph of
persistent pair kernels)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import DebyeOptions, ResaxsError, check, lib

__all__ = ["DebyeBatch"]


class DebyeBatch:
    def __init__(self, q, factors, member_sizes, *, device: int = -1, q_slab: int = 0,
                 autotune: bool = False, force_general_q: bool = False, pair_tables: bool = True,
                 pairs_per_step: int = 0):
        self.q = np.ascontiguousarray(q, np.float32)
        factors = np.ascontiguousarray(factors, np.float32)
        self.sizes = np.ascontiguousarray(member_sizes, np.int32)
        self.n_members = len(self.sizes)
        self.n_q = len(self.q)
        self.n_total = int(self.sizes.sum())
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        opts = DebyeOptions()
        lib().rsx_debye_default_options(ctypes.byref(opts))
        opts.device = device
        opts.q_slab = q_slab
        opts.autotune = int(autotune)
        opts.force_general_q = int(force_general_q)
        opts.no_pair_tables = int(not pair_tables)
        opts.pairs_per_step = int(pairs_per_step)
        h = ctypes.c_void_p()
        check(lib().rsx_batch_create(self.q, self.n_q, factors.reshape(-1), factors.shape[1],
                                     self.sizes, self.n_members, ctypes.byref(opts),
                                     ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().rsx_batch_destroy(self._h)
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

    def _pack(self, members):
        if isinstance(members, np.ndarray):
            b = np.ascontiguousarray(members, np.float32).reshape(-1)
        else:
            b = np.ascontiguousarray(np.concatenate(members, axis=0), np.float32).reshape(-1)
        # the C calls read every member's bodies, 4 floats each
        if b.size < 4 * self.n_total:
            raise ResaxsError(_lib.RSX_INVALID_ARG,
                              f"need {self.n_total} bodies over all members, got {b.size // 4}")
        return b

    def forward(self, members) -> np.ndarray:
        b = self._pack(members)
        out = np.zeros((self.n_members, self.n_q), np.float32)
        check(lib().rsx_batch_forward(self._h, b.reshape(-1), out.reshape(-1)))
        return out

    def set_factors(self, factors):
        f = np.ascontiguousarray(factors, np.float32)
        # the C call reads n_q rows of n_factors values
        if f.ndim != 2 or f.shape[0] != self.n_q:
            raise ResaxsError(_lib.RSX_INVALID_ARG, "factor table must be [n_q][n_factors]")
        check(lib().rsx_batch_set_factors(self._h, f.reshape(-1), f.shape[1]))

    def set_water(self, weight: float, water_index: int, rsasa=None):
        """Implicit water for every member; rsasa: one value per body, members
        concatenated (None keeps the values already set)."""
        ptr = None
        if rsasa is not None:
            if not isinstance(rsasa, np.ndarray):
                rsasa = np.concatenate([np.asarray(r, np.float32).reshape(-1) for r in rsasa])
            keep = np.ascontiguousarray(rsasa, np.float32).reshape(-1)
            # the C call reads one value per body
            if keep.size != self.n_total:
                raise ResaxsError(_lib.RSX_INVALID_ARG, "rsasa needs one value per body")
            self._rsasa_keep = keep
            ptr = keep.ctypes.data
        check(lib().rsx_batch_set_water(self._h, float(weight), int(water_index), ptr))

    def set_targets(self, targets, sigma):
        t = np.ascontiguousarray(targets, np.float32).reshape(-1)
        s = np.ascontiguousarray(sigma, np.float32).reshape(-1)
        # the C call reads n_members x n_q values from each
        if t.size < self.n_members * self.n_q or s.size < self.n_members * self.n_q:
            raise ResaxsError(_lib.RSX_INVALID_ARG, "targets and sigma must be n_members x n_q")
        check(lib().rsx_batch_set_targets(self._h, t, s))

    def forward_chi2_backward(self, members):
        b = self._pack(members)
        out = np.zeros((self.n_members, self.n_q), np.float32)
        chi2 = np.zeros(self.n_members, np.float64)
        grad = np.zeros((self.n_total, 3), np.float32)
        check(lib().rsx_batch_forward_chi2_backward(self._h, b.reshape(-1), out.ctypes.data,
                                                    chi2.ctypes.data, grad.ctypes.data))
        return out, chi2, grad

    def timing(self) -> float:
        ms = ctypes.c_float()
        check(lib().rsx_batch_timing(self._h, ctypes.byref(ms)))
        return ms.value

    def config(self):
        v = [ctypes.c_int() for _ in range(4)]
        check(lib().rsx_batch_config(self._h, *[ctypes.byref(x) for x in v]))
        return {"q_slab": v[0].value, "n_items": v[1].value, "persistent_ctas": v[2].value,
                "uniform_q": bool(v[3].value)}
