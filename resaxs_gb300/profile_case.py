"""Runs one hot-path case on cuda:0 for profiling (ncu / timing by hand).

    python -m resaxs_gb300.profile_case forward --config 2 [--n N] [--reps R]
    python -m resaxs_gb300.profile_case recalc  --config 2 [--k 50] [--reps R]
    python -m resaxs_gb300.profile_case adjoint --config 3 [--n N]
    python -m resaxs_gb300.profile_case sasa    --config 2 [--dots 960]

`--general` forces the general (non-recurrence) q path; `--water W` turns
the implicit water term on with weight W, seeded rsasa in [0, 1] and the
last factor column as the water factor.

Uses the seeded synthetic workloads of resaxs_gb300.workloads; prints one
line with the wall time per repetition.  Exits non-zero on any librsx error.
"""
from __future__ import annotations

import argparse
import sys
import time

import numpy as np


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("path", choices=["forward", "recalc", "adjoint", "sasa", "batch"])
    p.add_argument("--config", type=int, default=2)
    p.add_argument("--n", type=int, default=None)
    p.add_argument("--reps", type=int, default=2)
    p.add_argument("--k", type=int, default=50)
    p.add_argument("--dots", type=int, default=960)
    p.add_argument("--q-slab", type=int, default=0)
    p.add_argument("--general", action="store_true")
    p.add_argument("--water", type=float, default=0.0)
    a = p.parse_args(argv)
    from . import workloads as W
    from .saxs import Debye

    if a.path == "sasa":
        from .sasa import DotSphereSasa
        w = W.make_config(a.config, seed=0, n_override=a.n)
        rng = np.random.default_rng(0)
        radii = rng.uniform(1.2, 1.9, w.n).astype(np.float32)
        with DotSphereSasa(w.n, n_dots=a.dots, probe=1.4) as s:
            t0 = time.perf_counter()
            for _ in range(a.reps):
                counts = s.counts(w.bodies, radii)
            dt = (time.perf_counter() - t0) / a.reps
        print(f"sasa N={w.n} dots={a.dots}: {dt * 1e3:.3f} ms/rep, exposed={int(counts.sum())}")
        return 0
    if a.path == "batch":
        from .batch import DebyeBatch
        q, ff, members = W.batch_members(n_members=a.k, scale=(a.n or 30000) / 30000)
        with DebyeBatch(q, ff, [len(m) for m in members]) as b:
            t0 = time.perf_counter()
            for _ in range(a.reps):
                b.forward(members)
            dt = (time.perf_counter() - t0) / a.reps
        print(f"batch members={len(members)}: {dt * 1e3:.3f} ms/rep")
        return 0

    w = W.make_config(a.config, seed=0, n_override=a.n)
    with Debye(w.q, w.ff, w.n, q_slab=a.q_slab, force_general_q=a.general) as d:
        if a.water != 0.0:
            rs = np.random.default_rng(2).uniform(0, 1, w.n).astype(np.float32)
            d.set_water(a.water, w.ff.shape[1] - 1, rs)
        d.calc(w.bodies)
        rng = np.random.default_rng(1)
        t0 = time.perf_counter()
        for _ in range(a.reps):
            if a.path == "forward":
                d.forward_resident()
                d.sync()
            elif a.path == "recalc":
                idx = rng.choice(w.n, size=a.k, replace=False).astype(np.uint32)
                moved = w.bodies[idx].copy()
                moved[:, :3] += rng.normal(0, 0.5, (a.k, 3)).astype(np.float32)
                d.recalc_indices(moved, idx)
            else:
                d.backward(rng.normal(size=len(w.q)).astype(np.float32))
        dt = (time.perf_counter() - t0) / a.reps
    print(f"{a.path} config={a.config} N={w.n} Q={len(w.q)}: {dt * 1e3:.3f} ms/rep")
    return 0


if __name__ == "__main__":
    sys.exit(main())
