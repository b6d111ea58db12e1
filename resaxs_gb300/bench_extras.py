"""Secondary measurements of bench.py: one entry per benchmark configuration
besides the headline forward (incremental recalc + SASA, forward+adjoint,
the N = 20,000 forward, batching).  Every figure is a librsx timing on the
GPU.  Parity of these paths (drift of the running curve, SASA counts, per-q
error) is established by the GPU tests against the FP64 oracle
(tests/test_debye_gpu.py, tests/test_sasa_gpu.py, tests/test_recalc_gpu.py);
the drift figure below compares the running curve with a fresh GPU calculation."""
from __future__ import annotations

import statistics
import time

import numpy as np


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def recalc(device: int, steps: int = 1000, k: int = 50):
    """Config 2: N=20,000, Q=201; `steps` moves of k random bodies (Gaussian
    sigma 0.5 A) through rsx_debye_recalc_indices.  The API step time is the
    C entry point's, called through ctypes with the pointers of each step's
    arrays taken before the timed loop, on a handle without timing events;
    the Python wrapper's step (Debye.recalc_indices: array checks and
    marshalling) is timed separately.  A run of the same steps on a handle
    with events gives the kernel time and the GPU span of a call.  The FP64
    running curve is compared with a fresh full calculation at the end
    (drift)."""
    import ctypes

    from . import workloads as W
    from ._lib import check, lib
    from .saxs import Debye
    w = W.make_config(2, seed=0)
    rng = np.random.default_rng(42)
    bodies = w.bodies.copy()
    moves = []
    for _ in range(steps):
        idx = rng.choice(w.n, size=k, replace=False).astype(np.uint32)
        moved = bodies[idx].copy()
        moved[:, :3] += rng.normal(0, 0.5, (k, 3)).astype(np.float32)
        bodies[idx] = moved
        moves.append((idx, moved))
    raw = lib()["rsx_debye_recalc_indices"]  # a separate function object
    raw.restype = ctypes.c_int
    raw.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint,
                    ctypes.c_void_p]
    ptrs = [(m.ctypes.data, i.ctypes.data) for i, m in moves]
    out = np.zeros(len(w.q), np.float32)
    with Debye(w.q, w.ff, w.n, device=device) as d:
        d.calc(w.bodies)
        h, po, bad = d._h, out.ctypes.data, 0
        t0 = time.perf_counter()
        for pm, pi in ptrs:
            bad |= raw(h, pm, pi, k, po)
        wall = time.perf_counter() - t0
        check(bad)
        running = d.curve_f64()
    with Debye(w.q, w.ff, w.n, device=device) as d:
        d.calc(w.bodies)
        t0 = time.perf_counter()
        for idx, moved in moves:
            d.recalc_indices(moved, idx)
        wall_py = time.perf_counter() - t0
    kernel_ms, call_ms = [], []
    with Debye(w.q, w.ff, w.n, device=device, timing=True) as d:
        d.calc(w.bodies)
        full_ms = d.timing()[0]
        for idx, moved in moves:
            d.recalc_indices(moved, idx)
            kt, ct = d.timing()
            kernel_ms.append(kt)
            call_ms.append(ct)
    with Debye(w.q, w.ff, w.n, device=device) as d2:
        d2.calc(bodies)
        fresh = d2.curve_f64()
    terms = 2 * (k * (w.n - k) + k * (k - 1) // 2) * len(w.q)
    k_med = statistics.median(kernel_ms)
    return {"workload": "N=20000 Q=201, k=50 moved per step, sigma 0.5 A",
            "steps": steps, "step_ms_api": wall / steps * 1e3, "steps_per_s": steps / wall,
            "step_ms_python_wrapper": wall_py / steps * 1e3,
            "delta_kernel_ms": k_med, "gpu_call_ms": statistics.median(call_ms),
            "sinc_terms_per_step": terms,
            "delta_kernel_gterms_per_s": terms / (k_med * 1e-3) / 1e9,
            "full_forward_kernel_ms": full_ms,
            "speedup_vs_full_recompute_per_step": full_ms / (wall / steps * 1e3),
            "max_rel_drift_vs_fresh_full_calc": _rel(running, fresh)}


def sasa(device: int):
    """Config 2 SASA: 20,000 atoms, 960 Fibonacci dots, radii U[1.2,1.9], probe 1.4."""
    from . import workloads as W
    from .sasa import DotSphereSasa
    w = W.make_config(2, seed=0)
    radii = np.random.default_rng(0).uniform(1.2, 1.9, w.n).astype(np.float32)
    with DotSphereSasa(w.n, n_dots=960, probe=1.4, device=device) as s:
        s.counts(w.bodies, radii)
        times, kms = [], []
        for _ in range(5):
            t0 = time.perf_counter()
            c = s.counts(w.bodies, radii)
            times.append(time.perf_counter() - t0)
            tests, ms = s.stats()
            kms.append(ms)
    k_ms = statistics.median(kms)
    return {"workload": "N=20000 atoms, 960 dots, probe 1.4", "call_ms_api": statistics.median(times) * 1e3,
            "kernel_ms": k_ms, "occlusion_tests": int(tests),
            "gtests_per_s": tests / (k_ms * 1e-3) / 1e9, "dots_per_s": w.n * 960 / (k_ms * 1e-3),
            "exposed_dots": int(c.sum()),
            "parity": "bit-exact counts vs the strict-FP32 oracle, and vs the reference's own "
                      "CPU SASA on its dot sets (tests/test_sasa_gpu.py)"}


def adjoint(device: int):
    """Config 3: N=50,000, Q=256 on [0,0.6]; chi^2 against a copy displaced by
    sigma 1.0 A with sigma_q = 0.01 I_t: forward vs forward+adjoint time."""
    from . import workloads as W
    from .saxs import Debye
    w = W.make_config(3, seed=0)
    rng = np.random.default_rng(3)
    tb = w.bodies.copy()
    tb[:, :3] += rng.normal(0, 1.0, (w.n, 3)).astype(np.float32)
    with Debye(w.q, w.ff, w.n, device=device, timing=True) as d:
        target = d.calc(tb)
        sigma = (0.01 * target).astype(np.float32)
        d.calc(w.bodies)
        fwd, adj, tot = [], [], []
        for _ in range(3):
            t0 = time.perf_counter()
            d.calc(w.bodies)
            fwd.append(d.timing()[0])
            _, g = d.chi2_backward(target, sigma)
            adj.append(d.timing()[0])
            tot.append(time.perf_counter() - t0)
    f = statistics.median(fwd)
    a = statistics.median(adj)
    pq = w.pair_q
    return {"workload": "N=50000 Q=256", "forward_kernel_ms": f, "adjoint_kernel_ms": a,
            "fwd_plus_adjoint_over_fwd": (f + a) / f,
            "forward_gpairq_per_s": pq / (f * 1e-3) / 1e9,
            "adjoint_gpairq_per_s": pq / (a * 1e-3) / 1e9,
            "adjoint_method": "pair functions A(r), B(r) tabulated per type pair (FP64 sums over q) "
                              "and read by cubic Hermite interpolation: the per-pair cost does "
                              "not grow with Q, so adjoint pair*q/s is an effective rate; the "
                              "time includes the table build",
            "api_fwd_plus_adjoint_ms": statistics.median(tot) * 1e3,
            "grad_finite": bool(np.all(np.isfinite(g)))}


def forward_n20000(device: int, reps: int = 10):
    """Config 2's full forward (N = 20,000 compact chain, 5 types, 201 q on
    [0, 0.5]): pair kernels timed with CUDA events, median of ``reps``."""
    from . import workloads as W
    from .saxs import Debye
    w = W.make_config(2, seed=0)
    with Debye(w.q, w.ff, w.n, device=device, timing=True) as d:
        d.calc(w.bodies)
        for _ in range(3):
            d.forward_resident()
            d.sync()
        ms = []
        for _ in range(reps):
            d.forward_resident()
            d.sync()
            ms.append(d.timing()[0])
        t0 = time.perf_counter()
        for _ in range(reps):
            d.calc(w.bodies)
        api_ms = (time.perf_counter() - t0) / reps * 1e3
        cfg = d.config()
    k_ms = statistics.median(ms)
    return {"workload": W.CONFIG_NAMES[2], "pair_q": w.pair_q, "forward_kernel_ms": k_ms,
            "gpairq_per_s": w.pair_q / (k_ms * 1e-3) / 1e9, "api_ms": api_ms,
            "api_gpairq_per_s": w.pair_q / (api_ms * 1e-3) / 1e9, "config": cfg}


def _batching(device: int, n_members: int, n_lo: int, n_hi: int, seed: int = 0, reps: int = 3):
    """Both arms with the same statistic: the median of ``reps`` timed passes
    (batched) and, for every member, the median of ``reps`` timed forwards
    summed over the members (per conformation).  The batched pass picks its
    tile shape with the autotuner on the first pass."""
    from . import workloads as W
    from .batch import DebyeBatch
    from .saxs import Debye
    q, ff, members = W.batch_members(n_members=n_members, seed=seed, n_lo=n_lo, n_hi=n_hi)
    sizes = [len(m) for m in members]
    pair_q = sum(n * (n - 1) // 2 for n in sizes) * len(q)
    with DebyeBatch(q, ff, sizes, device=device, autotune=True) as b:
        out = b.forward(members)          # tunes, captures the graph
        b.forward(members)
        fwd, fwd_api = [], []
        for _ in range(reps):
            t0 = time.perf_counter()
            b.forward(members)
            fwd_api.append((time.perf_counter() - t0) * 1e3)
            fwd.append(b.timing())
        t = out * np.float32(1.01)
        b.set_targets(t, (0.01 * t + 1e-3).astype(np.float32))
        b.forward_chi2_backward(members)
        both = []
        for _ in range(reps):
            b.forward_chi2_backward(members)
            both.append(b.timing())
        cfg = b.config()
    # per-conformation launches: one handle per member; kernels (events around
    # the member's forward and assembly) and the API call a user makes per
    # member (host bodies in, curve out)
    per = 0.0
    api = 0.0
    for m in members:
        with Debye(q, ff, len(m), device=device, timing=True) as d:
            d.calc(m)
            ks, ws = [], []
            for _ in range(reps):
                t0 = time.perf_counter()
                d.calc(m)
                ws.append(time.perf_counter() - t0)
                d.forward_resident()
                d.sync()
                ks.append(d.timing()[1])
            per += statistics.median(ks)
            api += statistics.median(ws)
    f = statistics.median(fwd)
    fa = statistics.median(fwd_api)
    return {"workload": f"{n_members} members N~U[{n_lo},{n_hi}] Q={len(q)}", "pair_q": pair_q,
            "statistic": f"median of {reps} (batched passes; per member, summed)",
            "batched_forward_ms": f, "batched_gpairq_per_s": pair_q / (f * 1e-3) / 1e9,
            "batched_forward_api_ms": fa,
            "batched_fwd_plus_adjoint_ms": statistics.median(both),
            "per_conformation_forward_ms_sum": per,
            "per_conformation_api_ms_sum": api * 1e3,
            "speedup_vs_per_conformation_kernels": per / f,
            "speedup_vs_per_conformation_api": api * 1e3 / fa, "config": cfg}


def batching(device: int):
    """Config 5: 256 members, N ~ U[1000, 30000], Q=201: one graph-captured
    persistent pass (forward, and forward + per-member chi^2 adjoint) against
    per-conformation launches of the single-structure forward.  The same
    comparison on 256 small members (N ~ U[300, 3000]), where one structure
    cannot fill the GPU, is reported beside it."""
    out = _batching(device, 256, 1000, 30000)
    out["small_members"] = _batching(device, 256, 300, 3000, seed=1)
    return out


def run_all(device: int):
    out = {}
    for name, fn in (("forward_n20000_q201", forward_n20000), ("recalc", recalc),
                     ("sasa", sasa), ("adjoint", adjoint), ("batching", batching)):
        t0 = time.perf_counter()
        try:
            out[name] = fn(device)
        except Exception as e:  # report the failure in the line, do not hide it
            out[name] = {"error": repr(e)}
        out[name]["wall_s"] = time.perf_counter() - t0
    return out
