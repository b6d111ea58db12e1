"""Benchmark of the Debye hot path on GB300 (one JSON line on rank 0).

Workload (the largest configuration that fits one GPU): the full Debye forward
I(q) of N = 200,000 bodies, a random-walk chain folded into a 60 A sphere,
8 types (Z in {1,6,7,8,15,16,26,30}, f_t(q) = Z_t exp(-b_t q^2)), 512 q on
[0, 1.0] 1/A.  One step = one full forward of that structure: N(N-1)/2 x 512
= 1.024e13 pair*q terms f_i f_j sinc(q r_ij).

* ``value``   : pair*q/s with the bodies resident in HBM (kernels only), timed
                with CUDA events on librsx's stream; L2 is flushed (a 256 MB
                write) between timed steps, outside the events.
* ``e2e``     : the same metric through the C ABI call a user makes
                (rsx_debye_calc: host bodies in, host curve out, copies inside).
* ``roofline``: the pair kernel's pair*q/s against the FP32 issue bound of
                the recurrence: 3 FP32 lane-ops per pair*q (one FMA and one
                add advance sin(q r), one add accumulates it), at the FP32 FMA
                rate measured on this GPU (rsx_measure_fp32_fma_rate).  The
                bound of a direct evaluation (one SFU sine per pair*q, 16 per
                clock per SM = FMA rate / 8) is reported beside it.
* ``cpu_baseline``: the reference's host_debye<double,float> loop (the port in
                oracle/, bit-identical to the compiled original on x86) on the
                host cores over a bounded sample of the same workload: every
                sample is a set of rows of the lower triangle (all x < y for
                each sampled row y) over all 512 q.  The reference cannot run
                this structure whole: its N x N double matrix would take
                320 GB and is indexed with int (N <= 46,340).
* ``extras``  : the other configurations' figures (the N = 20,000 forward,
                incremental steps, SASA, forward+adjoint, batching).

With --gpus N under torchrun every rank computes its own independently seeded
structure (weak scaling, no collective); value = all ranks' pair*q / max time.
``--impl reference`` times the reference CPU path on the same workload
instead: every step is one row sample as above, every step timed; it also
runs one whole, un-extrapolated forward of the N = 20,000, 201-q structure.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "Debye Gpair\u00b7q/s & % FP32/SFU peak; fwd+adjoint vs plain fwd time at 1e-5 rel err"
UNIT = "Gpair\u00b7q/s"
HEADLINE = 4          # N = 200,000, 512 q
REF_ROWS = 32         # rows of the lower triangle per reference sample


def headline_config(w):
    """The ``config`` object both arms print (identical keys and values)."""
    from resaxs_gb300 import workloads as W
    return {"workload": W.CONFIG_NAMES[HEADLINE], "n_bodies": w.n, "n_q": len(w.q),
            "n_types": int(w.ff.shape[1]), "q_range": [float(w.q[0]), float(w.q[-1])],
            "structure": "random-walk chain folded into a 60 A sphere",
            "pair_q_per_step": w.pair_q,
            "l2": "GPU arm: flushed between timed steps by a 256 MB write outside the "
                  "events (the inputs, 3.2 MB, are L2-resident); CPU arm: not applicable"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--no-extras", action="store_true")
    p.add_argument("--cpu-threads", type=int, default=0)
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def ref_rows(n: int, n_rows: int, sample: int) -> np.ndarray:
    """Rows of the lower triangle timed in reference sample ``sample``: spread
    evenly over [1, n), shifted per sample so that the samples visit
    different rows.  Row y holds the y pairs (x, y), x < y."""
    base = np.linspace(1, n - 1, n_rows)
    shift = (sample * 7919) % max(1, (n - 1) // n_rows)
    return np.clip(np.round(base + shift), 1, n - 1).astype(np.int32)


def cpu_sample(w, threads: int, sample: int, n_rows: int = REF_ROWS):
    """One timed sample of the reference host_debye<double,float> loop (port
    in oracle/) on ``w``: the distance rows and the q loop of ``n_rows`` rows
    over every q, the q loop split over ``threads``.  Returns (pair*q, s)."""
    from oracle import oracle
    rows = ref_rows(w.n, n_rows, sample)
    t0 = time.perf_counter()
    oracle.refport_host_debye_rows(w.q, w.bodies, w.ff, rows, threads=threads)
    dt = time.perf_counter() - t0
    return int(rows.astype(np.int64).sum()) * len(w.q), dt


def cpu_baseline_forward(w, threads: int, samples: int = 4):
    """The reference CPU path on a bounded sample of the headline workload
    (``samples`` row samples; about 10 s on 16 cores)."""
    threads = threads or os.cpu_count() or 1
    pq = t = 0.0
    for s in range(samples):
        a, b = cpu_sample(w, threads, 1000 + s)
        pq += a
        t += b
    v = pq / t / 1e9
    return {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"host_debye<double,float> port over {samples} samples of {REF_ROWS} rows "
                      f"of the lower triangle (all x < y of each row, all {len(w.q)} q): "
                      f"{pq:.3e} pair*q in {t:.2f} s on {threads} threads",
            "seconds": t, "pair_q_timed": pq,
            "extrapolated_full_forward_s": w.pair_q / (v * 1e9)}


def cpu_full_forward_n20000(threads: int):
    """One whole, un-extrapolated host_debye<double,float> port forward of the
    N = 20,000, 201-q structure (its N x N matrix is 3.2 GB), q loop split
    over ``threads``."""
    from oracle import oracle
    from resaxs_gb300 import workloads as W
    w = W.make_config(2, seed=0)
    t0 = time.perf_counter()
    _, t_matrix = oracle.refport_host_debye(w.q, w.bodies, w.ff, threads=threads)
    dt = time.perf_counter() - t0
    return {"workload": W.CONFIG_NAMES[2], "n_bodies": w.n, "n_q": len(w.q),
            "pair_q": w.pair_q, "seconds": dt, "matrix_s": t_matrix,
            "value": w.pair_q / dt / 1e9, "unit": UNIT, "cores": threads,
            "what": "whole forward, every q, no extrapolation"}


def cpu_baseline_sasa(threads: int):
    """The SASA of config 2 (20,000 atoms, 960 Fibonacci dots, radii
    U[1.2, 1.9] A, probe 1.4 A) by the reference's CPU algorithm
    (rsasa_cpu_alg::calc_rsasa with its 6 A voxel grid; the port in oracle/,
    bit-identical to the compiled reference on x86), atoms split over the
    host threads.  The reference's neighbour prune assumes radii <= 1.5 A, so
    its counts may miss occluders of larger atoms: the dots where it differs
    from the exact counts are reported."""
    from oracle import oracle
    from resaxs_gb300 import workloads as W
    w = W.make_config(2, seed=0)
    radii = np.random.default_rng(0).uniform(1.2, 1.9, w.n).astype(np.float32)
    dots = oracle.fibonacci_unit_dots(960)
    t0 = time.perf_counter()
    counts = oracle.refport_rsasa_unit(w.bodies, radii, dots, 1.4, threads=threads)
    dt = time.perf_counter() - t0
    exact = oracle.sasa_counts(w.bodies, radii, dots, 1.4, threads=threads)
    return {"value": w.n * 960 / dt, "unit": "dots/s", "cores": threads, "kind": "port",
            "seconds": dt, "exposed_dots": int(counts.sum()),
            "atoms_differing_from_exact": int(np.sum(counts != exact)),
            "sample": "full config-2 SASA (20,000 atoms x 960 dots) by the port of the "
                      "reference's rsasa_cpu_alg (voxel grid, max_radius prune)"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from resaxs_gb300 import workloads as W
    w = W.make_config(HEADLINE, seed=0)
    threads = args.cpu_threads or os.cpu_count() or 1
    pq = t = 0.0
    for s in range(args.warmup + args.steps):
        a, b = cpu_sample(w, threads, s)
        if s >= args.warmup:
            pq += a
            t += b
    v = pq / t / 1e9
    cb = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
          "sample": f"every step: host_debye<double,float> port over {REF_ROWS} rows of the "
                    f"lower triangle (all x < y of each row, all {len(w.q)} q), {threads} "
                    f"threads; {pq:.3e} pair*q timed in {t:.2f} s over {args.steps} steps"}
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t / max(args.steps, 1) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": headline_config(w),
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "pair_q_per_timed_step": pq / max(args.steps, 1),
            "extrapolated": {"full_forward_s": w.pair_q / (v * 1e9),
                             "how": "the headline structure's N(N-1)/2 x 512 pair*q at the "
                                    "timed rate; not run (320 GB matrix, int-indexed)"}}
    if not args.no_extras:
        line["full_forward_n20000_q201"] = cpu_full_forward_n20000(threads)
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from resaxs_gb300 import _lib
    from resaxs_gb300 import workloads as W
    from resaxs_gb300.saxs import Debye

    w = W.make_config(HEADLINE, seed=rank)
    d = Debye(w.q, w.ff, w.n, device=local, timing=True)
    d.calc(w.bodies)                      # upload + first result
    stream = torch.cuda.ExternalStream(_lib.lib().rsx_debye_stream(d.handle),
                                       device=torch.device("cuda", local))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        d.forward_resident()
        d.sync()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    kernel_ms = []
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    launches0 = _lib.launch_count()
    t_wall0 = time.perf_counter()
    for s in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(s))
            ev[s][0].record(stream)
        d.forward_resident()
        with torch.cuda.stream(stream):
            ev[s][1].record(stream)
        d.sync()
        kernel_ms.append(d.timing()[0])
    barrier()
    t_wall = time.perf_counter() - t_wall0
    launches = _lib.launch_count() - launches0
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([total_ms], device=f"cuda:{local}", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * w.pair_q * args.steps / (total_ms * 1e-3) / 1e9

    # end to end through the C ABI with host buffers
    e2e_steps = max(3, args.steps // 2)
    d.calc(w.bodies)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        d.calc(w.bodies)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    if world > 1:
        t = torch.tensor([e2e_s], device=f"cuda:{local}", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": world * w.pair_q / e2e_s / 1e9, "unit": UNIT,
           "h2d_bytes_per_step": int(w.n * 16 + w.ff.nbytes),
           "d2h_bytes_per_step": int(len(w.q) * 4)}

    if rank == 0:
        import ctypes
        fma = ctypes.c_double()
        _lib.check(_lib.lib().rsx_measure_fp32_fma_rate(local, ctypes.byref(fma)))
        peak = fma.value / 3.0 / 1e9   # 3 FP32 lane-ops per pair*q
        sfu_peak = fma.value / 8.0 / 1e9  # one SFU sine per pair*q: 16 per clock per SM
        k_ms = statistics.median(kernel_ms)
        achieved = w.pair_q / (k_ms * 1e-3) / 1e9
        prof = os.path.join(ROOT, "profiles", "debye_forward_traffic_n200000_q512.json")
        traffic = None
        if os.path.exists(prof):
            traffic = json.load(open(prof)).get("dram_bytes_per_launch")
        cfg = d.config()
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": headline_config(w),
            "run": {"q_slab": cfg["q_slab"], "work_items": cfg["n_items"],
                    "uniform_q_recurrence": cfg["uniform_q"], "wall_s_timed_loop": t_wall,
                    "kernel_launches_per_step": launches / max(args.steps, 1)},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak,
                         "unit": UNIT, "frac": achieved / peak, "traffic": traffic,
                         "kernel_ms": k_ms,
                         "peak_source": "FP32 FMA rate measured on this GPU in this run / "
                                        "3 FP32 lane-ops per pair*q of the recurrence",
                         "fp32_fma_per_s": fma.value,
                         "sfu_direct_peak": sfu_peak,
                         "frac_of_sfu_direct_peak": achieved / sfu_peak},
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clk,
        }
        threads = args.cpu_threads or os.cpu_count() or 1
        try:
            line["cpu_baseline"] = cpu_baseline_forward(w, threads)
            if not args.no_extras:
                line["cpu_baseline"]["sasa"] = cpu_baseline_sasa(threads)
        except Exception as e:  # report, do not hide
            line["cpu_baseline"] = {"value": None, "error": repr(e)}
        if not args.no_extras:
            try:
                from resaxs_gb300 import bench_extras
                line["extras"] = bench_extras.run_all(local)
            except ImportError:
                pass
        print(json.dumps(line), flush=True)
    d.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
