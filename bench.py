"""Benchmark: particle force evaluations per second on one GB300.

Workload (the periodic gravity box): 128^3 = 2,097,152 equal-mass particles
on a unit-box lattice displaced by a Gaussian random field with P(k) ~ k^-2
(rms displacement 0.2 of the spacing), Ewald on, theta = 0.7, quadrupole
cells, eps = 1/(50*128), nBucket = 8.  One step = one full gravity force
evaluation (tree build, moments, walk + interactions, Ewald) of every
particle.  The headline path is FP32 on bucket-relative offsets; the plain
FP64 path is timed on the same input for the speed-up, and the FP32 path's
error is measured against it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With --impl reference the CPU oracle (this project's C restatement of the
reference's algorithm, the reference itself being unbuildable on the GPU
host) is timed on the host cores on the same workload.
Prints one JSON line (rank 0).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("particle force evals/s, 1 GB300: FP32+learned-h vs plain FP64 at "
          "99%ile err<1e-3")
UNIT = "particles/s"


def workload(ng=128, seed=2):
    from gasoline_gb300 import ics
    pos, vel, m = ics.lattice_box(ng, seed=seed, index=-2.0, rms_frac=0.2)
    soft = np.full(len(m), 1.0 / (50.0 * ng))
    return pos, m, soft


def config(ng, steps_flush="l2-flush"):
    return {"workload": f"periodic gravity box {ng}^3 lattice+GRF P(k)~k^-2, Ewald, "
                        f"theta=0.7, eps=1/(50*{ng}), nBucket=8",
            "n_particles": ng ** 3, "theta": 0.7, "iOrder": 2, "iEwOrder": 4,
            "nBucket": 8, "precision": "fp32 bucket-relative, fp64 positions",
            "l2": steps_flush, "parallelism": "replicas"}


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        time.sleep(0.25)
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except Exception:
            self.p.kill()
            out = ""
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def fma_peak_tflops(lib_ctx):
    """Measured FP32 FMA peak of this GPU (project microbenchmark)."""
    import ctypes
    t = ctypes.c_double()
    rc = lib_ctx.lib.tsph_fma_peak(lib_ctx._ctx, 1, ctypes.byref(t))
    return t.value if rc == 0 else None


def run_ours(args, rank, world, local_rank):
    import torch
    import gasoline_gb300 as g
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    ctx = g.Context(local_rank, stream=stream.cuda_stream)
    pos, m, soft = workload(args.ng)
    n = len(m)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # pinned host buffers for the end-to-end leg
    hpos = torch.from_numpy(np.ascontiguousarray(pos.reshape(-1))).pin_memory()
    hm = torch.from_numpy(np.ascontiguousarray(m)).pin_memory()
    hs = torch.from_numpy(np.ascontiguousarray(soft)).pin_memory()
    hacc = torch.empty(3 * n, dtype=torch.float64).pin_memory()

    ctx.set_particles(pos, m, soft)
    gp32 = g.grav_params(periodic=True, precision=g.FP32)
    gp64 = g.grav_params(periodic=True, precision=g.FP64)

    def timed(gp, steps, warmup, e2e=False):
        for _ in range(warmup):
            if e2e:
                ctx.set_particles_ptr(n, hpos.data_ptr(), hm.data_ptr(), hs.data_ptr())
            ctx.grav_all(gp)
            if e2e:
                ctx.get_gravity_ptr(hacc.data_ptr())
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        times, walk = [], []
        launches0 = ctx.launches()
        out = None
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            if e2e:
                ctx.set_particles_ptr(n, hpos.data_ptr(), hm.data_ptr(), hs.data_ptr())
            out = ctx.grav_all(gp)
            if e2e:
                ctx.get_gravity_ptr(hacc.data_ptr())
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            walk.append(ctx.timings())
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        launches = ctx.launches() - launches0
        return times, walk, out, launches

    clocks = Clocks(local_rank)
    # FP32 (headline), device-resident
    clocks.start()
    t32, w32, out32, launches32 = timed(gp32, args.steps, args.warmup)
    clk = clocks.stop()
    # FP32 end to end through the public API with host buffers
    te2e, _, _, _ = timed(gp32, args.steps, max(1, args.warmup // 2), e2e=True)
    # plain FP64 path on the same input
    k64 = max(1, args.steps // 2)
    t64, w64, out64, _ = timed(gp64, k64, max(1, args.warmup // 3))

    def agg(ts):
        ts = torch.tensor([sum(ts) / len(ts)], device=dev, dtype=torch.float64)
        if world > 1:
            torch.distributed.all_reduce(ts, op=torch.distributed.ReduceOp.MAX)
        return float(ts.item())

    ms32 = agg(t32)
    ms64 = agg(t64)
    mse2e = agg(te2e)
    result = None
    if rank == 0:
        # precision: FP32 vs FP64 accelerations on this input
        ctx.set_particles(pos, m, soft)
        ctx.grav_all(gp64)
        a64 = ctx.get_gravity()["acc"]
        ctx.grav_all(gp32)
        a32 = ctx.get_gravity()["acc"]
        rel = np.linalg.norm(a32 - a64, axis=1) / np.maximum(np.linalg.norm(a64, axis=1), 1e-300)
        walk_ms = statistics.mean(w["walk"] for w in w32)
        ew_ms = statistics.mean(w["ewald"] for w in w32)
        fgrav = out32["dFlop"] - out32["dFlopEwald"]
        peak = fma_peak_tflops(ctx)
        achieved = fgrav / (walk_ms * 1e-3) / 1e12
        value = world * n / (ms32 * 1e-3)
        result = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms32,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded lattice + Gaussian random field)",
            "config": config(args.ng),
            "clocks": clk,
            "e2e": {"value": world * n / (mse2e * 1e-3), "unit": UNIT,
                    "h2d_bytes_per_step": int(n * 5 * 8), "d2h_bytes_per_step": int(n * 3 * 8),
                    "ms_per_step": mse2e},
            "gpu_launches": int(launches32 // max(1, args.steps)) * args.steps,
            "roofline": {"bound": "fp32", "kernel": "k_walk<float> (fused walk + P-P/P-C)",
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": (achieved / peak) if peak else None, "traffic": None,
                         "flop_convention": "reference grav.c:246-247 (+,* = 1, 38 per P-P, "
                                            "76 per quadrupole cell)",
                         "walk_ms": walk_ms, "ewald_ms": ew_ms,
                         "phase_ms": {k: statistics.mean(w[k] for w in w32)
                                      for k in ("build", "moments", "walk", "ewald", "total")}},
            "fp64": {"value": world * n / (ms64 * 1e-3), "ms_per_step": ms64,
                     "walk_ms": statistics.mean(w["walk"] for w in w64)},
            "speedup_fp32_vs_fp64": ms64 / ms32,
            "precision_vs_fp64": {"rms": float(np.sqrt(np.mean(rel ** 2))),
                                  "p99": float(np.percentile(rel, 99)),
                                  "max": float(rel.max())},
            "interactions": {"dPartSum": out32["dPartSum"], "dCellSum": out32["dCellSum"],
                             "dSoftSum": out32["dSoftSum"], "exact_fallback_frac": out32["dExactFrac"]},
        }
        if not args.no_cpu:
            result["cpu_baseline"] = cpu_baseline(args, pos, m, soft)
    ctx.close()
    return result


def cpu_baseline(args, pos, m, soft):
    """The oracle (C restatement of the reference's algorithm) on the host
    cores, full workload, one evaluation."""
    import oracle
    nth = os.cpu_count() or 1
    gp = oracle.grav_params(periodic=True, ewald=True)
    o = oracle.oracle()
    t = time.perf_counter()
    o.grav(pos, m, soft, gp, nthreads=nth)
    dt = time.perf_counter() - t
    return {"value": len(m) / dt, "unit": UNIT, "cores": nth, "kind": "port",
            "sample": f"one full evaluation of the {round(len(m) ** (1/3))}^3 box "
                      f"({dt:.1f} s, OpenMP over buckets, serial tree build)"}


def run_reference(args):
    import oracle
    oracle.oracle()
    pos, m, soft = workload(args.ng)
    n = len(m)
    nth = os.cpu_count() or 1
    gp = oracle.grav_params(periodic=True, ewald=True)
    o = oracle.oracle()
    # bounded sample: a 64^3 box of the same construction per step
    ng_s = args.ref_ng
    ps, ms_, ss = workload(ng_s)
    for _ in range(min(1, args.warmup)):
        o.grav(ps, ms_, ss, gp, nthreads=nth)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        o.grav(ps, ms_, ss, gp, nthreads=nth)
        times.append(time.perf_counter() - t)
    sec = statistics.mean(times)
    value = len(ms_) / sec
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sec * 1e3 * n / len(ms_), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config(args.ng), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nth, "kind": "port",
                         "sample": f"{ng_s}^3 box of the same construction per step "
                                   f"(full {args.ng}^3 time scaled by particle count)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ng", type=int, default=128)
    ap.add_argument("--ref-ng", type=int, default=64)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    res = run_ours(args, rank, world, local_rank)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
