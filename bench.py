"""Benchmark: particle force evaluations per second on one GB300.

Workload (the periodic gravity box): 128^3 = 2,097,152 equal-mass particles
on a unit-box lattice displaced by a Gaussian random field with P(k) ~ k^-2
(rms displacement 0.2 of the spacing), Ewald on, theta = 0.7, quadrupole
cells, eps = 1/(50*128), nBucket = 16.  One step = a drift of every particle
(0.02 of the spacing rms) and one full gravity force evaluation (tree build,
moments, walk + interactions, Ewald) of every particle.  The headline path is
FP32 on bucket-relative offsets; the plain FP64 path is timed on the same
input for the speed-up, and the FP32 path's error is measured against it.
Outside the timed region the GPU's FP64 and FP32 evaluations of the box are
compared with the CPU oracle's evaluation of the same input (the `parity`
object), the oracle run that also gives `cpu_baseline`.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With --impl reference the CPU oracle (this project's C restatement of the
reference's algorithm; the reference's own sources are not on the GPU host)
is timed on all host cores on the same 128^3 box, one evaluation per step.
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
# bucket size of the box workload: the autotuner's choice on GB300 (16 beats
# 8 by ~12%: fewer walks, each over a wider bucket); fixed so both arms and
# the CPU baseline build the same tree
NBUCKET = 16


def workload(ng=128, seed=2, with_vel=False):
    from gasoline_gb300 import ics
    pos, vel, m = ics.lattice_box(ng, seed=seed, index=-2.0, rms_frac=0.2)
    soft = np.full(len(m), 1.0 / (50.0 * ng))
    if with_vel:
        return pos, vel, m, soft
    return pos, m, soft


# Each timed step drifts the particles before the force evaluation, as a KDK
# step does, so every tree build partitions moved particles.  The box's
# velocities equal its displacement field (rms 0.2 of the spacing), so a
# drift of DRIFT_DT moves particles by 0.02 of the spacing rms per step.
# The drift alternates in sign (forward, back): drifting one way only would
# grow the displacement field step after step and turn the box into a
# different, more clustered configuration than the one named.
DRIFT_DT = 0.1


def drifted(pos, vel, dt, box=1.0):
    """pos + vel * dt wrapped into [-box/2, box/2) (the drift of the timed
    end-to-end steps, precomputed on the host)."""
    p = pos + vel * dt
    p = (p + 0.5 * box) % box - 0.5 * box
    p[p >= 0.5 * box] -= box
    return p


def config(ng, steps_flush="l2-flush", nbucket=8):
    return {"workload": f"periodic gravity box {ng}^3 lattice+GRF P(k)~k^-2, Ewald, "
                        f"theta=0.7, eps=1/(50*{ng}), nBucket={nbucket} (autotuned)",
            "n_particles": ng ** 3, "theta": 0.7, "iOrder": 2, "iEwOrder": 4,
            "nBucket": nbucket, "precision": "fp32 bucket-relative, fp64 positions",
            "step": "one full force evaluation of every particle after a move of 0.02 of the "
                    f"spacing rms (device leg: a kick-drift-kick step, dt +-{DRIFT_DT} in turn, "
                    "replayed from one CUDA graph; end-to-end leg and CPU arm: the two position "
                    "sets a drift apart, in turn)",
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


def max_over_ranks(x, world, device="cpu"):
    """The largest of one float over all ranks (every rank gets it): the
    job's time is its slowest replica's."""
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_value(n_per_rank, world, ms):
    """Whole-job throughput of independent replicas: every rank's
    particles over the slowest rank's time."""
    return world * n_per_rank / (ms * 1e-3)


def fma_peak_tflops(lib_ctx, fp32=True):
    """Measured FP32 (or FP64) FMA peak of this GPU (project microbenchmark)."""
    import ctypes
    t = ctypes.c_double()
    rc = lib_ctx.lib.tsph_fma_peak(lib_ctx._ctx, 1 if fp32 else 0, ctypes.byref(t))
    return t.value if rc == 0 else None


# Algorithmic flops per neighbour pair of the SPH passes in the reference's
# convention (+, -, *, /, sqrt count one each), counted from the oracle's
# statement-by-statement restatement: DenDVDX (smoothfcn.c:3390-3627,
# M4 KERNEL/DKERNEL) and one symmetric SphPressureTerms pair
# (SphPressureTerms.h, both particles updated).
FLOP_DENDVDX_PAIR = 64
FLOP_PRESSURE_PAIR = 68
GRAV_FLOPS = ("reference grav.c:246-247 (+,* = 1, 38 per P-P, 82 per softened cell, "
              "76 per quadrupole cell)")


def walk_roofline(ctx, out, walk_ms, nbt):
    """The gravity walk (k_walk<float, nbt>): the reference's flop count of
    the evaluation over the kernel's event-timed duration, against the FP32
    FMA peak measured on this GPU."""
    fl = out["dFlop"] - out["dFlopEwald"]
    peak = fma_peak_tflops(ctx)
    ach = fl / (walk_ms * 1e-3) / 1e12
    return {"bound": "fp32", "kernel": f"k_walk<float, {nbt}> (fused walk + P-P/P-C)",
            "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak if peak else None,
            "traffic": None, "flop_convention": GRAV_FLOPS, "kernel_ms": walk_ms,
            "peak_source": "tsph_fma_peak (FP32 FMA, measured on this GPU)"}


def density_roofline(ctx, dens, density_ms, fp32):
    """The kNN + DenDVDX pass (k_knn_density): DenDVDX's flops per gathered
    pair over the kernel's event-timed duration (the kNN selection itself
    is comparisons and integer work, not counted), against the measured FMA
    peak of its precision."""
    peak = fma_peak_tflops(ctx, fp32)
    ach = dens["dPairs"] * FLOP_DENDVDX_PAIR / (density_ms * 1e-3) / 1e12
    return {"bound": "fp32" if fp32 else "fp64",
            "kernel": f"k_knn_density<{'f32' if fp32 else 'f64'}> (kNN + DenDVDX)",
            "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak if peak else None,
            "traffic": None, "flop_convention": f"{FLOP_DENDVDX_PAIR} per gathered pair (DenDVDX)",
            "kernel_ms": density_ms, "pairs": dens["dPairs"], "candidates": dens["dCandidates"],
            "peak_source": f"tsph_fma_peak ({'FP32' if fp32 else 'FP64'} FMA, measured on this GPU)"}


def oracle_seconds(fn):
    t = time.perf_counter()
    r = fn()
    return time.perf_counter() - t, r


def run_ours(args, rank, world, local_rank):
    import torch
    import gasoline_gb300 as g
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    # a dedicated stream: the library runs on it and the events bracket it
    stream = torch.cuda.Stream(dev)
    ctx = g.Context(local_rank, stream=stream.cuda_stream)
    pos, vel, m, soft = workload(args.ng, with_vel=True)
    n = len(m)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # pinned host buffers for the end-to-end leg: two position sets a drift
    # apart, used alternately, so each step's tree is built from moved
    # particles
    hpos = [torch.from_numpy(np.ascontiguousarray(p.reshape(-1))).pin_memory()
            for p in (pos, drifted(pos, vel, DRIFT_DT))]
    hm = torch.from_numpy(np.ascontiguousarray(m)).pin_memory()
    hs = torch.from_numpy(np.ascontiguousarray(soft)).pin_memory()
    hacc = torch.empty(3 * n, dtype=torch.float64).pin_memory()

    # the first evaluation of a new particle set builds its tree from the
    # caller's order (later ones start from the last tree's order); the
    # context's first call (kernel loading, allocations) is made beforehand
    gp_first = g.grav_params(periodic=True, precision=g.FP32, nBucket=NBUCKET)
    ctx.set_particles(pos, m, soft)
    ctx.grav_all(gp_first)
    ctx.set_particles(pos, m, soft)
    ctx.set_velocities(vel)
    first_ms = _cuda_ms(lambda: ctx.grav_all(gp_first), stream)
    first_build_ms = ctx.timings()["build"]
    ctx.set_particles(pos, m, soft)
    ctx.set_velocities(vel)
    # launch shapes and bucket size by the project's autotuner (a few
    # seconds); the FP64 path runs on the same bucket size, i.e. the same tree
    from gasoline_gb300 import autotune
    tuned, _ = autotune.tune_gravity(ctx, g.grav_params(periodic=True, precision=g.FP32),
                                     nbuckets=(NBUCKET,), walk_blocks=(4, 5),
                                     task_sizes=(0, 3072))
    gp32 = g.grav_params(periodic=True, precision=g.FP32, nBucket=tuned["nBucket"])
    gp64 = g.grav_params(periodic=True, precision=g.FP64, nBucket=tuned["nBucket"])

    def timed(gp, steps, warmup, e2e=False):
        # one step: move the particles (a device drift, forward and back in
        # turn; end to end, the other host position set), then one full
        # force evaluation
        k = [0]

        def one():
            k[0] ^= 1
            if e2e:
                ctx.update_particles_ptr(n, hpos[k[0]].data_ptr(), hm.data_ptr(), hs.data_ptr())
            else:
                ctx.drift(DRIFT_DT if k[0] else -DRIFT_DT, True, 1.0)
            o = ctx.grav_all(gp)
            if e2e:
                ctx.get_gravity_ptr(hacc.data_ptr())
            return o

        ctx.set_particles(pos, m, soft)
        ctx.set_velocities(vel)
        for _ in range(warmup):
            one()
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        times, walk = [], []
        launches0 = ctx.launches()
        out = None
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = one()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            walk.append(ctx.timings())
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        launches = ctx.launches() - launches0
        return times, walk, out, launches

    def timed_graph(gp, steps, warmup):
        # one step: a whole kick-drift-kick step (tsph_step) replayed from
        # one captured CUDA graph -- kick dt/2, drift dt, tree build,
        # moments, walk, Ewald, kick dt/2 -- with dt alternating +DRIFT_DT,
        # -DRIFT_DT: the leapfrog is time-reversible, so the box stays the
        # configuration named while every step moves the particles by 0.02 of
        # the spacing rms and rebuilds the tree on them
        sgn = [-1.0]

        def one():
            sgn[0] = -sgn[0]
            ctx.step(sgn[0] * DRIFT_DT, gp, None, graph=True)

        ctx.set_particles(pos, m, soft)
        ctx.set_velocities(vel)
        ctx.grav_all(gp)              # the opening kick's forces
        for _ in range(max(warmup, 2)):
            one()
        ctx.step_status()
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        times = []
        launches0 = ctx.launches()
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            one()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        ctx.step_status()
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        return times, ctx.launches() - launches0

    clocks = Clocks(local_rank)
    # FP32 (headline), device-resident: whole KDK steps as one CUDA graph
    clocks.start()
    tg, launchesg = timed_graph(gp32, args.steps, args.warmup)
    clk = clocks.stop()
    # the same force evaluation issued directly after a drift: per-phase
    # timings (the roofline's walk time) and pkdGravAll's counters
    t32, w32, out32, launches32 = timed(gp32, args.steps, args.warmup)
    # FP32 end to end through the public API with host buffers
    te2e, _, _, _ = timed(gp32, args.steps, max(1, args.warmup // 2), e2e=True)
    # plain FP64 path on the same input
    k64 = max(1, args.steps // 2)
    t64, w64, out64, _ = timed(gp64, k64, max(1, args.warmup // 3))
    # the reference's default cell order (iOrder 4: octopole and
    # hexadecapole cells), FP32, the same evaluation issued directly
    gp32o4 = g.grav_params(periodic=True, precision=g.FP32, nBucket=tuned["nBucket"], iOrder=4)
    t4, w4, out4, _ = timed(gp32o4, max(2, args.steps // 4), 2)

    def agg(ts):
        return max_over_ranks(sum(ts) / len(ts), world, dev)

    msg = agg(tg)
    ms32 = agg(t32)
    ms64 = agg(t64)
    ms4 = agg(t4)
    mse2e = agg(te2e)
    result = None
    if rank == 0:
        # precision: FP32 vs FP64 accelerations on this input
        ctx.set_particles(pos, m, soft)
        o64 = ctx.grav_all(gp64)
        g64 = ctx.get_gravity()
        a64 = g64["acc"]
        o32 = ctx.grav_all(gp32)
        g32 = ctx.get_gravity()
        a32 = g32["acc"]
        rel = np.linalg.norm(a32 - a64, axis=1) / np.maximum(np.linalg.norm(a64, axis=1), 1e-300)
        # total force error against an FP64 tree at theta = 0.3
        ctx.grav_all(g.grav_params(periodic=True, precision=g.FP64, theta=0.3,
                                   nBucket=tuned["nBucket"]))
        a03 = ctx.get_gravity()["acc"]
        n03 = np.maximum(np.linalg.norm(a03, axis=1), 1e-300)
        e32 = np.linalg.norm(a32 - a03, axis=1) / n03
        e64 = np.linalg.norm(a64 - a03, axis=1) / n03
        walk_ms = statistics.mean(w["walk"] for w in w32)
        ew_ms = statistics.mean(w["ewald"] for w in w32)
        fgrav = out32["dFlop"] - out32["dFlopEwald"]
        peak = fma_peak_tflops(ctx)
        achieved = fgrav / (walk_ms * 1e-3) / 1e12
        value = replica_value(n, world, msg)
        result = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": msg,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded lattice + Gaussian random field)",
            "config": config(args.ng, nbucket=tuned["nBucket"]),
            "clocks": clk,
            "e2e": {"value": replica_value(n, world, mse2e), "unit": UNIT,
                    "h2d_bytes_per_step": int(n * 5 * 8), "d2h_bytes_per_step": int(n * 3 * 8),
                    "ms_per_step": mse2e},
            "gpu_launches": int(launchesg),
            "direct_step": {"value": replica_value(n, world, ms32), "ms_per_step": ms32,
                            "step": "a drift (dt +-0.1 in turn) and tsph_grav_all issued directly",
                            "gpu_launches": int(launches32)},
            "roofline": {"bound": "fp32", "kernel": f"k_walk<float, {NBUCKET}> (fused walk + P-P/P-C)",
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": (achieved / peak) if peak else None,
                         # dram__bytes_read.sum + dram__bytes_write.sum of this kernel,
                         # one launch, ncu capture in profiles/k_walk_f32_box128.md
                         "traffic": 1.70719488e8, "traffic_unit": "bytes per launch",
                         "flop_convention": "reference grav.c:246-247 (+,* = 1, 38 per P-P, "
                                            "76 per quadrupole cell)",
                         "walk_ms": walk_ms, "ewald_ms": ew_ms,
                         "phase_ms": {k: statistics.mean(w[k] for w in w32)
                                      for k in ("build", "moments", "walk", "ewald", "total")}},
            "fp64": {"value": world * n / (ms64 * 1e-3), "ms_per_step": ms64,
                     "walk_ms": statistics.mean(w["walk"] for w in w64)},
            "fp32_iOrder4": {"value": world * n / (ms4 * 1e-3), "ms_per_step": ms4,
                             "walk_ms": statistics.mean(w["walk"] for w in w4),
                             "walk_tflops": (out4["dFlop"] - out4["dFlopEwald"]) /
                                            (statistics.mean(w["walk"] for w in w4) * 1e-3) / 1e12,
                             "note": "the reference's default cell order (octopole and hexadecapole "
                                     "cells); the evaluation issued directly after a drift"},
            "speedup_fp32_vs_fp64": ms64 / ms32,
            "precision_vs_fp64": {"rms": float(np.sqrt(np.mean(rel ** 2))),
                                  "p99": float(np.percentile(rel, 99)),
                                  "max": float(rel.max())},
            # the theta = 0.7 tree's own error on this near-uniform box (the
            # net force is a small residual of cancelling terms): FP64 and
            # FP32 alike; a pairwise Ewald sum confirms theta = 0.3 as the
            # reference (tests/test_gravity_gpu.py)
            "error_vs_fp64_theta_0.3": {
                "fp32_theta_0.7": {"rms": float(np.sqrt(np.mean(e32 ** 2))),
                                   "p99": float(np.percentile(e32, 99))},
                "fp64_theta_0.7": {"rms": float(np.sqrt(np.mean(e64 ** 2))),
                                   "p99": float(np.percentile(e64, 99))}},
            "tuned": tuned,
            "first_evaluation": {"ms": first_ms, "build_ms": first_build_ms,
                                 "note": "tree built from the caller's particle order (a new "
                                         "particle set); timed steps start from the last tree's"},
            "interactions": {"dPartSum": out32["dPartSum"], "dCellSum": out32["dCellSum"],
                             "dSoftSum": out32["dSoftSum"], "exact_fallback_frac": out32["dExactFrac"],
                             "opening_tests": out32["dTests"], "walk_visits": out32["dVisits"]},
        }
        if not args.no_cpu:
            base, ref = cpu_baseline(args, pos, m, soft)
            result["cpu_baseline"] = base
            import oracle
            with oracle.exact_rsqrt():
                _, ref_exact = cpu_baseline(args, pos, m, soft)
            result["parity"] = parity(o64, g64, o32, g32, ref, ref_exact)
    ctx.close()
    return result


def cpu_baseline(args, pos, m, soft):
    """The oracle (C restatement of the reference's algorithm) on the host
    cores, full workload, one evaluation; its result is kept for the parity
    check of the same input."""
    import oracle
    nth = os.cpu_count() or 1
    gp = oracle.grav_params(periodic=True, ewald=True, nBucket=NBUCKET)
    o = oracle.oracle()
    t = time.perf_counter()
    ref = o.grav(pos, m, soft, gp, nthreads=nth)
    dt = time.perf_counter() - t
    return ({"value": len(m) / dt, "unit": UNIT, "cores": nth, "kind": "port",
             "sample": f"one full evaluation of the {round(len(m) ** (1/3))}^3 box "
                       f"({dt:.1f} s, OpenMP over buckets, serial tree build)"}, ref)


# Parity bars at the headline size.  The reference takes 1/r from v_sqrt1,
# accurate to 2e-10 per term; in the periodic box the replica and Ewald sums
# cancel to a net force far smaller than the terms, which amplifies that
# error with N (oracle with v_sqrt1 against the same oracle with an exact
# 1/sqrt: acceleration rms 7.9e-9 at 16^3, 3.0e-8 at 64^3, 6.3e-8 at
# 128^3).  The CUDA FP64 path takes a correctly rounded rsqrt, so it is
# held to the oracle with an exact 1/sqrt (same tree, same lists, same
# terms; only the order of the sums differs), and its distance from the
# reference's own arithmetic is reported beside it.  The periodic potential
# crosses zero and is measured against max |pot|.  FP32: p99 bar.
PARITY_FP64_RMS = 1e-10
PARITY_POT_SCALED = 1e-10
PARITY_FP32_P99 = 3e-4


def _acc_err(a, ref):
    return np.linalg.norm(a - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-300)


def parity(o64, g64, o32, g32, ref, ref_exact):
    """The GPU's evaluations of the box (FP64 and FP32, same input) against
    the oracle's, outside the timed region: `ref` with the reference's own
    arithmetic (v_sqrt1), `ref_exact` with an exact 1/sqrt."""
    c = ref["counters"]
    counters = {}
    ok = True
    for name, o in (("fp64", o64), ("fp32", o32)):
        exact = (o["nActive"] == int(c[0]) and o["dPartSum"] == c[1] and o["dCellSum"] == c[2]
                 and o["dSoftSum"] == c[3])
        frel = abs(o["dFlop"] - c[4]) / abs(c[4])
        counters[name] = {"nActive_PP_cells_soft_exact": bool(exact), "dFlop_rel_diff": frel}
        ok = ok and exact
    ok = ok and counters["fp64"]["dFlop_rel_diff"] <= 1e-12
    pmax = float(np.max(np.abs(ref_exact["pot"])))
    e64x = _acc_err(g64["acc"], ref_exact["acc"])
    p64x = np.abs(g64["pot"] - ref_exact["pot"]) / pmax
    e64r = _acc_err(g64["acc"], ref["acc"])
    p64r = np.abs(g64["pot"] - ref["pot"]) / pmax
    eref = _acc_err(ref["acc"], ref_exact["acc"])
    e32 = _acc_err(g32["acc"], ref_exact["acc"])
    rms = lambda x: float(np.sqrt(np.mean(np.square(x))))  # noqa: E731
    res = {"against": "the oracle (a bit-exact restatement of the reference) on the same input, "
                      "one full evaluation each",
           "counters": counters,
           "oracle_counters": {"nActive": int(c[0]), "dPartSum": c[1], "dCellSum": c[2],
                               "dSoftSum": c[3], "dFlop": c[4]},
           "fp64_vs_oracle_exact_rsqrt": {"acc_rms": rms(e64x), "acc_max": float(e64x.max()),
                                          "pot_rms_over_max_pot": rms(p64x),
                                          "pot_max_over_max_pot": float(p64x.max())},
           "fp64_vs_oracle_v_sqrt1": {"acc_rms": rms(e64r), "acc_max": float(e64r.max()),
                                      "pot_max_over_max_pot": float(p64r.max())},
           "oracle_v_sqrt1_vs_exact_rsqrt": {"acc_rms": rms(eref), "acc_max": float(eref.max())},
           "fp32_vs_oracle_exact_rsqrt": {"acc_rms": rms(e32), "acc_p99": float(np.percentile(e32, 99))},
           "bars": {"fp64_acc_rms": PARITY_FP64_RMS, "fp64_pot_rms": PARITY_POT_SCALED,
                    "fp32_acc_p99": PARITY_FP32_P99,
                    "counters": "exact (FP64 dFlop to 1e-12; FP32 dFlop reported: its Ewald "
                                "real-space cut is tested in FP32)"}}
    ok = (ok and rms(e64x) <= PARITY_FP64_RMS and rms(p64x) <= PARITY_POT_SCALED
          and float(np.percentile(e32, 99)) <= PARITY_FP32_P99)
    res["pass"] = bool(ok)
    return res


def run_reference(args):
    """The CPU reference arm on the box the line names: the oracle port (a C
    restatement of the reference's algorithm, pinned bit for bit to the
    reference's own code where that compiles) on every host core, one full
    force evaluation of the same ng^3 box per step, `warmup` untimed steps
    then `steps` timed ones.  The reference's own build is single-rank and
    single-threaded (its null MDL) and its sources are not on the GPU host,
    so the port under OpenMP stands in for it: a stronger baseline."""
    import oracle
    pos, vel, m, soft = workload(args.ng, with_vel=True)
    # the two position sets a drift apart that the end-to-end leg uses
    sets = (drifted(pos, vel, DRIFT_DT), pos)
    n = len(m)
    nth = os.cpu_count() or 1
    gp = oracle.grav_params(periodic=True, ewald=True, nBucket=NBUCKET)
    o = oracle.oracle()
    for k in range(args.warmup):
        o.grav(sets[k & 1], m, soft, gp, nthreads=nth)
    times = []
    for k in range(args.steps):
        t = time.perf_counter()
        o.grav(sets[(args.warmup + k) & 1], m, soft, gp, nthreads=nth)
        times.append(time.perf_counter() - t)
    sec = statistics.mean(times)
    value = n / sec
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config(args.ng, nbucket=NBUCKET), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nth, "kind": "port",
                         "sample": f"one full evaluation of the {args.ng}^3 box per step, "
                                   "alternating between two position sets a drift apart "
                                   "(tree build serial, walk + Ewald OpenMP over buckets; "
                                   "FP64, the reference's own arithmetic)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ---------------------------------------------------------------------------
# the other workloads (each prints its own JSON line; the default run is the
# periodic box above)
# ---------------------------------------------------------------------------
def _cuda_ms(fn, stream):
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def run_profile(args):
    """The box's FP32 step alone, as the timed run takes it -- a
    kick-drift-kick step replayed from one CUDA graph, dt +-DRIFT_DT in
    turn -- `steps` times after `warmup` (no autotune, FP64, error or CPU
    legs): the command the ncu summaries use."""
    import torch
    import gasoline_gb300 as g
    stream = torch.cuda.Stream()
    ctx = g.Context(0, stream=stream.cuda_stream)
    # the knobs the timed run's autotuner picks for this box: the default
    # five walk blocks per SM, no walk groups, the fused walk (or the walk
    # mode asked for)
    ctx.set_tuning(walkGroup=-1, walkLists=args.walk_lists)
    pos, vel, m, soft = workload(args.ng, with_vel=True)
    ctx.set_particles(pos, m, soft)
    ctx.set_velocities(vel)
    gp = g.grav_params(periodic=True, precision=g.FP32, nBucket=NBUCKET, iOrder=args.iorder)
    ctx.grav_all(gp)
    sgn = -1.0
    for _ in range(args.warmup):
        sgn = -sgn
        ctx.step(sgn * DRIFT_DT, gp, None, graph=True)
    ms = []
    for _ in range(args.steps):
        sgn = -sgn
        ms.append(_cuda_ms(lambda: ctx.step(sgn * DRIFT_DT, gp, None, graph=True), stream))
    ctx.step_status()
    ctx.close()
    return {"profile": "box", "n_particles": len(m), "nBucket": NBUCKET, "iOrder": args.iorder,
            "ms_per_step": statistics.mean(ms)}


def run_gas(args):
    """One gravity + SPH force evaluation (density, pressure) of the 1/r gas
    sphere, N = collapse_n, `steps` times: the SPH kernels' profiling case."""
    import gasoline_gb300 as g
    n = args.collapse_n
    pos, vel, m, u = g.ics.gas_sphere(n, seed=41)
    soft = np.full(n, 0.01)
    ctx = g.Context(0)
    ctx.set_particles(pos, m, soft)
    ctx.set_velocities(vel, n, u)
    sp = g.sph_params(nSmooth=32, precision=g.FP32 if args.sph_fp32 else g.FP64)
    gp = g.grav_params(periodic=False, precision=g.FP32, nBucket=NBUCKET)
    rows = []
    for it in range(args.warmup + args.steps):
        ctx.grav_all(gp)
        tg = ctx.timings()
        d = ctx.smooth(g.SMX_DENDVDX, sp)
        ctx.smooth(g.SMX_SPHPRESSURETERMS, sp)
        t = ctx.timings()
        if it >= args.warmup:
            rows.append({"grav": tg["total"], "knn_tree": t["knn"], "density": t["density"],
                         "pressure": t["pressure"], "candidates_per_particle": d["dCandidates"] / n})
    ctx.close()
    return {"profile": "gas", "n_gas": n, "sph_precision": "fp32" if args.sph_fp32 else "fp64",
            "phase_ms": {k: statistics.mean(r[k] for r in rows) for k in rows[0]}}


def run_plummer(args):
    """Plummer sphere, N = 32768: one gravity evaluation plus one KDK step
    (dt = 1e-3) in FP64 and FP32, forces against the FP64 direct sum."""
    import torch
    import gasoline_gb300 as g
    import oracle
    pos, vel, m = g.ics.plummer(32768, seed=1)
    soft = np.full(len(m), 0.01)
    stream = torch.cuda.Stream()
    ctx = g.Context(0, stream=stream.cuda_stream)
    ctx.set_particles(pos, m, soft)
    ctx.set_velocities(vel)
    ad, _ = oracle.direct(pos, m, soft, np.arange(len(m)), nthreads=os.cpu_count() or 1)
    res = {}
    roof = None
    for name, prec in (("fp64", g.FP64), ("fp32", g.FP32)):
        gp = g.grav_params(periodic=False, precision=prec)
        for _ in range(args.warmup):
            ctx.grav_all(gp)
        ts, walk = [], []
        for _ in range(args.steps):
            box = {}
            ts.append(_cuda_ms(lambda: box.update(ctx.grav_all(gp)), stream))
            walk.append(ctx.timings()["walk"])
        if prec == g.FP32:
            roof = walk_roofline(ctx, box, statistics.mean(walk), 8)
        a = ctx.get_gravity()["acc"]
        e = np.linalg.norm(a - ad, axis=1) / np.linalg.norm(ad, axis=1)
        tk = [_cuda_ms(lambda: (ctx.kick(5e-4), ctx.drift(1e-3, False, 1.0), ctx.grav_all(gp),
                                ctx.kick(5e-4)), stream)]
        res[name] = {"grav_ms": statistics.mean(ts), "kdk_step_ms": tk[0],
                     "err_vs_direct_rms": float(np.sqrt(np.mean(e ** 2))),
                     "err_vs_direct_p99": float(np.percentile(e, 99))}
        if prec == g.FP32:
            # the same KDK step captured once as a CUDA graph and replayed:
            # at this size the directly launched step is launch-bound
            ctx.step(1e-3, gp, None, graph=True)
            ctx.step_status()
            tg = [_cuda_ms(lambda: ctx.step(1e-3, gp, None, graph=True), stream)
                  for _ in range(args.steps)]
            ctx.step_status()
            res[name]["kdk_step_graph_ms"] = statistics.mean(tg)
        ctx.set_particles(pos, m, soft)
        ctx.set_velocities(vel)
    ctx.close()
    # CPU baseline: the oracle's gravity evaluation of the same sphere on
    # every host core, and its KDK step
    nth = os.cpu_count() or 1
    tg, _ = oracle_seconds(lambda: oracle.oracle().grav(pos, m, soft, oracle.grav_params(periodic=False),
                                                          nthreads=nth))
    ms = res["fp32"]["grav_ms"]
    return {"metric": "particle force evals/s, Plummer N=32768 (gravity)", "value": 32768 / (ms * 1e-3),
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic Plummer sphere, seed 1",
            "config": {"workload": "Plummer N=32768, G=M=a=1, rmax=20a, theta=0.7, eps=0.01, "
                                   "nBucket=8, one eval + one KDK dt=1e-3"}, "paths": res,
            "roofline": roof,
            "cpu_baseline": {"value": 32768 / tg, "unit": UNIT, "cores": nth, "kind": "port",
                             "sample": f"one full gravity evaluation of the same sphere ({tg:.3f} s, "
                                       "FP64, tree build serial, walk OpenMP over buckets)"}}


def run_collapse(args):
    """Adiabatic collapse of a 1/r gas sphere, N = 262144, self-gravity + SPH
    over `--collapse-steps` KDK steps of `--collapse-dt` (0.002).  Run A collects the
    h-network's samples on the first 50 steps, trains it on the GPU and then
    seeds every kNN with its prediction; run B is the same simulation with
    the exact kNN alone.  Neighbour sets and fBall2 are compared bit for bit
    every step after training."""
    import gasoline_gb300 as g
    from gasoline_gb300.sim import Simulation
    n = args.collapse_n
    pos, vel, m, u = g.ics.gas_sphere(n, seed=41)
    soft = np.full(n, 0.01)
    kw = dict(ngas=n, u=u, nSmooth=32, precision=g.FP32, sph_precision=g.FP32)
    A = Simulation(pos, vel, m, soft, **kw)
    B = Simulation(pos, vel, m, soft, **kw)
    A.ctx.hnet_init(seed=3)
    A.ctx.hnet_mode(collect=True)
    A.forces()
    B.forces()
    # fixed step: 200 x 0.002 reaches t = 0.4, before the bounce near the
    # free-fall time (~1.1) where a fixed step would violate the Courant limit
    dt, ntrain = args.collapse_dt, 50
    rows = {"A": [], "B": []}
    mismatch = 0
    train = {}
    for step in range(args.collapse_steps):
        if step == ntrain:
            t0 = time.perf_counter()
            l0 = A.ctx.hnet_train(steps=0, batch=8192)
            l1 = A.ctx.hnet_train(steps=600, batch=8192, lr=3e-3)
            train = {"loss_before": l0, "loss_after": l1, "samples": A.ctx.hnet_info()[0],
                     "train_s": time.perf_counter() - t0, "adam_steps": 600, "batch": 8192}
            A.ctx.hnet_mode(collect=False, predict=True, margin=0.08)
            A.learned_h = True
        ra = A.step(dt)
        rb = B.step(dt)
        if step >= ntrain:
            for key, r in (("A", ra), ("B", rb)):
                rows[key].append((r["wall_s"], r["t_grav_ms"], r["t_knn_density_ms"],
                                  r["t_pressure_ms"], r["density"]["dCandidates"],
                                  r["density"]["nFallback"], r["density"]["bSeeded"],
                                  r["t_knn_tree_ms"], r["density"]["dPairs"]))
            sa, sb = A.ctx.get_sph(), B.ctx.get_sph()
            ha, hb = A.ctx.get_neighbour_hash(), B.ctx.get_neighbour_hash()
            if not (np.array_equal(sa["fBall2"], sb["fBall2"]) and np.array_equal(ha[1], hb[1])
                    and np.array_equal(ha[0], hb[0])):
                mismatch += 1
    def summ(rr):
        a = np.array(rr, dtype=np.float64)
        return {"step_ms": float(a[:, 0].mean() * 1e3), "grav_ms": float(a[:, 1].mean()),
                "density_ms": float(a[:, 2].mean()), "pressure_ms": float(a[:, 3].mean()),
                "candidates_per_particle": float(a[:, 4].mean() / n),
                "grown_balls_per_pass": float(a[:, 5].mean()), "seeded": bool(a[:, 6].all()),
                "knn_tree_ms": float(a[:, 7].mean()), "pairs_per_pass": float(a[:, 8].mean())}
    sa_, sb_ = summ(rows["A"]), summ(rows["B"])
    roof = density_roofline(A.ctx, {"dPairs": sa_["pairs_per_pass"],
                                    "dCandidates": sa_["candidates_per_particle"] * n},
                            sa_["density_ms"], True)
    A.ctx.close()
    B.ctx.close()
    # CPU baseline: the oracle's force evaluation of the initial sphere
    # (gravity, then both SPH passes) on every host core
    import oracle
    nth = os.cpu_count() or 1
    tg, _ = oracle_seconds(lambda: oracle.oracle().grav(pos, m, soft, oracle.grav_params(periodic=False),
                                                          nthreads=nth))
    tsph, _ = oracle_seconds(lambda: oracle.oracle().sph(pos, vel, m, soft, u, oracle.sph_params(nSmooth=32),
                                                           nthreads=nth))
    return {"metric": "gas particle force evals/s (gravity + SPH density + pressure), "
                      "adiabatic collapse N=262144, learned h", "value": n / (sa_["step_ms"] * 1e-3),
            "unit": UNIT, "n_gpus": 1, "steps": args.collapse_steps, "warmup": ntrain,
            "ms_per_step": sa_["step_ms"], "higher_is_better": True, "dtype": "f32 gravity, f32 SPH",
            "data": "synthetic 1/r gas sphere, seed 41",
            "roofline": roof,
            "cpu_baseline": {"value": n / (tg + tsph), "unit": UNIT, "cores": nth, "kind": "port",
                             "sample": f"one force evaluation of the initial sphere: gravity "
                                       f"{tg:.2f} s + SPH density and pressure passes {tsph:.2f} s "
                                       "(FP64, OpenMP)"},
            "config": {"workload": "adiabatic collapse, 262144 gas, M=R=G=1, u=0.05, gamma=5/3, "
                                   f"nSmooth=32, alpha=1, beta=2, dt={dt}, MLP trained on steps 0-49",
                       "timing": "host wall clock per KDK step incl. host round trips"},
            "learned_h": sa_, "exact_knn": sb_, "training": train,
            "density_speedup_learned_vs_exact": sb_["density_ms"] / sa_["density_ms"],
            "neighbour_sets_bit_exact": mismatch == 0, "steps_with_mismatch": mismatch}


def run_multistep(args):
    """Adaptive timesteps on the 1/r gas sphere (N = collapse_n): base step
    0.02 with up to 6 rungs (finest step 0.02/32), FP32 gravity + FP64 SPH,
    `steps` base steps after `warmup`.  Throughput counts the particles that
    received forces; the single-rung cost of the same time resolution is
    one all-active step at the finest step used, times 2^maxRung."""
    import torch
    import gasoline_gb300 as g
    n = args.collapse_n
    pos, vel, m, u = g.ics.gas_sphere(n, seed=41)
    soft = np.full(n, 0.01)
    stream = torch.cuda.Stream()
    ctx = g.Context(0, stream=stream.cuda_stream)
    ctx.set_particles(pos, m, soft)
    ctx.set_velocities(vel, ngas=n, u=u)
    gp = g.grav_params(periodic=False, precision=g.FP32)
    sp = g.sph_params(nSmooth=32)
    st = g.step_params(iMaxRung=6)
    dDelta = 0.02
    ctx.grav_all(gp)
    ctx.smooth(g.SMX_DENDVDX, sp)
    ctx.smooth(g.SMX_SPHPRESSURETERMS, sp)
    t = 0.0
    for _ in range(args.warmup):
        ctx.top_step_kdk(t, dDelta, gp, sp, st)
        t += dDelta
    outs, ts = [], []
    for _ in range(args.steps):
        box = {}
        ts.append(_cuda_ms(lambda: box.update(ctx.top_step_kdk(t, dDelta, gp, sp, st)), stream))
        outs.append(box)
        t += dDelta
    rungs = ctx.get_rungs()["rung"]
    maxr = max(o["iCurrMaxRung"] for o in outs)
    # single rung at the finest step, on the same state
    fine = dDelta / 2 ** maxr
    ctx.step(fine, gp, sp)
    ctx.step_status()
    t1 = [_cuda_ms(lambda: (ctx.step(fine, gp, sp), ctx.step_status()), stream) for _ in range(3)]
    ctx.close()
    ms = statistics.mean(ts)
    act = statistics.mean(o["nActiveSum"] for o in outs)
    single = statistics.mean(t1) * 2 ** maxr
    return {"metric": "particle force evals/s with adaptive timesteps, gas sphere N=262144",
            "value": act / (ms * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "dtype": "f32 gravity, f64 SPH", "data": "synthetic 1/r gas sphere, seed 41",
            "config": {"workload": f"1/r gas sphere N={n}, base step {dDelta}, iMaxRung 6, "
                                   "eta 0.1, eta_Courant 0.4, nSmooth 32",
                       "timing": "CUDA events around each base step (host recursion included)"},
            "force_passes_per_step": statistics.mean(o["nForcePasses"] for o in outs),
            "active_per_step": act, "max_rung": maxr,
            "rung_histogram": np.bincount(rungs, minlength=maxr + 1).tolist(),
            "single_rung_ms_per_base_step": single,
            "speedup_vs_single_rung_same_finest_step": single / ms}


def run_snapshot(args):
    """Tipsy snapshot I/O of the 128^3 box (2,097,152 dark particles, 75 MB):
    tsph_write_tipsy and tsph_read_tipsy through the C ABI, the file in the
    page cache, against the oracle's numpy reader on the same file."""
    import time
    import gasoline_gb300 as g
    from oracle import tipsy
    pos, m, soft = workload(args.ng)
    n = len(m)
    ctx = g.Context(0)
    ctx.set_particles(pos, m, soft)
    ctx.set_velocities(np.zeros((n, 3)))
    import tempfile
    tmpdir = tempfile.mkdtemp(prefix="tsph_snapshot_")
    path = os.path.join(tmpdir, "bench_snapshot.std")
    ctx.write_tipsy(path, 0.0)
    size = os.path.getsize(path)
    tw, tr = [], []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        ctx.write_tipsy(path, 0.0)
        t1 = time.perf_counter()
        ctx.read_tipsy(path)
        t2 = time.perf_counter()
        if k >= args.warmup:
            tw.append(t1 - t0)
            tr.append(t2 - t1)
    t0 = time.perf_counter()
    tipsy.read(path)
    tcpu = time.perf_counter() - t0
    ctx.close()
    os.remove(path)
    os.rmdir(tmpdir)
    r = statistics.mean(tr)
    return {"metric": "Tipsy snapshot read, particles/s (file in page cache -> device state)",
            "value": n / r, "unit": "particles/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r * 1e3, "higher_is_better": True,
            "dtype": "f32 file, f64 state", "data": "synthetic 128^3 box",
            "config": {"workload": f"standard (XDR) Tipsy file, {n} dark particles, {size} bytes",
                       "timing": "host wall clock per call"},
            "read_GBps": size / r / 1e9, "write_ms": statistics.mean(tw) * 1e3,
            "write_GBps": size / statistics.mean(tw) / 1e9,
            "cpu_baseline": {"value": n / tcpu, "unit": "particles/s", "cores": 1, "kind": "port",
                             "sample": "the oracle's numpy reader on the same file"}}


def _oracle_system_job(job):
    """One independent system by the oracle on one core (a pool worker):
    gravity and, for a system with gas, the density and pressure passes."""
    import oracle
    if job is None:
        oracle.oracle()
        return 0
    pos, vel, mass, soft, ng, nbucket = job
    o = oracle.oracle()
    o.grav(pos, mass, soft, oracle.grav_params(periodic=False, nBucket=nbucket), nthreads=1)
    if ng > 0:
        o.sph(pos[:ng], vel[:ng], mass[:ng], soft[:ng], np.full(ng, 0.05), oracle.sph_params(nSmooth=32),
              nthreads=1)
    return len(mass)


def run_batched(args):
    """512 independent Plummer/Hernquist spheres, N log-uniform in
    [1024, 65536], every other pair with a 0.2 gas fraction: one context, a
    forest of trees; launch shapes autotuned, then whole KDK steps replayed
    from one CUDA graph.  FP32 gravity against the FP64 direct sum on a
    sample of every system."""
    import torch
    import gasoline_gb300 as g
    from gasoline_gb300 import autotune
    import oracle
    systems = g.ics.batched_systems(nsys=args.nsys, seed=5)
    pos, vel, m, soft, ngas, u, so, index = g.ics.pack_systems(systems)
    n = len(m)
    stream = torch.cuda.Stream()
    ctx = g.Context(0, stream=stream.cuda_stream)
    ctx.set_particles(pos, m, soft)
    ctx.set_velocities(vel, ngas, u)
    ctx.set_systems(so)
    sp = g.sph_params(nSmooth=32, precision=g.FP32)
    best, table = autotune.tune_gravity(ctx, g.grav_params(periodic=False, precision=g.FP32))
    gp = g.grav_params(periodic=False, precision=g.FP32, nBucket=best["nBucket"])
    ctx.set_tuning(taskSize=best["taskSize"], walkBlocksPerSM=best["walkBlocksPerSM"],
                   walkGroup=best["walkGroup"], walkLists=best["walkLists"])
    gout = ctx.grav_all(gp)
    gtim = ctx.timings()
    roof = walk_roofline(ctx, gout, gtim["walk"], min(32, max(8, best["nBucket"])))
    acc = ctx.get_gravity()["acc"]
    errs = []
    for s_, d in enumerate(systems):
        q = np.linspace(0, len(d["mass"]) - 1, 16).astype(np.int64)
        ad, _ = oracle.direct(d["pos"], d["mass"], d["soft"], q, nthreads=os.cpu_count() or 1)
        e = np.linalg.norm(acc[index[s_][q]] - ad, axis=1) / np.linalg.norm(ad, axis=1)
        errs.append(float(np.sqrt(np.mean(e ** 2))))
    res = {}
    for graph in (False, True):
        ctx.step(1e-4, gp, sp, graph=graph)
        ctx.step_status()
        l0 = ctx.launches()
        ts = [_cuda_ms(lambda: ctx.step(1e-4, gp, sp, graph=graph), stream) for _ in range(args.steps)]
        ctx.step_status()
        res["graph" if graph else "direct"] = {"step_ms": statistics.mean(ts),
                                               "kernels_per_step": (ctx.launches() - l0) / args.steps}
    ctx.smooth(g.SMX_DENDVDX, sp)
    ctx.smooth(g.SMX_SPHPRESSURETERMS, sp)
    stim = ctx.timings()
    phases = {"gravity": {k: gtim[k] for k in ("build", "moments", "walk", "total")},
              "sph": {k: stim[k] for k in ("knn", "density", "pressure")}}
    ctx.close()
    # CPU baseline: independent systems, as the reference runs them (one job
    # each): every 4th system, gravity and (for the gas systems) both SPH
    # passes by the oracle, one single-threaded process per host core
    # (spawned, warmed up before the timed map)
    import multiprocessing
    nth = os.cpu_count() or 1
    sample = systems[::4]
    with multiprocessing.get_context("spawn").Pool(nth) as pool:
        pool.map(_oracle_system_job, [None] * nth)      # workers loaded
        t0 = time.perf_counter()
        pool.map(_oracle_system_job, [(d["pos"], d["vel"], d["mass"], d["soft"], d["ngas"], best["nBucket"])
                                      for d in sample], chunksize=1)
        t_cpu = time.perf_counter() - t0
    n_cpu = sum(len(d["mass"]) for d in sample)
    ms = res["graph"]["step_ms"]
    return {"metric": "particle force evals/s, 512 batched uneven systems (gravity + SPH), one CUDA graph per step",
            "value": n / (ms * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": 1, "ms_per_step": ms, "higher_is_better": True, "dtype": "f32 gravity, f32 SPH",
            "data": "synthetic Plummer/Hernquist spheres, seed 5",
            "config": {"workload": f"{args.nsys} systems, N log-uniform [1024, 65536], total {n}, "
                                   f"gas {ngas}, eps=0.01, theta=0.7, nSmooth=32",
                       "tuned": best},
            "autotune": table, "steps": res, "roofline": roof, "phase_ms": phases,
            "cpu_baseline": {"value": n_cpu / t_cpu, "unit": UNIT, "cores": nth, "kind": "port",
                             "sample": f"{len(sample)} of the {len(systems)} systems (every 4th, "
                                       f"{n_cpu} particles): oracle gravity + SPH per system, "
                                       f"{t_cpu:.2f} s (FP64, one single-threaded process per system "
                                       f"on {nth} cores)"},
            "per_system_err_vs_direct": {"max_rms": max(errs), "median_rms": float(np.median(errs))}}


def run_mixed(args):
    """Clustered periodic box, 2 x ng^3 (gas + dark matter) with 64 Plummer
    clumps: full gravity (FP32, Ewald) + SPH step with the learned h after
    two steps of sample collection and GPU training."""
    import gasoline_gb300 as g
    from gasoline_gb300.sim import Simulation
    ng = args.mixed_ng
    pos, vel, m, ngas, u = g.ics.mixed_box(ng, seed=6)
    n = len(m)
    soft = np.full(n, 1.0 / (50.0 * ng))
    sim = Simulation(pos, vel, m, soft, ngas=ngas, u=u, periodic=True, L=1.0, nSmooth=32,
                     precision=g.FP32, sph_precision=g.FP32)
    sim.ctx.hnet_init(seed=3)
    sim.ctx.hnet_mode(collect=True)
    sim.forces()
    for _ in range(2):
        sim.step(1e-4)
    loss = sim.ctx.hnet_train(steps=300, batch=8192, lr=3e-3)
    sim.ctx.hnet_mode(collect=False, predict=True, margin=0.08)
    sim.learned_h = True
    recs = [sim.step(1e-4) for _ in range(max(1, args.steps // 5))]
    r = recs[-1]
    roof = density_roofline(sim.ctx, r["density"], r["t_knn_density_ms"], True)
    # learned h against the exact kNN alone on the same particles: the
    # density pass seeded by the network and unseeded, twice each
    cmp = {}
    for learned in (True, False, True, False):
        sim.learned_h = learned
        sim.sp.bLearnedH = int(learned)
        d = sim.ctx.smooth(g.SMX_DENDVDX, sim.sp)
        t = sim.ctx.timings()
        cnt, hsh = sim.ctx.get_neighbour_hash()
        key = "learned_h" if learned else "exact_knn"
        cmp[key] = {"density_ms": t["density"], "knn_tree_ms": t["knn"],
                    "candidates_per_particle": d["dCandidates"] / ngas, "seeded": bool(d["bSeeded"]),
                    "grown_balls": d["nFallback"], "_hash": hsh, "_fb": sim.ctx.get_sph()["fBall2"]}
    same = (np.array_equal(cmp["learned_h"].pop("_hash"), cmp["exact_knn"].pop("_hash")) and
            np.array_equal(cmp["learned_h"].pop("_fb"), cmp["exact_knn"].pop("_fb")))
    cmp["neighbour_sets_and_fBall2_identical"] = bool(same)
    cmp["density_speedup"] = cmp["exact_knn"]["density_ms"] / cmp["learned_h"]["density_ms"]
    sim.learned_h = True
    sim.ctx.close()
    ms = statistics.mean(x["wall_s"] for x in recs) * 1e3
    # CPU baseline: one gravity evaluation (Ewald) of the same construction
    # at 2 x 128^3 by the oracle on every host core (the full box's serial
    # tree build alone takes the oracle minutes)
    import oracle
    nth = os.cpu_count() or 1
    ps, _, ms_, _, _ = g.ics.mixed_box(128, seed=6)
    ts_, _ = oracle_seconds(lambda: oracle.oracle().grav(ps, ms_, np.full(len(ms_), 1.0 / (50.0 * 128)),
                                                         oracle.grav_params(periodic=True, ewald=True),
                                                         nthreads=nth))
    return {"metric": "particle force evals/s, clustered mixed box 2x%d^3 (gravity + SPH), learned h" % ng,
            "value": n / (ms * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": len(recs), "warmup": 2,
            "ms_per_step": ms, "higher_is_better": True, "dtype": "f32 gravity, f32 SPH",
            "data": "synthetic two-lattice GRF box + 64 Plummer clumps, seed 6",
            "config": {"workload": f"2x{ng}^3 periodic box, gas fraction 0.16, 20% in clumps, "
                                   "Ewald, theta=0.7, nSmooth=32, learned h",
                       "timing": "host wall clock per KDK step"},
            "phases_ms": {"grav": r["t_grav_ms"], "density": r["t_knn_density_ms"],
                          "pressure": r["t_pressure_ms"]},
            "roofline": roof,
            "cpu_baseline": {"value": len(ms_) / ts_, "unit": UNIT, "cores": nth, "kind": "port",
                             "sample": f"one gravity evaluation (Ewald) of the 2x128^3 box of the same "
                                       f"construction, {len(ms_)} particles, {ts_:.1f} s (FP64, tree build "
                                       "serial, walk + Ewald OpenMP); the SPH passes are not in the sample"},
            "hnet_loss": loss, "seeded": r["density"]["bSeeded"],
            "learned_vs_exact_density_pass": cmp}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ng", type=int, default=128)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="box",
                    choices=["box", "plummer", "collapse", "batched", "mixed", "gas", "multistep",
                             "snapshot"])
    ap.add_argument("--profile", action="store_true",
                    help="box FP32 evaluations only (the ncu capture command)")
    ap.add_argument("--sph-fp32", action="store_true")
    ap.add_argument("--iorder", type=int, default=2,
                    help="cell multipole order of the profile leg (4: the reference's default)")
    ap.add_argument("--walk-lists", type=int, default=0,
                    help="--profile: the walk mode (tsph_tuning.walkLists; 1 = two passes)")
    ap.add_argument("--collapse-n", type=int, default=262144)
    ap.add_argument("--collapse-steps", type=int, default=200)
    ap.add_argument("--collapse-dt", type=float, default=0.002)
    ap.add_argument("--nsys", type=int, default=512)
    ap.add_argument("--mixed-ng", type=int, default=256)
    args = ap.parse_args()
    if args.profile:
        print(json.dumps(run_profile(args)), flush=True)
        return
    if args.workload != "box":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "workload": args.workload,
                              "unavailable": "the reference arm is timed on the periodic box only"}))
            return
        fn = {"plummer": run_plummer, "collapse": run_collapse, "batched": run_batched,
              "mixed": run_mixed, "gas": run_gas, "multistep": run_multistep,
              "snapshot": run_snapshot}[args.workload]
        print(json.dumps(fn(args)), flush=True)
        return
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
