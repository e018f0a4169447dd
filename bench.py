#!/usr/bin/env python3
"""ORB build benchmark on GB300: 2^27 uniform float32 particles into 2^16 leaf cells.

One step = one ORB build (orb_build through the C ABI) of the whole particle set, preceded
by a device-to-device restore of the unpartitioned input (the build partitions in place).

  value      particles/s with inputs resident in HBM (restore + build per step)
  e2e        particles/s through orb_build with pinned HOST buffers, as the reference's
             driver calls it: H2D of x,y,z, build, D2H of the reordered x,y,z, the cell heap
             and the range map (the reference has no permutation output); beside it the
             host link's own copy rate measured in the same run (its ceiling)
  roofline   the dominant kernel's algorithmic bytes / its CUDA-event time in the timed
             region (on the engine's stream) against the measured HBM copy bandwidth
  count_left every count-left launch of the same steps, timed with CUDA events in a second
             region right after the headline's (against the same peak)
  cpu_baseline  the CPU oracle with the reference's MDL semantics (one rank per host core,
             per-cell counts summed, per-rank Hoare partition) on a bounded sample; the same
             leg runs the single-rank oracle on the benchmark's own inputs (outside every
             timed region) as the checker of the GPU outputs: "parity"
  clustered  the same measurements for 2^26 Plummer-clustered particles into 2^18 leaves
  weighted   weighted ORB (integer weights per particle, a labelled mode) on 2^26 clustered
             particles into 2^16 leaves
  batched    128 uneven instances in one batched build against one build at a time
  served     a Poisson request stream through the continuous-batching server

--impl reference times the CPU implementation alone (rank 0), as the reference arm, with
the same config. With torchrun (N>1) every rank builds its own replica on its own GPU (the
path has no data exchange on one GPU per box): value sums the particles of all ranks.
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
PKG_DIR = os.path.join(ROOT, "gpu-load-balance_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
sys.path.insert(0, PKG_DIR)

N_PARTICLES = 1 << 27
LEAVES = 1 << 16
SEED = 20270
METRIC = "orb_build_particles_per_s"
WARM_WIDTH = 8.0  # warm rebuild: bracket factor (half-width = factor x extent / sqrt(n))
UNIT = "particles/s"
FALLBACK_HBM_GBS = 6800.0
CLUSTERED = (1 << 26, 1 << 18)
WEIGHTED = (1 << 26, 1 << 16)
TRAFFIC_PROFILE = "dram_traffic_part_swap_hist_classify_subtree_2p24_2p13.txt"
# every kernel kind that counts keys below a cut (the count-left family)
COUNT_LEFT_KERNELS = ("count_left_hist", "bisect_tile", "bisect_cta", "count_left_sample",
                      "count_left_sample_pick")
PARTITION_KERNELS = ("part_classify", "part_scan", "part_cells", "part_swap", "part_finish")


def workload_name(kind: str, n: int, d: int) -> str:
    lg = lambda v: f"2^{v.bit_length() - 1}" if v & (v - 1) == 0 else str(v)
    what = "uniform float32 particles in [-0.5,0.5)^3" if kind == "uniform" else \
        "float32 particles, 90% from 64 Plummer spheres + 10% uniform, in [-0.5,0.5)^3"
    return f"plain ORB, {lg(n)} {what}, {lg(d)} leaf cells"


def workload_config(n: int, d: int, world: int) -> dict:
    """The `config` both arms print (the same keys and values in both, so the lines compare)."""
    return {"workload": workload_name("uniform", n, d), "particles": n, "leaves": d,
            "levels": d.bit_length() - 1, "parallelism": f"replicas x{world}",
            "l2": "inputs 1.5 GB > 129 MB L2 (no flush needed)" if 12 * n > (129 << 20)
            else "inputs smaller than the 129 MB L2"}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str | None):
        self.rows = []
        self.proc = None
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
               "-lms", "200"]
        if gpu_id is not None:
            cmd += ["-i", gpu_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
        except Exception:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append((time.perf_counter(), parts))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0: float, t1: float):
        sel = [r for (t, r) in self.rows if t0 <= t <= t1] or [r for (_, r) in self.rows]
        if not sel:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"],
                    "samples": 0}

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None

        sm = [num(r[1]) for r in sel if num(r[1]) is not None]
        mx = [num(r[2]) for r in sel if num(r[2]) is not None]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in sel:
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sel)}


def traffic_ratio(kernel: str):
    """DRAM traffic per algorithmic byte of a kernel, from the committed ncu summary (a
    smaller case of the same workload; the ratio is per swapped pair / per key, so it scales
    with the units a launch processes)."""
    names = {"part_swap": "k_part_swap", "count_left_hist": "k_hist", "part_classify": "k_part_classify",
             "bisect_tile": "k_bisect_tile", "subtree": "k_subtree"}
    path = os.path.join(ROOT, "profiles", TRAFFIC_PROFILE)
    try:
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 3 and parts[0] == "traffic_per_algorithmic_byte" and parts[1] == names.get(kernel):
                    return float(parts[2])
    except OSError:
        pass
    return None


def gpu_id_for(local_rank: int):
    cvd = os.environ.get("CUDA_VISIBLE_DEVICES")
    if cvd:
        ids = [s.strip() for s in cvd.split(",") if s.strip()]
        if local_rank < len(ids):
            return ids[local_rank]
    return str(local_rank)


# ------------------------------------------------------------------------------------------
# CPU leg: the oracle as the timed CPU baseline (MDL semantics) and as the checker
# ------------------------------------------------------------------------------------------
def _oracle():
    sys.path.insert(0, ORACLE_DIR)
    import oracle as O  # the checker and the CPU baseline; never on the GPU path
    O.build()
    return O


def cpu_build_probe(n: int, d: int, threads: int):
    O = _oracle()
    x, y, z = O.gen_uniform(SEED, n, nthreads=threads)
    t = time.perf_counter()
    r = O.build_tree(x, y, z, d, nranks=threads, make_axis=True, copy=False, want_perm=False)
    return time.perf_counter() - t, r.stats


def cpu_sample_size(n: int, d: int, budget_s: float, steps: int, threads: int):
    """Largest (n, d) with the workload's particles-per-leaf whose run fits the budget."""
    t_probe, _ = cpu_build_probe(max(n >> 5, 1 << 12), max(d >> 5, 2), threads)
    per_step = t_probe * 32 * 1.15  # levels grow by 5 at full size
    while per_step * steps > budget_s and n > (1 << 20):
        n >>= 1
        d >>= 1
        per_step /= 2
    return n, d


def run_cpu(n_full: int, d_full: int, steps: int, warmup: int, budget_s: float):
    threads = os.cpu_count() or 1
    n, d = cpu_sample_size(n_full, d_full, budget_s, steps + warmup, threads)
    times = []
    stats = None
    for i in range(warmup + steps):
        t, stats = cpu_build_probe(n, d, threads)
        if i >= warmup:
            times.append(t)
    total = sum(times)
    value = n * len(times) / total
    sample = (f"oracle with MDL semantics ({threads} ranks = host threads, makeAxis gather on), "
              f"{n} particles / {d} leaves per step (same particles per leaf as the workload), "
              f"{len(times)} steps")
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
            "ms_per_step": 1e3 * total / len(times), "phase_s": {k: stats[k] for k in
            ("t_make_axis_s", "t_count_s", "t_partition_s", "t_total_s")}}


def check_parity(job):
    """The checker: the single-rank oracle (src/orbit.cpp:102-275 restated, cells in
    parallel) on the job's own inputs, compared bit for bit with the GPU's outputs."""
    import numpy as np
    O = _oracle()
    threads = os.cpu_count() or 1
    t = time.perf_counter()
    out = {"oracle": "single-rank restatement of the reference's CPU path, run on the "
                     "benchmark's own inputs", "compared": ["heap", "ranges", "perm", "x", "y", "z"]}
    ok, cells, particles = True, 0, 0
    weighted = "w" in job
    if weighted:
        out["compared"].append("w")
    for inst in job["instances"]:
        sl = slice(inst["offset"], inst["offset"] + inst["n"])
        x, y, z = job["x"][sl], job["y"][sl], job["z"][sl]
        if weighted:
            ref, wref = O.build_tree_weighted(x, y, z, job["w"][sl], inst["d"], threads=threads)
        else:
            ref = O.build_tree(x, y, z, inst["d"], threads=threads)
        heap, ranges, gx, gy, gz, perm = inst["gpu"][:6]
        same = (heap.tobytes() == ref.heap.tobytes() and np.array_equal(ranges, ref.ranges[0])
                and np.array_equal(perm, ref.perm)
                and all(np.array_equal(a.view(np.uint32), b.view(np.uint32))
                        for a, b in ((gx, ref.x), (gy, ref.y), (gz, ref.z))))
        if weighted:
            same = same and np.array_equal(inst["gpu"][6], wref)
        ok = ok and same
        cells += len(ref.heap)
        particles += inst["n"]
    out.update({"bit_exact": bool(ok), "instances": len(job["instances"]), "cells": cells,
                "particles": particles, "oracle_s": round(time.perf_counter() - t, 2)})
    if len(job["instances"]) == 1 and not weighted:
        # the keys the reference's plain count-left scan reads, level by level (every key of
        # every cell still searching, at every sweep): the count passes' reference-equivalent
        out["ref_key_reads_per_level"] = ref.stats["elements_per_level"]
    return out


def effective_count_left(count_left: dict, kernels: dict, parity, peak: float):
    """The count-left aggregate's reference-equivalent rate: 4 B x the keys the reference's
    plain scan would read on the levels the count passes run, over their measured time. It
    can exceed the peak: the engine reads far fewer keys (compaction, one pass bins several
    sweeps)."""
    if not parity or "ref_key_reads_per_level" not in parity or not count_left.get("ms_per_step"):
        return
    levels = kernels.get("part_swap", {}).get("launches", 0)  # levels run level by level
    reads = sum(parity.pop("ref_key_reads_per_level")[:levels])
    gbs = 4.0 * reads / (count_left["ms_per_step"] / 1e3) / 1e9
    count_left["effective"] = {
        "achieved": round(gbs, 1), "unit": "GB/s", "frac": round(gbs / peak, 4),
        "bytes_per_step": 4 * reads, "levels": levels,
        "note": "reference-equivalent: 4 B x the keys the reference's plain scan reads on these "
                "levels (every key of every cell still searching, at every sweep; counted by the "
                "oracle on the same inputs) over the count-left time; may exceed the peak"}


def reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    cpu = run_cpu(args.particles, args.leaves, args.steps, args.warmup, budget_s=150.0)
    line = {
        "impl": "reference", "metric": METRIC, "value": cpu["value"], "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": cpu["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded uniform)",
        "config": workload_config(args.particles, args.leaves, world),
        "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": cpu["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------------------
# One plain workload (headline or clustered): device-resident steps, per-kernel profile,
# roofline, count-left, e2e through pinned host buffers, GPU outputs for the checker
# ------------------------------------------------------------------------------------------
def measure_link(torch, dev, nbytes: int, reps: int = 3):
    """The host link's copy rate with one plain copy of nbytes each way (pinned host)."""
    h = torch.empty(nbytes // 4, dtype=torch.float32, pin_memory=True)
    dbuf = torch.empty(nbytes // 4, dtype=torch.float32, device=dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    dbuf.copy_(h, non_blocking=True)
    h.copy_(dbuf, non_blocking=True)
    torch.cuda.synchronize(dev)
    ev[0].record()
    for _ in range(reps):
        dbuf.copy_(h, non_blocking=True)
    ev[1].record()
    for _ in range(reps):
        h.copy_(dbuf, non_blocking=True)
    ev[2].record()
    torch.cuda.synchronize(dev)
    h2d = reps * nbytes / (ev[0].elapsed_time(ev[1]) / 1e3) / 1e9
    d2h = reps * nbytes / (ev[1].elapsed_time(ev[2]) / 1e3) / 1e9
    del h, dbuf
    return h2d, d2h


def run_plain(ctx, E, torch, dev, args, kind: str, n: int, d: int, seed: int, peak: float,
              peak_kind: str, tuning_arg, clocks_cb=None, with_warm=False):
    import numpy as np

    gen = E.ORB_GEN_UNIFORM if kind == "uniform" else E.ORB_GEN_PLUMMER
    x0, y0, z0 = (torch.empty(n, dtype=torch.float32, device=dev) for _ in range(3))
    ctx.generate(gen, seed, n, x0, y0, z0, device_pointers=True)
    x, y, z = (torch.empty_like(x0) for _ in range(3))
    perm = torch.empty(n, dtype=torch.int32, device=dev)
    # cell heap and range map land in pinned host buffers (the API's host outputs)
    heap_pin = torch.empty((2 * d - 1) * 52, dtype=torch.uint8, pin_memory=True)
    ranges_pin = torch.empty((2 * d - 1) * 2, dtype=torch.int32, pin_memory=True)
    heap_np = heap_pin.numpy().view(E.CELL_DTYPE)
    ranges_np = ranges_pin.numpy().view(np.uint32).reshape(-1, 2)

    def step(with_perm=False):
        # the reference's outputs: reordered x,y,z, cell heap, range map (it has no
        # permutation output; with_perm adds the engine's optional one)
        x.copy_(x0)
        y.copy_(y0)
        z.copy_(z0)
        torch.cuda.synchronize(dev)
        return ctx.build(x, y, z, d, perm=perm if with_perm else None, device_pointers=True,
                         heap_out=heap_np, ranges_out=ranges_np)

    # launch parameters from the engine's autotuner on this workload (before any timing; the
    # inputs are copied, every candidate's tree is checked equal)
    t0 = time.perf_counter()
    if tuning_arg:
        names = ("hist_blocks_per_sm", "part_blocks_per_sm", "tile_blocks_per_sm",
                 "sparse_keys_per_tile", "cta_min_cells", "subtree_levels", "predict_sigmas")
        ctx.set_tuning(**dict(zip(names, (int(v) for v in tuning_arg.split(",")))))
        tuning, tuned_by = ctx.get_tuning(), "--tuning"
    else:
        tuning, _ = ctx.autotune_batch(x0, y0, z0, [{"offset": 0, "n": n, "d": d}], reps=2,
                                       device_pointers=True)
        tuned_by = "orb_autotune_batch"
    tune_s = time.perf_counter() - t0

    # warm-up steps time every kernel: per-kernel breakdown and the dominant kernel
    ctx.profile_reset(timing=True)
    for _ in range(args.warmup):
        step()
    warm = ctx.profile()
    warm_timed = {k: v for k, v in warm.items() if v["total_ms"] > 0}
    dom = max(warm_timed, key=lambda k: warm_timed[k]["total_ms"])
    # timed steps: CUDA events only around the dominant kernel's launches (one untimed step
    # first, so the build's CUDA graph is captured outside the timed region)
    ctx.profile_reset(timing=[dom])
    step()
    ctx.profile_reset(timing=[dom])
    torch.cuda.synchronize(dev)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    if clocks_cb:
        clocks_cb("start")
    ev0.record()
    infos = []
    for _ in range(args.steps):
        infos.append(step().info)
    ev1.record()
    torch.cuda.synchronize(dev)
    if clocks_cb:
        clocks_cb("end")
    ms_total = ev0.elapsed_time(ev1)
    prof = ctx.profile()
    launches = sum(v["launches"] for v in prof.values())

    # roofline of the dominant kernel (its events in the timed region)
    dk = prof[dom]
    achieved = dk["bytes"] / (dk["total_ms"] / 1e3) / 1e9
    kern_ms_total = sum(v["total_ms"] for v in warm_timed.values())
    ratio = traffic_ratio(dom)
    roofline = {
        "bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
        "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} hbm_gbs",
        "traffic": (ratio * dk["bytes"] / dk["launches"]) if ratio else None,
        "traffic_source": "ncu dram bytes per algorithmic byte, 2^24/2^13 capture scaled per unit"
                          if ratio else None,
        "dram_gbs_equivalent": round(achieved * ratio, 1) if ratio else None,
        "bytes_per_launch": dk["bytes"] / dk["launches"],
        "ms_per_launch": dk["total_ms"] / dk["launches"],
        "share_of_kernel_time": round(warm_timed[dom]["total_ms"] / kern_ms_total, 4),
    }
    if dom == "part_swap":
        # the partition's 36 B per particle and level model (key 4 B + coordinates 12 B read +
        # 12 B written + index 4+4 B of an out-of-place scatter) over the levels this kernel
        # partitions, beside the swap's own 48 B per swapped pair
        lv = dk["launches"] / args.steps
        model = 36.0 * n * lv * args.steps / (dk["total_ms"] / 1e3) / 1e9
        roofline["algorithmic_bytes"] = "48 B per swapped pair (x,y,z of both read and written)"
        roofline["model_36BN"] = {"achieved": round(model, 1), "frac": round(model / peak, 4),
                                  "levels": lv, "bytes_per_level": 36 * n,
                                  "note": "36 B x particles per level over the swap's event time"}
    # count-left: every count-left launch of a second timed region of the same steps (events
    # around its ~50 launches a build cost about 0.5 ms a step inside a graph, so they stay
    # out of the headline's region)
    cl_kinds = [k for k in COUNT_LEFT_KERNELS if k in warm]
    ctx.profile_reset(timing=cl_kinds)
    step()
    ctx.profile_reset(timing=cl_kinds)
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize(dev)
    clp = ctx.profile()
    cl_names = [k for k in cl_kinds if clp[k]["total_ms"] > 0]
    cl_bytes = sum(clp[k]["bytes"] for k in cl_names) / args.steps
    cl_ms = sum(clp[k]["total_ms"] for k in cl_names) / args.steps
    cl_gbs = cl_bytes / (cl_ms / 1e3) / 1e9 if cl_ms else None
    count_left = {"kernels": cl_names, "bytes_per_step": cl_bytes, "ms_per_step": round(cl_ms, 4),
                  "achieved": round(cl_gbs, 1) if cl_gbs else None, "peak": peak, "unit": "GB/s",
                  "frac": round(cl_gbs / peak, 4) if cl_gbs else None,
                  "peak_source": f"{peak_kind} hbm_gbs",
                  "timed": f"CUDA events around every count-left launch of {args.steps} steps "
                           "after the headline's timed region (same inputs and tuning)",
                  "bytes": "4 B per key read + 4 B per key compacted (algorithmic, engine counters)",
                  "excluded": "the bisection inside k_subtree (the last levels' bisection and "
                              "partition run fused in one kernel, timed as `subtree`)"
                              if "subtree" in warm else None}
    wsteps = max(args.warmup, 1)
    kernels = {k: {"launches": v["launches"] // wsteps, "ms": round(v["total_ms"] / wsteps, 4),
                   "GBps": round(v["bytes"] / (v["total_ms"] / 1e3) / 1e9, 1) if v["total_ms"] else None}
               for k, v in warm.items()}
    part_ms = sum(warm[k]["total_ms"] for k in PARTITION_KERNELS if k in warm) / wsteps

    # the same step with the optional permutation output (one more array moved per swap); its
    # outputs are the checker's GPU side
    ctx.profile_reset(timing=False)
    step(with_perm=True)
    torch.cuda.synchronize(dev)
    ev0.record()
    for _ in range(args.steps):
        res = step(with_perm=True)
    ev1.record()
    torch.cuda.synchronize(dev)
    perm_ms_step = ev0.elapsed_time(ev1) / args.steps
    gpu_out = (heap_np.copy(), ranges_np.copy(), x.cpu().numpy(), y.cpu().numpy(), z.cpu().numpy(),
               perm.cpu().numpy().view(np.uint32))
    inputs = (x0.cpu().numpy(), y0.cpu().numpy(), z0.cpu().numpy())

    warm_rb = None
    if with_warm:
        # warm-started rebuild (labelled mode, not bit-identical with a cold build): the same
        # particles displaced by sigma = 1e-3 (seeded, clamped to the box), rebuilt cold and
        # from the previous tree's cuts
        prev_heap = gpu_out[0]
        g = torch.Generator(device=dev)
        g.manual_seed(seed + 11)
        hi = float(np.nextafter(np.float32(0.5), np.float32(0)))
        xd, yd, zd = ((a + 1e-3 * torch.randn(n, generator=g, device=dev)).clamp_(-0.5, hi)
                      for a in (x0, y0, z0))
        cold_ms, warm_ms, winfo = [], [], None
        for i in range(args.warmup + args.steps):
            for dst, src in ((x, xd), (y, yd), (z, zd)):
                dst.copy_(src)
            c = ctx.build(x, y, z, d, perm=None, device_pointers=True)
            for dst, src in ((x, xd), (y, yd), (z, zd)):
                dst.copy_(src)
            w = ctx.build_warm(x, y, z, d, prev_heap, WARM_WIDTH, perm=None, device_pointers=True)
            if i >= args.warmup:
                cold_ms.append(c.info["device_ms"])
                warm_ms.append(w.info["device_ms"])
                winfo = w.info
        del xd, yd, zd
        warm_rb = {"workload": f"{workload_name(kind, n, d)}, particles displaced by N(0, 1e-3^2) "
                               "per coordinate",
                   "width": WARM_WIDTH, "cold_build_ms": round(statistics.median(cold_ms), 3),
                   "warm_build_ms": round(statistics.median(warm_ms), 3),
                   "speedup": round(statistics.median(cold_ms) / statistics.median(warm_ms), 3),
                   "warm_cells": winfo["warm_cells"], "warm_resets": winfo["warm_resets"],
                   "note": "labelled mode: a valid ORB tree, not bit-identical with the cold build"}

    # end to end through the C ABI with pinned host buffers (copies inside the timed region)
    hx, hy, hz = (torch.empty(n, dtype=torch.float32, pin_memory=True) for _ in range(3))
    for h, src in ((hx, inputs[0]), (hy, inputs[1]), (hz, inputs[2])):
        h.numpy()[:] = src
    nx, ny, nz = hx.numpy(), hy.numpy(), hz.numpy()
    e2e_times = []
    if clocks_cb:
        clocks_cb("start_e2e")
    for i in range(args.warmup + args.steps):
        for a, s in zip((nx, ny, nz), inputs):
            np.copyto(a, s)
        t = time.perf_counter()
        ctx.build(nx, ny, nz, d, perm=None, heap_out=heap_np, ranges_out=ranges_np)
        if i >= args.warmup:
            e2e_times.append(time.perf_counter() - t)
    # one more build from host memory, outside the timed region, with every kernel timed:
    # the kernels of the staged path (per-coordinate swap instances, the gathers) and the rest
    for a, s_ in zip((nx, ny, nz), inputs):
        np.copyto(a, s_)
    ctx.profile_reset(timing=True)
    eb = ctx.build(nx, ny, nz, d, perm=None, heap_out=heap_np, ranges_out=ranges_np)
    e2e_kernels = {k: {"launches": v["launches"], "ms": round(v["total_ms"], 4),
                       "GBps": round(v["bytes"] / (v["total_ms"] / 1e3) / 1e9, 1) if v["total_ms"] > 0 else None}
                   for k, v in ctx.profile().items()}
    ctx.profile_reset(timing=False)
    e2e_copies = {"h2d_ms": round(eb.info["h2d_ms"], 3), "d2h_ms": round(eb.info["d2h_ms"], 3),
                  "device_ms": round(eb.info["device_ms"], 3)}
    if clocks_cb:
        clocks_cb("end_e2e")
    del hx, hy, hz, nx, ny, nz
    h2d_gbs, d2h_gbs = measure_link(torch, dev, 4 * n)
    heap_bytes = (2 * d - 1) * 52
    h2d_bytes, d2h_bytes = 12 * n, 12 * n + heap_bytes + 8 * (2 * d - 1)
    e2e_ms = 1e3 * sum(e2e_times) / len(e2e_times)
    link_floor_ms = 1e3 * (h2d_bytes / (h2d_gbs * 1e9) + d2h_bytes / (d2h_gbs * 1e9))
    e2e = {"value": n / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d_bytes,
           "d2h_bytes_per_step": d2h_bytes,
           "call": "orb_build(x,y,z host pinned, perm=NULL): reordered x,y,z + heap + ranges back",
           "ms_per_step": e2e_ms,
           "kernels_one_build": e2e_kernels, "copies_one_build": e2e_copies,
           "link_gbs": {"h2d": round(h2d_gbs, 1), "d2h": round(d2h_gbs, 1),
                        "how": "one plain copy of 4n bytes each way between pinned host and HBM, "
                               "CUDA events, same run"},
           "link_floor_ms": round(link_floor_ms, 3),
           "link_frac": round(link_floor_ms / e2e_ms, 4),
           "link_note": "link_floor_ms = the step's bytes in and out at the measured link rates "
                        "back to back; link_frac = that floor / the e2e step (1.0 = link-bound)"}

    del x0, y0, z0, x, y, z, perm
    torch.cuda.empty_cache()
    return {
        "n": n, "d": d, "kind": kind, "ms_total": ms_total, "ms_step": ms_total / args.steps,
        "build_ms_device": statistics.median(i["device_ms"] for i in infos),
        "with_perm_ms_per_step": round(perm_ms_step, 4), "tuning": tuning, "tuned_by": tuned_by,
        "tune_s": round(tune_s, 2), "roofline": roofline, "count_left": count_left,
        "kernels": kernels, "partition_ms_per_step": round(part_ms, 4), "launches": launches,
        "e2e": e2e, "passes": infos[-1]["count_passes"], "warm_rebuild": warm_rb,
        "parity_job": {"x": inputs[0], "y": inputs[1], "z": inputs[2],
                       "instances": [{"offset": 0, "n": n, "d": d, "gpu": gpu_out}]},
    }


# ------------------------------------------------------------------------------------------
# Weighted ORB: integer weights per particle (orb_build_weighted), a labelled mode
# ------------------------------------------------------------------------------------------
def bench_weighted(ctx, E, torch, dev, args, n: int, d: int, seed: int, peak: float):
    import numpy as np

    x0, y0, z0 = (torch.empty(n, dtype=torch.float32, device=dev) for _ in range(3))
    ctx.generate(E.ORB_GEN_PLUMMER, seed, n, x0, y0, z0, device_pointers=True)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    w0 = torch.randint(1, 64, (n,), generator=g, device=dev, dtype=torch.int32)
    x, y, z, w = (torch.empty_like(a) for a in (x0, y0, z0, w0))
    perm = torch.empty(n, dtype=torch.int32, device=dev)

    def step(with_perm=False):
        for dst, src in ((x, x0), (y, y0), (z, z0), (w, w0)):
            dst.copy_(src)
        torch.cuda.synchronize(dev)
        return ctx.build_weighted(x, y, z, w, d, perm=perm if with_perm else None,
                                  device_pointers=True)

    ctx.profile_reset(timing=True)
    for _ in range(max(args.warmup, 1)):
        step()
    prof = ctx.profile()
    ms = []
    for _ in range(args.steps):
        ms.append(step().info["device_ms"])
    res = step(with_perm=True)
    wsteps = max(args.warmup, 1)
    wh = prof.get("count_left_weighted", {"bytes": 0.0, "total_ms": 0.0})
    gbs = wh["bytes"] / (wh["total_ms"] / 1e3) / 1e9 if wh["total_ms"] else None
    gpu = (res.heap.copy(), res.ranges.copy(), x.cpu().numpy(), y.cpu().numpy(), z.cpu().numpy(),
           perm.cpu().numpy().view(np.uint32), w.cpu().numpy().view(np.uint32))
    job = {"x": x0.cpu().numpy(), "y": y0.cpu().numpy(), "z": z0.cpu().numpy(),
           "w": w0.cpu().numpy().view(np.uint32),
           "instances": [{"offset": 0, "n": n, "d": d, "gpu": gpu}]}
    kernels = {k: {"launches": v["launches"] // wsteps, "ms": round(v["total_ms"] / wsteps, 4)}
               for k, v in prof.items()}
    del x0, y0, z0, w0, x, y, z, w, perm
    torch.cuda.empty_cache()
    leaves = res.ranges[d - 1:]
    wp = gpu[6]
    sums = np.array([int(wp[b:e].sum()) for b, e in leaves], dtype=np.float64)
    return {
        "workload": f"{workload_name('plummer', n, d)}, integer weights uniform in 1..63 per particle",
        "build_ms_device": round(statistics.median(ms), 4),
        "particles_per_s": n / (statistics.median(ms) / 1e3),
        "count_left_weighted": {"achieved": round(gbs, 1) if gbs else None, "unit": "GB/s",
                                "frac": round(gbs / peak, 4) if gbs else None,
                                "bytes": "4 B per key and pass, 4 B per weight read (every weight in the first pass, the bracket keys' after it)"},
        "leaf_weight_spread": round(float((sums.max() - sums.min()) / sums.mean()), 5),
        "kernels_per_step_warmup": kernels,
        "note": "labelled mode (the reference never implemented weighted ORB): every level "
                "through the weighted passes, no subtree kernel",
    }, job


# ------------------------------------------------------------------------------------------
# Batched workload: 128 uneven instances, batched build vs one instance at a time
# ------------------------------------------------------------------------------------------
def bench_batched(ctx, E, torch, dev, steps: int, warmup: int, seed: int):
    import numpy as np
    import workloads as W

    specs = W.batched_instances(seed, 128)
    offs, total = [], 0
    for sp in specs:
        offs.append(total)
        total += sp.n
    x0, y0, z0 = (torch.empty(total, dtype=torch.float32, device=dev) for _ in range(3))
    for sp, off in zip(specs, offs):
        kind = E.ORB_GEN_UNIFORM if sp.kind == "uniform" else E.ORB_GEN_PLUMMER
        ctx.generate(kind, sp.seed, sp.n, x0[off:off + sp.n], y0[off:off + sp.n], z0[off:off + sp.n],
                     device_pointers=True)
    x, y, z = (torch.empty_like(x0) for _ in range(3))
    perm = torch.empty(total, dtype=torch.int32, device=dev)
    inst = [{"offset": off, "n": sp.n, "d": sp.d} for sp, off in zip(specs, offs)]
    outs = [(np.zeros(2 * sp.d - 1, E.CELL_DTYPE), np.zeros((2 * sp.d - 1, 2), np.uint32))
            for sp in specs]

    def restore():
        x.copy_(x0)
        y.copy_(y0)
        z.copy_(z0)
        torch.cuda.synchronize(dev)

    def batch_step():
        restore()
        return ctx.build_batch(x, y, z, inst, perm=perm, device_pointers=True)

    def plain_step():
        restore()
        for sp, off, (hp, rp) in zip(specs, offs, outs):
            sl = slice(off, off + sp.n)
            ctx.build(x[sl], y[sl], z[sl], sp.d, perm=perm[sl], device_pointers=True,
                      heap_out=hp, ranges_out=rp)

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        for _ in range(steps):
            r = fn()
        torch.cuda.synchronize(dev)
        return (time.perf_counter() - t) / steps, r

    ctx.profile_reset(timing=False)
    # launch parameters chosen by the engine's autotuner on this batch (every candidate's
    # trees checked equal); both forms below run under the chosen setting
    default_tuning = ctx.get_tuning()
    t0 = time.perf_counter()
    tuning, tuned_ms = ctx.autotune_batch(x0, y0, z0, inst, reps=3, device_pointers=True)
    tune_s = time.perf_counter() - t0
    t_batch, (parts, _, binfo) = timed(batch_step)
    bperm = perm.cpu().numpy().view(np.uint32)
    bx, by, bz = x.cpu().numpy(), y.cpu().numpy(), z.cpu().numpy()
    t_plain, _ = timed(plain_step)
    pperm = perm.cpu().numpy().view(np.uint32)
    same = all(hb.tobytes() == hp.tobytes() and np.array_equal(rb, rp)
               for (hb, rb), (hp, rp) in zip(parts, outs)) and np.array_equal(bperm, pperm)
    job_inst = []
    for (hb, rb), ins in zip(parts, inst):
        a, b = ins["offset"], ins["offset"] + ins["n"]
        job_inst.append({**ins, "gpu": (hb.copy(), rb.copy(), bx[a:b], by[a:b], bz[a:b], bperm[a:b])})
    job = {"x": x0.cpu().numpy(), "y": y0.cpu().numpy(), "z": z0.cpu().numpy(), "instances": job_inst}
    del x0, y0, z0, x, y, z, perm
    torch.cuda.empty_cache()
    return {
        "workload": "128 instances, particles log-uniform 2^14..2^22, leaves 2^6..2^12, "
                    "half uniform / half Plummer (seeded)",
        "particles": total, "instances": len(specs),
        "instances_per_s": len(specs) / t_batch,
        "plain_instances_per_s": len(specs) / t_plain,
        "speedup_vs_plain": t_plain / t_batch,
        "ms_per_batch": 1e3 * t_batch, "ms_plain_one_at_a_time": 1e3 * t_plain,
        "particles_per_s": total / t_batch,
        "bit_exact_vs_plain": bool(same),
        "autotune": {"chosen": tuning, "default": default_tuning,
                     "median_build_ms": round(tuned_ms, 3), "tuning_s": round(tune_s, 2)},
        "design": "each level's kernel sequence runs once over the cells of every instance "
                  "(one launch per kernel kind and level for the whole batch), all levels "
                  "captured in one CUDA graph",
    }, job


# ------------------------------------------------------------------------------------------
# Served workload: Poisson request stream, continuous batching vs one request at a time
# ------------------------------------------------------------------------------------------
def run_server_stream(E, device, reqs, budget, max_batch, lanes, paced=True):
    """Submits `reqs` at their arrival times (or all at once when paced=False); returns the
    per-request results and the server stats."""
    with E.Server(device, hbm_budget_bytes=budget, max_batch=max_batch, lanes=lanes) as sv:
        # warm-up: every lane allocates its build scratch once
        warm = [sv.submit_generate(E.ORB_GEN_UNIFORM, 1, 1 << 16, 64) for _ in range(2 * lanes)]
        for w in warm:
            sv.wait(w)
        for w in warm:
            sv.release(w)
        inst, rids = {}, []
        t0 = time.perf_counter()
        for i, r in enumerate(reqs):
            delay = t0 + r.t - time.perf_counter()
            if paced and delay > 0:
                time.sleep(delay)
            if r.kind == "build":
                kind = E.ORB_GEN_UNIFORM if r.spec.kind == "uniform" else E.ORB_GEN_PLUMMER
                rid = sv.submit_generate(kind, r.spec.seed, r.spec.n, r.spec.d)
                inst[i] = rid
            else:
                rid = sv.submit_rebalance(inst[r.target], r.seed, 1e-3)
            rids.append(rid)
        res = [sv.wait(rid) for rid in rids]
        stats = sv.stats()
    return res, stats


def bench_served(E, device, seed: int, rate: float = 2000.0, count: int = 2000):
    import workloads as W

    reqs = W.served_stream(seed, rate, count, rebalance_frac=0.5, sizes=(14, 22))
    budget = 96 << 30

    def summarize(res, stats):
        lat = sorted(r["done_s"] - r["submit_s"] for r in res)
        span = max(r["done_s"] for r in res) - min(r["submit_s"] for r in res)
        ok = all(r["status"] == 0 for r in res)
        return {"instances_per_s": len(res) / span, "p50_ms": 1e3 * lat[len(lat) // 2],
                "p99_ms": 1e3 * lat[min(len(lat) - 1, int(0.99 * len(lat)))],
                "batches": stats["batches"], "mean_batch": len(res) / max(stats["batches"], 1),
                "max_batch": stats["max_batch_seen"], "all_ok": ok}

    cb = summarize(*run_server_stream(E, device, reqs, budget, 0, 2))
    one = summarize(*run_server_stream(E, device, reqs, budget, 1, 1))
    # capacity: the same requests submitted all at once
    cb_sat = summarize(*run_server_stream(E, device, reqs, budget, 0, 2, paced=False))
    one_sat = summarize(*run_server_stream(E, device, reqs, budget, 1, 1, paced=False))
    return {
        "workload": f"Poisson arrivals at {rate:.0f} req/s, {count} requests, half new instances "
                    "(particles log-uniform 2^14..2^22, leaves 2^6..2^12, half uniform / half "
                    "Plummer, generated on the device) and half rebalances (sigma=1e-3) of "
                    "resident instances",
        "paced": {"continuous_batching": cb, "one_at_a_time": one,
                  "speedup_instances_per_s": cb["instances_per_s"] / one["instances_per_s"],
                  "note": "continuous batching keeps up with the arrival rate, which caps it"},
        "saturated": {"continuous_batching": cb_sat, "one_at_a_time": one_sat,
                      "speedup_instances_per_s": cb_sat["instances_per_s"] / one_sat["instances_per_s"]},
    }


# ------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------
def _section(r: dict, parity=None) -> dict:
    """The per-workload keys of a run_plain result (clustered section)."""
    return {"workload": workload_name(r["kind"], r["n"], r["d"]), "particles": r["n"],
            "leaves": r["d"], "ms_per_step": round(r["ms_step"], 4),
            "build_ms_device": round(r["build_ms_device"], 4),
            "particles_per_s": r["n"] / (r["ms_step"] / 1e3),
            "e2e": r["e2e"], "roofline": r["roofline"], "count_left": r["count_left"],
            "partition_ms_per_step": r["partition_ms_per_step"],
            "kernels_per_step_warmup": r["kernels"], "tuning": r["tuning"],
            "with_perm_ms_per_step": r["with_perm_ms_per_step"], "parity": parity}


def gpu_arm(args):
    import torch

    import orb_gb300 as E
    import replicas

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    E.build()
    n, d = args.particles, args.leaves
    ctx = E.Context(local, reserve_particles=n, reserve_leaves=d)
    dev = torch.device("cuda", local)
    peak, peak_kind = measured_peak()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    clocks = ClockSampler(gpu_id_for(local))
    marks = {}

    def mark(what):
        if what == "start":
            barrier()
        marks[what] = time.perf_counter()

    time.sleep(0.5)
    head = run_plain(ctx, E, torch, dev, args, "uniform", n, d, SEED + rank, peak, peak_kind,
                     args.tuning, clocks_cb=mark, with_warm=(rank == 0 and not args.no_warm))
    ms_total, _, value = replicas.whole_job(head["ms_total"], n * args.steps)
    ms_step = ms_total / args.steps
    e2e_ms, _, e2e_value = replicas.whole_job(head["e2e"]["ms_per_step"], n)
    head["e2e"]["value"] = e2e_value
    clock_summary = clocks.summary(marks["start"], marks["end_e2e"])
    clocks.stop()

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0

    clustered = None
    jobs = {"headline": head.pop("parity_job")}
    if not args.no_clustered:
        cn, cd = CLUSTERED
        cl = run_plain(ctx, E, torch, dev, args, "plummer", cn, cd, SEED + 33, peak, peak_kind, None)
        jobs["clustered"] = cl.pop("parity_job")
        clustered = cl
    weighted = None
    if not args.no_weighted:
        weighted, jobs["weighted"] = bench_weighted(ctx, E, torch, dev, args, *WEIGHTED, SEED + 55, peak)
    batched = None
    if not args.no_batched:
        batched, jobs["batched"] = bench_batched(ctx, E, torch, dev, max(2, min(args.steps, 5)), 1,
                                                 SEED + 77)
    ctx.close()
    served = None
    if not args.no_served:
        torch.cuda.empty_cache()
        served = bench_served(E, local, SEED + 99)

    # CPU leg: the checker on the benchmark's own inputs, then the timed CPU baseline
    parity = {}
    cpu = None
    if not args.no_cpu_baseline:
        for name, job in jobs.items():
            parity[name] = check_parity(job)
        jobs.clear()
        cpu = run_cpu(N_PARTICLES, LEAVES, 1, 0, budget_s=40.0)
        cpu = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    effective_count_left(head["count_left"], head["kernels"], parity.get("headline"), peak)
    if clustered is not None:
        effective_count_left(clustered["count_left"], clustered["kernels"], parity.get("clustered"), peak)
        clustered = _section(clustered, parity.get("clustered"))
    if batched is not None:
        batched["parity"] = parity.get("batched")
    if weighted is not None:
        weighted["parity"] = parity.get("weighted")

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded uniform, engine generator)",
        "config": workload_config(n, d, world),
        "step": {"what": "d2d restore of x,y,z + orb_build (device pointers)",
                 "outputs": "reordered x,y,z + cell heap + range map (as the reference; the "
                            "optional permutation is off, timed separately as with_perm)"},
        "parity": parity.get("headline"),
        "build_ms_device": head["build_ms_device"],
        "tuning": {"chosen": head["tuning"], "by": head["tuned_by"], "tuning_s": head["tune_s"]},
        "with_perm_ms_per_step": head["with_perm_ms_per_step"],
        "warm_rebuild": head["warm_rebuild"],
        "e2e": head["e2e"],
        "roofline": head["roofline"],
        "count_left": head["count_left"],
        "partition_ms_per_step": head["partition_ms_per_step"],
        "kernels_per_step_warmup": head["kernels"],
        "gpu_launches": head["launches"],
        "cpu_baseline": cpu,
        "clustered": clustered,
        "weighted": weighted,
        "batched": batched,
        "served": served,
        "clocks": clock_summary,
        "bisection_passes_per_build": head["passes"],
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--particles", type=int, default=N_PARTICLES)
    ap.add_argument("--leaves", type=int, default=LEAVES)
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the CPU leg (timed baseline and the oracle's parity check)")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-clustered", action="store_true")
    ap.add_argument("--no-warm", action="store_true")
    ap.add_argument("--no-weighted", action="store_true")
    ap.add_argument("--tuning", default=None,
                    help="hist,part,tile,sparse,cta,subtree[,predict]: use this launch tuning for the headline "
                         "instead of autotuning it (profiling runs reuse a chosen setting)")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
