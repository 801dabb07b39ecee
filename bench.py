#!/usr/bin/env python
"""Benchmark of the GB300 PBF timestep (particle-steps/s on the 1M scene).

Workload: the 1,000,000-particle falling block (100^3 lattice, spacing 0.02,
h = 0.04, 8x4x4 box, s_corr + XSPH + vorticity, 4 Jacobi iterations),
synthetic and seeded. One timed step = one full PBF timestep over that
scene's initial batch: before every step the initial state is restored
device-to-device (outside the timed region), so every step does the same
work (the lattice phase, ~28 neighbours per particle). The reference's own
run of this scene collapses to ~10^4 neighbours per particle within ~30
steps; `trajectory` reports that regime separately: step times and the
HBM fraction of steps 1-5 (the lattice, collapsing from step 2 on) and of
the last 5, and neighbour-count histograms at steps 1, 5 and the last.

  value   particle-steps/s, inputs resident in HBM, L2 flushed between steps,
          per-step CUDA events on the solver's stream, max over ranks.
  e2e     the same metric through the reference-facing call
          fluid_gb300_cuda_step (host SoA arrays in pinned memory copied in,
          stepped, copied out every step), host wall clock.
  roofline / pair_roofline  the dominant kernel against HBM bandwidth and
          against the FP32 issue rate, from per-launch CUDA events.
  cpu_baseline  the oracle (a CPU restatement of the reference step) on the
          host cores on a bounded sample, rank 0 at N = 1.
  parity_step1  that sample's first step on the GPU against the oracle
          (untimed): per-particle neighbour counts and their histogram,
          positions and velocities, bit for bit.
  configs c1 (4,096-particle dam break, all 240 steps) and c2 (250k double
          dam break, until its lists pass --c2-pair-budget entries) from
          their initial states with autotuned shapes (c1 also with the
          defaults); the oracle on the host over all of c1 and a prefix of
          c2, the states compared bit for bit.
  collapsed  one collapsed-phase step (the 125k falling block at step 21),
          the GPU (autotuned on that state, and default shapes) and the
          oracle from the same state.
  batched 64 scenes in one solver against 64 solvers stepped in turn.
  differentiable  the 60-step adjoint scene: forward and forward + adjoint
          times and gradient norms (FP64 checks in the CPU leg).
  output  one step plus one frame written per iteration at 1M, the
          reference's ASCII writer against the asynchronous binary one.

`--impl reference` times the reference's CPU step (the oracle restatement;
the reference binary is not buildable on the GPU host) on the host cores.
Multi-GPU (torchrun): independent replicas, one per rank, no collective on
the data path; scaling "weak".
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

N_SIDE = 100
METRIC = "particle-steps/s @1M"
# The workload both arms name in `config` (the reference arm times the same
# step on the host cores, on as many of the scene's particles as its budget
# allows; `particles` says how many).
WORKLOAD = ("falling_block_1M: 100^3 lattice, sp 0.02, h 0.04, 8x4x4 box, s_corr+XSPH+vorticity, "
            "4 iterations, one step over the initial batch per timed step")
UNIT = "particle-steps/s"

# Algorithmic bytes per particle per launch (compulsory per-particle array
# traffic; vec3 = 12 B, scalar / index = 4 B; neighbour gathers on chip).
ALGO_BYTES_PER_PARTICLE = {
    "k_bounds": 24,        # R x 12, v 12
    "k_keys": 28,          # R x 12, v 12; W key 4
    "k_reorder": 76,       # R key 4, index 4, slot 4, x 12, v 12; W x 12, v 12, p* 12, slot 4
    "k_nbr_build": 16,     # R p* 12; W count 4 (lists excluded)
    "k_lambda": 20,        # R p* 12; W lambda 4, rho 4
    "k_delta": 28,         # R p* 12, lambda 4; W p* 12
    "k_xsph": 40,          # R x 12, v 12, rho 4; W v 12
    "k_omega": 40,         # R x 12, v 12; W omega + |omega| 16
    "k_eta": 52,           # R x 12, omega 16, v 12; W v 12
}
# Per step, all three flags and 4 iterations (predict 44, sort 16, reorder 56,
# 4 x (lambda 16 + delta 28) + rho 4, commit + XSPH 52, omega 40, eta 52,
# permutation 12).
ALGO_BYTES_PER_STEP = 452
# FP32 operations per neighbour pair in k_delta (s_corr on): difference 3,
# r^2 5, sqrt 1, spiky factor 3, lambda sum 1, s_corr 9, accumulate 7.
DELTA_OPS_PER_PAIR = 29
FP32_LANES_PER_SM = 128
# Bin edges of the per-step neighbour-count histograms: [0, 8), [8, 16),
# [16, 32), ... [16384, 32768), [32768, inf). The lattice phase fills the
# bins below 64; the collapsed phase spreads over the thousands.
HIST_EDGES = [0, 8] + [16 << k for k in range(12)]


def neighbor_histogram(counts):
    """Particles per bin of HIST_EDGES (the last bin is open-ended)."""
    import numpy as np

    idx = np.searchsorted(np.asarray(HIST_EDGES), np.asarray(counts), side="right") - 1
    return np.bincount(idx, minlength=len(HIST_EDGES)).tolist()


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def profile_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summaries."""
    import glob
    import re

    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        with open(path) as f:
            for line in f:
                m = re.match(r"^traffic_bytes_per_launch\s+(\S+)\s+(\d+)", line)
                if m and m.group(1) == kernel:
                    return int(m.group(2))
    return None


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured", d
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback", {}


# --------------------------------------------------------------------------
# distributed helpers (replicas only)

def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(value: float, world: int, device=None) -> float:
    """Max over ranks (no-op at world size 1)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


# --------------------------------------------------------------------------
# clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------
# our arm

def run_ours(args, world, rank, local):
    import numpy as np
    import torch

    from fluidsimulator_gb300 import _capi, scenes
    from fluidsimulator_gb300 import build as lib_build
    from fluidsimulator_gb300.solver import Solver, cuda_step

    lib_build.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    stream = torch.cuda.Stream(dev)  # a real stream: the legacy NULL stream would not order with the solver
    torch.cuda.set_stream(stream)

    sc = scenes.falling_block(args.side, seed=0)
    n = sc.count
    pos0 = torch.from_numpy(sc.pos).to(dev)
    vel0 = torch.from_numpy(sc.vel).to(dev)
    l2_flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2
    torch.cuda.synchronize(dev)

    solver = Solver(local)
    solver.configure([sc.params], [n])
    solver.set_stream(stream.cuda_stream)
    solver.set_graphs(True)

    def restore():
        solver.upload(pos0, vel0)

    # warm-up (also sizes the neighbour lists and captures the graphs), then
    # the autotuner picks each kernel's launch shape on this state
    for _ in range(args.warmup):
        restore()
        solver.step(1)
    tuning = None
    if not args.no_autotune:
        restore()
        tuning = solver.autotune(2)
        for _ in range(args.warmup):
            restore()
            solver.step(1)
    sort_bits = solver.sort_bits()
    # The timed steps carry no per-kernel events (recorded between every two
    # kernels they cost ~0.1 ms per step); a second pass over the same K
    # steps records them for the per-kernel times and the rooflines.
    solver.set_profiling(False)
    launches0 = solver.stats()["kernel_launches"]
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)

    def timed_steps():
        ms = []
        for _ in range(args.steps):
            restore()
            l2_flush.zero_()
            ev0.record(stream)
            solver.step_async(1)
            ev1.record(stream)
            solver.synchronize()
            ms.append(ev0.elapsed_time(ev1))
        return ms

    barrier(world)
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(local)
    clocks.start()
    step_ms = timed_steps()
    torch.cuda.synchronize(dev)
    barrier(world)
    clk = clocks.stop()
    stats = solver.stats()
    launches = stats["kernel_launches"] - launches0
    total_ms = reduce_max(sum(step_ms), world, dev)
    value = world * n * args.steps / (total_ms / 1e3)
    solver.set_profiling(True)
    solver.kernel_times(reset=True)
    instrumented_ms = statistics.mean(timed_steps())
    stage = solver.kernel_times(reset=True)
    solver.set_profiling(False)

    # dominant kernel and its rooflines
    peak_gbs, peak_kind, peaks = measured_peaks()
    dom = max(stage, key=lambda k: stage[k][0])
    dom_ms, dom_launches = stage[dom]
    avg_ms = dom_ms / max(dom_launches, 1)
    roofline = None
    if dom in ALGO_BYTES_PER_PARTICLE and dom_launches:
        bytes_per_launch = ALGO_BYTES_PER_PARTICLE[dom] * n
        achieved = bytes_per_launch / (avg_ms / 1e3) / 1e9
        roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 2), "peak": peak_gbs,
                    "unit": "GB/s", "frac": round(achieved / peak_gbs, 5),
                    "traffic": args.traffic if args.traffic is not None else profile_traffic(dom),
                    "bytes_per_launch": bytes_per_launch, "avg_launch_ms": round(avg_ms, 4),
                    "launches": dom_launches, "share": round(dom_ms / max(sum(v[0] for v in stage.values()), 1e-9), 3),
                    "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured" else "fallback"}
    pair_roofline = None
    sm_mhz = clk["sm_mhz"] if clk else None
    if stage["k_delta"][1]:
        pairs = stats["neighbor_pairs"]
        d_ms = stage["k_delta"][0] / stage["k_delta"][1]
        props = torch.cuda.get_device_properties(dev)
        max_mhz = (clk or {}).get("sm_max_mhz") or float(peaks.get("sm_max_mhz", 2070.0))
        peak_ops = props.multi_processor_count * FP32_LANES_PER_SM * max_mhz * 1e6
        ops = pairs * DELTA_OPS_PER_PAIR / (d_ms / 1e3)
        pair_roofline = {"bound": "fp32_issue", "kernel": "k_delta", "pairs_per_launch": pairs,
                         "ops_per_pair": DELTA_OPS_PER_PAIR, "achieved": round(ops / 1e12, 3),
                         "peak": round(peak_ops / 1e12, 2), "unit": "TFLOP/s (non-FMA FP32)",
                         "frac": round(ops / peak_ops, 4), "avg_launch_ms": round(d_ms, 4)}
    step_frac = ALGO_BYTES_PER_STEP * n / (statistics.mean(step_ms) / 1e3) / 1e9 / peak_gbs

    # e2e through the reference-facing call, host arrays in pinned memory
    e2e = None
    if not args.no_e2e:
        hp = torch.empty((3, n), dtype=torch.float32, pin_memory=True)
        hv = torch.empty((3, n), dtype=torch.float32, pin_memory=True)
        hpn, hvn = hp.numpy(), hv.numpy()
        torch.cuda.set_device(local)
        for _ in range(args.warmup):
            np.copyto(hpn, sc.pos)
            np.copyto(hvn, sc.vel)
            cuda_step(sc.params, hpn, hvn, 0.0)
        e2e_s = []
        for _ in range(args.steps):
            np.copyto(hpn, sc.pos)
            np.copyto(hvn, sc.vel)
            l2_flush.zero_()
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            cuda_step(sc.params, hpn, hvn, 0.0)
            e2e_s.append(time.perf_counter() - t0)
        e2e_total = reduce_max(sum(e2e_s), world, dev)
        e2e = {"value": round(world * n * args.steps / e2e_total, 1), "unit": UNIT,
               "h2d_bytes_per_step": 24 * n, "d2h_bytes_per_step": 24 * n,
               "ms_per_step": round(1e3 * e2e_total / args.steps, 4),
               "call": "fluid_gb300_cuda_step (fluid::cuda_step semantics)"}

    # the real trajectory: lattice phase and collapse
    traj = None
    if args.trajectory > 0:
        restore()
        solver.set_profiling(True)  # per-kernel totals; ~0.1 ms a step against 10-200 ms steps
        solver.kernel_times(reset=True)
        t_ms, t_pairs, hists = [], [], {}
        hist_steps = {1, min(5, args.trajectory), args.trajectory}
        for k in range(1, args.trajectory + 1):
            ev0.record(stream)
            solver.step(1)
            ev1.record(stream)
            ev1.synchronize()
            t_ms.append(ev0.elapsed_time(ev1))
            t_pairs.append(solver.stats()["neighbor_pairs"])
            if k in hist_steps:  # outside the events; the step has completed
                hists[f"step{k}"] = neighbor_histogram(solver.read_debug(_capi.DEBUG_NEIGHBOR_COUNTS))
        st = solver.stats()
        first5, last5 = statistics.mean(t_ms[:5]), statistics.mean(t_ms[-5:])
        peak_gbs = measured_peaks()[0]
        traj = {"steps": args.trajectory, "ms_per_step_first5": round(first5, 3),
                "ms_per_step_last5": round(last5, 3),
                "hbm_frac_first5": round(ALGO_BYTES_PER_STEP * n / (first5 / 1e3) / 1e9 / peak_gbs, 5),
                "hbm_frac_last5": round(ALGO_BYTES_PER_STEP * n / (last5 / 1e3) / 1e9 / peak_gbs, 7),
                "neighbors_per_particle_step1": round(t_pairs[0] / n, 2),
                "neighbors_per_particle_last": round(t_pairs[-1] / n, 2), "neighbor_max_last": st["neighbor_max"],
                "neighbor_histogram": {"edges": HIST_EDGES, **hists},
                "particle_steps_per_s": round(n * len(t_ms) / (sum(t_ms) / 1e3), 1),
                "regrows": st["regrows"]}
        tail = solver.kernel_times(reset=True)
        traj["kernel_ms_total"] = {k: round(v[0], 2) for k, v in tail.items() if v[1]}
    solver.close()

    output = None
    if not args.no_output and rank == 0:
        output = run_output(sc, dev, stream, args)
    batched = None
    if not args.no_batched:
        batched = run_batched(args, dev, stream, l2_flush)
    differentiable = None
    if not args.no_adjoint:
        differentiable = run_differentiable(args, dev, stream)
    configs = collapsed = None
    if not args.no_configs:
        configs = run_configs(args, dev, stream)
        collapsed = run_collapsed(args, dev, stream)

    cpu = parity = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, parity = cpu_baseline(sc, budget_s=args.cpu_budget)
        if configs:
            cpu_configs(configs, args)
        if collapsed:
            cpu_collapsed(collapsed)
        if differentiable:
            differentiable["fp64_checks"] = gradient_checks(args)

    for part in (configs or {}).values():  # the CPU legs' inputs, left when they did not run
        for k in [k for k in part if k.startswith("_")]:
            part.pop(k)
    if collapsed:
        collapsed.pop("_state", None)
    out = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "particles": n, "neighbors_per_particle": round(stats["neighbor_pairs"] / n, 2),
                   "l2": "flushed (256 MB write) between timed steps", "parallelism": f"replicas x{world}",
                   "graphs": True, "exact_fp32": True,
                   "tuning": ({k: [v["unroll"], v["block"], v.get("lanes", 1)] for k, v in tuning.items()}
                              if tuning else "default"),
                   "sort_bits": sort_bits,
                   "kernel_timing": "per-kernel CUDA events in a second pass over the same steps (the timed pass "
                                    "has none); that pass's step time is ms_per_step_instrumented"},
        "ms_per_step_instrumented": round(instrumented_ms, 4),
        "roofline": roofline, "pair_roofline": pair_roofline,
        "step_roofline": {"bytes_per_particle_step": ALGO_BYTES_PER_STEP, "frac": round(step_frac, 5)},
        "kernel_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in stage.items() if v[1]},
        "cpu_baseline": cpu, "parity_step1": parity, "e2e": e2e, "clocks": clk, "gpu_launches": launches,
        "trajectory": traj, "configs": configs, "collapsed": collapsed,
        "batched": batched, "differentiable": differentiable, "output": output,
    }
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(_finite(out)), flush=True)


def _gpu_run(sc, steps, dev, stream, pair_budget=None, tune=False):
    """Runs up to `steps` steps of a scene from its initial state on a fresh
    solver (graphs on; shapes from fluid_solver_autotune on the initial state
    when `tune`, else the defaults), each step bracketed by CUDA events on the
    solver's stream; stops early once a step's lists hold more than
    `pair_budget` entries (the next steps of a collapse grow them further). A
    step that outgrows the list or grid capacity is re-run by synchronize()
    after a regrow, behind the closing event: such a step is timed to a third
    event recorded after synchronize() returns (its host turnaround
    included). Returns per-step ms, neighbours per particle per step, the
    final state, the stats and the shapes used."""
    import torch

    from fluidsimulator_gb300.solver import Solver

    s = Solver(dev.index)
    s.configure([sc.params], [sc.count])
    s.set_stream(stream.cuda_stream)
    s.upload(sc.pos, sc.vel)
    shapes = None
    if tune:
        tuned = s.autotune()
        shapes = {"sort_bits": s.sort_bits(),
                  **{k: [v["unroll"], v["block"], v["lanes"]] for k, v in tuned.items()}}
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ms, nbr = [], []
    regrows = s.stats()["regrows"]
    for _ in range(steps):
        ev[0].record(stream)
        s.step_async(1)
        ev[1].record(stream)
        s.synchronize()
        st = s.stats()
        if st["regrows"] != regrows:
            regrows = st["regrows"]
            ev[2].record(stream)
            ev[2].synchronize()
            ms.append(ev[0].elapsed_time(ev[2]))
        else:
            ms.append(ev[0].elapsed_time(ev[1]))
        pairs = st["neighbor_pairs"]
        nbr.append(pairs / sc.count)
        if pair_budget and pairs > pair_budget:
            break
    pos, vel = s.download()
    st = s.stats()
    s.close()
    return ms, nbr, pos, vel, st, shapes


def run_configs(args, dev, stream):
    """The two single-scene configurations besides the 1M throughput scene,
    each run over its full length on the GPU: c1, the plain dam break (4,096
    particles, 16^3 lattice, spacing 0.05, h 0.1, flags off, 240 steps), and
    c2, the double dam break (two 50^3 blocks, 250,000 particles, spacing
    0.025, h 0.05, all three flags, 480 steps). Both run with the shapes the
    autotuner picks on the initial state; c1 is also run with the default
    shapes. c2 collapses completely (with m = rho0 sp^3 the Jacobi update
    scales by 1/m = 64): each block's particles end up within h of nearly all
    others, ~125,000 neighbours each, so its lists would grow past 87e9
    entries (~350 GB, the reference's CSR alike). Its GPU run stops once a
    step's lists pass `--c2-pair-budget` entries and reports the steps it
    covered. The CPU side (cpu_configs) times the oracle over the whole of c1
    and a stated prefix of c2 on the host cores and checks the GPU's state
    after that prefix bit for bit."""
    from fluidsimulator_gb300 import scenes

    def summary(ms, nbr, st):
        ran, total = len(ms), sum(ms)
        return {"ms_total": round(total, 3), "ms_per_step": round(total / ran, 4),
                "particle_steps_per_s": round(sc.count * ran / (total / 1e3), 1),
                "ms_per_step_first5": round(statistics.mean(ms[:5]), 4),
                "ms_per_step_last5": round(statistics.mean(ms[-5:]), 4),
                "neighbors_per_particle_step1": round(nbr[0], 2),
                "neighbors_per_particle_last": round(nbr[-1], 2), "neighbor_max_last": st["neighbor_max"],
                "regrows": st["regrows"]}

    out = {}
    for key, sc, steps, budget, default_too in (
            ("c1_dam_break_4096", scenes.dam_break(16, seed=0), args.c1_steps, None, True),
            ("c2_double_dam_break_250k", scenes.double_dam_break(50, seed=0), args.c2_steps, args.c2_pair_budget,
             False)):
        if steps <= 0:
            continue
        _gpu_run(sc, min(steps, 3), dev, stream)  # warm-up: kernels loaded, graphs captured once
        ms, nbr, pos, vel, st, shapes = _gpu_run(sc, steps, dev, stream, budget, tune=True)
        ran = len(ms)
        out[key] = {"particles": sc.count, "steps": ran, "steps_of_config": steps,
                    "gpu": {**summary(ms, nbr, st), "shapes": shapes,
                            "timing": "per-step CUDA events on the solver's stream (a step re-run after a regrow "
                                      "timed to an event after synchronize), graphs on, autotuned shapes, whole "
                                      "run from the initial state"},
                    "_scene": sc, "_ms": ms}
        if default_too:
            dms, dnbr, _, _, dst, _ = _gpu_run(sc, steps, dev, stream, budget)
            out[key]["gpu_default_shapes"] = summary(dms, dnbr, dst)
        if ran < steps:
            out[key]["stopped"] = (f"after step {ran}: {nbr[-1]:.0f} neighbours per particle, lists past the "
                                   f"{budget:.3g}-entry budget (a complete collapse needs ~87e9)")
    return out


def run_collapsed(args, dev, stream):
    """One step of the collapsed phase on the GPU, for a CPU comparison on the
    same state: the 125,000-particle falling block (50^3, the 1M scene's
    spacing, h and flags) stepped `collapsed_at - 1` steps on the GPU, its
    state downloaded, then step `collapsed_at` timed from that state (re-
    uploaded before each of a few repetitions; median), first with the default
    shapes, then with the shapes fluid_solver_autotune picks on that state."""
    import numpy as np
    import torch

    from fluidsimulator_gb300 import scenes
    from fluidsimulator_gb300.solver import Solver

    if args.collapsed_at <= 1:
        return None
    sc = scenes.falling_block(args.collapsed_side, seed=0)
    s = Solver(dev.index)
    s.configure([sc.params], [sc.count])
    s.set_stream(stream.cuda_stream)
    s.upload(sc.pos, sc.vel)
    s.step(args.collapsed_at - 1)
    pos, vel = s.download()
    t0 = s.time()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def one_step_ms():
        ms = []
        for _ in range(4):
            s.upload(pos, vel)
            s.set_time(t0)
            ev[0].record(stream)
            s.step_async(1)
            ev[1].record(stream)
            s.synchronize()
            ms.append(ev[0].elapsed_time(ev[1]))
        return statistics.median(ms[1:])

    dms = one_step_ms()
    st = s.stats()
    after = s.download()
    s.upload(pos, vel)
    s.set_time(t0)
    tuned = s.autotune()
    shapes = {"sort_bits": s.sort_bits(), **{k: [v["unroll"], v["block"], v["lanes"]] for k, v in tuned.items()}}
    gms = one_step_ms()
    after_tuned = s.download()
    s.close()
    timing = "CUDA events around one step from the uploaded state; median of 3 after one warm-up"
    return {"scene": f"falling_block_{sc.count}", "particles": sc.count, "step": args.collapsed_at,
            "neighbors_per_particle": round(st["neighbor_pairs"] / sc.count, 2), "neighbor_max": st["neighbor_max"],
            "gpu": {"ms_per_step": round(gms, 4), "particle_steps_per_s": round(sc.count / (gms / 1e3), 1),
                    "shapes": shapes, "timing": timing + ", shapes autotuned on this state"},
            "gpu_default_shapes": {"ms_per_step": round(dms, 4),
                                   "particle_steps_per_s": round(sc.count / (dms / 1e3), 1), "timing": timing},
            "tuned_equals_default": bool(np.array_equal(after[0], after_tuned[0])
                                         and np.array_equal(after[1], after_tuned[1])),
            "_state": (sc, pos, vel, t0, after)}


def run_differentiable(args, dev, stream):
    """Differentiable PBF: 32^3 block (32,768 particles), XSPH c = 0.01 and
    s_corr on, initial velocity N(0, 0.1^2), 60 steps, loss |COM - (1.5, 0.3,
    1.0)|^2. Times the forward run and forward + adjoint (checkpoints every 10
    steps, recomputation in between) and reports the gradient's size per
    horizon. The checks of these gradients against the oracle (its FP64
    adjoint, central differences of its FP64 forward) run in the CPU leg
    (gradient_checks) and in tests/test_adjoint.py."""
    import numpy as np
    import torch

    from fluidsimulator_gb300 import scenes
    from fluidsimulator_gb300.solver import Solver

    sc = scenes.differentiable_block(32, seed=0)
    n = sc.count
    steps, every = args.adj_steps, 10
    target = np.array([1.5, 0.3, 1.0])
    s = Solver(dev.index)
    s.configure([sc.params], [n])
    s.set_stream(stream.cuda_stream)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)

    def grad(horizon):
        s.upload(sc.pos, sc.vel)
        s.record(horizon, every)
        x, _ = s.download()
        com = x.astype(np.float64).mean(axis=1)
        gxf = np.repeat((2.0 * (com - target) / n)[:, None], n, axis=1).astype(np.float32)
        return s.backward(gxf, np.zeros((3, n), np.float32))

    # timing: forward run vs forward + adjoint
    for _ in range(max(1, args.warmup)):
        s.upload(sc.pos, sc.vel)
        s.step(steps)
        grad(steps)
    fwd, both = [], []
    for _ in range(3):
        s.upload(sc.pos, sc.vel)
        torch.cuda.synchronize(dev)
        ev0.record(stream)
        s.step_async(steps)
        ev1.record(stream)
        s.synchronize()
        fwd.append(ev0.elapsed_time(ev1))
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        grad(steps)
        both.append(1e3 * (time.perf_counter() - t0))
    fwd_ms, both_ms = statistics.median(fwd), statistics.median(both)

    out = {"particles": n, "steps": steps, "checkpoint_every": every,
           "forward_ms": round(fwd_ms, 3), "forward_adjoint_ms": round(both_ms, 3),
           "adjoint_cost_ratio": round(both_ms / fwd_ms, 3),
           "timing": "forward: CUDA events around the 60 steps; forward+adjoint: host wall clock around record(60, 10) "
                     "+ final-state read + backward"}

    def norms(scene):
        """|dL/dv0| and dL/dc of the GPU adjoint per horizon (null where the
        FP32 gradient overflows)."""
        res = {}
        for horizon in sorted({1, 5, 10, 20, steps}):
            s.set_params([scene.params])
            s.upload(scene.pos, scene.vel)
            s.record(horizon, every)
            x, _ = s.download()
            com = x.astype(np.float64).mean(axis=1)
            gxf = np.repeat((2.0 * (com - target) / n)[:, None], n, axis=1).astype(np.float32)
            _, gv0, gc = s.backward(gxf, np.zeros((3, n), np.float32))
            res[str(horizon)] = {"grad_v0_norm": float(np.linalg.norm(gv0.astype(np.float64))),
                                 "dL_dc": float(gc[0])}
        s.set_params([sc.params])
        return res

    out["gradient_norms"] = {"as_specified": norms(sc),
                             "unit_mass": norms(scenes.differentiable_block(32, seed=0, unit_mass=True))}
    s.close()
    return out


def run_output(sc, dev, stream, args):
    """Frame output at 1M particles, per frame: the reference's path
    (synchronous read of the whole state, ASCII .vtp with 9 decimals) against
    an asynchronous frame copy into pinned memory overlapped with the next
    step, written as binary .vtp."""
    import tempfile

    import torch

    from fluidsimulator_gb300.solver import Solver, write_vtp

    n = sc.count
    s = Solver(dev.index)
    s.configure([sc.params], [n])
    s.set_stream(stream.cuda_stream)
    s.upload(sc.pos, sc.vel)
    s.step(2)
    frames = 3
    hp = torch.empty((3, n), dtype=torch.float32, pin_memory=True).numpy()
    with tempfile.TemporaryDirectory() as d:
        t0 = time.perf_counter()
        for k in range(frames):
            s.step(1)
            pos, _ = s.download()
            write_vtp(os.path.join(d, f"a{k}.vtp"), pos, binary=False)
        ascii_ms = 1e3 * (time.perf_counter() - t0) / frames
        s.upload(sc.pos, sc.vel)
        s.step(2)
        t0 = time.perf_counter()
        for k in range(frames):
            s.frame_begin(0, hp)
            s.step_async(1)  # the copy overlaps this step
            s.frame_wait(0)
            write_vtp(os.path.join(d, f"b{k}.vtp"), hp, binary=True)
            s.synchronize()
        binary_ms = 1e3 * (time.perf_counter() - t0) / frames
        size_a = os.path.getsize(os.path.join(d, "a0.vtp"))
        size_b = os.path.getsize(os.path.join(d, "b0.vtp"))
    s.close()
    return {"particles": n, "frames": frames,
            "reference_path_ms_per_step_and_frame": round(ascii_ms, 2),
            "async_binary_ms_per_step_and_frame": round(binary_ms, 2),
            "speedup": round(ascii_ms / binary_ms, 2), "ascii_bytes": size_a, "binary_bytes": size_b,
            "note": "one step plus one frame written per iteration, host wall clock, local disk"}


def run_batched(args, dev, stream, l2_flush):
    """64 independent dam-break scenes (2k-64k particles each, all flags):
    one batched solver (all scenes in the same launches, one CUDA graph per
    step, autotuned launch shapes) against the same scenes stepped serially by
    64 single-scene solvers enqueued back to back on one stream."""
    import torch

    from fluidsimulator_gb300 import scenes
    from fluidsimulator_gb300.solver import Solver

    scs = scenes.batched_scenes(args.batch_scenes, seed=0)
    counts = [sc.count for sc in scs]
    pos = torch.from_numpy(__import__("numpy").concatenate([sc.pos for sc in scs], axis=1)).to(dev)
    vel = torch.from_numpy(__import__("numpy").concatenate([sc.vel for sc in scs], axis=1)).to(dev)
    parts_p = [torch.from_numpy(sc.pos).to(dev) for sc in scs]
    parts_v = [torch.from_numpy(sc.vel).to(dev) for sc in scs]
    torch.cuda.synchronize(dev)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)

    big = Solver(dev.index)
    big.configure([sc.params for sc in scs], counts)
    big.set_stream(stream.cuda_stream)
    big.upload(pos, vel)
    shapes = big.autotune(1)
    sort_bits = big.sort_bits()
    small = []
    for sc, pp, vv in zip(scs, parts_p, parts_v):
        s = Solver(dev.index)
        s.configure([sc.params], [sc.count])
        s.set_stream(stream.cuda_stream)
        s.upload(pp, vv)
        s.set_tuning(shapes)
        s.set_sort_bits(sort_bits)
        small.append(s)

    ev2 = torch.cuda.Event(enable_timing=True)

    def timed_step(solvers):
        """One step of every solver between two events on the stream. A step
        that outgrows a capacity is re-run by synchronize() after a regrow,
        behind ev1: then the step is timed to an event recorded after the
        re-run (host turnaround included)."""
        before = sum(s.stats()["regrows"] for s in solvers)
        ev0.record(stream)
        for s in solvers:
            s.step_async(1)
        ev1.record(stream)
        for s in solvers:
            s.synchronize()
        if sum(s.stats()["regrows"] for s in solvers) != before:
            ev2.record(stream)
            ev2.synchronize()
            return ev0.elapsed_time(ev2)
        return ev0.elapsed_time(ev1)

    def time_batched(steps, restore):
        ms = []
        if not restore:
            big.upload(pos, vel)
        for _ in range(steps):
            if restore:
                big.upload(pos, vel)
            l2_flush.zero_()
            ms.append(timed_step([big]))
        return ms

    def time_serial(steps, restore):
        ms = []
        if not restore:
            for s, pp, vv in zip(small, parts_p, parts_v):
                s.upload(pp, vv)
        for _ in range(steps):
            if restore:
                for s, pp, vv in zip(small, parts_p, parts_v):
                    s.upload(pp, vv)
            l2_flush.zero_()
            ms.append(timed_step(small))
        return ms

    time_batched(args.warmup, True)
    time_serial(args.warmup, True)
    b = time_batched(args.steps, True)
    sr = time_serial(args.steps, True)
    out = {"scenes": len(scs), "particles": int(sum(counts)), "steps": args.steps,
           "batched_ms_per_step": round(statistics.mean(b), 4), "serial_ms_per_step": round(statistics.mean(sr), 4),
           "batched_scene_steps_per_s": round(len(scs) * 1e3 / statistics.mean(b), 1),
           "serial_scene_steps_per_s": round(len(scs) * 1e3 / statistics.mean(sr), 1),
           "speedup": round(statistics.mean(sr) / statistics.mean(b), 3),
           "workload": "one step over each scene's initial batch per timed step, L2 flushed between steps",
           "tuning": shapes, "sort_bits": sort_bits, }
    if args.batch_trajectory > 0:
        tb = time_batched(args.batch_trajectory, False)
        ts = time_serial(args.batch_trajectory, False)
        st = big.stats()
        out["trajectory"] = {"steps": args.batch_trajectory, "batched_ms_total": round(sum(tb), 3),
                             "serial_ms_total": round(sum(ts), 3), "speedup": round(sum(ts) / sum(tb), 3),
                             "neighbors_per_particle_last": round(st["neighbor_pairs"] / st["particles"], 2)}
    for s in small:
        s.close()
    big.close()
    return out


def _finite(x):
    """JSON-safe copy: non-finite floats (an overflowed gradient) become null."""
    import math

    if isinstance(x, dict):
        return {k: _finite(v) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [_finite(v) for v in x]
    if isinstance(x, float) and not math.isfinite(x):
        return None
    return x


# --------------------------------------------------------------------------
# CPU: oracle restatement of the reference step

def _cpu_sample(sc, particles):
    """The first `particles` particles of the lattice (whole z-layers)."""
    from fluidsimulator_gb300 import scenes

    layer = N_SIDE * N_SIDE
    k = max(1, min(N_SIDE, particles // layer)) * layer
    return scenes.Scene(sc.name, sc.params, sc.pos[:, :k].copy(), sc.vel[:, :k].copy())


def cpu_baseline(sc, budget_s=20.0, steps=None):
    from oracle import pyoracle

    pyoracle.build(ref=False)
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    probe = _cpu_sample(sc, 100_000)
    t0 = time.perf_counter()
    pyoracle.Oracle().run(probe.params, probe.pos, probe.vel, 0.0, 1)
    per_particle = (time.perf_counter() - t0) / probe.count
    reps = steps or 2
    particles = int(min(sc.count, budget_s / reps / max(per_particle, 1e-12)))
    sample = _cpu_sample(sc, particles)
    t0 = time.perf_counter()
    for _ in range(reps):
        pyoracle.Oracle().run(sample.params, sample.pos, sample.vel, 0.0, 1)
    dt = time.perf_counter() - t0
    out = {"value": round(sample.count * reps / dt, 1), "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{reps} x step 1 of the first {sample.count} particles (whole z-layers) of the 1M scene, "
                     f"oracle/pbf_oracle.cpp (restatement of core/src/core.cpp:119-615), OpenMP {threads} threads, "
                     f"{os.uname().machine}"}
    return out, step1_parity(sample)


def step1_parity(sample):
    """The sample's first step on the GPU against the oracle as checker (an
    untimed run): neighbour counts per particle and their histogram, and the
    positions and velocities, bit for bit; and the GPU's and the CPU FP32
    step's distance from an FP64 run of the oracle."""
    import numpy as np

    from fluidsimulator_gb300 import _capi
    from fluidsimulator_gb300.solver import Solver
    from oracle import pyoracle

    ref = pyoracle.Oracle().run(sample.params, sample.pos, sample.vel, 0.0, 1, dump=True)
    s = Solver(0)
    s.configure([sample.params], [sample.count])
    s.upload(sample.pos, sample.vel)
    s.step(1)
    counts = s.read_debug(_capi.DEBUG_NEIGHBOR_COUNTS)
    pos, vel = s.download()
    s.close()
    hist_gpu = np.bincount(counts)
    hist_ref = np.bincount(ref["neighbor_counts"])
    # Error of each FP32 result against an FP64 run of the same step.
    ref64 = pyoracle.Oracle(np.float64).run(sample.params, sample.pos.astype(np.float64),
                                            sample.vel.astype(np.float64), 0.0, 1)
    h = float(sample.params.h)

    def dx_stats(p32):
        d = np.max(np.abs(p32.astype(np.float64) - ref64["pos"]), axis=0) / h
        return {"median": float(np.median(d)), "p99": float(np.percentile(d, 99)), "max": float(d.max())}

    return {"particles": sample.count, "neighbor_counts_equal": bool(np.array_equal(counts, ref["neighbor_counts"])),
            "dx_vs_fp64_over_h": {"gpu": dx_stats(pos), "cpu_fp32": dx_stats(ref["pos"])},
            "histogram_equal": bool(np.array_equal(hist_gpu, hist_ref)),
            "neighbors_mean": round(float(counts.mean()), 2), "neighbors_max": int(counts.max()),
            "positions_equal": bool(np.array_equal(pos, ref["pos"])),
            "velocities_equal": bool(np.array_equal(vel, ref["vel"])),
            "max_abs_dx_over_h": float(np.max(np.abs(pos - ref["pos"]))) / float(sample.params.h)}


def cpu_configs(configs, args):
    """The oracle on the host cores over c1 (all steps) and a prefix of c2;
    the GPU's state after the same steps must equal the oracle's bit for bit.
    Fills configs[key]["cpu"] and drops the scene objects."""
    import numpy as np
    import torch

    from fluidsimulator_gb300.solver import Solver
    from oracle import pyoracle

    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    for key, c in configs.items():
        sc = c.pop("_scene")
        gms = c.pop("_ms")
        steps = c["steps"] if key.startswith("c1") else min(c["steps"], args.c2_cpu_steps)
        steps = min(steps, c["steps"])
        o = pyoracle.Oracle()
        t0 = time.perf_counter()
        r = o.run(sc.params, sc.pos, sc.vel, 0.0, steps, records=True)
        dt = time.perf_counter() - t0
        s = Solver(torch.cuda.current_device())
        s.configure([sc.params], [sc.count])
        s.upload(sc.pos, sc.vel)
        s.step(steps)
        pos, vel = s.download()
        s.close()
        c["cpu"] = {"steps": steps, "ms_per_step": round(1e3 * dt / steps, 3),
                    "particle_steps_per_s": round(sc.count * steps / dt, 1), "cores": threads, "kind": "port",
                    "neighbors_per_particle_last": round(float(r["neighbor_pairs"][-1]) / sc.count, 2),
                    "what": f"oracle/pbf_oracle.cpp (restatement of core/src/core.cpp:119-615), steps 1-{steps} "
                            f"from the initial state, OpenMP {threads} threads, {os.uname().machine}"}
        c["gpu_equals_cpu_after_cpu_steps"] = bool(np.array_equal(pos, r["pos"]) and np.array_equal(vel, r["vel"]))
        # like for like: the GPU's own time over the steps the CPU ran
        same = statistics.mean(gms[:steps])
        c["gpu_ms_per_step_same_steps"] = round(same, 4)
        c["gpu_over_cpu_same_steps"] = round(c["cpu"]["ms_per_step"] / same, 1)
        if steps < c["steps_of_config"]:
            c["cpu"]["note"] = f"prefix: steps 1-{steps} of {c['steps_of_config']}"


def cpu_collapsed(col):
    """The oracle timed on the collapsed state the GPU step started from; the
    GPU's step must equal the oracle's bit for bit."""
    import numpy as np

    from oracle import pyoracle

    sc, pos, vel, t0, after = col.pop("_state")
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    o = pyoracle.Oracle()
    t = time.perf_counter()
    r = o.run(sc.params, pos, vel, t0, 1, dump=True)
    dt = time.perf_counter() - t
    col["cpu"] = {"ms_per_step": round(1e3 * dt, 2), "particle_steps_per_s": round(sc.count / dt, 1),
                  "cores": threads, "kind": "port",
                  "what": f"oracle/pbf_oracle.cpp, one step from the GPU's state after step {col['step'] - 1}, "
                          f"OpenMP {threads} threads, {os.uname().machine}"}
    col["cpu_neighbors_per_particle"] = round(float(r["neighbor_counts"].mean()), 2)
    col["gpu_equals_cpu"] = bool(np.array_equal(after[0], r["pos"]) and np.array_equal(after[1], r["vel"]))
    col["gpu_over_cpu"] = round(col["gpu"]["particle_steps_per_s"] / col["cpu"]["particle_steps_per_s"], 1)


def gradient_checks(args):
    """The oracle as checker of the differentiable scene's gradients (unit-mass
    variant, where the GPU's FP32 adjoint stays in range): the GPU's dL/dv0,
    dL/dx0 and dL/dc over 60 steps (checkpoints every 10) against the
    oracle's FP64 adjoint of the same FP32 trajectory, and dL/dv0 at horizon
    10 against central differences of the FP64 forward (step 1e-8, 4 random
    directions). The full set (16 directions, horizons 10 and 20, dL/dc) is
    tests/test_adjoint.py."""
    import numpy as np
    import torch

    from fluidsimulator_gb300 import scenes
    from fluidsimulator_gb300.solver import Solver
    from oracle import pyoracle

    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    target = np.array([1.5, 0.3, 1.0])
    um = scenes.differentiable_block(32, seed=0, unit_mass=True)
    n = um.count

    def cot(x):
        com = np.asarray(x, np.float64).mean(axis=1)
        return np.repeat((2.0 * (com - target) / n)[:, None], n, axis=1)

    s = Solver(torch.cuda.current_device())
    s.configure([um.params], [n])
    out = {}
    for horizon in (10, args.adj_steps):
        s.upload(um.pos, um.vel)
        s.record(horizon, 10)
        x, _ = s.download()
        gx0, gv0, gc = s.backward(cot(x).astype(np.float32), np.zeros((3, n), np.float32))
        o = pyoracle.Oracle()
        states = [(um.pos, um.vel)]
        for _ in range(horizon):
            r = o.run(um.params, *states[-1], 0.0, 1)
            states.append((r["pos"], r["vel"]))
        g, gv, gcr = cot(states[-1][0]), np.zeros((3, n)), 0.0
        for t in reversed(range(horizon)):
            g, gv, c, _, _ = pyoracle.vjp(um.params, *states[t], g, gv, fwd32=True)
            gcr += c
        rel = lambda a, b: float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))  # noqa: E731
        e = {"grad_v0_norm": float(np.linalg.norm(gv0)),
             "rel_err_vs_fp64_adjoint": {"dL_dv0": rel(gv0, gv), "dL_dx0": rel(gx0, g),
                                         "dL_dc": abs(float(gc[0]) - gcr) / abs(gcr)}}
        if horizon == 10:
            o64 = pyoracle.Oracle(np.float64)
            x64, v64 = um.pos.astype(np.float64), um.vel.astype(np.float64)

            def loss(v0):
                r = o64.run(um.params, x64, v0, 0.0, horizon)
                return float(np.sum((r["pos"].mean(axis=1) - target) ** 2))

            rng = np.random.default_rng(7)
            rels = []
            for _ in range(4):
                d = rng.standard_normal((3, n))
                d /= np.sqrt(np.mean(d * d))
                fd = (loss(v64 + 1e-8 * d) - loss(v64 - 1e-8 * d)) / 2e-8
                ad = float(np.sum(gv0.astype(np.float64) * d))
                rels.append(abs(fd - ad) / max(abs(fd), abs(ad), 1e-30))
            e["fd_fp64_step1e-8_rel_err_max"] = max(rels)
            e["fd_directions"] = len(rels)
        out[f"unit_mass_h{horizon}"] = e
    s.close()
    out["note"] = ("unit-mass variant (m = 1, rho0 = 1/sp^3); the scene as specified leaves the FP32 range after "
                   "~10 steps (its gradient grows ~10^3 per step); FP64 adjoint = oracle reverse mode chained "
                   "over the same FP32 trajectory")
    return out


def run_reference(args, world, rank):
    if rank != 0:
        return
    from fluidsimulator_gb300 import scenes
    from oracle import pyoracle

    pyoracle.build(ref=False)
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    sc = scenes.falling_block(N_SIDE, seed=0)
    probe = _cpu_sample(sc, 100_000)
    t0 = time.perf_counter()
    pyoracle.Oracle().run(probe.params, probe.pos, probe.vel, 0.0, 1)
    per_particle = (time.perf_counter() - t0) / probe.count
    budget = args.cpu_budget * 6  # whole run within a few minutes
    particles = int(min(sc.count, budget / max(args.steps + args.warmup, 1) / max(per_particle, 1e-12)))
    sample = _cpu_sample(sc, particles)
    for _ in range(args.warmup):
        pyoracle.Oracle().run(sample.params, sample.pos, sample.vel, 0.0, 1)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        pyoracle.Oracle().run(sample.params, sample.pos, sample.vel, 0.0, 1)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = sample.count * args.steps / total
    desc = (f"each step: one PBF step (step 1) of the first {sample.count} particles (whole z-layers) of the 1M "
            f"scene on the host CPU, oracle/pbf_oracle.cpp (CPU restatement of core/src/core.cpp:119-615; the "
            f"reference binary itself builds only where its source tree is), OpenMP {threads} threads, "
            f"{os.uname().machine}")
    out = {"metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
           "config": {"workload": WORKLOAD, "particles": sample.count},
           "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": threads, "kind": "port", "sample": desc},
           "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--trajectory", type=int, default=24, help="steps of the real run to report (0 = skip)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of CPU work for cpu_baseline")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-scene batched vs serial measurement")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--batch-trajectory", type=int, default=30)
    ap.add_argument("--side", type=int, default=100, help="lattice side of the throughput scene (100 = 1M)")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the differentiable-scene measurement")
    ap.add_argument("--no-output", action="store_true", help="skip the frame-output measurement")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--adj-steps", type=int, default=60)
    ap.add_argument("--no-configs", action="store_true", help="skip c1 / c2 and the collapsed-phase comparison")
    ap.add_argument("--c1-steps", type=int, default=240)
    ap.add_argument("--c2-steps", type=int, default=480)
    ap.add_argument("--c2-cpu-steps", type=int, default=3, help="prefix of c2 the oracle runs on the host")
    ap.add_argument("--c2-pair-budget", type=float, default=3e9,
                    help="stop c2 once a step's lists hold more entries than this")
    ap.add_argument("--collapsed-side", type=int, default=50)
    ap.add_argument("--collapsed-at", type=int, default=21)
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per launch of the dominant kernel from an ncu capture")
    args = ap.parse_args(argv)
    world, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
