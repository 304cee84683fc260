#!/usr/bin/env python
"""Benchmark of the waves solver step: simulated seconds per wall second on the 310x48x80 beach.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--mg 32|16]

A "step" is one accepted solver step (CFL, three VOF sweeps, MacCormack, offshore forcing,
geometry, multigrid build, MGPCG to relative residual 1e-6, extension, acceptance; retries and
defect corrections included).  The state is resident in HBM; the device time of each trial comes
from CUDA events the library records on its own stream.  L2 is flushed (a 256 MiB write) between
timed steps.  `value` = simulated seconds advanced / device seconds.  `e2e` drives the same
solver frame by frame through the C ABI with host buffers: request_time, run, the telemetry
read-back and the accepted-surface export to host memory, timed with the host clock.

--impl reference times the CPU restatement of the reference's algorithm (the oracle, all host
threads) on the same configuration and prints the same line with "impl": "reference".
With torchrun (N > 1) every rank runs an independent replica of the beach (the solver step has
no data-parallel exchange; replicas only); value = total simulated seconds / max wall over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "sim-s per wall-s at 310x48x80; pressure ms/step, learned+BF16 vs plain FP32"
UNIT = "sim-s/wall-s"
TOL = 1e-6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mg", type=int, default=32, choices=[32, 16])
    ap.add_argument("--grid", default="beach", choices=["beach", "large"],
                    help="beach: 310x48x80 (the metric's grid); large: 620x96x160, spacing halved")
    ap.add_argument("--e2e-frames", type=int, default=-1,
                    help="1/60 s frames of the end-to-end run; -1: the timed window's simulated span, 0: none")
    ap.add_argument("--window-start", type=float, default=5.0,
                    help="accepted time (s) the timed steps start from, reached by an untimed run from rest "
                         "(5 s: waves developed; 0: from rest)")
    ap.add_argument("--host-window", action="store_true",
                    help="time the window on a host-scheduled handle that takes over the graph run's checkpoint at "
                         "the window start (every kernel launched one by one, visible to kernel profilers)")
    ap.add_argument("--no-compare", dest="compare", action="store_false",
                    help="skip the BF16-multigrid and BF16 + learned warm-start arms")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Clocks:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.stop = threading.Event()
        self.t = threading.Thread(target=self.run, daemon=True)

    def run(self):
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5).stdout
                for line in out.strip().splitlines():
                    self.rows.append([x.strip() for x in line.split(",")])
            except Exception:
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=6)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 4 + k and r[4 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


GRIDS = {"beach": {}, "large": {"n": (620, 96, 160), "spacing": (0.0125, 0.0125, 0.025)}}


def beach_config(mg, grid="beach"):
    import waves_gb300 as wg
    return wg.config("beach", pressure_tolerance=TOL, mg_precision=mg, **GRIDS[grid])


class Window:
    """One solver handle timed over K accepted steps: every trial's device time comes from the CUDA
    events the library records on its own stream; L2 is flushed (a 256 MiB write) before each
    step."""

    def __init__(self, cfg, torch, flush):
        import ctypes as C
        import waves_gb300 as wg
        self.C, self.torch, self.flush = C, torch, flush
        self.s = wg.WavesSolver(cfg)

    def timing(self, reset):
        C, s = self.C, self.s
        m, p, t = C.c_double(), C.c_double(), C.c_int64()
        s._ck(s.lib.waves_timing(s.h, C.byref(m), C.byref(p), C.byref(t), reset))
        return m.value, p.value, t.value

    def one_step(self):
        s = self.s
        c = s.control()
        target = int(c[2]) + 1
        s.request_steps(target)
        while True:
            s.advance(1)
            c = s.control()
            if c[2] >= target:
                return c
            if c[7] > .5 and not ((c[7] == 20 or 10 <= c[7] <= 12) and c[29] < 2):
                raise RuntimeError(f"solver halted with code {c[7]}")

    def advance_to(self, t_start):
        """Untimed run from rest to the accepted time t_start (the waves' window)."""
        if t_start > 0:
            self.s.request_time(t_start)
            st = self.s.run(8)
            if st != 0:
                raise RuntimeError(f"solver stopped with status {st} before t = {t_start}")

    def measure(self, steps, warmup, barrier=None, clocks=None, checkpoint=False):
        s = self.s
        for _ in range(max(warmup, 3)):
            self.one_step()
        # the state the timed steps start from (the end-to-end run replays the same span)
        self.start_state = s.save() if checkpoint else None
        self.timing(True)
        c0, stats0 = s.control(), s.stats()
        if barrier:
            barrier()
        self.torch.cuda.synchronize()
        wall0 = time.perf_counter()
        for _ in range(steps):
            self.flush.zero_()
            self.torch.cuda.synchronize()
            self.one_step()
        wall = time.perf_counter() - wall0
        self.torch.cuda.synchronize()
        motion, pressure, trials = self.timing(True)
        c1 = s.control()
        n = max(int(c1[2] - c0[2]), 1)
        return {"c0": c0, "c1": c1, "sim_s": c1[1] - c0[1], "device_s": (motion + pressure) / 1e3, "wall_s": wall,
                "steps": int(c1[2] - c0[2]), "trials": trials, "motion_ms": motion, "pressure_ms": pressure,
                "iters": c1[18] - c0[18], "rounds": (c1[32] - c0[32]) + (c1[103] - c0[103]),
                "active": c1[32] - c0[32], "mg_builds": s.stats()["mg_builds"] - stats0["mg_builds"],
                "window_s": [c0[1], c1[1]], "pressure_ms_per_step": pressure / n, "ms_per_step": (motion + pressure) / n,
                "cg_iterations_per_step": (c1[18] - c0[18]) / n,
                "warm_start_used": int(c1[102] - c0[102])}

    def close(self):
        self.s.close()


def summary(r):
    """The per-arm figures of the JSON line."""
    return {"sim_s_per_wall_s": r["sim_s"] / r["device_s"] if r["device_s"] > 0 else None,
            "ms_per_step": r["ms_per_step"], "pressure_ms_per_step": r["pressure_ms_per_step"],
            "motion_ms_per_step": r["motion_ms"] / max(r["steps"], 1),
            "cg_iterations_per_step": r["cg_iterations_per_step"], "steps": r["steps"], "trials": r["trials"],
            "mg_builds": r["mg_builds"], "window_s": r["window_s"], "warm_start_trials": r["warm_start_used"]}


def load_shipped_model(s):
    """The learned warm start committed with the package (waves_gb300/learned/model_beach.npz)."""
    import waves_gb300 as wg
    from waves_gb300.learned import load_model
    weights, biases, iscale, oscale = load_model(os.path.join(os.path.dirname(wg.__file__), "learned", "model_beach.npz"))
    s.set_warm_start(weights, biases, iscale, oscale)


def run_ours(args, world, rank, local):
    import torch
    import waves_gb300 as wg
    from waves_gb300.build import build
    if rank == 0:
        build()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.set_device(local)
    import ctypes as C
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    barrier = (lambda: torch.distributed.barrier()) if world > 1 else None

    def cfg_of(mg, warm=0):
        cfg = beach_config(mg, args.grid)
        cfg.device = local
        cfg.warm_start = warm
        return cfg

    # the headline arm: args.mg multigrid, from the waves' window start
    arm = Window(cfg_of(args.mg), torch, flush)
    arm.advance_to(args.window_start)
    if args.host_window:
        checkpoint = arm.s.save()
        arm.close()
        previous = os.environ.get("WAVES_SCHEDULE")
        os.environ["WAVES_SCHEDULE"] = "host"
        try:
            arm = Window(cfg_of(args.mg), torch, flush)
        finally:
            if previous is None:
                del os.environ["WAVES_SCHEDULE"]
            else:
                os.environ["WAVES_SCHEDULE"] = previous
        arm.s.load(checkpoint)
    s, lib, h = arm.s, arm.s.lib, arm.s.h
    with Clocks(local) as clk:
        res = arm.measure(args.steps, args.warmup, barrier, checkpoint=args.e2e_frames != 0)
    c1 = res["c1"]
    # Roofline of the dominant kernel: one further step, host-scheduled, with every launch of the
    # probed kernels bracketed by CUDA events on the solver's stream (outside the timed region).
    s.request_steps(int(c1[2]) + 1)
    probe_trials, probes = s.probe_trial()
    counts = (C.c_int32 * 8)()
    lib.waves_debug_launch_counts(h, counts)
    counts = list(counts)
    trials, active, rounds, iters = res["trials"], res["active"], res["rounds"], res["iters"]
    # per trial: begin + condition, and when active: motion, pressure set-up, conditions, trial end;
    # per defect round: CG set-up + conditions + post; per CG iteration: the iteration kernels
    launches = int(trials * (counts[0] + counts[7] * 2) + active * (counts[1] + counts[2] + counts[6] + counts[7])
                   + rounds * (counts[3] + counts[5] + 2 * counts[7]) + iters * counts[4])
    out = dict(res)
    out.update({"defect_rounds": rounds - active, "launches": launches, "clocks": clk.summary(), "t_end": c1[1],
                "probes": probes if probe_trials else [], "plan": wg.mg_plan(arm.s.cfg)})
    # e2e: frames through the public API with host buffers, over the timed steps' simulated span,
    # from the state the timed steps started from (restored from the checkpoint taken there)
    e2e = None
    if args.e2e_frames != 0:
        s.load(arm.start_state)
        frames = args.e2e_frames if args.e2e_frames > 0 else max(1, int(round(res["sim_s"] * 60.0)))
        # page-locked host buffers for the per-frame surface export, as a renderer that reads the
        # surface every frame would hold them
        planes = torch.empty(4 * s.N, dtype=torch.float32, pin_memory=True).numpy()
        kinds = torch.empty(s.N, dtype=torch.float32, pin_memory=True).numpy()
        t_sim0 = s.control()[1]
        arm.timing(True)
        w0 = time.perf_counter()
        for f in range(frames):
            s.request_time(t_sim0 + (f + 1) / 60.0)
            s.run(4)
            s.stats()
            lib.waves_export_surface(h, planes.ctypes.data_as(C.POINTER(C.c_float)), kinds.ctypes.data_as(C.POINTER(C.c_float)))
        w = time.perf_counter() - w0
        e_motion, e_pressure, e_trials = arm.timing(True)
        sim_e = s.control()[1] - t_sim0
        e2e = {"sim_s": sim_e, "wall_s": w, "frames": frames, "window_s": [t_sim0, s.control()[1]],
               "h2d": 8, "d2h": int(planes.nbytes + kinds.nbytes + 128 * 8),
               "device_s": (e_motion + e_pressure) / 1e3, "trials": e_trials}
    out["e2e"] = e2e
    out["render"] = time_render(s, torch)
    arm.close()
    # the same multigrid from rest (the first steps of the run: still water, forcing ramping up)
    arms = {}
    if args.window_start > 0:
        rest = Window(cfg_of(args.mg), torch, flush)
        arms["from_rest"] = summary(rest.measure(args.steps, args.warmup, barrier))
        rest.close()
    # the comparison the metric names: BF16 multigrid, and BF16 multigrid + learned warm start,
    # over the same window as the headline (each from rest to the window start on its own handle)
    if args.compare and args.grid == "beach":
        for name, mg, warm in (("bf16", 16, 0), ("bf16_learned", 16, 1)):
            w = Window(cfg_of(mg, warm), torch, flush)
            if warm:
                load_shipped_model(w.s)
            w.advance_to(args.window_start)
            arms[name] = summary(w.measure(args.steps, args.warmup, barrier))
            w.close()
    out["arms"] = arms
    return out


def time_render(s, torch, width=1280, height=720, frames=10):
    """Headless presentation: surface export + water ray-march of one 1280x720 frame into device
    buffers (waves_render_device), CUDA events on the solver's stream, after two warm-up frames."""
    p = s.render_params(width, height)
    rgba = torch.empty((height, width, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.ExternalStream(s.stream())
    for _ in range(2):
        s.render_device(p, rgba.data_ptr())
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(frames):
        s.render_device(p, rgba.data_ptr())
    b.record(stream)
    b.synchronize()
    return {"view": "water", "width": width, "height": height, "ms_per_frame": a.elapsed_time(b) / frames,
            "launches_per_frame": 2}


def measured_peaks():
    """HBM copy bandwidth (GB/s) measured on this GPU model, else the stated fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the probed kernels
    from the ncu captures summarised in profiles/dram_traffic.txt ('kernel bytes ...' lines)."""
    out = {}
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.txt")) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 2 and not line.startswith("#"):
                    try:
                        out[parts[0]] = float(parts[1])
                    except ValueError:
                        pass
    except OSError:
        pass
    return out


def roofline(probes):
    """HBM roofline of the kernel with the largest probed time in one trial: algorithmic bytes per
    launch / CUDA-event time per launch, against the measured copy bandwidth.  Each probed launch
    carries two nested event brackets; their cost per launch, measured on an empty kernel
    bracketed the same way (the 'empty' calibration), is taken off every probed launch (at most
    down to a tenth of its bracketed time), so short kernels are not ranked by the bracket."""
    cal = {p["kernel"]: p for p in probes}
    empty = cal.get("empty")
    bracket_us = 1e3 * empty["ms"] / empty["launches"] if empty and empty["launches"] else 0.0
    live = [p for p in probes if p["launches"] > 0 and p["ms"] > 0 and p["kernel"] not in ("all", "empty", "empty_inner")]
    if not live:
        return None, []
    peak, source = measured_peaks()
    table = []
    for p in live:
        raw_us = 1e3 * p["ms"] / p["launches"]
        us = max(raw_us - bracket_us, 0.1 * raw_us)
        gbs = p["bytes"] / p["launches"] / (us / 1e6) / 1e9
        table.append({"kernel": p["kernel"], "launches": p["launches"], "us_per_launch": us, "us_per_launch_bracketed": raw_us,
                      "bytes_per_launch": p["bytes"] / p["launches"], "achieved_gbs": gbs, "frac": gbs / peak})
    total = sum(t["us_per_launch"] * t["launches"] for t in table)
    for t in table:
        t["share_of_probed"] = t["us_per_launch"] * t["launches"] / total
    top = max(table, key=lambda t: t["us_per_launch"] * t["launches"])
    traffic = ncu_traffic().get(top["kernel"])
    return {"bound": "hbm", "kernel": top["kernel"], "achieved": top["achieved_gbs"], "peak": peak, "unit": "GB/s",
            "frac": top["frac"], "peak_source": f"{source} copy bandwidth (hbm_gbs)",
            "traffic": traffic, "bytes_per_launch": top["bytes_per_launch"], "us_per_launch": top["us_per_launch"],
            "launches": top["launches"],
            "timing": "CUDA events on the solver stream around each launch, one host-scheduled trial after the timed steps, "
                      f"less the {bracket_us:.2f} us per launch the brackets measure on an empty kernel"}, table


STEP_BYTES_FORMULA = ("152 N + builds/step * (28 N + sum_{l>=1} S_l n_l b_m) + CG iterations/step * "
                      "(72 N + sum_l [7 n_l (S_l b_m + 5 b_v) + 3 n_l b_v] + 8 n_c^2)")


def step_bytes_model(plan, iters_per_step, builds_per_step, bf16):
    """Algorithmic (compulsory) HBM bytes of one accepted step: each distinct array read once and
    each output written once at its storage precision, halos and cache re-reads excluded.  N = fine
    cells; per step the non-CG passes move 152 N (VOF sweeps 36 N, MacCormack 24 N, geometry and
    coefficients 40 N, projection set-up 16 N, gradient, extension and acceptance 36 N); a Galerkin
    rebuild reads the fine coefficients (28 N) and writes every coarse operator (S_l n_l b_m); a CG
    iteration moves 72 N outside the preconditioner (matvec 36 N, x and r updates 24 N, direction
    12 N) plus one V-cycle, per level 7 passes over the operator and 5 vectors and 3 over one vector,
    and the dense coarse factor (FP32, 2 reads of n_c^2).  b_m = b_v = 4 bytes (FP32 multigrid) or 2
    (BF16).  plan: waves_gb300.mg_plan(cfg)."""
    bm = bv = 2 if bf16 else 4
    n = [l["n"][0] * l["n"][1] * l["n"][2] for l in plan]
    N = n[0]
    vcycle = sum(7 * n_l * (l["stencil"] * bm + 5 * bv) + 3 * n_l * bv for n_l, l in zip(n, plan)) + 2 * 4 * n[-1] ** 2
    rebuild = 28 * N + sum(l["stencil"] * n_l * bm for n_l, l in zip(n[1:], plan[1:]))
    total = 152 * N + builds_per_step * rebuild + iters_per_step * (72 * N + vcycle)
    return {"bytes_per_step": total, "non_cg": 152 * N, "rebuild": rebuild, "cg_iteration": 72 * N + vcycle,
            "vcycle": vcycle, "cells": N}


def step_roofline(plan, iters_per_step, builds_per_step, bf16, ms_per_step):
    """The whole step against the HBM roofline: step_bytes_model bytes / device time per step."""
    model = step_bytes_model(plan, iters_per_step, builds_per_step, bf16)
    peak, source = measured_peaks()
    achieved = model["bytes_per_step"] / (ms_per_step / 1e3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": f"{source} copy bandwidth (hbm_gbs)", "bytes_per_step": model["bytes_per_step"],
            "cg_iteration_bytes": model["cg_iteration"], "rebuild_bytes": model["rebuild"],
            "non_cg_bytes": model["non_cg"], "formula": STEP_BYTES_FORMULA}


def oracle_sample(cfg, seconds, threads):
    """Accepted steps of the oracle (FP32) from rest until `seconds` of wall time have passed, on
    `threads` OpenMP threads (0: every processor): (sim-s per wall-s, threads, steps, sim-s, wall-s)."""
    from tests.oracle_ref import Oracle, lib
    used = lib().wo_set_threads(threads)
    o = Oracle(cfg, 32)
    t0 = time.perf_counter()
    steps = 0
    while time.perf_counter() - t0 < seconds or steps == 0:
        steps += 1
        o.request_steps(steps)
        o.run()
    wall = time.perf_counter() - t0
    sim = float(o.control()[1])
    return sim / wall, used, steps, sim, wall


def cpu_baseline(args, cfg_mg, seconds, single_core_seconds=0.0):
    """The oracle (CPU restatement, FP32) on the beach for a bounded sample on every host core, and
    optionally a second sample on one core.  The configuration comes from the oracle's own presets
    (oracle/wo_config.cpp): this leg loads nothing of the product library."""
    from tests.oracle_ref import lib, oracle_config
    cfg = oracle_config("beach", pressure_tolerance=TOL, mg_precision=cfg_mg)
    try:
        value, cores, steps, sim, wall = oracle_sample(cfg, seconds, 0)
        out = {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{steps} accepted steps of the 310x48x80 beach from rest ({sim:.4f} sim-s, {wall:.1f} s)"}
        if single_core_seconds > 0:
            v1, _, s1, sim1, w1 = oracle_sample(cfg, single_core_seconds, 1)
            out["single_core"] = {"value": v1, "unit": UNIT, "cores": 1,
                                  "sample": f"{s1} accepted steps from rest ({sim1:.4f} sim-s, {w1:.1f} s)"}
    finally:
        lib().wo_set_threads(0)
    return out


def main():
    args = parse()
    world, rank, local = dist_env()
    if args.impl == "reference":
        if rank != 0:
            return
        base = cpu_baseline(args, args.mg, max(args.cpu_seconds, 1.0))
        line = {"metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": "beach 310x48x80 (lab_runner.gd settings), plain FP32 MGPCG, tol 1e-6",
                           "cells": 1190400},
                "impl": "reference",
                "cpu_baseline": {"value": base["value"], "unit": UNIT, "cores": base["cores"], "kind": base["kind"],
                                 "sample": base["sample"]},
                "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    import torch
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    res = run_ours(args, world, rank, local)
    sim, dev = res["sim_s"], res["device_s"]
    from waves_gb300.replicas import aggregate
    e = res["e2e"] or {"sim_s": 0.0, "wall_s": 0.0}
    sim_total, dev_max, e2e_sim, e2e_wall = aggregate(sim, dev, e["sim_s"], e["wall_s"],
                                                      device=f"cuda:{local}" if world > 1 else None)
    if rank != 0:
        torch.distributed.destroy_process_group() if world > 1 else None
        return
    steps = max(res["steps"], 1)
    line = {
        "metric": METRIC,
        "value": sim_total / dev_max if dev_max > 0 else None,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dev_max * 1e3 / steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32" if args.mg == 32 else "f32+bf16mg",
        "data": "synthetic",
        "config": {"workload": ("beach 310x48x80 (lab_runner.gd settings), " if args.grid == "beach" else
                                "beach 620x96x160 (lab_runner.gd settings, spacing halved), ")
                               + ("plain FP32 MGPCG" if args.mg == 32 else "BF16 multigrid, FP32 CG") + ", tol 1e-6",
                   "cells": 1190400 if args.grid == "beach" else 9523200, "l2": "flushed between steps (256 MiB write)",
                   "sim_window_s": res["window_s"],
                   "window": (f"{args.steps} accepted steps after {max(args.warmup, 3)} untimed ones, from the state an "
                              f"untimed run from rest reached at t = {args.window_start:g} s (waves developed; the "
                              f"forcing ramp ends at 5.6 s)") if args.window_start > 0 else
                             f"{args.steps} accepted steps after {max(args.warmup, 3)} untimed ones from rest",
                   "parallelism": "replicas" if world > 1 else "single"},
        "pressure_ms_per_step": res["pressure_ms"] / steps,
        "motion_ms_per_step": res["motion_ms"] / steps,
        "cg_iterations_per_step": res["iters"] / steps,
        "defect_rounds": res["defect_rounds"],
        "mg_builds": res["mg_builds"],
        "trials": res["trials"],
        "clocks": res["clocks"],
        "gpu_launches": res["launches"],
        "render": res["render"],
    }
    roof, kernels = roofline(res["probes"])
    line["roofline"] = roof
    line["step_roofline"] = step_roofline(res["plan"], res["iters"] / steps, res["mg_builds"] / steps,
                                          args.mg == 16, line["ms_per_step"]) if line["ms_per_step"] > 0 else None
    line["probed_kernels"] = kernels
    every = [p for p in res["probes"] if p["kernel"] == "all"]
    if every and res["trials"]:
        # in-situ kernel time of one trial (all launches, back to back) against the graph's time
        line["kernel_ms_per_trial"] = every[0]["ms"]
        line["kernel_launches_per_trial"] = every[0]["launches"]
        line["graph_ms_per_trial"] = (res["motion_ms"] + res["pressure_ms"]) / res["trials"]
    if res["e2e"]:
        e = res["e2e"]
        line["e2e"] = {"value": e2e_sim / max(e2e_wall, 1e-12), "unit": UNIT, "h2d_bytes_per_step": e["h2d"],
                       "d2h_bytes_per_step": e["d2h"], "step": "one 1/60 s frame: request_time, run, stats, surface export",
                       "frames": e["frames"], "window_s": e["window_s"],
                       "window": "the timed steps' simulated span again, from the state they started from (restored)",
                       "device_sim_s_per_s": e["sim_s"] / e["device_s"] if e.get("device_s") else None,
                       "trials": e.get("trials")}
    arms = dict(res["arms"])
    arms[("fp32" if args.mg == 32 else "bf16") + "_headline"] = summary(res)
    line["arms"] = arms
    plain = arms.get("fp32_headline")
    mixed = arms.get("bf16_learned")
    if plain and mixed:
        # the metric's second half: pressure ms per accepted step, plain FP32 over BF16 + learned
        line["pressure_ms_ratio_plain_fp32_over_bf16_learned"] = plain["pressure_ms_per_step"] / mixed["pressure_ms_per_step"]
        line["sim_rate_ratio_bf16_learned_over_plain_fp32"] = mixed["sim_s_per_wall_s"] / plain["sim_s_per_wall_s"]
    if world == 1 and not args.no_cpu_baseline:
        try:
            base = cpu_baseline(args, args.mg, args.cpu_seconds, args.cpu_seconds / 2)
            line["cpu_baseline"] = base
        except Exception as ex:  # the oracle needs a C++ toolchain on the host
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "error": str(ex)[:200]}
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
