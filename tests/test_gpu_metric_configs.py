"""Parity on the benchmark's own configurations (sizes where the oracle needs seconds per step).

- The 310x48x80 beach (the lab_runner.gd:26 settings, CG relative residual 1e-6): three accepted
  steps from rest, and three from a developed-wave state at t = 5 s that the GPU reached and the
  oracle takes over (banks, control block, masks, geometry).  For the hand-over both run with the
  rebuild-every-trial multigrid maintenance, so no lagged hierarchy has to travel with the state.
- The 64x48x16 sloshing tank (surface 0.45 + 0.05 sin(2 pi x / 1.6), CFL 0.5, tolerance 1e-6):
  50 accepted steps bit for bit, and the drift from the FP64 oracle over its 200 steps.
- The error of one GPU step against one FP64 oracle step from the same state, every step of the
  tank's 200 and of the beach's first 0.5 simulated seconds (FP32 and BF16 multigrid: the
  mixed-precision configuration's first report interval), held to the per-step bars; and the
  tank's whole FP32 trajectory against the FP64 trajectory, recorded.

Bit for bit means: both banks, signed distance and kind of every cell, pressure masks, valid bands
and every decision entry of the control block, after every accepted step.
"""
import numpy as np
import pytest

import waves_gb300 as wg
from tests.oracle_ref import Oracle
from tests.test_gpu_accuracy import F_TOLERANCE, liquid_faces, split
from tests.test_gpu_parity import compare_state

# Per-step bars against the FP64 oracle from the same state.  F is held to 1e-5.  Velocity and
# pressure are held to what the reference's own convergence and acceptance tests allow: in FP32
# the CG recurrence residual meets the relative test sooner than in FP64 and the acceptance
# check then runs a defect correction (pressure_pass.glslinc:84-87), so the FP32 step may stop
# at another CG iterate than the FP64 one (on the tank, 2 + 2 iterations against 4); the two
# converged answers differ by up to a few 1e-3 m/s and a few 1e-3 of the pressure.
U_STEP = 1e-2  # m/s, liquid faces
P_STEP = 1e-2  # relative to the largest FP64 pressure in liquid cells


def beach(**kw):
    return wg.config("beach", pressure_tolerance=1e-6, **kw)


def tank(**kw):
    return wg.config("tank", **kw)


def lockstep(g, o, cfg, steps, tag):
    first = int(g.control()[2])
    assert first == int(o.control()[2])
    for step in range(first + 1, first + steps + 1):
        for s in (g, o):
            s.request_steps(step)
            s.run()
        problems = compare_state(g, o, cfg, f"{tag} step {step}")
        assert not problems, "\n".join(problems)
    assert g.control()[2] == first + steps


@pytest.mark.gpu
def test_beach_parity_from_rest(gpu_lib):
    cfg = beach()
    g, o = wg.WavesSolver(cfg), Oracle(cfg, 32)
    lockstep(g, o, cfg, 3, "beach from rest")
    g.close()
    o.close()


@pytest.mark.gpu
def test_beach_parity_from_developed_waves(gpu_lib):
    cfg = beach(mg_maintenance=0)
    g = wg.WavesSolver(cfg)
    g.request_time(5.0)
    assert g.run() == 0
    c = g.control()
    assert c[1] >= 5.0 and c[7] == 0
    o = Oracle(cfg, 32)
    o.set_control(c)
    for b in (0, 1):
        o.set_bank(b, g.bank(b))
    o.set_masks(*g.masks())
    o.set_geometry(*g.geometry())
    problems = compare_state(g, o, cfg, "hand-over at t = 5 s")
    assert not problems, "\n".join(problems)
    lockstep(g, o, cfg, 3, "beach from t = 5 s")
    g.close()
    o.close()


@pytest.mark.gpu
def test_tank_parity_50_steps(gpu_lib):
    cfg = tank()
    assert tuple(cfg.n) == (64, 48, 16)
    g, o = wg.WavesSolver(cfg), Oracle(cfg, 32)
    lockstep(g, o, cfg, 50, "tank")
    g.close()
    o.close()


def errors(g_bank, o_bank, n):
    """Worst |F - F64|, |u - u64| on liquid faces (m/s) and |p - p64| in liquid cells relative to
    the largest |p64| there, of a GPU bank against an FP64 oracle bank."""
    Fg, ug, pg = split(g_bank.astype(np.float64), n)
    Fo, uo, po = split(o_bank, n)
    lf, lc = liquid_faces(Fo, n), Fo > 0.5
    return (float(np.max(np.abs(Fg - Fo))),
            float(np.max(np.abs(ug - uo)[lf])) if lf.any() else 0.0,
            float(np.max(np.abs(pg - po)[lc]) / max(np.max(np.abs(po[lc])), 1e-30)) if lc.any() else 0.0,
            int(np.count_nonzero(np.abs(Fg - Fo) > F_TOLERANCE)))


def per_step_report(cfg, steps=None, until=None):
    """The error of one GPU step against one FP64 oracle step from the same state: before every
    step the FP64 oracle takes over the GPU's state (both banks, control block, masks, geometry),
    then both take one accepted step and the results are compared.  With the rebuild-every-trial
    multigrid maintenance both build their hierarchy from that state, so the difference is the
    FP32 (or BF16) arithmetic of one step alone."""
    n = tuple(cfg.n)
    g = wg.WavesSolver(cfg)
    o = Oracle(cfg, 64)
    rows = []
    while True:
        c = g.control()
        o.set_control(c)
        for b in (0, 1):
            o.set_bank(b, g.bank(b))
        o.set_masks(*g.masks())
        o.set_geometry(*g.geometry())
        step = int(c[2]) + 1
        for s in (g, o):
            s.request_steps(step)
            s.run()
        cg, co = g.control(), o.control()
        assert cg[2] == co[2] == step
        rows.append((co[1],) + errors(g.bank(), o.bank_d(), n)[:3] + (abs(cg[1] - co[1]),))
        if (steps is not None and step >= steps) or (until is not None and co[1] >= until):
            break
    g.close()
    o.close()
    return np.array(rows)


def trajectory_report(cfg, steps):
    """The GPU run and an FP64 oracle run from the same initial state, compared at every accepted
    step count (the two trajectories are free to part where a threshold decision of the VOF
    update falls differently in the two precisions)."""
    n = tuple(cfg.n)
    g = wg.WavesSolver(cfg)
    o = Oracle(cfg, 64)
    rows = []
    for step in range(1, steps + 1):
        for s in (g, o):
            s.request_steps(step)
            s.run()
        cg, co = g.control(), o.control()
        assert cg[2] == co[2] == step
        rows.append((co[1],) + errors(g.bank(), o.bank_d(), n) + (abs(cg[1] - co[1]),))
    g.close()
    o.close()
    return np.array(rows)


def summarize(name, r, interval=None):
    worst = r[:, 1:4].max(axis=0)
    print(f"{name}: {len(r)} steps to t = {r[-1, 0]:.4f} s; max|F - F64| {worst[0]:.3e}, max|u - u64| {worst[1]:.3e} m/s, "
          f"max|p - p64|/max|p64| {worst[2]:.3e}, max|t - t64| {r[:, -1].max():.3e} s")
    if interval:
        lo = 0.0
        for hi in np.arange(interval, r[-1, 0] + interval, interval):
            sel = (r[:, 0] > lo) & (r[:, 0] <= hi + 1e-9)
            if sel.any():
                w = r[sel, 1:4].max(axis=0)
                print(f"  t in ({lo:.2f}, {hi:.2f}] s: F {w[0]:.3e}, u {w[1]:.3e}, p {w[2]:.3e}")
            lo = hi
    return worst


@pytest.mark.gpu
def test_tank_per_step_error_from_fp64_over_200_steps(gpu_lib):
    r = per_step_report(tank(mg_maintenance=0), steps=200)
    worst = summarize("tank 64x48x16, FP32, one step from the GPU's state", r, interval=0.5)
    assert worst[0] <= F_TOLERANCE and worst[1] <= U_STEP and worst[2] <= P_STEP, worst


@pytest.mark.gpu
def test_tank_trajectory_against_fp64(gpu_lib):
    """Recorded, not held to the per-step bars: the two runs accept the same steps at the same
    times, and their states part only where a threshold decision falls differently."""
    r = trajectory_report(tank(), steps=200)
    worst = summarize("tank 64x48x16, FP32 trajectory vs FP64 trajectory", r, interval=0.5)
    print(f"  cells with |F - F64| > 1e-5: at most {int(r[:, 4].max())} of {64 * 48 * 16}")
    assert r[:, -1].max() == 0.0  # identical accepted times
    assert worst[0] <= 0.25 and worst[1] <= 0.05 and worst[2] <= 1e-2, worst


@pytest.mark.gpu
@pytest.mark.parametrize("mg", [32, 16])
def test_beach_per_step_error_from_fp64_first_half_second(gpu_lib, mg):
    label = "FP32" if mg == 32 else "BF16"
    r = per_step_report(beach(mg_precision=mg, mg_maintenance=0), until=0.5)
    worst = summarize(f"beach 310x48x80, {label} multigrid, one step from the GPU's state", r, interval=0.25)
    assert worst[0] <= F_TOLERANCE and worst[1] <= U_STEP and worst[2] <= P_STEP, worst
