"""Parity on the benchmark's own configurations (sizes where the oracle needs seconds per step).

- The 310x48x80 beach (the lab_runner.gd:26 settings, CG relative residual 1e-6): three accepted
  steps from rest, and three from a developed-wave state at t = 5 s that the GPU reached and the
  oracle takes over (banks, control block, masks, geometry).  For the hand-over both run with the
  rebuild-every-trial multigrid maintenance, so no lagged hierarchy has to travel with the state.
- The 64x48x16 sloshing tank (surface 0.45 + 0.05 sin(2 pi x / 1.6), CFL 0.5, tolerance 1e-6):
  50 accepted steps bit for bit, and the drift from the FP64 oracle over its 200 steps.
- The beach's drift from the FP64 oracle over its first 0.5 simulated seconds, with the FP32 and
  the BF16 multigrid (the mixed-precision configuration's first report interval).

Bit for bit means: both banks, signed distance and kind of every cell, pressure masks, valid bands
and every decision entry of the control block, after every accepted step.
"""
import numpy as np
import pytest

import waves_gb300 as wg
from tests.oracle_ref import Oracle
from tests.test_gpu_accuracy import F_TOLERANCE, P_TOLERANCE, U_TOLERANCE, liquid_faces, split
from tests.test_gpu_parity import compare_state


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


def drift_report(cfgs, steps=None, until=None):
    """Each GPU run in `cfgs` against one FP64 oracle run of cfgs[0], compared at every accepted
    step count: the worst |F - F64|, |u - u64| on liquid faces (m/s), |p - p64| in liquid cells
    relative to the largest |p64| there, and |t - t64|, overall and per `interval` of simulated
    time.  The configurations may differ only in the multigrid precision."""
    n = tuple(cfgs[0].n)
    gs = [wg.WavesSolver(c) for c in cfgs]
    o = Oracle(cfgs[0], 64)
    rows = [[] for _ in cfgs]
    step = 0
    while True:
        step += 1
        o.request_steps(step)
        o.run()
        co = o.control()
        assert co[2] == step
        Fo, uo, po = split(o.bank_d(), n)
        lf, lc = liquid_faces(Fo, n), Fo > 0.5
        for k, g in enumerate(gs):
            g.request_steps(step)
            g.run()
            cg = g.control()
            assert cg[2] == step
            Fg, ug, pg = split(g.bank().astype(np.float64), n)
            rows[k].append((co[1], float(np.max(np.abs(Fg - Fo))),
                            float(np.max(np.abs(ug - uo)[lf])) if lf.any() else 0.0,
                            float(np.max(np.abs(pg - po)[lc]) / max(np.max(np.abs(po[lc])), 1e-30)) if lc.any() else 0.0,
                            abs(cg[1] - co[1])))
        if (steps is not None and step >= steps) or (until is not None and co[1] >= until):
            break
    for g in gs:
        g.close()
    o.close()
    return [np.array(r) for r in rows]


def summarize(name, r, interval=None):
    worst = r[:, 1:].max(axis=0)
    print(f"{name}: {len(r)} steps to t = {r[-1, 0]:.4f} s; max|F - F64| {worst[0]:.3e}, max|u - u64| {worst[1]:.3e} m/s, "
          f"max|p - p64|/max|p64| {worst[2]:.3e}, max|t - t64| {worst[3]:.3e} s")
    if interval:
        edges = np.arange(interval, r[-1, 0] + interval, interval)
        lo = 0.0
        for hi in edges:
            sel = (r[:, 0] > lo) & (r[:, 0] <= hi + 1e-9)
            if sel.any():
                w = r[sel, 1:].max(axis=0)
                print(f"  t in ({lo:.2f}, {hi:.2f}] s: F {w[0]:.3e}, u {w[1]:.3e}, p {w[2]:.3e}, t {w[3]:.3e}")
            lo = hi
    return worst


@pytest.mark.gpu
def test_tank_drift_from_fp64_over_200_steps(gpu_lib):
    (r,) = drift_report([tank()], steps=200)
    worst = summarize("tank 64x48x16, FP32", r, interval=0.5)
    assert worst[0] <= F_TOLERANCE and worst[1] <= U_TOLERANCE and worst[2] <= P_TOLERANCE, worst


@pytest.mark.gpu
def test_beach_drift_from_fp64_first_half_second(gpu_lib):
    r32, r16 = drift_report([beach(), beach(mg_precision=16)], until=0.5)
    w32 = summarize("beach 310x48x80, FP32 multigrid", r32, interval=0.25)
    w16 = summarize("beach 310x48x80, BF16 multigrid", r16, interval=0.25)
    for w in (w32, w16):
        assert w[0] <= F_TOLERANCE and w[1] <= U_TOLERANCE and w[2] <= P_TOLERANCE, w
