"""GPU solver (FP32 CG; FP32 or BF16 multigrid) against the FP64 instantiation of the oracle.

The FP32 parity tests pin the kernels bit for bit to the FP32 restatement; this file measures how
far the FP32 arithmetic (and the BF16 preconditioner) drifts from the same algorithm in FP64.
Each step is compared at the same accepted-step count: the volume fraction F within 1e-5 is the
bar the mixed-precision build is held to; velocities on liquid faces and pressures in liquid cells
are held to absolute (u, m/s) and relative (p) bars; the worst values are printed.
"""
import numpy as np
import pytest

import waves_gb300 as wg
from tests.cases import beach_slope, tank_small
from tests.oracle_ref import Oracle

STEPS = 8
F_TOLERANCE = 1e-5   # volume fraction, absolute
U_TOLERANCE = 1e-4   # m/s on liquid faces (the forced beach moves at ~0.1 m/s; the tank rests)
P_TOLERANCE = 1e-4   # pressure in liquid cells, relative to the largest FP64 pressure there


def split(bank, n):
    nx, ny, nz = n
    N = nx * ny * nz
    NF = (nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1)
    return bank[:N], bank[N:N + NF], bank[N + NF:N + NF + N]


def liquid_faces(F, n):
    """Faces with liquid (F > 1/2) on both sides, in bank face order (u, v, w; x fastest)."""
    nx, ny, nz = n
    wet = F.reshape(nz, ny, nx) > 0.5
    u = np.zeros((nz, ny, nx + 1), bool)
    u[:, :, 1:nx] = wet[:, :, :-1] & wet[:, :, 1:]
    v = np.zeros((nz, ny + 1, nx), bool)
    v[:, 1:ny, :] = wet[:, :-1, :] & wet[:, 1:, :]
    w = np.zeros((nz + 1, ny, nx), bool)
    w[:nz] = wet & np.roll(wet, 1, axis=0)  # z is periodic: face z sits between cells z-1 and z
    w[nz] = w[0]
    return np.concatenate([u.ravel(), v.ravel(), w.ravel()])


def drift(cfg, steps=STEPS):
    g = wg.WavesSolver(cfg)
    o = Oracle(cfg, 64)
    worst = {"F": 0.0, "u": 0.0, "p": 0.0, "t": 0.0}
    for step in range(1, steps + 1):
        g.request_steps(step)
        g.run()
        o.request_steps(step)
        o.run()
        cg, co = g.control(), o.control()
        assert cg[2] == co[2] == step
        Fg, ug, pg = split(g.bank().astype(np.float64), tuple(cfg.n))
        Fo, uo, po = split(o.bank_d(), tuple(cfg.n))
        worst["F"] = max(worst["F"], float(np.max(np.abs(Fg - Fo))))
        # velocities and pressures where the solver resolves them: liquid faces and cells (air
        # faces carry extrapolated values whose band membership is itself a threshold decision)
        lf, lc = liquid_faces(Fo, tuple(cfg.n)), Fo > 0.5
        if lf.any():
            worst["u"] = max(worst["u"], float(np.max(np.abs(ug - uo)[lf])))
        if lc.any():
            worst["p"] = max(worst["p"], float(np.max(np.abs(pg - po)[lc]) / max(np.max(np.abs(po[lc])), 1e-30)))
        worst["t"] = max(worst["t"], abs(cg[1] - co[1]))
    g.close()
    o.close()
    return worst


@pytest.mark.gpu
@pytest.mark.parametrize("name,make,mg", [("tank", tank_small, 32), ("beach_slope", beach_slope, 32),
                                          ("beach_slope_bf16", beach_slope, 16)])
def test_drift_from_fp64(gpu_lib, name, make, mg):
    worst = drift(make(mg_precision=mg))
    print(f"{name}: max|F - F64| {worst['F']:.3e}, max|u - u64| {worst['u']:.3e} m/s, "
          f"max|p - p64|/max|p64| {worst['p']:.3e}, max|t - t64| {worst['t']:.3e} s")
    assert worst["F"] <= F_TOLERANCE, worst
    assert worst["u"] <= U_TOLERANCE and worst["p"] <= P_TOLERANCE, worst
