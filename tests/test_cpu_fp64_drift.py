"""The beach's one-step error against the FP64 oracle every half simulated second, on the CPU.

The kernels match the FP32 oracle bit for bit on the 310x48x80 beach itself
(tests/test_gpu_metric_configs.py, from rest and from a developed-wave state; the whole run from
rest to its halt at step 771 takes the same CG iteration count in both), so the FP32 oracle's
trajectory stands for the kernels'.  This test runs it from rest with the rebuild-every-trial
multigrid maintenance and CG relative residual 1e-6 and, at every half simulated second, hands its
state (both banks, control block, masks, geometry) to the FP64 oracle; both take one accepted step
and F, u and p are compared, as the GPU tests do step by step over the first half second.  It
takes about an hour on eight cores, so it runs only with WAVES_LONG=1:

    WAVES_LONG=1 python -m pytest tests/test_cpu_fp64_drift.py -s -q
"""
import os

import numpy as np
import pytest

from tests.oracle_ref import Oracle, lib, oracle_config
from tests.test_gpu_accuracy import F_TOLERANCE, liquid_faces, split

U_STEP = 1e-2  # m/s on liquid faces: what the reference's stopping tests allow (see test_gpu_metric_configs)
P_STEP = 1e-2  # relative to the largest FP64 pressure in liquid cells
INTERVAL = 0.5
SPAN = 10.0


def errors(b32, b64, n):
    F3, u3, p3 = split(b32.astype(np.float64), n)
    F6, u6, p6 = split(b64, n)
    lf, lc = liquid_faces(F6, n), F6 > 0.5
    return (float(np.max(np.abs(F3 - F6))),
            float(np.max(np.abs(u3 - u6)[lf])) if lf.any() else 0.0,
            float(np.max(np.abs(p3 - p6)[lc]) / max(np.max(np.abs(p6[lc])), 1e-30)) if lc.any() else 0.0)


@pytest.mark.skipif(os.environ.get("WAVES_LONG") != "1", reason="about an hour of CPU time: set WAVES_LONG=1")
def test_beach_error_from_fp64_every_half_second():
    lib().wo_set_threads(0)
    cfg = oracle_config("beach", pressure_tolerance=1e-6, mg_maintenance=0)
    n = tuple(cfg.n)
    o32, o64 = Oracle(cfg, 32), Oracle(cfg, 64)
    rows, halted = [], None
    mark = INTERVAL
    while mark <= SPAN + 1e-9:
        o32.request_time(mark)
        o32.run()
        c = o32.control()
        if c[7] > 0.5:
            halted = (float(c[1]), int(c[2]), int(c[7]))
            break
        o64.set_control(c)
        for b in (0, 1):
            o64.set_bank(b, o32.bank(b))
        o64.set_masks(*o32.masks())
        o64.set_geometry(*o32.geometry())
        step = int(c[2]) + 1
        for s in (o32, o64):
            s.request_steps(step)
            s.run()
        c32, c64 = o32.control(), o64.control()
        if c32[7] > 0.5 or c64[7] > 0.5:
            halted = (float(c32[1]), int(c32[2]), int(max(c32[7], c64[7])))
            break
        assert c32[2] == c64[2] == step
        e = errors(o32.bank(), o64.bank_d(), n)
        rows.append((float(c64[1]), step) + e + (abs(float(c32[1]) - float(c64[1])),))
        print(f"t = {c64[1]:.4f} s (step {step}): max|F - F64| {e[0]:.3e}, max|u - u64| {e[1]:.3e} m/s, "
              f"max|p - p64|/max|p64| {e[2]:.3e}, |t - t64| {rows[-1][-1]:.1e} s", flush=True)
        mark += INTERVAL
    if halted:
        print(f"halted at t = {halted[0]:.4f} s, step {halted[1]}, code {halted[2]}")
    o32.close()
    o64.close()
    assert len(rows) >= 10
    worst = np.array(rows)[:, 2:5].max(axis=0)
    print(f"worst over {len(rows)} reports: F {worst[0]:.3e}, u {worst[1]:.3e} m/s, p {worst[2]:.3e}")
    assert worst[0] <= F_TOLERANCE and worst[1] <= U_STEP and worst[2] <= P_STEP, worst
