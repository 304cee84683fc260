"""The oracle against the reference's own outputs, without the reference checkout.

tests/golden/ holds runs of the reference's compute shaders alone (their FP32 control block and
workgroup sums; written by tests/golden/make_reference_fixtures.py): for the 24x16x8 tank at the
reference's CFL 0.45 and the 62x24x8 coarse beach, the control block after each of 24 accepted
steps and the bank after the listed steps.  A solver run from the same configuration must accept
the same steps with the same rejections and no failure, at accepted times within the FP32
rounding of the reference's clock, and its banks must stay within the bounds below.  The tank
stays within 1e-7 of the reference; on the coarse beach the reference's FP32 sums pass the CG
convergence test at step 6 with no iteration where the FP64 sums of the oracle (and of the
kernels) take two, and the runs then part by the solver's tolerance, so its step-24 bounds are the
tolerance's.  The kernels reach the fixtures through the oracle, which they match bit for bit
(tests/test_gpu_parity.py, on these two grids among others).
"""
import os

import numpy as np
import pytest

from tests.oracle_ref import Oracle
from tests.test_gpu_accuracy import liquid_faces, split
from waves_gb300.abi import WavesConfig

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# bank step -> bounds on max |F - F_ref|, max |u - u_ref| on liquid faces (m/s) and
# max |p - p_ref| in liquid cells relative to the largest |p_ref| there
BOUNDS = {
    "tank_24x16x8": {24: (1e-6, 1e-6, 1e-6)},
    "beach_62x24x8": {5: (1e-7, 2e-6, 1e-6), 24: (1e-2, 1e-3, 1e-3)},
}


def load(name):
    z = np.load(os.path.join(GOLDEN, f"reference_{name}.npz"))
    return WavesConfig.from_buffer_copy(z["config"].tobytes()), z


def bank_errors(bank, ref, n):
    F, u, p = split(bank.astype(np.float64), n)
    Fr, ur, pr = split(ref.astype(np.float64), n)
    lf, lc = liquid_faces(Fr, n), Fr > 0.5
    return (float(np.max(np.abs(F - Fr))),
            float(np.max(np.abs(u - ur)[lf])) if lf.any() else 0.0,
            float(np.max(np.abs(p - pr)[lc]) / max(np.max(np.abs(pr[lc])), 1e-30)) if lc.any() else 0.0)


def check_against_reference(make_solver, name):
    """Runs make_solver(config) through the fixture's steps and checks each against the reference."""
    cfg, z = load(name)
    n = tuple(cfg.n)
    s = make_solver(cfg)
    for step, r in enumerate(z["controls"], start=1):
        s.request_steps(step)
        s.run()
        c = s.control()
        assert int(c[2]) == int(r[2]) == step, (name, step, c[2], r[2])
        assert int(c[3]) == int(r[3]) and int(c[7]) == int(r[7]) == 0, (name, step, c[3], r[3], c[7], r[7])
        assert abs(float(c[1]) - float(r[1])) <= 1e-6 * float(c[1]), (name, step, c[1], r[1])
        if f"bank_{step}" in z.files:
            e = bank_errors(s.bank(), z[f"bank_{step}"], n)
            print(f"{name} step {step}: F {e[0]:.3e}, u {e[1]:.3e} m/s, p {e[2]:.3e}")
            assert all(a <= b for a, b in zip(e, BOUNDS[name][step])), (name, step, e)
    s.close()


@pytest.mark.parametrize("name", list(BOUNDS))
def test_fp32_oracle_against_the_reference_outputs(name):
    check_against_reference(lambda cfg: Oracle(cfg, 32), name)
