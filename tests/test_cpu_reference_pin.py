"""The oracle pinned to the reference's own shaders (tests/reference_pin.py), on the CPU.

The reference's GLSL compute programs are translated to C++ where they lie in the reference
checkout (oracle/glsl/translate.py) and run on the host (oracle/glsl/glsl.hpp).  In lockstep with
the FP32 oracle, every dispatch unit of the reference's command lists starts from the oracle's
state, runs through the reference's shader code and through the oracle, and every buffer is
compared: all must agree bit for bit, except control-block sums of the reference's FP32 workgroup
reductions (against the oracle's FP64 sums) and Galerkin products (float atomics in dispatch order
against a fixed gather), which are held to 1e-4 relative; every decision entry must agree exactly.
The configurations are the parity cases the reference can express: its push constants have no
surface phase and its CFL number is 0.45.
"""
import math
import os

import numpy as np
import pytest

from tests.oracle_ref import oracle_config
from tests.reference_pin import FreeReference, Lockstep, available

pytestmark = pytest.mark.skipif(not available(), reason="needs the reference checkout's shader sources")


def tank(**kw):
    return oracle_config("tank", n=(24, 16, 8), corrugation_phase=0.0, cfl=0.45, **kw)


def fixture(shape, **kw):
    return oracle_config("default", n=(24, 16, 8), shape=shape, pressure_tolerance=1e-6, **kw)


def beach_coarse(**kw):
    return oracle_config("beach", n=(62, 24, 8), spacing=(0.125, 0.05, 0.25), **kw)


def beach_slope(**kw):
    return oracle_config("beach", n=(64, 40, 8), origin=(0.5, -0.6, -0.2), **kw)


CASES = {
    "tank": (tank, 5),
    "tank_periodic_x": (lambda: tank(periodic_x=1), 3),
    "tank_height_normals": (lambda: tank(height_normals=1), 3),
    "tank_linear_air": (lambda: tank(linear_air=1, corrugation=0.1), 3),
    "tank_plain_transport": (lambda: tank(transport_cache=0, active_advection=0, corrugation=0.1), 3),
    "tank_interior_fast": (lambda: tank(transport_interior=1, corrugation=0.1), 3),
    "tank_jacobi_rebuild": (lambda: tank(mg_smoother=0, mg_smoothing=2, mg_maintenance=0), 3),
    "tank_structure": (lambda: tank(mg_maintenance=1), 3),
    "tank_aggregate_from_3": (lambda: tank(mg_aggregate_from=3), 3),
    "dam_break": (lambda: fixture(1), 4),
    "box_pool": (lambda: fixture(2), 3),
    "inflow": (lambda: fixture(3), 3),
    "jets": (lambda: fixture(4), 4),
    "wave_periodic": (lambda: oracle_config("default", n=(32, 16, 8), shape=5, periodic_x=1,
                                            wave=(0.03, 2 * math.pi / 0.8, math.sqrt(9.81 * 2 * math.pi / 0.8 * math.tanh(2 * math.pi / 0.8 * 0.45)), 0.45),
                                            stokes_second=1), 3),
    "beach_coarse": (beach_coarse, 2),
    "beach_slope": (beach_slope, 2),
    "beach_coarse_jacobi_rebuild": (lambda: beach_coarse(mg_smoother=0, mg_smoothing=2, mg_maintenance=0), 2),
    "absorber": (lambda: beach_coarse(shape=6), 2),
}


@pytest.mark.skipif(os.environ.get("WAVES_LONG") != "1", reason="about 35 minutes of one core: set WAVES_LONG=1")
def test_oracle_agrees_with_the_reference_shaders_on_the_full_beach():
    """The metric's own grid, the 310x48x80 beach of lab_runner.gd:26 (the oracle's preset), over
    its first two accepted steps, every dispatch unit, as the small cases below."""
    ls = Lockstep(oracle_config("beach"))
    ls.run_steps(2)
    bad, report = ls.report()
    totals = ls.totals()
    print(f"beach 310x48x80: {totals}")
    assert ls.control()[2] == 2
    assert bad == 0, report
    ls.close()


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_agrees_with_the_reference_shaders_unit_by_unit(name):
    make, steps = CASES[name]
    ls = Lockstep(make())
    ls.run_steps(steps)
    bad, report = ls.report()
    totals = ls.totals()
    print(f"{name}: {totals}")
    assert ls.control()[2] == steps or ls.control()[7] > 0
    assert totals["units"] > 100 and totals["exact"] > 0.9 * totals["units"]
    assert bad == 0, report
    ls.close()


def test_free_reference_and_oracle_accept_the_same_steps():
    """The reference's shaders alone (FP32 control block and workgroup sums) against the oracle
    (FP64 control block and sums, as the CUDA build): over 12 steps of the tank both accept every
    step at the same simulated times (to FP32 rounding of the accumulated clock); their CG
    iteration counts and defect-correction rounds may differ, and are printed."""
    from tests.oracle_ref import Oracle
    cfg = tank()
    r, o = FreeReference(cfg), Oracle(cfg, 32)
    differing = []
    for step in range(1, 13):
        for s in (r, o):
            s.request_steps(step)
            s.run()
        cr, co = r.control(), o.control()
        assert cr[2] == co[2] == step and cr[3] == co[3] and cr[7] == co[7] == 0
        assert abs(float(cr[1]) - co[1]) <= 1e-6 * co[1]
        differing += [(step, k, float(cr[k]), co[k]) for k in (8, 18, 58) if cr[k] != co[k]]
    print("differing (step, entry, reference, oracle):", differing)
    r.close()


@pytest.mark.skipif(os.environ.get("WAVES_LONG") != "1", reason="about 15 minutes: set WAVES_LONG=1")
def test_free_reference_and_oracle_over_two_seconds_of_the_coarse_beach():
    """The free run against the oracle over the first 240 accepted steps (2 simulated seconds) of
    the coarse beach: every step accepted on both sides with no rejection, retry or halt, at
    accepted times that differ only by the FP32 accumulation of the reference's clock; the CG
    iteration totals, the steps whose defect-correction flag differs and the largest bank
    difference are printed."""
    from tests.oracle_ref import Oracle
    cfg = beach_coarse()
    r, o = FreeReference(cfg), Oracle(cfg, 32)
    iters_r = iters_o = 0
    defect_steps, worst_dt, worst_bank = 0, 0.0, 0.0
    for step in range(1, 241):
        for s in (r, o):
            s.request_steps(step)
            s.run()
        cr, co = r.control(), o.control()
        assert cr[2] == co[2] == step and cr[3] == co[3] == 0 and cr[7] == co[7] == 0, step
        worst_dt = max(worst_dt, abs(float(cr[1]) - co[1]))
        iters_r += int(cr[8])
        iters_o += int(co[8])
        defect_steps += int(cr[58] != co[58])
        worst_bank = max(worst_bank, float(np.max(np.abs(r.bank().astype(np.float64) - o.bank().astype(np.float64)))))
    print(f"coarse beach, 240 steps to t = {co[1]:.4f} s: CG iterations reference {iters_r}, oracle {iters_o}; "
          f"defect-correction flag differs in {defect_steps} steps; max |t - t_ref| {worst_dt:.2e} s; "
          f"largest bank difference {worst_bank:.3g}")
    assert worst_dt <= 1e-5
    r.close()
    o.close()
