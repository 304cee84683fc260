"""Writes the reference fixtures of tests/golden/ from the reference's own compute shaders.

The reference's GLSL programs, translated to C++ where they lie in its checkout and run on the host
(oracle/glsl, built into oracle/_ref/libwaves_ref.so by tests/reference_pin.py), run alone from
their own initial commands, with their own FP32 control block and workgroup sums (the free run of
tests/reference_pin.py).  Each fixture keeps, for one configuration the reference's push constants
can express, the configuration (the raw WavesConfig bytes), the reference's control block after
every accepted step and its current bank after the steps listed (on the coarse beach also after
step 5: at step 6 the reference's FP32 sums pass the CG convergence test at zero iterations where
the FP64 sums of the oracle and the kernels take two, and the two runs part by the solver's
tolerance from there).  tests/test_cpu_golden.py holds the oracle to them where the reference
checkout is absent.  Run from the repository root, in a checkout with the reference present:

    python -m tests.golden.make_reference_fixtures
"""
import ctypes as C
import os

import numpy as np

from tests.oracle_ref import oracle_config
from tests.reference_pin import FreeReference, available

HERE = os.path.dirname(os.path.abspath(__file__))


def tank():
    return oracle_config("tank", n=(24, 16, 8), corrugation_phase=0.0, cfl=0.45)


def beach_coarse():
    return oracle_config("beach", n=(62, 24, 8), spacing=(0.125, 0.05, 0.25))


FIXTURES = {"tank_24x16x8": (tank, 24, (24,)), "beach_62x24x8": (beach_coarse, 24, (5, 24))}


def make(name, build, steps, bank_steps):
    cfg = build()
    r = FreeReference(cfg)
    controls, banks = [], {}
    for step in range(1, steps + 1):
        r.request_steps(step)
        r.run()
        c = r.control()
        assert int(c[2]) == step and c[7] == 0, (name, step, c[2], c[7])
        controls.append(c.copy())
        if step in bank_steps:
            banks[f"bank_{step}"] = r.bank()
    r.close()
    path = os.path.join(HERE, f"reference_{name}.npz")
    np.savez_compressed(path, config=np.frombuffer(C.string_at(C.addressof(cfg), C.sizeof(cfg)), dtype=np.uint8),
                        controls=np.array(controls, dtype=np.float32), **banks)
    print(f"{path}: {steps} steps to t = {controls[-1][1]:.6f} s, banks after steps {bank_steps}")


if __name__ == "__main__":
    assert available(), "needs the reference checkout's shader sources"
    for name, (build, steps, bank_steps) in FIXTURES.items():
        make(name, build, steps, bank_steps)
