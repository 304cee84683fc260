"""GPU (CUDA library through the C ABI) versus the FP32 oracle on small grids.

Every per-cell FP32 operation is ordered identically in the kernels (-fmad=false) and in the
oracle (-ffp-contract=off); reductions are FP64 on both sides.  The decisions (accept, reject,
retry, defect correction, iteration counts), the wet/solid masks and both banks are therefore
required to match bit for bit after every accepted step.
"""
import numpy as np
import pytest

import waves_gb300 as wg
from tests.cases import CASES
from tests.compare import bank_locator, control_report, first_mismatch
from tests.oracle_ref import Oracle

STEPS = 6


def compare_state(g, o, cfg, tag):
    problems = []
    cg, co = g.control(), o.control()
    problems += control_report(cg, co)
    where = bank_locator(tuple(cfg.n))
    for b in (0, 1):
        m = first_mismatch(g.bank(b), o.bank(b), where)
        if m:
            problems.append(f"bank{b}: {m}")
    phi_g, kind_g = g.geometry()
    phi_o, kind_o = o.geometry()
    m = first_mismatch(kind_g, kind_o)
    if m:
        problems.append(f"kind: {m}")
    m = first_mismatch(phi_g, phi_o)
    if m:
        problems.append(f"phi: {m}")
    pg, vg = g.masks()
    po, vo = o.masks()
    m = first_mismatch(pg, po)
    if m:
        problems.append(f"pressure masks: {m}")
    m = first_mismatch(vg, vo)
    if m:
        problems.append(f"valid bands: {m}")
    return [f"{tag}: {p}" for p in problems]


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_initial_state_parity(gpu_lib, name):
    cfg = CASES[name]()
    g = wg.WavesSolver(cfg)
    o = Oracle(cfg, 32)
    problems = compare_state(g, o, cfg, "initial")
    assert not problems, "\n".join(problems)


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_step_parity(gpu_lib, name):
    cfg = CASES[name]()
    g = wg.WavesSolver(cfg)
    o = Oracle(cfg, 32)
    for step in range(1, STEPS + 1):
        g.request_steps(step)
        g.run()
        o.request_steps(step)
        o.run()
        problems = compare_state(g, o, cfg, f"step {step}")
        assert not problems, "\n".join(problems)
    assert g.control()[2] == STEPS


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["beach_slope", "beach_slope_bf16"])
@pytest.mark.parametrize("variant", ["WAVES_MG_ROWS_BELOW=0", "WAVES_MG_BOTTOM_GLOBAL=1"])
def test_step_parity_kernel_variants(gpu_lib, name, variant, monkeypatch):
    """Kernel forms that the small grids above do not reach: the level >= 1 sweeps with one
    thread per row (large levels use it; small ones use the product-parallel rows), and the
    bottom levels solved from global memory (used when they do not fit the shared-memory stage)."""
    key, value = variant.split("=")
    monkeypatch.setenv(key, value)
    cfg = CASES[name]()
    g = wg.WavesSolver(cfg)
    o = Oracle(cfg, 32)
    for step in range(1, 4):
        g.request_steps(step)
        g.run()
        o.request_steps(step)
        o.run()
        problems = compare_state(g, o, cfg, f"step {step}")
        assert not problems, "\n".join(problems)
