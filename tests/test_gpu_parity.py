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
@pytest.mark.parametrize("variant", ["WAVES_MG_ROWS_BELOW=0", "WAVES_MG_ROWS_BELOW=0,WAVES_MG_LANES=1",
                                     "WAVES_MG_BOTTOM_GLOBAL=1", "WAVES_MG_COARSE=1", "WAVES_MG_LEG=1"])
def test_step_parity_kernel_variants(gpu_lib, name, variant, monkeypatch):
    """Kernel forms that the small grids above do not reach: the level >= 1 sweeps of the large
    levels (four lanes per active row, and with WAVES_MG_LANES=1 one thread per row; small levels
    use the product-parallel rows), the bottom levels solved from global memory (used when they do
    not fit the shared-memory stage), the coarse levels as one cooperative launch, and the coarse
    leg as one thread-block cluster launch, instead of level by level."""
    for setting in variant.split(","):
        key, value = setting.split("=")
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


@pytest.mark.gpu
def test_step_parity_cluster_leg_jacobi(gpu_lib, monkeypatch):
    """The one-cluster coarse leg with Jacobi smoothing, over two levels and the bottom (the
    coarse beach), bit for bit against the oracle."""
    monkeypatch.setenv("WAVES_MG_LEG", "1")
    cfg = CASES["beach_coarse_jacobi"]()
    g = wg.WavesSolver(cfg)
    o = Oracle(cfg, 32)
    for step in range(1, 4):
        g.request_steps(step)
        g.run()
        o.request_steps(step)
        o.run()
        problems = compare_state(g, o, cfg, f"step {step}")
        assert not problems, "\n".join(problems)


@pytest.mark.gpu
def test_injected_rejection_parity(gpu_lib):
    """Host-side fault injection: c19 (waves_inject_rejection) forces code 4 at the next
    acceptance (pressure_pass.glslinc:268); the GPU rolls back and halts exactly as the oracle."""
    cfg = CASES["tank_small"]()
    g = wg.WavesSolver(cfg)
    o = Oracle(cfg, 32)
    g.request_steps(1)
    g.run()
    o.request_steps(1)
    o.run()
    g.inject_rejection()
    c = o.control()
    c[19] = 1
    o.set_control(c)
    g.request_steps(2)
    assert g.run() == 4  # WAVES_SOLVER_FAILED
    o.request_steps(2)
    o.run()
    cg = g.control()
    assert cg[7] == 4 and cg[3] == 1 and cg[2] == 1 and g.stats()["failure"] == 4
    problems = compare_state(g, o, cfg, "after injected rejection")
    assert not problems, "\n".join(problems)


@pytest.mark.gpu
def test_poisoned_fraction_retry_parity(gpu_lib):
    """A volume fraction of 1.5 fails the sweep bound (codes 10-12), the trial is rolled back and
    retried at half dt (coupled_motion.glslinc:351-355), on the GPU exactly as on the oracle."""
    cfg = CASES["tank_small"]()
    g = wg.WavesSolver(cfg)
    o = Oracle(cfg, 32)
    for s in (g, o):
        b = s.bank(0)
        b[5] = 1.5
        s.set_bank(0, b)
    g.request_steps(1)
    g.run()
    o.request_steps(1)
    o.run()
    cg, co = g.control(), o.control()
    assert cg[33] in (10.0, 11.0, 12.0) or cg[7] in (10.0, 11.0, 12.0)
    problems = compare_state(g, o, cfg, "after poisoned fraction")
    assert not problems, "\n".join(problems)


def check_export(g, o):
    """Host export bit for bit against the oracle's op 19; the device export (caller buffers) equal
    to the host one, with the surface clock of surface_clock.glsl:7."""
    import torch
    planes, kinds = g.export_surface()
    po, ko = o.export()
    m = first_mismatch(planes.ravel(), po.ravel())
    assert not m, f"planes: {m}"
    assert np.array_equal(kinds, ko)
    pd = torch.full((g.N, 4), -7.0, dtype=torch.float32, device="cuda")
    kd = torch.full((g.N,), -7.0, dtype=torch.float32, device="cuda")
    clock = torch.full((4,), -7.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    g.export_surface_device(pd.data_ptr(), kd.data_ptr(), clock.data_ptr())
    g.synchronize()
    assert np.array_equal(pd.cpu().numpy(), planes) and np.array_equal(kd.cpu().numpy(), kinds)
    c = g.control()
    assert clock.cpu().numpy().tolist() == [np.float32(c[1]), np.float32(c[2]), 0.0, 0.0]


@pytest.mark.gpu
def test_surface_export_parity(gpu_lib):
    """Op 19 export and the surface clock after accepted steps and after a rejected trial (the
    clock keeps the committed time, coastal_view.gd:19-23)."""
    cfg = CASES["beach_slope"]()
    g = wg.WavesSolver(cfg)
    o = Oracle(cfg, 32)
    for s in (g, o):
        s.request_steps(3)
        s.run()
    check_export(g, o)
    g.inject_rejection()
    c = o.control()
    c[19] = 1
    o.set_control(c)
    for s in (g, o):
        s.request_steps(4)
        s.run()
    assert g.control()[2] == 3 and g.control()[7] == 4
    check_export(g, o)
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["beach_slope", "tank_small"])
def test_history_parity(gpu_lib, name):
    """Telemetry history read back through waves_get_history against the oracle: per-trial sweep and
    trial rows, the coastal ledger and gauge rows, and the hierarchy audit words."""
    cfg = CASES[name]()
    g = wg.WavesSolver(cfg)
    o = Oracle(cfg, 32)
    for s in (g, o):
        s.request_steps(STEPS)
        s.run()
    trials, steps = int(g.control()[32]), int(g.control()[2])
    assert trials == int(o.control()[32]) and steps == STEPS
    hg, cg, ag = g.history()
    ho, co = o.history()
    ao = o.audit()
    for t in range(trials):
        sweeps_g, sweeps_o = hg[4 * t:4 * t + 3], ho[4 * t:4 * t + 3]
        assert np.array_equal(sweeps_g[:, :2], sweeps_o[:, :2]), (t, sweeps_g, sweeps_o)  # min / max F
        assert np.allclose(sweeps_g[:, 2:], sweeps_o[:, 2:], rtol=1e-6, atol=1e-12), (t, sweeps_g, sweeps_o)
        assert np.array_equal(hg[4 * t + 3], ho[4 * t + 3]), (t, hg[4 * t + 3], ho[4 * t + 3])
    if cfg.coastal:
        rows_g, rows_o = cg[:5 * steps], co[:5 * steps]
        assert np.abs(rows_o).sum() > 0
        assert np.allclose(rows_g, rows_o, rtol=1e-6, atol=1e-9), np.argwhere(~np.isclose(rows_g, rows_o, rtol=1e-6, atol=1e-9))[:5]
    builds = int(ag[13])
    assert builds >= 1 and builds == int(ao[13])
    words = 64 + 32 * builds
    m = first_mismatch(ag[:words].astype(np.int64), ao[:words].astype(np.int64))
    assert not m, f"audit: {m}"
    g.close()


@pytest.mark.gpu
def test_halting_parity(gpu_lib):
    """A run the algorithm halts: the periodic Stokes wave at CG tolerance 1e-6, whose true residual
    does not converge within the four defect corrections, fails acceptance (code 4) at the same
    trial on the GPU and on the oracle, with the same rolled-back state."""
    from tests.cases import wave_periodic
    cfg = wave_periodic(pressure_tolerance=1e-6)
    g = wg.WavesSolver(cfg)
    o = Oracle(cfg, 32)
    g.request_steps(STEPS)
    assert g.run() == 4  # WAVES_SOLVER_FAILED
    o.request_steps(STEPS)
    o.run()
    cg, co = g.control(), o.control()
    assert cg[7] == co[7] == 4 and cg[2] == co[2] < STEPS
    problems = compare_state(g, o, cfg, "halted")
    assert not problems, "\n".join(problems)
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["dam_break", "jets"])
def test_long_run_parity(gpu_lib, name):
    """24 accepted steps with rejections, retries and a multigrid rebuild at most trials: the state
    and the hierarchy audit words agree with the oracle at the end."""
    cfg = CASES[name]()
    g = wg.WavesSolver(cfg)
    o = Oracle(cfg, 32)
    for s in (g, o):
        s.request_steps(24)
        s.run()
    problems = compare_state(g, o, cfg, "24 steps")
    assert not problems, "\n".join(problems)
    assert g.control()[2] == 24 and g.control()[3] > 0  # rejections happened
    ag, ao = g.history()[2], o.audit()
    words = 64 + 32 * int(ag[13])
    assert int(ag[13]) == int(ao[13]) and np.array_equal(ag[:words], ao[:words])
    g.close()
