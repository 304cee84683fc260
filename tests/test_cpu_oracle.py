"""The oracle against the known answers the reference shaders encode (the reference has no tests,
golden vectors or fixtures; parity with it is pinned only by these analytic cases)."""
import math

import numpy as np
import pytest

import waves_gb300 as wg
from tests.cases import CASES
from tests.oracle_ref import Oracle, lib


def cube_volume_exact(n, alpha, samples=60):
    """Midpoint-rule volume of the unit cube under n.x <= alpha (independent check)."""
    g = (np.arange(samples) + 0.5) / samples
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    return float(np.mean(n[0] * X + n[1] * Y + n[2] * Z <= alpha))


def test_cube_volume_limits_and_symmetry():
    L = lib()
    rng = np.random.default_rng(1)
    for _ in range(200):
        n = rng.normal(size=3)
        n /= np.abs(n).sum()
        lo = sum(min(x, 0) for x in n)
        hi = sum(max(x, 0) for x in n)
        assert L.wo_cube_volume_d(*n, lo - 1e-3) == 0.0
        assert L.wo_cube_volume_d(*n, hi + 1e-3) == 1.0
        a = rng.uniform(lo, hi)
        v = L.wo_cube_volume_d(*n, a)
        # central symmetry: V(n, a) + V(-n, -a) = 1  (plic_math.glslinc:8-9)
        assert abs(v + L.wo_cube_volume_d(*(-n), -a) - 1.0) < 1e-12
        assert abs(v - cube_volume_exact(n, a)) < 0.02


def test_inverse_volume_round_trip():
    L = lib()
    rng = np.random.default_rng(2)
    for _ in range(200):
        n = rng.normal(size=3)
        n /= np.abs(n).sum()
        f = rng.uniform(0.01, 0.99)
        a = L.wo_inverse_volume_d(*n, f)
        assert abs(L.wo_cube_volume_d(*n, a) - f) < 1e-6
    # exact half-volume tie at the centre (plic_math.glslinc:32)
    n = np.array([0.2, 0.5, 0.3])
    assert L.wo_inverse_volume(*n.astype(np.float32), 0.5) == np.float32(0.5 * 0.2 + 0.5 * 0.5 + 0.5 * 0.3)


def test_dispersion_and_probe_formulas():
    k = wg.dispersion_k(1.4, 0.45)
    omega = 2 * math.pi / 1.4
    assert abs(9.81 * k * math.tanh(k * 0.45) - omega ** 2) < 1e-9
    cfg = wg.config("beach", n=(62, 24, 8), spacing=(0.125, 0.05, 0.25))
    o = Oracle(cfg, 64)
    p = o.probes()
    # coastal_pass.glslinc:78-83: Stokes-2 surface/velocity of the ramped target
    a0, kk, w, h = [float(x) for x in cfg.wave]
    for i in range(8):
        t = cfg.ramp_periods * 2 * math.pi / w * (0.37 if i < 4 else 1.0)
        q = min(max(t * w / (2 * math.pi * cfg.ramp_periods), 0), 1)
        a = a0 * q ** 3 * (10 + q * (-15 + 6 * q))
        x = cfg.origin[0] + 0.17 + i * 0.23
        y = -h + i * 0.07
        sig = math.tanh(kk * h)
        second = kk * a * a * (3 - sig * sig) / (4 * sig ** 3)
        ph = kk * (x - cfg.origin[0]) - w * t
        eta = a * math.cos(ph) + second * math.cos(2 * ph)
        s = math.sinh(kk * h)
        u = a * w / s * math.cosh(kk * (y + h)) * math.cos(ph) + 0.75 * a * a * w * kk / s ** 4 * math.cosh(2 * kk * (y + h)) * math.cos(2 * ph)
        assert abs(p[i, 0] - eta) < 1e-6 and abs(p[i, 2] - u) < 1e-6


def test_beach_level_plan():
    cfg = wg.config("beach")
    o = Oracle(cfg, 32) if False else None  # the full beach oracle is built lazily below
    levels = Oracle(wg.config("beach", n=(310, 48, 80)), 32).levels()
    dims = [d for d, _ in levels]
    sts = [s for _, s in levels]
    assert dims == [(310, 48, 80), (155, 24, 80), (78, 12, 40), (39, 6, 20), (20, 3, 10), (10, 2, 5), (5, 2, 5)]
    assert sts == [7, 39, 125, 27, 27, 27, 27]


@pytest.mark.parametrize("name", sorted(CASES))
def test_product_level_plan_matches_the_oracle(name):
    """The library's level plan (waves_mg_plan, the host function waves_create uses) against the
    oracle's (pressure_multigrid.gd:37-69, :181-198) for every parity configuration: level sizes
    and Galerkin stencil sizes (periodic x, odd extents, aggregation from level 2 or 3)."""
    cfg = CASES[name]()
    plan = wg.mg_plan(cfg)
    assert [(l["n"], l["stencil"]) for l in plan] == Oracle(cfg, 32).levels()
    for a, b in zip(plan, plan[1:]):
        assert b["n"] == tuple((n + f - 1) // f for n, f in zip(a["n"], a["f"]))
    assert [l["aggregate"] for l in plan] == [l >= cfg.mg_aggregate_from for l in range(len(plan))]


def flat_tank(**kw):
    return wg.config("tank", n=(24, 24, 8), corrugation=0.0, eta=0.3, **kw)


def test_still_water_stays_still_and_hydrostatic():
    o = Oracle(flat_tank(), 32)
    o.request_steps(5)
    o.run()
    c = o.control()
    assert c[2] == 5 and c[7] == 0
    assert c[15] < 1e-3          # max face speed (m/s)
    assert c[16] < 0.05 * 9810 * 0.025  # hydrostatic error well below one cell of head


def test_volume_conservation_ledger():
    for name, cfg in (("tank", wg.config("tank", n=(24, 16, 8))),
                      ("beach", wg.config("beach", n=(62, 24, 8), spacing=(0.125, 0.05, 0.25)))):
        o = Oracle(cfg, 64)
        o.request_steps(6)
        o.run()
        c = o.control()
        assert c[2] == 6, name
        assert abs(c[100]) <= 1e-10 * c[26], (name, c[100], c[26])


def test_oracle_is_deterministic_and_thread_count_invariant():
    """The same run twice on all threads and once on one thread: identical banks and control
    block (the parallel loops write disjoint outputs; every floating-point sum is sequential)."""
    cfg = wg.config("beach", n=(64, 40, 8), origin=(0.5, -0.6, -0.2))
    runs = []
    try:
        for threads in (0, 0, 1):
            assert lib().wo_set_threads(threads) >= 1
            o = Oracle(cfg, 32)
            o.request_steps(3)
            o.run()
            runs.append(np.concatenate([o.bank(0), o.bank(1), o.control()]))
    finally:
        lib().wo_set_threads(0)
    assert np.array_equal(runs[0], runs[1]) and np.array_equal(runs[0], runs[2])


def test_injected_rejection_and_retry_paths():
    """Host-side fault injection on the oracle: c19 forces code 4 at the next acceptance
    (pressure_pass.glslinc:268), and a poisoned F of 1.5 fails the sweep bound (code 10-12) and
    retries at half dt (coupled_motion.glslinc:351-355)."""
    cfg = wg.config("tank", n=(24, 16, 8))
    o = Oracle(cfg, 32)
    o.request_steps(1)
    o.run()
    c = o.control()
    c[19] = 1
    o.set_control(c)
    o.request_steps(2)
    o.run()
    c = o.control()
    assert c[7] == 4 and c[3] == 1 and c[2] == 1
    o2 = Oracle(cfg, 32)
    b = o2.bank(0)
    b[5] = 1.5
    o2.set_bank(0, b)
    o2.request_steps(1)
    o2.run()
    c = o2.control()
    assert c[33] in (10.0, 11.0, 12.0) or c[7] in (10.0, 11.0, 12.0)


def flat_pool(level=0.43, n=(8, 8, 4), h=0.1):
    """Op-19 export of still water at y = level over a flat floor (no bed), box from the origin."""
    from waves_gb300.abi import WavesConfig
    cfg = WavesConfig()
    for k in range(3):
        cfg.n[k], cfg.spacing[k], cfg.origin[k] = n[k], h, 0.0
    cfg.slope = 0.0
    nx, ny, nz = n
    planes = np.zeros((nz, ny, nx, 4), dtype=np.float32)
    kinds = np.zeros((nz, ny, nx), dtype=np.float32)
    full = int(level // h)
    kinds[:, :full, :] = 1.0
    frac = level / h - full
    kinds[:, full, :] = 2.0
    planes[:, full, :] = (0.0, 1.0, 0.0, frac)  # liquid where n . x <= alpha in cell units
    return cfg, planes.reshape(-1, 4), kinds.ravel()


def top_view(mode):
    from waves_gb300.abi import WavesRenderParams
    p = WavesRenderParams()
    p.width, p.height, p.mode, p.orthographic = 16, 16, mode, 1
    p.eye[:] = (0.4, 2.0, 0.2)
    p.target[:] = (0.4, 0.0, 0.2)
    p.up[:] = (0.0, 0.0, -1.0)
    p.size = 0.6
    p.water_tint[:] = (0.02745, 0.56078, 0.62353)
    p.attenuation_distance, p.ripple_strength, p.surface_roughness = 0.18, 0.0025, 0.3
    p.sun_direction[:] = (-0.45, 0.65, -0.63)
    p.contact_correction, p.clock_ready = 1, 1
    return p


def test_render_oracle_known_answers():
    """Straight down through still water (clay.gdshader / water.gdshader): the first entry is the
    eye height above the surface, the occupied length the water depth, the clay shade the Lambert
    term of an upward normal; rays outside the box footprint miss."""
    from tests.oracle_ref import render
    cfg, planes, kinds = flat_pool()
    img, tr = render(planes, kinds, cfg, top_view(0), 0.0)
    hit = tr[..., 0] >= 0
    # rows sample z = -0.081 + 0.0375 k over the box's [0, 0.4]: rows 3..12 hit
    assert hit.sum() == 10 * 16 and np.all(hit[3:13]) and np.all(img[~hit] == 0)
    assert np.allclose(tr[hit, 0], 2.0 - 0.43, atol=2e-6)
    light = np.array([-0.4, 0.8, 0.5]) / np.linalg.norm([-0.4, 0.8, 0.5])
    assert np.allclose(img[hit, :3], 0.54 * (0.28 + 0.72 * light[1]), atol=1e-6)
    assert np.all(img[hit, 3] == 1)
    img, tr = render(planes, kinds, cfg, top_view(1), 0.0)
    hit = tr[..., 0] >= 0
    assert hit.sum() == 10 * 16
    assert np.allclose(tr[hit, 0], 2.0 - 0.43, atol=2e-6)
    assert np.allclose(tr[hit, 1], 0.43, atol=2e-6)  # occupied: surface to floor
    assert np.allclose(tr[hit, 2], 2.0, atol=2e-6)  # one interval, leaving through the floor
    # deeper water is darker in red (absorption 1.4 / 0.18 per metre) than the sky behind a miss
    assert np.all(img[hit, 0] < img[~hit, 0].min())


def test_fixture5_velocity_is_the_discrete_curl_of_the_stokes_streamfunction():
    """Op 40, fixture 5 (coupled_motion.glslinc:203-207,258-266; the surface eta of
    pressure_core.glslinc:52-58): the initial x and y face velocities are centred differences of the
    second-order Stokes streamfunction across each face, on faces up to three cells above the wave
    surface that are not walls, and zero elsewhere; the initial commands that follow
    (coupled_gpu.gd:34-37) do not touch velocities.  Evaluated independently here in FP64, against
    the FP64 oracle; and since each velocity is a difference of one vertex streamfunction, every
    cell with all four x/y faces set has zero discrete divergence."""
    from tests.cases import wave_periodic
    cfg = wave_periodic()
    nx, ny, nz = cfg.n
    hx, hy, _ = (float(v) for v in cfg.spacing)
    ox, oy, _ = (float(v) for v in cfg.origin)
    a, k, w, d = (float(v) for v in cfg.wave)
    eta0 = float(cfg.eta)
    N = nx * ny * nz
    nu = (nx + 1) * ny * nz
    bank = Oracle(cfg, 64).bank_d()
    u = bank[N:N + nu].reshape(nz, ny, nx + 1)
    v = bank[N + nu:N + nu + nx * (ny + 1) * nz].reshape(nz, ny + 1, nx)

    def psi(x, y):
        s = a * w / (k * math.sinh(k * d)) * np.sinh(k * (y + d)) * np.cos(k * x)
        return s + 0.375 * a * a * w / math.sinh(k * d) ** 4 * np.sinh(2 * k * (y + d)) * np.cos(2 * k * x)

    sigma = math.tanh(k * d)
    second = k * a * a * (3 - sigma * sigma) / (4 * sigma ** 3)
    eta = lambda qx: eta0 + a * np.cos(k * (ox + (qx + 0.5) * hx)) + second * np.cos(2 * k * (ox + (qx + 0.5) * hx))
    # x faces (periodic in x: no walls; the floor is below y = 0): position of face (qx, qy)
    qx, qy = np.meshgrid(np.arange(nx + 1), np.arange(ny), indexing="xy")
    fx, fy = ox + qx * hx, oy + (qy + 0.5) * hy
    band_u = fy < eta(qx) + 3 * hy
    want_u = np.where(band_u, (psi(fx, fy + 0.5 * hy) - psi(fx, fy - 0.5 * hy)) / hy, 0.0)
    # y faces: the bottom row (qy = 0) is a wall face
    qx, qy = np.meshgrid(np.arange(nx), np.arange(ny + 1), indexing="xy")
    fx, fy = ox + (qx + 0.5) * hx, oy + qy * hy
    band_v = (fy < eta(qx) + 3 * hy) & (qy > 0)
    want_v = np.where(band_v, -(psi(fx + 0.5 * hx, fy) - psi(fx - 0.5 * hx, fy)) / hx, 0.0)
    scale = max(np.abs(want_u).max(), np.abs(want_v).max())
    assert scale > 1e-3 and band_u.sum() > nx * 4
    for z in range(nz):
        assert np.abs(u[z] - want_u).max() <= 1e-9 * scale
        assert np.abs(v[z] - want_v).max() <= 1e-9 * scale
    assert np.abs(bank[N + nu + nx * (ny + 1) * nz:N + nu + nx * (ny + 1) * nz + nx * ny * (nz + 1)]).max() == 0.0
    full = band_u[:, :-1] & band_u[:, 1:] & band_v[:-1, :] & band_v[1:, :]
    div = (u[:, :, 1:] - u[:, :, :-1]) / hx + (v[:, 1:, :] - v[:, :-1, :]) / hy
    assert full.sum() > nx and np.abs(div[:, full]).max() <= 1e-9 * scale / hx


def tank_with(poison):
    """The 24x16x8 tank (dt 1/120, CFL 0.5 summed over axes) with both banks poisoned on the host."""
    cfg = wg.config("tank", n=(24, 16, 8))
    o = Oracle(cfg, 32)
    b = o.bank(0)
    poison(b, cfg)
    o.set_bank(0, b)
    o.set_bank(1, b.copy())
    o.request_steps(1)
    o.run()
    return cfg, o.control()


def test_cfl_substep_control_shrinks_dt_for_a_fast_face():
    """CFL control (coupled_motion.glslinc:364, ops 43/1): one x face at 40 m/s in the liquid makes
    the trial's dt at most CFL * hx / 40, and the step is accepted without a failure."""
    def fast(b, cfg):
        nx, ny, nz = cfg.n
        b[nx * ny * nz + (4 * ny + 3) * (nx + 1) + 12] = 40.0
    cfg, c = tank_with(fast)
    assert c[7] == 0 and c[2] == 1 and c[3] == 0
    assert 0.0 < c[20] <= cfg.cfl * cfg.spacing[0] / 40.0 * (1 + 1e-6)
    assert c[20] > 0.5 * cfg.cfl * cfg.spacing[0] / 40.0


@pytest.mark.parametrize("value", [float("nan"), -0.5])
def test_retries_exhaust_and_halt_on_a_poisoned_fraction(value):
    """A volume fraction outside [0, 1] (or NaN) fails the sweep bound (code 10,
    coupled_motion.glslinc:407); the trial is retried at half dt twice (c29 = 2 retries, dt 1/120
    -> 1/480), then the third rejection halts the solver with code 10 and no accepted step."""
    def poison(b, cfg):
        nx, ny, nz = cfg.n
        b[(4 * ny + 3) * nx + 12] = value
    cfg, c = tank_with(poison)
    assert c[7] == 10 and c[33] == 10 and c[29] == 2 and c[3] == 3 and c[2] == 0
    assert c[20] == pytest.approx(cfg.dt / 4, rel=1e-6)


def test_initial_surface_is_the_still_water_ramp_with_corrugation():
    """Op 0 (pressure_pass.glslinc:14-17) with the corrugated surface of pressure_core.glslinc:61:
    F = clamp(0.5 - (y_c - eta(x))/hy, 0, 1) with eta = eta0 + corrugation cos(2 pi (qx + 1/2)/nx)
    (the shader's 6.28318530718), unchanged by the rest of the initial commands; and the initial
    volume c26 is the sum of F times the cell volume.  Independent FP64 evaluation against the FP64
    oracle."""
    cfg = wg.config("default", n=(24, 24, 8), corrugation=0.03, corrugation_phase=0.0)
    nx, ny, nz = cfg.n
    hx, hy, hz = (float(v) for v in cfg.spacing)
    o = Oracle(cfg, 64)
    F = o.bank_d()[:nx * ny * nz].reshape(nz, ny, nx)
    eta = float(cfg.eta) + float(cfg.corrugation) * np.cos(6.28318530718 * (np.arange(nx) + 0.5) / nx)
    yc = float(cfg.origin[1]) + (np.arange(ny) + 0.5) * hy
    want = np.clip(0.5 - (yc[:, None] - eta[None, :]) / hy, 0.0, 1.0)
    assert 0.0 < want.mean() < 1.0 and np.unique(want).size > 10
    for z in range(nz):
        assert np.abs(F[z] - want).max() <= 1e-12
    assert o.control()[26] == pytest.approx(F.sum() * hx * hy * hz, rel=1e-12)


@pytest.mark.parametrize("preset", ["default", "beach", "tank"])
def test_oracle_presets_equal_the_product_presets(preset):
    """The oracle builds its configurations itself (oracle/wo_config.cpp, restating
    lab_runner.gd:19-26 and the GDScript defaults), so the CPU baseline never loads the product
    library; both sets of presets fill the struct with the same bits."""
    import ctypes as C
    from tests.oracle_ref import oracle_config
    mine, product = oracle_config(preset), wg.config(preset)
    assert C.string_at(C.addressof(mine), C.sizeof(mine)) == C.string_at(C.addressof(product), C.sizeof(product))
    assert lib().wo_dispersion_k(1.4, 0.45) == wg.dispersion_k(1.4, 0.45)
