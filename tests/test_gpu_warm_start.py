"""Learned warm start: the tensor-core network against a PyTorch FP32 reference of the same op,
and the solver with a network loaded (the residual guard keeps plain MGPCG as the fallback)."""
import numpy as np
import pytest

import waves_gb300 as wg
from tests.cases import beach_slope
from tests.oracle_ref import Oracle
from tests.test_gpu_accuracy import F_TOLERANCE, split

CHANNELS = [(3, 16), (16, 16), (16, 16), (16, 1)]


def bf16_bits(a):
    """float32 -> BF16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def bf16_float(bits):
    return (np.asarray(bits, dtype=np.uint32) << 16).view(np.float32)


def random_model(seed):
    rng = np.random.default_rng(seed)
    weights, biases = [], []
    for ci, co in CHANNELS:
        w = rng.normal(0.0, 1.0 / np.sqrt(27 * ci), size=(co, 3, 3, 3, ci)).astype(np.float32)
        weights.append(bf16_bits(w))
        biases.append(rng.normal(0.0, 0.1, size=co).astype(np.float32))
    return weights, biases


def reference(F, b, p, kind, n, weights, biases, iscale, oscale):
    """The same network in PyTorch FP32 with the kernels' BF16 roundings (inputs, weights,
    activations between layers); zero padding; p + oscale * y on wet cells."""
    torch = pytest.importorskip("torch")
    nx, ny, nz = n
    grid = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32).reshape(nz, ny, nx))
    x = torch.stack([grid(F) * iscale[0], grid(b) * iscale[1], grid(p) * iscale[2]])[None]
    x = torch.from_numpy(bf16_float(bf16_bits(x.numpy())))
    for l, (ci, co) in enumerate(CHANNELS):
        w = torch.from_numpy(bf16_float(weights[l]).reshape(co, 3, 3, 3, ci)).permute(0, 4, 1, 2, 3).contiguous()
        x = torch.nn.functional.conv3d(x, w, torch.from_numpy(biases[l]), padding=1)
        if l < 3:
            x = torch.from_numpy(bf16_float(bf16_bits(torch.relu(x).numpy())))
    y = x[0, 0].numpy().ravel().astype(np.float64)
    return np.where(kind > 0, p + oscale * y, p)


@pytest.mark.gpu
@pytest.mark.parametrize("form,nx", [("tcgen05", 64), ("tcgen05", 200), ("sync", 64)])
def test_network_matches_fp32_reference(gpu_lib, monkeypatch, form, nx):
    """Both forms of the layers (tcgen05 with tensor-memory accumulators, the default; mma.sync):
    one block row of 128 cells partly past the grid's x extent (64 cells) and one spanning two
    blocks (200)."""
    monkeypatch.setenv("WAVES_NET_MMA", form)
    cfg = wg.config("beach", n=(nx, 40, 8), origin=(0.5, -0.6, -0.2), warm_start=1)
    s = wg.WavesSolver(cfg)
    weights, biases = random_model(7)
    iscale, oscale = (1.0, 1e-3, 1e-3), 10.0
    s.set_warm_start(weights, biases, iscale, oscale)
    s.request_steps(1)
    for phase in range(7):  # begin .. projection set-up (op 2)
        s.debug_phase(phase)
    n = tuple(cfg.n)
    N = n[0] * n[1] * n[2]
    cand = 1 - int(s.control()[0])
    bank = s.bank(cand)
    F, p_prev = bank[:N].astype(np.float64), bank[-N:].astype(np.float64)
    kind = s.geometry()[1]
    s.debug_phase(12)  # right-hand side, the four layers, the residual guard
    b = s.debug_read("b", N).astype(np.float64)
    p_net = s.debug_read("net_pressure", N).astype(np.float64)
    ref = reference(F, b, p_prev, kind, n, weights, biases, iscale, oscale)
    wet = kind > 0
    assert wet.any()
    scale = np.max(np.abs(ref - p_prev)[wet])
    err = np.abs(p_net - ref)
    # FP32 accumulation order differs (mma vs PyTorch); a BF16 rounding of an activation may then
    # land one step apart, so bound the worst case loosely and the typical case tightly
    assert np.max(err[wet]) <= 2e-2 * scale, (np.max(err[wet]), scale)
    assert np.median(err[wet]) <= 1e-4 * scale, (np.median(err[wet]), scale)
    assert np.array_equal(p_net[~wet], p_prev[~wet])
    s.close()


@pytest.mark.gpu
def test_solver_with_network_stays_within_fp64_bars(gpu_lib):
    """A (random) network either wins the residual comparison or is ignored; either way the CG
    converges to the same tolerance and F stays within the drift bar of the FP64 oracle."""
    cfg = beach_slope(warm_start=1)
    g = wg.WavesSolver(cfg)
    weights, biases = random_model(11)
    g.set_warm_start(weights, biases, (1.0, 1e-3, 1e-3), 1.0)
    o = Oracle(beach_slope(), 64)
    for step in range(1, 5):
        g.request_steps(step)
        g.run()
        o.request_steps(step)
        o.run()
        assert g.control()[2] == step and g.stats()["failure"] == 0
        Fg = split(g.bank().astype(np.float64), tuple(cfg.n))[0]
        Fo = split(o.bank_d(), tuple(cfg.n))[0]
        assert np.max(np.abs(Fg - Fo)) <= F_TOLERANCE
    print(f"warm start used in {g.stats()['warm_start_used']} of {int(g.control()[32])} trials")


@pytest.mark.gpu
def test_trained_network_gain_over_plain_mgpcg(gpu_lib):
    """What the shipped network (waves_gb300/learned/model_beach.npz) gains on a held-out beach
    (seed 101 of the capture's amplitude/period draws, 60 steps from t = 1 s, CG relres 1e-6):
    the same run with and without it.  The residual guard only takes the network where its
    initial residual is smaller, so it must not cost CG iterations; the gain is reported.
    Measured on a GB300: in these 60 steps the network is taken in 0 of 60 trials (13.78
    iterations per step both ways); over 120 steps, in 34 of 120 (14.24 against 14.35)."""
    import os
    from waves_gb300.learned import load_model
    from waves_gb300.learned.train import beach

    path = os.path.join(os.path.dirname(wg.__file__), "learned", "model_beach.npz")
    weights, biases, iscale, oscale = load_model(path)
    steps, out = 60, {}
    for warm in (0, 1):
        cfg, _, _ = beach(101, warm)
        s = wg.WavesSolver(cfg)
        if warm:
            s.set_warm_start(weights, biases, iscale, oscale)
        s.request_time(1.0)
        s.run()
        c0 = s.control()
        s.request_steps(int(c0[2]) + steps)
        s.run()
        c1 = s.control()
        assert c1[2] == c0[2] + steps and s.stats()["failure"] == 0
        out[warm] = ((c1[18] - c0[18]) / steps, int(c1[102] - c0[102]), int(c1[32] - c0[32]))
        s.close()
    (plain, _, _), (learned, used, trials) = out[0], out[1]
    print(f"plain {plain:.2f} it/step, learned {learned:.2f} it/step, network taken in {used} of {trials} trials")
    assert 0 <= used <= trials
    if used == 0:
        assert learned == plain  # never taken: the run is the plain run, bit for bit
    assert learned <= plain + 0.5
