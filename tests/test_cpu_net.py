"""The oracle's training step of the warm-start network (oracle/wo_net.cpp) against PyTorch
autograd in FP32 on the CPU: the same network with the same BF16 roundings (inputs, weights and
activations rounded, gradients passed through the roundings unchanged)."""
import numpy as np
import pytest

from tests.oracle_ref import NET_CHANNELS, net_gradients


def bf16(a):
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16).astype(np.uint32).view(np.float32)


def random_batch(seed, B=2, n=(6, 5, 7)):
    rng = np.random.default_rng(seed)
    nz, ny, nx = n
    x = rng.normal(size=(B, 3, nz, ny, nx)).astype(np.float32)
    t = rng.normal(size=(B, nz, ny, nx)).astype(np.float32)
    m = (rng.random(size=(B, nz, ny, nx)) < 0.7).astype(np.float32)
    weights, biases = [], []
    for ci, co in NET_CHANNELS:
        weights.append(rng.normal(0.0, 1.0 / np.sqrt(27 * ci), size=(co, 27, ci)).astype(np.float32))
        biases.append(rng.normal(0.0, 0.1, size=co).astype(np.float32))
    return x, t, m, weights, biases


def torch_reference(x, t, m, weights, biases):
    torch = pytest.importorskip("torch")

    class Round(torch.autograd.Function):
        @staticmethod
        def forward(ctx, v):
            return torch.from_numpy(bf16(v.detach().numpy()))

        @staticmethod
        def backward(ctx, g):
            return g

    ws = [torch.tensor(w, requires_grad=True) for w in weights]
    bs = [torch.tensor(b, requires_grad=True) for b in biases]
    a = Round.apply(torch.from_numpy(x))
    for l, (ci, co) in enumerate(NET_CHANNELS):
        # [co][27][ci] with tap t = (kz*3+ky)*3+kx -> conv3d weight [co][ci][kz][ky][kx]
        w = Round.apply(ws[l]).reshape(co, 3, 3, 3, ci).permute(0, 4, 1, 2, 3)
        z = torch.nn.functional.conv3d(a, w, bs[l], padding=1)
        a = Round.apply(torch.relu(z)) if l < 3 else z
    y = a[:, 0]
    mt, tt = torch.from_numpy(m), torch.from_numpy(t)
    loss = (mt * (y - tt) ** 2).sum() / max(float(m.sum()), 1.0)
    loss.backward()
    return float(loss.detach()), [w.grad.numpy() for w in ws], [b.grad.numpy() for b in bs], y.detach().numpy()


def close(a, ref, typical=1e-4, worst=2e-2):
    """FP32 accumulation orders differ (PyTorch vs the oracle), so a BF16 rounding of an activation
    may land one step apart: the typical element is held tightly, the worst one loosely."""
    scale = max(float(np.abs(ref).max()), 1e-12)
    err = np.abs(np.asarray(a, dtype=np.float64) - ref)
    return err.max() <= worst * scale and np.median(err) <= typical * scale


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_oracle_gradients_match_autograd(seed):
    x, t, m, weights, biases = random_batch(seed)
    loss, gw, gb, y = net_gradients(x, t, m, weights, biases)
    rloss, rgw, rgb, ry = torch_reference(x, t, m, weights, biases)
    assert close(y, ry)
    assert abs(loss - rloss) <= 1e-3 * abs(rloss)
    for l in range(4):
        assert close(gw[l], rgw[l]), l
        assert close(gb[l], rgb[l]), l
