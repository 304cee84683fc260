"""Training of the warm-start network on the GPU with the library's own kernels (k_train.cu), in
both arithmetics: gradients against the oracle's training step (oracle/wo_net.cpp, itself checked
against PyTorch autograd in tests/test_cpu_net.py), and Adam steps that fit a target."""
import numpy as np
import pytest

from tests.oracle_ref import net_gradients as oracle_gradients
from tests.test_cpu_net import close, random_batch
from waves_gb300.learned import CHANNELS, net_gradients, net_train


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [3, 4])
def test_gradients_match_oracle(gpu_lib, seed):
    """Same forward arithmetic (FP32, same order, BF16 roundings) and FP64 gradient sums in a
    different order: the output is identical and the gradients agree to 1e-5 of their scale."""
    x, t, m, weights, biases = random_batch(seed, B=2, n=(8, 6, 10))
    loss, gw, gb, y = net_gradients(x, t, m, weights, biases)
    oloss, ogw, ogb, oy = oracle_gradients(x, t, m, weights, biases)
    assert np.array_equal(y, oy)
    assert abs(loss - oloss) <= 1e-9 * abs(oloss)
    for l in range(4):
        for got, ref in ((gw[l], ogw[l]), (gb[l], ogb[l])):
            scale = max(float(np.abs(ref).max()), 1e-12)
            assert np.abs(got - ref).max() <= 1e-5 * scale, (l, np.abs(got - ref).max(), scale)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [3, 4])
def test_tensor_core_gradients_match_oracle(gpu_lib, seed):
    """WAVES_NET_TENSOR (implicit GEMM on mma.sync, BF16 gradients between layers) against the
    oracle's FP32 training step.  A numpy model of the BF16 gradient roundings puts the error at a
    median of 6e-4 and a maximum of 3.2e-3 of each gradient's scale on these batches; the bars
    leave a factor of 5 to 10 for the tensor cores' FP32 accumulation order."""
    x, t, m, weights, biases = random_batch(seed, B=2, n=(8, 6, 10))
    loss, gw, gb, y = net_gradients(x, t, m, weights, biases, tensor=True)
    oloss, ogw, ogb, oy = oracle_gradients(x, t, m, weights, biases)
    assert close(y, oy, typical=1e-4, worst=2e-2)
    assert abs(loss - oloss) <= 1e-3 * abs(oloss)
    for l in range(4):
        assert close(gw[l], ogw[l], typical=3e-3, worst=3e-2), l
        assert close(gb[l], ogb[l], typical=3e-3, worst=3e-2), l


@pytest.mark.gpu
@pytest.mark.parametrize("tensor", [False, True])
def test_adam_fits_a_teacher_network(gpu_lib, tensor):
    """Targets made by a random teacher network; a student started from other random weights
    loses more than half of the gap in 150 Adam steps on the GPU (measured with the exact
    arithmetic: 0.098 -> 0.030)."""
    x, _, m, teacher_w, teacher_b = random_batch(5, B=4, n=(12, 12, 12))
    m[:] = 1.0
    _, _, _, target = net_gradients(x, np.zeros_like(m), m, teacher_w, teacher_b)
    _, _, _, student_w, student_b = random_batch(6, B=1, n=(2, 2, 2))
    w, b, hist = net_train(x, target, m, student_w, student_b, 150, 3e-3, tensor=tensor)
    print(f"{'tensor' if tensor else 'exact'}: loss {hist[0]:.3e} -> {hist[-1]:.3e}")
    assert len(hist) == 150 and np.isfinite(hist).all()
    assert hist[-1] < 0.5 * hist[0], (hist[0], hist[-1])
    assert np.mean(hist[-10:]) < np.mean(hist[:10])
    loss_after, _, _, _ = net_gradients(x, target, m, w, b)
    assert loss_after <= hist[-1] * 1.5
    assert all(wl.shape == (co, 27, ci) for wl, (ci, co) in zip(w, CHANNELS))


@pytest.mark.gpu
@pytest.mark.parametrize("tensor", [False, True])
def test_training_is_bitwise_reproducible(gpu_lib, tensor):
    """Every sum of a training step (loss, weight and bias gradients) is reduced in a fixed order,
    so two runs of the same Adam steps give the same loss history and weights bit for bit."""
    x, t, m, weights, biases = random_batch(8, B=2, n=(10, 8, 12))
    runs = [net_train(x, t, m, weights, biases, 5, 3e-3, tensor=tensor) for _ in range(2)]
    (w0, b0, h0), (w1, b1, h1) = runs
    assert np.array_equal(h0, h1)
    for l in range(4):
        assert np.array_equal(w0[l], w1[l]) and np.array_equal(b0[l], b1[l]), l
