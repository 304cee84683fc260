"""Learned warm start: solve-pair capture, training and evaluation (waves_gb300.learned.train).

The network itself runs in the library (k_net.cu, waves_set_warm_start); this package produces
its weights, either with the library's own training kernels (k_train.cu: waves_net_gradients,
waves_net_train, wrapped below) or with PyTorch; the exported model is the BF16 weight layout of
include/waves.h.
"""
import ctypes as C

import numpy as np

CHANNELS = [(3, 16), (16, 16), (16, 16), (16, 1)]


def bf16_bits(a):
    """float32 -> BF16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def load_model(path):
    """(weights, biases, input_scale, output_scale) of a model file written by train.py."""
    z = np.load(path)
    weights = [z[f"w{l}"] for l in range(len(CHANNELS))]
    biases = [z[f"b{l}"] for l in range(len(CHANNELS))]
    return weights, biases, tuple(float(v) for v in z["input_scale"]), float(z["output_scale"])


def write_raw_model(npz_path, out_path):
    """The model of a train.py file as the raw file waves_run --model reads: b"WVNET1\\0\\0", per
    layer the BF16 weights [co][27][ci] (little-endian uint16) and the FP32 biases [co], then the
    three FP32 input scales and the FP32 output scale."""
    weights, biases, iscale, oscale = load_model(npz_path)
    with open(out_path, "wb") as f:
        f.write(b"WVNET1\0\0")
        for w, b, (ci, co) in zip(weights, biases, CHANNELS):
            w = np.asarray(w)
            bits = w.astype("<u2") if w.dtype == np.uint16 else bf16_bits(w).astype("<u2")
            assert bits.size == co * 27 * ci and np.asarray(b).size == co
            f.write(np.ascontiguousarray(bits).tobytes())
            f.write(np.asarray(b, dtype="<f4").tobytes())
        f.write(np.asarray(iscale, dtype="<f4").tobytes())
        f.write(np.asarray([oscale], dtype="<f4").tobytes())


def _batch(x, target, mask, tensor):
    from waves_gb300.abi import WAVES_NET_EXACT, WAVES_NET_TENSOR, WavesNetBatch
    fp = C.POINTER(C.c_float)
    x = np.ascontiguousarray(x, dtype=np.float32)
    target = np.ascontiguousarray(target, dtype=np.float32)
    mask = np.ascontiguousarray(mask, dtype=np.float32)
    B, ch, nz, ny, nx = x.shape
    assert ch == 3 and target.shape == (B, nz, ny, nx) and mask.shape == target.shape
    bt = WavesNetBatch(B, nz, ny, nx, x.ctypes.data_as(fp), target.ctypes.data_as(fp), mask.ctypes.data_as(fp),
                       WAVES_NET_TENSOR if tensor else WAVES_NET_EXACT)
    return bt, (x, target, mask)


def _ptrs(arrays):
    fp = C.POINTER(C.c_float)
    return (fp * len(arrays))(*[a.ctypes.data_as(fp) for a in arrays])


def net_gradients(x, target, mask, weights, biases, device=0, tensor=False):
    """One forward and backward pass on the GPU (waves_net_gradients): (loss, dL/dW per layer
    [co][27][ci], dL/db per layer, output y).  tensor: the tensor-core arithmetic
    (WAVES_NET_TENSOR) instead of the oracle's order (WAVES_NET_EXACT)."""
    import waves_gb300 as wg
    lib = wg.load()
    bt, keep = _batch(x, target, mask, tensor)
    ws = [np.ascontiguousarray(w, dtype=np.float32).reshape(co, 27, ci) for w, (ci, co) in zip(weights, CHANNELS)]
    bs = [np.ascontiguousarray(b, dtype=np.float32) for b in biases]
    gws = [np.zeros_like(w) for w in ws]
    gbs = [np.zeros_like(b) for b in bs]
    y = np.zeros(keep[1].shape, dtype=np.float32)
    loss = C.c_double()
    st = lib.waves_net_gradients(C.byref(bt), _ptrs(ws), _ptrs(bs), C.byref(loss), _ptrs(gws), _ptrs(gbs),
                                 y.ctypes.data_as(C.POINTER(C.c_float)), int(device))
    if st != 0:
        raise wg.WavesError(f"waves_net_gradients: status {st}")
    return loss.value, gws, gbs, y


def net_train(x, target, mask, weights, biases, iterations, learning_rate, device=0, tensor=False):
    """`iterations` Adam steps on the GPU (waves_net_train) from FP32 weights [co][27][ci] and biases;
    returns (weights, biases, loss per step).  tensor: as in net_gradients."""
    import waves_gb300 as wg
    lib = wg.load()
    bt, keep = _batch(x, target, mask, tensor)
    ws = [np.array(w, dtype=np.float32).reshape(co, 27, ci) for w, (ci, co) in zip(weights, CHANNELS)]
    bs = [np.array(b, dtype=np.float32) for b in biases]
    hist = np.zeros(max(int(iterations), 1), dtype=np.float64)
    st = lib.waves_net_train(C.byref(bt), _ptrs(ws), _ptrs(bs), int(iterations), float(learning_rate),
                             hist.ctypes.data_as(C.POINTER(C.c_double)), int(device))
    if st != 0:
        raise wg.WavesError(f"waves_net_train: status {st}")
    return ws, bs, hist[:int(iterations)]
