"""Learned warm start: solve-pair capture, training and evaluation (waves_gb300.learned.train).

The network itself runs in the library (k_net.cu, waves_set_warm_start); this package produces
its weights.  Training is offline and uses PyTorch on the GPU; the exported model is the BF16
weight layout of include/waves.h.
"""
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
