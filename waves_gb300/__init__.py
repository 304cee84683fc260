"""GB300-native waves solver step.

`load()` returns the in-tree C-ABI library (libwaves_gb300.so, built by waves_gb300/build.py);
`WavesSolver` is a thin Python handle over it, and `CoastalGPU` / `CoupledGPU` mirror the
GDScript classes of the reference (water/coastal_gpu.gd, water/coupled_gpu.gd,
water/pressure_gpu.gd) with the same method names and quota semantics.

There is no CPU fallback: every call goes through the CUDA library, and constructing a solver
without it (or without a CUDA device) raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .abi import WavesConfig, WavesStats, WAVES_CONTROL_SIZE

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libwaves_gb300.so")
_lib = None


def load(build_if_missing=False):
    """The product library, loaded once.  Raises if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError(f"waves_gb300 CUDA library missing: {LIB_PATH} (run waves_gb300/build.py)")
        from .build import build
        build()
    _lib = abi.declare(C.CDLL(LIB_PATH))
    return _lib


class WavesError(RuntimeError):
    pass


def _check(lib, status, h=None):
    if status != 0:
        msg = lib.waves_last_error(h)
        raise WavesError(f"{abi.STATUS.get(status, status)}: {msg.decode() if msg else ''}")


def config(preset="default", **overrides):
    """A WavesConfig from a preset ('default', 'beach', 'tank') with field overrides."""
    lib = load()
    cfg = WavesConfig()
    {"default": lib.waves_config_default, "beach": lib.waves_config_beach, "tank": lib.waves_config_tank}[preset](C.byref(cfg))
    for k, v in overrides.items():
        field = getattr(cfg, k)
        if hasattr(field, "__len__"):
            for i, x in enumerate(v):
                field[i] = x
        else:
            setattr(cfg, k, v)
    return cfg


def dispersion_k(period_s, depth_m):
    return load().waves_dispersion_k(period_s, depth_m)


def mg_plan(cfg):
    """The multigrid level plan waves_create builds for cfg (waves_mg_plan, no device needed): per
    level its size n, coarsening factors f, stencil size and whether its transfer aggregates."""
    lib = load()
    count = C.c_int32()
    _check(lib, lib.waves_mg_plan(C.byref(cfg), None, 0, C.byref(count)))
    out = (C.c_int32 * (8 * max(count.value, 1)))()
    _check(lib, lib.waves_mg_plan(C.byref(cfg), out, count.value, C.byref(count)))
    return [{"n": tuple(out[8 * l:8 * l + 3]), "f": tuple(out[8 * l + 3:8 * l + 6]), "stencil": out[8 * l + 6],
             "aggregate": bool(out[8 * l + 7])} for l in range(count.value)]


class WavesSolver:
    """One simulation on one CUDA device (a waves_handle)."""

    def __init__(self, cfg: WavesConfig):
        self.lib = load()
        self.cfg = cfg
        h = C.c_void_p()
        st = self.lib.waves_create(C.byref(cfg), C.byref(h))
        if st != 0:
            msg = self.lib.waves_last_error(None)
            raise WavesError(f"waves_create: {abi.STATUS.get(st, st)}: {msg.decode() if msg else ''}")
        self.h = h
        n = cfg.n
        self.N = n[0] * n[1] * n[2]
        self.NU = (n[0] + 1) * n[1] * n[2]
        self.NV = n[0] * (n[1] + 1) * n[2]
        self.NW = n[0] * n[1] * (n[2] + 1)
        self.NF = self.NU + self.NV + self.NW
        self.S = self.lib.waves_bank_floats(h)

    def close(self):
        if getattr(self, "h", None):
            self.lib.waves_destroy(self.h)
            self.h = None

    __del__ = close

    def _ck(self, st):
        _check(self.lib, st, self.h)

    def request_steps(self, steps):
        self._ck(self.lib.waves_request_steps(self.h, int(steps)))

    def request_time(self, seconds):
        self._ck(self.lib.waves_request_time(self.h, float(seconds)))

    def advance(self, trials):
        self._ck(self.lib.waves_advance(self.h, int(trials)))

    def run(self, trials_per_sync=4):
        st = self.lib.waves_run(self.h, int(trials_per_sync))
        if st not in (0, 4):
            self._ck(st)
        return st

    def frame(self, gpu_budget_ms=14.0, max_inflight=3, max_trials=96, cpu_budget_ms=4.0):
        """One frame of budgeted submission (waves_frame, after water/work_scheduler.gd:frame):
        never waits for the GPU; returns the frame report as a dict."""
        from .abi import WavesFrameBudget, WavesFrameReport
        b = WavesFrameBudget(float(gpu_budget_ms), int(max_inflight), int(max_trials), float(cpu_budget_ms))
        r = WavesFrameReport()
        self._ck(self.lib.waves_frame(self.h, C.byref(b), C.byref(r)))
        return r.as_dict()

    def frame_stats(self):
        """Telemetry of the latest retired frame submission (waves_frame_stats): no device access,
        no wait.  None while no submission has retired."""
        s = WavesStats()
        if self.lib.waves_frame_stats(self.h, C.byref(s)) != 0:
            return None
        return s.as_dict()

    def device_bytes(self):
        """Bytes of the handle's persistent device state (the size waves_save reports)."""
        n = C.c_size_t(0)
        self._ck(self.lib.waves_save(self.h, None, C.byref(n)))
        return int(n.value) - 16

    def synchronize(self):
        self._ck(self.lib.waves_synchronize(self.h))

    def stats(self):
        s = WavesStats()
        self._ck(self.lib.waves_stats(self.h, C.byref(s)))
        return s.as_dict()

    def control(self):
        c = (C.c_double * WAVES_CONTROL_SIZE)()
        self._ck(self.lib.waves_control(self.h, c, WAVES_CONTROL_SIZE))
        return np.frombuffer(c, dtype=np.float64).copy()

    def set_control(self, c):
        arr = np.ascontiguousarray(c, dtype=np.float64)
        self._ck(self.lib.waves_set_control(self.h, arr.ctypes.data_as(C.POINTER(C.c_double)), len(arr)))

    def set_warm_start(self, weights=None, biases=None, input_scale=(1.0, 1.0, 1.0), output_scale=1.0):
        """Load the warm-start network (waves_set_warm_start): weights[l] are BF16 bit patterns
        laid out [co][kz][ky][kx][ci] (channels 3, 16, 16, 16 in; 16, 16, 16, 1 out), biases[l]
        FP32; None turns the learned start off."""
        from .abi import WAVES_NET_LAYERS, WavesWarmStartModel
        if weights is None:
            self._ck(self.lib.waves_set_warm_start(self.h, None))
            return
        m = WavesWarmStartModel()
        keep = []
        for l in range(WAVES_NET_LAYERS):
            w = np.ascontiguousarray(weights[l], dtype=np.uint16).ravel()
            b = np.ascontiguousarray(biases[l], dtype=np.float32).ravel()
            keep += [w, b]
            m.weights[l] = w.ctypes.data_as(C.POINTER(C.c_uint16))
            m.bias[l] = b.ctypes.data_as(C.POINTER(C.c_float))
        for k in range(3):
            m.input_scale[k] = float(input_scale[k])
        m.output_scale = float(output_scale)
        self._ck(self.lib.waves_set_warm_start(self.h, C.byref(m)))

    def debug_phase(self, phase):
        self._ck(self.lib.waves_debug_phase(self.h, int(phase)))

    def debug_read(self, name, count, dtype=np.float32):
        out = np.empty(count, dtype=dtype)
        self._ck(self.lib.waves_debug_read(self.h, name.encode(), out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out

    def probe_trial(self):
        """Run one host-scheduled trial with kernel probes (waves_debug_probe_trial): per probed
        kernel, launches, summed CUDA-event milliseconds and summed algorithmic bytes."""
        from .abi import PROBE_KINDS, WavesKernelProbe
        out = (WavesKernelProbe * len(PROBE_KINDS))()
        trials = C.c_int32()
        self._ck(self.lib.waves_debug_probe_trial(self.h, out, len(PROBE_KINDS), C.byref(trials)))
        return trials.value, [{"kernel": PROBE_KINDS[k], "launches": out[k].launches, "ms": out[k].ms,
                               "bytes": out[k].bytes} for k in range(len(PROBE_KINDS))]

    def inject_rejection(self):
        self._ck(self.lib.waves_inject_rejection(self.h))

    def bank(self, which=-1):
        out = np.empty(self.S, dtype=np.float32)
        self._ck(self.lib.waves_get_bank(self.h, which, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def set_bank(self, which, data):
        arr = np.ascontiguousarray(data, dtype=np.float32)
        assert arr.size == self.S
        self._ck(self.lib.waves_set_bank(self.h, which, arr.ctypes.data_as(C.POINTER(C.c_float))))

    def geometry(self):
        phi = np.empty(self.N, dtype=np.float32)
        kind = np.empty(self.N, dtype=np.float32)
        self._ck(self.lib.waves_get_geometry(self.h, phi.ctypes.data_as(C.POINTER(C.c_float)),
                                             kind.ctypes.data_as(C.POINTER(C.c_float))))
        return phi, kind

    def masks(self):
        pm = np.empty(2 * self.N, dtype=np.float32)
        vb = np.empty(2 * self.NF, dtype=np.float32)
        self._ck(self.lib.waves_get_masks(self.h, pm.ctypes.data_as(C.POINTER(C.c_float)),
                                          vb.ctypes.data_as(C.POINTER(C.c_float))))
        return pm, vb

    def set_masks(self, pm, vb):
        pm = np.ascontiguousarray(pm, dtype=np.float32)
        vb = np.ascontiguousarray(vb, dtype=np.float32)
        self._ck(self.lib.waves_set_masks(self.h, pm.ctypes.data_as(C.POINTER(C.c_float)),
                                          vb.ctypes.data_as(C.POINTER(C.c_float))))

    def export_surface(self):
        planes = np.empty(4 * self.N, dtype=np.float32)
        kinds = np.empty(self.N, dtype=np.float32)
        self._ck(self.lib.waves_export_surface(self.h, planes.ctypes.data_as(C.POINTER(C.c_float)),
                                               kinds.ctypes.data_as(C.POINTER(C.c_float))))
        return planes.reshape(-1, 4), kinds

    def export_surface_device(self, planes_ptr, kinds_ptr, clock_ptr=None):
        """Enqueue the export into caller device buffers (waves_export_surface_device): planes
        float4[N], kinds float[N], clock float4 (accepted time, accepted steps, 0, 0) or None.
        Does not wait; order against other streams through `stream()`."""
        self._ck(self.lib.waves_export_surface_device(self.h, C.c_void_p(planes_ptr), C.c_void_p(kinds_ptr),
                                                      C.c_void_p(clock_ptr) if clock_ptr else None))

    def history(self):
        """waves_get_history: (per-trial rows (4 cap, 4), coastal rows (5 cap, 4), audit words)."""
        cap = max(self.cfg.history_capacity, 1)
        hist = np.empty(16 * cap, dtype=np.float32)
        coast = np.empty(20 * cap, dtype=np.float32)
        audit = np.empty(64 + 32 * cap, dtype=np.uint32)
        self._ck(self.lib.waves_get_history(self.h, hist.ctypes.data_as(C.POINTER(C.c_float)),
                                            coast.ctypes.data_as(C.POINTER(C.c_float)),
                                            audit.ctypes.data_as(C.POINTER(C.c_uint32))))
        return hist.reshape(-1, 4), coast.reshape(-1, 4), audit

    def render_params(self, width=1280, height=720, **overrides):
        """waves_render_params_default for this configuration, with field overrides."""
        from .abi import WavesRenderParams
        p = WavesRenderParams()
        self.lib.waves_render_params_default(C.byref(p), C.byref(self.cfg), int(width), int(height))
        for k, v in overrides.items():
            field = getattr(p, k)
            if hasattr(field, "__len__"):
                for i, x in enumerate(v):
                    field[i] = x
            else:
                setattr(p, k, v)
        return p

    def render(self, params=None, trace=False):
        """Export + ray-march (waves_render): an (H, W, 4) float32 RGBA image, and with trace=True
        also the (H, W, 4) trace image (first entry, occupied length, first exit, queries)."""
        p = params if params is not None else self.render_params()
        img = np.empty((p.height, p.width, 4), dtype=np.float32)
        tr = np.empty((p.height, p.width, 4), dtype=np.float32) if trace else None
        self._ck(self.lib.waves_render(self.h, C.byref(p), img.ctypes.data_as(C.POINTER(C.c_float)),
                                       tr.ctypes.data_as(C.POINTER(C.c_float)) if trace else None))
        return (img, tr) if trace else img

    def render_device(self, params, rgba_ptr, trace_ptr=None):
        self._ck(self.lib.waves_render_device(self.h, C.byref(params), C.c_void_p(rgba_ptr),
                                              C.c_void_p(trace_ptr) if trace_ptr else None))

    def stream(self):
        return self.lib.waves_stream(self.h)

    def save(self):
        n = C.c_size_t(0)
        self._ck(self.lib.waves_save(self.h, None, C.byref(n)))
        buf = np.empty(n.value, dtype=np.uint8)
        self._ck(self.lib.waves_save(self.h, buf.ctypes.data_as(C.c_void_p), C.byref(n)))
        return buf

    def load(self, buf):
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        self._ck(self.lib.waves_load(self.h, buf.ctypes.data_as(C.c_void_p), buf.size))

    def split_bank(self, b):
        """F, u, v, w, p views of a bank array (x-fastest flat arrays)."""
        N, NU, NV, NW = self.N, self.NU, self.NV, self.NW
        return b[:N], b[N:N + NU], b[N + NU:N + NU + NV], b[N + NU + NV:N + NU + NV + NW], b[N + NU + NV + NW:]


from .gd import CoastalGPU, CoupledGPU, PressureGPU  # noqa: E402,F401
