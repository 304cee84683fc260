"""Test-side access to the CPU oracle (oracle/libwaves_oracle.so via ctypes).

Tests compare the CUDA library against the oracle; nothing in the product imports it.  `build()` compiles it with oracle/Makefile when the library is missing or stale.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from waves_gb300.abi import WavesConfig, WavesRenderParams, WAVES_CONTROL_SIZE

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB = os.path.join(ORACLE_DIR, "_build", "libwaves_oracle.so")
_lib = None


def build():
    srcs = [os.path.join(ORACLE_DIR, f) for f in os.listdir(ORACLE_DIR) if f.startswith("wo_")]
    srcs.append(os.path.join(ROOT, "include", "waves.h"))
    if not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in srcs):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, dp, fp = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_float)
        sig = {
            "wo_create": (vp, [C.POINTER(WavesConfig), C.c_int]),
            "wo_destroy": (None, [vp]),
            "wo_set_quota": (None, [vp, C.c_double]),
            "wo_run": (C.c_int, [vp, C.c_int]),
            "wo_batch": (None, [vp]),
            "wo_get_control": (None, [vp, dp]),
            "wo_set_control": (None, [vp, dp]),
            "wo_bank_floats": (C.c_size_t, [vp]),
            "wo_get_bank": (None, [vp, C.c_int, fp]),
            "wo_get_bank_d": (None, [vp, C.c_int, dp]),
            "wo_set_bank": (None, [vp, C.c_int, fp]),
            "wo_get_geometry": (None, [vp, fp, fp]),
            "wo_get_masks": (None, [vp, fp, fp]),
            "wo_set_masks": (None, [vp, fp, fp]),
            "wo_set_geometry": (None, [vp, fp, fp]),
            "wo_get_export": (None, [vp, fp, fp]),
            "wo_render": (None, [fp, fp, C.POINTER(WavesConfig), C.POINTER(WavesRenderParams), C.c_float, fp, fp]),
            "wo_get_probes": (None, [vp, fp]),
            "wo_mg_levels": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
            "wo_mg_stencil": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int)]),
            "wo_mg_state": (None, [vp, C.POINTER(C.c_uint32)]),
            "wo_get_history": (None, [vp, fp, fp]),
            "wo_mg_audit": (None, [vp, C.POINTER(C.c_uint32), C.c_size_t]),
            "wo_net_gradients": (C.c_double, [C.c_int, C.c_int, C.c_int, C.c_int, fp, fp, fp, C.POINTER(fp),
                                              C.POINTER(fp), C.POINTER(fp), C.POINTER(fp), fp]),
            "wo_cube_volume": (C.c_float, [C.c_float] * 4),
            "wo_inverse_volume": (C.c_float, [C.c_float] * 4),
            "wo_cube_volume_d": (C.c_double, [C.c_double] * 4),
            "wo_inverse_volume_d": (C.c_double, [C.c_double] * 4),
            "wo_time_batches": (C.c_double, [vp, C.c_int]),
            "wo_set_threads": (C.c_int, [C.c_int]),
            "wo_phase": (None, [vp, C.c_int]),
            "wo_read": (C.c_int, [vp, C.c_char_p, fp]),
            "wo_dispersion_k": (C.c_double, [C.c_double, C.c_double]),
            "wo_config_default": (None, [C.POINTER(WavesConfig)]),
            "wo_config_beach": (None, [C.POINTER(WavesConfig)]),
            "wo_config_tank": (None, [C.POINTER(WavesConfig)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def oracle_config(preset="default", **overrides):
    """A WavesConfig from the oracle's own presets (oracle/wo_config.cpp: 'default', 'beach',
    'tank'), with field overrides; the product library is not loaded."""
    L = lib()
    cfg = WavesConfig()
    {"default": L.wo_config_default, "beach": L.wo_config_beach, "tank": L.wo_config_tank}[preset](C.byref(cfg))
    for k, v in overrides.items():
        field = getattr(cfg, k)
        if hasattr(field, "__len__"):
            for i, x in enumerate(v):
                field[i] = x
        else:
            setattr(cfg, k, v)
    return cfg


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Oracle:
    """One oracle simulation (precision 32 = FP32 decision parity, 64 = FP64 error reference)."""

    def __init__(self, cfg: WavesConfig, precision=32):
        self.L = lib()
        self.cfg = cfg
        self.h = self.L.wo_create(C.byref(cfg), precision)
        n = cfg.n
        self.N = n[0] * n[1] * n[2]
        self.NF = (n[0] + 1) * n[1] * n[2] + n[0] * (n[1] + 1) * n[2] + n[0] * n[1] * (n[2] + 1)
        self.S = self.L.wo_bank_floats(self.h)
        self.cap = max(cfg.history_capacity, 0)

    def close(self):
        if self.h:
            self.L.wo_destroy(self.h)
            self.h = None

    __del__ = close

    def request_steps(self, n):
        self.L.wo_set_quota(self.h, float(n))

    def request_time(self, t):
        self.L.wo_set_quota(self.h, -float(t))

    def run(self, max_batches=100000):
        return self.L.wo_run(self.h, max_batches)

    def control(self):
        c = np.zeros(WAVES_CONTROL_SIZE)
        self.L.wo_get_control(self.h, c.ctypes.data_as(C.POINTER(C.c_double)))
        return c

    def set_control(self, c):
        c = np.ascontiguousarray(c, dtype=np.float64)
        self.L.wo_set_control(self.h, c.ctypes.data_as(C.POINTER(C.c_double)))

    def bank(self, which=-1):
        if which < 0:
            which = int(self.control()[0])
        out = np.empty(self.S, dtype=np.float32)
        self.L.wo_get_bank(self.h, which, _fp(out))
        return out

    def bank_d(self, which=-1):
        if which < 0:
            which = int(self.control()[0])
        out = np.empty(self.S, dtype=np.float64)
        self.L.wo_get_bank_d(self.h, which, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def set_bank(self, which, data):
        self.L.wo_set_bank(self.h, which, _fp(np.ascontiguousarray(data, dtype=np.float32)))

    def geometry(self):
        phi = np.empty(self.N, dtype=np.float32)
        kind = np.empty(self.N, dtype=np.float32)
        self.L.wo_get_geometry(self.h, _fp(phi), _fp(kind))
        return phi, kind

    def set_geometry(self, phi, kind):
        self.L.wo_set_geometry(self.h, _fp(np.ascontiguousarray(phi, dtype=np.float32)),
                               _fp(np.ascontiguousarray(kind, dtype=np.float32)))

    def masks(self):
        pm = np.empty(2 * self.N, dtype=np.float32)
        vb = np.empty(2 * self.NF, dtype=np.float32)
        self.L.wo_get_masks(self.h, _fp(pm), _fp(vb))
        return pm, vb

    def set_masks(self, pm, vb):
        self.L.wo_set_masks(self.h, _fp(np.ascontiguousarray(pm, dtype=np.float32)),
                            _fp(np.ascontiguousarray(vb, dtype=np.float32)))

    def export(self):
        planes = np.empty(4 * self.N, dtype=np.float32)
        kinds = np.empty(self.N, dtype=np.float32)
        self.L.wo_get_export(self.h, _fp(planes), _fp(kinds))
        return planes.reshape(-1, 4), kinds

    def phase(self, k):
        self.L.wo_phase(self.h, k)

    def read(self, name, count):
        out = np.empty(count, dtype=np.float32)
        assert self.L.wo_read(self.h, name.encode(), _fp(out)), name
        return out

    def probes(self):
        out = np.empty(32, dtype=np.float32)
        self.L.wo_get_probes(self.h, _fp(out))
        return out.reshape(8, 4)

    def history(self):
        h = np.empty(16 * self.cap, dtype=np.float32)
        ch = np.empty(20 * self.cap, dtype=np.float32)
        self.L.wo_get_history(self.h, _fp(h), _fp(ch))
        return h.reshape(-1, 4), ch.reshape(-1, 4)

    def audit(self):
        words = 64 + 32 * max(self.cap, 1)
        out = np.zeros(words, dtype=np.uint32)
        self.L.wo_mg_audit(self.h, out.ctypes.data_as(C.POINTER(C.c_uint32)), words)
        return out

    def levels(self):
        dims = (C.c_int * 36)()
        st = (C.c_int * 12)()
        n = self.L.wo_mg_levels(self.h, dims, st)
        return [((dims[3 * l], dims[3 * l + 1], dims[3 * l + 2]), st[l]) for l in range(n)]

    def mg_state(self):
        out = (C.c_uint32 * 32)()
        self.L.wo_mg_state(self.h, out)
        return list(out)


def render(planes, kinds, cfg, params, clock_time):
    """The oracle's ray-march of an op-19 export (oracle/wo_render.cpp): (H, W, 4) RGBA and trace."""
    L = lib()
    fp = C.POINTER(C.c_float)
    planes = np.ascontiguousarray(planes, dtype=np.float32)
    kinds = np.ascontiguousarray(kinds, dtype=np.float32)
    img = np.empty((params.height, params.width, 4), dtype=np.float32)
    tr = np.empty_like(img)
    L.wo_render(planes.ctypes.data_as(fp), kinds.ctypes.data_as(fp), C.byref(cfg), C.byref(params),
                float(np.float32(clock_time)), img.ctypes.data_as(fp), tr.ctypes.data_as(fp))
    return img, tr


NET_CHANNELS = [(3, 16), (16, 16), (16, 16), (16, 1)]


def net_gradients(x, target, mask, weights, biases):
    """The oracle's training step (oracle/wo_net.cpp): loss, per-layer dL/dW [co][27][ci] and dL/db,
    and the output, for a batch x[b][3][z][y][x] with FP32 weights."""
    L = lib()
    fp = C.POINTER(C.c_float)
    x = np.ascontiguousarray(x, dtype=np.float32)
    B, _, nz, ny, nx = x.shape
    target = np.ascontiguousarray(target, dtype=np.float32)
    mask = np.ascontiguousarray(mask, dtype=np.float32)
    ws = [np.ascontiguousarray(w, dtype=np.float32) for w in weights]
    bs = [np.ascontiguousarray(b, dtype=np.float32) for b in biases]
    gws = [np.zeros_like(w) for w in ws]
    gbs = [np.zeros_like(b) for b in bs]
    y = np.zeros((B, nz, ny, nx), dtype=np.float32)
    arr = lambda lst: (fp * len(lst))(*[a.ctypes.data_as(fp) for a in lst])
    loss = L.wo_net_gradients(B, nz, ny, nx, x.ctypes.data_as(fp), target.ctypes.data_as(fp), mask.ctypes.data_as(fp),
                              arr(ws), arr(bs), arr(gws), arr(gbs), y.ctypes.data_as(fp))
    return loss, gws, gbs, y
