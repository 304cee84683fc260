"""Test-side access to the reference's own shaders run on the host (oracle/_ref/libwaves_ref.so,
built by oracle/glsl/Makefile from the reference checkout's GLSL sources).

Two uses:
- lockstep: every dispatch unit of the reference's command lists runs through the reference's
  shader code and through the oracle from the same state, and every buffer is compared
  (oracle/glsl/ref_lockstep.cpp);
- free run: the reference's shaders alone, on their own FP32 control block and workgroup sums, to
  compare its decisions with the oracle's (FP64 control block and sums) over a long run.

The library exists only where the reference checkout does (this container): callers skip without
it.  It is test infrastructure, like the oracle.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from waves_gb300.abi import WavesConfig

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHADERS = os.environ.get("WAVES_REFERENCE_SHADERS", "/root/reference/water/shaders/compute")
LIB = os.path.join(ROOT, "oracle", "_ref", "libwaves_ref.so")
_lib = None


def available():
    return os.path.isdir(SHADERS)


def lib():
    global _lib
    if _lib is None:
        subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle", "glsl"), f"REF={SHADERS}"], check=True)
        L = C.CDLL(LIB)
        vp = C.c_void_p
        sig = {
            "ref_create": (vp, [C.POINTER(WavesConfig)]),
            "ref_free_create": (vp, [C.POINTER(WavesConfig)]),
            "ref_destroy": (None, [vp]),
            "ref_set_quota": (None, [vp, C.c_double]),
            "ref_run": (C.c_int, [vp, C.c_int]),
            "ref_free_run": (C.c_int, [vp, C.c_double, C.c_int]),
            "ref_free_control": (None, [vp, C.POINTER(C.c_float)]),
            "ref_free_bank": (None, [vp, C.c_int, C.POINTER(C.c_float)]),
            "ref_get_control": (None, [vp, C.POINTER(C.c_double)]),
            "ref_report": (C.c_int, [vp, C.c_char_p, C.c_int]),
            "ref_totals": (None, [vp, C.POINTER(C.c_long)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def reference_expressible(cfg):
    """The reference's push constants have no surface phase and hard-code the CFL number 0.45
    (pressure_core.glslinc:80, coupled_motion.glslinc:364)."""
    return cfg.corrugation_phase == 0.0 and abs(cfg.cfl - 0.45) < 1e-7


class Lockstep:
    """The oracle and the reference's shaders in lockstep (one comparison per dispatch unit)."""

    def __init__(self, cfg):
        assert reference_expressible(cfg)
        self.L = lib()
        self.h = self.L.ref_create(C.byref(cfg))

    def run_steps(self, steps):
        self.L.ref_set_quota(self.h, float(steps))
        return self.L.ref_run(self.h, 100000)

    def control(self):
        c = np.zeros(128)
        self.L.ref_get_control(self.h, c.ctypes.data_as(C.POINTER(C.c_double)))
        return c

    def report(self):
        buf = C.create_string_buffer(1 << 20)
        bad = self.L.ref_report(self.h, buf, len(buf))
        return bad, buf.value.decode()

    def totals(self):
        t = (C.c_long * 4)()
        self.L.ref_totals(self.h, t)
        return {"units": t[0], "exact": t[1], "within": t[2], "mismatched": t[3]}

    def close(self):
        if self.h:
            self.L.ref_destroy(self.h)
            self.h = None

    __del__ = close


class FreeReference:
    """The reference's shaders alone, from their own initial commands."""

    def __init__(self, cfg):
        assert reference_expressible(cfg)
        self.L = lib()
        self.h = self.L.ref_free_create(C.byref(cfg))
        n = cfg.n
        N = n[0] * n[1] * n[2]
        self.S = 2 * N + (n[0] + 1) * n[1] * n[2] + n[0] * (n[1] + 1) * n[2] + n[0] * n[1] * (n[2] + 1)

    def request_steps(self, steps):
        self.quota = float(steps)

    def run(self):
        return self.L.ref_free_run(self.h, self.quota, 100000)

    def control(self):
        c = np.zeros(96, dtype=np.float32)
        self.L.ref_free_control(self.h, c.ctypes.data_as(C.POINTER(C.c_float)))
        return c

    def bank(self, which=-1):
        if which < 0:
            which = int(self.control()[0])
        out = np.empty(self.S, dtype=np.float32)
        self.L.ref_free_bank(self.h, which, out.ctypes.data_as(C.POINTER(C.c_float)))
        return out

    def close(self):
        if self.h:
            self.L.ref_destroy(self.h)
            self.h = None

    __del__ = close
