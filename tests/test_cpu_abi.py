"""The C-ABI library loads and exports every function that include/*.h declares (no GPU calls)."""
import ctypes
import os
import re

import waves_gb300
from waves_gb300.abi import WAVES_ABI_SYMBOLS
from waves_gb300.build import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(waves_\w+)\s*\(", text))


def test_library_exports_every_declared_symbol():
    lib_path = build()
    lib = ctypes.CDLL(lib_path)
    names = declared("waves.h") | declared("waves_debug.h")
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_symbol_list_matches_header():
    assert set(WAVES_ABI_SYMBOLS) == declared("waves.h")


def test_probe_kind_names_match_the_library():
    """One name per probe kind of the library (kernels.h numbers them up to kProbeCount), in the
    order the debug header lists them."""
    from waves_gb300.abi import PROBE_KINDS
    text = open(os.path.join(ROOT, "waves_gb300", "csrc", "kernels.h")).read()
    kinds = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(kProbe\w+)\s*=\s*(\d+)", text)}
    assert kinds["kProbeCount"] == len(PROBE_KINDS)
    assert PROBE_KINDS[kinds["kProbeRowThread"]] == "k_mgl4"
    assert PROBE_KINDS[kinds["kProbeRows"]] == "k_mgl_rows"
    assert PROBE_KINDS[kinds["kProbeLeg"]] == "k_mg_leg"


def test_presets_without_gpu():
    lib = waves_gb300.load(build_if_missing=True)
    beach = waves_gb300.config("beach")
    assert tuple(beach.n) == (310, 48, 80)
    assert abs(beach.wave[1] - 2.52502) < 1e-4  # lab_runner.gd:19-25 dispersion, T = 1.4 s, h = 0.45 m
    tank = waves_gb300.config("tank")
    assert tank.coastal == 0 and abs(tank.cfl - 0.5) < 1e-7 and abs(tank.pressure_tolerance - 1e-6) < 1e-12
    assert abs(lib.waves_dispersion_k(1.4, 0.45) - 2.525) < 1e-3


def test_create_rejects_invalid_configurations_before_touching_a_device():
    """waves_create checks the configuration before it looks for a device: every invalid field
    gives WAVES_INVALID_ARG (1) with no handle, here as on a GPU host; a valid one without a GPU
    gives WAVES_NO_DEVICE (3), never a CPU fallback."""
    import ctypes as C
    lib = waves_gb300.load(build_if_missing=True)
    bad = [("n", (1, 16, 8)), ("n", (16, 1, 8)), ("n", (16, 16, 0)), ("spacing", (0.0, 0.05, 0.05)),
           ("spacing", (0.05, -0.05, 0.05)), ("spacing", (0.05, 0.05, float("nan"))), ("dt", 0.0),
           ("mg_smoothing", 0), ("mg_smoothing", 9), ("mg_lag", 0), ("mg_precision", 8),
           ("iterations_per_batch", 0)]
    for field, value in bad:
        cfg = waves_gb300.config("tank")
        if isinstance(value, tuple):
            for i, x in enumerate(value):
                getattr(cfg, field)[i] = x
        else:
            setattr(cfg, field, value)
        h = C.c_void_p(1)
        assert lib.waves_create(C.byref(cfg), C.byref(h)) == 1, (field, value)
        assert not h.value, (field, value)
    assert lib.waves_create(None, C.byref(C.c_void_p())) == 1
    import torch
    if not torch.cuda.is_available():
        h = C.c_void_p(1)
        assert lib.waves_create(C.byref(waves_gb300.config("tank")), C.byref(h)) == 3
        assert not h.value


def test_create_without_device_fails_cleanly(monkeypatch):
    # No GPU in this container: waves_create must report an error, not crash or fall back.
    import torch
    if torch.cuda.is_available():
        return
    import pytest
    with pytest.raises(waves_gb300.WavesError):
        waves_gb300.WavesSolver(waves_gb300.config("tank"))


def test_harness_argument_and_device_errors():
    """The C harness (built by build()) exits 1 on a bad argument and 2, with the library's
    message, when there is no usable device."""
    import subprocess
    from waves_gb300.build import HARNESS, build
    build()
    r = subprocess.run([HARNESS, "--bogus"], capture_output=True, text=True)
    assert r.returncode == 1 and "usage" in r.stderr
    import torch
    r = subprocess.run([HARNESS, "--preset", "ocean"], capture_output=True, text=True)
    assert r.returncode == 1 and "unknown preset" in r.stderr
    if not torch.cuda.is_available():
        for preset in ("tank", "beach", "large"):
            r = subprocess.run([HARNESS, "--preset", preset, "--steps", "1"], capture_output=True, text=True)
            assert r.returncode == 2 and "waves_create" in r.stderr, preset


def test_render_defaults_without_gpu():
    """waves_render_params_default: water.gdshader's look and presentation.gd's camera_preset(1),
    the wide view when the domain is deeper than 1 m in z."""
    import ctypes as C
    from waves_gb300.abi import WavesRenderParams
    lib = waves_gb300.load(build_if_missing=True)
    p = WavesRenderParams()
    beach = waves_gb300.config("beach")
    lib.waves_render_params_default(C.byref(p), C.byref(beach), 640, 360)
    assert (p.width, p.height, p.mode, p.orthographic) == (640, 360, 1, 1)
    assert max(abs(a - b) for a, b in zip(p.target, (2.15, -0.12, 0.0))) < 1e-6
    assert max(abs(a - b) for a, b in zip(p.eye, (2.15 + 2.5, -0.12 + 4.45, 5.7))) < 1e-5 and abs(p.size - 5.25) < 1e-6
    assert abs(p.attenuation_distance - 0.18) < 1e-7 and abs(p.surface_roughness - 0.3) < 1e-7
    tank = waves_gb300.config("tank")  # 16 x 0.05 m = 0.8 m deep in z: the close view
    lib.waves_render_params_default(C.byref(p), C.byref(tank), 64, 64)
    assert max(abs(a - b) for a, b in zip(p.target, (3.45, -0.08, 0.0))) < 1e-6 and abs(p.size - 1.5) < 1e-6


def test_training_calls_check_their_arguments_and_need_a_device():
    """waves_net_gradients / waves_net_train validate the batch before any CUDA call (bad sizes,
    missing buffers, an unknown arithmetic, a tensor-core grid beyond 65,535 crop planes:
    WAVES_INVALID_ARG), and without a GPU a valid batch is WAVES_NO_DEVICE, never a CPU fallback."""
    import ctypes as C
    import numpy as np
    import torch
    from waves_gb300.abi import WAVES_NET_EXACT, WAVES_NET_TENSOR, WavesNetBatch
    from waves_gb300.learned import CHANNELS
    lib = waves_gb300.load(build_if_missing=True)
    fp = C.POINTER(C.c_float)
    x = np.zeros((1, 3, 4, 4, 4), np.float32)
    t = np.zeros((1, 4, 4, 4), np.float32)
    ws = [np.zeros((co, 27, ci), np.float32) for ci, co in CHANNELS]
    bs = [np.zeros(co, np.float32) for _, co in CHANNELS]
    ptrs = lambda arrays: (fp * 4)(*[a.ctypes.data_as(fp) for a in arrays])
    loss = C.c_double()

    def grads(crops=1, nz=4, arithmetic=WAVES_NET_EXACT, mask=True):
        bt = WavesNetBatch(crops, nz, 4, 4, x.ctypes.data_as(fp), t.ctypes.data_as(fp),
                           t.ctypes.data_as(fp) if mask else None, arithmetic)
        return lib.waves_net_gradients(C.byref(bt), ptrs(ws), ptrs(bs), C.byref(loss), ptrs(ws), ptrs(bs), None, 0)

    assert grads(crops=0) == 1 and grads(nz=0) == 1 and grads(mask=False) == 1
    assert grads(arithmetic=2) == 1 and grads(arithmetic=-1) == 1
    assert grads(crops=1000, nz=70, arithmetic=WAVES_NET_TENSOR) == 1  # 70,000 crop planes
    bt = WavesNetBatch(1, 4, 4, 4, x.ctypes.data_as(fp), t.ctypes.data_as(fp), t.ctypes.data_as(fp), 0)
    assert lib.waves_net_train(C.byref(bt), ptrs(ws), ptrs(bs), -1, 1e-3, None, 0) == 1
    assert lib.waves_net_train(C.byref(bt), ptrs(ws), ptrs(bs), 1, 0.0, None, 0) == 1
    if not torch.cuda.is_available():
        assert grads() == 3 and grads(arithmetic=WAVES_NET_TENSOR) == 3
        assert lib.waves_net_train(C.byref(bt), ptrs(ws), ptrs(bs), 1, 1e-3, None, 0) == 3


def test_mg_plan_arguments():
    """waves_mg_plan: the level count with no output buffer, only `capacity` levels written, and
    WAVES_INVALID_ARG for a missing count, a negative capacity or an empty grid."""
    import ctypes as C
    lib = waves_gb300.load(build_if_missing=True)
    cfg = waves_gb300.config("beach")
    count = C.c_int32()
    assert lib.waves_mg_plan(C.byref(cfg), None, 0, C.byref(count)) == 0 and count.value == 7
    out = (C.c_int32 * 24)(*([-7] * 24))
    assert lib.waves_mg_plan(C.byref(cfg), out, 2, C.byref(count)) == 0 and count.value == 7
    assert list(out[:8]) == [310, 48, 80, 2, 2, 1, 7, 0] and list(out[16:]) == [-7] * 8
    assert lib.waves_mg_plan(C.byref(cfg), out, 2, None) == 1
    assert lib.waves_mg_plan(C.byref(cfg), out, -1, C.byref(count)) == 1
    assert lib.waves_mg_plan(C.byref(cfg), None, 2, C.byref(count)) == 1
    cfg.n[1] = 0
    assert lib.waves_mg_plan(C.byref(cfg), out, 2, C.byref(count)) == 1


def test_headers_compile_as_c99_and_cpp11(tmp_path):
    """include/waves.h and include/waves_debug.h are plain C: a C99 host, a C++11 host and FFI
    generators (cgo, JNI, ctypes) read them, so they compile warning-free under -pedantic."""
    import shutil
    import subprocess
    import pytest
    inc = os.path.join(ROOT, "include")
    for compiler, std, ext in (("gcc", "c99", "c"), ("g++", "c++11", "cpp")):
        if not shutil.which(compiler):
            pytest.skip(f"{compiler} missing")
        src = tmp_path / f"h.{ext}"
        src.write_text('#include "waves.h"\n#include "waves_debug.h"\nint main(void) { return 0; }\n')
        r = subprocess.run([compiler, f"-std={std}", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", inc,
                            "-fsyntax-only", str(src)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_harness_reads_the_raw_model_file(tmp_path):
    """waves_run --model: the raw file of waves_gb300.learned.write_raw_model (31,324 bytes for the
    3-16-16-16-1 network) is read and checked before any device call; a truncated file, trailing
    bytes or a wrong tag exit 1, and a valid file gets as far as waves_create (exit 2 without a
    GPU)."""
    import subprocess
    import torch
    from waves_gb300.build import HARNESS, build
    from waves_gb300.learned import write_raw_model
    build()
    good = tmp_path / "model.bin"
    write_raw_model(os.path.join(ROOT, "waves_gb300", "learned", "model_beach.npz"), good)
    data = good.read_bytes()
    assert len(data) == 8 + sum(co * 27 * ci * 2 + co * 4 for ci, co in [(3, 16), (16, 16), (16, 16), (16, 1)]) + 16
    bad = {"short": data[:-4], "long": data + b"\0", "tag": b"WVNET2\0\0" + data[8:]}
    for name, content in bad.items():
        path = tmp_path / f"{name}.bin"
        path.write_bytes(content)
        r = subprocess.run([HARNESS, "--preset", "tank", "--steps", "1", "--model", str(path)], capture_output=True,
                           text=True)
        assert r.returncode == 1 and "bad model file" in r.stderr, name
    if not torch.cuda.is_available():
        r = subprocess.run([HARNESS, "--preset", "beach", "--steps", "1", "--model", str(good)], capture_output=True,
                           text=True)
        assert r.returncode == 2 and "waves_create" in r.stderr
