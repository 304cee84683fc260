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


def test_presets_without_gpu():
    lib = waves_gb300.load(build_if_missing=True)
    beach = waves_gb300.config("beach")
    assert tuple(beach.n) == (310, 48, 80)
    assert abs(beach.wave[1] - 2.52502) < 1e-4  # lab_runner.gd:19-25 dispersion, T = 1.4 s, h = 0.45 m
    tank = waves_gb300.config("tank")
    assert tank.coastal == 0 and abs(tank.cfl - 0.5) < 1e-7 and abs(tank.pressure_tolerance - 1e-6) < 1e-12
    assert abs(lib.waves_dispersion_k(1.4, 0.45) - 2.525) < 1e-3


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
    if not torch.cuda.is_available():
        r = subprocess.run([HARNESS, "--preset", "tank", "--steps", "1"], capture_output=True, text=True)
        assert r.returncode == 2 and "waves_create" in r.stderr


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
