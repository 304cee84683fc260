"""The standalone C harness drives the solver through the C ABI only."""
import json
import subprocess

import pytest

from waves_gb300.build import HARNESS, build


@pytest.mark.gpu
def test_harness_runs_tank(gpu_lib, tmp_path):
    build()
    surface = tmp_path / "surface.bin"
    r = subprocess.run([HARNESS, "--preset", "tank", "--steps", "3", "--surface", str(surface)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["accepted_steps"] == 3 and line["failure"] == 0 and line["accepted_time"] > 0
    n = line["n"][0] * line["n"][1] * line["n"][2]
    assert surface.stat().st_size == 5 * 4 * n


@pytest.mark.gpu
def test_harness_writes_image(gpu_lib, tmp_path):
    build()
    image = tmp_path / "beach.ppm"
    r = subprocess.run([HARNESS, "--preset", "beach", "--steps", "2", "--image", str(image), "--size", "64x36"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    data = image.read_bytes()
    header = b"P6\n64 36\n255\n"
    assert data.startswith(header) and len(data) == len(header) + 64 * 36 * 3
    assert len(set(data[len(header):])) > 8  # not a flat colour
