"""Host-side logic without a GPU: the settings mapping of the GDScript mirror and the bench's
roofline arithmetic."""
import importlib.util
import os

import pytest

import waves_gb300 as wg
from waves_gb300.gd import settings_to_config

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_settings_to_config_maps_lab_runner_keys():
    """lab_runner.gd:26 keys land in the C config; coastal_gpu.gd turns Stokes-2 on by default."""
    wg.load(build_if_missing=True)
    s = {"n": (310, 48, 80), "spacing": (0.025, 0.025, 0.025), "origin": (-1.75, -0.6, -2.0), "shape": 7,
         "slope": 6.0, "wave": (0.08, 2.52502, 4.48799, 0.45), "periodic_x": False, "mg_smoother": "jacobi",
         "mg_maintenance": "structure", "iterations_per_batch": 6}
    cfg = settings_to_config(s, coastal=True)
    assert tuple(cfg.n) == (310, 48, 80) and cfg.shape == 7 and cfg.coastal == 1 and cfg.stokes_second == 1
    assert abs(cfg.origin[0] + 1.75) < 1e-6 and abs(cfg.slope - 6.0) < 1e-6 and abs(cfg.wave[1] - 2.52502) < 1e-5
    assert cfg.mg_smoother == 0 and cfg.mg_maintenance == 1 and cfg.iterations_per_batch == 6 and cfg.periodic_x == 0
    wall = settings_to_config({"n": (64, 48, 16)}, coastal=False)
    assert wall.coastal == 0 and wall.stokes_second == 0 and wall.mg_smoother == 1 and wall.mg_maintenance == 2


def test_bench_roofline_picks_the_largest_probed_time():
    bench = load_bench()
    probes = [
        {"kernel": "k_a", "launches": 10, "ms": 0.5, "bytes": 10 * 40e6},
        {"kernel": "k_b", "launches": 2, "ms": 1.0, "bytes": 2 * 100e6},
        {"kernel": "all", "launches": 50, "ms": 9.0, "bytes": 0.0},
        {"kernel": "k_c", "launches": 0, "ms": 0.0, "bytes": 0.0},
    ]
    roof, table = bench.roofline(probes)
    peak, _ = bench.measured_peaks()
    assert roof["kernel"] == "k_b" and len(table) == 2
    assert roof["achieved"] == pytest.approx(200e6 / 1e-3 / 1e9)  # 200 MB in 1 ms = 200 GB/s
    assert roof["frac"] == pytest.approx(roof["achieved"] / peak)
    assert sum(t["share_of_probed"] for t in table) == pytest.approx(1.0)
    assert bench.roofline([]) == (None, [])
