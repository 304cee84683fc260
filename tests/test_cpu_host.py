"""Host-side logic without a GPU: the settings mapping of the GDScript mirror, the multigrid level
plan (waves_mg_plan), and the bench's roofline arithmetic and step byte model."""
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
    # with the bracket calibration (8 us per bracketed empty launch) the ten short launches of
    # k_a (50 us each bracketed -> 42 us) outweigh the two long ones of k_b (500 -> 492 us)? no:
    # 10 x 42 = 420 < 2 x 492 = 984; k_b stays on top, and each time loses the bracket
    cal = probes + [{"kernel": "empty", "launches": 64, "ms": 64 * 0.008, "bytes": 0.0},
                    {"kernel": "empty_inner", "launches": 64, "ms": 64 * 0.004, "bytes": 0.0}]
    roof, table = bench.roofline(cal)
    a = next(t for t in table if t["kernel"] == "k_a")
    assert roof["kernel"] == "k_b" and roof["us_per_launch"] == pytest.approx(492.0)
    assert a["us_per_launch"] == pytest.approx(42.0) and a["us_per_launch_bracketed"] == pytest.approx(50.0)
    assert roof["achieved"] == pytest.approx(100e6 / 492e-6 / 1e9)


def test_bench_traffic_table_covers_the_probed_kernels():
    """profiles/dram_traffic.txt gives a DRAM figure for every probed kernel the bench can report as
    the dominant one, under the name the library's probe list uses."""
    from waves_gb300.abi import PROBE_KINDS
    traffic = load_bench().ncu_traffic()
    for name in ("k_mac", "k_mg0_cheb", "k_mgl_rows", "k_mgl4", "k_sweep_update"):
        assert name in PROBE_KINDS
        assert traffic.get(name, 0.0) > 0.0, name


def test_mg_plan_of_the_beach_and_the_large_grid():
    """waves_mg_plan (no device): the level plan of pressure_multigrid.gd:37-69 for the 310x48x80
    beach (x and y halved first, z kept at hz = 2 hx; aggregation from level 2) and the 620x96x160
    grid (8 levels), with the Galerkin stencil sizes 7 / 39 / 125 / 27."""
    wg.load(build_if_missing=True)
    plan = wg.mg_plan(wg.config("beach"))
    assert [l["n"] for l in plan] == [(310, 48, 80), (155, 24, 80), (78, 12, 40), (39, 6, 20), (20, 3, 10),
                                      (10, 2, 5), (5, 2, 5)]
    assert [l["stencil"] for l in plan] == [7, 39, 125, 27, 27, 27, 27]
    assert [l["aggregate"] for l in plan] == [False, False] + [True] * 5
    assert plan[0]["f"] == (2, 2, 1) and plan[1]["f"] == (2, 2, 2)
    large = wg.mg_plan(wg.config("beach", n=[620, 96, 160], spacing=[0.0125, 0.0125, 0.025]))
    assert len(large) == 8 and large[0]["n"] == (620, 96, 160) and large[2]["n"] == (155, 24, 80)
    bad = wg.config("beach", n=[0, 48, 80])
    with pytest.raises(wg.WavesError):
        wg.mg_plan(bad)


def test_step_bytes_model_reproduces_the_algorithmic_byte_table():
    """The compulsory-traffic model of one accepted step at the beach: non-CG 152 N = 180.9 MB, one
    FP32 V-cycle 926 MB (778 N), BF16 half of the operator and vector bytes (463 MB), a CG iteration
    72 N + V; the 620x96x160 grid's FP32 V-cycle 7.40 GB."""
    bench = load_bench()
    wg.load(build_if_missing=True)
    plan = wg.mg_plan(wg.config("beach"))
    N = 310 * 48 * 80
    m32 = bench.step_bytes_model(plan, 0.0, 0.0, False)
    m16 = bench.step_bytes_model(plan, 0.0, 0.0, True)
    assert m32["cells"] == N and m32["bytes_per_step"] == 152 * N == pytest.approx(180.9e6, rel=1e-3)
    assert m32["vcycle"] == pytest.approx(926.2e6, rel=1e-3) and round(m32["vcycle"] / N) == 778
    assert m16["vcycle"] == pytest.approx(463.1e6, rel=2e-3)
    assert m32["cg_iteration"] == 72 * N + m32["vcycle"]
    step = bench.step_bytes_model(plan, 14.0, 0.5, False)
    assert step["bytes_per_step"] == 152 * N + 0.5 * m32["rebuild"] + 14.0 * m32["cg_iteration"]
    large = wg.mg_plan(wg.config("beach", n=[620, 96, 160], spacing=[0.0125, 0.0125, 0.025]))
    assert bench.step_bytes_model(large, 0.0, 0.0, False)["vcycle"] == pytest.approx(7.40e9, rel=2e-3)
    roof = bench.step_roofline(plan, 14.0, 0.5, False, 12.5)
    assert roof["achieved"] == pytest.approx(step["bytes_per_step"] / 12.5e-3 / 1e9)
    assert roof["frac"] == pytest.approx(roof["achieved"] / bench.measured_peaks()[0])


def test_crop_bank_cuts_consistent_crops_and_scales_over_every_wet_cell():
    """waves_gb300.learned.train.CropBank (crops cut while pairs are captured): every field of a
    crop comes from the same offset of the same pair, the mask is the wet cells at least `edge`
    inside, the scales are the population standard deviations over all wet cells of all pairs (as
    if the pairs had been kept), and `rate` crops per pair are cut on average."""
    import numpy as np
    from waves_gb300.learned.train import CropBank
    nx, ny, nz = 30, 12, 20
    rng = np.random.default_rng(1)
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    pairs = []
    for k in range(6):
        wet = (y < 7 + k % 3) & (rng.random((nz, ny, nx)) < 0.9)
        pairs.append({"F": (x + 100 * y + 10000 * z + 1e6 * k).astype(np.float32).ravel(),
                      "b": rng.normal(3.0, 2.0, (nz, ny, nx)).astype(np.float32).ravel(),
                      "p_prev": rng.normal(900.0, 300.0, (nz, ny, nx)).astype(np.float32).ravel(),
                      "p_star": rng.normal(905.0, 301.0, (nz, ny, nx)).astype(np.float32).ravel(),
                      "kind": np.where(wet, 1.0, 0.0).astype(np.float32).ravel()})
    bank = CropBank((nx, ny, nz), 1.5, crop=(8, 8, 8), edge=2, seed=3)
    for p in pairs:
        bank.add(p)
    assert 6 <= len(bank.raw) <= 12
    xs, ys, ms, (s_b, s_p, s_out) = bank.batch()
    wet_all = np.concatenate([p["kind"] > 0 for p in pairs])
    cat = lambda key: np.concatenate([p[key] for p in pairs]).astype(np.float64)
    dp = np.concatenate([p["p_star"] - p["p_prev"] for p in pairs]).astype(np.float64)
    assert s_b == pytest.approx(1.0 / cat("b")[wet_all].std(), rel=1e-9)
    assert s_p == pytest.approx(1.0 / cat("p_prev")[wet_all].std(), rel=1e-9)
    assert s_out == pytest.approx(dp[wet_all].std(), rel=1e-9)
    inner = np.zeros((8, 8, 8), bool)
    inner[2:6, 2:6, 2:6] = True
    for i in range(len(xs)):
        code = int(xs[i, 0, 0, 0, 0])
        k, oz, oy, ox = code // 1000000, (code // 10000) % 100, (code // 100) % 100, code % 100
        assert 0 <= ox <= nx - 8 and 0 <= oy <= ny - 8 and 0 <= oz <= nz - 8
        sl = (slice(oz, oz + 8), slice(oy, oy + 8), slice(ox, ox + 8))
        g = lambda key: pairs[k][key].reshape(nz, ny, nx)[sl]
        assert np.array_equal(xs[i, 0], g("F"))
        assert np.array_equal(xs[i, 1], g("b") * np.float32(s_b))
        assert np.array_equal(xs[i, 2], g("p_prev") * np.float32(s_p))
        assert np.array_equal(ys[i], (g("p_star") - g("p_prev")) / np.float32(s_out))
        assert np.array_equal(ms[i] > 0, (g("kind") > 0) & inner)
    sparse = CropBank((nx, ny, nz), 0.25, crop=(8, 8, 8), seed=4)
    for _ in range(10):
        for p in pairs[:4]:
            sparse.add(p)
    assert sparse.pairs == 40 and 3 <= len(sparse.raw) <= 20


def test_bench_json_line_contract(monkeypatch, capsys):
    """bench.py's single JSON line from a stubbed measurement (the GPU part replaced): the keys the
    line must carry, value = simulated seconds / device seconds, ms_per_step from the device time,
    the kernel and whole-step rooflines, e2e with its copied bytes, and the clock record."""
    import json
    import sys
    bench = load_bench()
    wg.load(build_if_missing=True)

    def arm(pressure_ms_per_step):
        return {"sim_s_per_wall_s": 0.6, "ms_per_step": 12.0, "pressure_ms_per_step": pressure_ms_per_step,
                "motion_ms_per_step": 2.0, "cg_iterations_per_step": 12.0, "steps": 240, "trials": 245,
                "mg_builds": 60, "window_s": [5.0, 7.0], "warm_start_trials": 0}

    def measured(args, world, rank, local):
        assert args.window_start == 5.0 and args.compare
        return {"sim_s": 2.0, "device_s": 3.0, "wall_s": 3.1, "steps": 240, "trials": 245, "motion_ms": 500.0,
                "pressure_ms": 2500.0, "iters": 3103.0, "defect_rounds": 1, "launches": 123456,
                "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": []}, "t_end": 7.0, "mg_builds": 63,
                "probes": [{"kernel": "k_mgl_rows", "launches": 100, "ms": 1.5, "bytes": 100 * 8e6},
                           {"kernel": "all", "launches": 900, "ms": 11.0, "bytes": 0.0}],
                "plan": wg.mg_plan(wg.config("beach")), "window_s": [5.0, 7.0],
                "ms_per_step": 12.5, "pressure_ms_per_step": 2500.0 / 240, "cg_iterations_per_step": 3103.0 / 240,
                "warm_start_used": 0,
                "arms": {"from_rest": arm(8.0), "bf16": arm(10.0), "bf16_learned": arm(12.5)},
                "e2e": {"sim_s": 2.0, "wall_s": 3.2, "frames": 120, "h2d": 8, "d2h": 23809032, "window_s": [7.0, 9.0]},
                "render": None}

    monkeypatch.setattr(bench, "run_ours", measured)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--no-cpu-baseline"])
    bench.main()
    lines = [l for l in capsys.readouterr().out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "roofline", "step_roofline", "e2e", "clocks",
                "gpu_launches"):
        assert key in d, key
    assert d["value"] == pytest.approx(2.0 / 3.0) and d["ms_per_step"] == pytest.approx(3000.0 / 240)
    assert d["n_gpus"] == 1 and d["higher_is_better"] is True and d["gpu_launches"] == 123456
    assert "workload" in d["config"] and "model" not in d["config"]
    assert d["roofline"]["kernel"] == "k_mgl_rows" and d["roofline"]["unit"] == "GB/s"
    step = bench.step_bytes_model(wg.mg_plan(wg.config("beach")), 3103.0 / 240, 63 / 240, False)
    assert d["step_roofline"]["bytes_per_step"] == pytest.approx(step["bytes_per_step"])
    assert d["e2e"]["value"] == pytest.approx(2.0 / 3.2) and d["e2e"]["d2h_bytes_per_step"] == 23809032
    # the metric's second half: pressure ms per step of plain FP32 against BF16 + learned warm start
    assert set(d["arms"]) == {"from_rest", "bf16", "bf16_learned", "fp32_headline"}
    assert d["pressure_ms_ratio_plain_fp32_over_bf16_learned"] == pytest.approx((2500.0 / 240) / 12.5)
    assert d["config"]["sim_window_s"] == [5.0, 7.0] and "t = 5 s" in d["config"]["window"]


def test_gdscript_mirror_frame_packet_and_quota_without_a_gpu():
    """The mirror's frame() against a fake solver: quota forwarding, the budget defaults of
    work_scheduler.gd, and the packets lab_runner.gd:_process (:49-60) reads after merging them
    (:29-31): accepted_steps, accepted_time, pending, failure (recoverable codes masked, as
    coupled_gpu.gd:61-62), replayed here the way the GDScript does."""
    from waves_gb300.abi import WavesStats
    from waves_gb300.gd import CoastalGPU

    def control_stats(steps, time, pending, failure, trial_failure, retries):
        st = WavesStats().as_dict()
        st.update(accepted_steps=steps, accepted_time=time, pending=pending, failure=failure,
                  trial_failure=trial_failure, retry_count=retries, trial_count=steps + 1)
        return st

    class Fake:
        def __init__(self):
            self.calls = []
            self.report = {"trials_submitted": 3, "queue_depth": 2, "predicted_gpu_ms": 1.5, "gpu_ms_total": 4.0,
                           "r_fluid": 0.9, "accepted_steps": 7, "accepted_time": 0.05, "idle": 0, "halted": 0,
                           "submissions_retired": 1}
            self.retired = control_stats(7, 0.05, 1, 0, 0, 0)

        def request_steps(self, n):
            self.calls.append(("steps", n))

        def request_time(self, t):
            self.calls.append(("time", t))

        def frame(self, **budget):
            self.calls.append(("frame", budget))
            return dict(self.report)

        def frame_stats(self):
            return dict(self.retired)

        def device_bytes(self):
            return 1234

        def close(self):
            self.calls.append(("close",))

    packets = []
    g = CoastalGPU({"n": (310, 48, 80)})
    g.connect(packets.append)
    g.solver = fake = Fake()

    # lab_runner.gd state and _process, on the merged telemetry dictionary
    lab = {"stats": {}, "requested": 0, "requested_time": 0.0, "single_pending": False, "paused": False}

    def on_packet(p):
        lab["stats"].update(p)
    g.connect(on_packet)

    def process(wall_time):
        stats = lab["stats"]
        lab["requested_time"] = wall_time
        completed = stats.get("accepted_steps", stats.get("steps", 0))
        elapsed = stats.get("accepted_time", completed / 120.0)
        if lab["single_pending"] and completed >= lab["requested"]:
            lab["single_pending"] = False
            lab["requested_time"] = max(lab["requested_time"], elapsed)
        if not lab["paused"] and stats.get("failure", 0) == 0:
            g.request_time(lab["requested_time"])
        status = "PAUSED" if lab["paused"] else "RUNNING"
        if lab["paused"] and (stats.get("pending", False) or lab["single_pending"]):
            status = "PAUSING"
        if stats.get("failure", 0) > 0:
            status = "STOPPED"
        return status, completed, elapsed

    assert process(1.0) == ("RUNNING", 0, 0.0)
    assert g.frame() is True
    assert fake.calls[0] == ("time", 1.0) and fake.calls[1][0] == "frame"
    assert fake.calls[1][1] == {"gpu_budget_ms": 14.0, "max_inflight": 3, "max_trials": 96, "cpu_budget_ms": 4.0}
    stats = lab["stats"]
    assert stats["accepted_steps"] == 7 and stats["accepted_time"] == 0.05 and stats["pending"] is True
    assert stats["failure"] == 0 and stats["coupled"] is True and stats["allocated_bytes"] == 1234
    assert stats["submission_chunks"] == 3 and stats["queue_depth"] == 2 and stats["submission_accepted_steps"] == 7
    assert stats["gpu_ns"] == pytest.approx(4.0e6) and stats["R_fluid"] == pytest.approx(4.0e-3 / 0.05)
    assert "gauges_m" in stats and "forcing_momentum_kg_mps" in stats and "staged_forcing_volume_m3" in stats
    assert process(1.1) == ("RUNNING", 7, 0.05)

    # pause with a trial pending, then single-step: N requests accepted_steps + 1 (lab_runner.gd:64-72)
    lab["paused"] = True
    g.request(stats["accepted_steps"])
    assert process(1.2)[0] == "PAUSING"
    lab["requested"] = stats["accepted_steps"] + 1
    lab["single_pending"] = True
    g.request(lab["requested"])
    fake.report.update(submissions_retired=2)
    fake.retired = control_stats(8, 0.0583, 0, 0, 0, 0)
    g.frame()
    assert ("steps", 8) in fake.calls
    assert process(1.3) == ("PAUSED", 8, 0.0583) and lab["single_pending"] is False

    # a recoverable trial failure (code 11 with retries left) reads 0; a halt reads the code
    lab["paused"] = False
    fake.report.update(submissions_retired=3)
    fake.retired = control_stats(8, 0.0583, 1, 0, 11, 1)
    g.frame()
    assert stats["failure"] == 0 and stats["trial_failure"] == 11 and process(1.4)[0] == "RUNNING"
    fake.report.update(submissions_retired=4, halted=1)
    fake.retired = control_stats(8, 0.0583, 0, 4, 4, 0)
    assert g.frame() is False
    assert stats["failure"] == 4 and process(1.5)[0] == "STOPPED"
    # no new retirement: no new _stats packet, only the cost packet
    n = len(packets)
    g.frame()
    assert len(packets) == n + 1 and set(packets[-1]) == {"record_us", "gpu_ns", "R_fluid"}
    g.request(12)
    fake.report["idle"] = 1
    assert g.frame() is False and ("steps", 12) in fake.calls
    with pytest.raises(AssertionError):
        g.request_time(float("nan"))
    g.close()
    assert ("close",) in fake.calls and g.frame() is False and g.solver is None


def test_train_cli_flow_with_fakes(tmp_path, monkeypatch):
    """python -m waves_gb300.learned.train with the GPU parts replaced (capture feeds synthetic pairs
    into the crop bank; net_train / net_gradients are fakes): the CUDA-trainer flow cuts the
    requested number of crops on average, trains on them with the tensor arithmetic, and writes a
    model file load_model reads back, with the pair count."""
    import sys
    import numpy as np
    import waves_gb300.learned as learned
    import waves_gb300.learned.train as train
    nx, ny, nz = 310, 48, 80
    seen = {}

    def fake_capture(seeds, pairs, t0, gap, sink=None, with_coef=True):
        assert sink is not None and with_coef is False
        rng = np.random.default_rng(0)
        count = 0
        for _ in seeds:
            for _ in range(pairs):
                f = rng.random(nx * ny * nz).astype(np.float32)
                sink({"F": f, "b": f - 0.5, "p_prev": 2 * f, "p_star": 2 * f + 0.1 * f * f, "kind": (f > 0.3).astype(np.float32)})
                count += 1
        return count

    def fake_train(x, target, mask, weights, biases, iterations, lr, device=0, tensor=False):
        seen.update(crops=x.shape[0], shape=x.shape[1:], tensor=tensor, iterations=iterations)
        return weights, biases, np.linspace(1.0, 0.5, iterations)

    def fake_gradients(x, target, mask, weights, biases, device=0, tensor=False):
        return 0.25, None, None, None

    monkeypatch.setattr(train, "capture", fake_capture)
    monkeypatch.setattr(learned, "net_train", fake_train)
    monkeypatch.setattr(learned, "net_gradients", fake_gradients)
    out = tmp_path / "m.npz"
    monkeypatch.setattr(sys, "argv", ["train", "--seeds", "2", "--pairs", "3", "--crops", "12", "--steps", "5",
                                      "--eval-seeds", "0", "--out", str(out)])
    train.main()
    assert seen["tensor"] is True and seen["iterations"] == 5 and seen["shape"] == (3, 24, 24, 24)
    assert 6 <= seen["crops"] <= 18  # 2 crops per pair on average
    weights, biases, iscale, oscale = learned.load_model(str(out))
    assert [w.shape for w in weights] == [(co, 27, ci) for ci, co in learned.CHANNELS] and weights[0].dtype == np.uint16
    assert iscale[0] == 1.0 and oscale > 0 and int(np.load(out)["pairs"]) == 6
