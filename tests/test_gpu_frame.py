"""Frame-budgeted submission (waves_frame, after water/work_scheduler.gd:frame): bounded queue,
budgeted trial counts, telemetry, and results identical to the synchronous driver."""
import time

import numpy as np
import pytest

import waves_gb300 as wg
from tests.cases import beach_slope


def drive(s, steps, **budget):
    """Frames until the quota is met with nothing in flight; every report kept."""
    s.request_steps(steps)
    reports = []
    deadline = time.monotonic() + 300
    while time.monotonic() < deadline:
        r = s.frame(**budget)
        reports.append(r)
        assert not r["halted"]
        if r["idle"]:
            return reports
        time.sleep(0.002)
    raise AssertionError("frames did not reach the quota")


@pytest.mark.gpu
def test_frames_match_synchronous_run(gpu_lib):
    steps = 6
    ref = wg.WavesSolver(beach_slope())
    ref.request_steps(steps)
    assert ref.run() == 0
    s = wg.WavesSolver(beach_slope())
    reports = drive(s, steps, gpu_budget_ms=14.0, max_inflight=3, max_trials=96)
    assert max(r["queue_depth"] for r in reports) <= 3
    assert reports[0]["trials_submitted"] == 1  # no cost measured yet: one trial
    assert all(r["trials_submitted"] == 0 for r in reports if r["queue_depth"] == 0)
    last = reports[-1]
    assert last["accepted_steps"] == steps and last["queue_depth"] == 0
    assert last["trial_cost_ms"] > 0 and last["gpu_ms_total"] > 0
    assert last["r_fluid"] == pytest.approx(last["gpu_ms_total"] / 1e3 / last["accepted_time"])
    assert last["submissions_retired"] == sum(1 for r in reports if r["trials_submitted"] > 0)
    # trials past the quota are no-ops on the device: same state as the synchronous driver
    assert np.array_equal(s.bank(), ref.bank())
    c, cr = s.control(), ref.control()
    assert c[1] == cr[1] and c[2] == cr[2]
    s.close()
    ref.close()


@pytest.mark.gpu
def test_frame_budget_bounds_trials(gpu_lib):
    """Once a trial cost is measured, a submission predicts no more than the budget (one trial at
    least), and the queue never exceeds max_inflight."""
    s = wg.WavesSolver(beach_slope())
    s.request_steps(40)
    budget = 3.0
    seen_cost = False
    for _ in range(400):
        r = s.frame(gpu_budget_ms=budget, max_inflight=2, max_trials=8, cpu_budget_ms=0)
        assert r["queue_depth"] <= 2 and r["trials_submitted"] <= 8
        if r["trials_submitted"] > 1:
            assert r["predicted_gpu_ms"] <= budget + 1e-9
        if r["trial_cost_ms"] > 0:
            seen_cost = True
        if r["idle"]:
            break
        time.sleep(0.001)
    assert seen_cost and r["idle"] and r["accepted_steps"] == 40
    with pytest.raises(wg.WavesError):
        s.frame(max_inflight=0)
    with pytest.raises(wg.WavesError):
        s.frame(gpu_budget_ms=0)
    s.close()


@pytest.mark.gpu
def test_gdscript_mirror_frames(gpu_lib):
    """The CoastalGPU mirror driven the way lab_runner.gd drives coastal_view: request, then one
    frame() per rendered frame until it reports nothing left; telemetry packets carry the
    scheduler's keys and the accepted steps reach the quota."""
    from waves_gb300.gd import CoastalGPU
    solver = CoastalGPU({"n": (64, 40, 8), "origin": (0.5, -0.6, -0.2), "spacing": (0.025, 0.025, 0.025),
                         "shape": 7, "slope": 6.0, "wave": (0.08, 2.52502, 4.48799, 0.45)})
    packets = []
    solver.connect(packets.append)
    solver.start()
    solver.request(4)
    deadline = time.monotonic() + 300
    while solver.frame(gpu_budget_ms=5.0) and time.monotonic() < deadline:
        time.sleep(0.002)
    assert packets[0].get("initialized") and len(packets) > 2
    assert max(p.get("queue_depth", 0) for p in packets) <= 3
    # lab_runner.gd:29-31 merges every packet into one dictionary and reads it in _process (:49-60)
    stats = {}
    for p in packets:
        stats.update(p)
    assert stats["accepted_steps"] == 4 and stats["failure"] == 0 and stats["pending"] is False
    assert stats["accepted_time"] > 0 and stats["R_fluid"] > 0
    assert stats["submission_accepted_steps"] == 4 and "gauges_m" in stats and "trial_count" in stats
    solver.close()
