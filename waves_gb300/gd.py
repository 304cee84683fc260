"""Python mirror of the reference's GDScript solver classes.

water/pressure_gpu.gd, water/coupled_gpu.gd and water/coastal_gpu.gd expose to their callers
(water/lab_runner.gd, water/water_controller.gd):

    solver = coastal_view.new(settings)     # lab_runner.gd:27
    solver.telemetry.connect(callback)       # :29-31
    solver.start()                           # :31, pressure_gpu.gd:45-47
    solver.request(steps)                    # :68,72, pressure_gpu.gd:48-49
    solver.request_time(seconds)             # :57,  pressure_gpu.gd:52-54
    solver.close()                           # :16,75, pressure_gpu.gd:55-59
    solver.planes / solver.kinds             # accepted-surface textures (pressure_gpu.gd:4-5)

These classes keep those names and semantics over the C ABI.  `frame()` plays the role of the
render-thread work of work_scheduler.gd:41-87: one budgeted submission per call (waves_frame),
never a wait for the GPU, and one telemetry packet; `run()` submits until the quota is met.  The
settings dictionary uses the keys of lab_runner.gd:26.
"""
import math

from . import WavesSolver, config


def settings_to_config(settings, coastal):
    cfg = config("default")
    s = dict(settings)
    if "n" in s:
        for i, v in enumerate(s["n"]):
            cfg.n[i] = int(v)
    for key, field in (("spacing", "spacing"), ("origin", "origin")):
        if key in s:
            for i, v in enumerate(s[key]):
                getattr(cfg, field)[i] = float(v)
    if "wave" in s:
        for i, v in enumerate(s["wave"]):
            cfg.wave[i] = float(v)
    for key in ("eta", "dt", "slope", "corrugation", "gravity", "pressure_tolerance", "zone_length", "damping_rate",
                "ramp_periods", "right_absorption", "cfl"):
        if key in s:
            setattr(cfg, key, float(s[key]))
    for key in ("shape", "history_capacity", "mg_lag", "mg_aggregate_from", "mg_smoothing", "iterations_per_batch",
                "mg_precision", "device"):
        if key in s:
            setattr(cfg, key, int(s[key]))
    for key in ("periodic_x", "max_face_cfl", "linear_air", "height_normals", "active_advection", "transport_cache",
                "transport_interior"):
        if key in s:
            setattr(cfg, key, 1 if s[key] else 0)
    cfg.coastal = 1 if coastal else 0
    # coastal_gpu.gd:25 defaults Stokes-2 on; coupled_gpu.gd:21 off.
    cfg.stokes_second = 1 if s.get("stokes_second", coastal) else 0
    if "mg_smoother" in s:
        cfg.mg_smoother = {"jacobi": 0, "chebyshev": 1}[s["mg_smoother"]]
    if "mg_maintenance" in s:
        cfg.mg_maintenance = {"rebuild": 0, "structure": 1, "lagged": 2}[s["mg_maintenance"]]
    return cfg


class PressureGPU:
    """water/pressure_gpu.gd public surface over the C ABI."""

    coastal = False

    def __init__(self, settings):
        self.config = dict(settings)
        self.n = tuple(settings.get("n", (64, 48, 16)))
        self.spacing = tuple(settings.get("spacing", (0.025, 0.025, 0.05)))
        self.origin = tuple(settings.get("origin", (0.0, 0.0, 0.0)))
        self._callbacks = []
        self._target = 0.0
        self.solver = None
        self.closed = False
        self.planes = None
        self.kinds = None
        self.last_stats = {}

    # signal telemetry(packet: Dictionary)
    def connect(self, callback):
        self._callbacks.append(callback)

    def _emit(self, packet):
        for cb in self._callbacks:
            cb(packet)

    def start(self):
        self.solver = WavesSolver(settings_to_config(self.config, self.coastal))
        self._emit({"initialized": True, "pressure_backend": "multigrid"})

    def request(self, steps: int):
        self._target = float(steps)

    def request_time(self, seconds: float):
        assert math.isfinite(seconds) and seconds >= 0
        self._target = -float(seconds)

    def frame(self, gpu_budget_ms=14.0, max_inflight=3, max_trials=96, cpu_budget_ms=4.0):
        """One rendered frame of water/work_scheduler.gd:frame through waves_frame: trials toward the
        current quota within the GPU and CPU budgets, at most max_inflight unfinished submissions,
        never a wait for the GPU; emits the frame's telemetry (work_scheduler.gd:40,86 keys).
        Returns False once the quota is met with nothing in flight, or the solver halted."""
        if self.solver is None or self.closed:
            return False
        if self._target >= 0:
            self.solver.request_steps(int(self._target))
        else:
            self.solver.request_time(-self._target)
        r = self.solver.frame(gpu_budget_ms=gpu_budget_ms, max_inflight=max_inflight, max_trials=max_trials,
                              cpu_budget_ms=cpu_budget_ms)
        packet = {"submission_chunks": r["trials_submitted"], "queue_depth": r["queue_depth"],
                  "predicted_gpu_ns": r["predicted_gpu_ms"] * 1e6, "gpu_ns": r["gpu_ms_total"] * 1e6,
                  "R_fluid": r["r_fluid"], "submission_accepted_steps": r["accepted_steps"],
                  "submission_accepted_time": r["accepted_time"], "failure": r["halted"]}
        self.last_stats.update({"accepted_steps": r["accepted_steps"], "accepted_time": r["accepted_time"]})
        self._emit(packet)
        return not (r["idle"] or r["halted"])

    def run(self, trials_per_sync=4):
        if self._target >= 0:
            self.solver.request_steps(int(self._target))
        else:
            self.solver.request_time(-self._target)
        self.solver.run(trials_per_sync)
        self.last_stats = self.solver.stats()
        self._emit(self.last_stats)
        return self.last_stats

    def export(self):
        self.planes, self.kinds = self.solver.export_surface()
        return self.planes, self.kinds

    def close(self):
        if self.closed:
            return
        self.closed = True
        if self.solver is not None:
            self.solver.close()
            self.solver = None


class CoupledGPU(PressureGPU):
    """water/coupled_gpu.gd: VOF transport + projection, wall variant."""

    coastal = False


class CoastalGPU(CoupledGPU):
    """water/coastal_gpu.gd: offshore forcing, ocean ghost at x < 0."""

    coastal = True
