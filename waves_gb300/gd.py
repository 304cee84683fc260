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
never a wait for the GPU; when a submission has retired, the telemetry of its control-block copy is
emitted as the reference's _stats packets (pressure_gpu.gd:133-137, coupled_gpu.gd:58-65,
coastal_gpu.gd:34-37, with their key names), followed by the submission packet
(work_scheduler.gd:82) and the cost packet (:40).  `run()` submits until the quota is met and emits
the same _stats packets.  The settings dictionary uses the keys of lab_runner.gd:26.
"""
import math

from . import WavesSolver, config


def stats_packets(st, coastal, record_us=0.0, gpu_ns=0.0, batches_last_frame=0, iterations_per_batch=8,
                  transport_cache=True, allocated_bytes=0):
    """The packets the reference's _stats chain emits for one control-block read-back, built from a
    waves_stats_t dict: pressure_gpu.gd:135 (failure masked for recoverable codes, as
    coupled_gpu.gd:61-62 passes it on), coupled_gpu.gd:64 and, for the coastal class,
    coastal_gpu.gd:37."""
    t = st["accepted_time"]
    pressure = {"pressure_backend": "multigrid", "batches_last_frame": batches_last_frame,
                "iterations_per_batch": iterations_per_batch, "accepted_index": int(st["accepted_index"]),
                "accepted_time": t, "accepted_steps": int(st["accepted_steps"]), "rejections": int(st["rejections"]),
                "pending": bool(st["pending"]), "converged": bool(st["converged"]), "failure": int(st["failure"]),
                "iterations": int(st["iterations"]), "relative_residual": st["relative_residual"],
                "max_dt_divergence": st["max_dt_divergence"], "max_face_speed": st["max_face_speed"],
                "hydrostatic_error_pa": st["hydrostatic_error_pa"], "volume_m3": st["volume_m3"],
                "total_iterations": int(st["total_iterations"]), "record_us": record_us, "gpu_ns": gpu_ns,
                "R_fluid": gpu_ns / 1e9 / t if t > 0 else -1}
    coupled = {"transport_cache": bool(transport_cache),
               "rhs_integrated_divergence_l2": st["rhs_integrated_divergence_l2"],
               "residual_integrated_divergence_l2": st["residual_integrated_divergence_l2"],
               "true_relative_residual": st["true_relative_residual"],
               "pressure_defect_corrections": int(st["pressure_defect_corrections"]),
               "boundary_outflow_m3": st["boundary_outflow_m3"], "tentative_outflow_m3": st["tentative_outflow_m3"],
               "raw_compression_volume_m3": st["raw_compression_volume_m3"],
               "compression_volume_m3": st["compression_volume_m3"],
               "compression_coverage_errors": int(st["compression_coverage_errors"]),
               "step_start_volume_m3": st["step_start_volume_m3"], "trial_count": int(st["trial_count"]),
               "trial_failure": int(st["trial_failure"]), "retry_count": int(st["retry_count"]),
               "last_rejection_code": int(st["last_rejection_code"]), "last_rejected_dt": st["last_rejected_dt"],
               "dt": st["dt"], "signed_roundoff_m3": st["signed_roundoff_m3"],
               "absolute_roundoff_m3": st["absolute_roundoff_m3"], "max_CFL": st["max_CFL"],
               "mass_defect_m3": st["mass_defect_m3"], "initial_volume_m3": st["initial_volume_m3"], "coupled": True,
               "allocated_bytes": allocated_bytes}
    out = [pressure, coupled]
    if coastal:
        out.append({"forcing_min_F": st["forcing_min_F"], "forcing_max_F": st["forcing_max_F"],
                    "forcing_volume_m3": st["forcing_volume_m3"], "ocean_inflow_m3": st["ocean_inflow_m3"],
                    "ocean_outflow_m3": st["ocean_outflow_m3"],
                    "forcing_momentum_kg_mps": list(st["forcing_momentum"]),
                    "staged_forcing_volume_m3": st["staged_forcing_volume_m3"],
                    "staged_ocean_inflow_m3": st["staged_ocean_inflow_m3"],
                    "staged_ocean_outflow_m3": st["staged_ocean_outflow_m3"], "gauges_m": list(st["gauges_m"])})
    return out


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
        self._retired = 0
        self._submission = 0
        self._max_queue = 0
        self._record_us = 0.0

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
        never a wait for the GPU.  When a submission has retired since the last frame, its
        telemetry is emitted as the _stats packets, then the submission packet
        (work_scheduler.gd:82 keys) and the cost packet (work_scheduler.gd:40 keys).
        Returns False once the quota is met with nothing in flight, or the solver halted."""
        import time
        if self.solver is None or self.closed:
            return False
        if self._target >= 0:
            self.solver.request_steps(int(self._target))
        else:
            self.solver.request_time(-self._target)
        t0 = time.perf_counter()
        r = self.solver.frame(gpu_budget_ms=gpu_budget_ms, max_inflight=max_inflight, max_trials=max_trials,
                              cpu_budget_ms=cpu_budget_ms)
        record_us = (time.perf_counter() - t0) * 1e6
        self._record_us += record_us
        if r["trials_submitted"] > 0:
            self._submission += 1
        self._max_queue = max(self._max_queue, r["queue_depth"])
        gpu_ns = r["gpu_ms_total"] * 1e6
        if r["submissions_retired"] > self._retired:
            self._retired = r["submissions_retired"]
            st = self.solver.frame_stats()
            if st is not None:
                for packet in stats_packets(st, self.coastal, record_us=self._record_us, gpu_ns=gpu_ns,
                                            batches_last_frame=r["trials_submitted"],
                                            iterations_per_batch=int(self.config.get("iterations_per_batch", 8)),
                                            transport_cache=self.config.get("transport_cache", True),
                                            allocated_bytes=self._allocated()):
                    self.last_stats.update(packet)
                    self._emit(packet)
                self._emit({"submission_id": self._submission, "submission_chunks": r["trials_submitted"],
                            "submission_accepted_steps": int(st["accepted_steps"]),
                            "submission_accepted_time": st["accepted_time"],
                            "submission_iterations": int(st["iterations"]), "queue_depth": r["queue_depth"],
                            "maximum_queue_depth": self._max_queue, "record_us_submission": record_us,
                            "predicted_gpu_ns": r["predicted_gpu_ms"] * 1e6, "work_schedule": "trials"})
        elapsed = self.last_stats.get("accepted_time", 0.0)
        self._emit({"record_us": self._record_us, "gpu_ns": gpu_ns,
                    "R_fluid": gpu_ns / 1e9 / elapsed if elapsed > 0 else -1})
        return not (r["idle"] or r["halted"])

    def _allocated(self):
        try:
            return self.solver.device_bytes()
        except Exception:
            return 0

    def run(self, trials_per_sync=4):
        if self._target >= 0:
            self.solver.request_steps(int(self._target))
        else:
            self.solver.request_time(-self._target)
        self.solver.run(trials_per_sync)
        st = self.solver.stats()
        for packet in stats_packets(st, self.coastal, iterations_per_batch=int(self.config.get("iterations_per_batch", 8)),
                                    transport_cache=self.config.get("transport_cache", True),
                                    allocated_bytes=self._allocated()):
            self.last_stats.update(packet)
            self._emit(packet)
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
