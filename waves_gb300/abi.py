"""ctypes mirror of the C ABI structs in include/waves.h.

The field order and types follow include/waves.h exactly; `WAVES_ABI_SYMBOLS` lists every
function the header declares (used by the CPU test that checks the built library exports them).
"""
import ctypes as C

WAVES_CONTROL_SIZE = 128
WAVES_NET_LAYERS = 4
WAVES_NET_HIDDEN = 16
WAVES_NET_EXACT = 0
WAVES_NET_TENSOR = 1

STATUS = {
    0: "WAVES_OK",
    1: "WAVES_INVALID_ARG",
    2: "WAVES_CUDA_ERROR",
    3: "WAVES_NO_DEVICE",
    4: "WAVES_SOLVER_FAILED",
    5: "WAVES_NOT_READY",
    6: "WAVES_OUT_OF_MEMORY",
}


class WavesConfig(C.Structure):
    _fields_ = [
        ("n", C.c_int32 * 3),
        ("spacing", C.c_float * 3),
        ("origin", C.c_float * 3),
        ("eta", C.c_float),
        ("dt", C.c_float),
        ("periodic_x", C.c_int32),
        ("slope", C.c_float),
        ("corrugation", C.c_float),
        ("corrugation_phase", C.c_float),
        ("shape", C.c_int32),
        ("gravity", C.c_float),
        ("max_face_cfl", C.c_int32),
        ("history_capacity", C.c_int32),
        ("wave", C.c_float * 4),
        ("pressure_tolerance", C.c_float),
        ("linear_air", C.c_int32),
        ("stokes_second", C.c_int32),
        ("height_normals", C.c_int32),
        ("active_advection", C.c_int32),
        ("transport_cache", C.c_int32),
        ("transport_interior", C.c_int32),
        ("coastal", C.c_int32),
        ("zone_length", C.c_float),
        ("damping_rate", C.c_float),
        ("ramp_periods", C.c_float),
        ("right_absorption", C.c_float),
        ("mg_smoother", C.c_int32),
        ("mg_smoothing", C.c_int32),
        ("mg_maintenance", C.c_int32),
        ("mg_lag", C.c_int32),
        ("mg_aggregate_from", C.c_int32),
        ("iterations_per_batch", C.c_int32),
        ("cfl", C.c_float),
        ("mg_precision", C.c_int32),
        ("warm_start", C.c_int32),
        ("device", C.c_int32),
    ]


class WavesStats(C.Structure):
    _fields_ = [
        ("accepted_index", C.c_int32),
        ("accepted_time", C.c_double),
        ("accepted_steps", C.c_int64),
        ("rejections", C.c_int64),
        ("pending", C.c_int32),
        ("converged", C.c_int32),
        ("failure", C.c_int32),
        ("trial_failure", C.c_int32),
        ("iterations", C.c_int64),
        ("relative_residual", C.c_double),
        ("max_dt_divergence", C.c_double),
        ("max_face_speed", C.c_double),
        ("hydrostatic_error_pa", C.c_double),
        ("volume_m3", C.c_double),
        ("total_iterations", C.c_int64),
        ("dt", C.c_double),
        ("signed_roundoff_m3", C.c_double),
        ("absolute_roundoff_m3", C.c_double),
        ("initial_volume_m3", C.c_double),
        ("max_CFL", C.c_double),
        ("mass_defect_m3", C.c_double),
        ("retry_count", C.c_int32),
        ("trial_count", C.c_int64),
        ("last_rejection_code", C.c_int32),
        ("last_rejected_dt", C.c_double),
        ("compression_volume_m3", C.c_double),
        ("compression_coverage_errors", C.c_int64),
        ("step_start_volume_m3", C.c_double),
        ("raw_compression_volume_m3", C.c_double),
        ("tentative_outflow_m3", C.c_double),
        ("boundary_outflow_m3", C.c_double),
        ("pressure_defect_corrections", C.c_int32),
        ("true_relative_residual", C.c_double),
        ("rhs_integrated_divergence_l2", C.c_double),
        ("residual_integrated_divergence_l2", C.c_double),
        ("forcing_volume_m3", C.c_double),
        ("ocean_inflow_m3", C.c_double),
        ("ocean_outflow_m3", C.c_double),
        ("forcing_momentum", C.c_double * 3),
        ("gauges_m", C.c_double * 8),
        ("forcing_min_F", C.c_double),
        ("forcing_max_F", C.c_double),
        ("conservation_residual_m3", C.c_double),
        ("mg_builds", C.c_int64),
        ("mg_structure_builds", C.c_int64),
        ("mg_levels", C.c_int32),
        ("warm_start_used", C.c_int64),
        ("staged_forcing_volume_m3", C.c_double),
        ("staged_ocean_inflow_m3", C.c_double),
        ("staged_ocean_outflow_m3", C.c_double),
    ]

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            if hasattr(v, "__len__"):
                v = list(v)
            out[name] = v
        return out


class WavesWarmStartModel(C.Structure):
    _fields_ = [
        ("weights", C.POINTER(C.c_uint16) * WAVES_NET_LAYERS),
        ("bias", C.POINTER(C.c_float) * WAVES_NET_LAYERS),
        ("input_scale", C.c_float * 3),
        ("output_scale", C.c_float),
    ]


class WavesNetBatch(C.Structure):
    _fields_ = [
        ("crops", C.c_int32),
        ("nz", C.c_int32),
        ("ny", C.c_int32),
        ("nx", C.c_int32),
        ("x", C.POINTER(C.c_float)),
        ("target", C.POINTER(C.c_float)),
        ("mask", C.POINTER(C.c_float)),
        ("arithmetic", C.c_int32),
    ]


class WavesRenderParams(C.Structure):
    _fields_ = [
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("mode", C.c_int32),
        ("orthographic", C.c_int32),
        ("eye", C.c_float * 3),
        ("target", C.c_float * 3),
        ("up", C.c_float * 3),
        ("size", C.c_float),
        ("fov_y_deg", C.c_float),
        ("water_tint", C.c_float * 3),
        ("attenuation_distance", C.c_float),
        ("ripple_strength", C.c_float),
        ("surface_roughness", C.c_float),
        ("sun_direction", C.c_float * 3),
        ("contact_correction", C.c_int32),
        ("clock_ready", C.c_int32),
    ]


class WavesFrameBudget(C.Structure):
    _fields_ = [
        ("gpu_budget_ms", C.c_double),
        ("max_inflight", C.c_int32),
        ("max_trials", C.c_int32),
        ("cpu_budget_ms", C.c_double),
    ]


class WavesFrameReport(C.Structure):
    _fields_ = [
        ("trials_submitted", C.c_int32),
        ("queue_depth", C.c_int32),
        ("idle", C.c_int32),
        ("halted", C.c_int32),
        ("predicted_gpu_ms", C.c_double),
        ("trial_cost_ms", C.c_double),
        ("gpu_ms_total", C.c_double),
        ("r_fluid", C.c_double),
        ("accepted_time", C.c_double),
        ("accepted_steps", C.c_int64),
        ("submissions_retired", C.c_int64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class WavesKernelProbe(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("launches", C.c_int32),
        ("ms", C.c_double),
        ("bytes", C.c_double),
    ]


# Kinds of waves_debug_probe_trial (include/waves_debug.h): the kernel each probes.
PROBE_KINDS = ["k_mac", "k_mg0_cheb", "k_mgl_rows", "k_mgl4", "k_sweep_update", "all", "empty", "empty_inner", "k_mg_leg"]


# Every function declared in include/waves.h.
WAVES_ABI_SYMBOLS = [
    "waves_config_default",
    "waves_config_beach",
    "waves_config_tank",
    "waves_dispersion_k",
    "waves_mg_plan",
    "waves_create",
    "waves_destroy",
    "waves_request_steps",
    "waves_request_time",
    "waves_advance",
    "waves_frame",
    "waves_frame_stats",
    "waves_run",
    "waves_synchronize",
    "waves_stream",
    "waves_timing",
    "waves_stats",
    "waves_control",
    "waves_set_control",
    "waves_export_surface",
    "waves_export_surface_device",
    "waves_get_history",
    "waves_render_params_default",
    "waves_render",
    "waves_render_device",
    "waves_bank_floats",
    "waves_get_bank",
    "waves_set_bank",
    "waves_get_geometry",
    "waves_get_masks",
    "waves_set_masks",
    "waves_inject_rejection",
    "waves_save",
    "waves_load",
    "waves_set_warm_start",
    "waves_net_gradients",
    "waves_net_train",
    "waves_last_error",
    "waves_liquid_volume_noalloc",
]


def declare(lib):
    """Attach argtypes/restype to the product library's functions."""
    P = C.POINTER
    cfgp = P(WavesConfig)
    h = C.c_void_p
    sig = {
        "waves_config_default": (None, [cfgp]),
        "waves_config_beach": (None, [cfgp]),
        "waves_config_tank": (None, [cfgp]),
        "waves_dispersion_k": (C.c_double, [C.c_double, C.c_double]),
        "waves_mg_plan": (C.c_int, [P(WavesConfig), P(C.c_int32), C.c_int32, P(C.c_int32)]),
        "waves_create": (C.c_int, [cfgp, P(C.c_void_p)]),
        "waves_destroy": (None, [h]),
        "waves_request_steps": (C.c_int, [h, C.c_int64]),
        "waves_request_time": (C.c_int, [h, C.c_double]),
        "waves_advance": (C.c_int, [h, C.c_int32]),
        "waves_run": (C.c_int, [h, C.c_int32]),
        "waves_frame": (C.c_int, [h, P(WavesFrameBudget), P(WavesFrameReport)]),
        "waves_frame_stats": (C.c_int, [h, P(WavesStats)]),
        "waves_synchronize": (C.c_int, [h]),
        "waves_stream": (C.c_void_p, [h]),
        "waves_timing": (C.c_int, [h, P(C.c_double), P(C.c_double), P(C.c_int64), C.c_int32]),
        "waves_stats": (C.c_int, [h, P(WavesStats)]),
        "waves_control": (C.c_int, [h, P(C.c_double), C.c_int32]),
        "waves_set_control": (C.c_int, [h, P(C.c_double), C.c_int32]),
        "waves_export_surface": (C.c_int, [h, P(C.c_float), P(C.c_float)]),
        "waves_export_surface_device": (C.c_int, [h, C.c_void_p, C.c_void_p, C.c_void_p]),
        "waves_render_params_default": (None, [P(WavesRenderParams), cfgp, C.c_int32, C.c_int32]),
        "waves_get_history": (C.c_int, [h, P(C.c_float), P(C.c_float), P(C.c_uint32)]),
        "waves_render": (C.c_int, [h, P(WavesRenderParams), P(C.c_float), P(C.c_float)]),
        "waves_render_device": (C.c_int, [h, P(WavesRenderParams), C.c_void_p, C.c_void_p]),
        "waves_bank_floats": (C.c_size_t, [h]),
        "waves_get_bank": (C.c_int, [h, C.c_int32, P(C.c_float)]),
        "waves_set_bank": (C.c_int, [h, C.c_int32, P(C.c_float)]),
        "waves_get_geometry": (C.c_int, [h, P(C.c_float), P(C.c_float)]),
        "waves_get_masks": (C.c_int, [h, P(C.c_float), P(C.c_float)]),
        "waves_set_masks": (C.c_int, [h, P(C.c_float), P(C.c_float)]),
        "waves_inject_rejection": (C.c_int, [h]),
        "waves_save": (C.c_int, [h, C.c_void_p, P(C.c_size_t)]),
        "waves_load": (C.c_int, [h, C.c_void_p, C.c_size_t]),
        "waves_set_warm_start": (C.c_int, [h, P(WavesWarmStartModel)]),
        "waves_net_gradients": (C.c_int, [P(WavesNetBatch), P(P(C.c_float)), P(P(C.c_float)), P(C.c_double),
                                          P(P(C.c_float)), P(P(C.c_float)), P(C.c_float), C.c_int32]),
        "waves_net_train": (C.c_int, [P(WavesNetBatch), P(P(C.c_float)), P(P(C.c_float)), C.c_int32, C.c_float,
                                      P(C.c_double), C.c_int32]),
        "waves_last_error": (C.c_char_p, [h]),
        "waves_liquid_volume_noalloc": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_float,
                                                  C.c_float, C.c_void_p, C.c_void_p]),
    }
    sig["waves_debug_phase"] = (C.c_int, [h, C.c_int32])
    sig["waves_debug_sample"] = (C.c_int, [h, P(C.c_float), C.c_int32, C.c_int32, P(C.c_float)])
    sig["waves_debug_launch_counts"] = (C.c_int, [h, P(C.c_int32)])
    sig["waves_debug_read"] = (C.c_int, [h, C.c_char_p, C.c_void_p, C.c_size_t])
    sig["waves_debug_probe_trial"] = (C.c_int, [h, P(WavesKernelProbe), C.c_int32, P(C.c_int32)])
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib
