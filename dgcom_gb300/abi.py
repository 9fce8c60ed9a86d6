"""ctypes mirror of the C ABI in ``include/dgswe.h`` and the loader of the
in-tree CUDA library ``libdgswe.so``.

The structs below are the header's, field for field; ``Library`` binds the
entry points of any shared library that exports this ABI under a symbol
prefix (``dgswe_`` for the CUDA library)."""

from __future__ import annotations

import ctypes as C
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIBRARY_PATH = HERE / "libdgswe.so"

ABI_VERSION = 4

# dgswe_status
OK, ERR_INVALID, ERR_CUDA, ERR_NONFINITE, ERR_DT_MIN, ERR_MAX_STEPS, ERR_STOPPED, \
    ERR_UNSUPPORTED, ERR_NO_DEVICE = range(9)
# dgswe_formulation
WET_DRY, ENTROPY_STABLE, ENTROPY_CONSERVATIVE = range(3)
# dgswe_boundary_kind
BC_WALL, BC_CHARACTERISTIC, BC_NODE_TIDES, BC_PARENT = range(4)
# dgswe_elevation_only
AT_REST, INCOMING_WAVE = range(2)
# dgswe_friction
FRICTION_NONE, FRICTION_MANNING, FRICTION_MANNING_NODES = range(3)
# dgswe_drag
DRAG_CONSTANT, DRAG_LARGE_POND, DRAG_WU, DRAG_SMITH, DRAG_YELLAND_TAYLOR = range(5)
# dgswe_scheme
SSP_RK3, SSP_RK43 = range(2)
# dgswe_numerics
NUMERICS_FAST, NUMERICS_EXACT = range(2)

STATE = 0
N_BUFFERS = 6

_dp = C.POINTER(C.c_double)


class TideConstituent(C.Structure):
    _fields_ = [
        ("amplitude", C.c_double),
        ("period", C.c_double),
        ("phase", C.c_double),
        ("f", C.c_double),
        ("f_rate", C.c_double),
        ("u_deg", C.c_double),
        ("u_rate_deg", C.c_double),
        ("v0_deg", C.c_double),
    ]


class NodeTides(C.Structure):
    _fields_ = [
        ("n_constituents", C.c_int32),
        ("omega", _dp),
        ("f_rate", _dp),
        ("n_slots", C.c_int64),
        ("positions", _dp),
        ("coefficients", _dp),
        ("mean", _dp),
        ("source_depth", _dp),
        ("slot_of_node", C.POINTER(C.c_uint32)),
        ("velocity", C.c_int32),
        ("use_mean", C.c_int32),
        ("max_transport_ratio", C.c_double),
        ("ramp_duration", C.c_double),
    ]


class ParentSeries(C.Structure):
    _fields_ = [
        ("n_slots", C.c_int64),
        ("positions", _dp),
        ("on_boundary", C.POINTER(C.c_uint8)),
        ("slot_of_node", C.POINTER(C.c_uint32)),
        ("n_times", C.c_int64),
        ("times", _dp),
        ("values", C.POINTER(C.c_float)),
        ("parent_depth", _dp),
        ("cubic", C.c_int32),
        ("velocity", C.c_int32),
        ("reference_level", C.c_double),
        ("max_transport_ratio", C.c_double),
        ("ramp_duration", C.c_double),
    ]


class Relaxation(C.Structure):
    _fields_ = [
        ("parent", C.POINTER(ParentSeries)),
        ("weight", _dp),
        ("rate", C.c_double),
        ("wet_depth", C.c_double),
        ("momentum_only", C.c_int32),
    ]


class Atmosphere(C.Structure):
    _fields_ = [
        ("n_times", C.c_int64),
        ("times", _dp),
        ("epoch_unix", C.c_double),
        ("values", C.POINTER(C.c_float)),
        ("source", C.c_int32),
        ("wind", C.c_int32),
        ("pressure", C.c_int32),
        ("level", C.c_int32),
        ("drag", C.c_int32),
        ("drag_cd", C.c_double),
        ("rho_air", C.c_double),
        ("rho_water", C.c_double),
        ("h_min", C.c_double),
        ("ramp_duration", C.c_double),
    ]


class Tuning(C.Structure):
    _fields_ = [
        ("face_threads", C.c_int32),
        ("stage_threads", C.c_int32),
        ("face_ms", C.c_double * 3),
        ("stage_ms", C.c_double * 3),
    ]


class Boundary(C.Structure):
    _fields_ = [
        ("tag", C.c_int32),
        ("kind", C.c_int32),
        ("wall_h_min", C.c_double),
        ("elevation_only", C.c_int32),
        ("n_constituents", C.c_int32),
        ("constituents", C.POINTER(TideConstituent)),
        ("mean_elevation", C.c_double),
        ("ramp_duration", C.c_double),
        ("node_tides", C.POINTER(NodeTides)),
        ("parent", C.POINTER(ParentSeries)),
        ("raise_", C.c_int32),
        ("raise_factor", C.c_double),
    ]


class Form(C.Structure):
    _fields_ = [
        ("abi_version", C.c_uint32),
        ("order", C.c_int32),
        ("n_vertices", C.c_int64),
        ("vertices", _dp),
        ("n_elements", C.c_int64),
        ("elements", C.POINTER(C.c_int64)),
        ("n_periodic", C.c_int64),
        ("periodic", C.POINTER(C.c_int64)),
        ("face_tags", C.POINTER(C.c_int32)),
        ("bathymetry", _dp),
        ("g", C.c_double),
        ("h_min", C.c_double),
        ("formulation", C.c_int32),
        ("subcell_depth", C.c_double),
        ("subcell_h_dry", C.c_double),
        ("has_wet_dry", C.c_int32),
        ("wet_dry_h_dry", C.c_double),
        ("wet_dry_relaxation_time", C.c_double),
        ("wet_dry_max_velocity", C.c_double),
        ("positivity_h_dry", C.c_double),
        ("friction", C.c_int32),
        ("friction_g", C.c_double),
        ("manning_n", C.c_double),
        ("manning_h_min", C.c_double),
        ("manning_n_nodes", _dp),
        ("has_coriolis", C.c_int32),
        ("coriolis_f0", C.c_double),
        ("coriolis_beta", C.c_double),
        ("coriolis_y0", C.c_double),
        ("n_boundaries", C.c_int32),
        ("boundaries", C.POINTER(Boundary)),
        ("numerics", C.c_int32),
        ("has_line_local", C.c_int32),
        ("line_local_depth", C.c_double),
        ("relaxation", C.POINTER(Relaxation)),
        ("atmosphere", C.POINTER(Atmosphere)),
    ]


class StagePlan(C.Structure):
    _fields_ = [
        ("base", C.c_int32),
        ("input", C.c_int32),
        ("out", C.c_int32),
        ("acc", C.c_int32),
        ("time", C.c_double),
        ("a", C.c_double),
        ("b", C.c_double),
        ("c", C.c_double),
        ("accumulate", C.c_int32),
        ("w", C.c_double),
        ("keep", C.c_double),
    ]


class RunConfig(C.Structure):
    _fields_ = [
        ("scheme", C.c_int32),
        ("cfl", C.c_double),
        ("t_start", C.c_double),
        ("t_end", C.c_double),
        ("interval", C.c_double),
        ("dt_max", C.c_double),
        ("dt_min", C.c_double),
        ("max_steps", C.c_int64),
        ("stop", C.POINTER(C.c_int32)),
        ("levels", C.c_int32),
    ]


MAX_LEVELS = 8  # DGSWE_MAX_LEVELS


class MultirateStage(C.Structure):
    """dgswe_multirate_stage: one stage pass of a multirate coarse step."""
    _fields_ = [
        ("t", C.c_double),
        ("dt", C.c_double),
        ("finest", C.c_int32),
        ("substep", C.c_int32),
        ("depth", C.c_int32),
        ("stage", C.c_int32),
        ("last", C.c_int32),
        ("start", C.c_double),
        ("input", C.c_double),
        ("beta", C.c_double),
        ("c", C.c_double),
        ("base", C.c_int32),
        ("input_buffer", C.c_int32),
        ("out", C.c_int32),
        ("acc", C.c_int32),
    ]


class MultirateStats(C.Structure):
    _fields_ = [
        ("steps", C.c_int64),
        ("element_evaluations", C.c_int64),
        ("global_evaluations", C.c_int64),
        ("finest_level", C.c_int32),
        ("model_seconds", C.c_double),
        ("ideal_evaluations", C.c_double),
        ("level_evaluations", C.c_double),
        ("line_local_elements", C.c_int64),
        ("plans", C.c_int64),
        ("plan_seconds", C.c_double),
        ("device_seconds", C.c_double),
    ]


class PlanResult(C.Structure):
    _fields_ = [
        ("dt", C.c_double),
        ("stable_step", C.c_double),
        ("finest", C.c_int32),
        ("evaluations", C.c_int64),
        ("level_evaluations", C.c_int64),
        ("inverse_dt_sum", C.c_double),
    ]


class Report(C.Structure):
    _fields_ = [
        ("success", C.c_int32),
        ("final_time", C.c_double),
        ("n_steps", C.c_int64),
        ("dt_min_used", C.c_double),
        ("dt_max_used", C.c_double),
        ("wall_time", C.c_double),
        ("negative_depth_clips", C.c_int64),
        ("message", C.c_char * 256),
        ("device", C.c_char * 128),
    ]


class Profile(C.Structure):
    _fields_ = [
        ("steps", C.c_int64),
        ("total_ms", C.c_double),
        ("face_ms", C.c_double),
        ("stage_ms", C.c_double),
        ("dt_ms", C.c_double),
        ("control_ms", C.c_double),
        ("face_launches", C.c_int64),
        ("stage_launches", C.c_int64),
        ("dt_launches", C.c_int64),
        ("control_launches", C.c_int64),
        ("t_final", C.c_double),
    ]


class FormInfo(C.Structure):
    _fields_ = [
        ("n_elements", C.c_int64),
        ("n_interior_edges", C.c_int64),
        ("n_periodic_edges", C.c_int64),
        ("n_boundary_faces", C.c_int64),
        ("n_affine", C.c_int64),
        ("min_jacobian", C.c_double),
        ("area", C.c_double),
        ("table_checksum", C.c_double),
    ]


MAX_CONSTITUENTS = 8  # DGSWE_MAX_CONSTITUENTS


class AdjointConfig(C.Structure):
    _fields_ = [
        ("scheme", C.c_int32),
        ("cfl", C.c_double),
        ("t_start", C.c_double),
        ("n_steps", C.c_int64),
        ("n_stations", C.c_int32),
        ("stations", _dp),
        ("memory_budget", C.c_double),
        ("station_member", C.POINTER(C.c_int32)),
        ("checkpoint_every", C.c_int64),
    ]


class AdjointStats(C.Structure):
    _fields_ = [
        ("J", C.c_double),
        ("forward_ms", C.c_double),
        ("reverse_ms", C.c_double),
        ("forward_wall_s", C.c_double),
        ("reverse_wall_s", C.c_double),
        ("stride", C.c_int64),
        ("full_segments", C.c_int32),
        ("recomputed_steps", C.c_int64),
        ("stored_states", C.c_int64),
        ("stored_bytes", C.c_double),
    ]


CALLBACK = C.CFUNCTYPE(None, C.c_void_p, C.c_double, _dp, _dp, _dp, C.c_int64)

# entry points shared by every library with this ABI: name → (restype, argtypes)
ENTRY_POINTS = {
    "create": (C.c_int, [C.POINTER(Form), C.c_int, C.POINTER(C.c_void_p)]),
    "destroy": (None, [C.c_void_p]),
    "n_values": (C.c_int64, [C.c_void_p]),
    "upload": (C.c_int, [C.c_void_p, C.c_int32, _dp, _dp, _dp, C.c_int64]),
    "download": (C.c_int, [C.c_void_p, C.c_int32, _dp, _dp, _dp, C.c_int64]),
    "compute_rhs": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, _dp, _dp, _dp, C.c_int64]),
    "compute_rhs_mass_fluxes": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, _dp, _dp, _dp,
                                          C.c_int64, _dp, C.c_int64, _dp, C.c_int64]),
    "stage": (C.c_int, [C.c_void_p, C.POINTER(StagePlan)]),
    "finish": (C.c_int, [C.c_void_p, C.c_int32]),
    "implicit_damping": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_double]),
    "post_process": (C.c_int, [C.c_void_p, C.c_int32]),
    "element_dt": (C.c_int, [C.c_void_p, C.c_double, C.c_int32, _dp, _dp]),
    "step": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double]),
    "run": (C.c_int, [C.c_void_p, C.POINTER(RunConfig), CALLBACK, C.c_void_p, C.POINTER(Report)]),
    "negative_depth_clips": (C.c_int64, [C.c_void_p]),
}
# the CUDA library's own
CUDA_ONLY = {
    "abi_version": (C.c_uint32, []),
    "check_form": (C.c_int, [C.POINTER(Form), C.POINTER(FormInfo), C.c_char_p, C.c_size_t]),
    "status_string": (C.c_char_p, [C.c_int]),
    "last_error": (C.c_char_p, [C.c_void_p]),
    "profile_steps": (C.c_int, [C.c_void_p, C.POINTER(RunConfig), C.c_int64, C.POINTER(Profile)]),
    # local time stepping: the last run's work counts; the level planner (host only)
    "multirate_stats_get": (C.c_int, [C.c_void_p, C.POINTER(MultirateStats)]),
    # the LocalTimeStepping passes of a host-planned coarse step
    "begin_coarse_step": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_uint8),
                                    C.POINTER(C.c_uint8)]),
    "stage_where": (C.c_int, [C.c_void_p, C.POINTER(MultirateStage)]),
    "finish_where": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "depth_flags": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_double,
                              C.POINTER(C.c_uint8)]),
    "planner_create": (C.c_int, [C.POINTER(Form), C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "planner_destroy": (None, [C.c_void_p]),
    "planner_assign": (C.c_int, [C.c_void_p, _dp, C.POINTER(C.c_uint8), C.c_double, C.c_double,
                                 C.POINTER(PlanResult), C.POINTER(C.c_uint8),
                                 C.POINTER(C.c_uint8), C.POINTER(C.c_int32)]),
    "planner_spread": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint8), C.c_int32,
                                 C.POINTER(C.c_uint8), C.POINTER(C.c_uint8)]),
    # a step of a host state: upload, dt, step, download overlapped
    "step_host": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_double, _dp, _dp,
                            _dp, C.c_int64, _dp]),
    # device pointers in and out; working memory in the library's own array
    "autotune": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.POINTER(Tuning)]),
    "compute_rhs_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]),
    # the Standard-kernel helpers of the reference's RHS bench, batched over
    # elements on device arrays
    "apply_diff_matrix": (C.c_int, [C.c_int] + [C.c_void_p] * 7 + [C.c_int64, C.c_int64]),
    "apply_lift": (C.c_int, [C.c_int] + [C.c_void_p] * 7 + [C.c_int64, C.c_int64, C.c_void_p,
                                                            C.c_int64]),
    "coriolis_source": (C.c_int, [C.c_int] + [C.c_void_p] * 4 + [C.c_double, C.c_int64]),
    "combine_derivatives": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)] + [C.c_void_p] * 4
                            + [C.c_int64, C.c_int64]),
    "helpers_last_error": (C.c_char_p, []),
    # ensembles of independent members
    "ensemble_create": (C.c_int, [C.POINTER(Form), C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "ensemble_destroy": (None, [C.c_void_p]),
    "ensemble_last_error": (C.c_char_p, [C.c_void_p]),
    "ensemble_n_members": (C.c_int, [C.c_void_p]),
    "ensemble_n_values": (C.c_int64, [C.c_void_p, C.c_int]),
    "ensemble_upload": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_int64]),
    "ensemble_download": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_int64]),
    "ensemble_run": (C.c_int, [C.c_void_p, C.POINTER(RunConfig), C.c_int64, C.POINTER(Report),
                               C.POINTER(Profile)]),
    # the discrete adjoint
    "adjoint_create": (C.c_int, [C.POINTER(Form), C.c_int, C.POINTER(AdjointConfig),
                                 C.POINTER(C.c_void_p)]),
    "adjoint_create_ensemble": (C.c_int, [C.POINTER(Form), C.c_int, C.c_int,
                                          C.POINTER(AdjointConfig), C.POINTER(C.c_void_p)]),
    "adjoint_member_offset": (C.c_int64, [C.c_void_p, C.c_int]),
    "adjoint_member_misfit": (C.c_int, [C.c_void_p, _dp]),
    "adjoint_destroy": (None, [C.c_void_p]),
    "adjoint_last_error": (C.c_char_p, [C.c_void_p]),
    "adjoint_n_values": (C.c_int64, [C.c_void_p]),
    "adjoint_stations": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), _dp]),
    "adjoint_forward": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "adjoint_reverse": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp]),
    "adjoint_set_parameters": (C.c_int, [C.c_void_p, _dp, _dp]),
    "adjoint_get_stats": (C.c_int, [C.c_void_p, C.POINTER(AdjointStats)]),
}


class Library:
    """The entry points of a shared library exporting this ABI under
    ``prefix`` (``prefix_create``, ``prefix_stage``, …)."""

    def __init__(self, cdll: C.CDLL, prefix: str, extra: dict | None = None):
        self.cdll = cdll
        self.prefix = prefix
        table = dict(ENTRY_POINTS)
        table.update(extra or {})
        for name, (res, args) in table.items():
            fn = getattr(cdll, f"{prefix}_{name}")
            fn.restype = res
            fn.argtypes = args
            setattr(self, name, fn)
        self.has_last_error = hasattr(self, "last_error")

    def error_text(self, handle, status: int) -> str:
        text = ""
        if self.has_last_error and handle:
            raw = self.last_error(handle)
            text = raw.decode() if raw else ""
        return text or f"status {status}"


_cuda_library: Library | None = None


def cuda_library() -> Library:
    """The in-tree CUDA library. Fails loudly if it has not been built: there
    is no CPU fallback."""
    global _cuda_library
    if _cuda_library is None:
        if not LIBRARY_PATH.exists():
            raise RuntimeError(
                f"{LIBRARY_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        cdll = C.CDLL(str(LIBRARY_PATH))
        lib = Library(cdll, "dgswe", CUDA_ONLY)
        if lib.abi_version() != ABI_VERSION:
            raise RuntimeError("libdgswe ABI version mismatch: rebuild it")
        _cuda_library = lib
    return _cuda_library


def exported_symbols() -> list[str]:
    """Every entry point the C header declares, as ``dgswe_<name>``."""
    return sorted(f"dgswe_{n}" for n in list(ENTRY_POINTS) + list(CUDA_ONLY))
