"""ctypes view of include/watercube.h and the loader of libwatercube.so.

The library is the product; this module only declares its C ABI for Python callers. Loading
fails loudly (WatercubeError) when the shared library has not been built: there is no
fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libwatercube.so"

# wc_status
WC_OK = 0
WC_ERR_INVALID_ARG = 1
WC_ERR_OOM = 2
WC_ERR_CUDA = 3
WC_ERR_TIMEOUT = 4
WC_ERR_NUMERIC = 5
WC_ERR_STATE = 6
WC_ERR_UNSUPPORTED = 7

WC_EOS_DESBRUN_CUBIC = 0
WC_EOS_LINEAR = 1

WC_FLAG_WALL_DENSITY = 1 << 0
WC_FLAG_WALL_FORCE = 1 << 1
WC_FLAG_SPEED_CLAMP = 1 << 2
WC_FLAG_MOUSE_FORCE = 1 << 3
WC_FLAG_TRACK_IDS = 1 << 4
WC_FLAG_NEIGHBOR_COUNTS = 1 << 5
WC_FLAG_WALL_WEIGHTS = 1 << 6
WC_FLAG_CELL_TEAMS = 1 << 7
WC_PASSES_TEAM = 0
WC_PASSES_LANE = 1
WC_LOCAL_STALE = 0
WC_LOCAL_TAYLOR = 1
WC_LOCAL_NETWORK = 2
WC_FLAGS_REFERENCE = WC_FLAG_WALL_DENSITY | WC_FLAG_WALL_FORCE | WC_FLAG_SPEED_CLAMP | WC_FLAG_MOUSE_FORCE

WC_BUFFER_STATE = 1
WC_BUFFER_SORTED = 2

WC_UINTS_CELL_KEYS = 1
WC_UINTS_PERMUTATION = 2
WC_UINTS_CELL_COUNTS = 3
WC_UINTS_CELL_OFFSETS = 4
WC_UINTS_NEIGHBOR_COUNTS = 5
WC_UINTS_PARTICLE_IDS = 6

WC_NOALLOC_MAX_PARTICLES = 1 << 18
WC_NOALLOC_MAX_CELLS = 1 << 18


class WatercubeError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[status {status}] {message}")
        self.status = status


class Params(C.Structure):
    _fields_ = [
        ("num_particles", C.c_uint32),
        ("grid_res", C.c_uint32),
        ("size", C.c_float),
        ("particle_radius", C.c_float),
        ("kernel_radius", C.c_float),
        ("particle_mass", C.c_float),
        ("rest_density", C.c_float),
        ("rest_pressure", C.c_float),
        ("stiffness", C.c_float),
        ("viscosity", C.c_float),
        ("gravity", C.c_float * 3),
        ("time_scale", C.c_float),
        ("eos", C.c_uint32),
        ("flags", C.c_uint32),
        ("max_speed", C.c_float),
        ("wall_damping", C.c_float),
        ("wall_border", C.c_float),
        ("mouse_origin", C.c_float * 3),
        ("mouse_dir", C.c_float * 3),
        ("bin_size", C.c_float),
        ("poly6_const", C.c_float),
        ("spiky_const", C.c_float),
        ("visc_const", C.c_float),
        ("reserved", C.c_uint32 * 4),
    ]

    def copy(self) -> "Params":
        p = Params()
        C.memmove(C.byref(p), C.byref(self), C.sizeof(Params))
        return p

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


class DeviceBuffers(C.Structure):
    _fields_ = [
        ("state_pos_density", C.c_void_p),
        ("state_vel_pressure", C.c_void_p),
        ("sorted_pos_density", C.c_void_p),
        ("sorted_vel_pressure", C.c_void_p),
        ("cell_keys", C.c_void_p),
        ("permutation", C.c_void_p),
        ("cell_start", C.c_void_p),
        ("neighbor_counts", C.c_void_p),
        ("particle_ids", C.c_void_p),
        ("stream", C.c_void_p),
        ("num_particles", C.c_uint32),
        ("num_cells", C.c_uint32),
    ]


class SceneSpec(C.Structure):
    _fields_ = [
        ("num_particles", C.c_uint32),
        ("block_min", C.c_float * 3),
        ("block_max", C.c_float * 3),
        ("stiffness", C.c_float),
        ("velocity_sigma", C.c_float),
        ("seed", C.c_uint64),
    ]


class Tuning(C.Structure):
    _fields_ = [
        ("density_blocks_per_sm", C.c_uint32),
        ("force_blocks_per_sm", C.c_uint32),
        ("stream_blocks_per_sm", C.c_uint32),
        ("cell_factor", C.c_float),
        ("step_ms", C.c_float),
        ("trials", C.c_uint32),
        ("pass_variant", C.c_uint32),
    ]


class LocalConfig(C.Structure):
    _fields_ = [
        ("ages", C.c_uint32),
        ("seed", C.c_uint32),
        ("accel_scale", C.c_float),
        ("velocity_scale", C.c_float),
        ("capacity", C.c_uint64),
    ]


class GemmDesc(C.Structure):
    _fields_ = [
        ("m", C.c_uint32), ("n", C.c_uint32), ("k", C.c_uint32), ("k_chunk", C.c_uint32),
        ("a", C.c_void_p), ("a2", C.c_void_p), ("a_rows", C.c_void_p),
        ("lda", C.c_uint32), ("lda2", C.c_uint32), ("k_split", C.c_uint32), ("a_transposed", C.c_int),
        ("b", C.c_void_p), ("ldb", C.c_uint32), ("b_rowmajor", C.c_int),
        ("bias", C.c_void_p), ("add1", C.c_void_p), ("add1_idx", C.c_void_p), ("add2", C.c_void_p),
        ("add2_idx", C.c_void_p), ("ld_add", C.c_uint32), ("relu", C.c_int),
        ("c_f32", C.c_void_p), ("c_bf16", C.c_void_p), ("ldc", C.c_uint32), ("split_stride", C.c_size_t),
        ("accumulate", C.c_int), ("ln_gamma", C.c_void_p), ("ln_beta", C.c_void_p), ("ln_resid", C.c_void_p),
    ]


class SnapshotHeader(C.Structure):
    _fields_ = [
        ("magic", C.c_char * 8),
        ("version", C.c_uint32),
        ("header_bytes", C.c_uint32),
        ("num_particles", C.c_uint64),
        ("step", C.c_uint64),
        ("seed", C.c_uint64),
        ("has_ids", C.c_uint32),
        ("reserved", C.c_uint32),
        ("params", Params),
    ]


class SurfaceParams(C.Structure):
    _fields_ = [("grid_res", C.c_uint32), ("iso", C.c_float), ("radius", C.c_float), ("reserved", C.c_uint32)]


class SurrogateConfig(C.Structure):
    _fields_ = [
        ("layers", C.c_uint32),
        ("seed", C.c_uint64),
        ("velocity_scale", C.c_float),
        ("accel_scale", C.c_float),
    ]


class RolloutStats(C.Structure):
    _fields_ = [
        ("steps", C.c_uint32), ("sph_steps", C.c_uint32), ("surrogate_steps", C.c_uint32),
        ("judged", C.c_uint32), ("reverted", C.c_uint32), ("reserved", C.c_uint32),
        ("mean_density_error", C.c_double), ("max_density_error", C.c_double),
        ("ms_device", C.c_double), ("ms_wall", C.c_double), ("particle_steps_per_s", C.c_double),
        ("diag_start", C.c_double * 6), ("diag_end", C.c_double * 6),
    ]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if name.startswith("diag") else v
        return out


# numpy view of `struct wc_particle` (the reference's std430 Particle, 32 bytes)
PARTICLE_DTYPE = np.dtype(
    [("position", np.float32, (3,)), ("density", np.float32), ("velocity", np.float32, (3,)), ("pressure", np.float32)]
)
assert PARTICLE_DTYPE.itemsize == 32

_lib = None


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _declare(lib) -> None:
    S = C.c_int
    P = C.c_void_p
    pp = C.POINTER(Params)
    sig = {
        "wc_params_reference_defaults": (None, [pp]),
        "wc_params_dam_break": (None, [pp, C.c_uint32]),
        "wc_params_finalize": (S, [pp]),
        "wc_cull_threshold": (C.c_float, [C.c_float]),
        "wc_generate_reference_lattice": (S, [pp, C.c_uint64, P, C.c_uint32]),
        "wc_generate_dam_break": (S, [pp, C.c_uint64, P, C.c_uint32]),
        "wc_fluid_create": (S, [pp, C.POINTER(P)]),
        "wc_fluid_setup": (S, [P, P, C.c_uint32]),
        "wc_fluid_update": (S, [P, C.c_double]),
        "wc_fluid_step": (S, [P, C.c_float, C.c_uint32]),
        "wc_fluid_sort": (S, [P]),
        "wc_fluid_density": (S, [P]),
        "wc_fluid_integrate": (S, [P, C.c_float]),
        "wc_fluid_set_mouse_ray": (S, [P, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
        "wc_fluid_set_gravity": (S, [P, C.POINTER(C.c_float)]),
        "wc_fluid_get_particles": (S, [P, C.c_int, P, C.c_uint32]),
        "wc_fluid_set_particles": (S, [P, C.c_int, P, C.c_uint32]),
        "wc_fluid_update_host": (S, [P, C.c_double, P, P, C.c_uint32]),
        "wc_batch_step_host": (S, [P, C.c_float, P, P, C.c_uint64]),
        "wc_fluid_get_uints": (S, [P, C.c_int, P, C.c_size_t]),
        "wc_fluid_get_params": (S, [P, pp]),
        "wc_fluid_get_device_buffers": (S, [P, C.POINTER(DeviceBuffers)]),
        "wc_fluid_synchronize": (S, [P]),
        "wc_fluid_step_count": (C.c_uint64, [P]),
        "wc_fluid_destroy": (None, [P]),
        "wc_step_kernel_count": (C.c_uint32, []),
        "wc_step_kernel_name": (C.c_char_p, [C.c_uint32]),
        "wc_fluid_time_steps": (S, [P, C.c_float, C.c_uint32, C.c_int, P, P]),
        "wc_generate_batch_specs": (S, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(SceneSpec)]),
        "wc_scene_params": (S, [C.POINTER(SceneSpec), pp]),
        "wc_generate_scene": (S, [C.POINTER(SceneSpec), pp, P]),
        "wc_batch_create": (S, [pp, C.c_uint32, C.POINTER(P)]),
        "wc_batch_setup": (S, [P, P, C.c_uint64]),
        "wc_batch_step": (S, [P, C.c_float, C.c_uint32]),
        "wc_batch_get_particles": (S, [P, P, C.c_uint64]),
        "wc_batch_set_particles": (S, [P, P, C.c_uint64]),
        "wc_batch_scene_offsets": (S, [P, C.POINTER(C.c_uint64)]),
        "wc_batch_num_scenes": (C.c_uint32, [P]),
        "wc_batch_num_particles": (C.c_uint64, [P]),
        "wc_batch_diagnostics": (S, [P, C.POINTER(C.c_double)]),
        "wc_batch_time_steps": (S, [P, C.c_float, C.c_uint32, C.c_int, P]),
        "wc_batch_device_buffers": (S, [P, C.POINTER(DeviceBuffers)]),
        "wc_batch_set_recording": (S, [P, S]),
        "wc_batch_get_accelerations": (S, [P, P, C.c_uint64]),
        "wc_batch_get_ids": (S, [P, P, C.c_uint64]),
        "wc_fluid_set_recording": (S, [P, S]),
        "wc_fluid_get_accelerations": (S, [P, P, C.c_uint32]),
        "wc_batch_destroy": (None, [P]),
        "wc_batch_tune": (S, [P, C.c_float, C.POINTER(Tuning)]),
        "wc_batch_set_tuning": (S, [P, C.POINTER(Tuning)]),
        "wc_batch_get_tuning": (S, [P, C.POINTER(Tuning)]),
        "wc_nn_gemm": (S, [C.POINTER(GemmDesc), P, P]),
        "wc_fluid_save_snapshot": (S, [P, C.c_char_p, C.c_uint64]),
        "wc_snapshot_read_header": (S, [C.c_char_p, C.POINTER(SnapshotHeader)]),
        "wc_fluid_load_snapshot": (S, [P, C.c_char_p]),
        "wc_fluid_create_from_snapshot": (S, [C.c_char_p, C.POINTER(P)]),
        "wc_surface_create": (S, [C.POINTER(SurfaceParams), C.POINTER(P)]),
        "wc_surface_destroy": (None, [P]),
        "wc_surface_extract": (S, [P, P, C.POINTER(C.c_uint64)]),
        "wc_surface_get_triangles": (S, [P, P, C.c_uint64]),
        "wc_surface_get_field": (S, [P, P, C.c_uint64]),
        "wc_surface_timings": (S, [P, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
        "wc_surface_case_table": (S, [P, P]),
        "wc_surrogate_config_default": (None, [C.POINTER(SurrogateConfig)]),
        "wc_surrogate_create": (S, [C.POINTER(SurrogateConfig), C.POINTER(P)]),
        "wc_surrogate_destroy": (None, [P]),
        "wc_surrogate_num_params": (C.c_uint64, [P]),
        "wc_surrogate_get_params": (S, [P, P, C.c_uint64]),
        "wc_surrogate_set_params": (S, [P, P, C.c_uint64]),
        "wc_surrogate_get_grads": (S, [P, P, C.c_uint64]),
        "wc_surrogate_zero_grads": (S, [P]),
        "wc_surrogate_sample": (S, [P, P, C.c_float, P, P, P, C.c_uint32]),
        "wc_surrogate_forward_backward": (S, [P, S, C.POINTER(C.c_double)]),
        "wc_surrogate_predictions": (S, [P, P, C.c_uint32]),
        "wc_surrogate_adam": (S, [P, C.c_float, C.c_float]),
        "wc_surrogate_rollout": (S, [P, P, C.c_float, C.c_uint32, C.c_uint32, C.c_float, S, P,
                                     C.POINTER(RolloutStats)]),
        "wc_local_config_default": (None, [C.POINTER(LocalConfig)]),
        "wc_local_create": (S, [C.POINTER(LocalConfig), C.POINTER(P)]),
        "wc_local_destroy": (None, [P]),
        "wc_local_num_params": (C.c_uint64, [P]),
        "wc_local_get_params": (S, [P, P, C.c_uint64]),
        "wc_local_set_params": (S, [P, P, C.c_uint64]),
        "wc_local_record_fluid": (S, [P, P, C.c_float, C.c_uint32, C.c_int]),
        "wc_local_record_batch": (S, [P, P, C.c_float, C.c_uint32, C.c_int]),
        "wc_local_num_samples": (C.c_uint64, [P, C.c_int]),
        "wc_local_clear_samples": (S, [P]),
        "wc_local_train": (S, [P, C.c_uint32, C.c_uint32, C.c_float, P]),
        "wc_local_gradients": (S, [P, P, C.c_uint32, P, P]),
        "wc_local_get_samples": (S, [P, C.c_int, C.c_uint64, C.c_uint64, P, P]),
        "wc_local_evaluate": (S, [P, C.c_int, P, P, P]),
        "wc_local_predict": (S, [P, P, C.c_float, P, P]),
        "wc_local_rollout": (S, [P, P, C.c_float, C.c_uint32, C.c_uint32, C.c_float, C.POINTER(RolloutStats)]),
        "wc_local_rollout_mode": (S, [P, P, C.c_float, C.c_uint32, C.c_uint32, C.c_float, C.c_int,
                                      C.POINTER(RolloutStats)]),
        "wc_sort_cells_noalloc": (S, [P, C.c_uint32, C.c_uint32, C.c_float, P, P, P, P, P]),
        "wc_sort_cells_noalloc_status": (S, [P]),
        "wc_set_device": (S, [C.c_int]),
        "wc_debug_scan_stall": (S, [S, C.c_uint32]),
        "wc_debug_fail_allocations": (None, [C.c_longlong]),
        "wc_device_count": (C.c_int, []),
        "wc_alloc_host": (S, [C.c_size_t, C.POINTER(P)]),
        "wc_free_host": (None, [P]),
        "wc_last_error": (C.c_char_p, []),
        "wc_status_string": (C.c_char_p, [S]),
        "wc_build_info": (C.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def lib():
    """The loaded libwatercube.so. Raises WatercubeError when it is missing."""
    global _lib
    if _lib is None:
        path = Path(os.environ.get("WATERCUBE_LIB", LIB_PATH))
        if not path.is_file():
            raise WatercubeError(
                WC_ERR_UNSUPPORTED,
                f"{path} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`",
            )
        handle = C.CDLL(str(path))
        _declare(handle)
        _lib = handle
    return _lib


def check(status: int, what: str = "") -> None:
    if status != WC_OK:
        msg = lib().wc_last_error().decode() or lib().wc_status_string(status).decode()
        raise WatercubeError(status, f"{what}: {msg}" if what else msg)


def particles(n: int) -> np.ndarray:
    return np.zeros(n, dtype=PARTICLE_DTYPE)
