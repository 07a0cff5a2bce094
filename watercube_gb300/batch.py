"""Batches of independent scenes over the C ABI (wc_batch_*): one global sort and one launch per
stage for all scenes, replayed as one CUDA graph. No counterpart in the reference, which runs a
single scene."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from ._abi import Params, SceneSpec, Tuning, check, lib


def batch_specs(num_scenes: int = 512, n_min: int = 4096, n_max: int = 65536, seed: int = 0) -> list[SceneSpec]:
    """The batched workload's scene draw (log-uniform counts, random blocks, k in [2, 6])."""
    arr = (SceneSpec * num_scenes)()
    check(lib().wc_generate_batch_specs(seed, num_scenes, n_min, n_max, arr), "wc_generate_batch_specs")
    return list(arr)


def scene_params(spec: SceneSpec) -> Params:
    p = Params()
    check(lib().wc_scene_params(C.byref(spec), C.byref(p)), "wc_scene_params")
    return p


def scene_particles(spec: SceneSpec, p: Params) -> np.ndarray:
    out = A.particles(spec.num_particles)
    check(lib().wc_generate_scene(C.byref(spec), C.byref(p), A._ptr(out)), "wc_generate_scene")
    return out


class Batch:
    """Scenes given as finalized parameters and their initial states (one array per scene)."""

    DIAG_FIELDS = ("mass", "px", "py", "pz", "kinetic", "potential")

    def __init__(self, params: list[Params], initial: list[np.ndarray]):
        if len(params) != len(initial):
            raise A.WatercubeError(A.WC_ERR_INVALID_ARG, "one initial state per scene")
        arr = (Params * len(params))(*params)
        h = C.c_void_p()
        check(lib().wc_batch_create(arr, len(params), C.byref(h)), "wc_batch_create")
        self._h = h
        self.num_scenes = len(params)
        self.num_particles = int(lib().wc_batch_num_particles(h))
        state = np.ascontiguousarray(np.concatenate(initial) if initial else A.particles(0), dtype=A.PARTICLE_DTYPE)
        check(lib().wc_batch_setup(h, A._ptr(state), state.shape[0]), "wc_batch_setup")

    @classmethod
    def from_specs(cls, specs: list[SceneSpec]) -> "Batch":
        params = [scene_params(s) for s in specs]
        return cls(params, [scene_particles(s, p) for s, p in zip(specs, params)])

    def step(self, dt: float, nsteps: int = 1) -> None:
        check(lib().wc_batch_step(self._h, float(dt), int(nsteps)), "wc_batch_step")

    def particles(self) -> np.ndarray:
        out = A.particles(self.num_particles)
        check(lib().wc_batch_get_particles(self._h, A._ptr(out), self.num_particles), "wc_batch_get_particles")
        return out

    def set_particles(self, state: np.ndarray) -> None:
        state = np.ascontiguousarray(state, dtype=A.PARTICLE_DTYPE)
        check(lib().wc_batch_set_particles(self._h, A._ptr(state), state.shape[0]), "wc_batch_set_particles")

    def step_host(self, dt: float, inp: np.ndarray | None = None, out: np.ndarray | None = None) -> None:
        """set_particles(inp) (when given), one step and particles() into `out` (when given) in one
        call, the readback overlapping the step (wc_batch_step_host)."""
        n = self.num_particles
        for a, name in ((inp, "inp"), (out, "out")):
            if a is not None and (a.dtype != A.PARTICLE_DTYPE or a.shape != (n,) or not a.flags.c_contiguous):
                raise ValueError(f"{name} must be a contiguous array of {n} particles")
        if out is not None and not out.flags.writeable:
            raise ValueError("out must be writeable")
        check(lib().wc_batch_step_host(self._h, float(dt), A._ptr(inp) if inp is not None else None,
                                       A._ptr(out) if out is not None else None, n), "wc_batch_step_host")

    def ids(self) -> np.ndarray:
        """Per state slot, the particle's index in the initial state (all scenes concatenated)."""
        out = np.zeros(self.num_particles, np.uint32)
        check(lib().wc_batch_get_ids(self._h, A._ptr(out), self.num_particles), "wc_batch_get_ids")
        return out

    def offsets(self) -> np.ndarray:
        out = (C.c_uint64 * (self.num_scenes + 1))()
        check(lib().wc_batch_scene_offsets(self._h, out))
        return np.array(out[:], dtype=np.uint64)

    def scene(self, s: int, state: np.ndarray | None = None) -> np.ndarray:
        off = self.offsets()
        state = self.particles() if state is None else state
        return state[int(off[s]):int(off[s + 1])]

    def diagnostics(self) -> np.ndarray:
        """(num_scenes, 6) float64: mass, momentum x/y/z, kinetic, potential energy."""
        out = (C.c_double * (6 * self.num_scenes))()
        check(lib().wc_batch_diagnostics(self._h, out), "wc_batch_diagnostics")
        return np.array(out[:], dtype=np.float64).reshape(self.num_scenes, 6)

    def time_steps(self, dt: float, nsteps: int, flush_l2: bool = True) -> np.ndarray:
        ms = np.zeros(nsteps, np.float32)
        check(lib().wc_batch_time_steps(self._h, float(dt), nsteps, int(flush_l2), A._ptr(ms)), "time_steps")
        return ms

    def tune(self, dt: float) -> Tuning:
        t = Tuning()
        check(lib().wc_batch_tune(self._h, float(dt), C.byref(t)), "wc_batch_tune")
        return t

    def set_tuning(self, t: Tuning) -> None:
        check(lib().wc_batch_set_tuning(self._h, C.byref(t)), "wc_batch_set_tuning")

    def tuning(self) -> Tuning:
        t = Tuning()
        check(lib().wc_batch_get_tuning(self._h, C.byref(t)))
        return t

    def device_buffers(self) -> A.DeviceBuffers:
        b = A.DeviceBuffers()
        check(lib().wc_batch_device_buffers(self._h, C.byref(b)))
        return b

    def close(self) -> None:
        if self._h is not None:
            lib().wc_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def shard_scenes(num_scenes: int, rank: int, world: int) -> list[int]:
    """Scenes of one rank when a batch is split across processes (one per GPU): round-robin, so
    every rank gets a similar mix of large and small scenes. Scenes never exchange data."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return list(range(rank, num_scenes, world))
