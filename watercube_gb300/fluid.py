"""Python mirror of the reference's core::Fluid interface over the C ABI.

core::Fluid (src/core/Fluid.h:32-141) is driven as

    fluid = Fluid.create("fluid")
    fluid.numParticles(80000).gridRes(21) ... ; fluid.setup()
    fluid.update(frame_seconds)          # Scene::update -> Fluid::update (Fluid.cpp:342-354)

and so is this class. Method names and argument meanings follow the reference; the differences:
  * setters mutate this object and return it (the reference's setters return a copy of the
    object, Fluid.h:85, so a chained call's effect only survives through the returned copy);
  * rendering members (draw, renderMode, setCameraPosition, setLightPosition, position) only
    store their values: this solver is headless;
  * buffers are readable: particles() is util::getParticles (util.cpp:42-60), uints() is
    util::getUints (util.cpp:62-72) over the sort's tables (Sort.h:35-37).
Every call goes through libwatercube.so; there is no Python fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from ._abi import Params, check, lib


def reference_params() -> Params:
    """The reference's constructor defaults (src/core/Fluid.cpp:9-27)."""
    p = Params()
    lib().wc_params_reference_defaults(C.byref(p))
    return p


def dam_break_params(n: int) -> Params:
    """The dam-break preset at n particles (h scaled to keep particles per cell fixed)."""
    p = Params()
    lib().wc_params_dam_break(C.byref(p), n)
    return p


def finalize(p: Params) -> Params:
    q = p.copy()
    check(lib().wc_params_finalize(C.byref(q)), "wc_params_finalize")
    return q


def generate_dam_break(p: Params, seed: int = 0) -> np.ndarray:
    q = finalize(p)
    out = A.particles(q.num_particles)
    check(lib().wc_generate_dam_break(C.byref(q), seed, A._ptr(out), q.num_particles), "wc_generate_dam_break")
    return out


def generate_reference_lattice(p: Params, seed: int = 0) -> np.ndarray:
    q = finalize(p)
    out = A.particles(q.num_particles)
    check(
        lib().wc_generate_reference_lattice(C.byref(q), seed, A._ptr(out), q.num_particles),
        "wc_generate_reference_lattice",
    )
    return out


class Fluid:
    """core::Fluid on the GB300 solver."""

    def __init__(self, name: str = "fluid", params: Params | None = None):
        self.name = name
        self._params = (params or reference_params()).copy()
        self._handle = None
        self._gravity_dir = (0.0, -1.0, 0.0)
        self._gravity_strength = -self._params.gravity[1] if params is None else None
        self.render_mode = 0
        self.position_offset = (-0.5, -0.5, -0.5)
        self.camera_position = None
        self.light_position = None

    # ---- Fluid::create / setters (Fluid.h:37-59) ---------------------------------------------
    @staticmethod
    def create(name: str = "fluid", params: Params | None = None) -> "Fluid":
        return Fluid(name, params)

    def _set(self, field, value):
        if self._handle is not None:
            raise A.WatercubeError(A.WC_ERR_STATE, f"{field} must be set before setup()")
        setattr(self._params, field, value)
        return self

    def numParticles(self, n: int | None = None):
        if n is None:
            return int(self._params.num_particles)
        return self._set("num_particles", int(n))

    def gridRes(self, r: int):
        return self._set("grid_res", int(r))

    def size(self, s: float):
        return self._set("size", float(s))

    def particleRadius(self, r: float):
        return self._set("particle_radius", float(r))

    def viscosityCoefficient(self, c: float):
        return self._set("viscosity", float(c))

    def stiffness(self, s: float):
        return self._set("stiffness", float(s))

    def restDensity(self, d: float):
        return self._set("rest_density", float(d))

    def restPressure(self, p: float):
        return self._set("rest_pressure", float(p))

    def gravityStrength(self, g: float):
        self._gravity_strength = float(g)
        grav = [float(d) * self._gravity_strength for d in self._gravity_dir]
        self._params.gravity = (C.c_float * 3)(*grav)
        if self._handle is not None:
            check(lib().wc_fluid_set_gravity(self._handle, (C.c_float * 3)(*grav)), "set gravity")
        return self

    def position(self, p):
        self.position_offset = tuple(float(x) for x in p)
        return self

    def renderMode(self, m: int):
        self.render_mode = int(m)
        return self

    def setCameraPosition(self, p):
        self.camera_position = tuple(p)

    def setLightPosition(self, p):
        self.light_position = tuple(p)

    def setMouseRay(self, origin, direction):
        """Fluid::setMouseRay with the ray already in the fluid's frame."""
        o = (C.c_float * 3)(*map(float, origin))
        d = (C.c_float * 3)(*map(float, direction))
        self._params.mouse_origin = o
        self._params.mouse_dir = d
        if self._handle is not None:
            check(lib().wc_fluid_set_mouse_ray(self._handle, o, d), "set mouse ray")

    def setGravity(self, g):
        g3 = (C.c_float * 3)(*map(float, g))
        self._params.gravity = g3
        if self._handle is not None:
            check(lib().wc_fluid_set_gravity(self._handle, g3), "set gravity")
        return self

    def setFlags(self, flags: int):
        return self._set("flags", int(flags))

    @property
    def params(self) -> Params:
        if self._handle is not None:
            p = Params()
            check(lib().wc_fluid_get_params(self._handle, C.byref(p)))
            return p
        return finalize(self._params)

    # ---- lifecycle --------------------------------------------------------------------------------
    def setup(self, initial: np.ndarray | None = None, seed: int = 0) -> "Fluid":
        """Fluid::setup: derive constants, create device buffers, upload the initial state
        (the reference's lattice generator when `initial` is None)."""
        p = finalize(self._params)
        if initial is None:
            initial = generate_reference_lattice(p, seed)
        initial = np.ascontiguousarray(initial, dtype=A.PARTICLE_DTYPE)
        if initial.shape != (p.num_particles,):
            raise A.WatercubeError(A.WC_ERR_INVALID_ARG, f"initial state has shape {initial.shape}")
        if self._handle is None:
            h = C.c_void_p()
            check(lib().wc_fluid_create(C.byref(p), C.byref(h)), "wc_fluid_create")
            self._handle = h
        check(lib().wc_fluid_setup(self._handle, A._ptr(initial), p.num_particles), "wc_fluid_setup")
        return self

    def update(self, time: float) -> None:
        """Fluid::update(double time): one step of dt = float(time) * time_scale."""
        check(lib().wc_fluid_update(self._require(), float(time)), "wc_fluid_update")

    def step(self, dt: float, nsteps: int = 1) -> None:
        check(lib().wc_fluid_step(self._require(), float(dt), int(nsteps)), "wc_fluid_step")

    def sort(self) -> None:
        check(lib().wc_fluid_sort(self._require()), "wc_fluid_sort")

    def density(self) -> None:
        check(lib().wc_fluid_density(self._require()), "wc_fluid_density")

    def integrate(self, dt: float) -> None:
        check(lib().wc_fluid_integrate(self._require(), float(dt)), "wc_fluid_integrate")

    def draw(self) -> None:  # rendering is out of scope for the headless solver
        pass

    def reset(self) -> None:  # BaseObject::reset, a no-op in the reference (Fluid.h:57)
        pass

    def synchronize(self) -> None:
        check(lib().wc_fluid_synchronize(self._require()), "wc_fluid_synchronize")

    @property
    def step_count(self) -> int:
        return int(lib().wc_fluid_step_count(self._require()))

    # ---- buffer access --------------------------------------------------------------------------
    def particles(self, buffer: int = A.WC_BUFFER_STATE) -> np.ndarray:
        n = self.numParticles()
        out = A.particles(n)
        check(lib().wc_fluid_get_particles(self._require(), buffer, A._ptr(out), n), "wc_fluid_get_particles")
        return out

    def set_particles(self, arr: np.ndarray, buffer: int = A.WC_BUFFER_STATE) -> None:
        arr = np.ascontiguousarray(arr, dtype=A.PARTICLE_DTYPE)
        check(lib().wc_fluid_set_particles(self._require(), buffer, A._ptr(arr), arr.shape[0]), "set_particles")

    def update_host(self, time: float, inp: np.ndarray | None = None, out: np.ndarray | None = None) -> None:
        """set_particles(inp) (when given), update(time) and particles() into `out` (when given)
        in one call, the readback overlapping the step (wc_fluid_update_host). Arrays of
        PARTICLE_DTYPE with one row per particle; `out` in pinned memory (PinnedBuffer) lets
        the copies overlap."""
        n = self.numParticles()
        for a, name in ((inp, "inp"), (out, "out")):
            if a is not None and (a.dtype != A.PARTICLE_DTYPE or a.shape != (n,) or not a.flags.c_contiguous):
                raise ValueError(f"{name} must be a contiguous array of {n} particles")
        if out is not None and not out.flags.writeable:
            raise ValueError("out must be writeable")
        check(lib().wc_fluid_update_host(self._require(), float(time), A._ptr(inp) if inp is not None else None,
                                         A._ptr(out) if out is not None else None, n), "wc_fluid_update_host")

    def uints(self, which: int) -> np.ndarray:
        n = self.num_cells if which in (A.WC_UINTS_CELL_COUNTS, A.WC_UINTS_CELL_OFFSETS) else self.numParticles()
        out = np.zeros(n, dtype=np.uint32)
        check(lib().wc_fluid_get_uints(self._require(), which, A._ptr(out), n), "wc_fluid_get_uints")
        return out

    def keys(self):
        return self.uints(A.WC_UINTS_CELL_KEYS)

    def permutation(self):
        return self.uints(A.WC_UINTS_PERMUTATION)

    def cell_counts(self):
        return self.uints(A.WC_UINTS_CELL_COUNTS)

    def cell_offsets(self):
        return self.uints(A.WC_UINTS_CELL_OFFSETS)

    def neighbor_counts(self):
        return self.uints(A.WC_UINTS_NEIGHBOR_COUNTS)

    def particle_ids(self):
        return self.uints(A.WC_UINTS_PARTICLE_IDS)

    @property
    def num_cells(self) -> int:
        r = self.params.grid_res
        return int(r) ** 3

    def device_buffers(self) -> A.DeviceBuffers:
        b = A.DeviceBuffers()
        check(lib().wc_fluid_get_device_buffers(self._require(), C.byref(b)))
        return b

    def time_steps(self, dt: float, nsteps: int, flush_l2: bool = True, kernel_times: bool = False,
                   graph_steps: bool = True):
        """Device times (ms) of nsteps graph-launched steps; optionally per-kernel times of a
        further nsteps individually launched steps (graph_steps=False: those alone, and the
        step times returned are None). Advances the simulation."""
        if not graph_steps and not kernel_times:
            raise A.WatercubeError(A.WC_ERR_INVALID_ARG, "nothing to time")
        step_ms = np.zeros(nsteps, dtype=np.float32) if graph_steps else None
        nk = lib().wc_step_kernel_count()
        kern = np.zeros((nsteps, nk), dtype=np.float32) if kernel_times else None
        check(
            lib().wc_fluid_time_steps(
                self._require(), float(dt), nsteps, int(flush_l2), A._ptr(step_ms) if step_ms is not None else None,
                A._ptr(kern) if kern is not None else None,
            ),
            "wc_fluid_time_steps",
        )
        return step_ms, kern

    @staticmethod
    def kernel_names() -> list[str]:
        return [lib().wc_step_kernel_name(i).decode() for i in range(lib().wc_step_kernel_count())]

    # ---- teardown -------------------------------------------------------------------------------
    # ---- snapshots (no counterpart in the reference) -------------------------------------------
    def save_snapshot(self, path, seed: int = 0) -> None:
        check(lib().wc_fluid_save_snapshot(self._require(), str(path).encode(), int(seed)), "wc_fluid_save_snapshot")

    def load_snapshot(self, path) -> None:
        check(lib().wc_fluid_load_snapshot(self._require(), str(path).encode()), "wc_fluid_load_snapshot")

    @staticmethod
    def from_snapshot(path, name: str = "fluid") -> "Fluid":
        hdr = snapshot_header(path)
        f = Fluid(name, hdr.params)
        h = C.c_void_p()
        check(lib().wc_fluid_create_from_snapshot(str(path).encode(), C.byref(h)), "wc_fluid_create_from_snapshot")
        f._handle = h
        return f

    def close(self) -> None:
        if self._handle is not None:
            lib().wc_fluid_destroy(self._handle)
            self._handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _require(self):
        if self._handle is None:
            raise A.WatercubeError(A.WC_ERR_STATE, "setup() has not been called")
        return self._handle


class PinnedBuffer:
    """Page-locked host memory from the library (for timed host<->device copies)."""

    def __init__(self, nbytes: int):
        self.nbytes = nbytes
        p = C.c_void_p()
        check(lib().wc_alloc_host(nbytes, C.byref(p)), "wc_alloc_host")
        self.ptr = p.value

    def particles(self, n: int) -> np.ndarray:
        buf = (C.c_char * self.nbytes).from_address(self.ptr)
        return np.frombuffer(buf, dtype=A.PARTICLE_DTYPE, count=n)

    def free(self):
        if self.ptr:
            lib().wc_free_host(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def snapshot_header(path) -> A.SnapshotHeader:
    """The verified header of a snapshot file (magic, version, sizes and checksum checked)."""
    h = A.SnapshotHeader()
    check(lib().wc_snapshot_read_header(str(path).encode(), C.byref(h)), "wc_snapshot_read_header")
    return h
