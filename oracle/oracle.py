"""ctypes front end of the CPU oracle and of the parity reference. TEST INFRASTRUCTURE ONLY:
used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, never by the solver.

  Oracle  -> oracle/_build/liboracle.so  (wc_oracle.cpp: restatement, float and FP64)
  RefLib  -> oracle/_ref/libwcref.so     (the reference's own shaders compiled as C++,
                                          built by oracle/ref/make_ref.py; absent when
                                          neither the reference checkout nor its
                                          generated sources are present)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from watercube_gb300._abi import PARTICLE_DTYPE, Params

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
REF_LIB = HERE / "_ref" / "libwcref.so"

PARTICLE64_DTYPE = np.dtype(
    [("position", np.float64, (3,)), ("density", np.float64), ("velocity", np.float64, (3,)), ("pressure", np.float64)]
)


class Diagnostics(C.Structure):
    _fields_ = [("mass", C.c_double), ("momentum", C.c_double * 3), ("kinetic", C.c_double), ("potential", C.c_double)]


def build_oracle(force: bool = False) -> Path:
    src = HERE / "wc_oracle.cpp"
    hdr = HERE / "wc_oracle.h"
    if not force and LIB.exists() and LIB.stat().st_mtime > max(src.stat().st_mtime, hdr.stat().st_mtime):
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["g++", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-std=c++17",
           str(src), "-o", str(tmp)]
    subprocess.run(cmd, check=True, capture_output=True)
    os.replace(tmp, LIB)
    return LIB


def build_ref() -> Path | None:
    import importlib.util

    spec = importlib.util.spec_from_file_location("wc_make_ref", HERE / "ref" / "make_ref.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class Oracle:
    def __init__(self):
        self.lib = C.CDLL(str(build_oracle()))
        P, pp, u32 = C.c_void_p, C.POINTER(Params), C.c_uint32
        for name, res, args in [
            ("wco_sort", C.c_int, [pp, P, u32, P, P, P, P, P]),
            ("wco_sort64", C.c_int, [pp, P, u32, P, P, P, P, P]),
            ("wco_density_f32", C.c_int, [pp, P, u32, P, P, P, C.c_int]),
            ("wco_density_f64", C.c_int, [pp, P, u32, P, P, P, C.c_int]),
            ("wco_update_f32", C.c_int, [pp, P, P, u32, P, P, C.c_float, C.c_int]),
            ("wco_update_f64", C.c_int, [pp, P, P, u32, P, P, C.c_double, C.c_int]),
            ("wco_step_f32", C.c_int, [pp, P, u32, C.c_float, u32, P, C.c_int]),
            ("wco_step_f64", C.c_int, [pp, P, u32, C.c_double, u32, P, C.c_int]),
            ("wco_params_dam_break", C.c_int, [pp, u32]),
            ("wco_params_finalize", C.c_int, [pp]),
            ("wco_generate_dam_break", C.c_int, [pp, C.c_uint64, P, u32]),
            ("wco_generate_reference_lattice", C.c_int, [pp, C.c_uint64, P, u32]),
            ("wco_diagnostics_f32", C.c_int, [pp, P, u32, C.POINTER(Diagnostics)]),
            ("wco_diagnostics_f64", C.c_int, [pp, P, u32, C.POINTER(Diagnostics)]),
            ("wco_cull_threshold", C.c_float, [C.c_float]),
            ("wco_max_threads", C.c_int, []),
        ]:
            fn = getattr(self.lib, name)
            fn.restype = res
            fn.argtypes = args

    @staticmethod
    def ncells(p: Params) -> int:
        return int(p.grid_res) ** 3

    def sort(self, p: Params, state: np.ndarray):
        n = state.shape[0]
        out = np.zeros_like(state)
        keys = np.zeros(n, np.uint32)
        perm = np.zeros(n, np.uint32)
        counts = np.zeros(self.ncells(p), np.uint32)
        offsets = np.zeros(self.ncells(p), np.uint32)
        fn = self.lib.wco_sort64 if state.dtype == PARTICLE64_DTYPE else self.lib.wco_sort
        rc = fn(C.byref(p), _p(state), n, _p(out), _p(keys), _p(perm), _p(counts), _p(offsets))
        assert rc == 0
        return out, keys, perm, counts, offsets

    def density(self, p, sorted_state, counts, offsets, threads=0):
        """In place; returns neighbour counts."""
        n = sorted_state.shape[0]
        nc = np.zeros(n, np.uint32)
        fn = self.lib.wco_density_f64 if sorted_state.dtype == PARTICLE64_DTYPE else self.lib.wco_density_f32
        assert fn(C.byref(p), _p(sorted_state), n, _p(counts), _p(offsets), _p(nc), threads) == 0
        return nc

    def update(self, p, sorted_state, counts, offsets, dt, threads=0):
        out = np.zeros_like(sorted_state)
        if sorted_state.dtype == PARTICLE64_DTYPE:
            rc = self.lib.wco_update_f64(C.byref(p), _p(sorted_state), _p(out), sorted_state.shape[0], _p(counts),
                                         _p(offsets), float(dt), threads)
        else:
            rc = self.lib.wco_update_f32(C.byref(p), _p(sorted_state), _p(out), sorted_state.shape[0], _p(counts),
                                         _p(offsets), float(dt), threads)
        assert rc == 0
        return out

    def step(self, p, state, dt, nsteps, ids=None, threads=0):
        """In place on `state` (and `ids`)."""
        fn = self.lib.wco_step_f64 if state.dtype == PARTICLE64_DTYPE else self.lib.wco_step_f32
        assert fn(C.byref(p), _p(state), state.shape[0], float(dt), nsteps, _p(ids), threads) == 0

    def dam_break_params(self, n: int) -> Params:
        """The dam-break preset at n particles, finalized, computed by the oracle library alone
        (no solver library is loaded)."""
        p = Params()
        assert self.lib.wco_params_dam_break(C.byref(p), n) == 0
        assert self.lib.wco_params_finalize(C.byref(p)) == 0
        return p

    def generate_dam_break(self, p, seed=0):
        out = np.zeros(p.num_particles, PARTICLE_DTYPE)
        assert self.lib.wco_generate_dam_break(C.byref(p), seed, _p(out), p.num_particles) == 0
        return out

    def generate_reference_lattice(self, p, seed=0):
        out = np.zeros(p.num_particles, PARTICLE_DTYPE)
        assert self.lib.wco_generate_reference_lattice(C.byref(p), seed, _p(out), p.num_particles) == 0
        return out

    def diagnostics(self, p, state) -> dict:
        d = Diagnostics()
        fn = self.lib.wco_diagnostics_f64 if state.dtype == PARTICLE64_DTYPE else self.lib.wco_diagnostics_f32
        assert fn(C.byref(p), _p(state), state.shape[0], C.byref(d)) == 0
        return {"mass": d.mass, "momentum": list(d.momentum), "kinetic": d.kinetic, "potential": d.potential}

    def cull_threshold(self, h: float) -> float:
        return float(self.lib.wco_cull_threshold(h))

    def max_threads(self) -> int:
        return int(self.lib.wco_max_threads())


def to64(state: np.ndarray) -> np.ndarray:
    out = np.zeros(state.shape[0], PARTICLE64_DTYPE)
    for f in ("position", "density", "velocity", "pressure"):
        out[f] = state[f]
    return out


class RefLib:
    """The reference shaders compiled as C++ (dispatch order and uniforms of Sort.cpp/Fluid.cpp)."""

    def __init__(self, path: Path | None = None):
        path = path or REF_LIB
        if not path.is_file():
            raise FileNotFoundError(path)
        self.lib = C.CDLL(str(path))
        P, pp, u32 = C.c_void_p, C.POINTER(Params), C.c_uint32
        for name, args in [
            ("wcref_sort", [pp, P, P, P, P, u32, C.c_int]),
            ("wcref_perm", [pp, P, P, P, P, u32, C.c_int]),
            ("wcref_density", [pp, P, P, P, P, u32, C.c_int]),
            ("wcref_update", [pp, P, P, P, P, P, u32, C.c_float, C.c_int]),
            ("wcref_step", [pp, P, P, P, P, P, u32, C.c_float, u32, C.c_int]),
        ]:
            fn = getattr(self.lib, name)
            fn.restype = C.c_int
            fn.argtypes = args

    @staticmethod
    def _tables(p, n):
        c = max(int(p.grid_res) ** 3, n)
        return np.zeros(c, np.uint32), np.zeros(c, np.uint32)

    def sort(self, p: Params, state: np.ndarray, threads: int = 1):
        n = state.shape[0]
        inp = state.copy()
        out = np.zeros_like(state)
        counts, offsets = self._tables(p, n)
        assert self.lib.wcref_sort(C.byref(p), _p(inp), _p(out), _p(counts), _p(offsets), n, threads) == 0
        sorted_ids = np.zeros(n, np.uint32)
        assert self.lib.wcref_perm(C.byref(p), _p(inp), _p(counts), _p(offsets), _p(sorted_ids), n, threads) == 0
        C_ = int(p.grid_res) ** 3
        return out, sorted_ids, counts[:C_].copy(), offsets[:C_].copy()

    def density(self, p, sorted_state, counts, offsets, threads=1):
        n = sorted_state.shape[0]
        c2, o2 = self._tables(p, n)
        c2[: counts.size] = counts
        o2[: offsets.size] = offsets
        dbg = np.zeros(n, np.uint32)
        assert self.lib.wcref_density(C.byref(p), _p(sorted_state), _p(c2), _p(o2), _p(dbg), n, threads) == 0

    def update(self, p, sorted_state, counts, offsets, dt, threads=1):
        n = sorted_state.shape[0]
        c2, o2 = self._tables(p, n)
        c2[: counts.size] = counts
        o2[: offsets.size] = offsets
        dbg = np.zeros(n, np.uint32)
        out = np.zeros_like(sorted_state)
        inp = sorted_state.copy()
        assert self.lib.wcref_update(C.byref(p), _p(inp), _p(out), _p(c2), _p(o2), _p(dbg), n, float(dt), threads) == 0
        return out

    def step(self, p, state, dt, nsteps, threads=1):
        """Fluid::update nsteps times, in place on state (buffer 1)."""
        n = state.shape[0]
        buf2 = state.copy()
        counts, offsets = self._tables(p, n)
        dbg = np.zeros(n, np.uint32)
        assert self.lib.wcref_step(C.byref(p), _p(state), _p(buf2), _p(counts), _p(offsets), _p(dbg), n, float(dt),
                                   nsteps, threads) == 0
        return buf2


def ref_available() -> bool:
    return REF_LIB.is_file()
