"""Surface extraction over the C ABI (wc_surface_*): a colour field on a vertex grid and marching
cubes on the device, returned as a triangle soup. No counterpart in the reference."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from ._abi import check, lib
from .fluid import Fluid


def case_table() -> tuple[np.ndarray, np.ndarray]:
    """The generated marching-cubes table: counts[256], tris[256, 36] (edge ids, -1 unused)."""
    counts = np.zeros(256, np.uint8)
    tris = np.zeros((256, 36), np.int8)
    check(lib().wc_surface_case_table(A._ptr(counts), A._ptr(tris)), "wc_surface_case_table")
    return counts, tris


class Surface:
    """Buffers for one grid resolution; extract() may be called on any fluid, repeatedly."""

    def __init__(self, grid_res: int, iso: float = 0.5, radius: float = 0.0):
        p = A.SurfaceParams(grid_res=int(grid_res), iso=float(iso), radius=float(radius))
        h = C.c_void_p()
        check(lib().wc_surface_create(C.byref(p), C.byref(h)), "wc_surface_create")
        self._h = h
        self.grid_res = int(grid_res)
        self.num_triangles = 0

    def extract(self, fluid: Fluid) -> int:
        n = C.c_uint64(0)
        check(lib().wc_surface_extract(self._h, fluid._require(), C.byref(n)), "wc_surface_extract")
        self.num_triangles = int(n.value)
        return self.num_triangles

    def triangles(self) -> np.ndarray:
        """(T, 3, 3) float32 vertex positions, counter-clockwise seen from outside the fluid."""
        out = np.zeros((self.num_triangles, 3, 3), np.float32)
        check(lib().wc_surface_get_triangles(self._h, A._ptr(out), self.num_triangles), "wc_surface_get_triangles")
        return out

    def field(self) -> np.ndarray:
        """phi[z, y, x] of the last extraction."""
        G = self.grid_res
        out = np.zeros((G, G, G), np.float32)
        check(lib().wc_surface_get_field(self._h, A._ptr(out), out.size), "wc_surface_get_field")
        return out

    def timings(self) -> tuple[float, float]:
        a, b = C.c_float(0), C.c_float(0)
        check(lib().wc_surface_timings(self._h, C.byref(a), C.byref(b)), "wc_surface_timings")
        return a.value, b.value

    def close(self) -> None:
        if self._h is not None:
            lib().wc_surface_destroy(self._h)
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


def mesh_stats(tris: np.ndarray) -> dict:
    """Area, enclosed volume (divergence theorem; positive when the normals point outward),
    open_edges: edges whose uses do not cancel in direction (0 for a closed, consistently
    oriented surface), and nonmanifold_edges: edges used by more than two triangles (two
    sheets touching along a fan diagonal, closed all the same)."""
    t = np.asarray(tris, np.float64)
    if t.size == 0:
        return {"triangles": 0, "area": 0.0, "volume": 0.0, "open_edges": 0, "nonmanifold_edges": 0}
    a, b, c = t[:, 0], t[:, 1], t[:, 2]
    cr = np.cross(b - a, c - a)
    area = 0.5 * np.linalg.norm(cr, axis=1).sum()
    volume = np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0
    keys = {}
    flat = np.asarray(tris, np.float32).reshape(-1, 3)
    _, vid = np.unique(flat.view(np.dtype((np.void, 12))), return_inverse=True)
    vid = vid.reshape(-1, 3)
    for tri in vid:
        for k in range(3):
            u, v = int(tri[k]), int(tri[(k + 1) % 3])
            if u == v:
                continue
            key = (min(u, v), max(u, v))
            keys.setdefault(key, []).append(1 if u < v else -1)
    open_edges = sum(1 for d in keys.values() if sum(d) != 0)
    nonmanifold = sum(1 for d in keys.values() if len(d) > 2)
    return {"triangles": int(t.shape[0]), "area": float(area), "volume": float(volume), "open_edges": open_edges,
            "nonmanifold_edges": nonmanifold}
