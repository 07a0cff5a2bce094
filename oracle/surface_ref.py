"""CPU restatement of the surface extraction (colour field + marching cubes), for the parity tests.

Test infrastructure only: the product never imports this module. Surface extraction has no
counterpart in the reference (it draws the particles as points), so this oracle is not pinned to
reference outputs; it restates, independently of the CUDA path, the algorithm that path
implements, in float32 with the same operations in the same order so that the comparison can be
exact:

    field   phi(v) = fl(acc * scale), acc summed over the particles of the 27 cells around v
            (cell = trunc(coord / bin) clamped to the grid), rows in (dz, dy) order and sorted
            slots ascending within a row; term = (h2 - d2)^3 for d2 < h2,
            d2 = (dx*dx + dy*dy) + dz*dz, each operation rounded to float32;
            scale = float32(m / rho0 * 315 / (64 pi r^9)) computed in double.
    cases   for each of the 256 corner configurations (corner c at (c&1, c>>1&1, c>>2&1),
            inside = phi > iso): the iso-segments of the six faces (a face with two diagonal inside
            corners gets one segment around each inside corner), chained into loops, each loop
            oriented so that its Newell normal (edge midpoints) points from the inside corners
            of its edges to the outside ones, triangulated as a fan from its first edge.
    emit    cubes in x-fastest order, each vertex on edge (a, b), a < b:
            s = (iso - phi_a) / (phi_b - phi_a), p = p_a + s * (p_b - p_a) in float32.
"""
from __future__ import annotations

import math

import numpy as np

EDGE_A = (0, 2, 4, 6, 0, 1, 4, 5, 0, 1, 2, 3)
EDGE_B = (1, 3, 5, 7, 2, 3, 6, 7, 4, 5, 6, 7)
MAX_TRI = 12


def _edge(a: int, b: int) -> int:
    a, b = min(a, b), max(a, b)
    for e in range(12):
        if EDGE_A[e] == a and EDGE_B[e] == b:
            return e
    raise ValueError((a, b))


def _corner(c: int):
    return (c & 1, (c >> 1) & 1, (c >> 2) & 1)


def case_triangles(cfg: int) -> list[int]:
    inside = lambda c: (cfg >> c) & 1  # noqa: E731
    segs = []
    for a in range(3):
        u, v = (a + 1) % 3, (a + 2) % 3
        for s in range(2):
            cyc = [(s << a) | (du << u) | (dv << v) for du, dv in ((0, 0), (1, 0), (1, 1), (0, 1))]
            fe = [_edge(cyc[k], cyc[(k + 1) % 4]) for k in range(4)]
            cross = [inside(cyc[k]) != inside(cyc[(k + 1) % 4]) for k in range(4)]
            if sum(cross) == 2:
                es = [fe[k] for k in range(4) if cross[k]]
                segs.append((es[0], es[1]))
            elif sum(cross) == 4:
                for k in range(4):
                    if inside(cyc[k]):
                        segs.append((fe[(k + 3) % 4], fe[k]))
    used = [False] * len(segs)
    tris = []
    for first in range(len(segs)):
        if used[first]:
            continue
        used[first] = True
        start, cur = segs[first]
        loop = [start]
        while cur != start:
            loop.append(cur)
            for i, (x, y) in enumerate(segs):
                if not used[i] and (x == cur or y == cur):
                    used[i] = True
                    cur = y if x == cur else x
                    break
            else:
                break
        pts, din, dout = [], np.zeros(3), np.zeros(3)
        for e in loop:
            pa, pb = np.array(_corner(EDGE_A[e]), float), np.array(_corner(EDGE_B[e]), float)
            pts.append(0.5 * (pa + pb))
            if inside(EDGE_A[e]):
                din += pa
                dout += pb
            else:
                din += pb
                dout += pa
        nrm = np.zeros(3)
        for i in range(len(pts)):
            p, q = pts[i], pts[(i + 1) % len(pts)]
            nrm += ((p[1] - q[1]) * (p[2] + q[2]), (p[2] - q[2]) * (p[0] + q[0]), (p[0] - q[0]) * (p[1] + q[1]))
        if float(nrm @ (dout - din)) < 0:
            loop = [loop[0]] + loop[1:][::-1]
        for i in range(1, len(loop) - 1):
            tris += [loop[0], loop[i], loop[i + 1]]
    return tris


def case_table():
    counts = np.zeros(256, np.uint8)
    tris = np.full((256, MAX_TRI * 3), -1, np.int8)
    for cfg in range(256):
        t = case_triangles(cfg)
        counts[cfg] = len(t) // 3
        tris[cfg, :len(t)] = t
    return counts, tris


def field(sorted_pos: np.ndarray, start: np.ndarray, bin_: float, R: int, size: float, G: int, radius: float,
          m: float, rho0: float) -> np.ndarray:
    """phi[z, y, x] (float32). sorted_pos: (n, 3) float32 in sorted order; start: (R^3 + 1,)."""
    f32 = np.float32
    n = sorted_pos.shape[0]
    spacing = f32(size) / f32(G - 1)
    coords = (np.arange(G, dtype=np.float32) * spacing).astype(np.float32)
    h2 = f32(f32(radius) * f32(radius))
    r1 = float(f32(radius))
    r2 = r1 * r1
    r4 = r2 * r2
    r8 = r4 * r4
    scale = f32(float(f32(m)) / float(f32(rho0)) * (315.0 / (64.0 * math.pi * (r8 * r1))))

    def cell(q):
        f = (q / f32(bin_)).astype(np.float32)
        c = np.where(f >= 1.0, np.floor(f), 0).astype(np.int64)
        return np.minimum(c, R - 1)

    zz, yy, xx = np.meshgrid(np.arange(G), np.arange(G), np.arange(G), indexing="ij")
    px, py, pz = coords[xx.ravel()], coords[yy.ravel()], coords[zz.ravel()]
    cx, cy, cz = cell(px), cell(py), cell(pz)
    V = px.size
    acc = np.zeros(V, np.float32)
    # candidate lists per vertex, in the kernel's order
    lists = [[] for _ in range(V)]
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            z = cz + dz
            y = cy + dy
            ok = (z >= 0) & (z < R) & (y >= 0) & (y < R)
            x0 = np.maximum(cx - 1, 0)
            x1 = np.minimum(cx + 1, R - 1)
            row = (z * R + y) * R
            lo = np.where(ok, start[np.where(ok, row + x0, 0)], 0)
            hi = np.where(ok, np.minimum(start[np.where(ok, row + x1 + 1, 0)], n), 0)
            lo = np.minimum(lo, hi)
            for v in np.nonzero(hi > lo)[0]:
                lists[v].append(np.arange(lo[v], hi[v]))
    L = max((sum(len(a) for a in l) for l in lists), default=0)
    idx = np.full((V, max(L, 1)), -1, np.int64)
    for v, l in enumerate(lists):
        if l:
            c = np.concatenate(l)
            idx[v, :c.size] = c
    for col in range(L):
        k = idx[:, col]
        has = k >= 0
        q = sorted_pos[np.where(has, k, 0)]
        dx = (px - q[:, 0]).astype(np.float32)
        dy = (py - q[:, 1]).astype(np.float32)
        dz = (pz - q[:, 2]).astype(np.float32)
        d2 = ((dx * dx + dy * dy).astype(np.float32) + (dz * dz).astype(np.float32)).astype(np.float32)
        hit = has & (d2 < h2)
        t = (h2 - d2).astype(np.float32)
        w = ((t * t).astype(np.float32) * t).astype(np.float32)
        acc = np.where(hit, (acc + w).astype(np.float32), acc)
    return (acc * scale).astype(np.float32).reshape(G, G, G)


def march(phi: np.ndarray, size: float, iso: float, table=None) -> np.ndarray:
    """Triangles (T, 3, 3) float32 in the CUDA path's order."""
    counts, tris = table if table is not None else case_table()
    G = phi.shape[0]
    C = G - 1
    f32 = np.float32
    spacing = f32(size) / f32(G - 1)
    iso = f32(iso)
    out = []
    inside = phi > iso
    for iz in range(C):
        for iy in range(C):
            for ix in range(C):
                cfg = 0
                for c in range(8):
                    if inside[iz + ((c >> 2) & 1), iy + ((c >> 1) & 1), ix + (c & 1)]:
                        cfg |= 1 << c
                for t in range(int(counts[cfg])):
                    tri = []
                    for k in range(3):
                        e = int(tris[cfg, 3 * t + k])
                        a, b = EDGE_A[e], EDGE_B[e]
                        ia = (ix + (a & 1), iy + ((a >> 1) & 1), iz + ((a >> 2) & 1))
                        ib = (ix + (b & 1), iy + ((b >> 1) & 1), iz + ((b >> 2) & 1))
                        fa, fb = phi[ia[2], ia[1], ia[0]], phi[ib[2], ib[1], ib[0]]
                        s = f32(f32(iso - fa) / f32(fb - fa))
                        pa = [f32(f32(i) * spacing) for i in ia]
                        pb = [f32(f32(i) * spacing) for i in ib]
                        tri.append([f32(pa[d] + f32(s * f32(pb[d] - pa[d]))) for d in range(3)])
                    out.append(tri)
    return np.array(out, np.float32).reshape(-1, 3, 3)
