"""Surface extraction without a GPU: the library's generated case table against the oracle's
independent restatement, and size-independent properties of the marching-cubes construction
on analytic fields (closed, consistently oriented meshes; area and volume of a sphere)."""
import math

import numpy as np
import pytest

from oracle import surface_ref as R
from watercube_gb300.surface import case_table, mesh_stats


def test_case_table_matches_oracle(wclib):
    counts, tris = case_table()
    rc, rt = R.case_table()
    assert np.array_equal(counts, rc) and np.array_equal(tris, rt)
    assert counts[0] == 0 and counts[255] == 0
    assert counts.max() <= 5
    # complementary configurations cut the same edges
    for cfg in range(256):
        e1 = sorted(set(tris[cfg, :3 * counts[cfg]].tolist()))
        e2 = sorted(set(tris[255 - cfg, :3 * counts[255 - cfg]].tolist()))
        assert e1 == e2, cfg


def sphere_field(G, r, c=0.5):
    x = np.linspace(0.0, 1.0, G, dtype=np.float64)
    zz, yy, xx = np.meshgrid(x, x, x, indexing="ij")
    d = np.sqrt((xx - c) ** 2 + (yy - c) ** 2 + (zz - c) ** 2)
    return (1.0 - d / r).astype(np.float32)  # > 0 inside, iso 0 at the sphere


def test_sphere_is_closed_with_the_right_area_and_volume():
    r = 0.3
    phi = sphere_field(25, r)
    tris = R.march(phi, 1.0, 0.0)
    st = mesh_stats(tris)
    assert st["open_edges"] == 0
    assert st["volume"] == pytest.approx(4 / 3 * math.pi * r**3, rel=0.03)
    assert st["area"] == pytest.approx(4 * math.pi * r**2, rel=0.03)


@pytest.mark.parametrize("seed", range(4))
def test_random_fields_give_closed_oriented_meshes(seed):
    rng = np.random.default_rng(seed)
    G = 14
    phi = rng.normal(0.0, 1.0, (G, G, G)).astype(np.float32)
    phi[[0, -1], :, :] = -1.0  # outside on the domain boundary: every component is closed
    phi[:, [0, -1], :] = -1.0
    phi[:, :, [0, -1]] = -1.0
    st = mesh_stats(R.march(phi, 1.0, 0.0))
    assert st["triangles"] > 100
    assert st["open_edges"] == 0
    assert st["volume"] > 0  # normals point out of the inside region


def test_a_missing_triangle_is_detected():
    tris = R.march(sphere_field(17, 0.3), 1.0, 0.0)
    assert mesh_stats(tris)["open_edges"] == 0
    assert mesh_stats(tris[1:])["open_edges"] == 3
