"""Surface extraction on the GPU: the colour field and the triangle soup bit-exact against the
CPU restatement (oracle/surface_ref.py, fed by the oracle's own cell sort of the same state),
and a closed, outward-oriented mesh around a block of fluid."""
import numpy as np
import pytest

from oracle import surface_ref as R
from watercube_gb300 import _abi
from watercube_gb300.fluid import Fluid, dam_break_params, finalize, generate_dam_break
from watercube_gb300.surface import Surface, mesh_stats

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def evolved_state(gpu):
    p = finalize(dam_break_params(4096))
    st = generate_dam_break(p, 3)
    with Fluid("s", p) as f:
        f.setup(st)
        f.step(1e-3, 40)
        return p, f.particles()


@pytest.mark.parametrize("G", [17, 24])
def test_field_and_triangles_bit_exact(oracle, evolved_state, G):
    p, state = evolved_state
    with Fluid("s", p) as f, Surface(G, iso=0.5) as s:
        f.setup(state)
        nt = s.extract(f)
        phi = s.field()
        tris = s.triangles()
    sorted_state, _, _, counts, offsets = oracle.sort(p, state)
    start = np.append(offsets, np.uint32(state.shape[0]))
    ref_phi = R.field(sorted_state["position"].astype(np.float32), start, p.bin_size, p.grid_res, p.size, G,
                      p.kernel_radius, p.particle_mass, p.rest_density)
    assert np.array_equal(phi, ref_phi)
    ref = R.march(ref_phi, p.size, 0.5)
    assert nt == ref.shape[0] > 0
    assert np.array_equal(tris, ref)


def test_block_of_fluid_in_the_corner(gpu):
    p = finalize(dam_break_params(32768))
    st = generate_dam_break(p, 0)  # a resting block against three walls
    with Fluid("b", p) as f, Surface(64, iso=0.5) as s:
        f.setup(st)
        nt = s.extract(f)
        tris = s.triangles()
        ms_field, ms_mesh = s.timings()
    assert nt > 1000 and ms_field > 0 and ms_mesh > 0
    pos = st["position"]
    assert np.all(tris >= 0) and np.all(tris <= p.size)
    # every vertex lies within the field radius of the fluid's bounding box
    assert np.all(tris.max(axis=(0, 1)) <= pos.max(axis=0) + p.kernel_radius + 1e-6)
    m = mesh_stats(tris)
    assert m["area"] > 0 and m["volume"] > 0


def test_closed_blob(gpu):
    """A ball of particles in the middle of the box: closed, outward oriented, volume close to
    the particles' own volume (N s^3)."""
    p = finalize(dam_break_params(16384))
    s_ = 0.5 * p.kernel_radius
    g = np.arange(-12, 13) * s_
    xx, yy, zz = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], 1)
    pts = pts[np.linalg.norm(pts, axis=1) < 11.5 * s_] + 0.5 * p.size
    q = p.copy()
    q.num_particles = pts.shape[0]
    q = finalize(q)
    st = np.zeros(pts.shape[0], _abi.PARTICLE_DTYPE)
    st["position"] = pts.astype(np.float32)
    with Fluid("ball", q) as f, Surface(96, iso=0.5) as s:
        f.setup(st)
        s.extract(f)
        tris = s.triangles()
    m = mesh_stats(tris)
    assert m["open_edges"] == 0
    assert m["volume"] == pytest.approx(pts.shape[0] * s_**3, rel=0.25)


def test_no_surface_above_the_maximum(gpu, evolved_state):
    p, state = evolved_state
    with Fluid("s", p) as f, Surface(16, iso=1e9) as s:
        f.setup(state)
        assert s.extract(f) == 0
        assert s.triangles().shape == (0, 3, 3)


def test_rejects_a_radius_beyond_the_cell(gpu, evolved_state):
    p, state = evolved_state
    with Fluid("s", p) as f, Surface(16, radius=2 * p.kernel_radius) as s:
        f.setup(state)
        with pytest.raises(_abi.WatercubeError):
            s.extract(f)
