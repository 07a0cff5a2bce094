"""Snapshots on the GPU: a fluid resumed from a snapshot continues bit for bit (state, particle
ids, step count, gravity), through both load paths, and loading into a fluid with other
parameters is refused."""
import numpy as np
import pytest

from helpers import case
from watercube_gb300 import _abi
from watercube_gb300.fluid import Fluid, dam_break_params, finalize, generate_dam_break, snapshot_header

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("track_ids", [False, True])
def test_resume_is_bitwise_equal(gpu, tmp_path, track_ids):
    p = finalize(dam_break_params(16384))
    if track_ids:
        p.flags |= _abi.WC_FLAG_TRACK_IDS
    st = generate_dam_break(p, 4)
    snap = tmp_path / "s.wcsnap"
    with Fluid("a", p) as a:
        a.setup(st)
        a.step(1e-3, 25)
        a.setGravity((0.5, -9.0, 0.25))
        a.step(1e-3, 5)
        a.save_snapshot(snap, seed=4)
        a.step(1e-3, 20)
        ref = a.particles()
        ref_ids = a.particle_ids() if track_ids else None
        assert a.step_count == 50
    h = snapshot_header(snap)
    assert h.step == 30 and h.seed == 4 and h.num_particles == 16384 and h.has_ids == int(track_ids)
    assert np.allclose(list(h.params.gravity), [0.5, -9.0, 0.25])
    with Fluid.from_snapshot(snap) as b:
        assert b.step_count == 30
        b.step(1e-3, 20)
        assert b.particles().tobytes() == ref.tobytes()
        if track_ids:
            assert np.array_equal(b.particle_ids(), ref_ids)
        assert b.step_count == 50
    with Fluid("c", p) as c:
        c.setup(st)
        c.load_snapshot(snap)
        c.step(1e-3, 20)
        assert c.particles().tobytes() == ref.tobytes()


def test_load_refuses_other_parameters(gpu, tmp_path):
    p, st = case("dam16k")
    snap = tmp_path / "s.wcsnap"
    with Fluid("a", p) as a:
        a.setup(st)
        a.save_snapshot(snap)
    q = p.copy()
    q.stiffness = p.stiffness * 2
    with Fluid("b", q) as b:
        b.setup(st)
        with pytest.raises(_abi.WatercubeError):
            b.load_snapshot(snap)
    r = p.copy()
    r.flags |= _abi.WC_FLAG_TRACK_IDS
    with Fluid("c", r) as c:
        c.setup(st)
        with pytest.raises(_abi.WatercubeError):
            c.load_snapshot(snap)
