"""The core::Fluid-shaped API on the GPU: update(time) semantics, stage-by-stage calls equal
the graph-launched step, host copies, device buffers, timing."""
import ctypes as C

import numpy as np
import pytest

from helpers import case, fluid
from watercube_gb300 import _abi
from watercube_gb300.fluid import Fluid, finalize

pytestmark = pytest.mark.gpu


def test_reference_usage_pattern(gpu):
    """Fluid::create -> setters -> setup -> update(frame seconds), as WaterCubeApp drives it."""
    f = Fluid.create("fluid").numParticles(20000).gridRes(21).viscosityCoefficient(200).stiffness(100)
    f.setup()
    for _ in range(3):
        f.update(1.0 / 60.0)
    out = f.particles()
    f.synchronize()
    assert out.shape == (20000,) and np.isfinite(out["position"]).all()
    assert f.step_count == 3
    f.close()


def test_update_time_scale_equals_step(gpu):
    p, st = case("refdefaults")
    with fluid(p, st) as a, fluid(p, st) as b:
        a.update(1.0 / 60.0)
        b.step(np.float32(1.0 / 60.0) * np.float32(0.012), 1)
        assert a.particles().tobytes() == b.particles().tobytes()


def test_stages_equal_graph_step(gpu):
    p, st = case("dam16k")
    dts = [1e-3, 5e-4, 1e-3]
    with fluid(p, st) as a, fluid(p, st) as b:
        for dt in dts:
            a.step(dt, 1)  # graph, re-parameterised when dt changes
            b.sort()
            b.density()
            b.integrate(dt)
        assert a.particles().tobytes() == b.particles().tobytes()


def test_host_copies_round_trip(gpu):
    p, st = case("dam16k")
    with fluid(p, st) as f:
        assert f.particles().tobytes() == st.tobytes()
        st2 = st.copy()
        st2["velocity"] = 0.25
        f.set_particles(st2, _abi.WC_BUFFER_SORTED)
        assert f.particles(_abi.WC_BUFFER_SORTED).tobytes() == st2.tobytes()


def test_pinned_host_copies_round_trip(gpu):
    """Pinned host buffers (the end-to-end benchmark's) give the same results as pageable ones."""
    from watercube_gb300.fluid import PinnedBuffer

    p, st = case("dam16k")
    n = st.shape[0]
    hin, hout = PinnedBuffer(32 * n), PinnedBuffer(32 * n)
    try:
        a_in, a_out = hin.particles(n), hout.particles(n)
        a_in[:] = st
        a_in["velocity"] = 0.125
        with fluid(p, st) as f:
            f.set_particles(a_in)
            assert f.particles().tobytes() == a_in.tobytes()
            f.step(1e-3, 2)
            lib = _abi.lib()
            _abi.check(lib.wc_fluid_get_particles(f._handle, _abi.WC_BUFFER_STATE, a_out.ctypes.data, n))
            assert a_out.tobytes() == f.particles().tobytes()
            _abi.check(lib.wc_fluid_get_particles(f._handle, _abi.WC_BUFFER_SORTED, a_out.ctypes.data, n))
            assert a_out.tobytes() == f.particles(_abi.WC_BUFFER_SORTED).tobytes()
    finally:
        hin.free()
        hout.free()


@pytest.mark.parametrize("flags", [0, _abi.WC_FLAG_CELL_TEAMS, _abi.WC_FLAG_TRACK_IDS])
@pytest.mark.parametrize("pinned", [False, True])
def test_update_host_equals_the_three_calls(gpu, flags, pinned):
    """wc_fluid_update_host(time, in, out) = set_particles(in) + update(time) + particles(), bit
    for bit, whether the readback overlaps the force pass (lane passes: parts flagged by the
    pass) or follows the step (cell teams), into pageable or pinned memory; without `in` it
    steps the device state, without `out` it reads nothing back. The 1M case has parts of many
    chunks, the 16k case parts of a few."""
    from watercube_gb300.fluid import PinnedBuffer

    for name in ("dam16k", "dam1m"):
        p, st = case(name, flags)
        n = st.shape[0]
        bufs = [PinnedBuffer(32 * n), PinnedBuffer(32 * n)] if pinned else []
        try:
            a_in = bufs[0].particles(n) if pinned else np.empty(n, st.dtype)
            a_out = bufs[1].particles(n) if pinned else np.empty(n, st.dtype)
            with fluid(p, st) as a, fluid(p, st) as b:
                a_in[:] = st
                for k in range(4):
                    if k == 2:
                        a.update_host(1.0 / 60.0, None, a_out)  # the device state as it is
                        b.update(1.0 / 60.0)
                    elif k == 3:
                        a.update_host(1.0 / 60.0, a_in, None)  # no readback
                        b.set_particles(a_in)
                        b.update(1.0 / 60.0)
                        a_out[:] = a.particles()
                    else:
                        a.update_host(1.0 / 60.0, a_in, a_out)
                        b.set_particles(a_in)
                        b.update(1.0 / 60.0)
                    ref = b.particles()
                    assert a_out.tobytes() == ref.tobytes(), (name, k)
                    a_in[:] = a_out
                    a_in["velocity"] *= 0.5  # an input that differs from the device state
                assert a.step_count == b.step_count == 4
                if flags & _abi.WC_FLAG_TRACK_IDS:
                    assert np.array_equal(a.particle_ids(), b.particle_ids())
        finally:
            for buf in bufs:
                buf.free()


@pytest.mark.parametrize("n", [1, 45, 1000, 12345])
def test_update_host_ragged_sizes(gpu, n):
    """Particle counts that leave a partial last chunk of 32 slots and parts of one chunk or a few
    (the readback's part bookkeeping): the same bytes as set_particles + update + particles()."""
    from watercube_gb300.fluid import generate_reference_lattice, reference_params

    p = reference_params()
    p.num_particles = n
    p = finalize(p)
    st = generate_reference_lattice(p, 0)
    with fluid(p, st) as a, fluid(p, st) as b:
        cur = st.copy()
        out = np.empty_like(st)
        for _ in range(3):
            a.update_host(1.0 / 60.0, cur, out)
            b.set_particles(cur)
            b.update(1.0 / 60.0)
            assert out.tobytes() == b.particles().tobytes(), n
            cur = out.copy()


def test_update_host_checks_its_arguments(gpu):
    p, st = case("dam16k")
    with fluid(p, st) as f:
        lib = _abi.lib()
        assert lib.wc_fluid_update_host(f._handle, 1e-3, None, None, st.shape[0] - 1) == _abi.WC_ERR_INVALID_ARG
        with pytest.raises(ValueError):
            f.update_host(1e-3, st[:-1], None)


def test_set_particles_restarts_tracked_ids(gpu):
    p, st = case("dam16k", _abi.WC_FLAG_TRACK_IDS)
    with fluid(p, st) as f:
        f.step(1e-3, 2)
        ids = f.particle_ids()
        assert not np.array_equal(ids, np.arange(len(ids)))  # the sort moved the particles
        state = f.particles()
        f.set_particles(state)
        assert np.array_equal(f.particle_ids(), np.arange(len(ids)))
        f.step(1e-3, 1)
        out, ids2 = f.particles(), f.particle_ids()
        assert np.array_equal(np.sort(ids2), np.arange(len(ids)))
        moved = np.linalg.norm(out["position"] - state["position"][ids2], axis=1)
        assert moved.max() < 0.01 * p.kernel_radius  # each id follows its own particle (spacing 0.5 h)


def test_device_buffers(gpu):
    p, st = case("dam16k", _abi.WC_FLAG_TRACK_IDS | _abi.WC_FLAG_NEIGHBOR_COUNTS)
    with fluid(p, st) as f:
        b = f.device_buffers()
        assert b.num_particles == st.shape[0] and b.num_cells == p.grid_res**3
        for name in ("state_pos_density", "state_vel_pressure", "sorted_pos_density", "cell_start", "permutation",
                     "neighbor_counts", "particle_ids", "stream"):
            assert getattr(b, name)
        assert b.state_pos_density % 16 == 0


def test_gravity_and_mouse_setters(gpu):
    p, st = case("dam16k")
    with fluid(p, st) as a, fluid(p, st) as b:
        b.setGravity([0.0, 0.0, 0.0])
        a.step(1e-3, 2)
        b.step(1e-3, 2)
        va, vb = a.particles()["velocity"], b.particles()["velocity"]
        assert va[:, 1].mean() < vb[:, 1].mean()


def test_timing_entry_point(gpu):
    p, st = case("dam16k")
    with fluid(p, st) as f:
        ms, kern = f.time_steps(1e-3, 4, flush_l2=True, kernel_times=True)
        assert (ms > 0).all() and kern.shape == (4, 6) and (kern >= 0).all()
        assert Fluid.kernel_names() == ["bin_count", "scan_cells", "scatter_cells", "rank_gather", "density",
                                        "force_integrate"]
        assert f.step_count == 8
        none, kern2 = f.time_steps(1e-3, 3, kernel_times=True, graph_steps=False)
        assert none is None and kern2.shape == (3, 6) and (kern2 > 0).all()
        assert f.step_count == 11
