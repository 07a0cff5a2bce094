"""Edge cases on the GPU: empty and single-particle fluids, coincident particles, a particle
at p = size, all particles in one cell, non-finite input (reported, not faulted)."""
import numpy as np
import pytest

from helpers import case, fluid
from oracle.oracle import to64
from watercube_gb300 import _abi
from watercube_gb300.fluid import Fluid, dam_break_params, finalize

pytestmark = pytest.mark.gpu


def small(n, flags=_abi.WC_FLAG_NEIGHBOR_COUNTS):
    p = dam_break_params(16384)
    p.num_particles = n
    p.flags |= flags
    return finalize(p)


def states(positions):
    s = np.zeros(len(positions), _abi.PARTICLE_DTYPE)
    if len(positions):
        s["position"] = np.asarray(positions, np.float32)
    return s


def test_empty_fluid(gpu):
    p = small(0)
    with fluid(p, states([])) as f:
        f.step(1e-3, 3)
        f.synchronize()
        assert f.particles().shape == (0,)
        assert f.cell_counts().sum() == 0


def test_single_particle_free_fall(gpu, oracle):
    p = small(1)
    st = states([[0.5, 0.5, 0.5]])
    with fluid(p, st) as f:
        f.step(1e-3, 10)
        out = f.particles()
    ref = to64(st)
    oracle.step(p, ref, 1e-3, 10)
    assert np.allclose(out["position"], ref["position"], rtol=0, atol=1e-6)
    assert np.allclose(out["velocity"], ref["velocity"], rtol=1e-5)


def test_coincident_particles(gpu, oracle):
    p = small(3)
    st = states([[0.4, 0.4, 0.4], [0.4, 0.4, 0.4], [0.41, 0.4, 0.4]])
    with fluid(p, st) as f:
        f.sort()
        f.density()
        srt = f.particles(_abi.WC_BUFFER_SORTED)
        nc = f.neighbor_counts()
        f.integrate(1e-3)
        out = f.particles()
    assert list(nc) == [2, 2, 2]
    assert np.isfinite(out["position"]).all() and np.isfinite(out["velocity"]).all()
    s64, _, _, counts, offsets = oracle.sort(p, to64(st))
    oracle.density(p, s64, counts, offsets)
    assert np.allclose(srt["density"], s64["density"], rtol=1e-5)


def test_particle_at_box_faces(gpu, oracle):
    p = small(4)
    st = states([[1.0, 1.0, 1.0], [0.0, 0.0, 0.0], [1.0, 0.5, 0.0], [0.999, 0.999, 0.999]])
    with fluid(p, st) as f:
        f.step(1e-3, 1)
        out = f.particles()
        keys = f.keys()
    assert np.isfinite(out["position"]).all()
    border = np.float32(p.wall_border)
    assert (out["position"] >= border).all() and (out["position"] <= np.float32(1.0) - border).all()
    _, okeys, _, _, _ = oracle.sort(p, out)
    assert keys.shape == okeys.shape


def test_all_in_one_cell_density(gpu, oracle):
    p, st = case("dam16k", _abi.WC_FLAG_NEIGHBOR_COUNTS)
    n = 2000
    p = p.copy()
    p.num_particles = n
    rng = np.random.default_rng(2)
    b = float(p.bin_size)
    st = states(0.5 + rng.uniform(0.1 * b, 0.9 * b, size=(n, 3)))
    with fluid(p, st) as f:
        f.sort()
        f.density()
        srt = f.particles(_abi.WC_BUFFER_SORTED)
        nc = f.neighbor_counts()
    o_sorted, _, _, counts, offsets = oracle.sort(p, st)
    nc32 = oracle.density(p, o_sorted, counts, offsets)
    assert np.array_equal(nc, nc32)
    s64 = to64(srt)
    oracle.density(p, s64, counts, offsets)
    assert (np.abs(srt["density"] - s64["density"]) / np.abs(s64["density"])).max() <= 1e-5


def test_nonfinite_position_is_reported(gpu):
    p = small(64)
    rng = np.random.default_rng(3)
    st = states(rng.uniform(0.3, 0.6, size=(64, 3)))
    st["position"][5, 1] = np.nan
    with fluid(p, st) as f:
        f.step(1e-3, 1)
        with pytest.raises(_abi.WatercubeError) as e:
            f.synchronize()
        assert e.value.status == _abi.WC_ERR_NUMERIC
        # the error is reported once and cleared; the handle stays usable
        good = states(rng.uniform(0.3, 0.6, size=(64, 3)))
        f.set_particles(good)
        f.step(1e-3, 1)
        f.synchronize()


def test_wrong_sizes_rejected(gpu):
    p = small(10)
    with fluid(p, states(np.full((10, 3), 0.5))) as f:
        with pytest.raises(_abi.WatercubeError) as e:
            f.set_particles(states(np.full((11, 3), 0.5)))
        assert e.value.status == _abi.WC_ERR_INVALID_ARG
    f = Fluid.create("x", p)
    with pytest.raises(_abi.WatercubeError):
        f.setup(states(np.full((9, 3), 0.5)))
    f.close()


def crowd(n, p, seed=4):
    """n particles inside one cell of p's grid (cell (10, 10, 10))."""
    rng = np.random.default_rng(seed)
    b = float(p.bin_size)
    return states(10 * b + rng.uniform(0.1 * b, 0.9 * b, size=(n, 3)))


def test_overfull_cell_is_not_evaluated(gpu):
    """A cell of 3,000 particles (over the 2,048 limit; 2,000 is evaluated above): the neighbour
    passes skip it, the particles keep their state, and the step reports WC_ERR_NUMERIC instead
    of spending O(N^2) work on it. (Even unguarded this case would take well under a second.)"""
    p = small(3000)
    st = crowd(3000, p)
    with fluid(p, st) as f:
        f.step(1e-3, 3)
        with pytest.raises(_abi.WatercubeError) as e:
            f.synchronize()
        assert e.value.status == _abi.WC_ERR_NUMERIC and "2048" in str(e.value)
        out = f.particles()
    assert np.array_equal(np.sort(out["position"], axis=0), np.sort(st["position"], axis=0))


def test_nonfinite_state_is_bounded(gpu):
    """Every position NaN: all particles bin to cell 0; the step reports the non-finite input and
    the overfull cell without evaluating it."""
    p = small(3000)
    st = states(np.full((3000, 3), np.nan))
    with fluid(p, st) as f:
        f.step(1e-3, 5)
        with pytest.raises(_abi.WatercubeError) as e:
            f.synchronize()
        assert e.value.status == _abi.WC_ERR_NUMERIC


def test_overfull_cell_sort_is_bounded(gpu):
    """A million particles in one cell: the sort places a cell of more than 65,536 particles in
    arrival order instead of counting, for each member, the members before it (10^12 steps
    here), so the step ends promptly; the permutation is still a permutation of the input and
    the step reports WC_ERR_NUMERIC."""
    import time

    n = 1 << 20
    p = small(n, 0)
    st = crowd(n, p)
    with fluid(p, st) as f:
        t = time.perf_counter()
        f.step(1e-3, 2)
        with pytest.raises(_abi.WatercubeError) as e:
            f.synchronize()
        el = time.perf_counter() - t
        assert e.value.status == _abi.WC_ERR_NUMERIC
        perm = f.permutation()
    assert el < 5.0, f"two steps of a one-cell state took {el:.1f} s"
    assert np.array_equal(np.sort(perm), np.arange(n, dtype=np.uint32))


def test_overfull_rows_refused_by_surface_and_surrogate(gpu):
    from watercube_gb300.surface import Surface
    from watercube_gb300.surrogate import Surrogate

    n = 7000  # a row of more than 3 x 2,048 particles
    p = small(n)
    st = crowd(n, p)
    with fluid(p, st) as f, Surface(24) as s:
        with pytest.raises(_abi.WatercubeError) as e:
            s.extract(f)
        assert e.value.status == _abi.WC_ERR_NUMERIC
    with fluid(p, st) as f, Surrogate(layers=1) as sg:
        with pytest.raises(_abi.WatercubeError) as e:
            sg.sample(f, 1e-3, np.zeros((5, n, 4), np.float32))
        assert e.value.status == _abi.WC_ERR_NUMERIC


def test_scan_wait_that_runs_out_is_reported(gpu, wclib):
    """The look-back's bounded wait made to run out (it polls a descriptor nothing publishes):
    the step reports WC_ERR_TIMEOUT, the process and the handle stay usable, and with the hook
    off the next steps equal a fresh run's bit for bit."""
    p, st = case("dam16k")  # 21^3 cells: three scan tiles
    _abi.check(wclib.wc_debug_scan_stall(1, 64))
    try:
        with fluid(p, st) as f:
            f.step(1e-3, 2)
            with pytest.raises(_abi.WatercubeError) as e:
                f.synchronize()
            assert e.value.status == _abi.WC_ERR_TIMEOUT
            _abi.check(wclib.wc_debug_scan_stall(0, 0))
            f.set_particles(st)
            f.step(1e-3, 3)
            again = f.particles()
    finally:
        _abi.check(wclib.wc_debug_scan_stall(0, 0))
    with fluid(p, st) as g:
        g.step(1e-3, 3)
        assert g.particles().tobytes() == again.tobytes()


def test_allocation_failures_unwind_cleanly(gpu, wclib):
    """Every device allocation of fluid, batch, surface and surrogate creation made to fail in
    turn: each call reports WC_ERR_OOM, frees what it held, and the next creation succeeds."""
    torch = pytest.importorskip("torch")
    from watercube_gb300.batch import Batch, batch_specs, scene_params, scene_particles
    from watercube_gb300.surface import Surface
    from watercube_gb300.surrogate import Surrogate

    p, st = case("dam16k")
    specs = batch_specs(2, 1024, 2048, seed=1)
    prm = [scene_params(x) for x in specs]
    init = [scene_particles(x, q) for x, q in zip(specs, prm)]

    def make_fluid():
        f = Fluid.create("a", p)
        try:
            f.setup(st)
            f.step(1e-3, 1)
            f.synchronize()
        finally:
            f.close()

    def make_batch():
        with Batch(prm, init) as b:
            b.step(1e-3, 1)

    def make_surface():
        with fluid(p, st) as f, Surface(24) as s:
            s.extract(f)

    def make_surrogate():
        with Surrogate(layers=1) as s:
            pass

    for make in (make_fluid, make_batch, make_surface, make_surrogate):
        make()  # warm: lazily created library state is in place before the baseline
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        failures = 0
        for k in range(64):
            wclib.wc_debug_fail_allocations(k)
            try:
                make()
                break
            except _abi.WatercubeError as e:
                assert e.status == _abi.WC_ERR_OOM, (make.__name__, k, str(e))
                failures += 1
            finally:
                wclib.wc_debug_fail_allocations(-1)
        else:
            pytest.fail(f"{make.__name__} never succeeded")
        assert failures > 0, make.__name__
        make()
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        assert free0 - free1 < 16 << 20, (make.__name__, free0 - free1)  # nothing leaked
