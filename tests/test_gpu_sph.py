"""Density, pressure, forces and integration on the GPU against the oracle.

  * per-particle neighbour counts: bit-exact against the reference stage logic (FP32 oracle);
  * density: max relative error <= 1e-5 against the FP64 oracle on the same input state;
  * pressure: the same bound propagated through the equation of state;
  * one force + integration pass: velocity error <= 1e-4 of the largest velocity change, on
    the same input state, against the FP64 oracle;
  * 200 steps of the 16,384-particle dam break: position drift against the FP64 oracle.
"""
import numpy as np
import pytest

from helpers import case, evolved, fluid
from oracle.oracle import to64
from watercube_gb300 import _abi

pytestmark = pytest.mark.gpu

DENSITY_RTOL = 1e-5

CASES = [
    ("dam16k", 30, 1e-3),
    ("refdefaults", 20, 2e-4),
    ("dam16k_refphysics", 10, 2e-4),
    ("dam16k_walls", 30, 1e-3),
    ("dam1m", 4, 2.5e-4),
    # the end of the 1,000-step benchmark window: densities up to 6.7x rest, ~73 neighbours per
    # particle, 29% of the particles in cells of more than 32 (every dense path at full size)
    ("dam1m", 1000, 2.5e-4),
    ("compressed16k", 3, 1e-4),
]


def gpu_density(p, st):
    with fluid(p, st) as f:
        f.sort()
        f.density()
        return f.particles(_abi.WC_BUFFER_SORTED), f.neighbor_counts(), f.permutation()


def eos_tolerance(p, rho64):
    k = float(p.stiffness)
    if p.eos == _abi.WC_EOS_LINEAR:
        return DENSITY_RTOL * k * np.abs(rho64) + 1e-6
    x = rho64 / float(p.rest_density)
    return DENSITY_RTOL * 3.0 * k * np.abs(x) ** 3 + 1e-6


@pytest.mark.parametrize("variant", ["lane", "team"])
@pytest.mark.parametrize("name,steps,dt", CASES)
def test_density_pressure_neighbours(gpu, oracle, name, steps, dt, variant):
    """Both pass variants: one lane per target (the default) and a 32-lane team per cell."""
    p, st = evolved(name, steps, dt, _abi.WC_FLAG_NEIGHBOR_COUNTS)
    if variant == "team":
        p.flags |= _abi.WC_FLAG_CELL_TEAMS
    srt, nc, perm = gpu_density(p, st)
    o_sorted, _, o_perm, counts, offsets = oracle.sort(p, st)
    assert np.array_equal(perm, o_perm)
    nc32 = oracle.density(p, o_sorted, counts, offsets)
    assert np.array_equal(nc, nc32), f"neighbour counts differ at {np.flatnonzero(nc != nc32)[:10]}"
    s64 = to64(srt)
    oracle.density(p, s64, counts, offsets)
    rel = np.abs(srt["density"] - s64["density"]) / np.abs(s64["density"])
    assert rel.max() <= DENSITY_RTOL, f"max rel density err {rel.max():.3e}"
    # pressure uses the density without the wall term; compare through the EOS bound
    if p.flags & _abi.WC_FLAG_WALL_DENSITY:
        no_wall = p.copy()
        no_wall.flags &= ~_abi.WC_FLAG_WALL_DENSITY
        t64 = to64(srt)
        oracle.density(no_wall, t64, counts, offsets)
        rho_nw = t64["density"]
    else:
        rho_nw = s64["density"]
    perr = np.abs(srt["pressure"] - s64["pressure"])
    assert (perr <= eos_tolerance(p, rho_nw)).all(), f"max pressure err {perr.max():.3e}"


@pytest.mark.parametrize("variant", ["lane", "team"])
@pytest.mark.parametrize("name,steps,dt", CASES)
def test_force_integration_pass(gpu, oracle, name, steps, dt, variant):
    """Both pass variants: one lane per target (the default) and a 32-lane team per cell."""
    p, st = evolved(name, steps, dt)
    if variant == "team":
        p.flags |= _abi.WC_FLAG_CELL_TEAMS
    with fluid(p, st) as f:
        f.sort()
        f.density()
        srt = f.particles(_abi.WC_BUFFER_SORTED)
        f.integrate(dt)
        out = f.particles(_abi.WC_BUFFER_STATE)
    _, _, _, counts, offsets = oracle.sort(p, st)
    s64 = to64(srt)
    o64 = oracle.update(p, s64, counts, offsets, dt)
    dv = np.abs(o64["velocity"] - s64["velocity"]).max()
    verr = np.abs(out["velocity"] - o64["velocity"]).max()
    assert verr <= 1e-4 * dv + 1e-7, f"velocity err {verr:.3e} vs max change {dv:.3e}"
    # positions: the velocity bound times dt, plus the float spacing at the stored coordinate
    perr = np.abs(out["position"] - o64["position"])
    ptol = 1e-4 * dv * dt + np.spacing(np.abs(out["position"]).astype(np.float32)).astype(np.float64)
    assert (perr <= ptol).all(), f"position err {perr.max():.3e}"
    # density and pressure are carried through the update unchanged
    assert np.array_equal(out["density"], srt["density"])
    assert np.array_equal(out["pressure"], srt["pressure"])


def positions_by_id(state, ids):
    out = np.empty((state.shape[0], 3))
    out[ids] = state["position"]
    return out


def test_position_drift_200_steps(gpu, oracle):
    """The 16,384-particle dam break for 200 steps of 1 ms against the FP64 oracle.

    The reference's own FP32 arithmetic (the oracle's float path, bit-exact with the shaders)
    already departs from FP64 by ~1e-2 h at its worst particle after 200 steps: a rounding-level
    difference flips a wall-contact branch and the dynamics amplify it. So the bound checked is:
    the median particle within 1e-4 h, and the worst particle no further from FP64 than the
    reference arithmetic's own worst particle (x2)."""
    p, st = case("dam16k", _abi.WC_FLAG_TRACK_IDS)
    h = float(p.kernel_radius)
    n = st.shape[0]
    with fluid(p, st) as f:
        f.step(1e-3, 200)
        out = f.particles()
        ids = f.particle_ids()
    assert np.array_equal(np.sort(ids), np.arange(n, dtype=np.uint32))
    s64 = to64(st)
    ids64 = np.arange(n, dtype=np.uint32)
    oracle.step(p, s64, 1e-3, 200, ids64)
    s32 = st.copy()
    ids32 = np.arange(n, dtype=np.uint32)
    oracle.step(p, s32, np.float32(1e-3), 200, ids32)
    p64 = positions_by_id(s64, ids64)
    d_gpu = np.abs(positions_by_id(out, ids) - p64).max(axis=1) / h
    d_ref = np.abs(positions_by_id(s32, ids32) - p64).max(axis=1) / h
    print(f"200-step drift / h  GPU: median {np.median(d_gpu):.2e} p99 {np.percentile(d_gpu, 99):.2e} "
          f"max {d_gpu.max():.2e} | reference FP32: median {np.median(d_ref):.2e} "
          f"p99 {np.percentile(d_ref, 99):.2e} max {d_ref.max():.2e}")
    assert np.median(d_gpu) <= 1e-4
    assert d_gpu.max() <= max(2.0 * d_ref.max(), 1e-4)


def test_position_drift_50_steps_within_bound(gpu, oracle):
    """Over 50 steps every particle stays within 1e-4 h of the FP64 oracle."""
    p, st = case("dam16k", _abi.WC_FLAG_TRACK_IDS)
    h = float(p.kernel_radius)
    with fluid(p, st) as f:
        f.step(1e-3, 50)
        out = f.particles()
        ids = f.particle_ids()
    s64 = to64(st)
    ids64 = np.arange(st.shape[0], dtype=np.uint32)
    oracle.step(p, s64, 1e-3, 50, ids64)
    d = np.abs(positions_by_id(out, ids) - positions_by_id(s64, ids64)).max() / h
    assert d <= 1e-4, f"{d:.3e} h"


def test_reference_physics_tracks_oracle(gpu, oracle):
    """The reference's own physics (cubic EOS, wall terms, clamp) over several full steps."""
    p, st = case("refdefaults", _abi.WC_FLAG_TRACK_IDS)
    dt = 0.012 / 60.0
    with fluid(p, st) as f:
        for _ in range(5):
            f.update(1.0 / 60.0)  # dt = time * time_scale, as Fluid::update
        out = f.particles()
        ids = f.particle_ids()
    ref = st.copy()
    ids32 = np.arange(st.shape[0], dtype=np.uint32)
    oracle.step(p, ref, np.float32(1.0 / 60.0) * np.float32(0.012), 5, ids32)
    pg = np.empty((st.shape[0], 3))
    po = np.empty((st.shape[0], 3))
    pg[ids] = out["position"]
    po[ids32] = ref["position"]
    err = np.abs(pg - po).max()
    assert err <= 1e-5 * float(p.kernel_radius), f"{err:.3e}"
    assert dt > 0


def test_wall_weights_fill_the_density_deficit_at_the_walls(gpu):
    """A resting block against the floor and two walls: without boundary handling the particles
    within h of a wall miss part of their kernel's mass; with the wall weight functions their
    density matches the interior's."""
    out = {}
    for flags in (0, _abi.WC_FLAG_WALL_WEIGHTS):
        p, st = case("dam16k", flags | _abi.WC_FLAG_NEIGHBOR_COUNTS)
        srt, _, _ = gpu_density(p, st)
        pos, rho = srt["position"], srt["density"]
        h = p.kernel_radius
        near = (pos[:, 1] < 0.5 * h) & (pos[:, 0] > 2 * h) & (pos[:, 0] < 0.3) & (pos[:, 2] > 2 * h) & (pos[:, 2] < 0.3)
        inner = (pos[:, 1] > 3 * h) & (pos[:, 1] < 0.6) & (pos[:, 0] > 2 * h) & (pos[:, 0] < 0.3) & \
                (pos[:, 2] > 2 * h) & (pos[:, 2] < 0.3)
        out[flags] = (float(np.median(rho[near])), float(np.median(rho[inner])))
    floor0, inner0 = out[0]
    floor1, inner1 = out[_abi.WC_FLAG_WALL_WEIGHTS]
    assert inner1 == pytest.approx(inner0, rel=1e-6)  # the interior does not see the walls
    assert floor0 < 0.85 * inner0  # 0.81 on this lattice (the oracle's FP32 path)
    assert floor1 == pytest.approx(inner1, rel=0.05)  # 1.02


def test_wall_weights_keep_particles_off_the_walls(gpu):
    """300 steps of the 16,384-particle dam break: with the wall weight functions the fluid stays
    inside the box and fewer particles end on the clamp border (0.152 against 0.210 in the FP32
    oracle's run of the same steps; the dam-break stiffness k = 3 is soft, so the falling column
    reaches the floor in both)."""
    frac = {}
    for flags in (0, _abi.WC_FLAG_WALL_WEIGHTS):
        p, st = case("dam16k", flags)
        with fluid(p, st) as f:
            f.step(1e-3, 300)
            pos = f.particles()["position"]
        assert np.all(np.isfinite(pos))
        assert np.all((pos >= p.wall_border) & (pos <= p.size - p.wall_border))
        b = np.float32(p.wall_border)
        on = (pos == b) | (pos == np.float32(p.size) - b)
        frac[flags] = on.any(axis=1).mean()
    assert frac[_abi.WC_FLAG_WALL_WEIGHTS] < 0.85 * frac[0], frac


def test_pass_variants_agree(gpu):
    """The two force pass variants evaluate the same neighbour sets; over 50 steps of the 16,384
    particle dam break their trajectories differ only by rounding (the order of the sums)."""
    p, st = case("dam16k", _abi.WC_FLAG_TRACK_IDS)
    q = p.copy()
    q.flags |= _abi.WC_FLAG_CELL_TEAMS
    out = []
    for prm in (p, q):
        with fluid(prm, st) as f:
            f.step(1e-3, 50)
            pos = np.empty((st.shape[0], 3))
            pos[f.particle_ids()] = f.particles()["position"]
            out.append(pos)
    assert np.abs(out[0] - out[1]).max() <= 1e-4 * float(p.kernel_radius)
