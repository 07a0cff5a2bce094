"""Hand-computable cases for the oracle (the reference has no tests of its own; these pin the
equations of density.comp / update.comp and the sort's edge cases)."""
import math

import numpy as np
import pytest

from oracle.oracle import PARTICLE64_DTYPE, to64
from watercube_gb300 import _abi
from watercube_gb300.fluid import dam_break_params, finalize, reference_params


def config_params(n=2):
    p = dam_break_params(16384)
    p.num_particles = n
    return finalize(p)


def state_at(positions, velocities=None):
    s = np.zeros(len(positions), _abi.PARTICLE_DTYPE)
    s["position"] = np.asarray(positions, np.float32)
    if velocities is not None:
        s["velocity"] = np.asarray(velocities, np.float32)
    return s


def run_density64(oracle, p, s):
    s64 = to64(s)
    srt, keys, perm, counts, offsets = oracle.sort(p, s64)
    nc = oracle.density(p, srt, counts, offsets)
    return srt, perm, nc, counts, offsets


def consts64(p):
    h = float(p.kernel_radius)
    return h, 315.0 / (64 * math.pi * h**9), -45.0 / (math.pi * h**6), 45.0 / (math.pi * h**6)


def test_two_particles_density_and_eos(oracle):
    p = config_params(2)
    h, c6, _, _ = consts64(p)
    m = float(p.particle_mass)
    r = 0.37 * h
    s = state_at([[0.5, 0.5, 0.5], [0.5 + r, 0.5, 0.5]])
    srt, perm, nc, _, _ = run_density64(oracle, p, s)
    rr = float(np.float32(0.5 + r) - np.float32(0.5))
    expect = m * c6 * h**6 + m * c6 * (h * h - rr * rr) ** 3
    assert np.allclose(srt["density"], expect, rtol=1e-12)
    assert list(nc) == [1, 1]
    # linear EOS, p = k (rho - rho0) with the density that excludes the wall term
    assert np.allclose(srt["pressure"], float(p.stiffness) * (expect - float(p.rest_density)), rtol=1e-12)


def test_isolated_particle_and_cubic_eos(oracle):
    p = config_params(1)
    p.eos = _abi.WC_EOS_DESBRUN_CUBIC
    p.rest_pressure = 2.5
    h, c6, _, _ = consts64(p)
    m = float(p.particle_mass)
    srt, _, nc, _, _ = run_density64(oracle, p, state_at([[0.3, 0.4, 0.5]]))
    rho = m * c6 * h**6
    assert nc[0] == 0
    assert math.isclose(srt["density"][0], rho, rel_tol=1e-12)
    pr = 2.5 + float(p.stiffness) * ((rho / float(p.rest_density)) ** 3 - 1)
    assert math.isclose(srt["pressure"][0], pr, rel_tol=1e-12)


def test_pair_at_exactly_h_is_not_a_neighbour(oracle):
    p = config_params(2)
    h = np.float32(p.kernel_radius)
    # dist >= h is rejected (density.comp:117)
    x0 = np.float32(0.25)
    x1 = np.float32(x0 + h)
    s = state_at([[x0, 0.5, 0.5], [x1, 0.5, 0.5]])
    if np.float32(x1 - x0) >= h:
        _, _, nc, _, _ = oracle_density32(oracle, p, s)
        assert list(nc) == [0, 0]


def oracle_density32(oracle, p, s):
    srt, keys, perm, counts, offsets = oracle.sort(p, s)
    nc = oracle.density(p, srt, counts, offsets)
    return srt, perm, nc, counts, offsets


def test_wall_density_z_branch_tests_y(oracle):
    """density.comp:74 tests p.y where p.z is meant: a particle near the top (y > size-h) with a
    mid-box z gets m*W(size - z) added, a negative cube since size - z > h."""
    p = reference_params()
    p.num_particles = 1
    p = finalize(p)
    h, c6, _, _ = consts64(p)
    m = float(p.particle_mass)
    y = 1.0 - 0.5 * h
    z = 0.5
    srt, _, _, _, _ = run_density64(oracle, p, state_at([[0.5, y, z]]))
    wall = m * c6 * (h * h - (1.0 - y) ** 2) ** 3 + m * c6 * (h * h - (1.0 - z) ** 2) ** 3
    expect = m * c6 * h**6 + 4 * wall
    assert math.isclose(srt["density"][0], expect, rel_tol=1e-9)
    assert srt["density"][0] < 0  # the quirk is live


def test_pair_forces_are_opposite(oracle):
    p = config_params(2)
    h = float(p.kernel_radius)
    s = state_at([[0.5, 0.5, 0.5], [0.5 + 0.3 * h, 0.5 + 0.2 * h, 0.5]], [[0.1, 0, 0], [-0.1, 0.05, 0]])
    p.gravity[1] = 0.0
    s64 = to64(s)
    srt, keys, perm, counts, offsets = oracle.sort(p, s64)
    oracle.density(p, srt, counts, offsets)
    srt["pressure"] = 5.0  # positive pressure so the pressure term acts
    dt = 1e-4
    out = oracle.update(p, srt, counts, offsets, dt)
    dv = (out["velocity"] - srt["velocity"]) * srt["density"][:, None] / dt  # force
    assert np.allclose(dv[0], -dv[1], rtol=1e-9, atol=1e-9)


def test_free_fall_and_wall_bounce(oracle):
    p = config_params(2)
    dt = 1e-3
    s = state_at([[0.5, 0.5, 0.5], [0.2, 0.0015, 0.7]], [[0, 0, 0], [0, -2.0, 0]])
    s64 = to64(s)
    srt, keys, perm, counts, offsets = oracle.sort(p, s64)
    oracle.density(p, srt, counts, offsets)
    out = oracle.update(p, srt, counts, offsets, dt)
    i0 = int(np.where(perm == 0)[0][0])
    i1 = int(np.where(perm == 1)[0][0])
    g = float(np.float32(-9.81))
    assert math.isclose(out["velocity"][i0][1], g * dt, rel_tol=1e-9)
    assert math.isclose(out["position"][i0][1], 0.5 + g * dt * dt, rel_tol=1e-9)
    # particle 1 crosses y < border: clamped to border, velocity reflected with restitution 0.5
    border = float(np.float32(p.wall_border))
    assert out["position"][i1][1] == border
    assert math.isclose(out["velocity"][i1][1], -0.5 * (-2.0 + g * dt), rel_tol=1e-6)


def test_keys_edges(oracle):
    p = config_params(6)
    R = p.grid_res
    bin_ = np.float32(p.bin_size)
    s = state_at(
        [
            [0.0, 0.0, 0.0],  # origin
            [1.0, 1.0, 1.0],  # p = size -> clamped to R-1
            [-0.2, 0.5, 0.5],  # negative -> 0
            [np.float32(3) * bin_, 0.5, 0.5],  # on a cell face
            [np.nan, 0.5, 0.5],  # NaN -> 0
            [np.inf, -np.inf, 0.5],  # +inf -> R-1, -inf -> 0
        ]
    )
    _, keys, _, counts, _ = oracle.sort(p, s)
    mid = int(np.float32(0.5) / bin_)

    def key(x, y, z):
        return (z * R + y) * R + x

    face = int(np.float32(np.float32(3) * bin_) / bin_)
    assert list(keys) == [
        key(0, 0, 0),
        key(R - 1, R - 1, R - 1),
        key(0, mid, mid),
        key(face, mid, mid),
        key(0, mid, mid),
        key(R - 1, 0, mid),
    ]
    assert counts.sum() == 6


def test_sort_is_stable_all_in_one_cell(oracle):
    p = config_params(50)
    rng = np.random.default_rng(0)
    s = state_at(0.5 + rng.uniform(0, 0.5 * float(p.bin_size), size=(50, 3)))
    _, keys, perm, counts, offsets = oracle.sort(p, s)
    assert len(set(keys.tolist())) == 1
    assert list(perm) == list(range(50))
    assert counts.max() == 50


def test_sort_is_a_stable_counting_sort(oracle):
    p = config_params(5000)
    rng = np.random.default_rng(1)
    s = state_at(rng.uniform(-0.05, 1.05, size=(5000, 3)))
    _, keys, perm, counts, offsets = oracle.sort(p, s)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(perm, order)
    assert np.array_equal(np.cumsum(counts) - counts, offsets)


def test_cull_threshold(oracle):
    for h in [0.04, 0.0457, 0.011425, 1.0, 3.3e-3]:
        t = np.float32(oracle.cull_threshold(h))
        hf = np.float32(h)
        assert np.sqrt(t) < hf
        assert np.sqrt(np.nextafter(t, np.float32(np.inf))) >= hf


def test_generators(oracle):
    p = config_params(16384)
    s = oracle.generate_dam_break(p, 0)
    pos = s["position"]
    h = float(p.kernel_radius)
    assert pos.min() > 0 and pos[:, 0].max() < 21 * h / 2
    # 20 x 41 x 20 lattice, first 16,384 sites, x fastest then z then y
    assert np.allclose(pos[1] - pos[0], [h / 2, 0, 0], atol=0.03 * h)
    assert np.allclose(pos[20] - pos[0], [0, 0, h / 2], atol=0.03 * h)
    assert np.allclose(pos[400] - pos[0], [0, h / 2, 0], atol=0.03 * h)
    jit = pos - np.round(pos / (h / 2) - 0.5)[:, :] * 0  # noqa: F841
    q = reference_params()
    q.num_particles = 1000
    q = finalize(q)
    r = oracle.generate_reference_lattice(q, 0)
    d = 1.75 * float(q.particle_radius)
    assert np.allclose(r["position"][1] - r["position"][0], [d, 0, 0], atol=0.5 * d)


def test_fp64_types(oracle):
    p = config_params(2)
    s = to64(state_at([[0.5, 0.5, 0.5], [0.51, 0.5, 0.5]]))
    assert s.dtype == PARTICLE64_DTYPE
    oracle.step(p, s, 1e-3, 3)
    assert np.isfinite(s["position"]).all()
