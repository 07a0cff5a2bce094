"""The mouse-ray force on the GPU (update.comp:105-132: the slab test intersectAABB, then the
repulsion of particles within h of the ray, mouseForce), on the committed fixture whose ray
crosses the box: the reference's defaults at 800 particles, the ray entering at (0.1, 0.05)
along +z (tests/golden/mouse_ray_n800.npz, made from the reference's own shaders).

  * sort bit-exact against the reference build's tables;
  * density within 1e-5 of FP64, and of the reference build's FP32 densities;
  * one force + integration pass within 1e-4 of the largest velocity change against FP64;
  * three full steps within 1e-5 h of the reference arithmetic (the FP32 oracle, which equals
    the fixture's stepped state bit for bit);
  * the ray acts: without the mouse force flag the same pass gives different velocities, and
    only for particles within h of the ray.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from helpers import fluid
from oracle.oracle import to64
from watercube_gb300 import _abi

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def load_mouse_case():
    z = np.load(GOLDEN / "mouse_ray_n800.npz")
    p = _abi.Params()
    C.memmove(C.addressof(p), z["params"].tobytes(), C.sizeof(p))
    return p, z


def ray_distance(p, pos):
    o = np.array(p.mouse_origin, np.float64)
    d = np.array(p.mouse_dir, np.float64)
    d /= np.linalg.norm(d)
    t = pos.astype(np.float64) - o
    return np.linalg.norm(np.cross(t, d), axis=1)


def test_mouse_case_sort_and_density(gpu, oracle):
    p, z = load_mouse_case()
    assert p.flags & _abi.WC_FLAG_MOUSE_FORCE
    with fluid(p, z["state"]) as f:
        f.sort()
        f.density()
        srt = f.particles(_abi.WC_BUFFER_SORTED)
        perm, counts, offsets = f.permutation(), f.cell_counts(), f.cell_offsets()
    assert np.array_equal(perm, z["perm"])
    assert np.array_equal(counts, z["counts"]) and np.array_equal(offsets, z["offsets"])
    assert srt["position"].tobytes() == z["sorted"]["position"].tobytes()
    s64 = to64(srt)
    oracle.density(p, s64, counts, offsets)
    rel = np.abs(srt["density"] - s64["density"]) / np.abs(s64["density"])
    assert rel.max() <= 1e-5, f"{rel.max():.3e}"
    rel_ref = np.abs(srt["density"].astype(np.float64) - z["density"]["density"]) / np.abs(z["density"]["density"])
    assert rel_ref.max() <= 1e-5, f"{rel_ref.max():.3e}"


def force_pass(p, state, dt):
    with fluid(p, state) as f:
        f.sort()
        f.density()
        srt = f.particles(_abi.WC_BUFFER_SORTED)
        f.integrate(dt)
        return srt, f.particles(_abi.WC_BUFFER_STATE)


def test_mouse_force_pass_against_fp64(gpu, oracle):
    p, z = load_mouse_case()
    dt = float(z["dt"])
    srt, out = force_pass(p, z["state"], dt)
    s64 = to64(srt)
    o64 = oracle.update(p, s64, z["counts"], z["offsets"], dt)
    dv = np.abs(o64["velocity"] - s64["velocity"]).max()
    verr = np.abs(out["velocity"] - o64["velocity"]).max()
    assert verr <= 1e-4 * dv + 1e-7, f"velocity err {verr:.3e} vs max change {dv:.3e}"

    # the ray acts on the particles within h of it, and only on those
    q = p.copy()
    q.flags &= ~_abi.WC_FLAG_MOUSE_FORCE
    _, off = force_pass(q, z["state"], dt)
    moved = np.any(out["velocity"] != off["velocity"], axis=1)
    near = ray_distance(p, srt["position"]) <= float(p.kernel_radius) * (1 + 1e-5)
    assert moved.sum() > 0, "the mouse ray changed no velocity"
    assert not np.any(moved & ~near), "particles farther than h from the ray were pushed"


def test_mouse_ray_three_steps_track_the_reference(gpu, oracle):
    p, z = load_mouse_case()
    dt = np.float32(z["dt"])
    k = int(z["ksteps"])
    q = p.copy()
    q.flags |= _abi.WC_FLAG_TRACK_IDS
    st = z["state"]
    with fluid(q, st) as f:
        f.step(float(dt), k)
        out = f.particles()
        ids = f.particle_ids()
    ref = st.copy()
    ids32 = np.arange(st.shape[0], dtype=np.uint32)
    oracle.step(p, ref, dt, k, ids32)
    assert ref.tobytes() == z["stepped"].tobytes()  # the oracle is the reference's arithmetic here
    pg = np.empty((st.shape[0], 3))
    po = np.empty((st.shape[0], 3))
    pg[ids] = out["position"]
    po[ids32] = ref["position"]
    err = np.abs(pg - po).max()
    assert err <= 1e-5 * float(p.kernel_radius), f"{err:.3e}"
