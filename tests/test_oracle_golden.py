"""The oracle against the reference: committed golden fixtures (made from the reference's own
shaders by tests/golden/make_golden.py) and, where the reference checkout is present, a live
comparison with the shaders compiled as C++. Bit-exact on every stage."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import PARTICLE64_DTYPE, to64
from watercube_gb300 import _abi
from watercube_gb300.fluid import dam_break_params, finalize, generate_reference_lattice, reference_params

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load_case(name):
    z = np.load(GOLDEN / f"{name}.npz")
    p = _abi.Params()
    raw = z["params"].tobytes()
    C.memmove(C.addressof(p), raw, C.sizeof(p))
    return p, z


def test_fixtures_present():
    assert {"ref_defaults_n1500", "dam_refphysics_n2000", "mouse_ray_n800"} <= set(CASES)


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_fixture(oracle, name):
    p, z = load_case(name)
    state = z["state"]
    sorted_, keys, perm, counts, offsets = oracle.sort(p, state)
    assert sorted_.tobytes() == z["sorted"].tobytes()
    assert np.array_equal(perm, z["perm"])
    assert np.array_equal(counts, z["counts"])
    assert np.array_equal(offsets, z["offsets"])
    dens = sorted_.copy()
    oracle.density(p, dens, counts, offsets, threads=1)
    assert dens.tobytes() == z["density"].tobytes()
    upd = oracle.update(p, dens, counts, offsets, float(z["dt"]), threads=1)
    assert upd.tobytes() == z["update"].tobytes()
    stepped = state.copy()
    oracle.step(p, stepped, float(z["dt"]), int(z["ksteps"]), threads=1)
    assert stepped.tobytes() == z["stepped"].tobytes()


@pytest.mark.parametrize("name", CASES)
def test_oracle_threads_do_not_change_results(oracle, name):
    p, z = load_case(name)
    a = z["state"].copy()
    b = z["state"].copy()
    oracle.step(p, a, float(z["dt"]), 2, threads=1)
    oracle.step(p, b, float(z["dt"]), 2, threads=4)
    assert a.tobytes() == b.tobytes()


def test_mouse_case_exercises_mouse_force(oracle):
    p, z = load_case("mouse_ray_n800")
    q = p.copy()
    q.flags &= ~_abi.WC_FLAG_MOUSE_FORCE
    a = z["state"].copy()
    oracle.step(q, a, float(z["dt"]), int(z["ksteps"]), threads=1)
    assert a.tobytes() != z["stepped"].tobytes()


def test_live_reference_matches_oracle(oracle, reflib):
    """Live: reference shaders vs oracle on fresh inputs (only where the reference exists)."""
    for n, seed in [(3000, 11), (257, 5)]:
        p = reference_params()
        p.num_particles = n
        p = finalize(p)
        st = generate_reference_lattice(p, seed)
        a = st.copy()
        b = st.copy()
        oracle.step(p, a, 2e-4, 6, threads=1)
        reflib.step(p, b, 2e-4, 6)
        assert a.tobytes() == b.tobytes()
    p = dam_break_params(4096)
    p.eos = _abi.WC_EOS_DESBRUN_CUBIC
    p.flags = _abi.WC_FLAGS_REFERENCE
    p.wall_damping = 0.3  # update.comp:202-203 hard-code damping and border
    p = finalize(p)
    from watercube_gb300.fluid import generate_dam_break

    st = generate_dam_break(p, 1)
    a, b = st.copy(), st.copy()
    oracle.step(p, a, 1e-3, 5, threads=1)
    reflib.step(p, b, 1e-3, 5)
    assert a.tobytes() == b.tobytes()


@pytest.mark.parametrize("name", CASES)
def test_fp64_oracle_close_to_fp32(oracle, name):
    """The FP64 path evaluates the same equations: one density pass agrees to float rounding."""
    p, z = load_case(name)
    s32, _, _, counts, offsets = oracle.sort(p, z["state"])
    s64 = to64(s32)
    oracle.density(p, s32, counts, offsets)
    nc64 = oracle.density(p, s64, counts, offsets)
    assert s64.dtype == PARTICLE64_DTYPE
    rel = np.abs(s32["density"] - s64["density"]) / np.maximum(np.abs(s64["density"]), 1e-30)
    assert rel.max() < 2e-5
