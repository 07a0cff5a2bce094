"""Binning and sorting on the GPU, bit-exact against the reference stage logic (oracle, which
tests/test_oracle_golden.py pins to the reference's shaders): cell keys, the sorted
permutation, cell count/offset tables and the sorted particle buffer."""
import numpy as np
import pytest

from helpers import case, evolved, fluid
from watercube_gb300 import _abi

pytestmark = pytest.mark.gpu


def check_sort(oracle, p, state):
    with fluid(p, state) as f:
        f.sort()
        keys, perm = f.keys(), f.permutation()
        counts, offsets = f.cell_counts(), f.cell_offsets()
        srt = f.particles(_abi.WC_BUFFER_SORTED)
        f.synchronize()
    o_sorted, o_keys, o_perm, o_counts, o_offsets = oracle.sort(p, state)
    assert np.array_equal(keys, o_keys)
    assert np.array_equal(perm, o_perm)
    assert np.array_equal(counts, o_counts)
    assert np.array_equal(offsets, o_offsets)
    assert srt.tobytes() == o_sorted.tobytes()


@pytest.mark.parametrize("name", ["dam16k", "refdefaults", "dam1m"])
def test_sort_initial_state(gpu, oracle, name):
    p, st = case(name)
    check_sort(oracle, p, st)


@pytest.mark.parametrize("name,steps,dt", [("dam16k", 40, 1e-3), ("refdefaults", 30, 2e-4), ("dam1m", 8, 2.5e-4),
                                           ("dam1m", 1000, 2.5e-4)])
def test_sort_evolved_state(gpu, oracle, name, steps, dt):
    """Input already in last step's sorted order with particles migrating between cells."""
    p, st = evolved(name, steps, dt)
    check_sort(oracle, p, st)


def test_sort_shuffled_and_outside_box(gpu, oracle):
    p, st = case("dam16k")
    rng = np.random.default_rng(5)
    st = st[rng.permutation(st.shape[0])]
    st["position"][::7] = rng.uniform(-0.2, 1.2, size=st["position"][::7].shape).astype(np.float32)
    check_sort(oracle, p, st)


def test_sort_all_in_one_cell(gpu, oracle):
    p, st = case("dam16k")
    rng = np.random.default_rng(6)
    b = float(p.bin_size)
    st["position"] = (0.5 + rng.uniform(0.05 * b, 0.95 * b, size=(st.shape[0], 3))).astype(np.float32)
    check_sort(oracle, p, st)


def test_sort_cell_faces_and_box_faces(gpu, oracle):
    p, st = case("dam16k")
    b = np.float32(p.bin_size)
    k = np.arange(st.shape[0]) % p.grid_res
    st["position"][:, 0] = k.astype(np.float32) * b  # exactly on cell faces
    st["position"][::3, 1] = np.float32(p.size)  # exactly on the top face
    st["position"][1::3, 2] = 0.0
    check_sort(oracle, p, st)


def test_sort_repeated_is_stable(gpu, oracle):
    """Sorting an already sorted buffer is the identity permutation."""
    p, st = case("dam16k")
    o_sorted, *_ = oracle.sort(p, st)
    with fluid(p, o_sorted) as f:
        f.sort()
        assert np.array_equal(f.permutation(), np.arange(st.shape[0], dtype=np.uint32))
