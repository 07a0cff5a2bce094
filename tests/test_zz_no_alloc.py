"""wc_sort_cells_noalloc: the cell sort for callers that cannot allocate device memory while
they run (a frame loop where cudaMalloc would synchronise the GPU, a host application with a
fixed device memory budget). Its scratch is a fixed array inside the library, so the call only
takes the caller's buffers. Checked through the C ABI against the allocating path
(wc_fluid_sort) on two calls in a row, bit for bit: keys, permutation, cell table, sorted
positions. This file is collected last on purpose: it needs nothing from the other tests."""
import ctypes as C

import numpy as np
import pytest

from watercube_gb300 import _abi
from watercube_gb300.fluid import Fluid, dam_break_params, finalize, generate_dam_break, generate_reference_lattice, reference_params

pytestmark = pytest.mark.gpu


def allocating_sort(p, state):
    with Fluid.create("allocating", p) as f:
        f.setup(state)
        f.sort()
        srt = f.particles(_abi.WC_BUFFER_SORTED)
        return f.keys(), f.permutation(), f.cell_offsets(), f.cell_counts(), srt


def noalloc_sort(lib, torch, p, state):
    n = state.shape[0]
    R = int(p.grid_res)
    cells = R ** 3
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = state["position"]
    pos[:, 3] = state["density"]
    d_pos = torch.from_numpy(pos).cuda()
    d_keys = torch.zeros(n, dtype=torch.int32, device="cuda")
    d_perm = torch.zeros(n, dtype=torch.int32, device="cuda")
    d_start = torch.full((cells + 1,), -1, dtype=torch.int32, device="cuda")
    d_sorted = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.wc_sort_cells_noalloc(d_pos.data_ptr(), n, R, float(p.bin_size), d_keys.data_ptr(), d_perm.data_ptr(),
                                   d_start.data_ptr(), d_sorted.data_ptr(), None)
    assert rc == _abi.WC_OK, lib.wc_last_error().decode()
    torch.cuda.synchronize()
    start = d_start.cpu().numpy().view(np.uint32)
    return (d_keys.cpu().numpy().view(np.uint32), d_perm.cpu().numpy().view(np.uint32), start[:-1].copy(),
            np.diff(start).astype(np.uint32), d_sorted.cpu().numpy())


def test_noalloc_sort_matches_allocating_sort_twice(wclib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device for a GPU test")
    p1 = finalize(dam_break_params(16384))
    s1 = generate_dam_break(p1, 0)
    q = reference_params()
    q.num_particles = 20000
    p2 = finalize(q)
    s2 = generate_reference_lattice(p2, 4)
    s2 = s2[np.random.default_rng(1).permutation(s2.shape[0])]  # unsorted input
    for p, st in [(p1, s1), (p2, s2)]:  # two calls in a row share the scratch array
        keys, perm, offs, counts, srt = noalloc_sort(wclib, torch, p, st)
        e_keys, e_perm, e_offs, e_counts, e_srt = allocating_sort(p, st)
        assert np.array_equal(keys, e_keys)
        assert np.array_equal(perm, e_perm)
        assert np.array_equal(offs, e_offs)
        assert np.array_equal(counts, e_counts)
        assert srt[:, :3].tobytes() == np.ascontiguousarray(e_srt["position"]).tobytes()
        assert srt[:, 3].tobytes() == np.ascontiguousarray(e_srt["density"]).tobytes()


def test_noalloc_rejects_sizes_beyond_its_limit(wclib):
    rc = wclib.wc_sort_cells_noalloc(None, _abi.WC_NOALLOC_MAX_PARTICLES + 1, 16, 0.05, None, None, None, None, None)
    assert rc == _abi.WC_ERR_INVALID_ARG
    assert b"exceed" in wclib.wc_last_error()
    rc = wclib.wc_sort_cells_noalloc(None, 0, 65, 0.015, None, None, None, None, None)
    assert rc == _abi.WC_ERR_INVALID_ARG
    assert b"cells" in wclib.wc_last_error()


def test_noalloc_status_reports_device_errors(wclib):
    """The call only enqueues work; its device-side errors reach the caller through
    wc_sort_cells_noalloc_status, which allocates nothing either: a scan wait made to run out
    (the bounded-wait test hook) gives WC_ERR_TIMEOUT, a NaN position and a cell of more than
    65,536 particles give WC_ERR_NUMERIC, and a clean call afterwards reports WC_OK with tables
    equal to the allocating sort's."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device for a GPU test")
    p = finalize(dam_break_params(16384))  # 21^3 cells: three scan tiles
    st = generate_dam_break(p, 0)
    _abi.check(wclib.wc_debug_scan_stall(1, 64))
    try:
        noalloc_sort(wclib, torch, p, st)
        assert wclib.wc_sort_cells_noalloc_status(None) == _abi.WC_ERR_TIMEOUT
        assert b"invalid" in wclib.wc_last_error()
    finally:
        _abi.check(wclib.wc_debug_scan_stall(0, 0))

    bad = st.copy()
    bad["position"][[5, 700]] = np.nan
    noalloc_sort(wclib, torch, p, bad)
    assert wclib.wc_sort_cells_noalloc_status(None) == _abi.WC_ERR_NUMERIC
    assert b"non-finite" in wclib.wc_last_error()

    # a cell of 70,000 particles: beyond the 65,536 the stable rank is counted for, so its members
    # take arrival order; the permutation is still a permutation and the cell is reported
    q = reference_params()
    q.num_particles = 100000
    pc = finalize(q)
    crowd = generate_reference_lattice(pc, 2)
    rng = np.random.default_rng(3)
    b = float(pc.bin_size)
    crowd["position"][:70000] = 5 * b + rng.uniform(0.1 * b, 0.9 * b, size=(70000, 3))
    keys, perm, offs, counts, _ = noalloc_sort(wclib, torch, pc, crowd)
    assert wclib.wc_sort_cells_noalloc_status(None) == _abi.WC_ERR_NUMERIC
    assert b"65536" in wclib.wc_last_error()
    assert np.array_equal(np.sort(perm), np.arange(crowd.shape[0], dtype=np.uint32))
    big = int(np.argmax(counts))
    assert counts[big] >= 70000 and np.all(keys[perm[offs[big]:offs[big] + counts[big]]] == big)

    keys, perm, offs, counts, srt = noalloc_sort(wclib, torch, p, st)
    assert wclib.wc_sort_cells_noalloc_status(None) == _abi.WC_OK
    e_keys, e_perm, e_offs, e_counts, _ = allocating_sort(p, st)
    assert np.array_equal(perm, e_perm) and np.array_equal(offs, e_offs) and np.array_equal(keys, e_keys)
