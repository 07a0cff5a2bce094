"""Batched workload, host side: the scene draw, scene parameters, initial states, and the
multi-process split of a batch (round-robin scenes, no data exchange) on gloo ranks."""
import math
import os
import sys

import numpy as np
import pytest

from watercube_gb300 import batch_specs, scene_params, scene_particles, shard_scenes


def test_specs_follow_the_workload_rule(wclib):
    specs = batch_specs(512, 4096, 65536, seed=0)
    assert batch_specs(512, 4096, 65536, seed=0)[17].num_particles == specs[17].num_particles
    n = np.array([s.num_particles for s in specs])
    assert n.min() >= 4096 and n.max() <= 65536
    # log-uniform: the median count is near the geometric mean of the bounds (16,384)
    assert 11000 < np.median(n) < 24000
    assert 9e6 < n.sum() < 14e6
    for s in specs:
        sides = [s.block_max[a] - s.block_min[a] for a in range(3)]
        assert all(0.2 - 1e-6 <= x <= 0.7 + 1e-6 for x in sides)
        assert s.block_min[1] == 0.0 and all(0.0 <= s.block_min[a] and s.block_max[a] <= 1.0 + 1e-6 for a in (0, 2))
        assert 2.0 <= s.stiffness <= 6.0 and s.velocity_sigma == 0.5


def test_scene_params_and_particles(wclib):
    s = batch_specs(3, 4096, 65536, seed=2)[1]
    p = scene_params(s)
    vol = np.prod([s.block_max[a] - s.block_min[a] for a in range(3)])
    sp = (vol / s.num_particles) ** (1 / 3)
    assert math.isclose(p.kernel_radius, 2 * sp, rel_tol=1e-5)
    assert math.isclose(p.particle_mass, 1000 * sp**3, rel_tol=1e-5)
    assert p.grid_res == int(math.floor(1.0 / p.kernel_radius)) and p.bin_size >= p.kernel_radius
    assert math.isclose(p.stiffness, s.stiffness) and p.rest_density == 1000.0
    st = scene_particles(s, p)
    assert st.shape == (s.num_particles,)
    pos = st["position"]
    assert (pos[:, 0] >= s.block_min[0] - 0.01 * p.kernel_radius).all()
    assert (pos[:, 2] <= s.block_max[2] + p.kernel_radius).all()
    assert abs(st["velocity"].std() - 0.5) < 0.02


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_shards_cover_every_scene_once(world):
    parts = [shard_scenes(512, r, world) for r in range(world)]
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(512))
    assert max(map(len, parts)) - min(map(len, parts)) <= 1


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist

    import bench

    r, w, local, reduce_max, barrier = bench.dist_setup(world)
    assert (r, w, local) == (rank, world, rank)
    specs = batch_specs(64, 1000, 8000, seed=5)
    mine = {i: specs[i].num_particles for i in shard_scenes(64, r, w)}
    gathered = [None] * w
    dist.all_gather_object(gathered, mine)
    merged = {}
    for g in gathered:
        merged.update(g)
    slowest = reduce_max(float(rank + 1))
    barrier()
    if r == 0:
        ok = merged == {i: s.num_particles for i, s in enumerate(specs)} and slowest == float(w)
        open(os.path.join(out_dir, "result"), "w").write("ok" if ok else "bad")
    dist.destroy_process_group()


def test_sharded_batch_on_two_gloo_ranks(tmp_path, wclib):
    torch = pytest.importorskip("torch")
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    if torch.cuda.is_available():
        pytest.skip("gloo path is exercised on CPU-only hosts")
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    assert (tmp_path / "result").read_text() == "ok"
