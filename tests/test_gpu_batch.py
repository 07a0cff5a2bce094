"""Batched scenes on the GPU: one launch per stage over all scenes gives each scene exactly the
result of simulating it alone; FP64 per-scene diagnostics against the oracle; the autotuner
leaves the simulation state untouched and launch geometry does not change results."""
import ctypes as C

import numpy as np
import pytest

from helpers import fluid
from watercube_gb300 import _abi
from watercube_gb300.batch import Batch, batch_specs, scene_params, scene_particles

pytestmark = pytest.mark.gpu


def small_batch(num=4, seed=3):
    specs = batch_specs(num, 600, 6000, seed=seed)
    params = [scene_params(s) for s in specs]
    states = [scene_particles(s, p) for s, p in zip(specs, params)]
    return specs, params, states


def test_batch_equals_scenes_run_alone(gpu):
    _, params, states = small_batch()
    with Batch(params, states) as b:
        b.step(1e-3, 6)
        out = b.particles()
        for s, (p, st) in enumerate(zip(params, states)):
            with fluid(p, st) as f:
                f.step(1e-3, 6)
                alone = f.particles()
            assert b.scene(s, out).tobytes() == alone.tobytes(), f"scene {s}"


def test_batch_diagnostics_fp64(gpu, oracle):
    _, params, states = small_batch(5, seed=8)
    with Batch(params, states) as b:
        b.step(1e-3, 3)
        diag = b.diagnostics()
        out = b.particles()
        for s, p in enumerate(params):
            d = oracle.diagnostics(p, b.scene(s, out))
            ref = np.array([d["mass"], *d["momentum"], d["kinetic"], d["potential"]])
            scale = np.maximum(np.abs(ref), 1e-12 * np.abs(ref).max())
            assert (np.abs(diag[s] - ref) <= 1e-9 * scale + 1e-15).all(), (s, diag[s], ref)


def test_geometry_does_not_change_results(gpu):
    _, params, states = small_batch(3, seed=4)
    with Batch(params, states) as a, Batch(params, states) as b:
        t = b.tuning()
        t.density_blocks_per_sm = 1
        t.force_blocks_per_sm = 1
        t.stream_blocks_per_sm = 2
        b.set_tuning(t)
        a.step(1e-3, 4)
        b.step(1e-3, 4)
        assert a.particles().tobytes() == b.particles().tobytes()


def test_tuner_keeps_state_and_picks_valid_geometry(gpu):
    _, params, states = small_batch(6, seed=6)
    with Batch(params, states) as b:
        before = b.particles()
        t = b.tune(1e-3)
        assert b.particles().tobytes() == before.tobytes()
        assert t.trials >= 5 and t.step_ms > 0
        assert t.density_blocks_per_sm >= 1 and t.force_blocks_per_sm >= 1 and t.cell_factor in (1.0, 1.25)
        m0 = b.diagnostics()[:, 0].copy()
        b.step(1e-3, 3)
        after = b.particles()
        assert np.isfinite(after["position"]).all()
        assert np.array_equal(b.diagnostics()[:, 0], m0)


def test_workload_sample_runs(gpu):
    specs = batch_specs(512, 4096, 65536, seed=0)[:48]
    with Batch.from_specs(specs) as b:
        b.step(1e-3, 10)
        out = b.particles()
        assert np.isfinite(out["position"]).all()
        assert (out["position"] >= 0.0).all() and (out["position"] <= 1.0).all()
        off = b.offsets()
        assert off[-1] == out.shape[0] == sum(s.num_particles for s in specs)
