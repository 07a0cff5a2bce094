"""Batched scenes on the GPU: one launch per stage over all scenes gives each scene exactly the
result of simulating it alone; FP64 per-scene diagnostics against the oracle; the autotuner
leaves the simulation state untouched and launch geometry does not change results."""
import ctypes as C

import numpy as np
import pytest

from helpers import fluid
from oracle.oracle import to64
from watercube_gb300 import _abi
from watercube_gb300.fluid import finalize
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


@pytest.mark.parametrize("teams", [False, True])
def test_step_host_equals_the_three_calls(gpu, teams):
    """wc_batch_step_host(dt, in, out) = set_particles(in) + step(dt) + particles(), bit for bit,
    with the readback overlapping the force pass (lane passes) or following the step (teams);
    without `in` it steps the device state. 64 scenes: parts of many chunks across scenes."""
    specs = batch_specs(64, 600, 6000, seed=11)
    params = [scene_params(s) for s in specs]
    states = [scene_particles(s, p) for s, p in zip(specs, params)]
    with Batch(params, states) as a, Batch(params, states) as b:
        for x in (a, b):
            t = x.tuning()
            t.pass_variant = _abi.WC_PASSES_TEAM if teams else _abi.WC_PASSES_LANE
            x.set_tuning(t)
        n = a.num_particles
        cur = a.particles()
        out = np.empty(n, cur.dtype)
        for k in range(3):
            if k == 1:
                a.step_host(1e-3, None, out)
                b.step(1e-3, 1)
            else:
                a.step_host(1e-3, cur, out)
                b.set_particles(cur)
                b.step(1e-3, 1)
            assert out.tobytes() == b.particles().tobytes(), k
            cur = out.copy()
            cur["velocity"] *= 0.5


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
        assert t.pass_variant in (_abi.WC_PASSES_TEAM, _abi.WC_PASSES_LANE)
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


def test_every_tuned_geometry_keeps_the_densities(gpu, oracle):
    """Every geometry the tuner can pick: both cell edges (1.0 h and 1.25 h, which regrids every
    scene; the 27-cell search still covers every pair within h) and both neighbour-pass variants
    (a 32-lane team per cell, a lane per target). After one step each scene's densities (those of
    the step's density pass, carried in the state) stay within 1e-5 of the FP64 oracle on the
    scene's own 1.0 h grid, and the positions agree with the 1.0 h lane run to FP32 rounding (only
    the order of the neighbour sums changes). Blocks per SM change nothing at all
    (test_geometry_does_not_change_results)."""
    _, params, states = small_batch(4, seed=9)
    dt = 1e-3
    runs = {}
    for variant in (_abi.WC_PASSES_LANE, _abi.WC_PASSES_TEAM):
        for factor in (1.0, 1.25):
            with Batch(params, states) as b:
                t = b.tuning()
                t.cell_factor = factor
                t.pass_variant = variant
                b.set_tuning(t)
                assert b.tuning().cell_factor == factor and b.tuning().pass_variant == variant
                b.step(dt, 1)
                runs[variant, factor] = (b.particles(), b.ids(), b.offsets())
    base, base_ids, off = runs[_abi.WC_PASSES_LANE, 1.0]
    for s, (p, st) in enumerate(zip(params, states)):
        p = finalize(p)
        lo, hi = int(off[s]), int(off[s + 1])
        n = hi - lo
        o_sorted, _, o_perm, counts, offsets = oracle.sort(p, st)
        s64 = to64(o_sorted)
        oracle.density(p, s64, counts, offsets)
        rho64 = np.empty(n)
        rho64[o_perm] = s64["density"]
        ref = np.empty((n, 3))
        ref[base_ids[lo:hi] - lo] = base["position"][lo:hi]
        for key, (out, ids, off_k) in runs.items():
            assert int(off_k[s]) == lo and int(off_k[s + 1]) == hi
            rho = np.empty(n)
            rho[ids[lo:hi] - lo] = out["density"][lo:hi]
            rel = np.abs(rho - rho64) / np.abs(rho64)
            assert rel.max() <= 1e-5, (key, s, rel.max())
            pos = np.empty((n, 3))
            pos[ids[lo:hi] - lo] = out["position"][lo:hi]
            assert np.abs(pos - ref).max() <= 1e-5 * float(p.kernel_radius), (key, s)
