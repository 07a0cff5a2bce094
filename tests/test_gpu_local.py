"""The fast rollout on the GPU (csrc/wc_local.cu) against its FP64 restatement
(oracle/local_ref.py):

  * the judge step's feature output (SPH acceleration, its time derivative J with the
    neighbours' density and pressure rates, the density rate) and the network's 19 inputs,
    within the BF16 rounding of the inputs;
  * the fused tensor-core network (tcgen05, three layers in one kernel) against the FP64
    network with the same BF16 roundings;
  * the hand-written backward pass of a training step, per parameter block;
  * a rollout with tolerance 0 (every cycle reverted) equals plain SPH bit for bit, with and
    without the closing judge;
  * the Taylor extrapolation a + k dt J predicts the acceleration of every age better than the
    stale SPH acceleration, and its rollout drifts less from plain SPH;
  * trained on solver trajectories, the network (on top of the Taylor term) predicts the
    acceleration of every age better than the stale SPH acceleration on held-out samples.
"""
import numpy as np
import pytest

from helpers import case, fluid
from oracle import local_ref as L
from oracle.oracle import to64
from watercube_gb300 import _abi
from watercube_gb300.local import WC_LOCAL_NETWORK, WC_LOCAL_STALE, WC_LOCAL_TAYLOR, LocalNet, rollout

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


def test_judge_step_inputs_and_network_against_fp64(gpu, oracle):
    p, st = case("dam16k", _abi.WC_FLAG_TRACK_IDS)
    dt = 1e-3
    with fluid(p, st) as f, LocalNet(ages=3, seed=5) as net:
        f.step(dt, 30)
        before = f.particles()
        x, y = net.predict(f, dt)
        srt = f.particles(_abi.WC_BUFFER_SORTED)  # the judge step's sorted buffer, after its density pass
        assert f.particles().tobytes() == before.tobytes()  # predict does not advance the fluid
        w = net.params()
    cull = oracle.cull_threshold(float(p.kernel_radius))
    acc, jerk, rate = L.pair_sums(p, to64(srt), cull)
    ref = L.inputs(p, srt, acc, jerk, rate, dt)
    # BF16 inputs: 8 significant bits (relative rounding <= 2^-9 per element)
    for name, cols in [("acceleration", slice(0, 3)), ("J dt", slice(3, 6)), ("density rate", slice(6, 7)),
                       ("velocity", slice(7, 10)), ("density", slice(10, 11)), ("pressure", slice(11, 12)),
                       ("walls", slice(12, 18)), ("k", slice(18, 19))]:
        e = rel(x[:, cols], ref[:, cols])
        assert e <= 5e-3, f"{name}: relative L2 error {e:.2e}"
    assert np.all(x[:, 19:] == 0)
    # the fused network against the FP64 network on the same (BF16) inputs
    out = L.forward(w, x)[:, :9] * 10.0
    e = rel(y, out)
    assert e <= 1e-2, f"network outputs: relative L2 error {e:.2e}"


def recorded(net, cycles=2, held_out=False, seed=0, start=None):
    p, st = case("dam16k", _abi.WC_FLAG_TRACK_IDS)
    with fluid(p, st) as f:
        f.step(1e-3, start if start is not None else 20 + 10 * seed)
        net.record(f, 1e-3, cycles, held_out)


def test_training_gradients_against_fp64(gpu):
    with LocalNet(ages=3, seed=2, capacity=1 << 18) as net:
        recorded(net, cycles=1)
        assert net.num_samples() == 16384
        rng = np.random.default_rng(4)
        idx = rng.choice(16384, size=512, replace=False).astype(np.uint32)
        g, loss = net.gradients(idx)
        x, y = net.samples()
        w = net.params()
    ref_loss, ref = L.gradients(w, x[idx], y[idx], 9)
    assert loss == pytest.approx(ref_loss, rel=1e-2)
    for name, (a, b) in L.BLOCKS.items():
        e = rel(g[a:b], ref[a:b])
        assert e <= 3e-2, f"{name}: relative L2 error {e:.2e}"
    assert rel(g, ref) <= 1e-2


@pytest.mark.parametrize("nsteps", [13, 12])
def test_zero_tolerance_rollout_is_plain_sph(gpu, nsteps):
    """Tolerance 0: every judge reverts its cycle, whose steps are then recomputed by plain SPH
    from the state after the cycle's judge step; 12 steps end on skipped steps, which the
    closing judge reverts."""
    p, st = case("dam16k", _abi.WC_FLAG_TRACK_IDS)
    with fluid(p, st) as a, fluid(p, st) as b, LocalNet(ages=3, seed=1) as net:
        r = rollout(a, 1e-3, nsteps, ages=3, tolerance=0.0, net=net)
        b.step(1e-3, nsteps)
        assert r["steps"] == nsteps and r["surrogate_steps"] == 0 and r["sph_steps"] == nsteps
        assert r["reverted"] == r["judged"] > 0
        assert a.particles().tobytes() == b.particles().tobytes()
        assert np.array_equal(a.particle_ids(), b.particle_ids())
        assert a.step_count == b.step_count


def test_stale_rollout_is_judged_and_advances(gpu):
    p, st = case("dam16k", _abi.WC_FLAG_TRACK_IDS)
    with fluid(p, st) as f:
        r = rollout(f, 1e-3, 40, ages=3, tolerance=0.01, net=None)
        out = f.particles()
    assert r["steps"] == 40 and r["judged"] == 10 and r["sph_steps"] + r["surrogate_steps"] == 40
    assert 0.0 < r["mean_density_error"] < 0.01 and r["reverted"] == 0
    assert np.isfinite(out["position"]).all()
    assert (out["position"] >= p.wall_border).all() and (out["position"] <= p.size - p.wall_border).all()


def test_network_and_taylor_beat_stale_acceleration(gpu):
    """On the developed flow (from step 300 of the 16k dam break, when particles bounce off the
    floor every step), held-out samples: the Taylor term beats the stale acceleration at every
    age (the wall collisions it cannot foresee dominate the later ages) and the network trained
    on another stretch beats the stale acceleration too."""
    with LocalNet(ages=3, seed=3, capacity=1 << 21) as net:
        recorded(net, cycles=12, start=200)
        recorded(net, cycles=3, held_out=True, start=300)
        e_net0, e_stale, e_taylor = net.evaluate(held_out=True)
        loss = net.train(600, rows=4096, lr=2e-3)
        e_net, _, _ = net.evaluate(held_out=True)
    print("loss", loss[:10].mean(), "->", loss[-50:].mean())
    print("held-out relative error, network:", e_net, "(untrained", e_net0, ") stale:", e_stale, "taylor:", e_taylor)
    assert loss[-50:].mean() < 0.9 * loss[:10].mean()
    assert np.all(e_taylor < e_stale) and e_taylor[0] < 0.8 * e_stale[0], (e_taylor, e_stale)
    assert np.all(e_net < e_stale), (e_net, e_stale)


def test_taylor_rollout_drifts_less_than_stale(gpu):
    """40 steps in cycles of K = 4 on the 16k dam break: RMS position distance from plain SPH
    (by particle id) of the Taylor mode below that of the stale mode; both judged, none
    reverted, the density error within the tolerance."""
    p, st = case("dam16k", _abi.WC_FLAG_TRACK_IDS)
    dt = 1e-3
    with fluid(p, st) as f:
        f.step(dt, 40)
        plain = f.particles()["position"][np.argsort(f.particle_ids())]
    drift = {}
    for mode in (WC_LOCAL_STALE, WC_LOCAL_TAYLOR):
        with fluid(p, st) as f:
            r = rollout(f, dt, 40, ages=3, tolerance=0.01, mode=mode)
            pos = f.particles()["position"][np.argsort(f.particle_ids())]
        assert r["judged"] == 10 and r["reverted"] == 0 and r["mean_density_error"] < 0.01, (mode, r)
        drift[mode] = float(np.sqrt(np.mean(np.sum((pos - plain) ** 2, axis=1)))) / float(p.kernel_radius)
    print("RMS drift from plain SPH (h):", drift)
    assert drift[WC_LOCAL_TAYLOR] < drift[WC_LOCAL_STALE], drift


def test_network_mode_needs_a_network(gpu):
    p, st = case("dam16k", _abi.WC_FLAG_TRACK_IDS)
    with fluid(p, st) as f:
        with pytest.raises(_abi.WatercubeError):
            rollout(f, 1e-3, 8, ages=3, mode=WC_LOCAL_NETWORK)


def test_rollout_command_runs_each_mode(gpu, capsys):
    """python -m watercube_gb300.local: a short rollout of a small dam break in every mode."""
    import json

    from watercube_gb300.local import main

    for mode in ("stale", "taylor", "network"):
        assert main(["--particles", "16384", "--steps", "8", "--mode", mode]) == 0
        r = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
        assert r["mode"] == mode and r["steps"] == 8 and r["judged"] >= 1 and r["mean_density_error"] < 0.01
