"""What the trained network gains over the method without it.

The method without the network reuses the last SPH acceleration for the skipped steps of a
judged rollout (WC_ROLLOUT_STALE): with an SPH judge every K steps, a skipped step's
acceleration is 1 .. K-1 steps old. The network predicts the current step's acceleration from
the current state instead (WC_ROLLOUT_SURROGATE), or the change since that stale acceleration
from the current state, the stale acceleration and its age (WC_ROLLOUT_HYBRID). On scenes it
was not trained on (a different scene draw than the committed weights' training set):
  - the network alone beats the stale acceleration's mean per-step error at K = 8;
  - the hybrid beats the stale acceleration's per-step error at every age 1 .. 7, and so at
    K = 4 and K = 8;
  - the rollouts of every mode stay finite and inside the box, and the hybrid rollout ends
    closer to plain SPH than the plain surrogate's.
Against the stale method the closed-loop trajectory error is reported, not asserted: the
network's per-step error, though smaller, persists from step to step and accumulates in the
positions, while the stale acceleration's larger error mostly averages out, and both network
modes drift further from plain SPH than the stale method.
"""
import numpy as np
import pytest

from watercube_gb300 import _abi
from watercube_gb300.batch import batch_specs
from watercube_gb300.fluid import Fluid
from watercube_gb300.surrogate import (
    WC_ROLLOUT_HYBRID,
    WC_ROLLOUT_SPH,
    WC_ROLLOUT_STALE,
    WC_ROLLOUT_SURROGATE,
    Trainer,
    record_samples,
    rollout,
)
from watercube_gb300.train_surrogate import DEFAULT_WEIGHTS, hybrid_errors, load_weights, rel_error, stale_errors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained(gpu):
    if not DEFAULT_WEIGHTS.is_file():
        pytest.fail(f"trained weights missing: {DEFAULT_WEIGHTS}")
    s = load_weights()
    yield s
    s.close()


@pytest.fixture(scope="module")
def held_out(gpu):
    # the config-2 scene draw (4,096-65,536 particles) the committed weights were trained on,
    # with another seed (they were trained on seed 1)
    specs = batch_specs(6, 4096, 65536, seed=7)
    params, samples = record_samples(specs, steps=24, dt=1e-3, every=1, start=0)
    by = {(x.scene, x.step): x for x in samples}
    return params, samples, by


def test_network_beats_stale_acceleration_per_step(trained, held_out):
    params, samples, by = held_out
    evals = [x for x in samples if x.step >= 8][::3]
    t = Trainer(trained, params)
    try:
        t.index(samples)
        net = float(np.mean([rel_error(t.predict(x), x.target) for x in evals]))
        hyb = hybrid_errors(t, evals, by, 7)
    finally:
        t.close()
    stale = stale_errors(evals, by, 7)
    k4 = float(np.mean([stale[k] for k in range(1, 4)]))
    k8 = float(np.mean([stale[k] for k in range(1, 8)]))
    h4 = float(np.mean([hyb[k] for k in range(1, 4)]))
    h8 = float(np.mean([hyb[k] for k in range(1, 8)]))
    msg = (f"network {net:.4f}, stale K=4 {k4:.4f}, stale K=8 {k8:.4f}, hybrid K=4 {h4:.4f}, hybrid K=8 {h8:.4f}, "
           f"stale by age {stale}, hybrid by age {hyb}")
    print(msg)
    assert net < k8, msg
    assert net < 0.5, msg  # far better than gravity alone (about 0.75 on these scenes)
    assert all(hyb[k] < stale[k] for k in range(1, 8)), msg
    assert h4 < k4 and h8 < k8, msg


def test_rollouts_against_plain_sph(trained, held_out):
    params, samples, by = held_out
    report = []
    for sc in (0, 3):
        x = by[(sc, 8)]
        p = params[sc].copy()
        p.flags |= _abi.WC_FLAG_TRACK_IDS
        res = {}
        for mode, name in ((WC_ROLLOUT_SPH, "plain"), (WC_ROLLOUT_SURROGATE, "surrogate"), (WC_ROLLOUT_STALE, "stale"),
                           (WC_ROLLOUT_HYBRID, "hybrid")):
            with Fluid("g", p) as f:
                f.setup(x.state)
                st = rollout(f, x.dt, 16, 4, 1e9, mode, trained, x.hist)
                out, ids = f.particles(), f.particle_ids()
            pos = np.empty((len(ids), 3))
            pos[ids] = out["position"]
            assert np.all(np.isfinite(pos)) and np.all((pos >= 0) & (pos <= p.size))
            assert st["diag_end"][0] == st["diag_start"][0]
            res[name] = pos
        h = p.kernel_radius
        report.append({k: float(np.sqrt(((res[k] - res["plain"]) ** 2).sum(1).mean()) / h)
                       for k in ("surrogate", "stale", "hybrid")})
    print(report)
    # the comparison with the stale method is reported, not asserted (see the module docstring)
    assert all(np.isfinite(r["stale"]) for r in report), report
    assert all(r["hybrid"] < r["surrogate"] for r in report), report
