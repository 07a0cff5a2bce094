"""Train the surrogate on trajectories of the batched solver and save its weights.

    python -m watercube_gb300.train_surrogate --steps 3000 --out watercube_gb300/weights/surrogate_l8.npz

Training data: `--scenes` random scenes (the batched workload's scene draw at smaller particle
counts, seed `--seed`) run by wc_batch for `--frames` steps at dt = 1e-3 with acceleration
recording on; every frame of every scene is a sample. The last quarter of the scenes is held
out. Adam on batches of 8 samples (lr `--lr`, then lr / 3 for the last 30% of the steps), input
noise sigma = 3e-4 on positions. Each training sample carries, with probability
1 - `--p-no-stale`, the SPH acceleration of the same scene k steps earlier (k uniform in
1 .. `--stale-k-max`) and its age as inputs, as the hybrid rollout gives them (such a sample
is residual: the network learns the change of the acceleration since then); otherwise none, as
the plain surrogate rollout runs. The report printed at the end (and stored in the .npz) gives
the held-out per-step acceleration error of the network without that input, of the network
given the SPH acceleration k steps old (hybrid_k), and of the method without the network: the
SPH acceleration of k steps earlier reused (stale_k), as a judged rollout with interval K does
for k = 1 .. K-1.
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

from .batch import batch_specs
from .surrogate import Surrogate, Trainer, record_samples

DEFAULT_WEIGHTS = Path(__file__).resolve().parent / "weights" / "surrogate_l8.npz"


def rel_error(pred: np.ndarray, target: np.ndarray) -> float:
    return float(np.linalg.norm(pred[:, :3] - target[:, :3]) / np.linalg.norm(target[:, :3]))


def stale_errors(samples, by, kmax: int) -> dict[int, float]:
    """Mean relative error of the SPH acceleration k steps old, k = 1 .. kmax."""
    out = {}
    for k in range(1, kmax + 1):
        errs = [rel_error(by[(x.scene, x.step - k)].target, x.target) for x in samples if (x.scene, x.step - k) in by]
        out[k] = float(np.mean(errs))
    return out


def network_error(trainer: Trainer, samples, stale_k: int = 0) -> float:
    """Mean relative error of the network's acceleration, given the SPH acceleration of stale_k
    steps earlier (0: none). The trainer's index must hold the earlier samples."""
    return float(np.mean([rel_error(trainer.predict(x, stale_k), x.target) for x in samples]))


def hybrid_errors(trainer: Trainer, samples, by, kmax: int) -> dict[int, float]:
    out = {}
    for k in range(1, kmax + 1):
        have = [x for x in samples if (x.scene, x.step - k) in by]
        out[k] = network_error(trainer, have, k)
    return out


def report(trainer: Trainer, samples, by, K_values=(4, 8)) -> dict:
    kmax = max(K_values) - 1
    trainer.index(list(by.values()))
    stale = stale_errors(samples, by, kmax)
    hybrid = hybrid_errors(trainer, samples, by, kmax)
    net = network_error(trainer, samples)
    out = {"network": net, "stale_k": stale, "hybrid_k": hybrid}
    for K in K_values:
        out[f"stale_mean_K{K}"] = float(np.mean([stale[k] for k in range(1, K)]))
        out[f"hybrid_mean_K{K}"] = float(np.mean([hybrid[k] for k in range(1, K)]))
    return out


def save_weights(path: Path, s: Surrogate, meta: dict) -> None:
    path.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(path, params=s.params(), layers=np.int32(s.config.layers),
                        velocity_scale=np.float32(s.config.velocity_scale),
                        accel_scale=np.float32(s.config.accel_scale), meta=json.dumps(meta))


def load_weights(path: Path = DEFAULT_WEIGHTS) -> Surrogate:
    """A Surrogate with the weights and configuration stored at `path`."""
    z = np.load(path)
    s = Surrogate(layers=int(z["layers"]), velocity_scale=float(z["velocity_scale"]),
                  accel_scale=float(z["accel_scale"]))
    s.set_params(z["params"])
    return s


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--scenes", type=int, default=16)
    ap.add_argument("--n-min", type=int, default=2048)
    ap.add_argument("--n-max", type=int, default=8192)
    ap.add_argument("--frames", type=int, default=64)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--layers", type=int, default=8)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--velocity-noise", type=float, default=0.0)
    ap.add_argument("--p-no-stale", type=float, default=0.2)
    ap.add_argument("--stale-k-max", type=int, default=7)
    ap.add_argument("--out", type=Path, default=DEFAULT_WEIGHTS)
    args = ap.parse_args(argv)

    t0 = time.time()
    specs = batch_specs(args.scenes, args.n_min, args.n_max, seed=args.seed)
    params, samples = record_samples(specs, steps=args.frames, dt=1e-3, every=1, start=0)
    by = {(x.scene, x.step): x for x in samples}
    held_from = args.scenes - max(1, args.scenes // 4)
    train = [x for x in samples if x.scene < held_from]
    held = [x for x in samples if x.scene >= held_from and x.step >= 8][::4]
    t_data = time.time() - t0

    s = Surrogate(layers=args.layers, seed=args.seed)
    tr = Trainer(s, params, seed=args.seed, velocity_noise=args.velocity_noise, p_no_stale=args.p_no_stale,
                 stale_k_max=args.stale_k_max)
    t1 = time.time()
    losses = []
    cut = int(args.steps * 0.7)
    losses += tr.train(train, steps=cut, lr=args.lr, batch=args.batch)
    losses += tr.train(train, steps=args.steps - cut, lr=args.lr / 3, batch=args.batch)
    t_train = time.time() - t1
    rep = report(tr, held, by)
    meta = {
        "scenes": args.scenes, "n_range": [args.n_min, args.n_max], "frames": args.frames, "seed": args.seed,
        "steps": args.steps, "lr": args.lr, "batch": args.batch, "velocity_noise": args.velocity_noise,
        "p_no_stale": args.p_no_stale, "stale_k_max": args.stale_k_max,
        "held_out_scenes": list(range(held_from, args.scenes)), "train_seconds": t_train,
        "data_seconds": t_data, "final_train_loss": float(np.mean(losses[-50:])), "held_out": rep,
    }
    save_weights(args.out, s, meta)
    tr.close()
    s.close()
    print(json.dumps(meta))
    return meta


if __name__ == "__main__":
    main()
