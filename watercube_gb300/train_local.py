"""Train the learned fast rollout's per-particle network on solver trajectories and save it.

    python -m watercube_gb300.train_local [--ages 3] [--steps 20000] [--lr 1e-4] [--out watercube_gb300/weights/local_k4.npz]

Training data: scenes of the batched workload's draw (512 scenes, 4,096-65,536 particles each,
seed `--seed`): `--train-scenes` of them run together by wc_batch at dt = 1e-3, `--warmup` plain
steps, then `--cycles` cycles of (judge step, `ages` plain steps), each cycle giving one sample per
particle (the judge step's inputs; the residuals a(t + k) - a(t) - k dt J of the SPH
accelerations of the next `ages` steps, matched by particle id). The dam break the fast rollout is measured on (a smaller size with the same
particles per cell, its own dt) adds its own trajectory, `--dam-cycles` cycles, and so does the
full-size dam break (`--big-dam-n` particles, dt 2.5e-4, `--big-dam-cycles` cycles) started
from another jitter of the lattice (`--dam-seed`; the rollout is measured from seed 0). Held out:
other scenes of the draw and later stretches of the dam breaks. Adam on minibatches of `--rows`
samples (about eight scenes' particles), lr `--lr`, `--steps` steps. The report (printed, and
stored in the .npz) gives the held-out relative error of the acceleration at each age in the
three modes (the network on top of the Taylor term a + k dt J; the stale SPH acceleration; the
Taylor term alone), over all held-out samples and over a stretch of the full-size dam break from
a third jitter (`--dam-seed` + 1).
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

from . import _abi
from .batch import Batch, batch_specs, scene_params, scene_particles
from .fluid import Fluid, dam_break_params, finalize, generate_dam_break
from .local import DEFAULT_WEIGHTS, LocalNet, save_weights


def record_batch(net: LocalNet, specs, dt: float, warmup: int, cycles: int, held_out: bool) -> int:
    params = [scene_params(s) for s in specs]
    states = [scene_particles(s, p) for s, p in zip(specs, params)]
    with Batch(params, states) as b:
        b.step(dt, warmup)
        net.record(b, dt, cycles, held_out)
        return b.num_particles


def record_dam(net: LocalNet, n: int, warmup: int, cycles: int, held_out: bool, seed: int = 0) -> float:
    p = dam_break_params(n)
    p.flags |= _abi.WC_FLAG_TRACK_IDS
    p = finalize(p)
    dt = 2.5e-4 * (1048576.0 / n) ** (1.0 / 3.0)  # the same dt / h as the 1,048,576-particle workload
    with Fluid.create("train", p) as f:
        f.setup(generate_dam_break(p, seed))
        f.step(dt, warmup)
        net.record(f, dt, cycles, held_out)
    return dt


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--ages", type=int, default=3, help="skipped steps per cycle (K - 1)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--train-scenes", type=int, default=48)
    ap.add_argument("--held-scenes", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=40)
    ap.add_argument("--cycles", type=int, default=12)
    ap.add_argument("--dam-n", type=int, default=131072)
    ap.add_argument("--dam-cycles", type=int, default=24)
    ap.add_argument("--big-dam-n", type=int, default=1048576, help="0: no full-size dam break")
    ap.add_argument("--big-dam-cycles", type=int, default=6)
    ap.add_argument("--dam-seed", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--rows", type=int, default=176000)
    ap.add_argument("--lr", type=float, default=1e-4)
    ap.add_argument("--out", type=Path, default=DEFAULT_WEIGHTS)
    a = ap.parse_args(argv)
    _abi.check(_abi.lib().wc_set_device(0), "select device")
    t0 = time.perf_counter()
    specs = batch_specs(512, 4096, 65536, seed=a.seed)
    rng = np.random.default_rng(a.seed)
    order = rng.permutation(len(specs))
    train_specs = [specs[i] for i in order[:a.train_scenes]]
    held_specs = [specs[i] for i in order[a.train_scenes:a.train_scenes + a.held_scenes]]
    rows = (a.rows // 8) * 8
    net = LocalNet(ages=a.ages, seed=1 + a.seed, capacity=1 << 25)
    n_train = record_batch(net, train_specs, 1e-3, a.warmup, a.cycles, False)
    n_held = record_batch(net, held_specs, 1e-3, a.warmup, max(2, a.cycles // 4), True)
    dam_dt = record_dam(net, a.dam_n, a.warmup, a.dam_cycles, False, a.dam_seed)
    record_dam(net, a.dam_n, a.warmup + (a.ages + 1) * a.dam_cycles + 40, max(2, a.dam_cycles // 4), True, a.dam_seed)
    if a.big_dam_n:
        record_dam(net, a.big_dam_n, a.warmup, a.big_dam_cycles, False, a.dam_seed)
        record_dam(net, a.big_dam_n, a.warmup + (a.ages + 1) * a.big_dam_cycles + 80, 2, True, a.dam_seed)
    t_rec = time.perf_counter() - t0
    e_net0, e_stale, e_taylor = net.evaluate(held_out=True)
    t1 = time.perf_counter()
    loss = net.train(a.steps, rows=rows, lr=a.lr)
    t_train = time.perf_counter() - t1
    e_net, e_stale, e_taylor = net.evaluate(held_out=True)
    e_train, e_stale_train, e_taylor_train = net.evaluate(held_out=False)
    e_big, e_big_stale, e_big_taylor = [], [], []
    if a.big_dam_n:
        net.clear_samples()
        record_dam(net, a.big_dam_n, a.warmup + 200, 2, True, a.dam_seed + 1)
        e_big, e_big_stale, e_big_taylor = net.evaluate(held_out=True)
    report = {
        "samples_train": net.num_samples(False),
        "samples_held_out": net.num_samples(True),
        "train_scenes": a.train_scenes, "held_scenes": a.held_scenes, "batch_particles_train": n_train,
        "batch_particles_held": n_held, "dam_particles": a.dam_n, "dam_dt": dam_dt, "cycles": a.cycles,
        "steps": a.steps, "rows": rows, "lr": a.lr, "record_s": t_rec, "train_s": t_train,
        "loss_first": float(loss[:10].mean()), "loss_last": float(loss[-100:].mean()),
        "loss_curve": [float(loss[i:i + max(1, a.steps // 20)].mean()) for i in range(0, a.steps, max(1, a.steps // 20))],
        "held_out_error_network": [float(x) for x in e_net],
        "held_out_error_untrained": [float(x) for x in e_net0],
        "held_out_error_stale": [float(x) for x in e_stale],
        "held_out_error_taylor": [float(x) for x in e_taylor],
        "train_error_network": [float(x) for x in e_train],
        "train_error_stale": [float(x) for x in e_stale_train],
        "train_error_taylor": [float(x) for x in e_taylor_train],
        "big_dam_n": a.big_dam_n, "big_dam_cycles": a.big_dam_cycles, "dam_seed": a.dam_seed, "ages": a.ages,
        "big_dam_error_network": [float(x) for x in e_big],
        "big_dam_error_stale": [float(x) for x in e_big_stale],
        "big_dam_error_taylor": [float(x) for x in e_big_taylor],
    }
    save_weights(net, a.out, report=json.dumps(report))
    print(json.dumps(report, indent=1))
    net.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
