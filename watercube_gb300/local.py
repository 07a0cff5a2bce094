"""The fast rollout over the C ABI (wc_local_*): every K-th step is plain SPH (the judge) and
also computes each particle's density and pressure rates and the time derivative J of its
acceleration; the K - 1 steps after it run without neighbour passes on an extrapolated
acceleration, by mode: the judge's acceleration held (WC_LOCAL_STALE), a + k dt J
(WC_LOCAL_TAYLOR), or a + k dt J plus a per-particle network's residual (WC_LOCAL_NETWORK). The
next judge step checks the cycle by the carried density. No counterpart in the reference, which
only runs plain SPH.

The network, its fused tensor-core inference, training and the rollout are in
csrc/wc_local.cu; this module moves host arrays and drives training.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _abi as A
from ._abi import WC_LOCAL_NETWORK, WC_LOCAL_STALE, WC_LOCAL_TAYLOR, LocalConfig, RolloutStats, check, lib
from .batch import Batch
from .fluid import Fluid

IN, HIDDEN, OUT = 32, 64, 16
YW = 20  # a sample's target row: residuals of 5 ages, unused, (1 ms / dt)^2, dt J / a_s
INPUT_NAMES = ["a_x", "a_y", "a_z", "jdt_x", "jdt_y", "jdt_z", "rhodot", "v_x", "v_y", "v_z", "rho_rel", "p_rel",
               "wall_x0", "wall_x1", "wall_y0", "wall_y1", "wall_z0", "wall_z1", "k_rel"]
DEFAULT_WEIGHTS = Path(__file__).resolve().parent / "weights" / "local_k4.npz"


def default_config(**overrides) -> LocalConfig:
    c = LocalConfig()
    lib().wc_local_config_default(C.byref(c))
    for k, v in overrides.items():
        setattr(c, k, v)
    return c


class LocalNet:
    """One per-particle network: FP32 master weights, Adam state, sample sets and scratch."""

    def __init__(self, config: LocalConfig | None = None, **overrides):
        cfg = config if config is not None else default_config(**overrides)
        h = C.c_void_p()
        check(lib().wc_local_create(C.byref(cfg), C.byref(h)), "wc_local_create")
        self._h = h
        self.config = cfg
        self.ages = int(cfg.ages)
        self.num_params = int(lib().wc_local_num_params(h))

    # ---- parameters ---------------------------------------------------------------------------
    def params(self) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        check(lib().wc_local_get_params(self._h, A._ptr(out), self.num_params), "wc_local_get_params")
        return out

    def set_params(self, w: np.ndarray) -> None:
        w = np.ascontiguousarray(w, dtype=np.float32)
        check(lib().wc_local_set_params(self._h, A._ptr(w), w.size), "wc_local_set_params")

    # ---- samples and training -------------------------------------------------------------------
    def record(self, target, dt: float, cycles: int, held_out: bool = False) -> None:
        if isinstance(target, Batch):
            check(lib().wc_local_record_batch(self._h, target._h, float(dt), int(cycles), int(held_out)),
                  "wc_local_record_batch")
        else:
            check(lib().wc_local_record_fluid(self._h, target._require(), float(dt), int(cycles), int(held_out)),
                  "wc_local_record_fluid")

    def num_samples(self, held_out: bool = False) -> int:
        return int(lib().wc_local_num_samples(self._h, int(held_out)))

    def clear_samples(self) -> None:
        check(lib().wc_local_clear_samples(self._h), "wc_local_clear_samples")

    def samples(self, held_out: bool = False, first: int = 0, count: int | None = None):
        if count is None:
            count = self.num_samples(held_out) - first
        x = np.zeros((count, IN), np.float32)
        y = np.zeros((count, YW), np.float32)
        check(lib().wc_local_get_samples(self._h, int(held_out), first, count, A._ptr(x), A._ptr(y)),
              "wc_local_get_samples")
        return x, y

    def train(self, steps: int, rows: int = 8192, lr: float = 1e-3) -> np.ndarray:
        loss = np.zeros(steps, np.float32)
        check(lib().wc_local_train(self._h, int(steps), int(rows), float(lr), A._ptr(loss)), "wc_local_train")
        return loss

    def gradients(self, rows_idx: np.ndarray):
        idx = np.ascontiguousarray(rows_idx, dtype=np.uint32)
        g = np.zeros(self.num_params, np.float32)
        loss = np.zeros(1, np.float32)
        check(lib().wc_local_gradients(self._h, A._ptr(idx), idx.size, A._ptr(g), A._ptr(loss)), "wc_local_gradients")
        return g, float(loss[0])

    def evaluate(self, held_out: bool = True):
        """(network, stale, Taylor) errors per age: relative L2 of the acceleration."""
        a = np.zeros(self.ages, np.float32)
        b = np.zeros(self.ages, np.float32)
        c = np.zeros(self.ages, np.float32)
        check(lib().wc_local_evaluate(self._h, int(held_out), A._ptr(a), A._ptr(b), A._ptr(c)), "wc_local_evaluate")
        return a, b, c

    def predict(self, fluid: Fluid, dt: float):
        """(inputs [n, 32], the network's residuals of the acceleration changes [n, 3 ages]) of the
        fluid's current state, in the order of the judge step's sort; the fluid does not advance."""
        n = fluid.numParticles()
        x = np.zeros((n, IN), np.float32)
        y = np.zeros((n, 3 * self.ages), np.float32)
        check(lib().wc_local_predict(self._h, fluid._require(), float(dt), A._ptr(x), A._ptr(y)), "wc_local_predict")
        return x, y

    def close(self) -> None:
        if self._h is not None:
            lib().wc_local_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rollout(fluid: Fluid, dt: float, nsteps: int, ages: int = 3, tolerance: float = 0.01,
            net: LocalNet | None = None, mode: int | None = None) -> dict:
    """Cycles of one judge SPH step and `ages` extrapolated steps; mode WC_LOCAL_* (default: the
    network mode with a net, the stale mode without)."""
    st = RolloutStats()
    h = net._h if net is not None else None
    if mode is None:
        mode = WC_LOCAL_NETWORK if net is not None else WC_LOCAL_STALE
    check(lib().wc_local_rollout_mode(h, fluid._require(), float(dt), int(nsteps), int(ages), float(tolerance),
                                      int(mode), C.byref(st)), "wc_local_rollout_mode")
    return st.as_dict()


def save_weights(net: LocalNet, path: Path = DEFAULT_WEIGHTS, **meta) -> None:
    path.parent.mkdir(parents=True, exist_ok=True)
    np.savez(path, params=net.params(), ages=np.int32(net.ages), accel_scale=np.float32(net.config.accel_scale),
             velocity_scale=np.float32(net.config.velocity_scale), **meta)


def load_weights(path: Path = DEFAULT_WEIGHTS, **overrides) -> LocalNet:
    z = np.load(path)
    net = LocalNet(ages=int(z["ages"]), accel_scale=float(z["accel_scale"]), velocity_scale=float(z["velocity_scale"]),
                   **overrides)
    net.set_params(z["params"])
    return net


def main(argv=None) -> int:
    """python -m watercube_gb300.local: a fast rollout of the dam break (the benchmark's scene) in
    one mode, with its statistics printed as JSON."""
    import argparse
    import json

    from .fluid import dam_break_params, finalize, generate_dam_break

    ap = argparse.ArgumentParser(description=main.__doc__.split("\n")[0])
    ap.add_argument("--particles", type=int, default=1048576)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--ages", type=int, default=3, help="skipped steps per cycle (K - 1)")
    ap.add_argument("--mode", choices=["stale", "taylor", "network"], default="network")
    ap.add_argument("--tolerance", type=float, default=0.01)
    ap.add_argument("--weights", type=Path, default=None, help="default: weights/local_k{ages + 1}.npz")
    a = ap.parse_args(argv)
    check(lib().wc_set_device(0), "select device")
    p = finalize(dam_break_params(a.particles))
    dt = 2.5e-4 * (1048576.0 / a.particles) ** (1.0 / 3.0)
    mode = {"stale": WC_LOCAL_STALE, "taylor": WC_LOCAL_TAYLOR, "network": WC_LOCAL_NETWORK}[a.mode]
    net = None
    if mode == WC_LOCAL_NETWORK:
        net = load_weights(a.weights or DEFAULT_WEIGHTS.with_name(f"local_k{a.ages + 1}.npz"))
    with Fluid.create("rollout", p) as f:
        f.setup(generate_dam_break(p, 0))
        stats = rollout(f, dt, a.steps, ages=a.ages, tolerance=a.tolerance, net=net, mode=mode)
    if net is not None:
        net.close()
    print(json.dumps({"mode": a.mode, "particles": a.particles, "dt": dt, "K": a.ages + 1, **stats}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
