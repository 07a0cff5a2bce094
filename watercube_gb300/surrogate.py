"""The learned message-passing surrogate over the C ABI (wc_surrogate_*), its training data from
batched-solver trajectories, the training loop and the judged rollout. No counterpart in the
reference, which only runs plain SPH.

Network and kernels live in csrc/wc_surrogate.cu (driver), csrc/wc_nn_gemm.cu (tcgen05 GEMM) and
csrc/wc_nn_ops.cu (graph, features, LayerNorm, reductions, Adam); this module only moves host
arrays and drives the loop.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi as A
from ._abi import RolloutStats, SurrogateConfig, check, lib
from .batch import Batch, scene_params, scene_particles
from .fluid import Fluid

WC_ROLLOUT_SPH = 0
WC_ROLLOUT_SURROGATE = 1
WC_ROLLOUT_STALE = 2
WC_ROLLOUT_HYBRID = 3
HISTORY = 5  # velocities per node feature (current + 4 previous)


def default_config(**overrides) -> SurrogateConfig:
    c = SurrogateConfig()
    lib().wc_surrogate_config_default(C.byref(c))
    for k, v in overrides.items():
        setattr(c, k, v)
    return c


class Surrogate:
    """One network with its FP32 master weights, Adam state and activation workspaces."""

    def __init__(self, config: SurrogateConfig | None = None, **overrides):
        cfg = config if config is not None else default_config(**overrides)
        h = C.c_void_p()
        check(lib().wc_surrogate_create(C.byref(cfg), C.byref(h)), "wc_surrogate_create")
        self._h = h
        self.config = cfg
        self.num_params = int(lib().wc_surrogate_num_params(h))
        self._n = 0

    # ---- parameters --------------------------------------------------------------------------
    def params(self) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        check(lib().wc_surrogate_get_params(self._h, A._ptr(out), self.num_params), "get_params")
        return out

    def set_params(self, w: np.ndarray) -> None:
        w = np.ascontiguousarray(w, dtype=np.float32)
        check(lib().wc_surrogate_set_params(self._h, A._ptr(w), w.size), "set_params")

    def grads(self) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        check(lib().wc_surrogate_get_grads(self._h, A._ptr(out), self.num_params), "get_grads")
        return out

    def zero_grads(self) -> None:
        check(lib().wc_surrogate_zero_grads(self._h), "zero_grads")

    # ---- one sample ----------------------------------------------------------------------------
    def sample(self, fluid: Fluid, dt: float, hist: np.ndarray, target: np.ndarray | None = None,
               stale: np.ndarray | None = None, stale_age: int = 0) -> None:
        """Load the fluid's current particles with their velocity history hist (5, n, 4), steps
        dt apart, optional target accelerations (n, 4) and optionally the last SPH acceleration
        (n, 4) computed stale_age >= 1 steps earlier, all in the fluid's state order."""
        n = fluid.numParticles()
        hist = np.ascontiguousarray(hist, dtype=np.float32)
        if hist.shape != (HISTORY, n, 4):
            raise A.WatercubeError(A.WC_ERR_INVALID_ARG, f"history has shape {hist.shape}, want (5, {n}, 4)")
        tp = None
        if target is not None:
            target = np.ascontiguousarray(target, dtype=np.float32)
            if target.shape != (n, 4):
                raise A.WatercubeError(A.WC_ERR_INVALID_ARG, f"target has shape {target.shape}")
            tp = A._ptr(target)
        sp = None
        if stale is not None and stale_age > 0:
            stale = np.ascontiguousarray(stale, dtype=np.float32)
            if stale.shape != (n, 4):
                raise A.WatercubeError(A.WC_ERR_INVALID_ARG, f"stale acceleration has shape {stale.shape}")
            sp = A._ptr(stale)
        else:
            stale_age = 0
        check(lib().wc_surrogate_sample(self._h, fluid._require(), float(dt), A._ptr(hist), tp, sp, int(stale_age)),
              "wc_surrogate_sample")
        self._n = n

    def forward_backward(self, backward: bool = True) -> float:
        loss = C.c_double(0.0)
        check(lib().wc_surrogate_forward_backward(self._h, int(backward), C.byref(loss)), "forward_backward")
        return loss.value

    def predictions(self) -> np.ndarray:
        out = np.zeros((self._n, 4), np.float32)
        check(lib().wc_surrogate_predictions(self._h, A._ptr(out), self._n), "predictions")
        return out

    def adam(self, lr: float, grad_scale: float = 1.0) -> None:
        check(lib().wc_surrogate_adam(self._h, float(lr), float(grad_scale)), "adam")

    # ---- rollout -------------------------------------------------------------------------------
    def rollout(self, fluid: Fluid, dt: float, nsteps: int, K: int = 4, tolerance: float = 0.01,
                mode: int = WC_ROLLOUT_SURROGATE, hist: np.ndarray | None = None) -> dict:
        return rollout(fluid, dt, nsteps, K, tolerance, mode, self, hist)

    def close(self) -> None:
        if self._h is not None:
            lib().wc_surrogate_destroy(self._h)
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


def rollout(fluid: Fluid, dt: float, nsteps: int, K: int = 4, tolerance: float = 0.01,
            mode: int = WC_ROLLOUT_SPH, surrogate: Surrogate | None = None, hist: np.ndarray | None = None) -> dict:
    """Advance `fluid` nsteps in `mode` (WC_ROLLOUT_*) and return the rollout statistics. `hist`
    (5, n, 4), in the fluid's state order, seeds the surrogate's velocity history."""
    st = RolloutStats()
    h = surrogate._h if surrogate is not None else None
    hp = None
    if hist is not None:
        hist = np.ascontiguousarray(hist, dtype=np.float32)
        if hist.shape != (HISTORY, fluid.numParticles(), 4):
            raise A.WatercubeError(A.WC_ERR_INVALID_ARG, f"history has shape {hist.shape}")
        hp = A._ptr(hist)
    check(lib().wc_surrogate_rollout(h, fluid._require(), float(dt), int(nsteps), int(K), float(tolerance),
                                     int(mode), hp, C.byref(st)), "wc_surrogate_rollout")
    return st.as_dict()


# ---- training data ---------------------------------------------------------------------------

@dataclass
class Sample:
    """One scene at one time step, arrays in particle-id order."""

    scene: int
    step: int
    dt: float
    state: np.ndarray   # (n,) PARTICLE_DTYPE: positions and velocities before the step
    hist: np.ndarray    # (5, n, 4) velocities, hist[0] = state velocity
    target: np.ndarray  # (n, 4) SPH acceleration of the state (w = 0)


def record_samples(specs, steps: int, dt: float, every: int = 1, start: int = 0, sink=None,
                   keep: bool = True) -> tuple[list, list[Sample]]:
    """Run the batched solver on `specs` for `steps` steps with acceleration recording on and
    collect one Sample per scene every `every` steps from step `start`. Returns (params per
    scene, samples). `sink` (a DatasetWriter, or anything with write(Sample)) receives every
    sample as it is made; keep=False then holds none in memory."""
    params = [scene_params(s) for s in specs]
    initial = [scene_particles(s, p) for s, p in zip(specs, params)]
    samples: list[Sample] = []
    with Batch(params, initial) as b:
        total = b.num_particles
        off = b.offsets().astype(np.int64)
        check(lib().wc_batch_set_recording(b._h, 1), "wc_batch_set_recording")
        ids = np.zeros(total, np.uint32)
        acc = np.zeros((total, 4), np.float32)
        vel_by_id = np.zeros((total, 4), np.float32)
        state = b.particles()
        check(lib().wc_batch_get_ids(b._h, A._ptr(ids), total), "wc_batch_get_ids")
        vel_by_id[ids, :3] = state["velocity"]
        hist = np.repeat(vel_by_id[None], HISTORY, axis=0)
        for t in range(steps):
            state_by_id = np.empty(total, A.PARTICLE_DTYPE)
            state_by_id[ids] = state
            b.step(dt, 1)
            check(lib().wc_batch_get_accelerations(b._h, A._ptr(acc), total), "wc_batch_get_accelerations")
            check(lib().wc_batch_get_ids(b._h, A._ptr(ids), total), "wc_batch_get_ids")
            acc_by_id = np.zeros((total, 4), np.float32)
            acc_by_id[ids, :3] = acc[:, :3]
            if t >= start and (t - start) % every == 0:
                for s in range(len(specs)):
                    lo, hi = int(off[s]), int(off[s + 1])
                    smp = Sample(s, t, dt, state_by_id[lo:hi].copy(), hist[:, lo:hi].copy(), acc_by_id[lo:hi].copy())
                    if sink is not None:
                        sink.write(smp)
                    if keep:
                        samples.append(smp)
            state = b.particles()
            vel_by_id = np.zeros((total, 4), np.float32)
            vel_by_id[ids, :3] = state["velocity"]
            hist = np.concatenate([vel_by_id[None], hist[:-1]], axis=0)
    return params, samples


class Trainer:
    """Adam on batches of samples (gradients accumulated over the batch, averaged), one
    wc_fluid per scene holding the sample's particles for the graph build.

    The hybrid rollout feeds the network the last SPH acceleration and its age. Training shows
    it the same: for each sample, with probability 1 - p_no_stale, the target of the same
    scene k steps earlier (k uniform in 1 .. stale_k_max, when recorded) with age k, which makes
    the sample residual (the network learns the change since then); otherwise none, as the plain
    surrogate rollout runs."""

    def __init__(self, surrogate: Surrogate, params: list, position_noise: float = 3e-4, seed: int = 0,
                 velocity_noise: float = 0.0, p_no_stale: float = 0.2, stale_k_max: int = 7):
        self.s = surrogate
        self.params = params
        self.noise = position_noise
        # independent Gaussian noise on each velocity of the history (the state's velocity is
        # hist[0] and moves with it): robustness to the network's own past errors in a rollout
        self.vnoise = velocity_noise
        self.rng = np.random.default_rng(seed)
        self.p_no_stale = p_no_stale
        self.stale_k_max = stale_k_max
        self.by: dict[tuple[int, int], Sample] = {}
        self._fluids: dict[int, Fluid] = {}

    def index(self, samples: list[Sample]) -> None:
        """Make `samples` available as the source of earlier SPH accelerations."""
        for x in samples:
            self.by[(x.scene, x.step)] = x

    def stale_for(self, smp: Sample, k: int) -> np.ndarray | None:
        """The SPH acceleration of the same scene k steps before smp, if recorded."""
        src = self.by.get((smp.scene, smp.step - k)) if k > 0 else None
        return None if src is None else src.target

    def draw_stale(self, smp: Sample) -> tuple[np.ndarray | None, int]:
        if self.stale_k_max < 1 or self.rng.random() < self.p_no_stale:
            return None, 0
        k = int(self.rng.integers(1, self.stale_k_max + 1))
        st = self.stale_for(smp, k)
        return (st, k) if st is not None else (None, 0)

    def fluid(self, scene: int, state: np.ndarray) -> Fluid:
        f = self._fluids.get(scene)
        if f is None:
            f = Fluid(f"scene{scene}", self.params[scene])
            f.setup(state)
            self._fluids[scene] = f
        else:
            f.set_particles(state)
        return f

    def load(self, smp: Sample, noise: bool, stale_k: int | None = None) -> None:
        """Load smp; stale_k None draws the stale acceleration at random (training), an int
        gives its age (0: none)."""
        state, hist = smp.state, smp.hist
        if stale_k is None:
            stale, age = self.draw_stale(smp)
        else:
            stale, age = self.stale_for(smp, stale_k), stale_k
            if stale is None:
                age = 0
        if noise and self.vnoise > 0:
            hist = hist + np.pad(self.rng.normal(0.0, self.vnoise, hist[..., :3].shape),
                                 ((0, 0), (0, 0), (0, 1))).astype(np.float32)
            state = state.copy()
            state["velocity"] = hist[0, :, :3]
        if noise and self.noise > 0:
            state = state.copy()
            state["position"] += self.rng.normal(0.0, self.noise, state["position"].shape).astype(np.float32)
            size = self.params[smp.scene].size
            border = self.params[smp.scene].wall_border
            np.clip(state["position"], border, size - border, out=state["position"])
        f = self.fluid(smp.scene, state)
        self.s.sample(f, smp.dt, hist, smp.target, stale, age)

    def step(self, batch: list[Sample], lr: float) -> float:
        """One Adam step over `batch`; returns the mean loss."""
        losses = []
        for smp in batch:
            self.load(smp, noise=True, stale_k=None)
            losses.append(self.s.forward_backward(True))
        self.s.adam(lr, 1.0 / len(batch))
        return float(np.mean(losses))

    def evaluate(self, samples: list[Sample], stale_k: int = 0) -> float:
        """Mean loss over samples (no noise, no gradient), with the SPH acceleration of stale_k
        steps earlier as input (0: none)."""
        out = []
        for smp in samples:
            self.load(smp, noise=False, stale_k=stale_k)
            out.append(self.s.forward_backward(False))
        return float(np.mean(out))

    def predict(self, smp: Sample, stale_k: int = 0) -> np.ndarray:
        self.load(smp, noise=False, stale_k=stale_k)
        self.s.forward_backward(False)
        return self.s.predictions()

    def train(self, samples: list[Sample], steps: int, lr: float = 1e-4, batch: int = 8) -> list[float]:
        self.index(samples)
        hist = []
        for _ in range(steps):
            idx = self.rng.choice(len(samples), size=min(batch, len(samples)), replace=False)
            hist.append(self.step([samples[i] for i in idx], lr))
        return hist

    def close(self) -> None:
        for f in self._fluids.values():
            f.close()
        self._fluids.clear()


def main(argv=None) -> dict:
    """`python -m watercube_gb300.surrogate`: a judged rollout of the message-passing surrogate on
    the dam break from its initial state (the trained weights when present), printing the rollout
    statistics as one JSON line."""
    import argparse
    import json

    from .fluid import dam_break_params, finalize, generate_dam_break
    from .train_surrogate import DEFAULT_WEIGHTS, load_weights

    modes = {"sph": WC_ROLLOUT_SPH, "surrogate": WC_ROLLOUT_SURROGATE, "stale": WC_ROLLOUT_STALE,
             "hybrid": WC_ROLLOUT_HYBRID}
    ap = argparse.ArgumentParser(description="Judged rollout of the message-passing surrogate on the dam break "
                                             "(prints the rollout statistics as one JSON line)")
    ap.add_argument("--particles", type=int, default=1048576)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--K", type=int, default=4, help="a plain SPH judge step every K steps")
    ap.add_argument("--dt", type=float, default=2.5e-4)
    ap.add_argument("--mode", choices=sorted(modes), default="surrogate")
    args = ap.parse_args(argv)
    check(lib().wc_set_device(0), "wc_set_device")
    p = finalize(dam_break_params(args.particles))
    st = generate_dam_break(p, 0)
    s = load_weights() if DEFAULT_WEIGHTS.is_file() else Surrogate(layers=8, seed=1)
    try:
        with Fluid.create("rollout", p) as f:
            f.setup(st)
            r = rollout(f, args.dt, args.steps, args.K, 0.01, modes[args.mode], s)
    finally:
        s.close()
    r.update(particles=args.particles, mode=args.mode, K=args.K)
    print(json.dumps(r), flush=True)
    return r


if __name__ == "__main__":
    main()
