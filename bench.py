"""Benchmark of the plain SPH step at 1,048,576 particles (the dam break the solver is measured
on), printing one JSON line.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload dam1m|dam16k|batch512|rollout1m]

value      particle-steps/s of K graph-launched steps (the timed window: steps W+1 .. W+K of the
           workload from its initial state), inputs resident in HBM, device time from CUDA events
           around each step; L2 is flushed (a read of twice its size) before every timed step,
           outside the timed span.
e2e        the same metric over the same window through the C ABI with host buffers: each step
           is one wc_fluid_update_host call, which uploads the particle state from pinned host
           memory, runs the step and reads the state back (each eighth of the slots copied out
           as soon as the force pass has stored it, while the pass computes the rest).
roofline   the dominant kernel's algorithmic bytes per launch / its mean CUDA-event time over the
           same window (separately launched kernels), against the measured HBM copy bandwidth;
           `traffic` is its DRAM bytes per launch from ncu (profiles/ncu_traffic.json).
cpu_baseline  the CPU transcription of the reference's stages (oracle, FP32) on this host's
           cores, on a bounded sample of the same window (a few steps from states spread over it).
--advance N  runs N untimed steps before the warm-up, to time or profile a later window.
--impl reference  times the reference's own shader code compiled for the host CPU
           (oracle/_ref, when built) or else the oracle's transcription, all threads.
surface    surface extraction of the same state: colour field on 256^3 vertices and marching
           cubes, CUDA-event times.
rollout    rollouts at the same size from the same initial state, --rollout-steps steps each:
           plain SPH and the fast rollout's three modes (a judge SPH step every K steps, the
           K - 1 steps between on the judge's acceleration extrapolated to first order plus the
           network's residual ("learned"), to first order ("taylor"), or held ("stale")) for
           K = 4 and every other K with trained weights (5, 6), with the judge's density error
           and the position drift from plain SPH; the message-passing network's modes a few
           steps each. `--workload rollout1m` times them alone with --steps steps (default
           2,000) and reports the fastest learned mode within the density tolerance.
--workload batch512  512 scenes of 4,096-65,536 particles in one launch per stage, 500 steps
           after the autotuner (its choice in `tuning`).
Multi-GPU (torchrun): every rank runs an independent replica (the path has no exchange step);
the slowest rank's time is reported.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = "particle-steps/s at 1M particles (plain SPH step)"
UNIT = "particle-steps/s"

WORKLOADS = {
    # name: (particles, dt, description)
    "dam1m": (1048576, 2.5e-4, "dam break, 1,048,576 particles, h=0.011425, 87^3 cells, dt=2.5e-4"),
    "dam16k": (16384, 1e-3, "dam break, 16,384 particles, h=0.0457, 21^3 cells, dt=1e-3"),
}

# Algorithmic bytes per particle per launch (reads + writes the kernel must make once).
ALGO_BYTES = {
    "bin_count": 16.0,  # read position 12, write key 4
    "scan_cells": None,  # per cell: read count 4, write start 4, clear count 4 (x C/N)
    "scatter_cells": 12.0,  # read key 4 + rank 4, write slot 4
    "rank_gather": 40.0,  # read position 12 + velocity 12 (+ key), write 24 + permutation 4
    "density": 20.0,  # read position 12, write density + pressure 8
    "force_integrate": 56.0,  # read position, velocity, density, pressure 32, write position, velocity 24
}


def step_algo_bytes(n: int, cells: int) -> float:
    """Per particle-step algorithmic bytes of the whole step: 152 + 32 C/N (binning 16,
    histogram 4, reorder 56, density 20, force 56, cell tables 32 per cell)."""
    return 152.0 + 32.0 * cells / max(n, 1)


def measured_peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.is_file():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_capture(workload: str, window_mid: float):
    """The ncu capture of `workload` (profiles/ncu_traffic.json) whose step is nearest the middle
    of the timed window: per kernel its DRAM bytes and warp-instructions per launch. A step's
    cost changes as the fluid compresses, so the capture must match the window."""
    p = REPO / "profiles" / "ncu_traffic.json"
    if not p.is_file():
        return None
    caps = [c for c in json.loads(p.read_text()).get("captures", []) if c.get("workload") == workload]
    if not caps:
        return None
    return min(caps, key=lambda c: abs(float(c["step"]) - window_mid))


def sm_count(device: int) -> int:
    try:
        import torch

        return int(torch.cuda.get_device_properties(device).multi_processor_count)
    except Exception:
        return 152  # GB300


def issue_bound(cap: dict, kernel: str, ms: float, sms: int, sm_mhz: float, n: int):
    """The instruction-issue roofline of `kernel`: its warp-instructions per launch (ncu,
    smsp__inst_executed.sum of the matching capture) over its mean CUDA-event time, against the
    SMs' issue rate (4 schedulers x one warp-instruction per cycle each, at the median SM clock
    sampled during the timed region)."""
    inst = cap.get("warp_instructions", {}).get(kernel)
    if inst is None:
        return None
    achieved = float(inst) / (ms * 1e-3) / 1e9
    peak = sms * 4 * sm_mhz * 1e6 / 1e9
    return {"bound": "issue", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "G warp-instructions/s",
            "frac": achieved / peak, "warp_instructions_per_particle": float(inst) / n,
            "peak_source": f"{sms} SMs x 4 schedulers x {sm_mhz:.0f} MHz (median sampled SM clock)",
            "instructions_source": f"ncu smsp__inst_executed.sum, launch of step {cap['step']}"}


def workload_config(workload: str, n: int, grid_res: int, dt: float, first: int, last: int, world: int) -> dict:
    """The `config` object of both arms (identical for the same workload, window and N)."""
    return {
        "workload": WORKLOADS[workload][2],
        "particles_per_gpu": n,
        "grid_res": grid_res,
        "cells": grid_res ** 3,
        "dt": dt,
        "window": f"steps {first} .. {last} from the initial state",
        "l2": "GPU arm: flushed before every timed step (read of 2x L2), outside the timed span; "
              "CPU arm: not applicable",
        "parallelism": f"{world} independent replicas" if world > 1 else "1 GPU",
    }


class Clocks:
    """nvidia-smi sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"wc_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path.is_file():
            return None
        rows = [r.split(",") for r in self.path.read_text().strip().splitlines() if r.strip()]
        try:
            self.path.unlink()
        except OSError:
            pass
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except ValueError:
                continue
            for name, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(gpus: int):
    """(rank, world, local_rank, reduce_max) for torchrun launches; plain values for N=1."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world <= 1:
        return 0, 1, 0, (lambda x: x), (lambda: None)
    import torch
    import torch.distributed as dist

    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)

    def reduce_max(x: float) -> float:
        t = torch.tensor([x], dtype=torch.float64, device="cuda" if backend == "nccl" else "cpu")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    return rank, world, local, reduce_max, dist.barrier


def cpu_baseline(p, samples, dt, threads_all: int):
    """The oracle's FP32 transcription on a bounded sample of the timed window (about 20 s of CPU
    work at 1M particles): from each state in `samples` ((window step, particles) pairs spread
    evenly over the window, taken from the GPU run), 8 full steps on all threads and 1 on one
    thread. A step's cost grows as the fluid compresses, so the per-step times are averaged
    over the states, as the GPU's are over the window."""
    from oracle.oracle import Oracle

    o = Oracle()
    n = samples[0][1].shape[0]
    o.step(p, samples[0][1].copy(), dt, 1, threads=threads_all)  # warm-up (page-in, thread pool)
    k_all, k_one = 8, 1
    t_all, t_one = [], []
    for _, state in samples:
        s = state.copy()
        t = time.perf_counter()
        o.step(p, s, dt, k_all, threads=threads_all)
        t_all.append((time.perf_counter() - t) / k_all)
        s = state.copy()
        t = time.perf_counter()
        o.step(p, s, dt, k_one, threads=1)
        t_one.append((time.perf_counter() - t) / k_one)
    m_all, m_one = float(np.mean(t_all)), float(np.mean(t_one))
    at = ", ".join(str(k) for k, _ in samples)
    return {
        "value": n / m_all,
        "unit": UNIT,
        "cores": threads_all,
        "kind": "port",
        "sample": f"{k_all} full steps on all threads and {k_one} on one thread from each of {len(samples)} states of "
                  f"the timed window (window steps {at}; states from the GPU run), per-step times averaged over the "
                  f"states; the {n}-particle workload, the oracle's FP32 transcription of the reference's shader stages",
        "value_1thread": n / m_one,
        "ms_per_step": m_all * 1e3,
        "ms_per_step_1thread": m_one * 1e3,
        "ms_per_step_by_state": [x * 1e3 for x in t_all],
    }


REF_SAMPLE_STEPS = 20  # steps the reference arm times, at most


def run_reference(args):
    """--impl reference: the reference's CPU implementation of the path on this host. Only the
    oracle libraries are loaded (parameters and the initial lattice come from the oracle too):
    nothing of the solver runs in this arm."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return 0
    from oracle.oracle import Oracle, RefLib, build_ref, ref_available

    n, dt, desc = WORKLOADS[args.workload]
    o = Oracle()
    p = o.dam_break_params(n)
    st = o.generate_dam_break(p, 0)
    threads = os.cpu_count() or 1
    kind = "port"
    try:
        if not ref_available():
            build_ref()
        if ref_available():
            kind = "reference"
    except Exception:
        kind = "port"
    state = st.copy()
    if kind == "reference":
        ref = RefLib()

        def one_step():
            ref.step(p, state, dt, 1, threads=threads)
    else:
        def one_step():
            o.step(p, state, dt, 1, threads=threads)

    warm = args.advance + max(args.warmup, 3)
    for _ in range(warm):
        one_step()
    # a bounded sample of the window: its first REF_SAMPLE_STEPS steps (the window's late steps
    # cost up to ~1.3 s each on 16 cores; the full 1,000-step window took 11 minutes), so the rate
    # comes from the cheapest part of the workload and favours the reference
    sampled = min(args.steps, REF_SAMPLE_STEPS)
    t = time.perf_counter()
    for _ in range(sampled):
        one_step()
    el = time.perf_counter() - t
    value = n * sampled / el
    what = ("the reference's compute shaders (assets/sort/*.comp, assets/fluid/density.comp, update.comp) compiled "
            "as C++ and dispatched in Fluid::update order, OpenMP over invocations" if kind == "reference" else
            "the oracle's FP32 transcription of the reference's shader stages, OpenMP")
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": el / sampled * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": workload_config(args.workload, n, int(p.grid_res), dt, warm + 1, warm + args.steps, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": f"the first {sampled} full steps of the window (steps {warm + 1} .. {warm + sampled}) "
                                   f"of the {n}-particle workload, from its initial state: {what}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def by_id(f) -> np.ndarray:
    """Positions of a fluid's state buffer in particle-id order."""
    out = f.particles()
    ids = f.particle_ids()
    pos = np.empty((ids.size, 3))
    pos[ids] = out["position"]
    return pos


def run_rollouts(p, st, dt, steps: int, K: int = 4, tolerance: float = 0.01, gnn_steps: int = 8,
                 cycle_lengths=(4, 5, 6)) -> dict:
    """Rollouts of `steps` steps from `st`, each on a fresh fluid, against plain SPH over the same
    steps: cycles of one judge SPH step and K - 1 extrapolated steps in the three modes of the
    fast rollout: "learned" (a + k dt J plus the network's residual), "taylor" (a + k dt J) and
    "stale" (the judge's acceleration held), for each K of `cycle_lengths` whose trained weights
    (weights/local_k{K}.npz) exist (K itself always runs; the others get the suffix "_k{K}"),
    with density error (the judge's), RMS and largest position drift from the plain SPH
    trajectory (in h) and FP64 momentum / energy change; then the message-passing network's
    judged modes, `gnn_steps` steps each (its step costs hundreds of plain steps at this size)."""
    from watercube_gb300 import _abi
    from watercube_gb300.fluid import Fluid
    from watercube_gb300.local import DEFAULT_WEIGHTS as LOCAL_WEIGHTS
    from watercube_gb300.local import WC_LOCAL_NETWORK, WC_LOCAL_STALE, WC_LOCAL_TAYLOR, LocalNet, load_weights
    from watercube_gb300.local import rollout as local_rollout
    from watercube_gb300.surrogate import (
        WC_ROLLOUT_HYBRID,
        WC_ROLLOUT_SPH,
        WC_ROLLOUT_STALE,
        WC_ROLLOUT_SURROGATE,
        Surrogate,
        rollout,
    )
    from watercube_gb300.train_surrogate import DEFAULT_WEIGHTS, load_weights as load_gnn

    q = p.copy()
    q.flags |= _abi.WC_FLAG_TRACK_IDS
    h = float(p.kernel_radius)
    keep = ("particle_steps_per_s", "ms_device", "steps", "sph_steps", "surrogate_steps", "judged", "reverted",
            "mean_density_error", "max_density_error")

    def diag_changes(r):
        d0, d1 = np.array(r["diag_start"]), np.array(r["diag_end"])
        return {"momentum_change": float(np.linalg.norm(d1[1:4] - d0[1:4])),  # gravity and walls act on it
                "energy_change_rel": float(abs((d1[4] + d1[5]) - (d0[4] + d0[5])) / max(abs(d0[4] + d0[5]), 1e-30))}

    out = {"steps": steps, "K": K, "tolerance": tolerance}
    with Fluid.create("rollout", q) as f:
        f.setup(st)
        f.step(dt, 2)
        f.setup(st)
        r = rollout(f, dt, steps, K, tolerance, WC_ROLLOUT_SPH, None)
        plain_pos = by_id(f)
        out["plain"] = {**{k: r[k] for k in keep}, **diag_changes(r)}
    best = None
    for k_len in sorted(set(cycle_lengths) | {K}):
        path = LOCAL_WEIGHTS.with_name(f"local_k{k_len}.npz")
        trained = path.is_file()
        if not trained and k_len != K:
            continue
        net = load_weights(path) if trained else LocalNet(ages=k_len - 1, seed=1)
        suffix = "" if k_len == K else f"_k{k_len}"
        out["weights" + suffix] = path.relative_to(REPO).as_posix() if trained else "untrained (seed 1)"
        for name, mode in (("learned", WC_LOCAL_NETWORK), ("taylor", WC_LOCAL_TAYLOR), ("stale", WC_LOCAL_STALE)):
            model = net if mode == WC_LOCAL_NETWORK else None
            with Fluid.create("rollout", q) as f:
                f.setup(st)
                local_rollout(f, dt, 2 * k_len, ages=k_len - 1, tolerance=tolerance, net=model, mode=mode)  # warm-up
                f.setup(st)
                r = local_rollout(f, dt, steps, ages=k_len - 1, tolerance=tolerance, net=model, mode=mode)
                d = np.linalg.norm(by_id(f) - plain_pos, axis=1) / h
                e = {"K": k_len, **{k: r[k] for k in keep}}
                e.update(diag_changes(r))
                e["rms_drift_h"] = float(np.sqrt(np.mean(d * d)))
                e["max_drift_h"] = float(d.max())
                e["vs_plain"] = e["particle_steps_per_s"] / out["plain"]["particle_steps_per_s"]
                out[name + suffix] = e
                if (name == "learned" and trained and e["mean_density_error"] <= tolerance
                        and (best is None or e["vs_plain"] > best["vs_plain"])):
                    best = {"mode": name + suffix, **{x: e[x] for x in ("K", "vs_plain", "mean_density_error",
                                                                         "rms_drift_h", "reverted")}}
        net.close()
    out["best_learned"] = best
    out["judge"] = ("every K-th step is plain SPH; it compares each particle's density carried through the "
                    "skipped steps (the judge step's density plus its rate) with the SPH density of the same "
                    "particles and reverts the cycle when the mean |rho_carried / rho_SPH - 1| exceeds the tolerance")
    # the message-passing network (width 128, 8 layers) in its one-step-judged modes
    gnn = {"steps": gnn_steps, "K": K}
    trained_gnn = DEFAULT_WEIGHTS.is_file()
    s = load_gnn() if trained_gnn else Surrogate(layers=8, seed=1)
    gnn["weights"] = DEFAULT_WEIGHTS.relative_to(REPO).as_posix() if trained_gnn else "untrained (seed 1)"
    for mode, name in ((WC_ROLLOUT_SURROGATE, "surrogate"), (WC_ROLLOUT_HYBRID, "hybrid"),
                       (WC_ROLLOUT_STALE, "stale_one_step_judge")):
        with Fluid.create("rollout", p) as f:
            f.setup(st)
            rollout(f, dt, 1 if mode == WC_ROLLOUT_SURROGATE else 2, K, tolerance, mode, s)
            f.setup(st)
            r = rollout(f, dt, gnn_steps, K, tolerance, mode, s)
            e = {k: r[k] for k in keep}
            e["vs_plain"] = e["particle_steps_per_s"] / out["plain"]["particle_steps_per_s"]
            gnn[name] = e
    s.close()
    out["message_passing"] = gnn
    out["learned_vs_plain"] = out["learned"]["vs_plain"]
    out["taylor_vs_plain"] = out["taylor"]["vs_plain"]
    out["stale_vs_plain"] = out["stale"]["vs_plain"]
    return out


def run_surface(p, st, grid_res: int = 256, reps: int = 5) -> dict:
    """Surface extraction (colour field on grid_res^3 vertices + marching cubes) of the
    workload's state, CUDA-event times of the field and of classify + scan + emit (median of
    `reps` extractions after one warm-up)."""
    from watercube_gb300.fluid import Fluid
    from watercube_gb300.surface import Surface

    with Fluid.create("surface", p) as f, Surface(grid_res, iso=0.5) as s:
        f.setup(st)
        s.extract(f)
        fields, meshes = [], []
        for _ in range(reps):
            ntri = s.extract(f)
            a, b = s.timings()
            fields.append(a)
            meshes.append(b)
    V = grid_res**3
    mf, mm = float(np.median(fields)), float(np.median(meshes))
    return {"grid_res": grid_res, "triangles": ntri, "ms_field": mf, "ms_mesh": mm,
            "vertices_per_s": V / (mf * 1e-3), "cubes_per_s": (grid_res - 1) ** 3 / (mm * 1e-3)}


def run_rollout_workload(args):
    """--workload rollout1m: the rollouts at 1,048,576 particles from the dam break's initial
    state (dt = 2.5e-4, 1% density tolerance, K = 4 and every other cycle length with trained
    weights), --steps steps each (default 2,000, the workload's length); the value is the
    particle-steps/s of the fastest learned rollout whose mean density error stays within the
    tolerance (K = 4 when none does)."""
    from watercube_gb300 import _abi
    from watercube_gb300.fluid import dam_break_params, finalize, generate_dam_break

    _abi.check(_abi.lib().wc_set_device(0), "select device")
    n, dt, desc = WORKLOADS["dam1m"]
    p = finalize(dam_break_params(n))
    st = generate_dam_break(p, 0)
    with Clocks(0) as clocks:
        r = run_rollouts(p, st, dt, args.steps)
    mode = r["best_learned"]["mode"] if r["best_learned"] else "learned"
    learned = r[mode]
    line = {
        "metric": f"particle-steps/s at 1M particles, learned rollout (K={learned['K']}, 1% density tolerance)",
        "value": learned["particle_steps_per_s"],
        "unit": UNIT,
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": learned["ms_device"] / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 solver, bf16 network (fp32 accumulate)",
        "data": "synthetic",
        "config": {"workload": desc + ", rollout from the initial state", "particles": n, "dt": dt,
                   "K": learned["K"], "mode": mode, "tolerance": 0.01},
        "vs_plain": learned["vs_plain"],
        "rollout": r,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    rank, world, local, reduce_max, barrier = dist_setup(args.gpus)
    from watercube_gb300 import _abi
    from watercube_gb300.fluid import Fluid, PinnedBuffer, dam_break_params, finalize, generate_dam_break

    _abi.check(_abi.lib().wc_set_device(local), "select device")
    n, dt, desc = WORKLOADS[args.workload]
    p = finalize(dam_break_params(n))
    st = generate_dam_break(p, rank)
    cells = int(p.grid_res) ** 3
    f = Fluid.create("bench", p)
    f.setup(st)
    if args.advance:
        f.step(dt, args.advance)
    # warm-up: graph capture, clocks up
    f.step(dt, max(args.warmup, 3))
    f.synchronize()

    barrier()
    clocks = Clocks(local)
    with clocks:
        step_ms, _ = f.time_steps(dt, args.steps, flush_l2=True, kernel_times=False)
    barrier()
    total_ms = reduce_max(float(step_ms.sum()))
    clock_summary = clocks.summary()
    value = world * n * args.steps / (total_ms * 1e-3)

    def restart():
        """Back to the timed window's first state: the initial particles and the warm-up steps
        (steps are deterministic, so the window repeats bit for bit)."""
        f.set_particles(st)
        f.step(dt, args.advance + max(args.warmup, 3))
        f.synchronize()

    # Per-kernel CUDA-event times over the same window (separately launched steps, L2 flushed
    # before each), in four parts; each part's first state is kept for the CPU sample.
    restart()
    samples, kern_parts, done = [], [], 0
    for i in range(4):
        k = args.steps * (i + 1) // 4 - done
        if k == 0:
            continue
        samples.append((done, f.particles()))
        _, kp = f.time_steps(dt, k, flush_l2=True, kernel_times=True, graph_steps=False)
        kern_parts.append(kp)
        done += k
    kern = np.concatenate(kern_parts)
    names = Fluid.kernel_names()
    kmean = {k: float(np.mean(kern[:, i])) for i, k in enumerate(names)}
    dom = max(kmean, key=kmean.get)
    peak, peak_kind = measured_peaks()
    algo = ALGO_BYTES[dom] * n if ALGO_BYTES.get(dom) else 12.0 * cells
    achieved = algo / (kmean[dom] * 1e-3) / 1e9
    step_mean_ms = total_ms / args.steps
    step_gbs = step_algo_bytes(n, cells) * n / (step_mean_ms * 1e-3) / 1e9
    first = args.advance + max(args.warmup, 3) + 1
    last = first + args.steps - 1
    cap = ncu_capture(args.workload, 0.5 * (first + last))
    sm_mhz = (clock_summary or {}).get("sm_mhz") or 2070.0
    issue = issue_bound(cap, dom, kmean[dom], sm_count(local), sm_mhz, n) if cap else None

    # end to end through the C ABI with host buffers
    nbytes = n * 32
    hin = PinnedBuffer(nbytes)
    hout = PinnedBuffer(nbytes)
    ain = hin.particles(n)
    aout = hout.particles(n)
    ain[:] = f.particles()
    lib = _abi.lib()
    e2e_steps = args.steps  # the same window as the device-timed steps

    def e2e_step(src, dst):
        _abi.check(lib.wc_fluid_update_host(f._handle, dt / float(p.time_scale), src.ctypes.data, dst.ctypes.data, n))

    for _ in range(2):
        e2e_step(ain, aout)
        ain, aout = aout, ain
    restart()
    ain[:] = f.particles()
    barrier()
    t = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step(ain, aout)
        ain, aout = aout, ain
    el = reduce_max(time.perf_counter() - t)
    e2e_value = world * n * e2e_steps / el

    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": step_mean_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": workload_config(args.workload, n, int(p.grid_res), dt, first, last, world),
        "roofline": {
            "bound": "hbm",
            "kernel": dom,
            "achieved": achieved,
            "peak": peak,
            "unit": "GB/s",
            "frac": achieved / peak,
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
            "algorithmic_bytes_per_launch": algo,
            "traffic": float(cap["dram_bytes"][dom]) if cap and dom in cap.get("dram_bytes", {}) else None,
            "traffic_source": (f"ncu, launch of step {cap['step']} (the capture nearest the window's middle, "
                               "profiles/ncu_traffic.json)") if cap else None,
            "step": {"algorithmic_bytes_per_particle": step_algo_bytes(n, cells), "achieved": step_gbs,
                     "frac": step_gbs / peak},
            "issue": issue,
        },
        "kernels_ms": kmean,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": e2e_steps,
                "pattern": "wc_fluid_update_host(pinned host in, pinned host out): upload, step, readback "
                           "overlapping the force pass"},
        "gpu_launches": 6 * args.steps,
        "clocks": clock_summary,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(p, samples, dt, os.cpu_count() or 1)
    if rank == 0 and world == 1 and not args.no_rollout and args.workload == "dam1m":
        line["rollout"] = run_rollouts(p, st, dt, args.rollout_steps)
        line["surface"] = run_surface(p, st)
    f.close()
    hin.free()
    hout.free()
    if rank == 0:
        print(json.dumps(line))
    return 0


def batch_cpu_baseline(specs, params, states, dt, threads_all: int, scenes: int = 8, steps: int = 2) -> dict:
    """The oracle's FP32 transcription on a bounded sample of the batched workload: `steps` full
    steps of `scenes` scenes spread over the draw (every 64th), all threads, per scene in turn."""
    from oracle.oracle import Oracle

    o = Oracle()
    pick = list(range(0, len(specs), max(1, len(specs) // scenes)))[:scenes]
    n = 0
    el = 0.0
    for s in pick:
        st = states[s].copy()
        o.step(params[s], st, dt, 1, threads=threads_all)  # page-in, thread pool
        t = time.perf_counter()
        o.step(params[s], st, dt, steps, threads=threads_all)
        el += time.perf_counter() - t
        n += st.shape[0] * steps
    return {"value": n / el, "unit": UNIT, "cores": threads_all, "kind": "port",
            "sample": f"{steps} full steps of each of {len(pick)} scenes (every {max(1, len(specs) // scenes)}th of the "
                      f"512-scene draw, {n // steps} particles), one scene at a time on all threads, after one "
                      "warm-up step: the oracle's FP32 transcription of the reference's shader stages"}


def run_batch(args):
    """The 512-scene batched workload (4,096-65,536 particles per scene, log-uniform, seed 0):
    autotuned, then timed like the single-scene step; the scenes' SPH arithmetic is the plain
    step's, so the same algorithmic bytes per particle-step apply."""
    from watercube_gb300 import _abi
    from watercube_gb300.batch import Batch, batch_specs, scene_params, scene_particles
    from watercube_gb300.fluid import PinnedBuffer

    _abi.check(_abi.lib().wc_set_device(0), "select device")
    specs = batch_specs(512, 4096, 65536, seed=0)
    dt = 1e-3
    params = [scene_params(x) for x in specs]
    states = [scene_particles(x, q) for x, q in zip(specs, params)]
    b = Batch(params, states)
    n = b.num_particles
    t0 = time.perf_counter()
    tuning = b.tune(dt)
    tune_s = time.perf_counter() - t0
    warm = max(args.warmup, 3)
    b.step(dt, warm)
    with Clocks(0) as clocks:
        ms = b.time_steps(dt, args.steps, flush_l2=True)
    total_ms = float(ms.sum())
    d = b.diagnostics()
    value = n * args.steps / (total_ms * 1e-3)
    peak, peak_kind = measured_peaks()
    cells = sum(int(q.grid_res) ** 3 for q in params)
    step_gbs = step_algo_bytes(n, cells) * n / (total_ms / args.steps * 1e-3) / 1e9

    # end to end through the public API with host buffers (pinned), the same number of steps
    # from the same state: upload every scene's particles, step, read them back
    state0 = b.particles()
    nbytes = n * 32
    hin, hout = PinnedBuffer(nbytes), PinnedBuffer(nbytes)
    ain, aout = hin.particles(n), hout.particles(n)
    lib = _abi.lib()
    b.set_particles(states_concat(states))
    b.step(dt, warm)
    ain[:] = b.particles()
    e2e_steps = min(args.steps, 100)
    t = time.perf_counter()
    for _ in range(e2e_steps):
        _abi.check(lib.wc_batch_step_host(b._h, dt, ain.ctypes.data, aout.ctypes.data, n))
        ain, aout = aout, ain
    el = time.perf_counter() - t
    line = {
        "metric": "particle-steps/s, 512 batched scenes (plain SPH step)",
        "value": value,
        "unit": UNIT,
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "512 scenes, 4,096-65,536 particles each (log-uniform, seed 0), random blocks, "
                               "v ~ N(0, 0.5), k ~ U[2, 6], dt=1e-3", "particles": n, "cells": cells,
                   "window": f"steps {warm + 1} .. {warm + args.steps} from the initial states",
                   "l2": "flushed before every timed step (read of 2x L2), outside the timed span"},
        "roofline": {"bound": "hbm", "kernel": "whole step", "achieved": step_gbs, "peak": peak, "unit": "GB/s",
                     "frac": step_gbs / peak,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
                     "algorithmic_bytes_per_particle": step_algo_bytes(n, cells), "traffic": None},
        "tuning": {"density_blocks_per_sm": tuning.density_blocks_per_sm,
                   "force_blocks_per_sm": tuning.force_blocks_per_sm,
                   "stream_blocks_per_sm": tuning.stream_blocks_per_sm, "cell_factor": tuning.cell_factor,
                   "pass_variant": "lane per target" if tuning.pass_variant == _abi.WC_PASSES_LANE else "team per cell",
                   "trials": tuning.trials, "tune_seconds": tune_s},
        "e2e": {"value": n * e2e_steps / el, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": e2e_steps,
                "pattern": "wc_batch_step_host(pinned host in, pinned host out): upload, step, readback "
                           "overlapping the force pass"},
        "gpu_launches": 6 * args.steps,
        "clocks": clocks.summary(),
        "mass_total": float(d[:, 0].sum()),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = batch_cpu_baseline(specs, params, states, dt, os.cpu_count() or 1)
    del state0
    b.close()
    hin.free()
    hout.free()
    print(json.dumps(line))
    return 0


def states_concat(states):
    return np.concatenate(states)


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 1000 for the single scenes, 500 for batch512, 2000 for rollout1m; "
                         "the same for --impl reference)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["batch512", "rollout1m"], default="dam1m")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-rollout", action="store_true")
    ap.add_argument("--rollout-steps", type=int, default=200)
    ap.add_argument("--advance", type=int, default=0, help="untimed steps before the warm-up (single scenes)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.steps is None:
        # both arms default to the workload's own window, so that their configs agree (the
        # reference arm's 1,000 CPU steps of the 1M dam break take about two minutes on 16 cores)
        args.steps = {"batch512": 500, "rollout1m": 2000}.get(args.workload, 1000)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch512":
        return run_batch(args)
    if args.workload == "rollout1m":
        return run_rollout_workload(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
