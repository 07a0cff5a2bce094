"""Generate the golden fixtures in this directory from the reference itself.

The reference's compute shaders (assets/sort/*.comp, assets/fluid/{density,update}.comp) are
compiled as C++ by oracle/ref/make_ref.py and driven in the reference's dispatch order
(oracle/ref/ref_driver.cpp). For each case this script stores the input state, the parameters
(raw wc_params bytes) and the reference's outputs of every stage:

  sort:    sorted particles (reorder.comp), permutation (sort.comp), counts, offsets
  density: the sorted buffer after density.comp (density + pressure)
  update:  the state after update.comp
  steps:   the state after K full Fluid::update steps

Run in a checkout next to the reference: python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle.oracle import RefLib, build_ref  # noqa: E402
from watercube_gb300 import _abi  # noqa: E402
from watercube_gb300.fluid import dam_break_params, finalize, generate_dam_break, generate_reference_lattice, reference_params  # noqa: E402


def params_bytes(p: _abi.Params) -> np.ndarray:
    return np.frombuffer(C.string_at(C.addressof(p), C.sizeof(p)), dtype=np.uint8).copy()


def make_case(ref: RefLib, name: str, p: _abi.Params, state: np.ndarray, dt: float, ksteps: int) -> None:
    sorted_, perm, counts, offsets = ref.sort(p, state)
    dens = sorted_.copy()
    ref.density(p, dens, counts, offsets)
    upd = ref.update(p, dens, counts, offsets, dt)
    stepped = state.copy()
    ref.step(p, stepped, dt, ksteps)
    np.savez_compressed(
        HERE / f"{name}.npz",
        params=params_bytes(p),
        state=state,
        dt=np.float32(dt),
        ksteps=np.int32(ksteps),
        sorted=sorted_,
        perm=perm,
        counts=counts,
        offsets=offsets,
        density=dens,
        update=upd,
        stepped=stepped,
    )
    print(f"{name}: n={state.shape[0]} R={p.grid_res} -> {HERE / (name + '.npz')}")


def main() -> None:
    lib = build_ref()
    if lib is None:
        raise SystemExit("reference shaders not found (set WC_REFERENCE_ROOT)")
    ref = RefLib(lib)

    # 1. The reference's own defaults (Fluid.cpp:9-27) at 1,500 particles, its lattice.
    p = reference_params()
    p.num_particles = 1500
    p = finalize(p)
    make_case(ref, "ref_defaults_n1500", p, generate_reference_lattice(p, 0), dt=0.012 / 60.0, ksteps=5)

    # 2. The dam-break block at 2,000 particles with the reference's physics switched on
    #    (cubic EOS, wall density and force, speed clamp, mouse force) so the shaders apply.
    p = dam_break_params(2000)
    p.eos = _abi.WC_EOS_DESBRUN_CUBIC
    p.flags = _abi.WC_FLAGS_REFERENCE
    p.stiffness = 100.0
    p.gravity[1] = -900.0
    p.wall_damping = 0.3  # update.comp:202-203 hard-code these two
    p.wall_border = 0.001
    p = finalize(p)
    make_case(ref, "dam_refphysics_n2000", p, generate_dam_break(p, 7), dt=2.0e-4, ksteps=4)

    # 3. A mouse ray through the box (update.comp:116-132 active), 800 particles.
    p = reference_params()
    p.num_particles = 800
    p.mouse_origin[:] = [0.1, 0.05, -1.0]
    p.mouse_dir[:] = [0.0, 0.0, 1.0]
    p = finalize(p)
    st = generate_reference_lattice(p, 3)
    st["velocity"][:] = np.random.default_rng(3).normal(0.0, 0.5, size=(800, 3)).astype(np.float32)
    make_case(ref, "mouse_ray_n800", p, st, dt=2.0e-4, ksteps=3)


if __name__ == "__main__":
    main()
