"""Shared builders for the tests: parameter sets and initial states of the two dam-break sizes,
the reference's defaults, and the reference's physics on the dam-break block."""
import numpy as np

from watercube_gb300 import _abi
from watercube_gb300.fluid import Fluid, dam_break_params, finalize, generate_dam_break, generate_reference_lattice, reference_params


def reference_physics(p: _abi.Params) -> _abi.Params:
    """The reference shader's behaviour on any geometry: cubic EOS, wall density and force,
    speed clamp 50, mouse force, damping 0.3 and border 0.001 (update.comp:5,202-203)."""
    p.eos = _abi.WC_EOS_DESBRUN_CUBIC
    p.flags |= _abi.WC_FLAGS_REFERENCE
    p.max_speed = 50.0
    p.wall_damping = 0.3
    p.wall_border = 0.001
    return p


def case(name: str, extra_flags: int = 0):
    """(finalized params, initial state) of a named workload."""
    if name == "dam16k":
        p = dam_break_params(16384)
        p.flags |= extra_flags
        p = finalize(p)
        return p, generate_dam_break(p, 0)
    if name == "dam1m":
        p = dam_break_params(1048576)
        p.flags |= extra_flags
        p = finalize(p)
        return p, generate_dam_break(p, 0)
    if name == "dam16k_walls":
        p = dam_break_params(16384)
        p.flags |= _abi.WC_FLAG_WALL_WEIGHTS | extra_flags
        p = finalize(p)
        return p, generate_dam_break(p, 0)
    if name == "refdefaults":
        p = reference_params()
        p.flags |= extra_flags
        p = finalize(p)
        return p, generate_reference_lattice(p, 0)
    if name == "dam16k_refphysics":
        p = reference_physics(dam_break_params(16384))
        p.stiffness = 100.0
        p.flags |= extra_flags
        p = finalize(p)
        return p, generate_dam_break(p, 0)
    raise KeyError(name)


def fluid(p, state) -> Fluid:
    f = Fluid.create("fluid", p)
    f.setup(state)
    return f


def by_input_index(values: np.ndarray, perm: np.ndarray) -> np.ndarray:
    """values[k] belongs to input particle perm[k]; return them in input order."""
    out = np.empty_like(values)
    out[perm] = values
    return out


def evolved(name: str, steps: int, dt: float, extra_flags: int = 0):
    """A state after `steps` GPU steps (velocities and pressures non-trivial)."""
    p, st = case(name, extra_flags)
    with fluid(p, st) as f:
        f.step(dt, steps)
        return p, f.particles()
