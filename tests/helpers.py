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
    if name == "compressed16k":
        # A dense block (spacing 0.3 h: ~37 particles per cell, ~1,000 candidates) and a denser
        # one (0.2 h: ~125 per cell, ~3,400 candidates): candidate lists longer than the stage,
        # cells of more than 32 particles, bit strings kept in pieces and bit strings that do
        # not fit the slot -- every dense path of the two neighbour passes, beside the block
        # edges' ordinary cells.
        p = dam_break_params(16384)
        p.flags |= extra_flags
        p = finalize(p)
        st = generate_dam_break(p, 0)
        rng = np.random.default_rng(7)
        h = float(p.kernel_radius)

        def block(count, spacing, origin):
            k = int(np.ceil(count ** (1.0 / 3.0)))
            g = np.stack(np.meshgrid(*[np.arange(k)] * 3, indexing="ij"), -1).reshape(-1, 3)[:count]
            return origin + g * spacing + rng.uniform(-0.01 * h, 0.01 * h, (count, 3))

        st["position"] = np.concatenate([block(12000, 0.3 * h, 0.05), block(4384, 0.2 * h, 0.6)]).astype(np.float32)
        st["velocity"] = rng.normal(0.0, 0.2, (16384, 3)).astype(np.float32)
        return p, st
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
