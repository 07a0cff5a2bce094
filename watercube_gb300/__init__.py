"""GB300 SPH water solver: the WaterCube simulation path (core::Fluid + core::Sort and their
compute shaders) as hand-written sm_103a CUDA behind a C ABI (include/watercube.h)."""
from ._abi import PARTICLE_DTYPE, Params, WatercubeError  # noqa: F401
from .fluid import (  # noqa: F401
    Fluid,
    PinnedBuffer,
    dam_break_params,
    finalize,
    generate_dam_break,
    generate_reference_lattice,
    reference_params,
)
from .batch import Batch, batch_specs, scene_params, scene_particles, shard_scenes  # noqa: F401,E402
