"""C ABI checks that need no GPU: every declared symbol is exported, parameter presets and
derivation, generators (bit-exact with the oracle's restatement), and error behaviour."""
import ctypes as C
import math
import re
from pathlib import Path

import numpy as np
import pytest

from watercube_gb300 import _abi
from watercube_gb300.fluid import Fluid, dam_break_params, finalize, generate_dam_break, generate_reference_lattice, reference_params

HEADER = Path(__file__).resolve().parent.parent / "include" / "watercube.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"WC_API\s+[\w\s\*]+?\b(wc_\w+)\s*\(", text)))


def test_header_symbols_exported(wclib):
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(wclib, s)]
    assert not missing, missing


def test_build_info(wclib):
    assert b"sm_103a" in wclib.wc_build_info()


def test_reference_defaults():
    p = finalize(reference_params())
    assert p.num_particles == 80000 and p.grid_res == 21
    assert math.isclose(p.kernel_radius, 0.04, rel_tol=1e-6)  # 4 r
    assert math.isclose(p.particle_mass, 0.08, rel_tol=1e-6)  # 8 r
    assert p.bin_size == np.float32(1.0) / np.float32(21)
    h = float(p.kernel_radius)
    assert p.poly6_const == np.float32(315.0 / (64.0 * math.pi * h**9))
    assert p.spiky_const == np.float32(-45.0 / (math.pi * h**6))
    assert p.visc_const == np.float32(45.0 / (math.pi * h**6))
    assert list(p.gravity) == [0.0, -900.0, 0.0]
    assert math.isclose(p.time_scale, 0.012, rel_tol=1e-6)
    assert p.flags == _abi.WC_FLAGS_REFERENCE and p.eos == _abi.WC_EOS_DESBRUN_CUBIC


@pytest.mark.parametrize("n,h,R", [(16384, 0.0457, 21), (1048576, 0.011425, 87)])
def test_dam_break_presets(n, h, R):
    p = finalize(dam_break_params(n))
    assert math.isclose(p.kernel_radius, h, rel_tol=1e-6)
    assert p.grid_res == R
    assert p.bin_size >= p.kernel_radius
    assert math.isclose(p.particle_mass, 1000 * (h / 2) ** 3, rel_tol=1e-5)
    assert p.eos == _abi.WC_EOS_LINEAR and p.flags == 0
    assert p.rest_density == 1000 and p.stiffness == 3 and math.isclose(p.viscosity, 3.5)
    assert math.isclose(p.wall_damping, 0.5)


def test_finalize_rejects_bad_params(wclib):
    p = reference_params()
    p.size = 0.0
    with pytest.raises(_abi.WatercubeError) as e:
        finalize(p)
    assert e.value.status == _abi.WC_ERR_INVALID_ARG and "size" in str(e.value)
    p = reference_params()
    p.particle_radius = 0.0
    with pytest.raises(_abi.WatercubeError):
        finalize(p)
    p = reference_params()
    p.grid_res = 5000
    with pytest.raises(_abi.WatercubeError):
        finalize(p)


def test_cull_threshold_matches_oracle(wclib, oracle):
    for h in [0.04, 0.0457, 0.011425, 0.5]:
        assert np.float32(wclib.wc_cull_threshold(h)) == np.float32(oracle.cull_threshold(h))


@pytest.mark.parametrize("n,seed", [(16384, 0), (1000, 9), (3, 1)])
def test_generators_match_oracle(oracle, n, seed):
    p = finalize(dam_break_params(n))
    assert generate_dam_break(p, seed).tobytes() == oracle.generate_dam_break(p, seed).tobytes()
    q = reference_params()
    q.num_particles = n
    q = finalize(q)
    assert generate_reference_lattice(q, seed).tobytes() == oracle.generate_reference_lattice(q, seed).tobytes()


def test_fluid_api_state_errors(wclib):
    f = Fluid.create("fluid")
    assert f.numParticles() == 80000
    assert f.numParticles(100) is f
    with pytest.raises(_abi.WatercubeError) as e:
        f.update(0.016)
    assert e.value.status == _abi.WC_ERR_STATE


def test_null_arguments(wclib):
    assert wclib.wc_fluid_create(None, None) == _abi.WC_ERR_INVALID_ARG
    assert b"null" in wclib.wc_last_error()
    assert wclib.wc_fluid_update(None, 0.1) == _abi.WC_ERR_INVALID_ARG
    assert wclib.wc_fluid_synchronize(None) == _abi.WC_ERR_INVALID_ARG
    assert wclib.wc_status_string(_abi.WC_ERR_TIMEOUT) == b"device wait timed out"


def test_create_without_device_fails_cleanly(wclib):
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    p = dam_break_params(10)
    h = C.c_void_p()
    rc = wclib.wc_fluid_create(C.byref(p), C.byref(h))
    assert rc == _abi.WC_ERR_CUDA
    assert h.value is None
