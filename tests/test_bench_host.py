"""bench.py's host-side pieces without a GPU: the reference arm's JSON line (the reference's CPU
implementation of the step on a small workload) and the CPU baseline over sampled states."""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_its_line():
    r = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--workload", "dam16k",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["steps"] == 2
    assert line["unit"] == "particle-steps/s" and line["higher_is_better"] is True
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_cpu_baseline_averages_sampled_states():
    sys.path.insert(0, str(REPO))
    import bench
    from watercube_gb300.fluid import dam_break_params, finalize, generate_dam_break

    p = finalize(dam_break_params(4096))
    st = generate_dam_break(p, 0)
    moved = st.copy()
    moved["velocity"] = 0.1
    out = bench.cpu_baseline(p, [(0, st), (10, moved)], 1e-3, 2)
    assert out["kind"] == "port" and out["cores"] == 2 and out["value"] > 0 and out["value_1thread"] > 0
    assert len(out["ms_per_step_by_state"]) == 2 and "window steps 0, 10" in out["sample"]
    assert np.isclose(out["value"], 4096 / (np.mean(out["ms_per_step_by_state"]) * 1e-3), rtol=1e-2)


def test_reference_arm_loads_no_solver_library():
    """The reference arm takes its parameters and initial lattice from the oracle library: the
    process never maps libwatercube.so, and its config equals the GPU arm's for the same window."""
    code = (
        "import argparse, json, sys; sys.path.insert(0, '.'); import bench\n"
        "a = argparse.Namespace(workload='dam16k', steps=1, warmup=3, advance=0, gpus=1)\n"
        "bench.run_reference(a)\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'loaded': 'libwatercube' in maps}))\n"
    )
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.strip().splitlines()]
    assert lines[-1] == {"loaded": False}
    sys.path.insert(0, str(REPO))
    import bench

    assert lines[0]["config"] == bench.workload_config("dam16k", 16384, lines[0]["config"]["grid_res"], 1e-3, 4, 4, 1)


def test_oracle_params_equal_the_solver_params():
    from oracle.oracle import Oracle
    from watercube_gb300.fluid import dam_break_params, finalize

    o = Oracle()
    for n in (1, 4096, 16384, 1048576):
        a = o.dam_break_params(n)
        b = finalize(dam_break_params(n))
        assert bytes(a) == bytes(b), n
