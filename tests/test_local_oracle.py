"""The FP64 restatement of the learned fast rollout (oracle/local_ref.py), on the CPU: its
hand-written backward pass against central differences in plain float64, the BF16 rounding
helper, and its pair sums against finite differences of the SPH acceleration and density in time
(the definitions the force pass's feature output follows)."""
import numpy as np
import pytest

from oracle import local_ref as L


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2**-8, 1.0 + 2**-7, 1.0 + 3 * 2**-8, -2.5, 0.0], np.float32)
    r = L.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2**-7 and r[3] == 1.0 + 2**-6 and r[4] == -2.5 and r[5] == 0


def test_backward_matches_central_differences():
    rng = np.random.default_rng(0)
    w = rng.normal(0, 0.3, L.NPARAMS)
    x = rng.normal(0, 1, (24, L.IN))
    y = rng.normal(0, 1, (24, L.OUT))
    nout = 9
    loss, g = L.gradients(w, x, y, nout, rounding=False)
    eps = 1e-6
    for name, (a, b) in L.BLOCKS.items():
        idx = rng.choice(np.arange(a, b), size=min(6, b - a), replace=False)
        for k in idx:
            wp, wm = w.copy(), w.copy()
            wp[k] += eps
            wm[k] -= eps
            lp, _ = L.gradients(wp, x, y, nout, rounding=False)
            lm, _ = L.gradients(wm, x, y, nout, rounding=False)
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (name, k, fd, g[k])
    assert loss > 0


def test_pair_sums_are_the_time_derivatives():
    """J and the density rate are d/dt of the SPH acceleration's pair sums and of the Poly6
    density when positions move with their velocities and pressures and densities are held."""
    scipy = pytest.importorskip("scipy")
    del scipy
    from oracle.oracle import Oracle
    from watercube_gb300.fluid import dam_break_params, finalize, generate_dam_break

    o = Oracle()
    p = o.dam_break_params(4096)
    st = o.generate_dam_break(p, 0)
    st["velocity"] = np.random.default_rng(1).normal(0.0, 0.3, (4096, 3)).astype(np.float32)
    srt, _, _, counts, offsets = o.sort(p, st)
    o.density(p, srt, counts, offsets)
    from oracle.oracle import to64

    s64 = to64(srt)
    cull = o.cull_threshold(float(p.kernel_radius))
    acc, jerk, rate = L.pair_sums(p, s64, cull)
    tau = 1e-7
    moved = s64.copy()
    moved["position"] = s64["position"] + tau * s64["velocity"]
    acc2, _, _ = L.pair_sums(p, moved, cull)
    fd = (acc2 - acc) / tau
    # pairs near |r| = h may enter or leave the sum between the two states: compare the bulk
    err = np.linalg.norm(fd - jerk, axis=1)
    assert np.median(err) <= 1e-3 * np.median(np.linalg.norm(jerk, axis=1))
    # density rate against the FP64 oracle density of the moved state
    a64, b64 = s64.copy(), moved.copy()
    o.density(p, a64, counts, offsets)
    o.density(p, b64, counts, offsets)
    fdr = (b64["density"] - a64["density"]) / tau
    assert np.median(np.abs(fdr - rate)) <= 1e-3 * np.median(np.abs(rate))
