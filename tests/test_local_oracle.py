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
    """J and the density rate are d/dt of the SPH acceleration's pressure term and of the Poly6
    density when the positions move with their velocities and the density pass recomputes the
    densities and pressures of the moved state: finite differences of the FP64 oracle's density
    pass and of the pair sums without viscosity (J leaves the viscosity term's derivative out),
    for both equations of state."""
    scipy = pytest.importorskip("scipy")
    del scipy
    from oracle.oracle import Oracle, to64

    o = Oracle()
    for eos in (1, 0):  # WC_EOS_LINEAR, WC_EOS_DESBRUN_CUBIC
        p = o.dam_break_params(4096)
        p.eos = eos
        p.viscosity = 0.0
        st = o.generate_dam_break(p, 0)
        st["velocity"] = np.random.default_rng(1).normal(0.0, 0.3, (4096, 3)).astype(np.float32)
        srt, _, _, counts, offsets = o.sort(p, st)
        s64 = to64(srt)
        o.density(p, s64, counts, offsets)
        cull = o.cull_threshold(float(p.kernel_radius))
        acc, jerk, rate = L.pair_sums(p, s64, cull)
        tau = 1e-7
        moved = s64.copy()
        moved["position"] = s64["position"] + tau * s64["velocity"]
        o.density(p, moved, counts, offsets)  # a move this small keeps every particle in its cell
        fdr = (moved["density"] - s64["density"]) / tau
        assert np.median(np.abs(fdr - rate)) <= 1e-3 * np.median(np.abs(rate)), eos
        acc2, _, _ = L.pair_sums(p, moved, cull)
        fd = (acc2 - acc) / tau
        # pairs near |r| = h may enter or leave the sum between the two states: compare the bulk
        err = np.linalg.norm(fd - jerk, axis=1)
        assert np.median(err) <= 1e-3 * np.median(np.linalg.norm(jerk, axis=1)), eos
