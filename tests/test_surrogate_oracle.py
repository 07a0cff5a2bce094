"""The surrogate's FP64 oracle on its own (no GPU): parameter layout, graph and features, and that
the gradient comparison of tests/test_gpu_surrogate.py would catch a missing backward term."""
import numpy as np
import pytest

from oracle import surrogate_ref as R
from watercube_gb300.fluid import dam_break_params, finalize

torch = pytest.importorskip("torch")

BLOCK_TOL = 3e-2  # the GPU test's per-block bound


def test_layout_sizes():
    lin = lambda k, n, b=True: k * n + (n if b else 0)  # noqa: E731
    ln = 2 * 128
    per_layer = lin(128, 128) + 2 * lin(128, 128, False) + lin(128, 128) + ln + lin(256, 128) + lin(128, 128) + ln
    enc = lin(32, 128) + lin(128, 128) + ln + lin(16, 128) + lin(128, 128) + ln
    dec = lin(128, 128) + lin(128, 16)
    for L in (1, 8):
        assert R.num_params(L) == enc + L * per_layer + dec
    w = np.arange(R.num_params(2), dtype=np.float64)
    assert np.array_equal(R.flatten(R.unflatten(w, 2), 2), w)


def test_cull_threshold_matches_solver_oracle(oracle):
    for h in (0.0457, 0.011425, 0.04, 0.0213):
        assert R.cull_threshold(h) == np.float32(oracle.cull_threshold(h))


def test_radius_graph():
    rng = np.random.default_rng(0)
    pos = rng.uniform(0.0, 0.2, (400, 3)).astype(np.float32)
    h = 0.03
    recv, send = R.radius_graph(pos, R.cull_threshold(h))
    assert np.all(recv != send)
    pairs = set(zip(recv.tolist(), send.tolist()))
    assert all((j, i) in pairs for i, j in pairs)  # symmetric
    d = np.sqrt(((pos[:, None, :].astype(np.float64) - pos[None, :, :]) ** 2).sum(-1))
    within = (d < h) & ~np.eye(len(pos), dtype=bool)
    near = np.abs(d - h) < 1e-6  # FP32 rounding may decide these either way
    got = np.zeros_like(within)
    got[recv, send] = True
    assert np.all((got == within) | near)
    assert np.all(recv[1:] >= recv[:-1])  # receiver-major, like the CSR of the CUDA path


def test_features():
    p = finalize(dam_break_params(64))
    pos = np.array([[0.0, 0.5, 0.02], [0.99, 0.01, 0.5]], np.float32)
    hist = np.zeros((5, 2, 4), np.float32)
    hist[0, :, :3] = [[1.0, -2.0, 0.5], [0.0, 0.0, 3.0]]
    hist[1, :, :3] = [[0.99, -2.0, 0.5], [0.0, 0.01, 3.0]]
    xn = R.node_features(pos, hist, 1.0, p.kernel_radius, 7.0, 2.0, 1e-3, 10.0)
    assert xn.shape == (2, 32)
    assert np.allclose(xn[0, :3], [0.5, -1.0, 0.25])
    assert np.allclose(xn[0, 3:6], [1.0, 0.0, 0.0], atol=1e-4)  # (v0 - v1) / (dt a_scale)
    assert np.allclose(xn[1, 3:6], [0.0, -1.0, 0.0], atol=1e-4)
    assert np.allclose(xn[:, 6:9], hist[1, :, :3] * 100.0, rtol=1e-5)  # v1 - v2 with v2 = 0
    assert np.all(xn[:, 9:15] == 0.0)  # v2 - v3 = v3 - v4 = 0
    assert xn[0, 15] == 0.0 and xn[0, 16] == 1.0  # at the x = 0 wall; far from x = size
    assert xn[1, 16] == pytest.approx(0.01 / p.kernel_radius, rel=1e-5) or xn[1, 16] == 1.0
    assert np.all(xn[:, 21] == 7.0) and np.all(xn[:, 22:] == 0.0)
    xe = R.edge_features(pos, np.array([0]), np.array([1]), 0.5)
    d = (pos[0] - pos[1]) / np.float32(0.5)
    assert np.allclose(xe[0, :3], d) and xe[0, 3] == pytest.approx(np.linalg.norm(d), rel=1e-6)


def small_case(layers, n=300, seed=0):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0.0, 0.25, (n, 3)).astype(np.float32)
    hist = rng.normal(0.0, 0.3, (5, n, 4)).astype(np.float32)
    h = 0.05
    recv, send = R.radius_graph(pos, R.cull_threshold(h))
    xn = R.node_features(pos, hist, 1.0, h, 0.6, 1.0, 1e-3, 10.0)
    xe = R.edge_features(pos, recv, send, h)
    target = rng.normal(0.0, 5.0, (n, 4)).astype(np.float32)
    w = rng.normal(0.0, 0.08, R.num_params(layers))
    return xn, xe, recv, send, target, w


def block_errors(g, ref, layers):
    out, off = {}, 0
    for name, shape in R.layout(layers):
        size = int(np.prod(shape))
        a, b = g[off:off + size], ref[off:off + size]
        off += size
        out[name] = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
    return out


def test_planted_backward_mistake_is_caught():
    """Dropping the sender-side gradient (the reverse-edge segment sum of the CUDA backward)
    changes the sender weights' gradient far beyond the GPU test's tolerance."""
    layers = 2
    xn, xe, recv, send, target, w = small_case(layers)
    _, good, _ = R.Net(w, layers).loss_and_grads(xn, xe, recv, send, target, 10.0)
    _, bad, _ = R.Net(w, layers, drop_sender_grad=True).loss_and_grads(xn, xe, recv, send, target, 10.0)
    err = block_errors(bad, good, layers)
    assert err["mp0.e1s.w"] > 10 * BLOCK_TOL
    assert err["mp1.e1s.w"] > 10 * BLOCK_TOL
    assert err["d2.w"] == 0.0  # the last layer does not see the mistake


def test_oracle_gradient_matches_finite_differences():
    """The oracle's autograd against central differences of its own loss, in plain float64 (the
    BF16 emulation makes the loss piecewise constant, so it is switched off here)."""
    layers = 1
    xn, xe, recv, send, target, w = small_case(layers, n=120, seed=3)
    loss, g, _ = R.Net(w, layers, bf16=False).loss_and_grads(xn, xe, recv, send, target, 10.0)
    names = dict()
    off = 0
    for name, shape in R.layout(layers):
        names[name] = (off, int(np.prod(shape)))
        off += int(np.prod(shape))
    rng = np.random.default_rng(1)
    for name in ("d2.b", "d1.b", "mp0.lnn.g", "mp0.e2.b", "lne0.beta", "mp0.e1s.w", "mp0.e1i.w", "mp0.n1.w",
                 "ee1.w", "ne1.w"):
        o, size = names[name]
        for idx in rng.choice(size, 3, replace=False):
            k = o + idx
            if name == "d2.b" and idx >= 3:
                continue
            eps = 1e-6
            wp, wm = w.copy(), w.copy()
            wp[k] += eps
            wm[k] -= eps
            fp = R.Net(wp, layers, bf16=False).loss_and_grads(xn, xe, recv, send, target, 10.0)[0]
            fm = R.Net(wm, layers, bf16=False).loss_and_grads(xn, xe, recv, send, target, 10.0)[0]
            fd = (fp - fm) / (2 * eps)
            assert fd == pytest.approx(g[k], rel=2e-3, abs=1e-7), (name, idx)
