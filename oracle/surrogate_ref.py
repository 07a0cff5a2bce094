"""FP64 CPU restatement of the learned surrogate, for the gradient and prediction checks.

Test infrastructure only: the product never imports this module. The surrogate has no
counterpart in the reference (which runs plain SPH), so this oracle is not pinned to reference
outputs; it is an independent restatement of the network the CUDA path implements, evaluated in
float64 with torch autograd for the gradients.

Network (latent width 128, L message-passing steps), parameters in one flat FP32 vector in
this order (each block's weight is [in x out] row-major, then its bias):
    node encoder   ne1 32->128 (+b), ne2 128->128 (+b), LayerNorm (gamma, beta)
    edge encoder   ee1 16->128 (+b), ee2 128->128 (+b), LayerNorm
    L times:       e1e 128->128 (+b), e1i 128->128, e1s 128->128, e2 128->128 (+b), LayerNorm,
                   n1 256->128 (+b), n2 128->128 (+b), LayerNorm
    decoder        d1 128->128 (+b), d2 128->16 (+b)
    e' = e + LN(e2 relu(e1e e + e1i h_recv + e1s h_send + b))
    h' = h + LN(n2 relu(n1 [h | sum over in-edges of e'] + b))
    a  = accel_scale * d2 relu(d1 h)   (first 3 outputs)
Graph: ordered pairs (i, j), i != j, with d2 <= cull, d2 = fma(dz, dz, fma(dy, dy, dx * dx)) in
FP32 (cull = largest float whose square root is below h), edge features from receiver i to
sender j. Features: node = current velocity / velocity_scale, the four successive velocity
differences / (dt accel_scale) (FP32), 6 wall distances / h clipped to [0, 1], stiffness /
rest density * 200, the last SPH acceleration / accel_scale and its age in steps / 8 (zeros when
none is given), zeros to 32. With a stale acceleration the sample is residual: the loss target
is target - stale and the acceleration is stale + output (the caller subtracts and adds it); edge = (x_i - x_j) / h, |x_i - x_j| / h,
zeros to 16.

Emulated BF16 rounding: the CUDA path keeps features, weights and the stored activations in
BF16 (FP32 accumulation). The oracle rounds exactly those values to BF16 in the forward pass
(identity in the backward pass, as a straight-through estimator, since the CUDA path takes the
weight gradients with respect to the BF16 copies and the activation gradients through them);
everything else is float64.
"""
from __future__ import annotations

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover - torch is present wherever the tests run
    torch = None

W = 128
NODE_IN, EDGE_IN, OUT = 32, 16, 16


def layout(layers: int) -> list[tuple[str, tuple[int, ...]]]:
    """(name, shape) of every parameter block, in storage order."""
    out: list[tuple[str, tuple[int, ...]]] = []

    def lin(name, kin, nout, bias=True):
        out.append((name + ".w", (kin, nout)))
        if bias:
            out.append((name + ".b", (nout,)))

    def ln(name):
        out.append((name + ".g", (W,)))
        out.append((name + ".beta", (W,)))

    lin("ne1", NODE_IN, W)
    lin("ne2", W, W)
    ln("lnn0")
    lin("ee1", EDGE_IN, W)
    lin("ee2", W, W)
    ln("lne0")
    for l in range(layers):
        p = f"mp{l}."
        lin(p + "e1e", W, W)
        lin(p + "e1i", W, W, bias=False)
        lin(p + "e1s", W, W, bias=False)
        lin(p + "e2", W, W)
        ln(p + "lne")
        lin(p + "n1", 2 * W, W)
        lin(p + "n2", W, W)
        ln(p + "lnn")
    lin("d1", W, W)
    lin("d2", W, OUT)
    return out


def num_params(layers: int) -> int:
    return int(sum(int(np.prod(s)) for _, s in layout(layers)))


def unflatten(flat: np.ndarray, layers: int) -> dict[str, np.ndarray]:
    out, off = {}, 0
    for name, shape in layout(layers):
        size = int(np.prod(shape))
        out[name] = flat[off:off + size].reshape(shape)
        off += size
    assert off == flat.size, (off, flat.size)
    return out


def flatten(blocks: dict, layers: int) -> np.ndarray:
    return np.concatenate([np.asarray(blocks[name], np.float64).reshape(-1) for name, _ in layout(layers)])


def radius_graph(pos: np.ndarray, cull: float) -> tuple[np.ndarray, np.ndarray]:
    """(recv, send) of every ordered pair within the cull distance, FP32 distance as the solver
    computes it (fma emulated exactly: a float32 square is exact in float64)."""
    p = np.asarray(pos, np.float32)
    dx = (p[:, None, 0] - p[None, :, 0]).astype(np.float32)
    dy = (p[:, None, 1] - p[None, :, 1]).astype(np.float32)
    dz = (p[:, None, 2] - p[None, :, 2]).astype(np.float32)
    d2 = (dx * dx).astype(np.float32)
    d2 = (dy.astype(np.float64) ** 2 + d2.astype(np.float64)).astype(np.float32)
    d2 = (dz.astype(np.float64) ** 2 + d2.astype(np.float64)).astype(np.float32)
    hit = d2 <= np.float32(cull)
    np.fill_diagonal(hit, False)
    recv, send = np.nonzero(hit)
    return recv.astype(np.int64), send.astype(np.int64)


def node_features(pos, hist, size, h, k_feature, velocity_scale, dt, accel_scale, stale=None,
                  stale_age: int = 0) -> np.ndarray:
    pos = np.asarray(pos, np.float32)
    n = pos.shape[0]
    f = np.zeros((n, NODE_IN), np.float32)
    inv_v = np.float32(1.0) / np.float32(velocity_scale)
    inv_dv = np.float32(1.0) / (np.float32(dt) * np.float32(accel_scale))
    v = [np.asarray(hist[s][:, :3], np.float32) for s in range(5)]
    f[:, 0:3] = v[0] * inv_v
    for s in range(1, 5):
        f[:, 3 * s:3 * s + 3] = (v[s - 1] - v[s]) * inv_dv
    inv_h = np.float32(1.0) / np.float32(h)
    walls = [pos[:, 0], np.float32(size) - pos[:, 0], pos[:, 1], np.float32(size) - pos[:, 1], pos[:, 2],
             np.float32(size) - pos[:, 2]]
    for a, w in enumerate(walls):
        f[:, 15 + a] = np.clip(w.astype(np.float32) * inv_h, 0.0, 1.0)
    f[:, 21] = np.float32(k_feature)
    if stale is not None and stale_age > 0:
        inv_a = np.float32(1.0) / np.float32(accel_scale)
        f[:, 22:25] = np.asarray(stale, np.float32)[:, :3] * inv_a
        f[:, 25] = np.float32(stale_age) * np.float32(0.125)
    return f


def edge_features(pos, recv, send, h) -> np.ndarray:
    pos = np.asarray(pos, np.float32)
    inv_h = np.float32(1.0) / np.float32(h)
    d = (pos[recv] - pos[send]).astype(np.float32) * inv_h
    f = np.zeros((recv.size, EDGE_IN), np.float32)
    f[:, :3] = d
    f[:, 3] = np.sqrt((d.astype(np.float64) ** 2).sum(1))
    return f


def _bf(x):
    """Round to BF16 in the forward pass, identity in the backward pass."""
    return x + (x.to(torch.bfloat16).to(torch.float64) - x).detach()


def _ln(y, g, b):
    mu = y.mean(1, keepdim=True)
    var = ((y - mu) ** 2).mean(1, keepdim=True)
    return (y - mu) / torch.sqrt(var + 1e-5) * g + b


class Net:
    """The surrogate in float64 (torch), parameters as leaf tensors named as in `layout`."""

    def __init__(self, flat: np.ndarray, layers: int, drop_sender_grad: bool = False, bf16: bool = True):
        if torch is None:
            raise RuntimeError("the surrogate oracle needs torch")
        self.layers = layers
        self.bf16 = bf16  # False: plain float64 (for checking the autograd itself)
        blocks = unflatten(np.asarray(flat, np.float64), layers)
        self.p = {k: torch.tensor(v, dtype=torch.float64, requires_grad=True) for k, v in blocks.items()}
        # planted mistake for the sensitivity test: no gradient through the sender term
        self.drop_sender_grad = drop_sender_grad

    def w(self, name):
        return self.r(self.p[name + ".w"])

    def r(self, x):
        return _bf(x) if self.bf16 else x

    def forward(self, xn: np.ndarray, xe: np.ndarray, recv: np.ndarray, send: np.ndarray):
        P = self.p
        _bf = self.r
        n = xn.shape[0]
        x = _bf(torch.tensor(xn, dtype=torch.float64))
        xe_t = _bf(torch.tensor(xe, dtype=torch.float64))
        recv_t = torch.tensor(recv, dtype=torch.int64)
        send_t = torch.tensor(send, dtype=torch.int64)
        z = _bf(torch.relu(x @ self.w("ne1") + P["ne1.b"]))
        h = _bf(_ln(z @ self.w("ne2") + P["ne2.b"], P["lnn0.g"], P["lnn0.beta"]))
        z = _bf(torch.relu(xe_t @ self.w("ee1") + P["ee1.b"]))
        e = _bf(_ln(z @ self.w("ee2") + P["ee2.b"], P["lne0.g"], P["lne0.beta"]))
        for l in range(self.layers):
            p = f"mp{l}."
            hi = _bf(h @ self.w(p + "e1i"))
            hs = _bf(h @ self.w(p + "e1s"))
            if self.drop_sender_grad:
                hs = hs.detach()
            ze = _bf(torch.relu(e @ self.w(p + "e1e") + P[p + "e1e.b"] + hi[recv_t] + hs[send_t]))
            e = _bf(e + _ln(ze @ self.w(p + "e2") + P[p + "e2.b"], P[p + "lne.g"], P[p + "lne.beta"]))
            agg = torch.zeros((n, W), dtype=torch.float64).index_add(0, recv_t, e)
            agg = _bf(agg)
            zn = _bf(torch.relu(torch.cat([h, agg], 1) @ self.w(p + "n1") + P[p + "n1.b"]))
            h = _bf(h + _ln(zn @ self.w(p + "n2") + P[p + "n2.b"], P[p + "lnn.g"], P[p + "lnn.beta"]))
        zd = _bf(torch.relu(h @ self.w("d1") + P["d1.b"]))
        return zd @ self.w("d2") + P["d2.b"]  # [n x 16], normalised accelerations

    def loss_and_grads(self, xn, xe, recv, send, target: np.ndarray, accel_scale: float):
        """Mean squared error over 3 components of (output - target / accel_scale), and its
        gradient as a flat vector in storage order."""
        out = self.forward(xn, xe, recv, send)
        t = torch.tensor(np.asarray(target, np.float64)[:, :3] / accel_scale, dtype=torch.float64)
        loss = ((out[:, :3] - t) ** 2).mean()
        loss.backward()
        loss = loss.detach()
        grads = {k: (v.grad.numpy() if v.grad is not None else np.zeros(v.shape)) for k, v in self.p.items()}
        return float(loss), flatten(grads, self.layers), out.detach().numpy()[:, :3] * accel_scale


def cull_threshold(h: float) -> np.float32:
    """Largest float32 x with sqrtf(x) < h (IEEE square root is correctly rounded)."""
    h = np.float32(h)
    x = np.float32(h * h)
    while np.sqrt(x) >= h:
        x = np.nextafter(x, np.float32(0))
    while np.sqrt(np.nextafter(x, np.float32(np.inf))) < h:
        x = np.nextafter(x, np.float32(np.inf))
    return x


def sample_inputs(state: np.ndarray, hist: np.ndarray, params, velocity_scale: float, dt: float, accel_scale: float,
                  stale=None, stale_age: int = 0):
    """Graph and features of one sample (state: PARTICLE_DTYPE, hist: (5, n, 4), stale: (n, 4) or
    None), as the CUDA path builds them from the same particles."""
    pos = np.asarray(state["position"], np.float32)
    cull = cull_threshold(params.kernel_radius)
    recv, send = radius_graph(pos, cull)
    k_feature = np.float32(params.stiffness) / np.float32(params.rest_density) * np.float32(200.0)
    xn = node_features(pos, hist, params.size, params.kernel_radius, k_feature, velocity_scale, dt, accel_scale,
                       stale, stale_age)
    xe = edge_features(pos, recv, send, params.kernel_radius)
    return xn, xe, recv, send
