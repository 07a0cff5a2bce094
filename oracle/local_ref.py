"""FP64 restatement of the learned fast rollout's quantities. TEST INFRASTRUCTURE ONLY: used by
tests/ to check the CUDA path, never by the solver.

  pair_sums    the judge step's pass sums per particle: the SPH acceleration (the update
               shader's pressure, viscosity and gravity terms, assets/fluid/update.comp:149-195),
               the Poly6 density rate -6 m c6 sum (cull - d2)^2 (r . (v_i - v_j)), and
               J = d a / dt of the pressure term when the positions move with their velocities
               and the densities and pressures follow them (the density pass's rates); the
               viscosity term's derivative is not in J. Neighbours are the pairs the solver's test
               selects (float32 d2 <= cull, the reference's |r| < h), evaluated in float64.
  inputs       the network's 19 inputs (unrounded).
  forward      the network with the BF16 roundings of the tensor-core path (inputs, weights and
               hidden activations rounded to BF16, sums in float64).
  gradients    the loss and the hand-written backward pass of the training step, with the same
               roundings (the BF16 operands of the GEMMs: output gradient, masked hidden gradients).
"""
from __future__ import annotations

import numpy as np

IN, HID, OUT = 32, 64, 16
OFF_W1 = 0
OFF_B1 = OFF_W1 + IN * HID
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID * OUT
NPARAMS = OFF_B3 + OUT


def bf16(x) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w: np.ndarray):
    w = np.asarray(w, np.float64)
    return (w[OFF_W1:OFF_B1].reshape(IN, HID), w[OFF_B1:OFF_W2], w[OFF_W2:OFF_B2].reshape(HID, HID), w[OFF_B2:OFF_W3],
            w[OFF_W3:OFF_B3].reshape(HID, OUT), w[OFF_B3:NPARAMS])


def neighbour_pairs(pos32: np.ndarray, h: float, cull: float):
    """(i, j) with i != j and float32 d2 <= cull (the solver's and the reference's neighbour test)."""
    from scipy.spatial import cKDTree

    tree = cKDTree(pos32.astype(np.float64))
    pairs = tree.query_pairs(h * (1.0 + 1e-5), output_type="ndarray")
    i = np.concatenate([pairs[:, 0], pairs[:, 1]])
    j = np.concatenate([pairs[:, 1], pairs[:, 0]])
    d = (pos32[i] - pos32[j]).astype(np.float32)
    d2 = np.float32(d[:, 2] * d[:, 2]) + (np.float32(d[:, 1] * d[:, 1]) + np.float32(d[:, 0] * d[:, 0]))
    keep = d2 <= np.float32(cull)
    return i[keep], j[keep]


def pair_sums(p, sorted_state: np.ndarray, cull: float):
    """Per particle of a sorted state (density and pressure from the density pass): the SPH
    acceleration, J and the density rate, all float64. The equation of state's dp/drho turns
    the density rate into the pressure rate (linear: k; cubic: 3 k rho^2 / rho0^3)."""
    x = sorted_state["position"].astype(np.float64)
    v = sorted_state["velocity"].astype(np.float64)
    rho = sorted_state["density"].astype(np.float64)
    pr = sorted_state["pressure"].astype(np.float64)
    n = x.shape[0]
    h = float(p.kernel_radius)
    m = float(p.particle_mass)
    fp_scale = -m * float(p.spiky_const)
    fv_scale = m * float(p.visc_const) * float(p.viscosity)
    c6 = float(p.poly6_const)
    i, j = neighbour_pairs(sorted_state["position"].astype(np.float32), h, cull)
    r = x[i] - x[j]
    d = np.linalg.norm(r, axis=1)
    inv_d = np.where(d > 0, 1.0 / np.where(d > 0, d, 1.0), 0.0)
    hd = h - d
    pres = (pr[i] + pr[j]) * 0.5 / rho[j]
    pos_p = pres > 0
    coef = np.where(pos_p, pres * hd * hd * inv_d, 0.0)
    u = v[i] - v[j]
    ru = np.einsum("ij,ij->i", r, u)
    dp = ru * inv_d
    dcoef = np.where(pos_p, -pres * hd * inv_d * (2.0 + hd * inv_d), 0.0)
    # the density pass's rates
    w = np.maximum(float(cull) - np.einsum("ij,ij->i", r, r), 0.0)
    rr = np.zeros(n)
    np.add.at(rr, i, w * w * ru)
    rate = -6.0 * m * c6 * rr
    rho0, k = float(p.rest_density), float(p.stiffness)
    dpdrho = np.full(n, k) if int(p.eos) == 1 else 3.0 * k * rho * rho / rho0**3  # 1: WC_EOS_LINEAR
    pdot = dpdrho * rate
    dpres = np.where(pos_p, (pdot[i] + pdot[j]) * 0.5 / rho[j] - pres * rate[j] / rho[j], 0.0)
    fp = np.zeros((n, 3))
    fv = np.zeros((n, 3))
    jp = np.zeros((n, 3))
    np.add.at(fp, i, coef[:, None] * r)
    np.add.at(fv, i, (v[j] - v[i]) * (hd / rho[j])[:, None])
    np.add.at(jp, i, (dcoef * dp + dpres * hd * hd * inv_d)[:, None] * r + coef[:, None] * u)
    g = np.array(list(p.gravity), np.float64)
    inv = 1.0 / (rho + 1e-16)
    pressure_acc = fp_scale * fp * inv[:, None]
    acc = pressure_acc + fv_scale * fv * inv[:, None] + g[None, :] * (rho * inv)[:, None]
    jerk = fp_scale * jp * inv[:, None] - (rate * inv)[:, None] * pressure_acc
    return acc, jerk, rate


def inputs(p, sorted_state: np.ndarray, acc, jerk, rate, dt: float = 1e-3, accel_scale: float = 10.0,
           velocity_scale: float = 1.0) -> np.ndarray:
    """The network's inputs [n, 32] (19 used), float64; J and the density rate enter times the
    network's time unit `dt` (1 ms, whatever the solver's time step)."""
    x = sorted_state["position"].astype(np.float64)
    v = sorted_state["velocity"].astype(np.float64)
    rho = sorted_state["density"].astype(np.float64)
    pr = sorted_state["pressure"].astype(np.float64)
    n = x.shape[0]
    h, size, rho0, k = float(p.kernel_radius), float(p.size), float(p.rest_density), float(p.stiffness)
    out = np.zeros((n, IN))
    out[:, 0:3] = acc / accel_scale
    out[:, 3:6] = jerk * dt / accel_scale
    out[:, 6] = 100.0 * rate * dt / rho
    out[:, 7:10] = v / velocity_scale
    out[:, 10] = rho / rho0 - 1.0
    out[:, 11] = pr / (k * rho0)
    walls = np.stack([x[:, 0], size - x[:, 0], x[:, 1], size - x[:, 1], x[:, 2], size - x[:, 2]], 1) / h
    out[:, 12:18] = np.clip(walls, 0.0, 1.0)
    out[:, 18] = 100.0 * k / rho0
    return out


def _round(rounding: bool):
    return bf16 if rounding else (lambda a: np.asarray(a, np.float64))


def forward(w: np.ndarray, x: np.ndarray, keep: bool = False, rounding: bool = True):
    """Outputs [n, 16] (units of accel_scale) of inputs x [n, 32] (BF16-rounded inside unless
    rounding is False: plain float64)."""
    R = _round(rounding)
    W1, b1, W2, b2, W3, b3 = unpack(w)
    xb = R(x)
    z1 = xb @ R(W1) + b1
    h1 = R(np.maximum(z1, 0.0))
    z2 = h1 @ R(W2) + b2
    h2 = R(np.maximum(z2, 0.0))
    y = h2 @ R(W3) + b3
    if keep:
        return y, (xb, h1, h2)
    return y


def gradients(w: np.ndarray, x: np.ndarray, y: np.ndarray, nout: int, rounding: bool = True):
    """(loss, gradient of every parameter) of the mean squared error over the first nout outputs."""
    bf = _round(rounding)
    W1, b1, W2, b2, W3, b3 = unpack(w)
    rows = x.shape[0]
    yp, (xb, h1, h2) = forward(w, x, keep=True, rounding=rounding)
    e = np.zeros_like(yp)
    e[:, :nout] = yp[:, :nout] - y[:, :nout]
    loss = float((e[:, :nout] ** 2).sum() / (rows * nout))
    dy = 2.0 * e / (rows * nout)
    dy16 = bf(dy)
    g = np.zeros(NPARAMS)
    g[OFF_W3:OFF_B3] = (h2.T @ dy16).ravel()
    g[OFF_B3:NPARAMS] = dy.sum(0)
    dh2 = dy16 @ bf(W3).T
    dz2 = np.where(h2 > 0, dh2, 0.0)
    dz2b = bf(dz2)
    g[OFF_W2:OFF_B2] = (h1.T @ dz2b).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    dh1 = dz2b @ bf(W2).T
    dz1 = np.where(h1 > 0, dh1, 0.0)
    dz1b = bf(dz1)
    g[OFF_W1:OFF_B1] = (xb.T @ dz1b).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    return loss, g


BLOCKS = {"W1": (OFF_W1, OFF_B1), "b1": (OFF_B1, OFF_W2), "W2": (OFF_W2, OFF_B2), "b2": (OFF_B2, OFF_W3),
          "W3": (OFF_W3, OFF_B3), "b3": (OFF_B3, NPARAMS)}
