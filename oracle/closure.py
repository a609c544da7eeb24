"""CPU oracle of the learned subgrid closure (test infrastructure only).

A numpy restatement, in binary64 with the network's bfloat16 roundings
emulated, of the project's closure (no counterpart in the reference): the nine
inputs, the 9 -> 32 -> 32 -> 1 forward pass, its mean-squared-error gradients,
one Adam step, and the training data of a fine run (2x2x2 box filter, subgrid
stress, finite-difference strain, wall distance, target c*).  The GPU kernels
compute in binary32 with the hardware tanh approximation, so comparisons use
tolerances.
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID = 9, 32
W1, B1 = 0, N_HID * N_IN
W2 = B1 + N_HID
B2 = W2 + N_HID * N_HID
W3 = B2 + N_HID
B3 = W3 + N_HID
N_PARAMS = B3 + 1
WALL_CAP = 8.0


def bf16(a):
    """Round binary32 values to bfloat16 (nearest, ties to even), as binary64."""
    f = np.ascontiguousarray(np.asarray(a, np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    out = r.view(np.float32).astype(np.float64)
    nan = np.isnan(f)
    out[nan] = np.nan
    return out


def unpack(w):
    w = np.asarray(w, np.float64)
    return (w[W1:B1].reshape(N_HID, N_IN), w[B1:W2], w[W2:B2].reshape(N_HID, N_HID), w[B2:W3], w[W3:B3], w[B3])


def features(s, rho, ux, uy, uz, wall, nu0, nu_s, u_in):
    """The nine inputs (pw_closure.cuh `features`); s is (N, 6): xx, yy, zz, xy, xz, yz."""
    s = np.asarray(s, np.float64)
    a, b, c, d, e, f = (s[:, k] for k in range(6))
    ss = a * a + b * b + c * c + 2 * (d * d + e * e + f * f)
    off = 2 * (d * d + e * e + f * f)
    t3 = a ** 3 + b ** 3 + c ** 3 + 3 * ((a + b) * d * d + (a + c) * e * e + (b + c) * f * f) + 6 * d * e * f
    mag = np.sqrt(2 * ss)
    uu = np.sqrt(ux * ux + uy * uy + uz * uz)
    x = np.empty((len(a), N_IN))
    x[:, 0] = 100 * mag
    x[:, 1] = t3 / (ss * np.sqrt(ss) + 1e-30)
    x[:, 2] = off / (ss + 1e-30)
    x[:, 3] = uu / u_in
    x[:, 4] = ux / u_in
    x[:, 5] = 0.1 * (rho - 1) / (u_in * u_in)
    x[:, 6] = np.minimum(wall, WALL_CAP) / WALL_CAP
    x[:, 7] = 10 * nu_s / nu0
    x[:, 8] = 200 * nu0
    return x


def forward(w, X):
    w1, b1, w2, b2, w3, b3 = unpack(w)
    xb = bf16(X)
    h1 = bf16(np.tanh(xb @ bf16(w1).T + b1))
    h2 = bf16(np.tanh(h1 @ bf16(w2).T + b2))
    out = h2 @ bf16(w3) + b3
    return out, (xb, h1, h2)


def gradients(w, X, Y):
    """Mean squared error and its parameter gradients; the bfloat16 roundings
    pass gradients unchanged and tanh' is 1 - h^2 of the rounded activation."""
    w1, b1, w2, b2, w3, b3 = unpack(w)
    out, (xb, h1, h2) = forward(w, X)
    n = len(Y)
    err = out - np.asarray(Y, np.float64)
    d3 = 2 * err / n
    d2 = (d3[:, None] * bf16(w3)[None, :]) * (1 - h2 * h2)
    d1 = (d2 @ bf16(w2)) * (1 - h1 * h1)
    g = np.zeros(N_PARAMS)
    g[W1:B1] = (d1.T @ xb).reshape(-1)
    g[B1:W2] = d1.sum(0)
    g[W2:B2] = (d2.T @ h1).reshape(-1)
    g[B2:W3] = d2.sum(0)
    g[W3:B3] = h2.T @ d3
    g[B3] = d3.sum()
    return float(np.mean(err * err)), g


def adam(w, m, v, g, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    w = w - lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
    return w, m, v


# ---------------------------------------------------------------- training data
def coarsen(macros, walls, dims):
    """2x2x2 means of rho and u, the subgrid stress mean((u - ubar)(u - ubar)),
    and the any-wall mask, on the coarse grid."""
    nx, ny, nz = dims
    m = np.asarray(macros, np.float64).reshape(nz, ny, nx, 4)
    w = np.asarray(walls, bool).reshape(nz, ny, nx)

    def box(a):
        return a.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2).mean(axis=(1, 3, 5))

    rho, ux, uy, uz = (m[..., k] for k in range(4))
    means = [box(rho), box(ux), box(uy), box(uz)]

    def spread(a):
        return np.repeat(np.repeat(np.repeat(a, 2, axis=0), 2, axis=1), 2, axis=2)

    dx, dy, dz = ux - spread(means[1]), uy - spread(means[2]), uz - spread(means[3])
    q = means + [box(dx * dx), box(dy * dy), box(dz * dz), box(dx * dy), box(dx * dz), box(dy * dz)]
    solid = w.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2).any(axis=(1, 3, 5))
    return q, solid


def wall_distance(solid, cap_steps=8):
    """6-neighbour steps to the nearest wall (x bounded, y and z periodic), as the
    kernel's eight relaxation passes compute it."""
    d = np.where(solid, 0, 255).astype(np.int64)
    for _ in range(cap_steps):
        e = d.copy()
        e[:, :, 1:] = np.minimum(e[:, :, 1:], d[:, :, :-1] + 1)
        e[:, :, :-1] = np.minimum(e[:, :, :-1], d[:, :, 1:] + 1)
        e = np.minimum(e, np.roll(d, 1, axis=1) + 1)
        e = np.minimum(e, np.roll(d, -1, axis=1) + 1)
        e = np.minimum(e, np.roll(d, 1, axis=0) + 1)
        e = np.minimum(e, np.roll(d, -1, axis=0) + 1)
        d = np.minimum(e, 255)
    return d


def samples(q, dist, nu0, u_in):
    """(inputs, targets) of the coarse cells in cell order, as pw_closure_dataset_add."""
    rho, ux, uy, uz, txx, tyy, tzz, txy, txz, tyz = q
    nz, ny, nx = rho.shape
    u = [ux, uy, uz]
    grad = np.zeros((3, 3) + rho.shape)
    for b in range(3):
        grad[0, b][:, :, 1:-1] = 0.5 * (u[b][:, :, 2:] - u[b][:, :, :-2])
        grad[1, b] = 0.5 * (np.roll(u[b], -1, axis=1) - np.roll(u[b], 1, axis=1))
        grad[2, b] = 0.5 * (np.roll(u[b], -1, axis=0) - np.roll(u[b], 1, axis=0))
    s = np.stack([grad[0, 0], grad[1, 1], grad[2, 2], 0.5 * (grad[0, 1] + grad[1, 0]),
                  0.5 * (grad[0, 2] + grad[2, 0]), 0.5 * (grad[1, 2] + grad[2, 1])], axis=-1)
    t = np.stack([txx, tyy, tzz, txy, txz, tyz], axis=-1)
    ss = (s[..., :3] ** 2).sum(-1) + 2 * (s[..., 3:] ** 2).sum(-1)
    ts = (t[..., :3] * s[..., :3]).sum(-1) + 2 * (t[..., 3:] * s[..., 3:]).sum(-1)
    nu_s = 0.01 * np.sqrt(2 * ss)
    xidx = np.broadcast_to(np.arange(nx)[None, None, :], rho.shape)
    keep = (xidx >= 2) & (xidx + 3 <= nx) & (dist >= 2) & (nu_s > 1e-9)
    with np.errstate(divide="ignore", invalid="ignore"):
        nu_t = np.maximum(0.0, -ts / (2 * ss))
        y = np.clip(nu_t / nu_s - 1, -1, 3)
    k = keep.reshape(-1)
    x = features(s.reshape(-1, 6)[k], rho.reshape(-1)[k], ux.reshape(-1)[k], uy.reshape(-1)[k], uz.reshape(-1)[k],
                 dist.reshape(-1)[k].astype(np.float64), nu0, nu_s.reshape(-1)[k], u_in)
    return x, y.reshape(-1)[k]
