"""CPU restatement of the learned cloth surrogate -- TEST INFRASTRUCTURE ONLY.

Used by tests/ (and nothing else) as the oracle of the CUDA surrogate in
feriphys_gb300/csrc/surrogate.cu: the per-vertex input features, the MLP
54 -> 128 -> 128 -> 3 with the bf16 roundings the tensor-core kernels make,
its gradient of the mean squared error (the gradient check the training
kernels are held to), the Adam update and the coarse integration step.

The surrogate has no counterpart in the reference (jalberse/feriphys); this
module restates the specification written in feriphys_gb300/csrc/surrogate.h.
Its backward pass is itself pinned by a finite-difference check in float64
with the roundings switched off (tests/test_surrogate_oracle.py).

Conventions (as on the GPU):
  * bf16 = round-to-nearest-even of the f32 value to 8 significant bits;
  * z = bf16(x) @ bf16(W)^T accumulated in f32 (here: f64, then f32) + b;
  * h = bf16(gelu(z)), slope g = bf16(gelu'(z)) with the tanh form of GELU;
  * dY = bf16((y - t) * 2 / (3 n)), dZ = bf16(dH * g), dH = dZ_next @ bf16(W);
  * weight gradients dW = dZ^T @ H of the bf16 operands; bias gradients are
    column sums of the same bf16 dZ.
"""
from __future__ import annotations

import numpy as np

N_FEAT = 54
N_HID = 128
N_OUT = 3
NEIGHBOURS = ((-1, -1), (-1, 0), (-1, 1), (0, -1), (0, 1), (1, -1), (1, 0), (1, 1))
GELU_C = np.float32(0.797884560802865356)
GELU_A = np.float32(0.044715)
INV_PI = np.float32(0.318309873342514038)


def bf16(x):
    """Round float32 values to bfloat16 (nearest even) and back to float32."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).copy()
    nan = np.isnan(a)
    out[nan] = a[nan]
    return out.reshape(np.shape(x))


def gelu(x, tanh=np.tanh):
    x = np.asarray(x)
    t = x.dtype.type
    x2 = x * x
    u = t(GELU_C) * (x + t(GELU_A) * (x2 * x))
    th = tanh(u)
    return (t(0.5) * x) * (t(1) + th)


def gelu_slope(x, tanh=np.tanh):
    x = np.asarray(x)
    t = x.dtype.type
    x2 = x * x
    u = t(GELU_C) * (x + t(GELU_A) * (x2 * x))
    th = tanh(u)
    g = (t(0.5) * x) * (t(1) + th)
    dg = t(0.5) * (t(1) + th) + ((t(0.5) * x) * (t(1) - th * th)) * (t(GELU_C) * (t(1) + (t(3) * t(GELU_A)) * x2))
    return g, dg


# ---- parameters ------------------------------------------------------------

def split_params(flat):
    """Public flat layout -> (W1[128,54], b1[128], W2[128,128], b2, W3[3,128], b3[3])."""
    f = np.asarray(flat)
    o = 0

    def take(n, shape):
        nonlocal o
        a = f[o:o + n].reshape(shape)
        o += n
        return a

    W1 = take(N_HID * N_FEAT, (N_HID, N_FEAT))
    b1 = take(N_HID, (N_HID,))
    W2 = take(N_HID * N_HID, (N_HID, N_HID))
    b2 = take(N_HID, (N_HID,))
    W3 = take(N_OUT * N_HID, (N_OUT, N_HID))
    b3 = take(N_OUT, (N_OUT,))
    assert o == f.size
    return W1, b1, W2, b2, W3, b3


def join_params(W1, b1, W2, b2, W3, b3):
    return np.concatenate([np.ravel(a) for a in (W1, b1, W2, b2, W3, b3)])


# ---- network ---------------------------------------------------------------

def _mm(a, b, dtype):
    """a @ b accumulated in float64, rounded to the working type."""
    return (a.astype(np.float64) @ b.astype(np.float64)).astype(dtype)


def forward(params, x, rounding=True, dtype=np.float32):
    """Outputs y[n,3] (standardised units, bias included) for standardised
    inputs x[n,54]; with rounding=False and dtype=float64 the exact network."""
    R = bf16 if rounding else (lambda a: np.asarray(a, dtype))
    W1, b1, W2, b2, W3, b3 = [np.asarray(a, dtype) for a in split_params(params)]
    xb = R(np.asarray(x, dtype))
    z1 = _mm(xb, R(W1).T, dtype) + b1
    h1 = R(gelu(z1))
    z2 = _mm(h1, R(W2).T, dtype) + b2
    h2 = R(gelu(z2))
    return _mm(h2, R(W3).T, dtype) + b3


def gradients(params, x, t, rounding=True, dtype=np.float32):
    """(flat gradient of mean((y - t)^2), loss) with the GPU's roundings."""
    R = bf16 if rounding else (lambda a: np.asarray(a, dtype))
    W1, b1, W2, b2, W3, b3 = [np.asarray(a, dtype) for a in split_params(params)]
    n = x.shape[0]
    xb = R(np.asarray(x, dtype))
    W1b, W2b, W3b = R(W1), R(W2), R(W3)
    z1 = _mm(xb, W1b.T, dtype) + b1
    g1v, s1 = gelu_slope(z1)
    h1, g1 = R(g1v), R(s1)
    z2 = _mm(h1, W2b.T, dtype) + b2
    g2v, s2 = gelu_slope(z2)
    h2, g2 = R(g2v), R(s2)
    y = _mm(h2, W3b.T, dtype) + b3
    r = y - np.asarray(t, dtype)
    loss = float(np.mean(r.astype(np.float64) ** 2))
    dscale = dtype(2.0) / (dtype(3.0) * dtype(n))
    dy = R(r * dscale)
    dW3 = _mm(dy.T, h2, dtype)
    db3 = dy.astype(np.float64).sum(0).astype(dtype)
    dH2 = _mm(dy, W3b, dtype)
    dZ2 = R(dH2 * g2)
    dW2 = _mm(dZ2.T, h1, dtype)
    db2 = dZ2.astype(np.float64).sum(0).astype(dtype)
    dH1 = _mm(dZ2, W2b, dtype)
    dZ1 = R(dH1 * g1)
    dW1 = _mm(dZ1.T, xb, dtype)
    db1 = dZ1.astype(np.float64).sum(0).astype(dtype)
    return join_params(dW1, db1, dW2, db2, dW3, db3), loss


def adam(params, grad, m, v, t, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step in f32 (t = step count after this step)."""
    f = np.float32
    c1 = f(1.0 / (1.0 - 0.9 ** t))
    c2 = f(1.0 / (1.0 - 0.999 ** t))
    g = np.asarray(grad, f)
    m = f(beta1) * m + (f(1) - f(beta1)) * g
    v = f(beta2) * v + (f(1) - f(beta2)) * (g * g)
    p = params - f(lr) * (m * c1) / (np.sqrt(v * c2) + f(eps))
    return p.astype(f), m.astype(f), v.astype(f)


# ---- features and the coarse step -------------------------------------------

def spacing(construction_positions, rows, cols):
    """Rest spacing: mean distance of horizontal neighbours at construction
    (vertical ones in a single column), f64 arithmetic, then f32."""
    p = np.asarray(construction_positions, np.float64).reshape(rows, cols, 3)
    d = p[:, 1:] - p[:, :-1] if cols >= 2 else p[1:, :] - p[:-1, :]
    return np.float32(np.sqrt((d ** 2).sum(-1)).mean())


def features(pos, vel, rows, cols, h, T, wind, rest):
    """Raw inputs [n,54] of every vertex (f32, the GPU's operation order).

    pos[n,4] = (x, y, z, mass), vel[n,4] = (vx, vy, vz, pinned), rest[n,3] =
    the positions the mesh was built from (the first 24 inputs are the
    stencil's deformation from its rest shape)."""
    f32 = np.float32
    P = np.asarray(pos, f32).reshape(rows, cols, 4)
    V = np.asarray(vel, f32).reshape(rows, cols, 4)
    P0 = np.asarray(rest, f32).reshape(rows, cols, 3)
    ih = f32(1) / f32(h)
    s = f32(T) / f32(h)
    out = np.zeros((rows, cols, N_FEAT), f32)
    q = {}
    for k, (dr, dc) in enumerate(NEIGHBOURS):
        Pn = P[:, :, :3].copy()
        Vn = V[:, :, :3].copy()
        Rn = P0.copy()
        has = np.zeros((rows, cols), bool)
        r0, r1 = max(0, -dr), rows - max(0, dr)
        c0, c1 = max(0, -dc), cols - max(0, dc)
        Pn[r0:r1, c0:c1] = P[r0 + dr:r1 + dr, c0 + dc:c1 + dc, :3]
        Vn[r0:r1, c0:c1] = V[r0 + dr:r1 + dr, c0 + dc:c1 + dc, :3]
        Rn[r0:r1, c0:c1] = P0[r0 + dr:r1 + dr, c0 + dc:c1 + dc]
        has[r0:r1, c0:c1] = True
        q[k] = Pn
        rel_p = ((Pn - P[:, :, :3]) - (Rn - P0)) * ih
        rel_v = (Vn - V[:, :, :3]) * s
        out[:, :, 3 * k:3 * k + 3] = np.where(has[..., None], rel_p, f32(0))
        out[:, :, 24 + 3 * k:24 + 3 * k + 3] = np.where(has[..., None], rel_v, f32(0))
    out[:, :, 48] = np.where(V[:, :, 3] != 0, f32(1), f32(0))
    w = np.asarray(wind, f32)
    for d in range(3):
        out[:, :, 49 + d] = (w[d] - V[:, :, d]) * s
    a = q[4] - q[3]
    b = q[6] - q[1]
    nx = a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1]
    ny = a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2]
    nz = a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]
    ln = np.sqrt((nx * nx + ny * ny) + nz * nz)
    good = (ln > 0) & np.isfinite(ln)
    with np.errstate(divide="ignore", invalid="ignore"):
        il = np.where(good, f32(1) / np.where(good, ln, f32(1)), f32(0))
    ux = np.where(good, nx * il, f32(0))
    uy = np.where(good, ny * il, f32(0))
    uz = np.where(good, nz * il, f32(1))
    out[:, :, 52] = np.arccos(np.clip(uy, f32(-1), f32(1))).astype(f32) * INV_PI
    out[:, :, 53] = np.arctan2(uz, ux).astype(f32) * INV_PI
    return out.reshape(rows * cols, N_FEAT)


def coarse_step(pos, vel, rows, cols, h, T, wind, rest, params, in_mean, in_std, out_mean, out_std):
    """One surrogate coarse step without obstacles: v' = v + dv,
    p' = p + (v + v') T / 2,
    pinned vertices unchanged.  Returns (pos', vel') as [n,4] f32."""
    f32 = np.float32
    P = np.asarray(pos, f32).reshape(-1, 4)
    V = np.asarray(vel, f32).reshape(-1, 4)
    x = features(P, V, rows, cols, h, T, wind, rest)
    inv_std = f32(1) / np.asarray(in_std, f32)
    xn = (x - np.asarray(in_mean, f32)) * inv_std
    y = forward(params, xn)
    inv_sv = f32(h) / f32(T)
    dv = (y * np.asarray(out_std, f32) + np.asarray(out_mean, f32)) * inv_sv
    nv = V[:, :3] + dv
    npos = P[:, :3] + (V[:, :3] + nv) * (f32(0.5) * f32(T))
    pinned = V[:, 3] != 0
    Po, Vo = P.copy(), V.copy()
    Po[~pinned, :3] = npos[~pinned]
    Vo[~pinned, :3] = nv[~pinned]
    Vo[~pinned, 3] = 0
    return Po, Vo
