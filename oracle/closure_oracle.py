"""CPU oracle of the learned closure (test infrastructure only).

A float64 numpy statement of every piece of the closure that the CUDA kernels
compute: the periodic 3-D convolution net (forward, backward), GELU, the
edge-EMF curl that carries the B correction and its adjoint, the loss and its
gradient, the coarse-graining box filter, the input features, the correction
step and AdamW.  The tests compare the BF16 tensor-core kernels with these
functions; nothing in the product imports this file.

The reference has no learned closure; conventions follow the solver's state
layout (C/mhd.c:26-41): u(5,n,n,n) = (rho, mx, my, mz, E), b(3,n,n,n) on the
faces at i, j, k of cell (i,j,k), component index fastest.

Tensor conventions (shared with the kernels):
  * boxes are periodic cubes; a batch of NB boxes is an array (NB, n, n, n, C)
    indexed [box, k, j, i, channel] (channels innermost, like the state);
  * a conv weight is (Cout, KS, KS, KS, Cin) indexed [co, dk, dj, di, ci] and
    reads the input at (k+dk-h, j+dj-h, i+di-h) with h = KS//2;
  * edge EMFs E[...,0] = Ex at (i+1/2, j, k), E[...,1] = Ey at (i, j+1/2, k),
    E[...,2] = Ez at (i, j, k+1/2), in cell units.
"""
from __future__ import annotations

import math

import numpy as np

try:
    from scipy.special import erf as _erf
except ImportError:  # pragma: no cover
    _erf = np.vectorize(math.erf)

GAMMA = 5.0 / 3.0


# ---------------------------------------------------------------- layers

def conv3d(x: np.ndarray, w: np.ndarray, bias: np.ndarray) -> np.ndarray:
    """Periodic 3-D convolution (cross-correlation), float64."""
    nb, n = x.shape[0], x.shape[1]
    co, ks = w.shape[0], w.shape[1]
    h = ks // 2
    y = np.zeros((nb, n, n, n, co))
    for dk in range(ks):
        for dj in range(ks):
            for di in range(ks):
                xs = np.roll(x, shift=(h - dk, h - dj, h - di), axis=(1, 2, 3))
                y += np.einsum("bkjic,oc->bkjio", xs, w[:, dk, dj, di, :], optimize=True)
    return y + bias


def conv3d_backward(x: np.ndarray, w: np.ndarray, dy: np.ndarray):
    """Gradients of conv3d: (dx, dw, dbias)."""
    ks = w.shape[1]
    h = ks // 2
    dx = np.zeros_like(x, dtype=np.float64)
    dw = np.zeros_like(w, dtype=np.float64)
    for dk in range(ks):
        for dj in range(ks):
            for di in range(ks):
                xs = np.roll(x, shift=(h - dk, h - dj, h - di), axis=(1, 2, 3))
                dw[:, dk, dj, di, :] = np.einsum("bkjio,bkjic->oc", dy, xs, optimize=True)
                g = np.einsum("bkjio,oc->bkjic", dy, w[:, dk, dj, di, :], optimize=True)
                dx += np.roll(g, shift=(dk - h, dj - h, di - h), axis=(1, 2, 3))
    return dx, dw, dy.sum(axis=(0, 1, 2, 3))


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    bits = a.view(np.uint32).astype(np.uint64)
    bits = (bits + 0x7FFF + ((bits >> 16) & 1)) & 0xFFFF0000
    return bits.astype(np.uint32).view(np.float32).astype(np.float64)


# ---------------------------------------------------------------- the net

def net_forward(params, x, round_bf16: bool = False):
    """params: list of (w, b) for the hidden 3^3 layers then the 1^3 head.
    Returns (out, cache); the hidden layers apply GELU."""
    q = bf16 if round_bf16 else (lambda t: t)
    a = q(x)
    cache = []
    for w, b in params[:-1]:
        z = conv3d(a, q(w), b)
        cache.append((a, z))
        a = q(gelu(q(z)))
    w, b = params[-1]
    out = conv3d(a, q(w), b)
    cache.append((a, None))
    return out, cache


def net_backward(params, cache, dout):
    """Gradients [(dw, db)] of every layer, for d loss / d out = dout."""
    grads = [None] * len(params)
    a, _ = cache[-1]
    da, dw, db = conv3d_backward(a, params[-1][0], dout)
    grads[-1] = (dw, db)
    for li in range(len(params) - 2, -1, -1):
        a, z = cache[li]
        dz = da * gelu_grad(z)
        da, dw, db = conv3d_backward(a, params[li][0], dz)
        grads[li] = (dw, db)
    return grads


# ------------------------------------------------------- EMF and its curl

def curl_faces(e: np.ndarray) -> np.ndarray:
    """dB = -curl E on the faces from edge EMFs (both (..., n, n, n, 3))."""
    ex, ey, ez = e[..., 0], e[..., 1], e[..., 2]
    K, J, I = -3, -2, -1  # axes of k, j, i of one component (..., k, j, i)

    def nxt(f, ax):  # f at index+1 along ax
        return np.roll(f, -1, axis=ax)

    dbx = -(nxt(ez, J) - ez) + (nxt(ey, K) - ey)
    dby = -(nxt(ex, K) - ex) + (nxt(ez, I) - ez)
    dbz = -(nxt(ey, I) - ey) + (nxt(ex, J) - ex)
    return np.stack([dbx, dby, dbz], axis=-1)


def curl_faces_adjoint(r: np.ndarray) -> np.ndarray:
    """Adjoint of curl_faces: <curl_faces(E), r> = <E, curl_faces_adjoint(r)>."""
    rx, ry, rz = r[..., 0], r[..., 1], r[..., 2]
    K, J, I = -3, -2, -1

    def prv(f, ax):  # f at index-1 along ax
        return np.roll(f, 1, axis=ax)

    gx = ry - prv(ry, K) + prv(rz, J) - rz
    gy = prv(rx, K) - rx + rz - prv(rz, I)
    gz = rx - prv(rx, J) + prv(ry, I) - ry
    return np.stack([gx, gy, gz], axis=-1)


def loss_and_grad(out: np.ndarray, tu: np.ndarray, tb: np.ndarray):
    """loss = (sum r_f^2 + sum r_b^2) / (8 N) with r_f = out[..., :5] - tu and
    r_b = curl_faces(out[..., 5:]) - tb; returns (loss, d loss / d out)."""
    nvox = out.shape[0] * out.shape[1] ** 3
    rf = out[..., :5] - tu
    rb = curl_faces(out[..., 5:]) - tb
    loss = (np.sum(rf * rf) + np.sum(rb * rb)) / (8.0 * nvox)
    d = np.zeros_like(out)
    d[..., :5] = 2.0 * rf / (8.0 * nvox)
    d[..., 5:] = curl_faces_adjoint(2.0 * rb / (8.0 * nvox))
    return loss, d


# ------------------------------------------------------ states and data

def state_arrays(u, b, n):
    """(n,n,n,5) and (n,n,n,3) float64 views of a flat state."""
    return (np.asarray(u, dtype=np.float64).reshape(n, n, n, 5),
            np.asarray(b, dtype=np.float64).reshape(n, n, n, 3))


def cell_b(B: np.ndarray) -> np.ndarray:
    """Cell-centred B (face means) of (..., n, n, n, 3) faces."""
    return 0.5 * (B + np.stack([np.roll(B[..., c], -1, axis=-1 - c) for c in range(3)], axis=-1))


def features(u, b, n, mean, inv_std):
    """(n,n,n,16) net input: (rho, m, E, B_cell) standardised, 8 zero channels."""
    U, B = state_arrays(u, b, n)
    raw = np.concatenate([U, cell_b(B)], axis=-1)
    x = np.zeros((n, n, n, 16))
    x[..., :8] = (raw - np.asarray(mean)) * np.asarray(inv_std)
    return x


def box_filter(u, b, n, f):
    """Coarse-grain a fine state by f: u averaged over f^3 cells, each face
    component over the f^2 fine faces that make the coarse face."""
    U, B = state_arrays(u, b, n)
    m = n // f
    uc = U.reshape(m, f, m, f, m, f, 5).mean(axis=(1, 3, 5))
    bx = B[:, :, ::f, 0].reshape(m, f, m, f, m).mean(axis=(1, 3))
    by = B[:, ::f, :, 1].reshape(m, f, m, m, f).mean(axis=(1, 4))
    bz = B[::f, :, :, 2].reshape(m, m, f, m, f).mean(axis=(2, 4))
    return uc.reshape(-1), np.stack([bx, by, bz], axis=-1).reshape(-1)


def targets(u_fine_next, b_fine_next, u_coarse, b_coarse, n, oscale, bscale):
    """Normalised targets (n,n,n,8): fluid difference / oscale, face difference / bscale."""
    Uf, Bf = state_arrays(u_fine_next, b_fine_next, n)
    Uc, Bc = state_arrays(u_coarse, b_coarse, n)
    t = np.zeros((n, n, n, 8))
    t[..., :5] = (Uf - Uc) / np.asarray(oscale)
    t[..., 5:] = (Bf - Bc) / bscale
    return t


def apply_correction(u, b, out, n, oscale, bscale, alpha=1.0):
    """u + alpha oscale (out[:5] - box mean); b + alpha bscale curl_faces(out[5:])."""
    U, B = state_arrays(u, b, n)
    O = np.asarray(out, dtype=np.float64).reshape(n, n, n, 8)
    fl = O[..., :5] - O[..., :5].mean(axis=(0, 1, 2))
    U2 = U + alpha * fl * np.asarray(oscale)
    B2 = B + alpha * bscale * curl_faces(O[..., 5:])
    return U2.reshape(-1), B2.reshape(-1)


def pressure(u, b, n):
    U, B = state_arrays(u, b, n)
    Bc = cell_b(B)
    ek = 0.5 * (U[..., 1:4] ** 2).sum(-1) / U[..., 0]
    return (GAMMA - 1.0) * (U[..., 4] - ek - 0.5 * (Bc ** 2).sum(-1))


def adamw(p, g, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8, wd=1e-4):
    """One AdamW update (decoupled weight decay); returns (p, m, v)."""
    m = beta1 * m + (1 - beta1) * g
    v = beta2 * v + (1 - beta2) * g * g
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    p = p - lr * (mh / (np.sqrt(vh) + eps) + wd * p)
    return p, m, v
