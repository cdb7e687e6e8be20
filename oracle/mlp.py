"""numpy restatement of the learned warm start: node descriptors and the BF16 MLP with its
gradients.

TEST INFRASTRUCTURE ONLY: tests/ check the library's descriptor kernel and its tensor-core
forward/backward kernels against these functions; the product never imports this module.

The reference has no learned component (its start density is the atomic superposition,
SuperposAtRho, src/ilsdft.h:269).  The model is stated here in full:

Descriptors of a grid point x (64 per point).  Over the atom images J with r_J = |x - X_J| <
R_CUT = 8 bohr: radial Gaussians g_n(r) = exp(-(r - mu_n)^2 / (2 sigma^2)) fc(r) with 16
centres mu_n = 8 n / 15 and sigma = 0.5 bohr, smooth cutoff fc(r) = (cos(pi r / R_CUT) + 1)/2,
times the real spherical harmonics Y_lm(x - X_J) of l <= 3 (the reference's constants,
src/lsdft_tools.cc:156-370; at r = 0 only l = 0):
    c_{n,lm} = sum_J g_n(r_J) Y_lm,   feature[4 n + l] = sqrt(sum_m c_{n,lm}^2).

MLP 64 - 128 - 128 - 1 with SiLU activations on standardised features; the output is the
standardised correction rho_SCF - rho_0 to the atomic superposition.  BF16 enters exactly
where the tensor-core kernels round: features X, weights W1, W2, w3, the hidden activations
h1 (operand of the second product) and the back-propagated dz2, dz1 (operands of the
gradient products).  Products of BF16 numbers are exact in FP32 and sums are FP32 on the GPU
(float64 here).  Loss L = mean over the batch of (y - t)^2.
"""
import math

import numpy as np

R_CUT = 8.0
N_RAD = 16
SIGMA = 0.5
MU = np.arange(N_RAD) * (R_CUT / (N_RAD - 1))
N_FEAT = 64
N_HID = 128

_Y0 = 0.282094791773878  # 1 / (2 sqrt(pi))


def bf16(a):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def real_ylm(dx, dy, dz):
    """The 16 real spherical harmonics (l <= 3) of unit direction (dx,dy,dz), [..., 16]."""
    x, y, z = dx, dy, dz
    return np.stack([
        np.full_like(x, _Y0),
        0.488602511902920 * y, 0.488602511902920 * z, 0.488602511902920 * x,
        1.092548430592079 * x * y, 1.092548430592079 * y * z,
        0.315391565252520 * (2 * z * z - x * x - y * y), 1.092548430592079 * z * x,
        0.546274215296040 * (x * x - y * y),
        0.590043589926644 * (3 * x * x - y * y) * y, 2.890611442640554 * x * y * z,
        0.457045799464466 * y * (4 * z * z - x * x - y * y),
        0.373176332590115 * z * (2 * z * z - 3 * x * x - 3 * y * y),
        0.457045799464466 * x * (4 * z * z - x * x - y * y),
        1.445305721320277 * z * (x * x - y * y), 0.590043589926644 * x * (x * x - 3 * y * y),
    ], axis=-1)


def descriptors(points, atoms, cell):
    """Descriptors [n_points, 64] of points [n, 3] for the periodic cell of side lengths
    cell[3] with atoms [natoms, 3] (all images within R_CUT)."""
    points = np.asarray(points, dtype=np.float64)
    cell = np.asarray(cell, dtype=np.float64)
    c = np.zeros((len(points), N_RAD, 16))
    reps = [int(math.ceil(R_CUT / cell[a])) + 1 for a in range(3)]
    for X in np.asarray(atoms, dtype=np.float64):
        for P in range(-reps[0], reps[0] + 1):
            for Q in range(-reps[1], reps[1] + 1):
                for R in range(-reps[2], reps[2] + 1):
                    d = points - (X + np.array([P, Q, R]) * cell)
                    r = np.sqrt(np.sum(d * d, axis=1))
                    sel = r < R_CUT
                    if not np.any(sel):
                        continue
                    rs, ds = r[sel], d[sel]
                    fc = 0.5 * (np.cos(math.pi * rs / R_CUT) + 1.0)
                    g = np.exp(-(rs[:, None] - MU[None, :]) ** 2 / (2 * SIGMA * SIGMA)) * fc[:, None]
                    inv = np.where(rs > 1e-12, 1.0 / np.where(rs > 1e-12, rs, 1.0), 0.0)
                    Y = real_ylm(ds[:, 0] * inv, ds[:, 1] * inv, ds[:, 2] * inv)
                    Y[rs <= 1e-12, 1:] = 0.0
                    c[sel] += g[:, :, None] * Y[:, None, :]
    lsl = [slice(0, 1), slice(1, 4), slice(4, 9), slice(9, 16)]
    feat = np.stack([np.sqrt(np.sum(c[:, :, s] ** 2, axis=2)) for s in lsl], axis=2)
    return feat.reshape(len(points), N_FEAT)  # [n, 16 radial, 4 l] -> feature 4 n + l


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward_backward(params, x, t, mask=None, rounding=True):
    """Loss and gradients of the BF16 MLP on standardised features x [n, 64] and targets
    t [n]; params = dict(W1 [64,128], b1 [128], W2 [128,128], b2 [128], w3 [128], b3 [1])
    (float master values; the BF16 rounding is applied here, or skipped with rounding=False
    for exact float64 gradients).  mask [n] weights rows (0 for padding); the mean runs over
    the rows with weight 1.  Returns (loss, grads, y)."""
    rnd = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    n = len(x)
    m = np.ones(n) if mask is None else np.asarray(mask, dtype=np.float64)
    cnt = max(1.0, m.sum())
    X = rnd(x)
    W1, W2, w3 = rnd(params["W1"]), rnd(params["W2"]), rnd(params["w3"])
    z1 = X @ W1 + params["b1"]
    h1 = rnd(silu(z1))
    z2 = h1 @ W2 + params["b2"]
    h2 = silu(z2)
    y = h2 @ w3 + params["b3"][0]
    r = (y - t) * m
    loss = float(np.sum(r * r) / cnt)
    dy = 2.0 * r / cnt
    dz2 = dy[:, None] * w3[None, :] * dsilu(z2)
    dz2b = rnd(dz2)
    dh1 = dz2b @ W2.T
    dz1 = dh1 * dsilu(z1)
    dz1b = rnd(dz1)
    grads = {"W1": X.T @ dz1b, "b1": dz1.sum(0), "W2": h1.T @ dz2b, "b2": dz2.sum(0),
             "w3": h2.T @ dy, "b3": np.array([dy.sum()])}
    return loss, grads, y


def forward(params, x):
    """Network output y [n] (standardised units) for standardised features x [n, 64]."""
    X = bf16(x)
    h1 = bf16(silu(X @ bf16(params["W1"]) + params["b1"]))
    h2 = silu(h1 @ bf16(params["W2"]) + params["b2"])
    return h2 @ bf16(params["w3"]) + params["b3"][0]
