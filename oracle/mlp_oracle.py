"""CPU oracle of the learned start value's network (TEST INFRASTRUCTURE ONLY).

float64 numpy restatement of the 6-32-32-1 SiLU network of
asteriy_2d_gb300/csrc/mlp.cuh: forward pass, mean-squared-error loss, the
analytic gradient by backpropagation, and a central finite-difference
gradient to check it.  The parameter block layout is the one of mlp.cuh.
"""
import numpy as np

SHIFT, SCALE, W1, B1, W2, B2, W3, B3, NPARAM = 0, 6, 12, 204, 236, 1260, 1292, 1324, 1325


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[SHIFT:SHIFT + 6], p[SCALE:SCALE + 6], p[W1:B1].reshape(32, 6), p[B1:W2],
            p[W2:B2].reshape(32, 32), p[B2:W3], p[W3:B3], p[B3])


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def input_map(x):
    """The network's fixed input map: log of the positive ratios (features 0,
    1, 3), asinh of the velocity jump (feature 2)."""
    x = np.array(x, dtype=np.float64)
    x[:, [0, 1, 3]] = np.log(x[:, [0, 1, 3]])
    x[:, 2] = np.arcsinh(x[:, 2])
    return x


def forward(p, x):
    shift, scale, w1, b1, w2, b2, w3, b3 = unpack(p)
    xn = (input_map(x) - shift) * scale
    z1 = xn @ w1.T + b1
    h1 = silu(z1)
    z2 = h1 @ w2.T + b2
    h2 = silu(z2)
    return h2 @ w3 + b3, (xn, z1, h1, z2, h2)


def loss(p, x, t):
    y, _ = forward(p, x)
    return np.mean((y - t) ** 2)


def grad(p, x, t):
    """Analytic gradient of the mean-squared error (shift/scale slots zero)."""
    shift, scale, w1, b1, w2, b2, w3, b3 = unpack(p)
    y, (xn, z1, h1, z2, h2) = forward(p, x)
    n = len(x)
    dy = 2.0 * (y - t) / n
    g = np.zeros(NPARAM)
    g[W3:B3] = dy @ h2
    g[B3] = dy.sum()
    dz2 = dy[:, None] * w3[None, :] * silu_grad(z2)
    g[W2:B2] = (dz2.T @ h1).ravel()
    g[B2:W3] = dz2.sum(0)
    dz1 = (dz2 @ w2) * silu_grad(z1)
    g[W1:B1] = (dz1.T @ xn).ravel()
    g[B1:W2] = dz1.sum(0)
    return g


def fd_grad(p, x, t, idx, h=1e-6):
    p = np.asarray(p, dtype=np.float64)
    out = []
    for i in idx:
        a = p.copy(); a[i] += h
        b = p.copy(); b[i] -= h
        out.append((loss(a, x, t) - loss(b, x, t)) / (2 * h))
    return np.array(out)
