"""CPU restatement of the learned proposal's network (TEST INFRASTRUCTURE ONLY).

Only tests/ and bench.py's checks use this module, as the checker of the
library's tensor-core forward and backward kernels (lyapunov3d_gb300/csrc/
lyap_net.cu); the product package never imports it.  The network has no
reference counterpart (the reference marches every sample, kernel.cu:326-363);
this file restates the published definitions the library's header gives
(include/lyap_gb300.h, LyapNet):

    u = (P - lo) / (hi - lo)
    f[2*(3k+j)] = sin(pi 2^k u_j), f[2*(3k+j)+1] = cos(pi 2^k u_j)   k < 8, j < 3
    h1 = gelu(W1 f + b1), h2 = gelu(W2 h1 + b2), out = w3 . h2 + b3
    gelu(x) = x/2 (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))

in float64, with the roundings the GPU applies to the tensor-core operands:
f, W1, h1, W2 and w3 rounded to nearest-even BF16 (the products then exact
in float64; the GPU accumulates them in FP32).  The gradient of the loss
(1/n) sum (out - t)^2 is the exact derivative of this rounded forward pass
(roundings treated as identity in the backward), which is what the GPU's
backward computes up to its own BF16 rounding of dz1, dz2.  `fd_check`
verifies the analytic gradient against central differences, so the oracle
is pinned by calculus rather than by the library.
"""
import numpy as np

NF, NH = 48, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + NH * NF
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NH
NPARAM = OFF_B3 + 1
assert NPARAM == 7361

K0 = np.sqrt(2.0 / np.pi)
K1 = 0.044715


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64).reshape(a.shape)


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    return (p[OFF_W1:OFF_B1].reshape(NH, NF), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(NH, NH),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3], p[OFF_B3])


def pack(w1, b1, w2, b2, w3, b3):
    return np.concatenate([np.ravel(w1), b1, np.ravel(w2), b2, w3, [b3]])


def features(u):
    u = np.asarray(u, dtype=np.float64).reshape(-1, 3)
    f = np.empty((u.shape[0], NF))
    for k in range(8):
        for j in range(3):
            a = np.pi * (2.0 ** k) * u[:, j]
            f[:, 2 * (3 * k + j)] = np.sin(a)
            f[:, 2 * (3 * k + j) + 1] = np.cos(a)
    return f


def gelu(x):
    th = np.tanh(K0 * (x + K1 * x ** 3))
    return 0.5 * x * (1.0 + th), th


def gelu_grad(x, th):
    return 0.5 * (1.0 + th) + 0.5 * x * (1.0 - th * th) * K0 * (1.0 + 3.0 * K1 * x * x)


def to_unit(xyz, lo, hi):
    xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    return (xyz - np.asarray(lo, dtype=np.float64)) / (np.asarray(hi, dtype=np.float64) - np.asarray(lo))


def forward(params, u, rounding=True):
    """out[n] and the intermediates (f, z1, h1, z2, h2) at unit-box points u[n, 3]."""
    w1, b1, w2, b2, w3, b3 = unpack(params)
    r = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    f = r(features(u))
    z1 = f @ r(w1).T + b1
    h1, _ = gelu(z1)
    h1r = r(h1)
    z2 = h1r @ r(w2).T + b2
    h2, _ = gelu(z2)
    out = h2 @ r(w3) + b3
    return out, (f, z1, h1r, z2, h2)


def loss_grad(params, u, target, rounding=True):
    """(loss, grad[NPARAM]) of (1/n) sum (out - t)^2."""
    w1, b1, w2, b2, w3, b3 = unpack(params)
    r = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    out, (f, z1, h1r, z2, h2) = forward(params, u, rounding)
    t = np.asarray(target, dtype=np.float64)
    n = t.size
    err = out - t
    g = 2.0 * err / n
    _, th2 = gelu(z2)
    gw3 = g @ h2
    gb3 = g.sum()
    dz2 = np.outer(g, r(w3)) * gelu_grad(z2, th2)
    gw2 = dz2.T @ h1r
    gb2 = dz2.sum(0)
    dh1 = dz2 @ r(w2)
    _, th1 = gelu(z1)
    dz1 = dh1 * gelu_grad(z1, th1)
    gw1 = dz1.T @ f
    gb1 = dz1.sum(0)
    return float(np.mean(err ** 2)), pack(gw1, gb1, gw2, gb2, gw3, gb3)


def fd_check(params, u, target, n_probe=40, eps=1e-6, seed=0):
    """Largest relative difference between the analytic gradient (no
    rounding) and central differences of the loss at n_probe parameters."""
    _, g = loss_grad(params, u, target, rounding=False)
    rng = np.random.default_rng(seed)
    idx = rng.choice(NPARAM, size=n_probe, replace=False)
    worst = 0.0
    p = np.asarray(params, dtype=np.float64).copy()
    for i in idx:
        old = p[i]
        p[i] = old + eps
        lp, _ = loss_grad(p, u, target, rounding=False)
        p[i] = old - eps
        lm, _ = loss_grad(p, u, target, rounding=False)
        p[i] = old
        fd = (lp - lm) / (2 * eps)
        worst = max(worst, abs(fd - g[i]) / max(1e-8, abs(fd) + abs(g[i])))
    return worst


def init_params(seed=0):
    """He-normal weights, zero biases (any initialisation serves the checks)."""
    rng = np.random.default_rng(seed)
    w1 = rng.standard_normal((NH, NF)) * np.sqrt(2.0 / NF)
    w2 = rng.standard_normal((NH, NH)) * np.sqrt(2.0 / NH)
    w3 = rng.standard_normal(NH) * np.sqrt(1.0 / NH)
    return pack(w1, np.zeros(NH), w2, np.zeros(NH), w3, 0.0)
