"""CPU oracle of the coarse-grid correction network — TEST INFRASTRUCTURE ONLY.

numpy restatement of the network liblbm_cuda.so trains on the tensor cores
(4 layers of 3x3 'same' convolutions with zero padding, channels
4 -> 32 -> 32 -> 32 -> 9, GELU in its tanh form between layers, MSE loss), used by the
tests as the checker of the GPU forward pass and gradients.  With bf16=True
it rounds where the GPU stores bf16: weights, every layer input, the stored
pre-activations and the loss gradient; sums are exact (f64).  With
bf16=False it is the plain f64 network, whose analytic gradients the tests
check against central finite differences.

Parameter layout (as lbm_cnn_get_params): per layer the weights
W[tap = ky*3 + kx][cin][cout], then the biases[cout].
"""
from __future__ import annotations

import numpy as np

CIN = (4, 32, 32, 32)
COUT = (32, 32, 32, 9)


def bf16(x):
    """Round to bfloat16 (nearest, ties to even), returned as float32/64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


K_GELU = np.sqrt(2.0 / np.pi)
C_GELU = 0.044715


def gelu(x):
    """GELU, tanh form: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))."""
    return 0.5 * x * (1.0 + np.tanh(K_GELU * (x + C_GELU * x ** 3)))


def gelu_grad(x):
    t = np.tanh(K_GELU * (x + C_GELU * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * K_GELU * (1.0 + 3.0 * C_GELU * x * x)


def unpack(params):
    ws, bs, k = [], [], 0
    for ci, co in zip(CIN, COUT):
        w = np.asarray(params[k:k + 9 * ci * co], dtype=np.float64).reshape(9, ci, co)
        k += 9 * ci * co
        b = np.asarray(params[k:k + co], dtype=np.float64)
        k += co
        ws.append(w)
        bs.append(b)
    return ws, bs


def pack(ws, bs):
    return np.concatenate([np.concatenate([w.ravel(), b.ravel()]) for w, b in zip(ws, bs)])


def _shift(x, dy, dx):
    """y[..., i, j] = x[..., i + dy, j + dx], zero outside."""
    B, C, H, W = x.shape
    out = np.zeros_like(x)
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(W, W - dx)
    out[:, :, ys:ye, xs:xe] = x[:, :, ys + dy:ye + dy, xs + dx:xe + dx]
    return out


def conv(x, w):
    """'same' 3x3 convolution (cross-correlation): out[b, o, i, j] =
    sum_{t, c} x[b, c, i + ky - 1, j + kx - 1] w[t, c, o]."""
    out = 0.0
    for t in range(9):
        ky, kx = divmod(t, 3)
        out = out + np.einsum("bchw,co->bohw", _shift(x, ky - 1, kx - 1), w[t])
    return out


def conv_input_grad(g, w):
    """Gradient of conv wrt its input: dx[b, c] = sum_t shift(g, -(t)) w[t]^T."""
    out = 0.0
    for t in range(9):
        ky, kx = divmod(t, 3)
        out = out + np.einsum("bohw,co->bchw", _shift(g, 1 - ky, 1 - kx), w[t])
    return out


def conv_weight_grad(x, g):
    dw = np.zeros((9, x.shape[1], g.shape[1]))
    for t in range(9):
        ky, kx = divmod(t, 3)
        dw[t] = np.einsum("bchw,bohw->co", _shift(x, ky - 1, kx - 1), g)
    return dw


def forward(params, x, bf16_rounding=True):
    """Returns (out, cache) for input x (B, 4, H, W)."""
    r = bf16 if bf16_rounding else (lambda v: np.asarray(v, dtype=np.float64))
    ws, bs = unpack(params)
    ws = [r(w) for w in ws]
    xs, zs = [r(x)], []
    out = None
    for l in range(4):
        z = conv(xs[l], ws[l]) + bs[l][None, :, None, None]
        if l < 3:
            zs.append(r(z))
            xs.append(r(gelu(z)))
        else:
            out = z
    return out, (ws, bs, xs, zs)


def gradients(params, x, target, bf16_rounding=True):
    """(loss, flat gradient) of the mean squared error."""
    r = bf16 if bf16_rounding else (lambda v: np.asarray(v, dtype=np.float64))
    out, (ws, bs, xs, zs) = forward(params, x, bf16_rounding)
    n = out.size
    d = out - target
    loss = float(np.mean(d * d))
    g = r(2.0 * d / n)
    dws, dbs = [None] * 4, [None] * 4
    for l in range(3, -1, -1):
        dws[l] = conv_weight_grad(xs[l], g)
        dbs[l] = g.sum(axis=(0, 2, 3))
        if l == 0:
            break
        g = r(conv_input_grad(g, ws[l]) * gelu_grad(zs[l - 1]))
    return loss, pack(dws, dbs)


def init_params(seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    ws, bs = [], []
    for l, (ci, co) in enumerate(zip(CIN, COUT)):
        lim = np.sqrt(6.0 / (9.0 * ci)) * (0.1 if l == 3 else 1.0) * scale
        ws.append(rng.uniform(-lim, lim, size=(9, ci, co)))
        bs.append(rng.uniform(-0.05, 0.05, size=co))
    return pack(ws, bs)
