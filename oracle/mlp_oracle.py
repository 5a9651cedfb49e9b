"""CPU oracle of the troubled-cell MLP (test infrastructure only): the forward
pass, loss and gradients in float64 numpy with the same BF16 rounding points as
the GPU kernels (inputs, W1, W2, the layer-2 operand a1, the weight-gradient
operands dz1 and dz2, and W2 in the backward matmul), so that GPU and CPU
gradients agree to FP32 accumulation round-off."""
import math

import numpy as np

H = 64


def bf16(x):
    """Round float values to bfloat16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    rounded = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


def bf16_bits_to_float(bits):
    return (np.asarray(bits).astype(np.uint16).astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def unpack(params, kpad):
    p = np.asarray(params, dtype=np.float64)
    o = 0
    W1 = p[o:o + H * kpad].reshape(H, kpad); o += H * kpad
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


GELU_C = 2.0 * math.sqrt(2.0 / math.pi)


def _sigmoid(z):
    with np.errstate(over="ignore"):
        return 1.0 / (1.0 + np.exp(-z))


def gelu(x):
    """GELU, tanh form: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))) = x sigmoid(z)."""
    return x * _sigmoid(GELU_C * (x + 0.044715 * x ** 3))


def gelu_grad(x):
    s = _sigmoid(GELU_C * (x + 0.044715 * x ** 3))
    return s + x * s * (1.0 - s) * GELU_C * (1.0 + 3.0 * 0.044715 * x * x)


def forward(params, X, kpad):
    W1, b1, W2, b2, w3, b3 = unpack(params, kpad)
    z1 = X @ bf16(W1).T + b1
    a1 = gelu(z1)
    z2 = bf16(a1) @ bf16(W2).T + b2
    a2 = gelu(z2)
    z3 = a2 @ w3 + b3
    return 1.0 / (1.0 + np.exp(-z3)), (z1, a1, z2, a2)


def loss_and_grad(params, X, y, kpad):
    """Mean BCE and its gradient (flat, the layout of the parameter vector)."""
    W1, b1, W2, b2, w3, b3 = unpack(params, kpad)
    B = X.shape[0]
    p, (z1, a1, z2, a2) = forward(params, X, kpad)
    yy = y.astype(np.float64)
    loss = -np.mean(yy * np.log(np.maximum(p, 1e-12)) + (1 - yy) * np.log(np.maximum(1 - p, 1e-12)))
    d3 = (p - yy) / B
    dz2 = d3[:, None] * w3[None, :] * gelu_grad(z2)
    da1 = bf16(dz2) @ bf16(W2)
    dz1 = da1 * gelu_grad(z1)
    g = np.zeros_like(np.asarray(params, dtype=np.float64))
    o = 0
    g[o:o + H * kpad] = (bf16(dz1).T @ X).reshape(-1); o += H * kpad
    g[o:o + H] = dz1.sum(0); o += H
    g[o:o + H * H] = (bf16(dz2).T @ bf16(a1)).reshape(-1); o += H * H
    g[o:o + H] = dz2.sum(0); o += H
    g[o:o + H] = a2.T @ d3; o += H
    g[o] = d3.sum()
    return loss, g
