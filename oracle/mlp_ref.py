"""ORACLE (test infrastructure only): numpy restatement of the warm-start MLP of
libgdx-jbullet_gb300/csrc/mlp.cuh / mlp.cu, the checker of its forward pass and gradients.

24 -> 64 -> 64 -> 3, inputs through asinh((x - mean) * scale), GELU in its tanh form, mean
squared error of normalised outputs.  With
`bf16=True` every tensor-core operand is rounded to bfloat16 (round to nearest even) exactly
where the kernels round it: normalised inputs, weights, activations, dY, dZ2, dZ1; sums are
taken in float64.  With `bf16=False` the same function in float64 is differentiable by finite
differences (the check of the analytic backward pass itself)."""
import numpy as np

N_IN, N_H, N_OUT = 24, 64, 3
OFF_W1 = 0
OFF_B1 = OFF_W1 + N_H * N_IN
OFF_W2 = OFF_B1 + N_H
OFF_B2 = OFF_W2 + N_H * N_H
OFF_W3 = OFF_B2 + N_H
OFF_B3 = OFF_W3 + N_OUT * N_H
N_PARAM = OFF_B3 + N_OUT
K_GELU = 0.7978845608028654


def bf16(x):
    """Round float32 values to the nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    out = r.view(np.float32)
    return np.where(np.isnan(a), a, out)


def unpack(p):
    p = np.asarray(p, np.float64)
    W1 = p[OFF_W1:OFF_B1].reshape(N_H, N_IN)
    W2 = p[OFF_W2:OFF_B2].reshape(N_H, N_H)
    W3 = p[OFF_W3:OFF_B3].reshape(N_OUT, N_H)
    return W1, p[OFF_B1:OFF_W2], W2, p[OFF_B2:OFF_W3], W3, p[OFF_B3:N_PARAM]


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(K_GELU * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    th = np.tanh(K_GELU * (x + 0.044715 * x ** 3))
    return 0.5 * (1.0 + th) + 0.5 * x * (1.0 - th * th) * K_GELU * (1.0 + 3.0 * 0.044715 * x * x)


def _r(x, on):
    return bf16(x).astype(np.float64) if on else np.asarray(x, np.float64)


N_NORM = 2 * N_IN + 2 * N_OUT + 1


def normalise(norm, x):
    norm = np.asarray(norm, np.float32)
    return np.arcsinh((np.asarray(x, np.float32) - norm[:N_IN]) * norm[N_IN:2 * N_IN])


def forward(p, norm, x, bf16=True):
    """Raw outputs and the intermediate tensors for the backward pass."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    xn = _r(normalise(norm, x), bf16)
    z1 = xn @ _r(W1, bf16).T + b1
    h1 = _r(gelu(z1), bf16)
    z2 = h1 @ _r(W2, bf16).T + b2
    h2 = _r(gelu(z2), bf16)
    y = h2 @ _r(W3, bf16).T + b3
    norm = np.asarray(norm, np.float64)
    raw = y * norm[2 * N_IN + N_OUT:2 * N_IN + 2 * N_OUT] + norm[2 * N_IN:2 * N_IN + N_OUT]
    return raw, (xn, z1, h1, z2, h2, y)


def loss_and_grad(p, norm, x, t, bf16=True):
    """Mean squared error of the normalised outputs over all samples and outputs, and its
    gradient with respect to the packed parameters."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    _, (xn, z1, h1, z2, h2, y) = forward(p, norm, x, bf16)
    norm = np.asarray(norm, np.float64)
    tn = (np.asarray(t, np.float64) - norm[2 * N_IN:2 * N_IN + N_OUT]) / norm[2 * N_IN + N_OUT:2 * N_IN + 2 * N_OUT]
    n = len(x)
    r = y - tn
    loss = float(np.mean(r * r))
    dy = 2.0 * r / (n * N_OUT)
    dyb = _r(dy, bf16)
    g = np.zeros(N_PARAM)
    g[OFF_W3:OFF_B3] = (dyb.T @ h2).ravel()
    g[OFF_B3:N_PARAM] = dy.sum(0)
    dz2 = _r((dyb @ _r(W3, bf16)) * gelu_grad(z2), bf16)
    g[OFF_W2:OFF_B2] = (dz2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    dz1 = _r((dz2 @ _r(W2, bf16)) * gelu_grad(z1), bf16)
    g[OFF_W1:OFF_B1] = (dz1.T @ xn).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    return loss, g
