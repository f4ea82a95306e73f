"""CPU reference of the learned anisotropic filter's MLP (numpy, float64).

ORACLE / TEST INFRASTRUCTURE: only tests/ load this module.  It restates the
network the GPU kernels run -- 24 -> 64 -> 64 -> 5, GELU (tanh form), RGBA plus a
confidence logit -- and its training loss and gradients, in float64.  With
`bf16_ops=True` it rounds the operands the GPU feeds to its tensor cores
(inputs, weights, hidden activations) to BF16 and evaluates GELU in BF16
steps as the GPU does, so forward outputs can be compared closely; gradients
are compared against the exact float64 ones at a stated tolerance.

Parameter layout (fp32 masters, W[out][in]): W1 [64 x 24], b1 [64],
W2 [64 x 64], b2 [64], W3 [5 x 64], b3 [5].

Prediction: colour = the mean of the four bilinear taps (features 8-23, in
float32 as the GPU forms it) + the network's colour outputs; confidence =
sigmoid of the fifth output.

Training loss per sample (mean over the batch):
    sum_c (out_c - y_c)^2 for the 4 colour channels of the prediction
  + binary cross-entropy of sigmoid(out_4) against exp(-CONF_K * e), where
    e is the largest absolute colour error of the sample (not differentiated).
"""
import math

import numpy as np

F, H, O = 24, 64, 5
CONF_K = 32.0
OFFS = {"W1": (0, (H, F)), "b1": (H * F, (H,)), "W2": (H * F + H, (H, H)), "b2": (H * F + H + H * H, (H,)),
        "W3": (H * F + 2 * H + H * H, (O, H)), "b3": (H * F + 2 * H + H * H + O * H, (O,))}
NPARAMS = H * F + H + H * H + H + O * H + O


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return {k: p[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in OFFS.items()}


def pack(d):
    out = np.zeros(NPARAMS, dtype=np.float64)
    for k, (o, s) in OFFS.items():
        out[o:o + int(np.prod(s))] = np.asarray(d[k]).ravel()
    return out


def bf16(x):
    """Round to BF16 (nearest even) and back, elementwise."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


# GELU, tanh form (Hendrycks and Gimpel 2016), in float64
K0 = math.sqrt(2.0 / math.pi)
K1 = K0 * 0.044715


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(x * (K0 + K1 * x * x)))


def gelu_bf16(x):
    """The GPU's forward GELU, step by step in BF16 arithmetic (each product
    or fused multiply-add rounded once; tanh in float64 where the GPU's
    tanh.approx differs by about one BF16 step)."""
    k0, k1 = bf16(np.float32(K0)), bf16(np.float32(K1))
    x = bf16(x)
    u = bf16(x * bf16(bf16(x * x) * k1 + k0))
    t = bf16(np.tanh(u))
    h = bf16(x * 0.5)
    return bf16(h * t + h)


def gelu_grad(x):
    t = np.tanh(x * (K0 + K1 * x * x))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * (K0 + 3.0 * K1 * x * x)


def tap_mean(x):
    """The residual's base: 0.25 * ((t0 + t1) + (t2 + t3)) per channel, float32."""
    x = np.asarray(x, dtype=np.float32)
    s = (x[:, 8:12] + x[:, 12:16]) + (x[:, 16:20] + x[:, 20:24])
    return (np.float32(0.25) * s).astype(np.float64)


def forward(params, x, bf16_ops=False):
    """Returns (out [n x 5]: the predicted colour and the confidence as a
    probability, cache).  `bf16_ops` rounds the network's operands to BF16
    (the tap mean stays float32)."""
    P = unpack(params)
    r = bf16 if bf16_ops else (lambda v: np.asarray(v, dtype=np.float64))
    skip = tap_mean(x)
    act = gelu_bf16 if bf16_ops else gelu
    x = r(x)
    h1p = x @ r(P["W1"]).T + P["b1"]
    h1 = act(h1p)
    h2p = r(h1) @ r(P["W2"]).T + P["b2"]
    h2 = act(h2p)
    o = r(h2) @ r(P["W3"]).T + P["b3"]
    out = o.copy()
    out[:, :4] += skip
    out[:, 4] = 1.0 / (1.0 + np.exp(-o[:, 4]))
    return out, (x, h1p, h1, h2p, h2, o)


def loss_and_grads(params, x, y, bf16_inputs=False):
    """Mean loss over the batch and its exact float64 gradient; with
    `bf16_inputs` the network reads the features rounded to BF16, as the GPU
    does (weights and activations stay exact)."""
    P = unpack(params)
    skip = tap_mean(x)
    out, (x, h1p, h1, h2p, h2, o) = forward(params, bf16(x) if bf16_inputs else x)
    n = x.shape[0]
    err = (o[:, :4] + skip) - y
    e = np.max(np.abs(err), axis=1)
    c_t = np.exp(-CONF_K * e)
    c = out[:, 4]
    eps = 1e-12
    loss = np.sum(err ** 2, axis=1) - (c_t * np.log(c + eps) + (1 - c_t) * np.log(1 - c + eps))
    do = np.zeros_like(o)
    do[:, :4] = 2.0 * err / n
    do[:, 4] = (c - c_t) / n
    g = {}
    g["W3"] = do.T @ h2
    g["b3"] = do.sum(0)
    dh2p = (do @ P["W3"]) * gelu_grad(h2p)
    g["W2"] = dh2p.T @ h1
    g["b2"] = dh2p.sum(0)
    dh1p = (dh2p @ P["W2"]) * gelu_grad(h1p)
    g["W1"] = dh1p.T @ x
    g["b1"] = dh1p.sum(0)
    return float(loss.mean()), pack(g)
