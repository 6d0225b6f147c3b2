"""CPU oracle for the noise-surrogate network (TEST INFRASTRUCTURE ONLY).

The reference has no learned component: the surrogate that maps noise
parameters to a fixed circuit's outcome distribution is an extension of
this engine, trained on distributions that the batched simulator
produces.  This module restates the network's arithmetic in numpy so the
GPU kernels can be checked against it (forward, loss, gradients, Adam,
ensemble statistics).  There is no reference implementation to pin it to;
its own checks are finite differences (``tests/test_mlp_oracle.py``).

Network, per ensemble member (all widths fixed by the kernels):
    x (6 features, zero-padded to 64) -> 256 -> 256 -> 256 -> 1024
    hidden layers  h = gelu(W h_prev + b)   (tanh form of GELU)
    output         q = softmax(W4 h3 + b4)
    loss           mean over the batch of KL(t || q) = sum_j t_j (log t_j - log q_j)
Matrix products take BF16-rounded operands (round to nearest even) and
accumulate in FP32 or better; weights are FP32 master copies.

Only ``tests/`` and ``bench.py``'s CPU legs may import this module.
"""
import numpy as np

WIDTHS = (64, 256, 256, 256, 1024)      # input (padded), three hidden layers, outcomes
N_FEATURES = 6
GELU_C = 0.7978845608028654             # sqrt(2 / pi)
GELU_A = 0.044715


def bf16(x):
    """Round float32 values to the nearest bfloat16 (ties to even); returns float32."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out).reshape(a.shape)


def gelu(u):
    return 0.5 * u * (1.0 + np.tanh(GELU_C * (u + GELU_A * u ** 3)))


def gelu_grad(u):
    t = np.tanh(GELU_C * (u + GELU_A * u ** 3))
    return 0.5 * (1.0 + t) + 0.5 * u * (1.0 - t * t) * GELU_C * (1.0 + 3.0 * GELU_A * u * u)


def init_params(seed, widths=WIDTHS):
    """He-style initialisation (normal, std sqrt(2 / fan_in) over the 6 real inputs for layer 1)."""
    rng = np.random.default_rng(seed)
    params = []
    for li in range(4):
        fan_in, fan_out = widths[li], widths[li + 1]
        real_in = N_FEATURES if li == 0 else fan_in
        std = np.sqrt(2.0 / real_in) if li < 3 else np.sqrt(1.0 / real_in)
        W = np.zeros((fan_out, fan_in), dtype=np.float32)
        W[:, :real_in] = rng.normal(0.0, std, size=(fan_out, real_in))
        b = np.zeros(fan_out, dtype=np.float32)
        params += [W, b]
    return params


def pad_features(x):
    x = np.asarray(x, dtype=np.float32)
    out = np.zeros((x.shape[0], WIDTHS[0]), dtype=np.float32)
    out[:, :x.shape[1]] = x
    return out


def _exact(x):
    return np.asarray(x, dtype=np.float64)


def forward(params, x16, rnd=bf16, dtype=np.float32):
    """Returns (pre-activations, activations, softmax output).

    ``rnd`` rounds the matrix-product operands (BF16 by default; ``_exact``
    for the finite-difference checks, with ``dtype`` float64).
    """
    pres, acts = [], [x16]
    h = x16
    for li in range(4):
        W, b = params[2 * li], params[2 * li + 1]
        u = (rnd(h).astype(np.float64) @ rnd(W).astype(np.float64).T + b).astype(dtype)
        pres.append(u)
        if li < 3:
            h = gelu(u.astype(np.float64)).astype(dtype)
            acts.append(h)
    z = pres[-1].astype(np.float64)
    z = z - z.max(axis=1, keepdims=True)
    e = np.exp(z)
    q = e / e.sum(axis=1, keepdims=True)
    return pres, acts, q


def kl_loss(q, t):
    t = np.asarray(t, dtype=np.float64)
    with np.errstate(divide='ignore', invalid='ignore'):
        terms = np.where(t > 0, t * (np.log(np.where(t > 0, t, 1.0)) - np.log(q)), 0.0)
    return float(terms.sum(axis=1).mean())


def backward(params, x16, t, rnd=bf16, dtype=np.float32):
    """Loss and gradients (same order as params) of the mean KL over the batch."""
    pres, acts, q = forward(params, x16, rnd, dtype)
    B = x16.shape[0]
    loss = kl_loss(q, t)
    grads = [None] * 8
    d = ((q - t) / B).astype(dtype)                 # dL/dz
    for li in range(3, -1, -1):
        W = params[2 * li]
        grads[2 * li] = (rnd(d).astype(np.float64).T @ rnd(acts[li]).astype(np.float64)).astype(dtype)
        grads[2 * li + 1] = rnd(d).astype(np.float64).sum(axis=0).astype(dtype)
        if li > 0:
            dh = rnd(d).astype(np.float64) @ rnd(W).astype(np.float64)
            d = (dh * gelu_grad(pres[li - 1].astype(np.float64))).astype(dtype)
    return loss, grads


def adam(params, grads, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step in place (FP32 state); ``step`` counts from 1."""
    c1 = 1.0 - beta1 ** step
    c2 = 1.0 - beta2 ** step
    for p, g, mm, vv in zip(params, grads, m, v):
        mm[...] = beta1 * mm + (1 - beta1) * g
        vv[...] = beta2 * vv + (1 - beta2) * g * g
        p[...] = p - lr * (mm / c1) / (np.sqrt(vv / c2) + eps)


def ensemble_stats(qs):
    """Mean distribution of the members and their spread (mean total-variation distance to the mean)."""
    qs = np.asarray(qs, dtype=np.float64)
    mean = qs.mean(axis=0)
    spread = 0.5 * np.abs(qs - mean[None]).sum(axis=2).mean(axis=0)
    return mean, spread


def tv(p, q):
    return 0.5 * np.abs(np.asarray(p, dtype=np.float64) - np.asarray(q, dtype=np.float64)).sum(axis=-1)
