"""TEST INFRASTRUCTURE - FP64 numpy restatement of the learned guiding
surrogate, the checker of the library's BF16 training and inference kernels
(rtx-pathtracer_gb300/csrc/pg_mlp.cu).  Used only by tests/ as the oracle.

The reference has no learned guide; this model is the project's surrogate of
its per-region vMF mixtures (src/PathGuiding.cpp:350-368 fits one mixture per
region).  Definition, shared with the kernels:

  x      = (p - box_lo) / (box_hi - box_lo)                 position in [0, 1]^3
  enc    = 112 features: for i in 0..47 (d = i % 3, k = i // 3) the pair
           sin(2^k pi x_d), cos(2^k pi x_d) at columns 2i, 2i + 1; x at
           columns 96..98; zeros at 99..111
  h1     = relu(W1 enc + b1)     W1: 64 x 112
  h2     = relu(W2 h1 + b2)      W2: 64 x 64
  h3     = relu(W3 h2 + b3)      W3: 64 x 64
  o      = W4 h3 + b4            W4: 80 x 64
  component j (16): logit o[5j], mean direction m = o[5j+1:5j+4] / |.|,
  kappa = exp(clamp(o[5j+4], S_MIN, S_MAX)); pi = softmax(logits)
  q(d)   = sum_j pi_j kappa_j / (2 pi (1 - e^{-2 kappa_j})) e^{kappa_j (mu_j . d - 1)}
  loss   = sum_i w_i (-log q(d_i)) / sum_i w_i                (weighted NLL: KL up to a constant)

Parameters are one flat float vector: W1, b1, W2, b2, W3, b3, W4, b4 (row-major,
output-major).  Training uses Adam (beta1 0.9, beta2 0.999, eps 1e-8) with
bias correction.
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID, N_OUT, N_COMP, N_FREQ = 112, 64, 80, 16, 16
S_MIN, S_MAX = -4.0, 9.0
SHAPES = [("W1", (N_HID, N_IN)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
          ("W3", (N_HID, N_HID)), ("b3", (N_HID,)), ("W4", (N_OUT, N_HID)), ("b4", (N_OUT,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(theta: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = theta[o:o + n].reshape(shape)
        o += n
    return out


def pack(p: dict) -> np.ndarray:
    return np.concatenate([np.asarray(p[name], dtype=np.float64).reshape(-1) for name, _ in SHAPES])


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def encode(pos: np.ndarray, box: np.ndarray) -> np.ndarray:
    """The kernels normalise the position in FP32 as (p - lo) * (1 / (hi - lo));
    the same rounding is reproduced here, the features then in FP64."""
    lo = np.asarray(box[:3], dtype=np.float32)
    inv = (np.float32(1.0) / (np.asarray(box[3:], dtype=np.float32) - lo)).astype(np.float32)
    x = ((np.asarray(pos, dtype=np.float32) - lo) * inv).astype(np.float64)
    enc = np.zeros((x.shape[0], N_IN))
    for i in range(48):
        d, k = i % 3, i // 3
        a = np.pi * (2.0 ** k) * x[:, d]
        enc[:, 2 * i] = np.sin(a)
        enc[:, 2 * i + 1] = np.cos(a)
    enc[:, 96:99] = x
    return enc


def forward(theta: np.ndarray, enc: np.ndarray, act_round=None) -> dict:
    """All layers; act_round (e.g. bf16) is applied to each layer's input as
    the kernels store activations in BF16."""
    p = unpack(theta)
    r = act_round or (lambda a: a)
    a0 = r(enc)
    z1 = a0 @ p["W1"].T + p["b1"]
    h1 = r(np.maximum(z1, 0.0))
    z2 = h1 @ p["W2"].T + p["b2"]
    h2 = r(np.maximum(z2, 0.0))
    z3 = h2 @ p["W3"].T + p["b3"]
    h3 = r(np.maximum(z3, 0.0))
    o = h3 @ p["W4"].T + p["b4"]
    return {"a0": a0, "z1": z1, "h1": h1, "z2": z2, "h2": h2, "z3": z3, "h3": h3, "o": o}


def mixture(o: np.ndarray) -> dict:
    """Mixture parameters from the raw outputs (N x 80)."""
    o = o.reshape(o.shape[0], N_COMP, 5)
    logit = o[:, :, 0]
    lm = logit - logit.max(axis=1, keepdims=True)
    pi = np.exp(lm)
    pi /= pi.sum(axis=1, keepdims=True)
    m = o[:, :, 1:4]
    mn = np.linalg.norm(m, axis=2, keepdims=True)
    mu = m / mn
    s = o[:, :, 4]
    kappa = np.exp(np.clip(s, S_MIN, S_MAX))
    return {"pi": pi, "mu": mu, "kappa": kappa, "m_norm": mn[..., 0], "s": s}


def log_vmf(mu, kappa, d):
    """log of the vMF pdf, per sample and component."""
    cos = np.einsum("njc,nc->nj", mu, d)
    return np.log(kappa) - np.log(2.0 * np.pi) - np.log(-np.expm1(-2.0 * kappa)) + kappa * (cos - 1.0)


def loss_and_dout(o: np.ndarray, d: np.ndarray, w: np.ndarray):
    """Weighted NLL and its gradient with respect to the raw outputs."""
    mx = mixture(o)
    lf = log_vmf(mx["mu"], mx["kappa"], d)
    lp = np.log(mx["pi"]) + lf
    lmax = lp.max(axis=1, keepdims=True)
    logq = lmax[:, 0] + np.log(np.exp(lp - lmax).sum(axis=1))
    W = w.sum()
    loss = float((w * -logq).sum() / W)
    r = np.exp(lp - logq[:, None])          # responsibilities
    sc = (w / W)[:, None]
    dlogit = (mx["pi"] - r) * sc
    cos = np.einsum("njc,nc->nj", mx["mu"], d)
    kap = mx["kappa"]
    # d(-log q)/dm = -r kappa (d - (mu.d) mu) / |m|
    dm = -(r * kap / mx["m_norm"])[..., None] * (d[:, None, :] - cos[..., None] * mx["mu"]) * sc[..., None]
    # d(-log q)/ds = -r (1 - 2 kappa / expm1(2 kappa) + kappa (mu.d - 1)) inside the clamp
    inside = (mx["s"] > S_MIN) & (mx["s"] < S_MAX)
    # 2 kappa / (e^{2 kappa} - 1), written with e^{-2 kappa} so it cannot overflow
    t = 2.0 * kap * np.exp(-2.0 * kap) / -np.expm1(-2.0 * kap)
    ds = -r * (1.0 - t + kap * (cos - 1.0)) * sc * inside
    do = np.zeros((o.shape[0], N_COMP, 5))
    do[:, :, 0] = dlogit
    do[:, :, 1:4] = dm
    do[:, :, 4] = ds
    return loss, do.reshape(o.shape[0], N_OUT)


def loss_and_grad(theta, pos, d, w, box, act_round=None):
    """Loss and parameter gradient (flat), by hand-written backpropagation."""
    p = unpack(theta)
    f = forward(theta, encode(pos, box), act_round)
    loss, do = loss_and_dout(f["o"], np.asarray(d, dtype=np.float64), np.asarray(w, dtype=np.float64))
    g = {}
    g["W4"] = do.T @ f["h3"]
    g["b4"] = do.sum(0)
    dh3 = (do @ p["W4"]) * (f["z3"] > 0)
    g["W3"] = dh3.T @ f["h2"]
    g["b3"] = dh3.sum(0)
    dh2 = (dh3 @ p["W3"]) * (f["z2"] > 0)
    g["W2"] = dh2.T @ f["h1"]
    g["b2"] = dh2.sum(0)
    dh1 = (dh2 @ p["W2"]) * (f["z1"] > 0)
    g["W1"] = dh1.T @ f["a0"]
    g["b1"] = dh1.sum(0)
    return loss, pack(g)


def init_params(seed: int) -> np.ndarray:
    """He-uniform hidden layers, a small output layer, log-kappa biases at
    log 5 (lightpmm's initial kappa); columns of the zero features are 0."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, (o, i) in (("W1", (N_HID, N_IN)), ("W2", (N_HID, N_HID)), ("W3", (N_HID, N_HID))):
        lim = np.sqrt(6.0 / (99 if name == "W1" else i))
        p[name] = rng.uniform(-lim, lim, size=(o, i))
    p["W1"][:, 99:] = 0.0
    lim = np.sqrt(6.0 / N_HID) * 0.1
    p["W4"] = rng.uniform(-lim, lim, size=(N_OUT, N_HID))
    for b in ("b1", "b2", "b3"):
        p[b] = np.zeros(N_HID)
    b4 = np.zeros((N_COMP, 5))
    b4[:, 4] = np.log(5.0)
    # spread the initial mean directions (spherical Fibonacci points)
    j = np.arange(N_COMP) + 0.5
    z = 1.0 - 2.0 * j / N_COMP
    phi = np.pi * (3.0 - np.sqrt(5.0)) * j
    rr = np.sqrt(1.0 - z * z)
    b4[:, 1], b4[:, 2], b4[:, 3] = rr * np.cos(phi), rr * np.sin(phi), z
    p["b4"] = b4.reshape(-1)
    return pack(p).astype(np.float32)


def adam(theta, grad, m, v, t, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (t counts from 1); returns new theta, m, v."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return theta - lr * mh / (np.sqrt(vh) + eps), m, v
