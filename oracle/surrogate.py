"""ORACLE (test infrastructure only): numpy restatement of the learned
thick-cell surrogate, used by the tests as the checker of the GPU kernels.
Nothing in the product imports it.

  features / knots / inv_cdf / sample_outcome   the model's input map and its
      inverse-transform sampling (the CUDA header imc_surrogate.cuh states the
      same functions for the transport kernel)
  forward(P, x)                  FP64 forward pass of the 4-64-64-64-64 ReLU net
  forward_bf16(P, x)             the tensor-core pass: BF16 weights and inputs of
                                 every layer (round to nearest even), FP32 sums
  loss_and_grad(P, x, cls, tgt)  mean training loss and its gradient in FP64:
                                 cross entropy of the outcome plus the pinball
                                 losses of the outcome's two quantile heads

The walk the network learns is the in-cell part of Transport.MC's loop
(src/imc_transport.jl:72-193) in mean free paths; its CPU restatement is
orc_surr_walk in imc_oracle.cpp.
"""
import numpy as np

K_IN, K_HID, K_OUT = 4, 64, 64
W1 = 0
B1 = W1 + K_HID * K_IN
W2 = B1 + K_HID
B2 = W2 + K_HID * K_HID
W3 = B2 + K_HID
B3 = W3 + K_HID * K_HID
W4 = B3 + K_HID
B4 = W4 + K_OUT * K_HID
N_PARAMS = B4 + K_OUT
assert N_PARAMS == 12800

QL, QM, QP = 12, 6, 6
NEAR_L = 3
NEAR_M = NEAR_L + QL
FAR_L = NEAR_M + QM
FAR_M = FAR_L + QL
TR_P = FAR_M + QM
TR_M = TR_P + QP
NEAR, FAR, TRUNC = 0, 1, 2
HEADS = {NEAR: ((NEAR_L, QL), (NEAR_M, QM)), FAR: ((FAR_L, QL), (FAR_M, QM)), TRUNC: ((TR_P, QP), (TR_M, QM))}


def unpack(P):
    P = np.asarray(P, dtype=np.float64)
    return [(P[W1:B1].reshape(K_HID, K_IN), P[B1:W2]), (P[W2:B2].reshape(K_HID, K_HID), P[B2:W3]),
            (P[W3:B3].reshape(K_HID, K_HID), P[B3:W4]), (P[W4:B4].reshape(K_OUT, K_HID), P[B4:])]


def features(state):
    """(d_n, d_f, mu', lmax) rows -> network inputs."""
    s = np.asarray(state, dtype=np.float64)
    dn, df, mu, L = s[:, 0], s[:, 1], s[:, 2], s[:, 3]
    g = lambda d: np.minimum(np.log1p(d / np.sqrt(L)) / np.log(11.0), 1.0)
    return np.stack([g(dn), g(df), mu, (np.log10(L) - 2.0) * 0.5], axis=1)


def forward(P, x):
    a = np.asarray(x, dtype=np.float64)
    layers = unpack(P)
    for li, (W, b) in enumerate(layers):
        z = a @ W.T + b
        a = np.maximum(z, 0.0) if li < 3 else z
    return a


def bf16(v):
    """Round float32 values to bfloat16 (nearest, ties to even), as float32."""
    f = np.ascontiguousarray(np.asarray(v, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(f.shape)


def forward_bf16(P, x):
    """The kernel's pass: BF16 operands, products summed in FP32 (order-free
    up to FP32 rounding), FP32 bias and ReLU."""
    a = bf16(np.asarray(x, dtype=np.float32))
    layers = unpack(np.asarray(P, dtype=np.float32))
    for li, (W, b) in enumerate(layers):
        z = (a.astype(np.float64) @ bf16(W.astype(np.float32)).astype(np.float64).T).astype(np.float32)
        z = z + b.astype(np.float32)
        a = bf16(np.maximum(z, 0.0)) if li < 3 else z
    return a


def softplus(v):
    return np.where(v > 20.0, v, np.log1p(np.exp(np.minimum(v, 20.0))))


def level(k, K):
    return (k + 0.5) / K


def knots(h):
    """Monotone knots q_0 = h_0, q_k = q_{k-1} + softplus(h_k) along the last axis."""
    h = np.asarray(h, dtype=np.float64)
    q = np.empty_like(h)
    q[..., 0] = h[..., 0]
    q[..., 1:] = h[..., :1] + np.cumsum(softplus(h[..., 1:]), axis=-1)
    return q


def inv_cdf(q, u):
    """Piecewise-linear quantile function through (level(k), q_k), extended
    linearly by half a knot spacing to u = 0 and u = 1."""
    K = len(q)
    pos = u * K - 0.5
    k = min(max(int(np.floor(pos)), 0), K - 2)
    return q[k] + (pos - k) * (q[k + 1] - q[k])


def expected_collisions(d_n, d_f, lmax):
    return min(1.5 * d_n * d_f, 1.95 * d_n * np.sqrt(lmax), lmax)


def sample_outcome(out, u0, u1, u2):
    m = max(out[0], out[1], out[2])
    e = np.exp(np.asarray(out[:3], dtype=np.float64) - m)
    z = u0 * e.sum()
    c = NEAR if z < e[0] else (FAR if z < e[0] + e[1] else TRUNC)
    (h0, k0), (h1, k1) = HEADS[c]
    return c, inv_cdf(knots(out[h0:h0 + k0]), u1), inv_cdf(knots(out[h1:h1 + k1]), u2)


def class_probs(out):
    o = np.asarray(out, dtype=np.float64)[:, :3]
    e = np.exp(o - o.max(axis=1, keepdims=True))
    return e / e.sum(axis=1, keepdims=True)


def loss_and_grad(P, x, cls, tgt):
    """Mean loss over the samples and d(mean loss)/dP, in FP64."""
    x = np.asarray(x, dtype=np.float64)
    cls = np.asarray(cls)
    tgt = np.asarray(tgt, dtype=np.float64)
    n = len(x)
    layers = unpack(P)
    acts = [x]
    a = x
    for li, (W, b) in enumerate(layers):
        z = a @ W.T + b
        a = np.maximum(z, 0.0) if li < 3 else z
        acts.append(a)
    out = acts[-1]
    dout = np.zeros_like(out)
    p = class_probs(out)
    loss = -np.log(p[np.arange(n), cls]).sum()
    dout[:, :3] = p
    dout[np.arange(n), cls] -= 1.0
    for c in (NEAR, FAR, TRUNC):
        rows = np.nonzero(cls == c)[0]
        if len(rows) == 0:
            continue
        for hh, (h0, K) in enumerate(HEADS[c]):
            h = out[rows, h0:h0 + K]
            q = knots(h)
            tau = level(np.arange(K), K)
            u = tgt[rows, hh][:, None] - q
            loss += np.where(u >= 0.0, tau * u, (tau - 1.0) * u).sum()
            dq = (u < 0.0).astype(np.float64) - tau
            tail = np.cumsum(dq[:, ::-1], axis=1)[:, ::-1]  # tail[:, k] = sum_{j>=k} dq_j
            sg = 1.0 / (1.0 + np.exp(-h[:, 1:]))
            dout[rows, h0 + 1:h0 + K] = tail[:, 1:] * sg
            dout[rows, h0] = tail[:, 0]
    grads = []
    d = dout
    for li in range(3, -1, -1):
        W, _ = layers[li]
        a_in = acts[li]
        grads.append((d.T @ a_in, d.sum(axis=0)))
        if li > 0:
            d = (d @ W) * (acts[li] > 0.0)
    g = np.zeros(N_PARAMS)
    offs = [(W1, B1), (W2, B2), (W3, B3), (W4, B4)]
    for li, (gw, gb) in zip(range(3, -1, -1), grads):
        wo, bo = offs[li]
        g[wo:wo + gw.size] = gw.ravel()
        g[bo:bo + gb.size] = gb
    return loss / n, g / n
