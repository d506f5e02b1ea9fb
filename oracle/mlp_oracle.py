"""CPU oracle of the learned tuner (numpy, float64): feature statistics,
MLP forward / backward / AdamW, and BF16 tensor-core inference emulation.

TEST INFRASTRUCTURE: only tests and the benchmark's baseline import this
module, as the checker of the library's CUDA kernels; the library never
calls it.  The learned tuner has no counterpart in the reference; this is a
restatement of the definitions in include/faz_gb300.h ("Learned tuner").
"""
import numpy as np

N_FEATURES, HIDDEN, N_LOGITS, N_PARAMS = 64, 256, 27, 89371
HEADS = [(0, 4), (4, 4), (8, 4), (12, 4), (16, 5), (21, 4), (25, 2)]
FEB, MAX_BLOCKS = 33, 64


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    out = {}
    for name, shape in (("W1", (HIDDEN, N_FEATURES)), ("b1", (HIDDEN,)), ("W2", (HIDDEN, HIDDEN)), ("b2", (HIDDEN,)),
                        ("W3", (N_LOGITS, HIDDEN)), ("b3", (N_LOGITS,))):
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([d[k].reshape(-1) for k in ("W1", "b1", "W2", "b2", "W3", "b3")])


def forward(p, X):
    w = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    h1 = np.maximum(X @ w["W1"].T + w["b1"], 0)
    h2 = np.maximum(h1 @ w["W2"].T + w["b2"], 0)
    z = h2 @ w["W3"].T + w["b3"]
    return h1, h2, z


def loss_and_grad(p, X, labels):
    """Mean over rows of the summed softmax cross-entropy of the labelled
    heads (label -1 = unlabelled) and its gradient, as a flat array."""
    w = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    B = X.shape[0]
    h1, h2, z = forward(p, X)
    dz = np.zeros_like(z)
    loss = np.zeros(B)
    for h, (lo, n) in enumerate(HEADS):
        lab = np.asarray(labels)[:, h]
        zz = z[:, lo:lo + n]
        m = zz.max(1, keepdims=True)
        lse = m[:, 0] + np.log(np.exp(zz - m).sum(1))
        ok = (lab >= 0) & (lab < n)
        idx = np.where(ok)[0]
        loss[idx] += lse[idx] - zz[idx, lab[idx]]
        sm = np.exp(zz - lse[:, None])
        sm[idx, lab[idx]] -= 1
        sm[~ok] = 0
        dz[:, lo:lo + n] = sm / B
    g = {"W3": dz.T @ h2, "b3": dz.sum(0)}
    dh2 = (dz @ w["W3"]) * (h2 > 0)
    g["W2"], g["b2"] = dh2.T @ h1, dh2.sum(0)
    dh1 = (dh2 @ w["W2"]) * (h1 > 0)
    g["W1"], g["b1"] = dh1.T @ X, dh1.sum(0)
    return loss, pack(g)


def adam(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8, wd=0.0):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    c1, c2 = 1 - b1 ** t, 1 - b2 ** t
    p = p - lr * ((m / c1) / (np.sqrt(v / c2) + eps) + wd * p)
    return p, m, v


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def infer_bf16(p, mean, std, F):
    """Tensor-core inference: BF16 inputs and weights, wide accumulation,
    bias and ReLU in float32, activations rounded to BF16 between layers."""
    w = unpack(p)
    x = bf16((np.asarray(F, np.float32) - np.asarray(mean, np.float32)) / np.asarray(std, np.float32))
    h1 = bf16(np.maximum(x @ bf16(w["W1"]).T + w["b1"], 0))
    h2 = bf16(np.maximum(h1 @ bf16(w["W2"]).T + w["b2"], 0))
    return h2 @ bf16(w["W3"]).T + w["b3"]


def feature_origins(dims):
    allo = [(x, y, z) for x in range(0, dims[0] - FEB + 1, FEB - 1) for y in range(0, dims[1] - FEB + 1, FEB - 1)
            for z in range(0, dims[2] - FEB + 1, FEB - 1)]
    step = max(1, -(-len(allo) // MAX_BLOCKS))
    return allo[::step]


def features(x, eb, rng, rel):
    """The 64 features of a 3-D field `x` (float64 statistics)."""
    x = np.asarray(x)
    dims = x.shape
    org = feature_origins(dims)
    tot = np.zeros((22, 7))
    for (o0, o1, o2) in org:
        b = x[o0:o0 + FEB, o1:o1 + FEB, o2:o2 + FEB].astype(np.float64)
        for cfg in range(21):
            cubic = cfg >= 12
            c = cfg - 12 if cubic else cfg
            s, axis = 1 << (c // 3), c % 3
            reach = 3 * s if cubic else s
            if 2 * reach >= FEB:
                continue
            bb = np.moveaxis(b, axis, 0)
            v = bb[reach:FEB - reach]
            if cubic:
                pred = (-bb[0:FEB - 2 * reach] + 9.0 * bb[2 * s:FEB - 4 * s] + 9.0 * bb[4 * s:FEB - 2 * s]
                        - bb[2 * reach:]) / 16.0
            else:
                pred = (bb[0:FEB - 2 * s] + bb[2 * s:]) * 0.5
            r = v - pred
            ar = np.abs(r)
            tot[cfg] += [ar.sum(), (ar <= eb).sum(), r.size, (r * r).sum(), (ar <= 0.1 * eb).sum(),
                         (ar > 16.0 * eb).sum(), (r ** 4).sum()]
        tot[21] += [b.sum(), (b * b).sum(), b.size, (b[:, :, 1:] == b[:, :, :-1]).sum(), 0, 0, 0]
    f = np.zeros(64)
    S = lambda cfg, k: tot[cfg, k]
    mean_abs = lambda cfg: S(cfg, 0) / S(cfg, 2) if S(cfg, 2) > 0 else 0.0
    frac = lambda cfg, k: S(cfg, k) / S(cfg, 2) if S(cfg, 2) > 0 else 0.0
    lg = lambda v: np.log2(1.0 + v)
    for c in range(21):
        f[c] = lg(mean_abs(c) / eb)
        f[21 + c] = frac(c, 1)
    for a in range(3):
        f[42 + a] = lg(np.sqrt(frac(a, 3)) / eb)
        f[45 + a] = lg(np.sqrt(frac(12 + a, 3)) / eb)
        f[48 + a] = frac(a, 4)
        f[51 + a] = frac(a, 5)
    m2, m4 = frac(2, 3), frac(2, 6)
    f[54] = np.log2(m4 / (m2 * m2) + 1e-12) if m2 > 0 else 0.0
    n = S(21, 2)
    mean = S(21, 0) / n
    var = max(S(21, 1) / n - mean * mean, 0.0)
    f[55] = np.log2(max(rng, 1e-300) / eb)
    f[56] = lg(np.sqrt(var) / eb)
    f[57:60] = np.log2(np.array(dims, dtype=np.float64))
    f[60] = np.log10(rel)
    f[61] = S(21, 3) / n
    f[62] = np.log2(len(org))
    f[63] = (f[9] + f[10] + f[11] - f[0] - f[1] - f[2]) / 3.0
    return f
