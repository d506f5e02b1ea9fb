"""Learned tuner: a small MLP that predicts the QoZ tuner's decisions from
block statistics of a field, trained on the GPU by the library's own
forward / backward / Adam kernels (include/faz_gb300.h, "Learned tuner").

The network replaces the sampled trial compressions of the QoZ tuner
(include/QoZ/api/impl/SZInterp.hpp:1857-2113 per-level interpolator and
direction, 2194-2543 alpha/beta search); the quantiser enforces the error
bound point by point whatever it predicts, so a wrong prediction costs
compression ratio only.  The plain tuner stays available as its fallback
(low confidence, Lorenzo predicted) and as the judge of its regret.

Training data: seeded synthetic 3-D fields (spectral slope in [-4, -2],
per-axis correlation-length ratios up to 8, 0-5 % white noise, optional
piecewise-constant boxes, relative bounds 1e-4..1e-2), labelled by the GPU
QoZ tuner (bit-identical to the reference's decisions) and the GPU SZ3 tuner
(Lorenzo or interpolation).

    python -m faz_gb300.learned gen   --n 2048 --seed 1 --out data.npz
    python -m faz_gb300.learned train --data data.npz --out tuner_mlp.npz
"""
import argparse
import ctypes
import os
import time

import numpy as np

from .api import FazError, _check, library, tune_device
from .config import ALGO_LORENZO_REG, Config, EB_REL, FAZ_DOUBLE, FAZ_FLOAT, FazConfigStruct

N_FEATURES, HIDDEN, N_LOGITS, N_HEADS, N_LABELS, N_PARAMS = 64, 256, 27, 7, 8, 89371
HEADS = [(0, 4), (4, 4), (8, 4), (12, 4), (16, 5), (21, 4), (25, 2)]   # (first logit, classes)
ALPHAS = (1.0, 1.25, 1.5, 1.75, 2.0)
BETAS = (1.5, 2.0, 3.0, 4.0)
DEFAULT_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuner_mlp.npz")

# parameter offsets in the flat array: W1[H][F], b1, W2[H][H], b2, W3[L][H], b3
OFF = {}
_o = 0
for _name, _n in (("W1", HIDDEN * N_FEATURES), ("b1", HIDDEN), ("W2", HIDDEN * HIDDEN), ("b2", HIDDEN),
                  ("W3", N_LOGITS * HIDDEN), ("b3", N_LOGITS)):
    OFF[_name] = (_o, _n)
    _o += _n
assert _o == N_PARAMS


class TunerChoice(ctypes.Structure):
    _fields_ = [("used_plain", ctypes.c_int), ("confidence", ctypes.c_float), ("p_lorenzo", ctypes.c_float),
                ("logits", ctypes.c_float * N_LOGITS), ("tune_ms", ctypes.c_double)]


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream(device=None):
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _dtype_code(t):
    import torch
    dt = {torch.float32: FAZ_FLOAT, torch.float64: FAZ_DOUBLE}.get(t.dtype)
    if dt is None:
        raise TypeError("FAZ compresses float32 or float64 data")
    return dt


# ----------------------------------------------------------------- features
def features(conf, tensor, out=None):
    """The 64 features of a 3-D CUDA field (a float32 CUDA tensor, or a row of `out`)."""
    import torch
    t = tensor.contiguous()
    if out is None:
        out = torch.empty(N_FEATURES, dtype=torch.float32, device=t.device)
    s = conf.to_struct()
    with torch.cuda.device(t.device):
        _check(library().faz_tuner_features(ctypes.byref(s), _dtype_code(t), _ptr(t), _stream(t.device), _ptr(out)))
    return out


def labels_of(qoz_conf, label_conf_result):
    """Label row (int32[8]): the QoZ tuner's per-level interpolators and
    directions, alpha and beta, and whether the labelling configuration
    (label_conf) chose Lorenzo."""
    lab = np.full(N_LABELS, -1, dtype=np.int32)
    for l, (a, d) in enumerate(zip(qoz_conf.interpAlgo_list[:4], qoz_conf.interpDirection_list[:4])):
        lab[l] = 2 * int(a) + (1 if int(d) != 0 else 0)
    if qoz_conf.alpha in ALPHAS:
        lab[4] = ALPHAS.index(qoz_conf.alpha)
    if qoz_conf.beta in BETAS:
        lab[5] = BETAS.index(qoz_conf.beta)
    if label_conf_result is not None:
        lab[6] = 1 if label_conf_result.cmprAlgo == ALGO_LORENZO_REG else 0
    return lab


# --------------------------------------------------------------------- MLP
def init_params(seed=0):
    """He-initialised weights, zero biases (float32 flat array)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, dtype=np.float32)
    for name, fan_in, shape in (("W1", N_FEATURES, (HIDDEN, N_FEATURES)), ("W2", HIDDEN, (HIDDEN, HIDDEN)),
                                ("W3", HIDDEN, (N_LOGITS, HIDDEN))):
        o, n = OFF[name]
        p[o:o + n] = (rng.standard_normal(shape) * np.sqrt(2.0 / fan_in)).astype(np.float32).reshape(-1)
    return p


class MLP:
    """FP32 parameters, Adam state and activations on the GPU; every step runs
    the library's kernels (faz_mlp_forward / _backward / _adam)."""

    def __init__(self, params, device="cuda"):
        import torch
        self.device = torch.device(device)
        self.p = torch.as_tensor(np.asarray(params, dtype=np.float32)).to(self.device).contiguous()
        self.m = torch.zeros_like(self.p)
        self.v = torch.zeros_like(self.p)
        self.g = torch.zeros_like(self.p)
        self.t = 0

    def _acts(self, B):
        import torch
        f = dict(dtype=torch.float32, device=self.device)
        return torch.empty(B, HIDDEN, **f), torch.empty(B, HIDDEN, **f), torch.empty(B, N_LOGITS, **f)

    def forward(self, X):
        X = X.contiguous()
        h1, h2, z = self._acts(X.shape[0])
        with __import__("torch").cuda.device(self.device):
            _check(library().faz_mlp_forward(_ptr(self.p), _ptr(X), X.shape[0], _ptr(h1), _ptr(h2), _ptr(z),
                                             _stream(self.device)))
        return h1, h2, z

    def loss_and_grad(self, X, labels):
        """Mean summed cross-entropy and its gradient (in self.g)."""
        import torch
        X, labels = X.contiguous(), labels.contiguous()
        h1, h2, z = self.forward(X)
        loss = torch.empty(X.shape[0], dtype=torch.float32, device=self.device)
        with torch.cuda.device(self.device):
            _check(library().faz_mlp_backward(_ptr(self.p), _ptr(X), _ptr(labels), X.shape[0], _ptr(h1), _ptr(h2),
                                              _ptr(z), _ptr(self.g), _ptr(loss), _stream(self.device)))
        return loss.mean(), z

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=1e-4):
        import torch
        self.t += 1
        with torch.cuda.device(self.device):
            _check(library().faz_mlp_adam(_ptr(self.p), _ptr(self.g), _ptr(self.m), _ptr(self.v), N_PARAMS, lr,
                                          beta1, beta2, eps, self.t, weight_decay, _stream(self.device)))

    def params(self):
        return self.p.cpu().numpy().copy()


def head_predictions(logits):
    """Per-head argmax (numpy int array [B, 7])."""
    z = np.asarray(logits)
    return np.stack([z[:, lo:lo + n].argmax(1) for lo, n in HEADS], axis=1)


def head_accuracy(logits, labels):
    pred = head_predictions(logits)
    lab = np.asarray(labels)[:, :N_HEADS]
    out = []
    for h in range(N_HEADS):
        m = lab[:, h] >= 0
        out.append(float((pred[m, h] == lab[m, h]).mean()) if m.any() else float("nan"))
    return out


VAL_FRACTION, SPLIT_SEED = 0.125, 4242


def split(n, val_fraction=VAL_FRACTION, seed=SPLIT_SEED):
    """Deterministic train / validation indices of a dataset of n rows: the
    network is fitted on the first, its accuracy is quoted on the second."""
    perm = np.random.default_rng(seed).permutation(n)
    nv = int(round(n * val_fraction))
    return np.sort(perm[nv:]), np.sort(perm[:nv])


def majority_rates(labels):
    """Per head, the accuracy of always answering its most frequent label."""
    Y = np.asarray(labels)
    out = []
    for h, (lo, n) in enumerate(HEADS):
        lab = Y[:, h][Y[:, h] >= 0]
        out.append(float(np.bincount(lab, minlength=n).max() / lab.size) if lab.size else float("nan"))
    return out


def train(X, labels, epochs=40, batch=256, lr=2e-3, seed=0, weight_decay=1e-4, device="cuda", log=None):
    """Train from scratch on standardised features; returns (params, mean, std).
    40 epochs of the cosine schedule: longer runs fit the training fields
    better and the held-out ones worse (the alpha / beta heads fall below the
    majority rate by 300 epochs)."""
    import torch
    X = np.asarray(X, dtype=np.float32)
    mu = X.mean(0).astype(np.float32)
    sd = X.std(0).astype(np.float32)
    sd[sd < 1e-6] = 1.0
    Xs = torch.as_tensor((X - mu) / sd, device=device)
    L = torch.as_tensor(np.asarray(labels, dtype=np.int32), device=device)
    net = MLP(init_params(seed), device)
    rng = np.random.default_rng(seed)
    n = X.shape[0]
    for ep in range(epochs):
        perm = torch.as_tensor(rng.permutation(n), device=device)
        lr_ep = lr * 0.5 * (1 + np.cos(np.pi * ep / epochs))
        tot = 0.0
        for i in range(0, n, batch):
            idx = perm[i:i + batch]
            loss, _ = net.loss_and_grad(Xs[idx], L[idx])
            net.adam(lr=float(lr_ep), weight_decay=weight_decay)
            tot += float(loss) * idx.numel()
        if log and (ep % 10 == 0 or ep == epochs - 1):
            log(f"epoch {ep} loss {tot / n:.4f}")
    return net.params(), mu, sd


# --------------------------------------------------------------- inference
class TunerModel:
    """Trained network: FP32 parameters plus feature standardisation; the
    device copy (BF16 weights for the tensor cores) is made on first use."""

    def __init__(self, params, mean, std):
        self.params = np.ascontiguousarray(params, dtype=np.float32)
        self.mean = np.ascontiguousarray(mean, dtype=np.float32)
        self.std = np.ascontiguousarray(std, dtype=np.float32)
        if self.params.size != N_PARAMS or self.mean.size != N_FEATURES or self.std.size != N_FEATURES:
            raise ValueError("tuner model arrays have the wrong sizes")
        self._handles = {}

    @classmethod
    def load(cls, path=DEFAULT_MODEL):
        z = np.load(path)
        return cls(z["params"], z["mean"], z["std"])

    def save(self, path, **extra):
        np.savez_compressed(path, params=self.params, mean=self.mean, std=self.std, **extra)

    def handle(self, device=None):
        import torch
        dev = torch.cuda.current_device() if device is None else torch.device(device).index
        if dev not in self._handles:
            with torch.cuda.device(dev):
                h = library().faz_tuner_model_create(self.params.ctypes.data, self.mean.ctypes.data,
                                                     self.std.ctypes.data)
            if not h:
                raise FazError(-3, library().faz_last_error().decode(errors="replace"))
            self._handles[dev] = h
        return ctypes.c_void_p(self._handles[dev])

    def infer(self, F):
        """Logits of feature rows F ([B, 64] float32 CUDA) on the tensor cores."""
        import torch
        F = F.reshape(-1, N_FEATURES).contiguous()
        z = torch.empty(F.shape[0], N_LOGITS, dtype=torch.float32, device=F.device)
        with torch.cuda.device(F.device):
            _check(library().faz_tuner_infer(self.handle(F.device), _ptr(F), F.shape[0], _ptr(z), _stream(F.device)))
        return z

    def __del__(self):
        try:
            for h in self._handles.values():
                library().faz_tuner_model_destroy(ctypes.c_void_p(h))
        except Exception:
            pass


def learned_tune(conf, tensor, model=None, min_confidence=0.0):
    """The learned replacement of the QoZ tuner on a CUDA field: returns
    (tuned Config, choice dict).  `conf` must select the QoZ tuner (QoZ = 1)."""
    import torch
    model = model or TunerModel.load()
    t = tensor.contiguous()
    s, ch = conf.to_struct(), TunerChoice()
    with torch.cuda.device(t.device):
        _check(library().faz_learned_tune(ctypes.byref(s), _dtype_code(t), _ptr(t), _stream(t.device),
                                          model.handle(t.device), float(min_confidence), ctypes.byref(ch)))
    info = {"used_plain": ch.used_plain, "confidence": ch.confidence, "p_lorenzo": ch.p_lorenzo,
            "tune_ms": ch.tune_ms, "logits": list(ch.logits)}
    return Config.from_struct(s), info


# ------------------------------------------------------------------- data
def field_params(rng):
    """One draw of the synthetic field distribution."""
    dims = tuple(int(v) for v in rng.integers(16, 33, size=3) * 8)      # 128..256
    return dict(dims=dims, slope=float(rng.uniform(-4, -2)), aniso=tuple(float(2 ** rng.uniform(0, 3)) for _ in range(3)),
                noise=float(rng.uniform(0, 0.05)), piecewise=int(rng.integers(1, 5)) if rng.random() < 0.25 else 0,
                rel=float(10 ** rng.uniform(-4, -2)), seed=int(rng.integers(0, 2 ** 31 - 1)))


def make_field(fp, device="cuda"):
    from .fields import spectral_field
    return spectral_field(fp["dims"], slope=fp["slope"], aniso=fp["aniso"], noise=fp["noise"], seed=fp["seed"],
                          piecewise=fp["piecewise"], device=device)


def qoz_conf(dims, rel):
    c = Config(*dims)
    c.errorBoundMode, c.relErrorBound, c.QoZ = EB_REL, rel, 1
    return c


def label_conf(dims, rel):
    """The labelling configuration: QoZ = 0 with the INI [AlgoSettings]
    autoTuningRate = predictorTuningRate = 0.005, maxStep = 32,
    levelwisePredictionSelection = 4, sampleBlockSize = 32, testLorenzo = 1.
    Its interpolation decisions equal the QoZ tuner's (the same values are the
    QoZ defaults for 3-D data); at relative bounds <= 1e-3 it also tries the
    Lorenzo candidate, which gives the Lorenzo label."""
    c = Config(*dims)
    c.errorBoundMode, c.relErrorBound = EB_REL, rel
    c.autoTuningRate = c.predictorTuningRate = 0.005
    c.maxStep, c.levelwisePredictionSelection, c.sampleBlockSize, c.testLorenzo = 32, 4, 32, 1
    return c


def generate(n, seed, device="cuda", log=None):
    """Features, labels and field parameters of n synthetic fields (a field
    the tuners reject, e.g. for more than 65536 quantisation bins, is skipped)."""
    import torch
    rng = np.random.default_rng(seed)
    X, Y, P = [], [], []
    t0 = time.time()
    for i in range(n):
        fp = field_params(rng)
        x = make_field(fp, device)
        try:
            q = tune_device(qoz_conf(fp["dims"], fp["rel"]), x)
            z = tune_device(label_conf(fp["dims"], fp["rel"]), x)
        except FazError as e:
            if log:
                log(f"field {i} skipped: {e}")
            continue
        X.append(features(qoz_conf(fp["dims"], fp["rel"]), x).cpu().numpy())
        Y.append(labels_of(q, z))
        P.append(fp)
        del x
        if log and (i % 256 == 0 or i == n - 1):
            log(f"field {i} {time.time() - t0:.1f}s")
    torch.cuda.synchronize()
    return np.array(X, np.float32).reshape(-1, N_FEATURES), np.array(Y, np.int32).reshape(-1, N_LABELS), P


def relabel(path, device="cuda", log=None):
    """Lorenzo labels of a saved dataset recomputed with label_conf on the
    regenerated fields; returns (X, Y, params, stats)."""
    import ast
    import torch
    d = np.load(path)
    X, Y, P = d["X"], d["Y"].copy(), d["params"]
    changed = interp_diff = lorenzo = 0
    for i, ps in enumerate(P):
        fp = ast.literal_eval(str(ps))
        x = make_field(fp, device)
        z = tune_device(label_conf(fp["dims"], fp["rel"]), x)
        lab = 1 if z.cmprAlgo == ALGO_LORENZO_REG else 0
        lorenzo += lab
        changed += int(Y[i, 6] != lab)
        Y[i, 6] = lab
        if not lab:
            zl = labels_of(z, None)
            interp_diff += int(not np.array_equal(zl[:6], Y[i, :6]))
        del x
        if log and (i % 512 == 0 or i == len(P) - 1):
            log(f"field {i}: {lorenzo} Lorenzo, {changed} changed, {interp_diff} interpolation labels differ")
    torch.cuda.synchronize()
    return X, Y, P, dict(lorenzo=lorenzo, changed=changed, interp_diff=interp_diff, n=len(P))


def _timed(fn, reps=3):
    import torch
    best, out = None, None
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        best = t if best is None else min(best, t)
    return best, out


def evaluate(model, n, seed, device="cuda", min_confidence=0.0, reps=3, log=None):
    """Learned vs plain QoZ autotune on n held-out fields, end to end through
    compress_device (tuning + compression + zstd).  Also compresses each field
    untuned (ALGO_INTERP, cubic, direction 0: the method without a tuner).
    Returns per-field records and a summary."""
    from .api import compress_device
    from .config import ALGO_INTERP
    rng = np.random.default_rng(seed)
    recs = []
    for i in range(n):
        fp = field_params(rng)
        x = make_field(fp, device)
        qc = qoz_conf(fp["dims"], fp["rel"])
        try:
            t_plain, s_plain = _timed(lambda: compress_device(qc, x), reps)
        except FazError as e:
            if log:
                log(f"field {i} skipped: {e}")
            continue

        def learned():
            tuned, info = learned_tune(qc, x, model, min_confidence)
            return compress_device(tuned, x), info
        t_learn, (s_learn, info) = _timed(learned, reps)
        uc = qoz_conf(fp["dims"], fp["rel"])
        uc.QoZ, uc.cmprAlgo = 0, ALGO_INTERP
        s_untuned = compress_device(uc, x)
        nbytes = x.numel() * x.element_size()
        recs.append(dict(dims=fp["dims"], rel=fp["rel"], t_plain=t_plain, t_learned=t_learn,
                         cr_plain=nbytes / len(s_plain), cr_learned=nbytes / len(s_learn),
                         cr_untuned=nbytes / len(s_untuned), same_stream=s_plain == s_learn,
                         used_plain=info["used_plain"], confidence=info["confidence"]))
        if log:
            r = recs[-1]
            log(f"field {i} {fp['dims']} rel {fp['rel']:.1e}: plain {t_plain * 1e3:.1f} ms cr {r['cr_plain']:.3f} | "
                f"learned {t_learn * 1e3:.1f} ms cr {r['cr_learned']:.3f} ({'same' if r['same_stream'] else 'differs'}, "
                f"fallback {r['used_plain']}) | untuned cr {r['cr_untuned']:.3f}")
    if not recs:
        return recs, {}
    tp = sum(r["t_plain"] for r in recs)
    tl = sum(r["t_learned"] for r in recs)
    loss = [1 - r["cr_learned"] / r["cr_plain"] for r in recs]
    gain = [r["cr_learned"] / r["cr_untuned"] - 1 for r in recs]
    summary = dict(fields=len(recs), plain_ms=tp * 1e3, learned_ms=tl * 1e3, speedup=tp / tl,
                   cr_loss_mean=float(np.mean(loss)), cr_loss_max=float(np.max(loss)),
                   same_stream=float(np.mean([r["same_stream"] for r in recs])),
                   fallback=float(np.mean([r["used_plain"] != 0 for r in recs])),
                   cr_gain_over_untuned=float(np.mean(gain)))
    return recs, summary


def _main():
    ap = argparse.ArgumentParser(prog="python -m faz_gb300.learned")
    sub = ap.add_subparsers(dest="cmd", required=True)
    g = sub.add_parser("gen")
    g.add_argument("--n", type=int, default=2048)
    g.add_argument("--seed", type=int, default=1)
    g.add_argument("--out", required=True)
    e = sub.add_parser("eval")
    e.add_argument("--model", default=DEFAULT_MODEL)
    e.add_argument("--n", type=int, default=64)
    e.add_argument("--seed", type=int, default=999)
    r = sub.add_parser("relabel")
    r.add_argument("--data", required=True)
    r.add_argument("--out", required=True)
    t = sub.add_parser("train")
    t.add_argument("--data", required=True, nargs="+")
    t.add_argument("--out", default=DEFAULT_MODEL)
    t.add_argument("--epochs", type=int, default=40)
    t.add_argument("--seed", type=int, default=0)
    a = ap.parse_args()
    if a.cmd == "gen":
        X, Y, P = generate(a.n, a.seed, log=print)
        np.savez_compressed(a.out, X=X, Y=Y, params=np.array([repr(p) for p in P]))
    elif a.cmd == "relabel":
        X, Y, P, stats = relabel(a.data, log=print)
        np.savez_compressed(a.out, X=X, Y=Y, params=P)
        print(stats)
    elif a.cmd == "eval":
        _, summary = evaluate(TunerModel.load(a.model), a.n, a.seed, log=print)
        print(summary)
    else:
        X = np.concatenate([np.load(f)["X"] for f in a.data])
        Y = np.concatenate([np.load(f)["Y"] for f in a.data])
        tr, va = split(len(X))
        params, mu, sd = train(X[tr], Y[tr], epochs=a.epochs, seed=a.seed, log=print)
        m = TunerModel(params, mu, sd)
        import torch
        net = MLP(params)
        acc = {}
        for name, idx in (("train", tr), ("validation", va)):
            _, _, z = net.forward(torch.as_tensor((X[idx] - mu) / sd, device="cuda"))
            acc[name] = head_accuracy(z.cpu().numpy(), Y[idx])
            print(f"{name} accuracy per head ({len(idx)} fields)", [round(v, 4) for v in acc[name]])
        maj = majority_rates(Y[va])
        print("validation majority rate per head", [round(v, 4) for v in maj])
        m.save(a.out, val_accuracy=np.array(acc["validation"]), train_accuracy=np.array(acc["train"]),
               val_majority=np.array(maj), val_fraction=np.array(VAL_FRACTION), split_seed=np.array(SPLIT_SEED))


if __name__ == "__main__":
    _main()
