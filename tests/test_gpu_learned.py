"""Learned tuner on the GPU: feature kernel, MLP training kernels and BF16
tensor-core inference against the CPU oracle (oracle/mlp_oracle.py), and the
learned replacement of the QoZ tuner end to end."""
import os

import numpy as np
import pytest

import faz_gb300 as F
import faz_gb300.learned as L
from faz_gb300.fields import spectral_field

import oracle.mlp_oracle as M

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _resolved(conf, x):
    """(eb, rng, rel) the library resolves for a REL configuration."""
    xd = x.double()
    rng = float(xd.max() - xd.min())
    return conf.relErrorBound * rng, rng, conf.relErrorBound


@pytest.mark.parametrize("dims,dtype,rel", [((70, 66, 80), torch.float32, 1e-3), ((40, 97, 35), torch.float64, 1e-4),
                                            ((200, 140, 130), torch.float32, 1e-2)])
def test_gpu_features_match_oracle(dims, dtype, rel):
    x = spectral_field(dims, slope=-3.0, aniso=(1, 2, 4), noise=0.02, seed=sum(dims), piecewise=1,
                       device="cuda").to(dtype)
    conf = L.qoz_conf(dims, rel)
    f = L.features(conf, x).cpu().numpy().astype(np.float64)
    eb, rng, rel = _resolved(conf, x)
    ref = M.features(x.cpu().numpy(), eb, rng, rel)
    # float32 outputs of double statistics (sums in a different order)
    assert np.allclose(f, ref, rtol=1e-5, atol=1e-6), np.abs(f - ref).max()


def _random_problem(B, seed):
    rng = np.random.default_rng(seed)
    p = L.init_params(seed)
    p[L.OFF["b1"][0]:L.OFF["b1"][0] + 256] = rng.standard_normal(256) * 0.1
    X = rng.standard_normal((B, 64)).astype(np.float32)
    lab = np.full((B, 8), -1, np.int32)
    for h, (lo, n) in enumerate(L.HEADS):
        lab[:, h] = rng.integers(-1, n, size=B)
    return p, X, lab


@pytest.mark.parametrize("B", [1, 37, 300])
def test_gpu_mlp_forward_backward_match_oracle(B):
    p, X, lab = _random_problem(B, B)
    net = L.MLP(p)
    Xt, Lt = torch.as_tensor(X, device="cuda"), torch.as_tensor(lab, device="cuda")
    h1, h2, z = net.forward(Xt)
    r1, r2, rz = M.forward(p, X)
    assert np.allclose(z.cpu().numpy(), rz, rtol=1e-4, atol=1e-4)
    assert np.allclose(h2.cpu().numpy(), r2, rtol=1e-4, atol=1e-4)
    loss, _ = net.loss_and_grad(Xt, Lt)
    rl, rg = M.loss_and_grad(p, X, lab)
    assert abs(float(loss) - rl.mean()) <= 1e-4 * max(1.0, abs(rl.mean()))
    g = net.g.cpu().numpy().astype(np.float64)
    scale = np.abs(rg).max()
    assert np.abs(g - rg).max() <= 1e-4 * scale, (np.abs(g - rg).max(), scale)


def test_gpu_adam_matches_oracle():
    p, X, lab = _random_problem(64, 5)
    net = L.MLP(p)
    Xt, Lt = torch.as_tensor(X, device="cuda"), torch.as_tensor(lab, device="cuda")
    rp, rm, rv = p.astype(np.float64), np.zeros(p.size), np.zeros(p.size)
    for t in range(1, 4):
        net.loss_and_grad(Xt, Lt)
        g = net.g.cpu().numpy().astype(np.float64)
        net.adam(lr=1e-2, weight_decay=1e-3)
        rp, rm, rv = M.adam(rp, g, rm, rv, t, 1e-2, wd=1e-3)
        assert np.allclose(net.p.cpu().numpy(), rp, rtol=1e-5, atol=1e-6)


def test_gpu_training_fits_a_learnable_rule():
    """The training kernels drive the loss down on labels that are a fixed
    function of the features (every head)."""
    rng = np.random.default_rng(3)
    X = rng.standard_normal((1024, 64)).astype(np.float32)
    lab = np.zeros((1024, 8), np.int32)
    for h, (lo, n) in enumerate(L.HEADS):
        w = rng.standard_normal((64, n))
        lab[:, h] = (X @ w).argmax(1)
    lab[:, 7] = -1
    params, mu, sd = L.train(X, lab, epochs=60, batch=128, lr=3e-3, seed=1)
    net = L.MLP(params)
    _, _, z = net.forward(torch.as_tensor((X - mu) / sd, device="cuda"))
    acc = L.head_accuracy(z.cpu().numpy(), lab)
    assert min(acc) > 0.9, acc


@pytest.mark.parametrize("B", [1, 5, 130])
def test_gpu_tensor_core_inference_matches_oracle(B):
    p, X, _ = _random_problem(B, 11 + B)
    rng = np.random.default_rng(B)
    mu = rng.standard_normal(64).astype(np.float32) * 0.1
    sd = (1 + rng.random(64)).astype(np.float32)
    model = L.TunerModel(p, mu, sd)
    z = model.infer(torch.as_tensor(X, device="cuda")).cpu().numpy()
    ref = M.infer_bf16(p, mu, sd, X)
    # bf16 rounding of hidden activations may differ where the two
    # accumulation orders straddle a rounding boundary
    err = np.abs(z - ref).max()
    assert err <= 2e-2 * max(1.0, np.abs(ref).max()), err
    full = M.forward(p, (X - mu) / sd)[2]
    assert np.abs(z - full).max() <= 0.1 * max(1.0, np.abs(full).max())


def _some_model():
    if os.path.exists(L.DEFAULT_MODEL):
        return L.TunerModel.load()
    p = L.init_params(7)
    return L.TunerModel(p, np.zeros(64, np.float32), np.ones(64, np.float32))


def test_gpu_learned_tune_gives_a_valid_qoz_configuration():
    dims = (96, 128, 112)
    x = spectral_field(dims, slope=-3.0, aniso=(1, 2, 2), noise=0.01, seed=4, device="cuda")
    conf = L.qoz_conf(dims, 1e-3)
    tuned, info = L.learned_tune(conf, x, _some_model(), min_confidence=0.0)
    if info["used_plain"] == 0:
        assert tuned.cmprAlgo == F.ALGO_INTERP
        assert tuned.alpha in L.ALPHAS and tuned.beta in L.BETAS and tuned.alpha <= tuned.beta
        assert len(tuned.interpAlgo_list) == 4
    s = F.SZ_compress(tuned, x)
    out = torch.empty_like(x)
    F.decompress_device(s, out)
    assert (out.double() - x.double()).abs().max().item() <= tuned.absErrorBound


def test_gpu_learned_tune_falls_back_to_the_plain_tuner():
    dims = (80, 72, 90)
    x = spectral_field(dims, slope=-3.5, noise=0.0, seed=8, device="cuda")
    conf = L.qoz_conf(dims, 1e-3)
    tuned, info = L.learned_tune(conf, x, _some_model(), min_confidence=1.01)
    assert info["used_plain"] in (1, 2)
    plain = F.tune_device(conf, x)
    assert F.SZ_compress(tuned, x) == F.SZ_compress(plain, x) == F.SZ_compress(conf, x)


@pytest.mark.skipif(not os.path.exists(L.DEFAULT_MODEL), reason="no committed model")
def test_gpu_committed_network_on_held_out_fields():
    """Held-out fields (a seed outside the training set): the learned tuner
    cuts end-to-end compress time by at least 3x against the QoZ tuner at no
    more than 2 % mean compression-ratio loss, and beats untuned compression."""
    recs, s = L.evaluate(L.TunerModel.load(), 6, seed=4242, reps=2)
    assert s["fields"] == 6
    assert s["speedup"] >= 3.0, s
    assert s["cr_loss_mean"] <= 0.02, s
    assert s["cr_gain_over_untuned"] > 0, s
    for r in recs:
        # the error bound is the quantiser's: every stream decodes within it
        assert r["cr_learned"] > 1.0


DATA = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "faz_gb300", "tuner_c4_dataset.npz")


@pytest.mark.skipif(not os.path.exists(DATA), reason="no committed dataset")
def test_stored_labels_match_the_oracle_tuners():
    """Label audit: the 32 smallest of the 4096 training fields, regenerated
    on the GPU, go through the oracle's QoZ tuner (the tool's -q) and the
    labelling configuration (label_conf) on the CPU.  The labels stored in the
    dataset - per-level interpolator and direction, alpha, beta, Lorenzo or
    not, made by the library's GPU tuners - must equal the oracle's
    decisions."""
    import ast
    import oracle.oracle as O
    from conftest import parse_interp_header
    d = np.load(DATA)
    P = [ast.literal_eval(str(p)) for p in d["params"]]
    Y = d["Y"]
    order = sorted(range(len(P)), key=lambda i: int(np.prod(P[i]["dims"])))[:32]
    O.set_zstd(None)  # the library's tuners sized their trials with the host zstd
    mismatches = []
    for i in order:
        fp = P[i]
        x = L.make_field(fp).cpu().numpy()
        sq, pq = O.compress(L.qoz_conf(fp["dims"], fp["rel"]), x)
        sl, _ = O.compress(L.label_conf(fp["dims"], fp["rel"]), x)
        cq, cl = O.read_stream(sq)[0], O.read_stream(sl)[0]
        lab = np.full(L.N_LABELS, -1, np.int32)
        if cq.cmprAlgo != 0:  # an interpolation stream: its header holds the decisions
            h = parse_interp_header(pq, 3)
            cq.interpAlgo_list, cq.interpDirection_list = h["interp_list"], h["dir_list"]
            cq.alpha, cq.beta = h["alpha"], h["beta"]
            lab = L.labels_of(cq, cl)
            want = Y[i]
        else:  # the QoZ tuner chose Lorenzo: only the Lorenzo label applies
            lab[6] = 1 if cl.cmprAlgo == 0 else 0
            want = np.full(L.N_LABELS, -1, np.int32)
            want[6] = Y[i][6]
        if not np.array_equal(lab[:7], want[:7]):
            mismatches.append((i, lab[:7].tolist(), want[:7].tolist()))
    assert not mismatches, mismatches
