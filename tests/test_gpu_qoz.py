"""GPU QoZ tuner (QoZ = 1, the faz tool's -q) against the oracle and the
reference's -q streams: the per-level interpolators and directions, alpha and
beta, and the resulting interpolation stream."""
import numpy as np
import pytest

import faz_gb300 as F
from faz_gb300.fields import spectral_field
from conftest import (cli_config, golden_case, golden_input, golden_manifest, golden_stream, mask_first_size,
                      mask_fast_frontend_padding,
                      parse_interp_header)

import oracle.oracle as O

pytestmark = pytest.mark.gpu

QOZ_CASES = [c["name"] for c in golden_manifest() if c["ini"] is None and "-q" in c["flags"]]
KEYS = ("interp", "direction", "alpha", "beta", "maxStep", "interp_list", "dir_list")


@pytest.fixture(scope="module", autouse=True)
def system_zstd():
    O.set_zstd(None)
    yield


@pytest.mark.parametrize("name", QOZ_CASES)
def test_gpu_qoz_matches_reference(name):
    case = golden_case(name)
    x = golden_input(case)
    N = len(case["dims"])
    stream = F.SZ_compress(cli_config(case), x)
    _, p = O.read_stream(stream)
    _, rp = O.read_stream(golden_stream(case))
    h, hr = parse_interp_header(p, N), parse_interp_header(rp, N)
    assert {k: h[k] for k in KEYS} == {k: hr[k] for k in KEYS}
    assert p == rp
    ref, _ = O.compress(cli_config(case), x)
    assert mask_first_size(stream) == mask_first_size(ref)
    dec, c2 = F.SZ_decompress(None, stream, dtype=x.dtype)
    assert np.abs(dec.astype(np.float64) - x.astype(np.float64)).max() <= c2.absErrorBound


QOZ_RANDOM = [
    ((64, 80, 96), 1e-3, np.float32, -3.0),
    ((70, 70, 70), 1e-4, np.float32, -3.5),
    ((96, 64, 80), 5e-3, np.float32, -2.5),
    ((300, 420), 1e-3, np.float32, -3.0),
    ((50, 60, 70), 1e-6, np.float64, -3.0),
]


@pytest.mark.parametrize("dims,rel,dtype,slope", QOZ_RANDOM)
def test_gpu_qoz_matches_oracle(dims, rel, dtype, slope):
    conf = F.Config(*dims)
    conf.QoZ = 1
    conf.errorBoundMode = F.EB_REL
    conf.relErrorBound = rel
    x = spectral_field(dims, slope=slope, noise=0.01, seed=sum(dims) + 7, dtype=dtype)
    stream = F.SZ_compress(conf, x)
    ref, ref_payload = O.compress(conf, x)
    _, p = O.read_stream(stream)
    assert parse_interp_header(p, len(dims)) == parse_interp_header(ref_payload, len(dims))
    assert p == ref_payload
    assert mask_first_size(stream) == mask_first_size(ref)


# Tuning from the configuration's own rates (QoZ = 0, predictorTuningRate in
# (0, 1)): levelwisePredictionSelection 0 picks one interpolator and direction
# for every level by CompressTest ratio; a positive value picks per level.
RATE_RANDOM = [
    ((64, 80, 96), 1e-3, np.float32, 0, 0),
    ((56, 64, 72), 5e-3, np.float32, 3, 16),
    ((300, 420), 1e-3, np.float32, 0, 0),
    ((48, 56, 64), 1e-5, np.float64, 0, 0),
]


@pytest.mark.parametrize("dims,rel,dtype,levelwise,max_step", RATE_RANDOM)
def test_gpu_rate_tuning_matches_oracle(dims, rel, dtype, levelwise, max_step):
    conf = F.Config(*dims)
    conf.errorBoundMode = F.EB_REL
    conf.relErrorBound = rel
    conf.autoTuningRate = conf.predictorTuningRate = 0.01
    conf.levelwisePredictionSelection = levelwise
    conf.maxStep = max_step
    x = spectral_field(dims, slope=-3.0, noise=0.01, seed=sum(dims) + 11, dtype=dtype)
    stream = F.SZ_compress(conf, x)
    ref, ref_payload = O.compress(conf, x)
    _, p = O.read_stream(stream)
    assert parse_interp_header(p, len(dims)) == parse_interp_header(ref_payload, len(dims))
    assert p == ref_payload
    assert mask_first_size(stream) == mask_first_size(ref)


def test_gpu_2d_lorenzo_candidate_matches_oracle():
    """testLorenzo on 2-D data: the 2-D general frontend over the sampled
    blocks; a sum of 1-D functions selects Lorenzo."""
    dims = (300, 400)
    rng = np.random.default_rng(7)
    base = np.cumsum(rng.standard_normal((dims[0], 1)), 0) + np.cumsum(rng.standard_normal((1, dims[1])), 1)
    for x in (base.astype(np.float32), spectral_field(dims, slope=-2.5, noise=0.05, seed=5)):
        conf = F.Config(*dims)
        conf.errorBoundMode = F.EB_REL
        conf.relErrorBound = 1e-3
        conf.autoTuningRate = conf.predictorTuningRate = 0.01
        conf.testLorenzo = 1
        stream = F.SZ_compress(conf, x)
        ref, ref_payload = O.compress(conf, x)
        c1, p = O.read_stream(stream)
        c2, _ = O.read_stream(ref)
        assert (c1.cmprAlgo, c1.alpha, c1.beta, c1.blockSize, c1.quantbinCnt) == \
            (c2.cmprAlgo, c2.alpha, c2.beta, c2.blockSize, c2.quantbinCnt)
        assert p == ref_payload
    assert c1.cmprAlgo == 2 and O.read_stream(F.SZ_compress(conf, base.astype(np.float32)))[0].cmprAlgo == 0


def _sum_of_planes(shape, noise, seed, dtype):
    """f(i,j) + g(j,k) + h(i,k) plus white noise: the 3-D Lorenzo predictor
    reproduces sums of 2-D functions, so the tuner's Lorenzo candidate wins."""
    rng = np.random.default_rng(seed)
    base = (rng.standard_normal((shape[0], shape[1], 1)) + rng.standard_normal((1, shape[1], shape[2])) +
            rng.standard_normal((shape[0], 1, shape[2])))
    return (base + noise * rng.standard_normal(shape) * (base.max() - base.min())).astype(dtype)


# the learned tuner's labelling configuration (testLorenzo = 1): at relative
# bounds <= 1e-3 the Lorenzo candidate runs against the best alpha/beta point
LABEL_CASES = [
    ("planes", (64, 64, 64), 1e-3, np.float32, 1e-3),
    ("planes", (64, 72, 80), 1e-4, np.float32, 1e-5),
    ("planes", (48, 56, 64), 1e-3, np.float64, 1e-3),
    ("spectral", (64, 96, 80), 1e-3, np.float32, 0.01),
    ("spectral", (80, 64, 72), 2e-4, np.float32, 0.02),
]


@pytest.mark.parametrize("kind,dims,rel,dtype,noise", LABEL_CASES)
def test_gpu_lorenzo_candidate_matches_oracle(kind, dims, rel, dtype, noise):
    conf = F.Config(*dims)
    conf.errorBoundMode = F.EB_REL
    conf.relErrorBound = rel
    conf.autoTuningRate = conf.predictorTuningRate = 0.005
    conf.maxStep = 32
    conf.levelwisePredictionSelection = 4
    conf.sampleBlockSize = 32
    conf.testLorenzo = 1
    if kind == "planes":
        x = _sum_of_planes(dims, noise, sum(dims), dtype)
    else:
        x = spectral_field(dims, slope=-3.0, noise=noise, seed=sum(dims) + 5, dtype=dtype)
    stream = F.SZ_compress(conf, x)
    ref, ref_payload = O.compress(conf, x)
    c1, p = O.read_stream(stream)
    c2, _ = O.read_stream(ref)
    for f in ("cmprAlgo", "alpha", "beta", "interpAlgo", "interpDirection", "quantbinCnt", "blockSize", "pred_dim"):
        assert getattr(c1, f) == getattr(c2, f), f
    if kind == "planes":
        assert c1.cmprAlgo == 0  # ALGO_LORENZO_REG
        assert mask_fast_frontend_padding(p, x.itemsize) == mask_fast_frontend_padding(ref_payload, x.itemsize)
    else:
        assert p == ref_payload
    dec, c3 = F.SZ_decompress(None, stream, dtype=x.dtype)
    assert np.abs(dec.astype(np.float64) - x.astype(np.float64)).max() <= c3.absErrorBound


# predictor tuning alone (autoTuningRate 0): the interpolation and Lorenzo
# candidates compared by the compression ratio of CompressTests
PT_CASES = [
    ((64, 80, 96), 1e-3, np.float32, 4, 32, 1),
    ((56, 64, 72), 1e-4, np.float32, 0, 0, 1),
    ((300, 420), 1e-3, np.float32, 6, 64, 0),
    ((48, 56, 64), 1e-5, np.float64, 0, 0, 0),
]
# without autoTuningRate a 2-D field keeps sampleBlockSize 64, above the
# interpolation block (32) the GPU tuner's sampled blocks need: set it


@pytest.mark.parametrize("dims,rel,dtype,levelwise,max_step,test_lorenzo", PT_CASES)
def test_gpu_predictor_tuning_only_matches_oracle(dims, rel, dtype, levelwise, max_step, test_lorenzo):
    conf = F.Config(*dims)
    conf.errorBoundMode = F.EB_REL
    conf.relErrorBound = rel
    conf.predictorTuningRate = 0.01
    conf.levelwisePredictionSelection = levelwise
    conf.maxStep = max_step
    conf.testLorenzo = test_lorenzo
    if len(dims) == 2:
        conf.sampleBlockSize = 32
    x = spectral_field(dims, slope=-2.5, noise=0.02, seed=sum(dims) + 13, dtype=dtype)
    stream = F.SZ_compress(conf, x)
    ref, ref_payload = O.compress(conf, x)
    c1, p = O.read_stream(stream)
    c2, _ = O.read_stream(ref)
    for f in ("cmprAlgo", "interpAlgo", "interpDirection", "alpha", "beta", "quantbinCnt", "blockSize", "pred_dim"):
        assert getattr(c1, f) == getattr(c2, f), f
    if c1.cmprAlgo == 0 and len(dims) == 3:
        assert mask_fast_frontend_padding(p, x.itemsize) == mask_fast_frontend_padding(ref_payload, x.itemsize)
    else:
        assert p == ref_payload


def test_gpu_tuner_rejects_sampled_blocks_above_the_interpolation_block():
    """2-D predictor tuning without autoTuningRate keeps sampleBlockSize 64
    (above interpBlockSize 32): the GPU tuner fails loudly."""
    conf = F.Config(300, 420)
    conf.errorBoundMode = F.EB_REL
    conf.relErrorBound = 1e-3
    conf.predictorTuningRate = 0.01
    with pytest.raises(F.FazError, match="interpBlockSize"):
        F.SZ_compress(conf, spectral_field((300, 420), slope=-2.5, seed=3))


def _flat_outside(dims, frac, seed):
    x = spectral_field(dims, slope=-3.0, noise=0.02, seed=seed)
    m = np.zeros(dims, bool)
    m[tuple(slice(0, int(n * frac)) for n in dims)] = True
    return np.where(m, x, np.float32(1.0)).astype(np.float32)


# profiling-driven sampling (profiling = 1: blocks whose subsampled range is
# within the bound are left out, profiling_coeff scales the alpha/beta
# CompressTests) and a B-M sample of its own when the rates differ
PROF_CASES = [
    ((96, 128, 160), 1e-3, dict(autoTuningRate=0.01, predictorTuningRate=0.01, profiling=1,
                                levelwisePredictionSelection=4, maxStep=32, sampleBlockSize=32), 0.6),
    ((96, 128, 160), 1e-2, dict(autoTuningRate=0.005, predictorTuningRate=0.02, profiling=1, testLorenzo=1,
                                sampleBlockSize=16), 0.6),
    ((128, 128, 128), 1e-4, dict(autoTuningRate=0.01, predictorTuningRate=0.01, profiling=1, testLorenzo=1,
                                 levelwisePredictionSelection=4, maxStep=32, sampleBlockSize=32), 0.5),
    ((400, 500), 1e-3, dict(autoTuningRate=0.01, predictorTuningRate=0.01, profiling=1,
                            levelwisePredictionSelection=6, maxStep=64), 0.7),
    ((96, 128, 160), 5e-3, dict(autoTuningRate=0.02, predictorTuningRate=0.005, levelwisePredictionSelection=4,
                                maxStep=32, sampleBlockSize=16), 1.0),
]


@pytest.mark.parametrize("dims,rel,settings,frac", PROF_CASES)
def test_gpu_profiling_and_rates_match_oracle(dims, rel, settings, frac):
    conf = F.Config(*dims)
    conf.errorBoundMode = F.EB_REL
    conf.relErrorBound = rel
    for k, v in settings.items():
        setattr(conf, k, v)
    x = _flat_outside(dims, frac, sum(dims))
    stream = F.SZ_compress(conf, x)
    ref, ref_payload = O.compress(conf, x)
    _, p = O.read_stream(stream)
    assert parse_interp_header(p, len(dims)) == parse_interp_header(ref_payload, len(dims))
    assert p == ref_payload
    assert mask_first_size(stream) == mask_first_size(ref)


VARFIRST_CASES = [
    ((96, 128, 160), 1e-3, dict(autoTuningRate=0.01, predictorTuningRate=0.01, var_first=1,
                                levelwisePredictionSelection=4, maxStep=32, sampleBlockSize=32), 1.0),
    ((96, 128, 160), 1e-3, dict(autoTuningRate=0.01, predictorTuningRate=0.01, var_first=1, profiling=1,
                                levelwisePredictionSelection=4, maxStep=32, sampleBlockSize=16), 0.6),
    ((400, 500), 1e-3, dict(autoTuningRate=0.01, predictorTuningRate=0.01, var_first=1, profiling=1,
                            levelwisePredictionSelection=6, maxStep=64), 0.7),
]


@pytest.mark.parametrize("dims,rel,settings,frac", VARFIRST_CASES)
def test_gpu_var_first_sampling_matches_oracle(dims, rel, settings, frac):
    conf = F.Config(*dims)
    conf.errorBoundMode = F.EB_REL
    conf.relErrorBound = rel
    for k, v in settings.items():
        setattr(conf, k, v)
    x = _flat_outside(dims, frac, sum(dims) + 1) if frac < 1 else spectral_field(dims, slope=-2.5, noise=0.05,
                                                                                seed=sum(dims))
    stream = F.SZ_compress(conf, x)
    ref, ref_payload = O.compress(conf, x)
    _, p = O.read_stream(stream)
    assert p == ref_payload
    assert mask_first_size(stream) == mask_first_size(ref)


@pytest.mark.parametrize("dims,rel,kind", [((64, 80, 96), 1e-3, "spectral"), ((300, 420), 1e-3, "spectral"),
                                           ((64, 72, 80), 1e-3, "planes")])
def test_gpu_cr_target_matches_oracle(dims, rel, kind):
    """TUNING_TARGET_CR: the alpha/beta lists with -1 and bit rates compared alone."""
    conf = F.Config(*dims)
    conf.errorBoundMode = F.EB_REL
    conf.relErrorBound = rel
    conf.tuningTarget = 1
    conf.autoTuningRate = conf.predictorTuningRate = 0.01
    conf.testLorenzo = 1
    conf.sampleBlockSize = 16
    x = _sum_of_planes(dims, 1e-4, 7, np.float32) if kind == "planes" else \
        spectral_field(dims, slope=-2.5, noise=0.02, seed=sum(dims))
    stream = F.SZ_compress(conf, x)
    ref, ref_payload = O.compress(conf, x)
    c1, p = O.read_stream(stream)
    c2, _ = O.read_stream(ref)
    assert (c1.cmprAlgo, c1.alpha, c1.beta) == (c2.cmprAlgo, c2.alpha, c2.beta)
    if c1.cmprAlgo == 0 and len(dims) == 3:
        assert mask_fast_frontend_padding(p, x.itemsize) == mask_fast_frontend_padding(ref_payload, x.itemsize)
    else:
        assert p == ref_payload


# (dims, bound, target, field): every case but the planes one decides
# differently from the PSNR target on the oracle (alpha, beta or Lorenzo)
SSIM_AC_CASES = [
    ((64, 80, 96), 1e-4, 2, (-2.25, 0.0, 6)), ((300, 420), 1e-4, 2, (-2.25, 0.03, 1)),
    ((72, 64, 80), 1e-4, 2, (-2.25, 0.03, 1)),
    ((64, 80, 96), 1e-3, 3, (-3.5, 0.03, 179)), ((300, 420), 5e-3, 3, (-3.5, 0.03, 723)),
    ((64, 72, 80), 1e-3, 3, "planes"), ((48, 50, 52), 1e-5, 3, "f64"),
]


@pytest.mark.parametrize("dims,rel,target,kind", SSIM_AC_CASES)
def test_gpu_ssim_and_ac_targets_match_oracle(dims, rel, target, kind):
    """TUNING_TARGET_SSIM / TUNING_TARGET_AC: the alpha/beta search scores
    each CompressTest by the reconstructions' SSIM or 1 - autocorrelation
    (computed from the GPU's reconstructions); decisions and streams equal
    the oracle's.  The planes case also runs the Lorenzo candidate."""
    conf = F.Config(*dims)
    conf.errorBoundMode = F.EB_REL
    conf.relErrorBound = rel
    conf.tuningTarget = target
    conf.autoTuningRate = conf.predictorTuningRate = 0.01
    conf.testLorenzo = 1
    conf.sampleBlockSize = 16
    if kind == "planes":
        x = _sum_of_planes(dims, 1e-4, 9, np.float32)
    elif kind == "f64":
        x = spectral_field(dims, slope=-3.0, noise=0.02, seed=5, dtype=np.float64)
    else:
        x = spectral_field(dims, slope=kind[0], noise=kind[1], seed=kind[2])
    stream = F.SZ_compress(conf, x)
    ref, ref_payload = O.compress(conf, x)
    c1, p = O.read_stream(stream)
    c2, _ = O.read_stream(ref)
    assert (c1.cmprAlgo, c1.alpha, c1.beta) == (c2.cmprAlgo, c2.alpha, c2.beta)
    if c1.cmprAlgo == 0 and len(dims) == 3:
        assert mask_fast_frontend_padding(p, x.itemsize) == mask_fast_frontend_padding(ref_payload, x.itemsize)
    else:
        assert p == ref_payload


@pytest.mark.parametrize("ab", [1, 2])
def test_gpu_ablist_matches_oracle(ab):
    """abList 1 / 2: the alpha list runs to 2.5 / 3."""
    dims = (80, 96, 112)
    conf = F.Config(*dims)
    conf.errorBoundMode = F.EB_REL
    conf.relErrorBound = 1e-2
    conf.autoTuningRate = conf.predictorTuningRate = 0.01
    conf.abList = ab
    conf.sampleBlockSize = 16
    x = spectral_field(dims, slope=-3.5, noise=0.005, seed=ab)
    stream = F.SZ_compress(conf, x)
    ref, ref_payload = O.compress(conf, x)
    assert O.read_stream(stream)[1] == ref_payload
