"""GPU path of the default configuration (ALGO_INTERP_LORENZO: the SZ3 tuner)
and of the 3-D Lorenzo fast frontend, against the oracle and the reference's
golden streams.

Lorenzo payloads hold struct padding that the reference writes from
uninitialised memory, so they are compared with those bytes masked; the
tuner's decisions and every other byte must match.
"""
import hashlib

import numpy as np
import pytest

import faz_gb300 as F
from faz_gb300.fields import spectral_field
from conftest import (cli_config, golden_case, golden_dec_sha, golden_input, golden_manifest, golden_stream,
                      mask_fast_frontend_padding, mask_first_size)

import oracle.oracle as O

pytestmark = pytest.mark.gpu

ALGO_LORENZO_REG, ALGO_INTERP = 0, 2
DECISIONS = ("cmprAlgo", "interpAlgo", "interpDirection", "quantbinCnt", "blockSize", "pred_dim", "lorenzo",
             "lorenzo2", "regression")


def _rc(name):
    return O.read_stream(golden_stream(golden_case(name)))[0]


# default configuration, no QoZ tuning (1-D to 3-D fields)
SZ3_CASES = [c["name"] for c in golden_manifest()
             if c["ini"] is None and "-q" not in c["flags"] and len(c["dims"]) <= 3]
# Lorenzo / regression streams
LOR_DEC_CASES = [c["name"] for c in golden_manifest() if _rc(c["name"]).cmprAlgo == ALGO_LORENZO_REG]
# explicit ALGO_LORENZO_REG runs of the reference (INI), compressed on the GPU
LOR_INI_CASES = [c["name"] for c in golden_manifest()
                 if c["ini"] is not None and _rc(c["name"]).cmprAlgo == ALGO_LORENZO_REG]


@pytest.fixture(scope="module", autouse=True)
def system_zstd():
    O.set_zstd(None)  # the oracle uses the same host zstd as the library
    yield


def _same(stream, ref, itemsize):
    c1, p1 = O.read_stream(stream)
    c2, p2 = O.read_stream(ref)
    for f in DECISIONS:
        assert getattr(c1, f) == getattr(c2, f), f
    if c1.cmprAlgo == ALGO_LORENZO_REG and c1.N == 3:
        assert mask_fast_frontend_padding(p1, itemsize) == mask_fast_frontend_padding(p2, itemsize)
    elif c1.cmprAlgo == ALGO_LORENZO_REG:
        assert p1 == p2  # the general frontend's payload has no padding
    else:
        assert p1 == p2
        assert mask_first_size(stream) == mask_first_size(ref)


@pytest.mark.parametrize("name", SZ3_CASES)
def test_gpu_default_config_matches_oracle_and_reference(name):
    case = golden_case(name)
    x = golden_input(case)
    stream = F.SZ_compress(cli_config(case), x)
    ref, _ = O.compress(cli_config(case), x)
    _same(stream, ref, x.itemsize)
    # the reference's own decisions (its zstd may differ from the host's, but
    # not by enough to flip these cases)
    gc = _rc(name)
    c1, _ = O.read_stream(stream)
    for f in DECISIONS:
        assert getattr(c1, f) == getattr(gc, f), f
    dec, c2 = F.SZ_decompress(None, stream, dtype=x.dtype)
    ref_dec, _ = O.decompress(ref, dtype=x.dtype)
    assert np.array_equal(dec.view(np.uint8), ref_dec.view(np.uint8))
    assert np.abs(dec.astype(np.float64) - x.astype(np.float64)).max() <= c2.absErrorBound


@pytest.mark.parametrize("name", LOR_DEC_CASES)
def test_gpu_decodes_reference_lorenzo_streams(name):
    case = golden_case(name)
    dec, _ = F.SZ_decompress(None, golden_stream(case), dtype=np.dtype(case["dtype"]))
    assert hashlib.sha256(dec.tobytes()).hexdigest() == golden_dec_sha(case)


@pytest.mark.parametrize("name", LOR_INI_CASES)
def test_gpu_lorenzo_regression_matches_reference(name):
    case = golden_case(name)
    x = golden_input(case)
    stream = F.SZ_compress(cli_config(case), x)
    _, p1 = O.read_stream(stream)
    _, p2 = O.read_stream(golden_stream(case))
    if x.ndim == 3:
        assert mask_fast_frontend_padding(p1, x.itemsize) == mask_fast_frontend_padding(p2, x.itemsize)
    else:
        assert p1 == p2


def _lor_conf(dims, rel=None, abs_=None, bs=6, lo2=0, pd=None, qbins=65536, reg=0, lo=1):
    c = F.Config(*dims)
    c.cmprAlgo = F.ALGO_LORENZO_REG
    c.lorenzo, c.lorenzo2, c.regression, c.regression2 = lo, lo2, reg, 0
    c.blockSize = bs
    if pd is not None:
        c.pred_dim = pd
    c.quantbinCnt = qbins
    if rel is not None:
        c.errorBoundMode, c.relErrorBound = F.EB_REL, rel
    else:
        c.errorBoundMode, c.absErrorBound = F.EB_ABS, abs_
    return c


LOR_CASES = [
    ((37, 41, 29), dict(rel=1e-3), np.float32),
    ((64, 72, 80), dict(rel=1e-4, lo2=1), np.float32),
    ((30, 33, 35), dict(rel=1e-4, lo2=1, bs=5), np.float64),
    ((50, 40, 33), dict(rel=1e-2, lo2=1, pd=2), np.float32),
    ((17, 70, 9), dict(rel=1e-3, lo2=1, pd=1, bs=8), np.float32),
    ((1, 50, 60), dict(rel=1e-3, lo2=1, bs=4), np.float32),
    ((5, 6, 7), dict(abs_=0.5, bs=6, qbins=1024), np.float32),
    ((96, 64, 48), dict(rel=1e-5, lo2=1, qbins=4096), np.float32),
    # with linear regression blocks
    ((40, 44, 52), dict(rel=1e-3, reg=1), np.float32),
    ((37, 41, 29), dict(rel=1e-3, reg=1, lo2=1, bs=4), np.float32),
    ((30, 33, 35), dict(rel=1e-5, reg=1), np.float64),
    ((21, 22, 23), dict(rel=1e-2, reg=1, lo=0), np.float32),
    ((64, 64, 64), dict(rel=1e-4, reg=1, lo2=1, pd=2), np.float32),
    # more than 65536 quantisation bins: 32-bit codes
    ((40, 44, 52), dict(rel=1e-7, qbins=131072), np.float32),
    ((30, 33, 35), dict(rel=1e-7, qbins=131072, lo2=1, reg=1), np.float64),
]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_gpu_default_config_with_131072_bins(dtype):
    """A rough field at relative bound 1e-6: the default configuration's tuner
    chooses Lorenzo and its interval estimate asks for 131072 bins (the
    reference tool aborts on the float32 field; the oracle is the check)."""
    dims = (56, 60, 64)
    x = spectral_field(dims, slope=-1.5, noise=0.0, seed=56, dtype=dtype)
    conf = F.Config(*dims)
    conf.errorBoundMode, conf.relErrorBound = F.EB_REL, 1e-6
    stream = F.SZ_compress(conf, x)
    assert O.read_stream(stream)[0].quantbinCnt == 131072
    ref, _ = O.compress(conf, x)
    _same(stream, ref, np.dtype(dtype).itemsize)
    dec, c2 = F.SZ_decompress(None, stream, dtype=dtype)
    ref_dec, _ = O.decompress(ref, dtype=dtype)
    assert np.array_equal(dec.view(np.uint8), ref_dec.view(np.uint8))
    assert np.abs(dec.astype(np.float64) - x.astype(np.float64)).max() <= c2.absErrorBound


@pytest.mark.parametrize("dims,kw,dtype", LOR_CASES)
def test_gpu_lorenzo_matches_oracle(dims, kw, dtype):
    conf = _lor_conf(dims, **kw)
    x = spectral_field(dims, slope=-2.5, noise=0.02, seed=sum(dims), dtype=dtype)
    stream = F.SZ_compress(conf, x)
    ref, _ = O.compress(conf, x)
    _same(stream, ref, np.dtype(dtype).itemsize)
    dec, c2 = F.SZ_decompress(None, stream, dtype=dtype)
    ref_dec, _ = O.decompress(ref, dtype=dtype)
    assert np.array_equal(dec.view(np.uint8), ref_dec.view(np.uint8))
    assert np.abs(dec.astype(np.float64) - x.astype(np.float64)).max() <= c2.absErrorBound


def test_gpu_lorenzo_fast_path_agrees_with_double_path(monkeypatch):
    monkeypatch.setenv("FAZ_VERIFY_FASTPATH", "1")
    dims = (48, 56, 64)
    rng = np.random.default_rng(3)
    x = np.round(spectral_field(dims, slope=-2.0, seed=9).astype(np.float64) / 2 ** -7) * 2 ** -7
    x[rng.random(dims) < 0.01] = 0
    x = x.astype(np.float32)
    conf = _lor_conf(dims, abs_=2.0 ** -6, lo2=1)
    stream = F.SZ_compress(conf, x)  # raises on any disagreement
    dec, _ = F.SZ_decompress(None, stream, dtype=np.float32)
    ref, _ = O.compress(conf, x)
    _same(stream, ref, 4)


def test_gpu_lorenzo_rejects_what_it_does_not_implement():
    dims = (20, 20, 20)
    x = spectral_field(dims, slope=-3.0, seed=1)
    conf = _lor_conf(dims, rel=1e-3, bs=9)
    with pytest.raises(F.FazError):
        F.SZ_compress(conf, x)


GEN_CASES = [
    ((97, 131), dict(rel=1e-3, lo2=1, bs=16), np.float32),
    ((300, 257), dict(rel=1e-4, lo2=1, bs=5), np.float32),
    ((64, 80), dict(rel=1e-3, lo2=0, bs=16), np.float64),
    ((70, 45), dict(abs_=0.02, lo=0, lo2=1, bs=8), np.float32),
    ((33, 2), dict(rel=1e-2, lo2=1, bs=16), np.float32),
    ((1, 500), dict(rel=1e-3, lo2=1, bs=16), np.float32),
    ((129, 200), dict(rel=1e-5, lo2=1, bs=64, qbins=4096), np.float32),
    ((5000,), dict(rel=1e-3, lo2=1, bs=128), np.float32),
    ((3001,), dict(rel=1e-4, lo2=0, bs=2), np.float64),
    ((777,), dict(rel=1e-3, lo=0, lo2=1, bs=7), np.float32),
]


@pytest.mark.parametrize("dims,kw,dtype", GEN_CASES)
def test_gpu_general_frontend_matches_oracle(dims, kw, dtype):
    """1-D / 2-D ALGO_LORENZO_REG (general frontend, Lorenzo predictors)."""
    conf = _lor_conf(dims, reg=0, **kw)
    x = spectral_field(dims, slope=-2.5, noise=0.01, seed=sum(dims), dtype=dtype)
    stream = F.SZ_compress(conf, x)
    ref, _ = O.compress(conf, x)
    _same(stream, ref, np.dtype(dtype).itemsize)
    assert stream == ref
    dec, c2 = F.SZ_decompress(None, stream, dtype=dtype)
    ref_dec, _ = O.decompress(ref, dtype=dtype)
    assert np.array_equal(dec.view(np.uint8), ref_dec.view(np.uint8))
    assert np.abs(dec.astype(np.float64) - x.astype(np.float64)).max() <= c2.absErrorBound


# (dims, settings, dtype, noise): regression in the list (noisier fields make
# the regression predictor win more blocks)
GEN_REG_CASES = [
    ((97, 131), dict(rel=1e-3, bs=16), np.float32, 0.1),  # the default Config: Lorenzo + regression
    ((70, 45), dict(abs_=0.02, lo2=1, bs=8), np.float32, 0.05),  # Lorenzo + 2-layer Lorenzo + regression
    ((60, 77), dict(rel=1e-2, lo=0, lo2=1, bs=16), np.float32, 0.03),  # 2-layer Lorenzo + regression
    ((49, 65), dict(rel=1e-4, lo=0, bs=16), np.float64, 0.0),  # regression alone; one-row / -column edge blocks
    ((81, 66), dict(rel=1e-7, bs=16), np.float64, 0.3),  # unpredictable coefficients
    ((129, 200), dict(rel=1e-5, lo2=1, bs=64, qbins=4096), np.float32, 0.3),  # unpredictable points, blocks of 64
    ((300, 257), dict(rel=1e-3, bs=5), np.float32, 0.2),
    ((33, 2), dict(rel=1e-2, bs=16), np.float32, 0.1),
    ((1, 500), dict(rel=1e-3, bs=16), np.float32, 0.1),
    ((2, 2), dict(rel=1e-3, bs=16), np.float64, 0.0),
    ((20000,), dict(rel=1e-3, bs=128), np.float32, 0.0),
    ((3841,), dict(rel=1e-4, bs=128), np.float32, 0.0),  # one-point final block
    ((4033,), dict(rel=1e-5, lo=0, bs=64), np.float64, 0.0),  # regression alone, one-point final block
    ((777,), dict(rel=1e-3, lo=0, lo2=1, bs=7), np.float32, 0.05),
    ((5000,), dict(abs_=0.05, lo2=1, bs=16, qbins=256), np.float32, 0.1),
]


@pytest.mark.parametrize("dims,kw,dtype,noise", GEN_REG_CASES)
def test_gpu_general_frontend_regression_matches_oracle(dims, kw, dtype, noise):
    """1-D / 2-D ALGO_LORENZO_REG with the linear-regression predictor
    (RegressionPredictor.hpp, ComposedPredictor.hpp): stream and decoded array
    equal the oracle's bit for bit, the bound holds."""
    conf = _lor_conf(dims, reg=1, **kw)
    x = spectral_field(dims, slope=-3.5, noise=noise, seed=7 * sum(dims), dtype=dtype)
    stream = F.SZ_compress(conf, x)
    ref, _ = O.compress(conf, x)
    _same(stream, ref, np.dtype(dtype).itemsize)
    assert stream == ref
    dec, c2 = F.SZ_decompress(None, stream, dtype=dtype)
    ref_dec, _ = O.decompress(ref, dtype=dtype)
    assert np.array_equal(dec.view(np.uint8), ref_dec.view(np.uint8))
    assert np.abs(dec.astype(np.float64) - x.astype(np.float64)).max() <= c2.absErrorBound


def test_gpu_general_frontend_regression_on_a_batch_shape():
    """The default ALGO_LORENZO_REG Config on a 1800x3600 float32 field
    (one of the batch workload's 2-D shapes), against the oracle."""
    dims = (1800, 3600)
    conf = _lor_conf(dims, rel=1e-3, bs=16, reg=1)
    x = spectral_field(dims, slope=-3.0, noise=0.02, seed=1234)
    stream = F.SZ_compress(conf, x)
    ref, _ = O.compress(conf, x)
    assert stream == ref
    dec, c2 = F.SZ_decompress(None, stream, dtype=np.float32)
    ref_dec, _ = O.decompress(ref, dtype=np.float32)
    assert np.array_equal(dec.view(np.uint8), ref_dec.view(np.uint8))


def test_gpu_general_frontend_rejects_regression2():
    dims = (40, 50)
    conf = _lor_conf(dims, rel=1e-3, reg=1)
    conf.regression2 = 1
    with pytest.raises(F.FazError):
        F.SZ_compress(conf, spectral_field(dims, slope=-3.0, seed=2))


@pytest.mark.parametrize("dims,rel,dtype", [((400, 520), 1e-3, np.float32), ((700, 300), 1e-4, np.float64),
                                            ((60000,), 1e-3, np.float32)])
def test_gpu_default_config_on_sampled_1d_2d_fields(dims, rel, dtype):
    """The SZ3 tuner on sampled 1-D / 2-D fields (its Lorenzo trial runs the
    general frontend), Lorenzo-friendly fields so both branches are met."""
    rng = np.random.default_rng(sum(dims))
    if len(dims) == 2:
        x = (np.cumsum(rng.standard_normal((dims[0], 1)), 0) + np.cumsum(rng.standard_normal((1, dims[1])), 1))
        x = (x + 0.001 * rng.standard_normal(dims) * np.ptp(x)).astype(dtype)
    else:
        x = np.cumsum(rng.standard_normal(dims)).astype(dtype)
    for arr in (x, spectral_field(dims, slope=-4.0, seed=3, dtype=dtype)):
        conf = F.Config(*dims)
        conf.errorBoundMode, conf.relErrorBound = F.EB_REL, rel
        stream = F.SZ_compress(conf, arr)
        ref, _ = O.compress(conf, arr)
        _same(stream, ref, np.dtype(dtype).itemsize)
        dec, c2 = F.SZ_decompress(None, stream, dtype=dtype)
        assert np.abs(dec.astype(np.float64) - arr.astype(np.float64)).max() <= c2.absErrorBound
