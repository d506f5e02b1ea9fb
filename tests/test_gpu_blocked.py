"""ALGO_INTERP_BLOCKED on the GPU (SZ_compress_Interp_blocked,
include/QoZ/api/impl/SZInterp.hpp:3021-3500; compress_block / decompress_block,
include/QoZ/compressor/SZInterpolationCompressor.hpp:533-781, 201-323): the
stream, with its per-block interpolator and direction choices, and the
decoded array against the oracle bit for bit.  The reference tool's own
streams (blk_* in tests/golden) are covered by tests/test_gpu_parity.py.
"""
import numpy as np
import pytest

import faz_gb300 as F
from faz_gb300.fields import spectral_field
from conftest import mask_first_size

import oracle.oracle as O

pytestmark = pytest.mark.gpu

ALGO_INTERP_BLOCKED = 3


@pytest.fixture(scope="module", autouse=True)
def system_zstd():
    O.set_zstd(None)  # the oracle uses the same host zstd as the library
    yield


def _conf(dims, rel=None, abs_=None, **kw):
    c = F.Config(*dims)
    c.cmprAlgo = ALGO_INTERP_BLOCKED
    if rel is not None:
        c.errorBoundMode, c.relErrorBound = F.EB_REL, rel
    else:
        c.errorBoundMode, c.absErrorBound = F.EB_ABS, abs_
    for k, v in kw.items():
        setattr(c, k, v)
    return c


# (dims, settings, dtype, field slope, noise)
CASES = [
    ((40, 56, 72), dict(rel=1e-3), np.float32, -3.0, 0.0),
    ((33, 47, 65), dict(rel=1e-5, interpBlockSize=16), np.float64, -3.5, 0.0),
    ((48, 48, 48), dict(abs_=0.05, blockwiseSampleBlockSize=8), np.float32, -2.5, 0.02),
    ((64, 40, 50), dict(rel=1e-4, maxStep=16, alpha=1.5, beta=3.0), np.float32, -3.0, 0.0),
    ((17, 23, 130), dict(rel=1e-3, interpBlockSize=8, trimToZero=1), np.float32, -3.0, 0.0),
    ((65, 33, 97), dict(rel=1e-3, interpBlockSize=64), np.float32, -3.0, 0.01),
    ((1, 70, 90), dict(rel=1e-3), np.float32, -3.0, 0.0),
    ((2, 3, 200), dict(rel=1e-2, interpBlockSize=4), np.float32, -2.0, 0.0),
    ((31, 31, 31), dict(rel=1e-3, interpBlockSize=2, blockwiseSampleBlockSize=2), np.float32, -3.0, 0.0),
    ((50, 51, 52), dict(rel=1e-6, quantbinCnt=1024), np.float64, -2.0, 0.05),
    ((36, 60, 44), dict(rel=1e-2, alpha=0.5, beta=0.25, trimToZero=2), np.float32, -3.0, 0.0),
]


@pytest.mark.parametrize("dims,kw,dtype,slope,noise", CASES)
def test_gpu_blocked_matches_oracle(dims, kw, dtype, slope, noise):
    conf = _conf(dims, **kw)
    x = spectral_field(dims, slope=slope, noise=noise, seed=3 * sum(dims), dtype=dtype)
    if kw.get("trimToZero"):
        x = (x / np.abs(x).max()).astype(dtype)
    stream = F.SZ_compress(conf, x)
    ref, _ = O.compress(conf, x)
    c1, p1 = O.read_stream(stream)
    c2, p2 = O.read_stream(ref)
    assert c1.cmprAlgo == F.ALGO_INTERP and c1.blockwiseTuning == 1
    assert p1 == p2
    assert mask_first_size(stream) == mask_first_size(ref)
    dec, c3 = F.SZ_decompress(None, stream, dtype=dtype)
    ref_dec, _ = O.decompress(ref, dtype=dtype)
    assert np.array_equal(dec.view(np.uint8), ref_dec.view(np.uint8))
    assert np.abs(dec.astype(np.float64) - x.astype(np.float64)).max() <= c3.absErrorBound


def test_gpu_blocked_on_a_larger_field():
    """256x256x256 float32, default block-wise settings, against the oracle."""
    dims = (256, 256, 256)
    conf = _conf(dims, rel=1e-3)
    x = spectral_field(dims, slope=-3.0, noise=0.01, seed=2024)
    stream = F.SZ_compress(conf, x)
    ref, _ = O.compress(conf, x)
    assert O.read_stream(stream)[1] == O.read_stream(ref)[1]
    dec, _ = F.SZ_decompress(None, stream, dtype=np.float32)
    ref_dec, _ = O.decompress(ref, dtype=np.float32)
    assert np.array_equal(dec.view(np.uint8), ref_dec.view(np.uint8))


# ALGO_INTERP with a fixBlockSize that is not a multiple of 2^levels: the
# same block loop with the level's interpolator and direction everywhere
FIX_CASES = [
    ((30, 30, 30), dict(rel=1e-3, fixBlockSize=8), np.float32),
    ((70, 45), dict(rel=1e-3, fixBlockSize=16, interpDirection=1), np.float32),
    ((3000,), dict(rel=1e-3, fixBlockSize=32), np.float32),
    ((40, 50, 60), dict(rel=1e-4, fixBlockSize=4, interpAlgo=0, interpDirection=3), np.float64),
    ((33, 65, 17), dict(rel=1e-3, fixBlockSize=16, interpAlgo_list=[1, 0, 1], interpDirection_list=[0, 5, 2],
                        alpha=1.25, beta=2.0), np.float32),
    ((100, 120), dict(abs_=0.01, fixBlockSize=2, trimToZero=1), np.float32),
    ((64, 200), dict(rel=1e-3, fixBlockSize=8, interpAlgo=0), np.float32),
]


@pytest.mark.parametrize("dims,kw,dtype", FIX_CASES)
def test_gpu_unaligned_fix_block_size_matches_oracle(dims, kw, dtype):
    conf = _conf(dims, **kw)
    conf.cmprAlgo = F.ALGO_INTERP
    x = spectral_field(dims, slope=-3.0, seed=5 * sum(dims), dtype=dtype)
    if kw.get("trimToZero"):
        x = (x / np.abs(x).max()).astype(dtype)
    stream = F.SZ_compress(conf, x)
    ref, _ = O.compress(conf, x)
    assert O.read_stream(stream)[1] == O.read_stream(ref)[1]
    assert mask_first_size(stream) == mask_first_size(ref)
    dec, c3 = F.SZ_decompress(None, stream, dtype=dtype)
    ref_dec, _ = O.decompress(ref, dtype=dtype)
    assert np.array_equal(dec.view(np.uint8), ref_dec.view(np.uint8))
    # one of them through the batched entry point
    if dims == (30, 30, 30):
        import torch
        assert F.compress_batch([conf], [torch.from_numpy(x).cuda()])[0] == stream


@pytest.mark.parametrize("dims,kw", [((40, 50), {}), ((30, 30, 30), dict(autoTuningRate=0.01)),
                                     ((30, 30, 30), dict(crossBlock=1)), ((30, 30, 30), dict(interpBlockSize=24)),
                                     ((64, 64, 64), dict(maxStep=32, interpBlockSize=8))])
def test_gpu_blocked_rejects_what_it_does_not_implement(dims, kw):
    """Not 3-D, the alpha/beta search, crossBlock, a block edge that is not a
    power of two, and blocks smaller than maxStep (the anchors are coded twice
    and the reference's decoder reads past its codes)."""
    conf = _conf(dims, rel=1e-3, **kw)
    with pytest.raises(F.FazError):
        F.SZ_compress(conf, spectral_field(dims, slope=-3.0, seed=5))


def test_gpu_fix_block_size_below_max_step_is_refused():
    """ALGO_INTERP with an anchor grid and fixBlockSize below maxStep: the
    reference codes the anchors twice and cannot decode its own stream."""
    dims = (64, 64)
    conf = _conf(dims, rel=1e-3, fixBlockSize=8, maxStep=32)
    conf.cmprAlgo = F.ALGO_INTERP
    with pytest.raises(F.FazError):
        F.SZ_compress(conf, spectral_field(dims, slope=-3.0, seed=6))
