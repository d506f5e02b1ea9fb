"""The finest interpolation level's plane kernel (finest.cu) against the
oracle and against the block kernel it replaces.

The plane kernel runs for 3-D float fields on the exact float quantiser path
whose sweep order ends on the contiguous axis (directions 0 and 2), block
edges up to 32 that are multiples of 4 and rows of a multiple of four values.
By default it compresses and the block kernel decompresses.  Every case runs
both directions with the plane kernel (FAZ_FINEST_PLANES=2) and with the
block kernel (FAZ_FINEST_PLANES=0): the streams are equal byte for byte and
equal the oracle's; both decompressions equal the oracle's array bit for bit.
"""
import numpy as np
import pytest

import faz_gb300 as F
from faz_gb300.fields import spectral_field
from conftest import mask_first_size

import oracle.oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def system_zstd():
    O.set_zstd(None)
    yield


def _conf(dims, interp, direction, rel=None, abs_=None, **kw):
    c = F.Config(*dims)
    c.cmprAlgo = F.ALGO_INTERP
    c.interpAlgo = interp
    c.interpDirection = direction
    if rel is not None:
        c.errorBoundMode, c.relErrorBound = F.EB_REL, rel
    else:
        c.errorBoundMode, c.absErrorBound = F.EB_ABS, abs_
    for k, v in kw.items():
        setattr(c, k, v)
    return c


LIN, CUB = F.INTERP_ALGO_LINEAR, F.INTERP_ALGO_CUBIC
CASES = [
    # full and clipped blocks; dim - 1 a multiple of 32 (blocks of one point)
    ((64, 64, 64), CUB, 0, dict(rel=1e-3)),
    ((65, 66, 68), LIN, 0, dict(rel=1e-3)),
    ((65, 66, 68), CUB, 2, dict(rel=1e-4)),
    ((33, 33, 36), CUB, 0, dict(rel=1e-2)),
    ((34, 35, 40), LIN, 2, dict(rel=1e-3)),
    ((97, 40, 100), CUB, 0, dict(rel=1e-5)),
    ((40, 97, 44), LIN, 2, dict(rel=1e-2)),
    # block size 16 and 8 (interpBlockSize), anchors with alpha / beta
    ((70, 60, 52), CUB, 0, dict(rel=1e-3, interpBlockSize=16)),
    ((50, 45, 48), LIN, 2, dict(rel=1e-3, interpBlockSize=8)),
    ((96, 64, 64), CUB, 0, dict(rel=1e-3, maxStep=16, alpha=1.5, beta=3.0)),
    # tiny bound: codes reach the radius, many unpredictable points
    ((48, 48, 48), CUB, 0, dict(rel=1e-6)),
    ((48, 48, 48), LIN, 2, dict(rel=1e-6, quantbinCnt=1024)),
]


def _run(conf, x, planes, monkeypatch):
    # 2: the plane kernel for compression and decompression; 0: neither
    monkeypatch.setenv("FAZ_FINEST_PLANES", "2" if planes else "0")
    s = F.SZ_compress(conf, x)
    d, c2 = F.SZ_decompress(None, s, dtype=x.dtype)
    return s, d, c2


@pytest.mark.parametrize("dims,interp,direction,kw", CASES)
def test_plane_kernel_matches_block_kernel_and_oracle(dims, interp, direction, kw, monkeypatch):
    x = spectral_field(dims, slope=-3.0, noise=0.02, seed=sum(dims) + direction)
    if kw.get("rel", 1) <= 1e-6:
        rng = np.random.default_rng(3)
        x[rng.random(dims) < 0.01] *= 40.0  # spikes: unpredictable points
    conf = _conf(dims, interp, direction, **kw)
    s_plane, d_plane, c2 = _run(conf, x, True, monkeypatch)
    s_block, d_block, _ = _run(conf, x, False, monkeypatch)
    assert s_plane == s_block
    ref, _ = O.compress(conf, x)
    assert mask_first_size(s_plane) == mask_first_size(ref)
    ref_dec, _ = O.decompress(ref)
    assert np.array_equal(d_plane.view(np.uint32), ref_dec.view(np.uint32))
    assert np.array_equal(d_block.view(np.uint32), ref_dec.view(np.uint32))
    assert np.abs(d_plane.astype(np.float64) - x.astype(np.float64)).max() <= c2.absErrorBound


def test_plane_kernel_exact_float_path(monkeypatch):
    """Grid-valued data puts differences on quantiser boundaries; with
    FAZ_VERIFY_FASTPATH every point also runs the double computation and
    the call fails on any difference."""
    dims = (64, 72, 80)
    step = 2.0 ** -7
    x = spectral_field(dims, slope=-3.0, seed=9).astype(np.float64)
    x = (np.round(x / step) * step).astype(np.float32)
    monkeypatch.setenv("FAZ_VERIFY_FASTPATH", "1")
    for interp, direction in ((CUB, 0), (LIN, 2)):
        conf = _conf(dims, interp, direction, abs_=2.0 ** -6)
        s, d, _ = _run(conf, x, True, monkeypatch)
        ref, _ = O.compress(conf, x)
        assert mask_first_size(s) == mask_first_size(ref)
        ref_dec, _ = O.decompress(ref)
        assert np.array_equal(d.view(np.uint32), ref_dec.view(np.uint32))
