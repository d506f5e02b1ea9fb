"""4-D interpolation (interp4.cu) against the oracle.

block_interpolation for N = 4 (SZInterpolationCompressor.hpp:3363-3442):
four sweeps per block, 24 directions.  Streams are compared with the
oracle's byte for byte and decompressed arrays bit for bit; the reference's
own 4-D stream (fixture c4d_cubic) is covered by the golden parity tests.
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


LIN, CUB = F.INTERP_ALGO_LINEAR, F.INTERP_ALGO_CUBIC
CASES = [
    ((10, 33, 40, 20), CUB, 0, dict(rel=1e-3), np.float32),
    ((17, 9, 65, 12), LIN, 7, dict(rel=1e-2), np.float32),
    ((5, 6, 7, 70), CUB, 23, dict(rel=1e-4), np.float32),
    ((12, 20, 18, 16), CUB, 13, dict(rel=1e-3, interpBlockSize=8), np.float32),
    ((9, 40, 11, 21), LIN, 18, dict(rel=1e-5), np.float64),
    ((8, 16, 16, 16), CUB, 5, dict(rel=1e-3, interpAlgo_list=[1, 0, 1, 0, 1], interpDirection_list=[0, 23, 5, 12, 1]),
     np.float32),
    ((33, 3, 2, 35), CUB, 3, dict(rel=1e-3), np.float32),
]


@pytest.mark.parametrize("dims,interp,direction,kw,dtype", CASES)
def test_4d_matches_oracle(dims, interp, direction, kw, dtype):
    kw = dict(kw)
    lists = {k: kw.pop(k) for k in ("interpAlgo_list", "interpDirection_list") if k in kw}
    c = F.Config(*dims)
    c.cmprAlgo = F.ALGO_INTERP
    c.interpAlgo = interp
    c.interpDirection = direction
    c.errorBoundMode, c.relErrorBound = F.EB_REL, kw.pop("rel")
    for k, v in list(kw.items()) + list(lists.items()):
        setattr(c, k, v)
    x = spectral_field(dims, slope=-3.0, noise=0.02, seed=sum(dims) + direction, dtype=dtype)
    stream = F.SZ_compress(c, x)
    ref, _ = O.compress(c, x)
    assert mask_first_size(stream) == mask_first_size(ref)
    dec, c2 = F.SZ_decompress(None, stream, dtype=dtype)
    ref_dec, _ = O.decompress(ref, dtype=dtype)
    assert np.array_equal(dec.view(np.uint8), ref_dec.view(np.uint8))
    assert np.abs(dec.astype(np.float64) - x.astype(np.float64)).max() <= c2.absErrorBound


def test_4d_default_tuner_is_refused():
    dims = (8, 9, 10, 11)
    c = F.Config(*dims)
    c.errorBoundMode, c.relErrorBound = F.EB_REL, 1e-3
    x = spectral_field(dims, slope=-3.0, seed=2)
    with pytest.raises(F.FazError):
        F.SZ_compress(c, x)
