"""Parity at the configured sizes.

* 512x512x512 float32 spectral field (k^-3.5, correlation lengths 1:2:4, 1 %
  noise, scaled to [-50, 80]) - the benchmark's own field, made by the same
  generator with the same seed - at relative bounds 1e-2, 1e-3, 1e-4 and
  1e-5, with the default configuration (the SZ3 sampled autotune of
  include/QoZ/api/impl/SZInterp.hpp:2115-2187, 2561-2880 choosing
  interpolation or Lorenzo) and with plain ALGO_INTERP cubic: the tuner's
  decision, the pre-zstd payload, the whole stream (firstSize masked) and the
  decompressed array equal the oracle's bit for bit, and the error bound holds
  in FP64.  tests/test_c2_reference.py pins the oracle to the reference tool on
  a field of the same distribution.
* One field of each batch shape (2-D 1800x3600, 2-D 721x1440, 3-D 100x500x500,
  3-D 26x1800x3600) at relative bound 1e-3 through the batched entry point.
* One float64 256x384x384 field (k^-3 plus a Gaussian-bump background) per
  bound (1e-4, 1e-6): the QoZ tuner's stream, and the learned tuner's
  configuration through the batched entry point, against the oracle.
"""
import numpy as np
import pytest

import faz_gb300 as F
from faz_gb300.fields import spectral_field
from conftest import mask_fast_frontend_padding, mask_first_size

import oracle.oracle as O

pytestmark = pytest.mark.gpu

C2_DIMS = (512, 512, 512)
C2_SEED = 1000  # bench.py's field (rank 0)
RELS = [1e-2, 1e-3, 1e-4, 1e-5]
ALGO_LORENZO_REG = 0


@pytest.fixture(scope="module", autouse=True)
def system_zstd():
    O.set_zstd(None)  # the oracle uses the same host zstd as the library
    yield


@pytest.fixture(scope="module")
def c2_field():
    import torch
    x = spectral_field(C2_DIMS, slope=-3.5, aniso=(1, 2, 4), noise=0.01, seed=C2_SEED)  # numpy, as bench.py
    return torch.from_numpy(x).cuda(), x


def _payload(stream, conf, itemsize):
    pl = O.read_stream(stream)[1]
    if conf.cmprAlgo == ALGO_LORENZO_REG and len(conf.dims) == 3:
        pl = mask_fast_frontend_padding(pl, itemsize)
    return pl


def _check_against_oracle(conf, t, x, stream):
    """Decision, payload, stream and decompressed array against the oracle."""
    import torch
    ref, _ = O.compress(conf, x)
    got_conf, ref_conf = O.read_stream(stream)[0], O.read_stream(ref)[0]
    for k in ("cmprAlgo", "interpAlgo", "interpDirection", "quantbinCnt", "pred_dim", "blockSize", "lorenzo",
              "lorenzo2", "regression"):
        assert getattr(got_conf, k) == getattr(ref_conf, k), k
    assert _payload(stream, got_conf, x.itemsize) == _payload(ref, ref_conf, x.itemsize)
    if got_conf.cmprAlgo != ALGO_LORENZO_REG:
        assert mask_first_size(stream) == mask_first_size(ref)
    out = torch.empty_like(t)
    c2 = F.decompress_device(stream, out)
    ref_dec, _ = O.decompress(ref, dtype=x.dtype)
    got = out.cpu().numpy()
    assert np.array_equal(got.reshape(-1).view(np.uint8), ref_dec.reshape(-1).view(np.uint8))
    err = (out.double() - t.double()).abs().max().item()
    assert err <= c2.absErrorBound
    return got_conf


@pytest.mark.parametrize("rel", RELS)
def test_c2_default_configuration_matches_oracle(c2_field, rel):
    t, x = c2_field
    conf = F.Config(*C2_DIMS)
    conf.errorBoundMode, conf.relErrorBound = F.EB_REL, rel
    stream = F.SZ_compress(conf, t)
    _check_against_oracle(conf, t, x, stream)


@pytest.mark.parametrize("rel", RELS)
def test_c2_interp_cubic_matches_oracle(c2_field, rel):
    t, x = c2_field
    conf = F.Config(*C2_DIMS)
    conf.cmprAlgo, conf.interpAlgo = F.ALGO_INTERP, F.INTERP_ALGO_CUBIC
    conf.errorBoundMode, conf.relErrorBound = F.EB_REL, rel
    stream = F.SZ_compress(conf, t)
    _check_against_oracle(conf, t, x, stream)


BATCH_SHAPES = [(1800, 3600), (721, 1440), (100, 500, 500), (26, 1800, 3600)]


def test_c3_shapes_batched_match_oracle():
    """One field of each batch shape (slopes in [-4, -2], the last with 5 %
    sparse spikes), relative bound 1e-3, cubic ALGO_INTERP, through one
    batched call: every stream against the oracle's."""
    rng = np.random.default_rng(7)
    confs, ts = [], []
    for i, dims in enumerate(BATCH_SHAPES):
        ts.append(spectral_field(dims, slope=float(rng.uniform(-4, -2)), noise=0.01, seed=int(rng.integers(1 << 30)),
                                 spikes=0.05 if i == 3 else 0.0, device="cuda"))
        c = F.Config(*dims)
        c.cmprAlgo, c.errorBoundMode, c.relErrorBound = F.ALGO_INTERP, F.EB_REL, 1e-3
        confs.append(c)
    streams = F.compress_batch(confs, ts)
    for c, t, s in zip(confs, ts, streams):
        _check_against_oracle(c, t, t.cpu().numpy(), s)


C5_DIMS = (256, 384, 384)


@pytest.mark.parametrize("rel", [1e-4, 1e-6])
def test_c5_f64_matches_oracle(rel):
    """float64 256x384x384 (k^-3 plus three Gaussian bumps): the QoZ tuner's
    stream (compress_device) and the learned tuner's configuration compressed
    through the batched entry point, each against the oracle."""
    import numpy as _np
    import faz_gb300.learned as L
    t = spectral_field(C5_DIMS, slope=-3.0, noise=0.0, bumps=3, seed=int(rel * 1e9) + 11, dtype=_np.float64,
                       device="cuda")
    x = t.cpu().numpy()
    qc = L.qoz_conf(C5_DIMS, rel)
    _check_against_oracle(qc, t, x, F.compress_device(qc, t))
    tuned, _ = L.learned_tune(L.qoz_conf(C5_DIMS, rel), t, min_confidence=0.5)
    stream = F.compress_batch([tuned], [t])[0]
    _check_against_oracle(tuned, t, x, stream)
