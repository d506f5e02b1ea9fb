"""Batched compression (faz_compress_batch): every field's stream equals the
one the single-field device call writes, whatever the batch holds."""
import numpy as np
import pytest

import faz_gb300 as F
from faz_gb300.fields import spectral_field

import oracle.oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _conf(dims, rel=1e-3, **kw):
    c = F.Config(*dims)
    c.cmprAlgo = F.ALGO_INTERP
    c.errorBoundMode, c.relErrorBound = F.EB_REL, rel
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def _mixed():
    """(conf, cuda tensor) pairs: 1-D/2-D/3-D, anchors, level-wise lists,
    alpha/beta, ABS / REL / PSNR bounds, linear and cubic, odd extents."""
    out = []
    specs = [
        ((60, 70, 80), dict()),
        ((33, 17, 65), dict(interpAlgo=F.INTERP_ALGO_LINEAR, rel=1e-2)),
        ((300, 257), dict(interpDirection=1)),
        ((5000,), dict(rel=1e-4)),
        ((40, 40, 40), dict(maxStep=16, alpha=1.5, beta=2.0)),
        ((36, 28, 44), dict(alpha=0.5, beta=0.25)),
        ((2, 3, 4), dict()),
        ((128, 96, 64), dict(interpBlockSize=16, interpDirection=5)),
        ((90, 100), dict(errorBoundMode=F.EB_ABS, absErrorBound=0.05)),
        ((48, 56, 64), dict(errorBoundMode=F.EB_PSNR, psnrErrorBound=60.0)),
    ]
    for i, (dims, kw) in enumerate(specs):
        rel = kw.pop("rel", 1e-3)
        c = _conf(dims, rel=rel, **kw)
        x = spectral_field(dims, slope=-3.0, aniso=(1,) * len(dims), noise=0.01, seed=100 + i, device="cuda")
        out.append((c, x))
    lw = _conf((64, 64, 64))
    lw.interpAlgo_list = [0, 1, 1, 0]
    lw.interpDirection_list = [5, 0, 5, 0]
    lw.maxStep, lw.alpha, lw.beta = 32, 1.25, 1.5
    out.append((lw, spectral_field((64, 64, 64), slope=-3.5, seed=120, device="cuda")))
    return out


@pytest.mark.parametrize("threads", [0, 256, 128])
def test_gpu_batch_streams_equal_single_field_streams(threads):
    pairs = _mixed()
    streams = F.compress_batch([c for c, _ in pairs], [x for _, x in pairs], threads=threads)
    for (c, x), s in zip(pairs, streams):
        assert s == F.compress_device(c, x)
        out = torch.empty_like(x)
        c2 = F.decompress_device(s, out)
        assert (out.double() - x.double()).abs().max().item() <= c2.absErrorBound


def test_gpu_batch_with_tuned_and_lorenzo_fields():
    """Fields whose configuration runs a tuner or the Lorenzo frontend go
    through the single-field path inside the batch."""
    dims = (56, 60, 64)
    base = spectral_field(dims, slope=-3.0, seed=7, device="cuda")
    tuned = F.Config(*dims)
    tuned.errorBoundMode, tuned.relErrorBound = F.EB_REL, 1e-3
    lor = F.Config(*dims)
    lor.cmprAlgo, lor.errorBoundMode, lor.relErrorBound, lor.lorenzo2 = F.ALGO_LORENZO_REG, F.EB_REL, 1e-3, 1
    plain = _conf(dims)
    confs, xs = [tuned, lor, plain], [base, base * 0.5 + 1.0, base]
    streams = F.compress_batch(confs, xs)
    for c, x, s in zip(confs, xs, streams):
        assert s == F.compress_device(c, x)


def test_gpu_batch_many_small_fields_match_the_oracle():
    rng = np.random.default_rng(9)
    confs, xs, hs = [], [], []
    for i in range(40):
        nd = int(rng.integers(1, 4))
        dims = tuple(int(v) for v in rng.integers(3, 40, size=nd))
        a = spectral_field(dims, slope=float(rng.uniform(-4, -2)), noise=0.02, seed=200 + i)
        confs.append(_conf(dims, rel=float(10 ** rng.uniform(-4, -2)),
                           interpAlgo=int(rng.integers(0, 2))))
        xs.append(torch.as_tensor(a, device="cuda"))
        hs.append(a)
    O.set_zstd(None)
    streams = F.compress_batch(confs, xs)
    for c, a, s in zip(confs, hs, streams):
        ref, _ = O.compress(c, a)
        assert O.read_stream(s)[1] == O.read_stream(ref)[1]


def test_gpu_batch_rejects_mismatched_input():
    x = torch.zeros(10, device="cuda")
    with pytest.raises(ValueError):
        F.compress_batch([_conf((11,))], [x])


@pytest.mark.parametrize("multiframe", [False, True])
def test_gpu_batch_writes_the_same_zstd_frames(monkeypatch, multiframe):
    """With zstd's worker threads (one frame per stream; the batch's host
    threads compress with one worker each) and with independent frames, the
    batch writes the bytes a single-field call writes."""
    monkeypatch.setenv("FAZ_ZSTD_THREADS", "8")
    if multiframe:
        monkeypatch.setenv("FAZ_ZSTD_MULTIFRAME", "1")
    big = spectral_field((128, 256, 256), slope=-3.0, noise=0.01, seed=5, device="cuda")
    small = spectral_field((40, 50, 60), slope=-3.0, seed=6, device="cuda")
    confs = [_conf((128, 256, 256), rel=1e-4), _conf((40, 50, 60))]
    streams = F.compress_batch(confs, [big, small])
    assert streams[0] == F.compress_device(confs[0], big)
    assert streams[1] == F.compress_device(confs[1], small)
