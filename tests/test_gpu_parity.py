"""GPU path vs oracle and vs the reference's golden streams.

Integer/byte work (codes, Huffman bits, stream bytes) and the decompressed
arrays are compared bit for bit.  Full streams are compared where oracle and
library use the same host zstd; the pre-zstd payloads always.
"""
import hashlib

import numpy as np
import pytest

import faz_gb300 as F
from faz_gb300.fields import spectral_field
from conftest import (cli_config, golden_case, golden_input, golden_manifest, golden_stream, mask_first_size,
                      tuned_config)

import oracle.oracle as O

pytestmark = pytest.mark.gpu

# cases outside the GPU path (none: 4-D fields run through interp4.cu)
GPU_UNSUPPORTED = set()
ALGO_INTERP = 2


def _trailer_algo(name):
    return O.read_stream(golden_stream(golden_case(name)))[0].cmprAlgo


# interpolation streams (ALGO_INTERP in the trailer)
_INTERP = {c["name"] for c in golden_manifest() if _trailer_algo(c["name"]) == ALGO_INTERP}
INI_CASES = [c["name"] for c in golden_manifest()
             if c["ini"] is not None and c["name"] not in GPU_UNSUPPORTED and c["name"] in _INTERP]
TUNED_CASES = [c["name"] for c in golden_manifest() if c["ini"] is None and c["name"] in _INTERP]
DEC_CASES = [c["name"] for c in golden_manifest() if c["name"] not in GPU_UNSUPPORTED and c["name"] in _INTERP]


@pytest.fixture(scope="module", autouse=True)
def system_zstd():
    O.set_zstd(None)  # the oracle uses the same host zstd as the library
    yield


def payload_of(stream):
    return O.read_stream(stream)[1]


@pytest.mark.parametrize("name", INI_CASES)
def test_gpu_stream_matches_reference_payload(name):
    case = golden_case(name)
    x = golden_input(case)
    conf = cli_config(case)
    stream = F.SZ_compress(conf, x)
    assert payload_of(stream) == payload_of(golden_stream(case))
    ref, _ = O.compress(conf, x)
    assert mask_first_size(stream) == mask_first_size(ref)


@pytest.mark.parametrize("name", TUNED_CASES)
def test_gpu_payload_matches_tuned_reference(name):
    case = golden_case(name)
    conf = tuned_config(case)
    stream = F.SZ_compress(conf, golden_input(case))
    assert payload_of(stream) == payload_of(golden_stream(case))


@pytest.mark.parametrize("name", DEC_CASES)
def test_gpu_decompress_matches_reference(name):
    case = golden_case(name)
    dec, conf = F.SZ_decompress(None, golden_stream(case), dtype=np.dtype(case["dtype"]))
    assert hashlib.sha256(dec.tobytes()).hexdigest() == case["dec_sha256"]


def _conf(dims, rel=None, abs_=None, interp=F.INTERP_ALGO_CUBIC, direction=0, **kw):
    c = F.Config(*dims)
    c.cmprAlgo = F.ALGO_INTERP
    c.interpAlgo = interp
    c.interpDirection = direction
    if rel is not None:
        c.errorBoundMode = F.EB_REL
        c.relErrorBound = rel
    else:
        c.errorBoundMode = F.EB_ABS
        c.absErrorBound = abs_
    for k, v in kw.items():
        setattr(c, k, v)
    return c


RANDOM_CASES = [
    ((97, 130, 161), dict(rel=1e-3), np.float32, -3.0),
    ((64, 96, 128), dict(rel=1e-4, direction=5), np.float32, -2.5),
    ((65, 66, 67), dict(rel=1e-2, interp=F.INTERP_ALGO_LINEAR, direction=2), np.float32, -3.5),
    ((33, 200, 70), dict(rel=1e-5), np.float32, -2.0),
    ((300, 400), dict(rel=1e-3, direction=1), np.float32, -3.0),
    ((100000,), dict(rel=1e-3), np.float32, -2.0),
    ((48, 50, 52), dict(rel=1e-6), np.float64, -3.0),
    ((64, 64, 64), dict(rel=1e-3, maxStep=32, alpha=1.25, beta=2.0), np.float32, -3.0),
    ((70, 80, 90), dict(rel=1e-3, interpAlgo_list=[1, 0, 1, 1], interpDirection_list=[0, 5, 3, 1],
                        alpha=1.0, beta=1.5), np.float32, -3.0),
    # blocks that begin on the last element of an axis (dim - 1 a multiple of
    # the block edge), extents 1 and 2, every direction
    ((33, 65, 17), dict(rel=1e-3, direction=4), np.float32, -3.0),
    ((1, 33, 65), dict(rel=1e-3, direction=3), np.float32, -3.0),
    ((2, 33, 3), dict(rel=1e-3), np.float32, -3.0),
    ((129, 2, 33), dict(rel=1e-3, direction=5), np.float32, -3.0),
    ((65, 65, 65), dict(rel=1e-3, interp=F.INTERP_ALGO_LINEAR, direction=1), np.float64, -3.0),
    ((33,), dict(rel=1e-3), np.float32, -3.0),
    ((65, 1), dict(rel=1e-3, direction=1), np.float32, -3.0),
]


@pytest.mark.parametrize("dims,kw,dtype,slope", RANDOM_CASES)
def test_gpu_matches_oracle_random_fields(dims, kw, dtype, slope):
    lists = {k: kw.pop(k) for k in ("interpAlgo_list", "interpDirection_list") if k in kw}
    conf = _conf(dims, **kw)
    for k, v in lists.items():
        setattr(conf, k, v)
    x = spectral_field(dims, slope=slope, noise=0.02, seed=sum(dims), dtype=dtype)
    stream = F.SZ_compress(conf, x)
    ref, ref_payload = O.compress(conf, x)
    assert payload_of(stream) == ref_payload
    assert mask_first_size(stream) == mask_first_size(ref)
    dec, c2 = F.SZ_decompress(None, stream, dtype=dtype)
    ref_dec, _ = O.decompress(ref, dtype=dtype)
    assert np.array_equal(dec.view(np.uint8), ref_dec.view(np.uint8))
    assert np.abs(dec.astype(np.float64) - x.astype(np.float64)).max() <= c2.absErrorBound


def test_device_tensor_api_roundtrip():
    import torch
    dims = (80, 90, 100)
    x = spectral_field(dims, slope=-3.0, seed=5)
    conf = _conf(dims, rel=1e-3)
    t = torch.from_numpy(x).cuda()
    s1 = F.SZ_compress(conf, t)
    s2 = F.SZ_compress(conf, x)
    assert mask_first_size(s1) == mask_first_size(s2)
    out = torch.empty(dims, dtype=torch.float32, device="cuda")
    c = F.decompress_device(s1, out)
    ref_dec, _ = O.decompress(s1)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref_dec.view(np.uint32))
    small = torch.empty(10, dtype=torch.float32, device="cuda")
    with pytest.raises(F.FazError):
        F.decompress_device(s1, small)
    assert c.dims == list(dims)


def test_large_field_round_trip_properties():
    """512x512x256 float32: error bound holds everywhere, the stream decodes
    to the oracle's array, and compressing twice gives the same bytes."""
    import torch
    dims = (256, 512, 512)
    t = F.fields.spectral_field(dims, slope=-3.5, aniso=(1, 2, 4), noise=0.01, seed=11, device="cuda")
    conf = _conf(dims, rel=1e-3)
    s1 = F.SZ_compress(conf, t)
    s2 = F.SZ_compress(conf, t)
    assert s1 == s2
    out = torch.empty(dims, dtype=torch.float32, device="cuda")
    c = F.decompress_device(s1, out)
    err = (out.double() - t.double()).abs().max().item()
    assert err <= c.absErrorBound
    ref_dec, _ = O.decompress(s1)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref_dec.view(np.uint32))


@pytest.fixture
def verify_fast_path(monkeypatch):
    """Every float quantisation also runs the double path; the library fails
    the call if any point differs (FAZ_VERIFY_FASTPATH)."""
    monkeypatch.setenv("FAZ_VERIFY_FASTPATH", "1")
    yield


def _grid_field(dims, step, seed, lo=-50.0, hi=80.0):
    """Values on a grid of `step`: differences and linear predictions fall
    on exact multiples of the grid, i.e. on quantiser boundaries."""
    rng = np.random.default_rng(seed)
    x = spectral_field(dims, slope=-3.0, seed=seed, lo=lo, hi=hi).astype(np.float64)
    x = np.round(x / step) * step
    x[rng.random(dims) < 0.01] = 0.0
    return x.astype(np.float32)


ADVERSARIAL = [
    ("grid_pow2_eb", (64, 72, 80), 2.0 ** -6, dict(abs_=2.0 ** -6)),
    ("grid_half_eb", (64, 72, 80), 2.0 ** -7, dict(abs_=2.0 ** -6, interp=F.INTERP_ALGO_LINEAR)),
    ("grid_decimal_eb", (50, 60, 70), 1e-3, dict(abs_=1e-3)),
    ("grid_rel", (50, 60, 70), 1e-2, dict(rel=1e-4)),
    ("zeros_trim2", (40, 50, 60), 1e-3, dict(abs_=0.05, trimToZero=2)),
]


@pytest.mark.parametrize("name,dims,step,kw", ADVERSARIAL)
def test_fast_path_agrees_with_double_path(name, dims, step, kw, verify_fast_path):
    x = _grid_field(dims, step, seed=len(name))
    conf = _conf(dims, **kw)
    stream = F.SZ_compress(conf, x)  # raises FazError on any disagreement
    ref, _ = O.compress(conf, x)
    assert mask_first_size(stream) == mask_first_size(ref)
    dec, c2 = F.SZ_decompress(None, stream)
    ref_dec, _ = O.decompress(ref)
    assert np.array_equal(dec.view(np.uint32), ref_dec.view(np.uint32))


def test_fast_path_verified_on_golden_cases(verify_fast_path):
    for name in INI_CASES:
        case = golden_case(name)
        if case["dtype"] != "float32":
            continue
        stream = F.SZ_compress(cli_config(case), golden_input(case))
        assert payload_of(stream) == payload_of(golden_stream(case)), name
        dec, _ = F.SZ_decompress(None, golden_stream(case))
        assert hashlib.sha256(dec.tobytes()).hexdigest() == case["dec_sha256"], name


def test_double_path_only_matches(monkeypatch):
    """FAZ_FASTPATH=0 forces the double path; streams are identical."""
    dims = (60, 70, 80)
    x = spectral_field(dims, slope=-3.0, seed=3)
    conf = _conf(dims, rel=1e-3)
    s_fast = F.SZ_compress(conf, x)
    monkeypatch.setenv("FAZ_FASTPATH", "0")
    s_dp = F.SZ_compress(conf, x)
    assert s_fast == s_dp


def test_gpu_full_code_range():
    """Prediction errors spread over the whole quantisation range: codes
    cover 0..65535 (offset 0 and the top symbol 65535 both occur)."""
    dims = (40, 50, 60)
    rng = np.random.default_rng(7)
    eb = 1e-3
    x = (rng.integers(-70000, 70000, size=dims) * (eb * 1.0001)).astype(np.float32)
    conf = _conf(dims, abs_=eb, interp=F.INTERP_ALGO_LINEAR)
    codes, _, ref_payload = O.interp_codes(conf, x)
    assert codes.min() == 0 and codes.max() == 65535
    stream = F.SZ_compress(conf, x)
    assert payload_of(stream) == ref_payload
    dec, _ = F.SZ_decompress(None, stream, dtype=np.float32)
    ref_dec, _ = O.decompress(O.compress(conf, x)[0])
    assert np.array_equal(dec.view(np.uint32), ref_dec.view(np.uint32))


def _zstd_frames(stream):
    """Number of zstd frames in a stream's body (system libzstd)."""
    import ctypes
    z = ctypes.CDLL("libzstd.so.1")
    z.ZSTD_findFrameCompressedSize.restype = ctypes.c_size_t
    z.ZSTD_findFrameCompressedSize.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    z.ZSTD_isError.argtypes = [ctypes.c_size_t]
    body_end = len(stream) - 4 - int.from_bytes(stream[-4:], "little", signed=True)
    body = stream[8:body_end]
    n, off = 0, 0
    while off < len(body):
        fs = z.ZSTD_findFrameCompressedSize(body[off:], len(body) - off)
        assert not z.ZSTD_isError(fs)
        off += fs
        n += 1
    return n


def test_gpu_zstd_bodies_hold_the_same_payload(monkeypatch):
    """The three ways of writing the zstd body hold the same payload:
    FAZ_ZSTD_THREADS=0 is ZSTD_compress itself (one frame, the oracle's bytes);
    FAZ_ZSTD_THREADS > 0 is one level-3 frame written by zstd's worker
    threads, the same bytes for any worker count; FAZ_ZSTD_MULTIFRAME=1 writes
    independent frames in parallel.  Plain ZSTD_decompress (the oracle) and
    the library's decoder read all of them."""
    import torch
    dims = (128, 256, 256)
    t = F.fields.spectral_field(dims, slope=-3.0, noise=0.01, seed=5, device="cuda")
    conf = _conf(dims, rel=1e-4)
    monkeypatch.setenv("FAZ_ZSTD_THREADS", "0")
    s0 = F.SZ_compress(conf, t)
    assert _zstd_frames(s0) == 1
    ref, ref_payload = O.compress(conf, t.cpu().numpy())
    assert mask_first_size(s0) == mask_first_size(ref)
    monkeypatch.setenv("FAZ_ZSTD_THREADS", "8")
    s8 = F.SZ_compress(conf, t)
    monkeypatch.setenv("FAZ_ZSTD_THREADS", "3")
    s3 = F.SZ_compress(conf, t)
    assert s8 == s3
    assert _zstd_frames(s8) == 1
    monkeypatch.setenv("FAZ_ZSTD_MULTIFRAME", "1")
    smf = F.SZ_compress(conf, t)
    monkeypatch.delenv("FAZ_ZSTD_MULTIFRAME")
    assert _zstd_frames(smf) > 1
    for s in (s8, smf):
        assert payload_of(s) == ref_payload  # the oracle decodes every body
    ref_dec, _ = O.decompress(s0)
    for s in (s8, smf):
        for threads in ("8", "0"):
            monkeypatch.setenv("FAZ_ZSTD_THREADS", threads)
            out = torch.empty(dims, dtype=torch.float32, device="cuda")
            F.decompress_device(s, out)
            assert np.array_equal(out.cpu().numpy().view(np.uint32), ref_dec.view(np.uint32))


def test_gpu_c1_full_size_matches_oracle():
    """The CPU-runnable configuration at full size (100x500x500, cubic, REL
    1e-3): the GPU payload and decompressed array equal the oracle's, which
    test_c1_reference.py pins to the reference tool."""
    from test_c1_reference import c1_conf, c1_field
    x = c1_field()
    stream = F.SZ_compress(c1_conf(), x)
    ref, ref_payload = O.compress(c1_conf(), x)
    assert payload_of(stream) == ref_payload
    dec, c2 = F.SZ_decompress(None, stream)
    ref_dec, _ = O.decompress(ref)
    assert np.array_equal(dec.reshape(-1).view(np.uint32), ref_dec.reshape(-1).view(np.uint32))
    assert np.abs(dec.astype(np.float64) - x.astype(np.float64)).max() <= c2.absErrorBound
