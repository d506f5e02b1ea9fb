"""OpenMP streams (Config::openmp, SZ_compress_OMP / SZ_decompress_OMP,
include/QoZ/api/impl/SZImplOMP.hpp:10-149): the field cut into slabs along
its slowest axis, one per OpenMP thread, each compressed as a field of its
own with the whole field's error bound.  The reference tool's streams
(OMP_NUM_THREADS fixed per case) against the oracle (CPU) and the GPU path."""
import hashlib

import numpy as np
import pytest

from conftest import cli_config, golden_case, golden_input, golden_manifest, golden_stream, mask_omp
from faz_gb300.fields import spectral_field

import oracle.oracle as O

OMP_CASES = [c["name"] for c in golden_manifest(omp=True) if "omp_threads" in c]


@pytest.fixture
def ref_zstd():
    if O.os.path.exists(O.REF_ZSTD):
        O.set_zstd(O.REF_ZSTD)
        yield True
    else:
        O.set_zstd(None)
        yield False
    O.set_zstd(None)


def test_omp_cases_exist():
    assert len(OMP_CASES) >= 3


@pytest.mark.parametrize("name", OMP_CASES)
def test_oracle_reads_and_decodes_reference_omp_stream(name):
    case = golden_case(name)
    ref = golden_stream(case)
    conf, slabs = O.read_omp(ref)
    assert len(slabs) == case["omp_threads"]
    assert conf.openmp == 1 and conf.errorBoundMode == 0  # EB_ABS after calAbsErrorBound
    rows = sum(ct.dims[0] for ct, _ in slabs)
    assert rows == case["dims"][0]
    dec, _ = O.decompress(ref, np.dtype(case["dtype"]))
    assert hashlib.sha256(dec.tobytes()).hexdigest() == case["dec_sha256"]


@pytest.mark.parametrize("name", OMP_CASES)
def test_oracle_omp_stream_matches_reference(name, ref_zstd, monkeypatch):
    if not ref_zstd:
        pytest.skip("the reference's zstd build is not here")
    case = golden_case(name)
    monkeypatch.setenv("OMP_NUM_THREADS", str(case["omp_threads"]))
    stream, _ = O.compress(cli_config(case), golden_input(case))
    assert mask_omp(stream) == mask_omp(golden_stream(case))


def test_oracle_omp_slab_rows():
    # rows [t*d0//n, (t+1)*d0//n) cover the field with no gap
    for d0, n in [(10, 3), (7, 7), (100, 16), (5, 2)]:
        rows = [O._omp_rows(d0, t, n) for t in range(n)]
        assert rows[0][0] == 0 and rows[-1][1] == d0
        assert all(a[1] == b[0] and a[1] > a[0] for a, b in zip(rows, rows[1:]))


# ------------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("name", OMP_CASES)
def test_gpu_decompresses_reference_omp_stream(name):
    import faz_gb300 as F
    case = golden_case(name)
    dec, conf = F.SZ_decompress(None, golden_stream(case), dtype=np.dtype(case["dtype"]))
    assert conf.openmp == 1
    assert hashlib.sha256(np.ascontiguousarray(dec).tobytes()).hexdigest() == case["dec_sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", OMP_CASES)
def test_gpu_omp_stream_matches_oracle_and_reference(name, monkeypatch):
    import faz_gb300 as F
    O.set_zstd(None)  # the oracle uses the same host zstd as the library
    case = golden_case(name)
    x = golden_input(case)
    monkeypatch.setenv("OMP_NUM_THREADS", str(case["omp_threads"]))
    monkeypatch.setenv("FAZ_ZSTD_THREADS", "0")
    stream = F.SZ_compress(cli_config(case), x)
    ref, _ = O.compress(cli_config(case), x)
    assert mask_omp(stream) == mask_omp(ref)
    # slab by slab, the reference's payloads (pre-zstd) and Configs
    _, ours = O.read_omp(stream)
    _, theirs = O.read_omp(golden_stream(case))
    assert len(ours) == len(theirs) == case["omp_threads"]
    for (c1, s1), (c2, s2) in zip(ours, theirs):
        assert c1.dims == c2.dims and c1.cmprAlgo == c2.cmprAlgo
        assert O.read_stream(s1)[1] == O.read_stream(s2)[1]
    dec, c3 = F.SZ_decompress(None, stream, dtype=x.dtype)
    assert np.abs(dec.astype(np.float64) - x.astype(np.float64)).max() <= c3.absErrorBound


@pytest.mark.gpu
def test_gpu_omp_device_roundtrip(monkeypatch):
    import torch
    import faz_gb300 as F
    dims = (50, 60, 70)
    x = torch.from_numpy(spectral_field(dims, slope=-3.0, seed=9)).to("cuda:0")
    conf = F.Config(*dims)
    conf.cmprAlgo = F.ALGO_INTERP
    conf.errorBoundMode = F.EB_REL
    conf.relErrorBound = 1e-3
    conf.openmp = 1
    monkeypatch.setenv("OMP_NUM_THREADS", "6")
    s = F.compress_device(conf, x)
    assert len(O.read_omp(s)[1]) == 6
    out = torch.empty_like(x)
    c2 = F.decompress_device(s, out)
    assert (out.double() - x.double()).abs().max().item() <= c2.absErrorBound
