"""The seeded random configurations of tests/fuzz_cases.py on the GPU against
the oracle (same host zstd): tuner decisions, pre-zstd payload and stream
(the Lorenzo fast frontend's padding bytes and the trailer's firstSize
masked), and the decompressed field within the bound.  A case the GPU path
rejects as unsupported (for example a Lorenzo interval estimate above 65536
bins) is skipped, and so is one the oracle rejects."""
import numpy as np
import pytest

import faz_gb300 as F
from conftest import cli_config, mask_fast_frontend_padding, mask_first_size
from fuzz_cases import fuzz_cases

import oracle.oracle as O

pytestmark = pytest.mark.gpu

CASES = fuzz_cases()


@pytest.fixture(scope="module", autouse=True)
def system_zstd():
    O.set_zstd(None)
    yield


@pytest.mark.parametrize("idx", range(len(CASES)))
def test_gpu_matches_oracle_on_random_configuration(idx):
    case, x = CASES[idx]["case"], CASES[idx]["field"]()
    try:
        ref, ref_payload = O.compress(cli_config(case), x)
    except RuntimeError as e:
        pytest.skip(f"oracle: {e}")
    try:
        stream = F.SZ_compress(cli_config(case), x)
    except F.FazError as e:
        if "UNSUPPORTED" in str(e):
            pytest.skip(str(e))
        raise
    c1, p1 = O.read_stream(stream)
    c2, _ = O.read_stream(ref)
    for f in ("cmprAlgo", "interpAlgo", "interpDirection", "alpha", "beta", "quantbinCnt", "blockSize", "pred_dim",
              "maxStep"):
        assert getattr(c1, f) == getattr(c2, f), f
    if c1.cmprAlgo == 0 and len(case["dims"]) == 3:
        assert mask_fast_frontend_padding(p1, x.itemsize) == mask_fast_frontend_padding(ref_payload, x.itemsize)
    else:
        assert p1 == ref_payload
        assert mask_first_size(stream) == mask_first_size(ref)
    dec, c3 = F.SZ_decompress(None, stream, dtype=x.dtype)
    assert np.abs(dec.astype(np.float64) - x.astype(np.float64)).max() <= c3.absErrorBound
