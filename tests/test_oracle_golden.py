"""Pins the CPU oracle against streams written by the reference build.

The fixtures in tests/golden were made by the reference `faz` tool (see
tests/golden/make_golden.py).  With the reference's own zstd 1.4.5 at hand
(oracle/_ref/libzstd145.so, built by oracle/build_ref.sh) whole streams are
compared; otherwise the pre-zstd payloads and trailers are.
"""
import hashlib
import os

import numpy as np
import pytest

from conftest import (cli_config, golden_case, golden_input, golden_manifest, golden_stream, mask_first_size,
                      tuned_config)

import oracle.oracle as O

INI_CASES = [c["name"] for c in golden_manifest() if c["ini"] is not None]
TUNED_CASES = [c["name"] for c in golden_manifest() if c["ini"] is None]
ALL_CASES = [c["name"] for c in golden_manifest()]


@pytest.fixture(scope="module", autouse=True)
def zstd_lib():
    if os.path.exists(O.REF_ZSTD):
        O.set_zstd(O.REF_ZSTD)
        yield "1.4.5"
    else:
        O.set_zstd(None)
        yield "system"
    O.set_zstd(None)


def _same_stream(ours, ref, zstd_lib):
    if zstd_lib == "1.4.5":
        assert mask_first_size(ours) == mask_first_size(ref)
    else:
        c1, p1 = O.read_stream(ours)
        c2, p2 = O.read_stream(ref)
        assert p1 == p2
        # trailer bytes
        n1 = int.from_bytes(ours[-4:], "little", signed=True)
        n2 = int.from_bytes(ref[-4:], "little", signed=True)
        assert mask_first_size(ours)[-4 - n1:] == mask_first_size(ref)[-4 - n2:]


@pytest.mark.parametrize("name", INI_CASES)
def test_oracle_stream_matches_reference(name, zstd_lib):
    case = golden_case(name)
    stream, _ = O.compress(cli_config(case), golden_input(case))
    _same_stream(stream, golden_stream(case), zstd_lib)


@pytest.mark.parametrize("name", TUNED_CASES)
def test_oracle_payload_matches_tuned_reference(name, zstd_lib):
    """Compressor parity for tuner-written streams, given the tuner's decisions."""
    case = golden_case(name)
    conf = tuned_config(case)
    _, ref_payload = O.read_stream(golden_stream(case))
    _, payload = O.compress(conf, golden_input(case))
    assert payload == ref_payload


@pytest.mark.parametrize("name", ALL_CASES)
def test_oracle_decompress_matches_reference(name):
    case = golden_case(name)
    dec, conf = O.decompress(golden_stream(case), dtype=np.dtype(case["dtype"]))
    assert hashlib.sha256(dec.tobytes()).hexdigest() == case["dec_sha256"]
    x = golden_input(case)
    err = np.abs(dec.astype(np.float64) - x.astype(np.float64)).max()
    assert err <= conf.absErrorBound


def test_ska_order_small():
    """Keys 0..4 inserted in order: 4 keys fit 4 buckets; the 5th doubles to 8."""
    order = O.ska_order(np.array([32768, 32767, 32769, 32766, 32770], dtype=np.int32))
    assert sorted(order.tolist()) == [0, 1, 2, 3, 4]
    # bucket of key k with B buckets: top log2(B) bits of k * 0x9E3779B97F4A7C15
    keys = [32768, 32767, 32769, 32766, 32770]
    b = [((k * 11400714819323198485) % (1 << 64)) >> 61 for k in keys]
    # iteration visits buckets from high to low
    visited = [b[i] for i in order]
    assert visited == sorted(visited, reverse=True)
