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

from conftest import (cli_config, golden_case, golden_input, golden_manifest, golden_stream,
                      mask_fast_frontend_padding, mask_first_size, parse_interp_header, tuned_config)

import oracle.oracle as O

ALGO_INTERP, ALGO_LORENZO_REG = 2, 0


def _trailer_algo(name):
    return O.read_stream(golden_stream(golden_case(name)))[0].cmprAlgo


INI_CASES = [c["name"] for c in golden_manifest() if c["ini"] is not None]
TUNED_CASES = [c["name"] for c in golden_manifest() if c["ini"] is None and _trailer_algo(c["name"]) == ALGO_INTERP]
# default configuration (ALGO_INTERP_LORENZO) without QoZ tuning: the SZ3 tuner
SZ3_CASES = [c["name"] for c in golden_manifest() if c["ini"] is None and "-q" not in c["flags"]]
# QoZ tuning (-q)
QOZ_CASES = [c["name"] for c in golden_manifest() if c["ini"] is None and "-q" in c["flags"]]
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


def _same_stream(ours, ref, zstd_lib, itemsize=4):
    c1, p1 = O.read_stream(ours)
    c2, p2 = O.read_stream(ref)
    assert c1.cmprAlgo == c2.cmprAlgo
    if c1.cmprAlgo == ALGO_LORENZO_REG and c1.N == 3:
        # the reference writes uninitialised struct padding into the 3-D fast
        # frontend's payloads, so their zstd frames differ; payload and
        # trailer must not
        assert mask_fast_frontend_padding(p1, itemsize) == mask_fast_frontend_padding(p2, itemsize)
        n1 = int.from_bytes(ours[-4:], "little", signed=True)
        n2 = int.from_bytes(ref[-4:], "little", signed=True)
        assert mask_first_size(ours)[-4 - n1:] == mask_first_size(ref)[-4 - n2:]
        return
    if zstd_lib == "1.4.5":
        assert mask_first_size(ours) == mask_first_size(ref)
    else:
        assert p1 == p2
        # trailer bytes
        n1 = int.from_bytes(ours[-4:], "little", signed=True)
        n2 = int.from_bytes(ref[-4:], "little", signed=True)
        assert mask_first_size(ours)[-4 - n1:] == mask_first_size(ref)[-4 - n2:]


@pytest.mark.parametrize("name", INI_CASES)
def test_oracle_stream_matches_reference(name, zstd_lib):
    case = golden_case(name)
    x = golden_input(case)
    stream, _ = O.compress(cli_config(case), x)
    _same_stream(stream, golden_stream(case), zstd_lib, x.itemsize)


@pytest.mark.parametrize("name", SZ3_CASES)
def test_oracle_sz3_tuner_matches_reference(name, zstd_lib):
    """The whole default path: tuner decisions, then the chosen compressor."""
    case = golden_case(name)
    x = golden_input(case)
    ref = golden_stream(case)
    rc, _ = O.read_stream(ref)
    tuned = O.sz3_tune(cli_config(case), x)
    for f in ("cmprAlgo", "interpAlgo", "interpDirection", "quantbinCnt", "blockSize", "pred_dim", "lorenzo",
              "lorenzo2", "regression"):
        assert getattr(tuned, f) == getattr(rc, f), f
    stream, _ = O.compress(cli_config(case), x)
    _same_stream(stream, ref, zstd_lib, x.itemsize)


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
    """The reference's decoded array, bit for bit.  Where the reference tool
    cannot decode its own stream (reg1d_thin: its decoder reads a selection
    past the end of the list for the one-point final block that fell back to
    the one-layer Lorenzo predictor), the oracle's decode must equal the
    reconstruction the compressor made, which the error bound and the
    re-compression below pin."""
    case = golden_case(name)
    dec, conf = O.decompress(golden_stream(case), dtype=np.dtype(case["dtype"]))
    x = golden_input(case)
    if case["dec_sha256"] is not None:
        assert hashlib.sha256(dec.tobytes()).hexdigest() == case["dec_sha256"]
    else:
        assert "ref_decode" in case
    err = np.abs(dec.astype(np.float64) - x.astype(np.float64)).max()
    assert err <= conf.absErrorBound


def test_oracle_one_point_final_block_falls_back():
    """reg1d_thin (3841 points, blocks of 128): the composed predictor
    (Lorenzo, regression) picks regression for the one-point final block,
    regression refuses it (RegressionPredictor.hpp:48-56) and the frontend
    predicts it with the one-layer Lorenzo fallback without recording a
    selection (SZGeneralFrontend.hpp:48-54): the stream holds one selection
    fewer than blocks.  Decoding the last point with any other predictor would
    break its error bound."""
    import struct
    case = golden_case("reg1d_thin")
    conf, pl = O.read_stream(golden_stream(case))
    nb = (case["dims"][0] - 1) // conf.blockSize + 1
    p = 8 + 4 + 1 + 1  # dims, block size, Lorenzo id, regression id
    ncoef = struct.unpack_from("<Q", pl, p)[0]
    p += 8
    for _ in range(2):  # the two coefficient quantizers
        nun = struct.unpack_from("<Q", pl, p + 1 + 8 + 4)[0]
        p += 1 + 8 + 4 + 8 + 4 * nun
    assert ncoef > 0
    p = _skip_huffman(pl, p)  # the coefficient codes
    assert struct.unpack_from("<Q", pl, p)[0] == nb - 1  # selections
    dec, c2 = O.decompress(golden_stream(case), dtype=np.float32)
    x = golden_input(case)
    assert abs(float(dec[-1]) - float(x[-1])) <= c2.absErrorBound


def _skip_huffman(pl, p):
    """Offset past one HuffmanEncoder<int> save + encode (HuffmanEncoder.hpp:
    119-137, 150-227): offset, big-endian node count and state count, the
    endianness byte, left / right child arrays (1, 2 or 4 bytes an entry by
    node count), symbols, leaf flags, then the byte count and the bits."""
    import struct
    nc = struct.unpack_from(">i", pl, p + 4)[0]
    w = 1 if nc <= 256 else (2 if nc <= 65536 else 4)
    p += 4 + 4 + 4 + 1 + 2 * w * nc + 4 * nc + nc
    nbytes = struct.unpack_from("<Q", pl, p)[0]
    return p + 8 + nbytes


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


@pytest.mark.parametrize("name", QOZ_CASES)
def test_oracle_qoz_tuner_matches_reference(name, zstd_lib):
    """QoZ tuning: per-level interpolators and directions, alpha/beta, then
    the interpolation stream."""
    case = golden_case(name)
    x = golden_input(case)
    ref = golden_stream(case)
    rc, rp = O.read_stream(ref)
    stream, payload = O.compress(cli_config(case), x)
    h1 = parse_interp_header(rp, len(case["dims"]))
    h2 = parse_interp_header(payload, len(case["dims"]))
    assert h1 == h2
    assert payload == rp
    _same_stream(stream, ref, zstd_lib, x.itemsize)
