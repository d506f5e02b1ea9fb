import configparser
import json
import os
import struct
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
# Full-stream comparisons with the oracle need the frame single-threaded
# ZSTD_compress writes; the library's default compresses the final frame with
# worker threads (same payload, different frame).
os.environ.setdefault("FAZ_ZSTD_THREADS", "0")
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


def golden_manifest(omp=False):
    """The golden cases; OpenMP streams (slab containers, "omp_threads" in
    the manifest) only with omp=True."""
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        cases = json.load(f)["cases"]
    return [c for c in cases if omp or "omp_threads" not in c]


def golden_case(name):
    for c in golden_manifest(omp=True):
        if c["name"] == name:
            return c
    raise KeyError(name)


def golden_input(case):
    arr = np.fromfile(os.path.join(GOLDEN, case["name"] + ".in"), dtype=np.dtype(case["dtype"]))
    return arr.reshape(case["dims"])


def golden_stream(case):
    with open(os.path.join(GOLDEN, case["name"] + ".faz"), "rb") as f:
        return f.read()


def golden_dec_sha(case):
    """SHA-256 of the array the reference decodes from the case's stream.  For
    a stream the reference tool writes but cannot decode ("ref_decode" in the
    manifest) the oracle's decoder, which applies the compressor's own
    predictor choice, stands in."""
    if case["dec_sha256"] is not None:
        return case["dec_sha256"]
    import hashlib
    import oracle.oracle as O
    dec, _ = O.decompress(golden_stream(case), dtype=np.dtype(case["dtype"]))
    return hashlib.sha256(dec.tobytes()).hexdigest()


# INI keys of QoZ::Config::loadcfg (include/QoZ/utils/Config.hpp:91-233) used by the fixtures
_INI_INT = {"InterpDirection": "interpDirection", "InterpBlockSize": "interpBlockSize",
            "fixBlockSize": "fixBlockSize", "trimToZero": "trimToZero", "maxStep": "maxStep",
            "QuantizationBinTotal": "quantbinCnt", "blockOrder": "blockOrder", "BlockSize": "blockSize",
            "sampleBlockSize": "sampleBlockSize", "levelwisePredictionSelection": "levelwisePredictionSelection",
            "testLorenzo": "testLorenzo", "profiling": "profiling", "var_first": "var_first", "abList": "abList",
            "blockwiseSampleBlockSize": "blockwiseSampleBlockSize", "crossBlock": "crossBlock"}
_INI_REAL = {"alpha": "alpha", "beta": "beta", "autoTuningRate": "autoTuningRate",
             "predictorTuningRate": "predictorTuningRate"}
_INI_BOOL = {"Lorenzo": "lorenzo", "Lorenzo2ndOrder": "lorenzo2", "Regression": "regression",
             "Regression2ndOrder": "regression2"}


def cli_config(case):
    """Config as the reference CLI builds it from the case's flags and INI."""
    from faz_gb300.config import (Config, ALGO_STR, INTERP_ALGO_STR, EB_ABS, EB_REL, EB_ABS_AND_REL)
    conf = Config(*case["dims"])
    flags = list(case["flags"])
    if "-q" in flags:
        conf.QoZ = 1
    if "-C" in flags:
        conf.maxStep = int(flags[flags.index("-C") + 1])
    ini = case["ini"]
    if ini:
        cp = configparser.ConfigParser()
        cp.optionxform = str
        cp.read_dict(ini)
        g = cp["GlobalSettings"] if cp.has_section("GlobalSettings") else {}
        a = cp["AlgoSettings"] if cp.has_section("AlgoSettings") else {}
        if "CmprAlgo" in g:
            conf.cmprAlgo = ALGO_STR.index(g["CmprAlgo"])
        if "tuningTarget" in g:
            conf.tuningTarget = ["TUNING_TARGET_RD", "TUNING_TARGET_CR", "TUNING_TARGET_SSIM",
                                 "TUNING_TARGET_AC"].index(g["tuningTarget"])
        if "OpenMP" in g:
            conf.openmp = 1 if g["OpenMP"].strip().lower() in ("true", "yes", "on", "1") else 0
        if "InterpolationAlgo" in a:
            conf.interpAlgo = INTERP_ALGO_STR.index(a["InterpolationAlgo"])
        for k, f in _INI_INT.items():
            if k in a:
                setattr(conf, f, int(a[k]))
        for k, f in _INI_REAL.items():
            if k in a:
                setattr(conf, f, float(a[k]))
        for k, f in _INI_BOOL.items():
            if k in a:
                setattr(conf, f, 1 if a[k].strip().lower() in ("true", "yes", "on", "1") else 0)
    m = flags.index("-M")
    mode = flags[m + 1]
    val = flags[m + 2] if m + 2 < len(flags) and not flags[m + 2].startswith("-") else None
    if "-A" in flags:
        conf.absErrorBound = float(flags[flags.index("-A") + 1])
    if "-R" in flags:
        conf.relErrorBound = float(flags[flags.index("-R") + 1])
    if mode == "ABS":
        conf.errorBoundMode = EB_ABS
        if val:
            conf.absErrorBound = float(val)
    elif mode == "REL":
        conf.errorBoundMode = EB_REL
        if val:
            conf.relErrorBound = float(val)
    elif mode == "ABS_AND_REL":
        conf.errorBoundMode = EB_ABS_AND_REL
    else:
        raise ValueError(mode)
    return conf


def parse_interp_header(payload, N):
    """Decisions recorded in an interpolation stream header
    (include/QoZ/compressor/SZInterpolationCompressor.hpp:489-512)."""
    o = 8 * N
    bs, interp, direction = struct.unpack_from("<Iii", payload, o)
    o += 12
    alpha, beta, max_step = struct.unpack_from("<ddQ", payload, o)
    o += 24
    (nlist,) = struct.unpack_from("<i", payload, o)
    o += 4
    bwt = payload[o]
    o += 1
    (fixbs,) = struct.unpack_from("<i", payload, o)
    o += 4
    (cross,) = struct.unpack_from("<Q", payload, o)
    o += 8
    trim, border = struct.unpack_from("<ii", payload, o)
    o += 8
    il = list(payload[o:o + nlist])
    dl = list(payload[o + nlist:o + 2 * nlist])
    return dict(blocksize=bs, interp=interp, direction=direction, alpha=alpha, beta=beta, maxStep=max_step,
                nlist=nlist, blockwise=bwt, fixBlockSize=fixbs, crossBlock=cross, trimToZero=trim,
                blockOrder=border, interp_list=il, dir_list=dl)


def tuned_config(case):
    """Config that reproduces a tuner-written interpolation stream without
    running the tuner: the trailer's settings plus the header's decisions."""
    import oracle.oracle as O
    stream = golden_stream(case)
    conf, payload = O.read_stream(stream)
    h = parse_interp_header(payload, conf.N)
    conf.interpAlgo_list = h["interp_list"]
    conf.interpDirection_list = h["dir_list"]
    return conf


def write_ini(path, d):
    """An INI file in the layout tests/golden/make_golden.py gave the reference."""
    with open(path, "w") as f:
        for sec, kv in d.items():
            f.write(f"[{sec}]\n")
            for k, v in kv.items():
                f.write(f"{k} = {v}\n")


def mask_fast_frontend_padding(payload, itemsize):
    """Zero the padding bytes of the Lorenzo fast frontend's raw structs in a
    pre-zstd payload: meta_params (bytes 11 and 41-43 of its 44) and
    meanInfo<T> (the bytes after its bool), which the reference writes from
    uninitialised memory (include/QoZ/frontend/SZFastFrontend.hpp:48-53)."""
    b = bytearray(payload)
    for i in [11, 41, 42, 43] + list(range(53, 52 + itemsize)):
        b[i] = 0
    return bytes(b)


def mask_first_size(stream):
    """Zero the trailer's Config::firstSize bytes (never set by the reference)."""
    (cs,) = struct.unpack_from("<i", stream, len(stream) - 4)
    t0 = len(stream) - 4 - cs
    N = stream[t0]
    a, b = 102 + 8 * N, 110 + 8 * N
    return stream[:t0 + a] + b"\0" * (b - a) + stream[t0 + b:]


def mask_omp(stream):
    """An OpenMP stream with the firstSize bytes of every Config (the slabs'
    and the field's) zeroed."""
    import oracle.oracle as O
    conf, slabs = O.read_omp(stream)
    n = len(slabs)
    parts, confs = [], []
    for _, s in slabs:
        s = mask_first_size(s)
        (cs,) = struct.unpack_from("<i", s, len(s) - 4)
        parts.append(s[:len(s) - 4 - cs])
        confs.append(s[len(s) - 4 - cs:len(s) - 4])
    body = struct.pack("<i", n) + b"".join(confs) + b"".join(struct.pack("<Q", len(p)) for p in parts) + b"".join(parts)
    (cs,) = struct.unpack_from("<i", stream, len(stream) - 4)
    return body + mask_first_size(stream[len(stream) - 4 - cs:])
