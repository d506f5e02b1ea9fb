"""Seeded random configurations of the tuners and compressors: the oracle
against the reference tool (oracle/_ref/faz, built from the reference sources
by oracle/build_ref.sh, with its bundled zstd 1.4.5), run where that build
exists.  Each case draws a field (spectral, sum of lower-dimensional
functions, or random walk; 2-D or 3-D; float or double) and an INI / flag set
covering the default SZ3 tuner, QoZ (-q), QoZ-branch rates (with and without
autoTuningRate, level-wise selection, the Lorenzo candidate), explicit
ALGO_INTERP and ALGO_LORENZO_REG, and compares the streams (the Lorenzo fast
frontend's uninitialised padding bytes and the trailer's firstSize masked).
The GPU counterpart (tests/test_gpu_fuzz.py) replays the same cases against
the oracle."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import cli_config, mask_fast_frontend_padding, mask_first_size, write_ini

import oracle.oracle as O
from fuzz_cases import fuzz_cases

HERE = os.path.dirname(os.path.abspath(__file__))
FAZ = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "faz")

CASES = fuzz_cases()


def _reference_stream(case, x, td):
    inp = os.path.join(td, "in.bin")
    out = os.path.join(td, "out.faz")
    x.tofile(inp)
    dims = [str(d) for d in reversed(case["dims"])]
    cmd = [FAZ, "-f" if x.dtype == np.float32 else "-d", "-F", "0", "-i", inp, "-z", out,
           f"-{len(dims)}"] + dims + case["flags"]
    if case["ini"] is not None:
        ip = os.path.join(td, "cfg.ini")
        write_ini(ip, case["ini"])
        cmd += ["-c", ip]
    r = subprocess.run(cmd, cwd=td, capture_output=True, text=True)
    if r.returncode:
        return None  # the reference itself fails (e.g. its CompressTest overflows on noisy data)
    return open(out, "rb").read()


@pytest.mark.skipif(not (os.path.exists(FAZ) and os.path.exists(O.REF_ZSTD)), reason="reference build absent")
@pytest.mark.parametrize("idx", range(len(CASES)))
def test_oracle_matches_reference_tool_on_random_configuration(idx):
    case, x = CASES[idx]["case"], CASES[idx]["field"]()
    O.set_zstd(O.REF_ZSTD)
    try:
        with tempfile.TemporaryDirectory() as td:
            ref = _reference_stream(case, x, td)
        if ref is None:
            pytest.skip("the reference tool fails on this case")
        ours, _ = O.compress(cli_config(case), x)
        c1, p1 = O.read_stream(ours)
        c2, p2 = O.read_stream(ref)
        assert c1.cmprAlgo == c2.cmprAlgo
        if c1.cmprAlgo == 0 and len(case["dims"]) == 3:
            assert mask_fast_frontend_padding(p1, x.itemsize) == mask_fast_frontend_padding(p2, x.itemsize)
        else:
            assert p1 == p2
            assert mask_first_size(ours) == mask_first_size(ref)
    finally:
        O.set_zstd(None)
