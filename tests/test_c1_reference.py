"""The CPU-runnable configuration at full size (100x500x500 float32, spectral
k^-3 field plus 1% noise scaled to [-50, 80], cubic ALGO_INTERP, relative
bound 1e-3): the oracle's stream and decompressed array against the
reference tool's own (oracle/_ref/faz, built from the reference sources by
oracle/build_ref.sh, with its bundled zstd 1.4.5).  Runs where that build
exists; the GPU test of the same case compares the library with the oracle."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import faz_gb300 as F
from faz_gb300.fields import spectral_field
from conftest import mask_first_size

import oracle.oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
FAZ = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "faz")

C1_DIMS = (100, 500, 500)


def c1_field():
    return spectral_field(C1_DIMS, slope=-3.0, noise=0.01, seed=101)


def c1_conf():
    c = F.Config(*C1_DIMS)
    c.cmprAlgo, c.interpAlgo = F.ALGO_INTERP, F.INTERP_ALGO_CUBIC
    c.errorBoundMode, c.relErrorBound = F.EB_REL, 1e-3
    return c


@pytest.mark.skipif(not (os.path.exists(FAZ) and os.path.exists(O.REF_ZSTD)), reason="reference build absent")
def test_oracle_matches_reference_tool_on_the_full_c1_field():
    x = c1_field()
    O.set_zstd(O.REF_ZSTD)
    try:
        ours, _ = O.compress(c1_conf(), x)
        with tempfile.TemporaryDirectory() as td:
            inp, cmp_, dec = (os.path.join(td, n) for n in ("x.f32", "x.faz", "x.out"))
            x.tofile(inp)
            ini = os.path.join(td, "c.ini")
            with open(ini, "w") as f:
                f.write("[GlobalSettings]\nCmprAlgo = ALGO_INTERP\n[AlgoSettings]\nInterpolationAlgo = INTERP_ALGO_CUBIC\n")
            dims = ["-3", "500", "500", "100"]
            subprocess.check_call([FAZ, "-f", "-F", "0", "-i", inp, "-z", cmp_] + dims + ["-M", "REL", "1e-3", "-c", ini],
                                  cwd=td, stdout=subprocess.DEVNULL)
            subprocess.check_call([FAZ, "-f", "-z", cmp_, "-o", dec] + dims + ["-M", "ABS", "1"], cwd=td,
                                  stdout=subprocess.DEVNULL)
            ref = open(cmp_, "rb").read()
            ref_dec = np.fromfile(dec, dtype=np.float32)
        assert mask_first_size(ours) == mask_first_size(ref)
        odec, _ = O.decompress(ref)
        assert np.array_equal(odec.reshape(-1).view(np.uint32), ref_dec.view(np.uint32))
    finally:
        O.set_zstd(None)
