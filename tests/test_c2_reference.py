"""The oracle against the reference tool at the benchmark's size: a 512x512x512
float32 spectral field (k^-3.5, correlation lengths 1:2:4, 1 % noise, scaled
to [-50, 80], seeded; numpy's generator) at relative bound 1e-3 with the
default configuration, whose SZ3 sampled autotune
(include/QoZ/api/impl/SZInterp.hpp:2115-2187, 2561-2880) samples this field
with its full-size geometry.  The oracle's stream (with the reference's zstd
1.4.5) equals the stream of oracle/_ref/faz, built from the reference sources
by oracle/build_ref.sh, and the oracle decodes that stream to the tool's own
array.  Runs where that build exists; tests/test_gpu_scale.py compares the
library with the oracle on the benchmark's field at every bound."""
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

C2_DIMS = (512, 512, 512)


@pytest.mark.skipif(not (os.path.exists(FAZ) and os.path.exists(O.REF_ZSTD)), reason="reference build absent")
def test_oracle_matches_reference_tool_on_the_512_cube():
    x = spectral_field(C2_DIMS, slope=-3.5, aniso=(1, 2, 4), noise=0.01, seed=1000)
    conf = F.Config(*C2_DIMS)
    conf.errorBoundMode, conf.relErrorBound = F.EB_REL, 1e-3
    O.set_zstd(O.REF_ZSTD)
    try:
        ours, _ = O.compress(conf, x)
        with tempfile.TemporaryDirectory() as td:
            inp, cmp_, dec = (os.path.join(td, n) for n in ("x.f32", "x.faz", "x.out"))
            x.tofile(inp)
            dims = ["-3", "512", "512", "512"]
            subprocess.check_call([FAZ, "-f", "-F", "0", "-i", inp, "-z", cmp_] + dims + ["-M", "REL", "1e-3"],
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
