"""C ABI boundary checks that need no GPU: exports, struct layout, defaults,
INI loading, and that compute calls fail loudly without a device."""
import ctypes
import os
import re

import numpy as np
import pytest

import faz_gb300 as F
from faz_gb300.config import FazConfigStruct

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from faz_gb300 import build as B
    B.build()
    return F.library()


def declared_functions():
    src = open(os.path.join(ROOT, "include", "faz_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(faz_[a-z_0-9]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(F.api.EXPORTED)


def test_struct_layout_matches(lib):
    assert lib.faz_config_size() == ctypes.sizeof(FazConfigStruct)


def test_config_init_defaults_match_python_mirror(lib):
    for dims in ([100], [100, 200], [100, 200, 300], [2, 3, 4, 5]):
        s = FazConfigStruct()
        arr = (ctypes.c_uint64 * 4)(*dims, *([0] * (4 - len(dims))))
        assert lib.faz_config_init(ctypes.byref(s), len(dims), arr) == 0
        py = F.Config(*dims).to_struct()
        assert bytes(s) == bytes(py)
        # QoZ::Config defaults (include/QoZ/utils/Config.hpp:64-74, 394-499)
        assert s.cmprAlgo == F.ALGO_INTERP_LORENZO and s.quantbinCnt == 65536 and s.interpBlockSize == 32
        assert s.blockSize == {1: 128, 2: 16, 3: 6, 4: 6}[len(dims)]
        assert s.alpha == -1 and s.beta == -1 and s.sperr == -1 and s.pyBind == 1


def test_config_init_rejects_bad_rank(lib):
    s = FazConfigStruct()
    arr = (ctypes.c_uint64 * 4)(1, 1, 1, 1)
    assert lib.faz_config_init(ctypes.byref(s), 5, arr) == F.api.FazError(-1, "").code


def test_ini_loader(tmp_path, lib):
    p = tmp_path / "c.ini"
    p.write_text("[GlobalSettings]\nCmprAlgo = ALGO_INTERP\nErrorBoundMode = REL ; inline comment\n"
                 "RelErrorBound = 1e-4\n# comment\n[AlgoSettings]\nInterpolationAlgo = INTERP_ALGO_LINEAR\n"
                 "interpdirection = 5\nalpha = 1.25\nbeta = 3\nmaxStep = 0x10\nLorenzo = no\n")
    c = F.load_ini(F.Config(10, 20, 30), str(p))
    assert c.cmprAlgo == F.ALGO_INTERP and c.errorBoundMode == F.EB_REL and c.relErrorBound == 1e-4
    assert c.interpAlgo == F.INTERP_ALGO_LINEAR and c.interpDirection == 5
    assert c.alpha == 1.25 and c.beta == 3.0 and c.maxStep == 16 and c.lorenzo == 0
    with pytest.raises(F.FazError):
        F.load_ini(F.Config(10), str(tmp_path / "missing.ini"))


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device error path")
def test_compress_without_device_fails_loudly(lib):
    c = F.Config(8, 8, 8)
    c.cmprAlgo = F.ALGO_INTERP
    with pytest.raises(F.FazError) as ei:
        F.SZ_compress(c, np.zeros((8, 8, 8), np.float32))
    assert ei.value.code == -3


def test_decompress_rejects_garbage(lib):
    with pytest.raises(F.FazError):
        F.SZ_decompress(None, b"\x01\x02\x03")
    with pytest.raises(F.FazError):
        F.SZ_decompress(None, b"\x00" * 64)


def test_unsupported_algo_is_reported(lib):
    c = F.Config(8, 8, 8)  # default cmprAlgo = ALGO_INTERP_LORENZO
    c.absErrorBound = 0.1
    with pytest.raises(F.FazError) as ei:
        F.SZ_compress(c, np.zeros((8, 8, 8), np.float32))
    assert ei.value.code in (-2, -3)


@pytest.mark.parametrize("preset", [None, "4"])
def test_package_sets_work_queue_default(preset):
    """Importing the package defaults CUDA_DEVICE_MAX_CONNECTIONS to 32 (the
    tuner's concurrent trial streams) and keeps a value the caller set."""
    import subprocess
    import sys
    env = {k: v for k, v in os.environ.items() if k != "CUDA_DEVICE_MAX_CONNECTIONS"}
    if preset is not None:
        env["CUDA_DEVICE_MAX_CONNECTIONS"] = preset
    out = subprocess.run([sys.executable, "-c", "import os, faz_gb300; print(os.environ['CUDA_DEVICE_MAX_CONNECTIONS'])"],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == (preset or "32")
