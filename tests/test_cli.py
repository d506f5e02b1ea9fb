"""The `faz` command-line tool (faz_gb300/faz, flags and output of the
reference's test/faz.cpp) and, through it, the C++ API of
include/faz_gb300.hpp.

Without a GPU only argument handling is checked; the GPU tests run the tool
on the golden cases with the reference's own command lines and compare the
streams and decompressed arrays with the reference's.
"""
import hashlib
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, golden_case, golden_dec_sha, golden_manifest, mask_fast_frontend_padding, write_ini

import oracle.oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FAZ = os.path.join(ROOT, "faz_gb300", "faz")


@pytest.fixture(scope="module", autouse=True)
def built():
    from faz_gb300 import build as B
    B.build()
    assert os.path.exists(FAZ)


def run(args, cwd=None):
    return subprocess.run([FAZ] + [str(a) for a in args], capture_output=True, text=True, cwd=cwd, timeout=300)


def test_cli_version_and_usage():
    r = run(["-v"])
    assert r.returncode == 0 and "version: 0.1.0.0" in r.stdout
    r = run(["-h"])
    assert "Usage: faz <options>" in r.stdout
    r = run([])
    assert "Usage: faz <options>" in r.stdout


def test_cli_argument_errors(tmp_path):
    r = run(["-f", "-3", "4", "4", "4", "-M", "REL", "1e-3"])
    assert "specify either a raw binary data file or a compressed data file" in r.stdout
    x = np.zeros(64, dtype=np.float32)
    p = tmp_path / "x.dat"
    x.tofile(p)
    r = run(["-f", "-i", p, "-z", tmp_path / "x.faz", "-3", "4", "4", "4", "-M", "WRONG", "1e-3"])
    assert "wrong error bound mode" in r.stdout
    r = run(["-f", "-i", p, "-z", tmp_path / "x.faz", "-3", "4", "4", "4", "-M", "REL", "1e-3", "-T", "XYZ"])
    assert "wrong tuning target" in r.stdout


def _cli_case_args(case, td):
    """The reference's own command line for a golden case (make_golden.py)."""
    dims = case["dims"]
    args = ["-f" if case["dtype"] == "float32" else "-d", "-F", "0", "-i", os.path.join(GOLDEN, case["name"] + ".in"),
            "-z", os.path.join(td, "out.faz"), f"-{len(dims)}"] + [str(d) for d in reversed(dims)] + case["flags"]
    if case["ini"] is not None:
        ip = os.path.join(td, "cfg.ini")
        write_ini(ip, case["ini"])
        args += ["-c", ip]
    return args


def _gpu_cases():
    out = []
    for c in golden_manifest():
        rc = O.read_stream(open(os.path.join(GOLDEN, c["name"] + ".faz"), "rb").read())[0]
        if rc.cmprAlgo == 0 and rc.quantbinCnt > 65536:
            continue
        if c["ini"] is None and len(c["dims"]) != 3:
            continue
        out.append(c["name"])
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("name", _gpu_cases())
def test_cli_reproduces_reference_runs(name, tmp_path):
    case = golden_case(name)
    r = run(_cli_case_args(case, str(tmp_path)))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "compression ratio = " in r.stdout and "compressed data file = " in r.stdout
    ours = open(tmp_path / "out.faz", "rb").read()
    ref = open(os.path.join(GOLDEN, name + ".faz"), "rb").read()
    c1, p1 = O.read_stream(ours)
    c2, p2 = O.read_stream(ref)
    assert c1.cmprAlgo == c2.cmprAlgo
    itemsize = 4 if case["dtype"] == "float32" else 8
    if c1.cmprAlgo == 0:
        assert mask_fast_frontend_padding(p1, itemsize) == mask_fast_frontend_padding(p2, itemsize)
    else:
        assert p1 == p2
    # decompress the reference's stream with the tool, with the analysis report
    dims = case["dims"]
    dt = "-f" if case["dtype"] == "float32" else "-d"
    # (SZ2-style -s / -x: with -i and -z the tool would compress again)
    r = run([dt, "-s", os.path.join(GOLDEN, name + ".faz"), "-x", tmp_path / "out.dec", "-i",
             os.path.join(GOLDEN, name + ".in"), f"-{len(dims)}"] + [str(d) for d in reversed(dims)] + ["-a"])
    assert r.returncode == 0, r.stdout + r.stderr
    for key in ("Max absolute error = ", "PSNR = ", "decompression time = ", "decompressed file = "):
        assert key in r.stdout
    assert hashlib.sha256(open(tmp_path / "out.dec", "rb").read()).hexdigest() == golden_dec_sha(case)


@pytest.mark.gpu
def test_cli_round_trip_text_output_and_temp_stream(tmp_path):
    x = np.linspace(-3, 5, 20 * 30 * 40, dtype=np.float32).reshape(20, 30, 40)
    p = tmp_path / "x.dat"
    x.tofile(p)
    # -i with -o and no -z: compress to a temporary stream, decompress, remove it
    r = run(["-f", "-F", "0", "-i", p, "-o", tmp_path / "x.txt", "-t", "-3", 40, 30, 20, "-M", "ABS", "1e-2"])
    assert r.returncode == 0, r.stdout + r.stderr
    assert not os.path.exists(str(p) + ".faz.tmp")
    vals = np.loadtxt(tmp_path / "x.txt", dtype=np.float64)
    assert vals.size == x.size and np.abs(vals - x.reshape(-1)).max() <= 1e-2 * (1 + 1e-5)


@pytest.mark.gpu
def test_cli_reports_unimplemented_features(tmp_path):
    x = np.linspace(0, 1, 16 ** 3, dtype=np.float32)
    p = tmp_path / "x.dat"
    x.tofile(p)
    # -F 1 (the default) asks for the FAZ wavelet features
    r = run(["-f", "-i", p, "-z", tmp_path / "x.faz", "-3", 16, 16, 16, "-M", "REL", "1e-3"])
    assert r.returncode != 0 and "FZ = 0" in r.stderr
