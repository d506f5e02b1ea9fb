"""The exact float emulation of the quantiser's double steps
(faz_gb300/csrc/fastq.cuh), compiled for the CPU and checked against the
double computation on random and adversarial inputs."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_fast_quantiser_matches_double(tmp_path):
    exe = str(tmp_path / "fastq_check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                           os.path.join(ROOT, "tests", "fastq_check.cpp")])
    for seed in (11, 12):
        r = subprocess.run([exe, "3000000", str(seed)], stdout=subprocess.PIPE, text=True)
        assert r.returncode == 0, r.stdout
        assert "bad=0" in r.stdout
