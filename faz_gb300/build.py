"""Build libfaz_gb300.so in-tree for sm_103a (nvcc + g++, no cmake).

Translation units compile in parallel; objects land in faz_gb300/_build/ and
the shared library next to this file.  Run: python -m faz_gb300.build
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfaz_gb300.so")
CLI_SRC = os.path.join(HERE, "cli", "faz.cpp")
CLI = os.path.join(HERE, "faz")  # the command-line tool, linked against LIB

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false keeps every stencil and quantiser operation separately rounded,
# as in the reference's compiled C++; IEEE division/sqrt stay on (defaults).
NVCC_FLAGS = ["-O3", "-std=c++17", "-fmad=false", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-ffp-contract=off", "--expt-relaxed-constexpr"] + ARCH
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def cuda_include():
    return os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _headers_mtime():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "faz_gb300.h"))
    return max(os.path.getmtime(h) for h in hs)


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    cu, cpp = sources()
    hmt = _headers_mtime()
    jobs = []
    objs = []
    for f in cu + cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hmt):
            if f.endswith(".cu"):
                cmd = [nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj]
            else:
                cmd = ["g++"] + CXX_FLAGS + ["-I" + cuda_include(), "-c", src, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout)
        return r.stdout

    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(8, len(jobs) or 1))) as ex:
        for out in ex.map(run, jobs):
            if verbose and out.strip():
                print(out)
    if jobs or not os.path.exists(LIB):
        run([nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB] + objs + ["-ldl", "-lpthread"])
    hpp = os.path.join(ROOT, "include", "faz_gb300.hpp")
    if force or not os.path.exists(CLI) or os.path.getmtime(CLI) < max(
            os.path.getmtime(CLI_SRC), os.path.getmtime(hpp), os.path.getmtime(LIB)):
        run(["g++", "-O2", "-std=c++17", "-Wall", "-o", CLI, CLI_SRC, "-L" + HERE, "-lfaz_gb300",
             "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
