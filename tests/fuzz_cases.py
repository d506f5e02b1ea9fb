"""Seeded random cases shared by tests/test_fuzz_reference.py (oracle against
the reference tool, CPU) and tests/test_gpu_fuzz.py (GPU against the oracle).

A case is the manifest-style dict of a golden case (dims, dtype, flags, ini)
plus a function that builds its field."""
import numpy as np

from faz_gb300.fields import spectral_field

N_CASES = 36


def _planes(shape, noise, seed, dtype):
    """Sum of functions of one axis fewer than the field (what the Lorenzo
    predictor reproduces) plus white noise of `noise` x range."""
    rng = np.random.default_rng(seed)
    if len(shape) == 2:
        base = np.cumsum(rng.standard_normal((shape[0], 1)), 0) + np.cumsum(rng.standard_normal((1, shape[1])), 1)
    else:
        base = (rng.standard_normal((shape[0], shape[1], 1)) + rng.standard_normal((1, shape[1], shape[2])) +
                rng.standard_normal((shape[0], 1, shape[2])))
    return (base + noise * rng.standard_normal(shape) * (base.max() - base.min())).astype(dtype)


def _walk(shape, seed, dtype):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(shape)
    for ax in range(len(shape)):
        a = np.cumsum(a, axis=ax)
    return a.astype(dtype)


def fuzz_cases(n=N_CASES, seed=20261203):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        N = 2 if rng.random() < 0.3 else 3
        dims = [int(v) for v in (rng.integers(150, 420, 2) if N == 2 else rng.integers(36, 90, 3))]
        dtype = np.float64 if rng.random() < 0.2 else np.float32
        rel = float(10 ** rng.uniform(-5 if dtype == np.float64 else -4.3, -2))
        kind = rng.choice(["spectral", "spectral", "planes", "walk"])
        fseed = int(rng.integers(0, 2 ** 31 - 1))
        slope = float(rng.uniform(-4, -1.5))
        noise = float(rng.uniform(0, 0.08))
        mode = rng.choice(["sz3", "qoz", "rates", "rates", "interp", "lorenzo"])
        flags = ["-M", "REL", f"{rel:.6g}"]
        ini = None
        if mode == "qoz":
            flags = flags + ["-q"]
        elif mode == "rates":
            atr = float(rng.choice([0.0, 0.005, 0.01]))
            a = {"predictorTuningRate": "0.01", "autoTuningRate": f"{atr:g}",
                 "levelwisePredictionSelection": str(int(rng.choice([0, 3, 4]))),
                 "testLorenzo": str(int(rng.integers(0, 2))), "maxStep": str(int(rng.choice([0, 16, 32]))),
                 "profiling": str(int(rng.integers(0, 2)))}
            sbs = int(rng.choice([0, 16, 32]))
            if N == 2 and atr == 0 and sbs == 0:
                sbs = 32  # keeps the sampled blocks within one interpolation block
            if sbs:
                a["sampleBlockSize"] = str(sbs)
            ini = {"GlobalSettings": {}, "AlgoSettings": a}
        elif mode == "interp":
            a = {"InterpolationAlgo": str(rng.choice(["INTERP_ALGO_CUBIC", "INTERP_ALGO_LINEAR"])),
                 "InterpDirection": str(int(rng.choice([0, 1 if N == 2 else 5])))}
            ini = {"GlobalSettings": {"CmprAlgo": "ALGO_INTERP"}, "AlgoSettings": a}
        elif mode == "lorenzo":
            lo, lo2 = [("YES", "NO"), ("NO", "YES"), ("YES", "YES")][int(rng.integers(0, 3))]
            a = {"Lorenzo": lo, "Lorenzo2ndOrder": lo2, "Regression": "NO"}
            if N == 3 and rng.random() < 0.5:
                a["BlockSize"] = str(int(rng.choice([4, 5, 6])))
            ini = {"GlobalSettings": {"CmprAlgo": "ALGO_LORENZO_REG"}, "AlgoSettings": a}
        case = {"name": f"fuzz_{i}_{mode}", "dims": dims, "dtype": str(np.dtype(dtype)), "flags": flags, "ini": ini}

        def field(kind=kind, dims=tuple(dims), fseed=fseed, slope=slope, noise=noise, dtype=dtype):
            if kind == "planes":
                return _planes(dims, noise * 0.01, fseed, dtype)
            if kind == "walk":
                return _walk(dims, fseed, dtype)
            return spectral_field(dims, slope=slope, noise=noise, seed=fseed, dtype=dtype)

        out.append({"case": case, "field": field})
    return out
