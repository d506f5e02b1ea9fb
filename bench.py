#!/usr/bin/env python
"""FAZ interpolation compress/decompress benchmark on GB300.

Workload: one 512x512x512 float32 spectral field (k^-3.5, anisotropic
correlation lengths 1:2:4, 1% noise, scaled to [-50, 80], seeded, synthetic;
numpy's generator, so that both arms and the parity tests see the same
values), relative error bound 1e-3, the default configuration (the SZ3 sampled
autotune, then the compressor it chooses).  A step is one compression of the
field; decompression is timed the same way and reported beside it.

  value       compress GB/s (input bytes / time) with the field resident in
              HBM, through the GPU path up to the pre-zstd payload in host
              memory (CUDA events on the call's stream).
  e2e         compress GB/s through faz_compress, the C ABI (host input in pinned
              memory, host->device copy, GPU path, payload copy back, host
              zstd, trailer), host clock.  The body is one level-3 zstd frame
              (the reference's format), written by zstd's worker threads;
              e2e_zstd_single_thread writes it with ZSTD_compress on one
              thread (the reference's call, byte for byte), e2e_multiframe as
              independent frames (a format extension).
  roofline    the finest interpolation level kernel (the dominant kernel):
              algorithmic bytes per launch / CUDA-event duration vs the
              measured HBM copy bandwidth.
  compress_frac / decompress_frac
              (input bytes + payload bytes) / time / measured HBM bandwidth
              for the whole device-resident compression / decompression.
  eb_sweep    value, decompression, ratio and the tuner's choice at relative
              bounds 1e-2 .. 1e-5.
  cpu_baseline  the CPU oracle (a restatement of the reference) on a slab
              of the same field, one thread.

--impl reference times the CPU restatement of the reference on all host
cores: every worker process compresses and decompresses the whole field (the
same stream as the GPU arm's), independent replicas of the workload.
Under torchrun every rank compresses its own field (independent replicas,
weak scaling); rank 0 prints the line.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

# 32 hardware work queues for the autotune's concurrent trial streams (read
# when the CUDA context is created; faz_gb300 sets the same default)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "compress/decompress GB/s + ratio at rel eb 1e-3; learned vs sampled autotune"
L2_BYTES = 129e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--dims", default="512,512,512")
    ap.add_argument("--eb", type=float, default=1e-3)
    ap.add_argument("--interp", default="cubic", choices=["cubic", "linear"])
    ap.add_argument("--algo", default="auto", choices=["auto", "interp"],
                    help="auto: the default configuration (ALGO_INTERP_LORENZO, sampled autotune); "
                         "interp: ALGO_INTERP with --interp")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sweep", action="store_true", help="skip the relative-bound sweep 1e-2 .. 1e-5")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-vs-sampled autotune comparison")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched uneven-fields measurement")
    ap.add_argument("--no-combined", action="store_true", help="skip the combined f64 learned + batched workload")
    ap.add_argument("--combined-fields", type=int, default=64,
                    help="float64 256x384x384 fields per bound in the combined workload")
    ap.add_argument("--batch-fields", type=int, default=256,
                    help="fields in the batched measurement (the shapes cycle through the four batch shapes)")
    return ap.parse_args()


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.idx = gpu_index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        if self.p is None:
            return None
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def make_conf(F, dims, eb, interp, algo="auto"):
    c = F.Config(*dims)
    if algo == "interp":
        c.cmprAlgo = F.ALGO_INTERP
        c.interpAlgo = F.INTERP_ALGO_CUBIC if interp == "cubic" else F.INTERP_ALGO_LINEAR
    c.errorBoundMode = F.EB_REL
    c.relErrorBound = eb
    return c


# DRAM traffic of one finest-level compress launch (the plane kernel
# k_finest), measured with ncu (dram__bytes_read.sum + dram__bytes_write.sum =
# 335.69 MB + 95.54 MB) on a 256x512x512 float32 field, cubic, rel eb 1e-3;
# traffic grows with the number of values, so it is scaled to the benchmarked
# field by its value count.
FINEST_TRAFFIC_BYTES = 431225856
FINEST_TRAFFIC_VALUES = 256 * 512 * 512


def finest_level_bytes(dims, itemsize):
    """Algorithmic bytes of the finest level kernel: each target point read
    once and its 2-byte code written once, each coarse point read once."""
    n = 1
    coarse = 1
    for d in dims:
        n *= d
        coarse *= (d + 1) // 2
    return (n - coarse) * (itemsize + 2) + coarse * itemsize


def bench_field(dims, seed):
    """The benchmark's field (numpy generator, seeded)."""
    from faz_gb300.fields import spectral_field
    return spectral_field(dims, slope=-3.5, aniso=(1, 2, 4), noise=0.01, seed=seed)


def workload_name(dims, args):
    what = ("default configuration: SZ3 sampled autotune (Lorenzo vs interpolation trials) then the chosen "
            "compressor" if args.algo == "auto" else f"ALGO_INTERP {args.interp}")
    return f"{dims[0]}x{dims[1]}x{dims[2]} float32 spectral field, rel eb {args.eb:g}, {what}"


def bench_config(dims, args):
    """The `config` of the JSON line, the same in both arms."""
    nbytes = 4 * dims[0] * dims[1] * dims[2]
    l2 = ("inputs larger than L2" if nbytes > L2_BYTES else "inputs smaller than L2 (not flushed)")
    return {"workload": workload_name(dims, args), "eb_mode": "REL", "eb": args.eb,
            "l2": "%s (field %.0f MB vs 129 MB L2)" % (l2, nbytes / 1e6)}


DATA = "synthetic: seeded spectral field k^-3.5, aniso 1:2:4, 1% noise, scaled to [-50,80]"


# ------------------------------------------------------------- CPU oracle
def _oracle_conf(shape, eb, interp, algo):
    import faz_gb300.config as C
    conf = C.Config(*shape)
    if algo == "interp":
        conf.cmprAlgo = C.ALGO_INTERP
        conf.interpAlgo = C.INTERP_ALGO_CUBIC if interp == "cubic" else C.INTERP_ALGO_LINEAR
    conf.errorBoundMode = C.EB_REL
    conf.relErrorBound = eb
    return conf


def _cpu_slab_job(args):
    path, shape, offset, eb, interp, algo, reps = args
    import numpy as np
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    x = np.fromfile(path, dtype=np.float32, count=int(np.prod(shape)), offset=offset).reshape(shape)
    conf = _oracle_conf(shape, eb, interp, algo)
    tc = td = 0.0
    size = 0
    for _ in range(reps):
        t0 = time.perf_counter()
        s, _ = O.compress(conf, x)
        tc += time.perf_counter() - t0
        t0 = time.perf_counter()
        O.decompress(s)
        td += time.perf_counter() - t0
        size = len(s)
    return tc, td, size, x.nbytes


def cpu_oracle_single(field_np, slab, eb, interp, algo):
    """One thread, one slab of the field."""
    shape = (slab,) + tuple(field_np.shape[1:])
    with tempfile.NamedTemporaryFile(suffix=".f32", delete=False) as f:
        field_np[:slab].tofile(f)
        path = f.name
    try:
        tc, td, size, nb = _cpu_slab_job((path, shape, 0, eb, interp, algo, 1))
    finally:
        os.unlink(path)
    return nb / tc / 1e9, nb / td / 1e9, shape


# Worker state of the reference arm: the field (loaded once per process) and
# the last stream it compressed.
_REF = {}


def _ref_init(path, shape, eb, interp, algo):
    import numpy as np
    sys.path.insert(0, ROOT)
    _REF["x"] = np.fromfile(path, dtype=np.float32).reshape(shape)
    _REF["conf"] = _oracle_conf(shape, eb, interp, algo)


def _ref_compress(_):
    from oracle import oracle as O
    s, _ = O.compress(_REF["conf"], _REF["x"])
    _REF["s"] = s
    return len(s)


def _ref_decompress(_):
    from oracle import oracle as O
    O.decompress(_REF["s"])
    return 0


def reference_arm(args, dims):
    """The CPU restatement of the reference on all host cores: each worker
    process compresses, then decompresses, the whole field per step (the same
    field, configuration and stream as the GPU arm: independent replicas);
    compression and decompression are timed separately across all workers."""
    import multiprocessing as mp
    import numpy as np
    cores = os.cpu_count() or 1
    x = bench_field(dims, 1000)
    with tempfile.NamedTemporaryFile(suffix=".f32", delete=False, dir="/dev/shm" if os.path.isdir("/dev/shm") else None) as f:
        x.tofile(f)
        path = f.name
    nbytes = x.nbytes
    del x
    ctx = mp.get_context("spawn")
    times_c, times_d, sizes = [], [], []
    try:
        with ctx.Pool(cores, initializer=_ref_init, initargs=(path, dims, args.eb, args.interp, args.algo)) as pool:
            for step in range(args.warmup + args.steps):
                t0 = time.perf_counter()
                res = pool.map(_ref_compress, range(cores), chunksize=1)
                tc = time.perf_counter() - t0
                t0 = time.perf_counter()
                pool.map(_ref_decompress, range(cores), chunksize=1)
                td = time.perf_counter() - t0
                if step >= args.warmup:
                    times_c.append(tc)
                    times_d.append(td)
                    sizes.append(res[0])
    finally:
        os.unlink(path)
    tc = statistics.median(times_c)
    td = statistics.median(times_d)
    v = cores * nbytes / tc / 1e9
    sample = (f"{cores} worker processes, each compressing and decompressing the whole {dims[0]}x{dims[1]}x{dims[2]} "
              f"float32 field ({nbytes / 1e6:.0f} MB) per step")
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "GB/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(tc * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": DATA,
            "config": bench_config(dims, args),
            "cpu_baseline": {"value": round(v, 4), "unit": "GB/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": round(v, 4), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "decompress": {"value": round(cores * nbytes / td / 1e9, 4), "unit": "GB/s",
                           "ms_per_step": round(td * 1e3, 3)},
            "ratio": round(nbytes / statistics.median(sizes), 3)}
    return line


# ------------------------------------------------------------------ GPU arm
BATCH_SHAPES = [(1800, 3600), (721, 1440), (100, 500, 500), (26, 1800, 3600)]


def batched_fields(nfields, eb, seed=7):
    """Uneven fields compressed in one batched call against one call per
    field: shapes cycle through 2-D 1800x3600, 2-D 721x1440, 3-D 100x500x500
    and 3-D 26x1800x3600; each a seeded spectral field with slope in [-4, -2],
    every fourth with 5 % sparse spikes; relative bound `eb`, ALGO_INTERP
    (cubic).  Inputs stay in HBM; streams (zstd included) come back to the
    host."""
    import numpy as np
    import torch
    import faz_gb300 as F
    from faz_gb300.fields import spectral_field
    rng = np.random.default_rng(seed)
    # the batched call holds every field's reconstruction, codes and scratch
    # (2.5 times the inputs) at once: cap the fields at what the device holds
    free, _ = torch.cuda.mem_get_info()
    per_cycle = sum(4 * int(np.prod(d)) for d in BATCH_SHAPES) * 3.6 / len(BATCH_SHAPES)
    nfields = max(4, min(nfields, int(0.85 * free / per_cycle)))
    confs, xs = [], []
    for i in range(nfields):
        dims = BATCH_SHAPES[i % len(BATCH_SHAPES)]
        x = spectral_field(dims, slope=float(rng.uniform(-4, -2)), noise=0.01, seed=int(rng.integers(1 << 30)),
                           spikes=0.05 if i % 4 == 3 else 0.0, device="cuda")
        c = F.Config(*dims)
        c.cmprAlgo, c.errorBoundMode, c.relErrorBound = F.ALGO_INTERP, F.EB_REL, eb
        confs.append(c)
        xs.append(x)
    nbytes = sum(x.numel() * x.element_size() for x in xs)

    def timed(fn, reps=2):
        best = None
        out = None
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = fn()
            torch.cuda.synchronize()
            t = time.perf_counter() - t0
            best = t if best is None else min(best, t)
        return best, out

    F.compress_batch(confs[:4], xs[:4])  # warm-up
    # launch autotuner: the persistent launch's CTA size measured on one
    # cycle of the shapes (levels time of the batched call), the fastest kept
    tune = {}
    for th in (512, 256, 128):
        F.compress_batch(confs[:4], xs[:4], threads=th)
        tune[th] = round(F.last_timings()["predict_ms"], 3)
    threads = min(tune, key=tune.get)
    t_batch, sb = timed(lambda: F.compress_batch(confs, xs, threads=threads), reps=1)
    tmb = F.last_timings()
    t_one, so = timed(lambda: [F.compress_device(c, x) for c, x in zip(confs, xs)], reps=1)
    assert sb == so, "batched streams differ from single-field streams"
    return {"fields": nfields, "shapes": [list(d) for d in BATCH_SHAPES], "bytes": nbytes,
            "batched": {"value": round(nbytes / t_batch / 1e9, 3), "unit": "GB/s", "ms": round(t_batch * 1e3, 2),
                        "levels_ms": round(tmb["predict_ms"], 2)},
            "one_call_per_field": {"value": round(nbytes / t_one / 1e9, 3), "unit": "GB/s",
                                   "ms": round(t_one * 1e3, 2)},
            "launch_autotune": {"levels_ms_by_threads": tune, "threads": threads},
            "speedup": round(t_one / t_batch, 3),
            "ratio": round(nbytes / sum(len(s) for s in sb), 3),
            "identical_streams": True}


def combined_f64(nfields, rels=(1e-4, 1e-6), seed=11):
    """float64 256x384x384 fields (spectral k^-3 plus a smooth Gaussian-bump
    background, seeded): configurations from the learned tuner (the plain QoZ
    tuner where it falls back), all fields compressed in one batched call, every
    output checked in FP64 against its field's bound; against the plain path
    (QoZ tuner + compression, one call per field)."""
    import numpy as np
    import torch
    import faz_gb300 as F
    import faz_gb300.learned as L
    from faz_gb300.fields import spectral_field
    if not os.path.exists(L.DEFAULT_MODEL):
        return None
    model = L.TunerModel.load()
    dims = (256, 384, 384)
    rng = np.random.default_rng(seed)
    out = {"fields_per_bound": nfields, "dims": list(dims), "dtype": "f64"}
    for rel in rels:
        xs = [spectral_field(dims, slope=-3.0, noise=0.0, bumps=3, seed=int(rng.integers(1 << 30)),
                             dtype=np.float64, device="cuda") for _ in range(nfields)]
        nbytes = sum(x.numel() * 8 for x in xs)
        qcs = [L.qoz_conf(dims, rel) for _ in xs]
        F.compress_device(qcs[0], xs[0])  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plain = [F.compress_device(c, x) for c, x in zip(qcs, xs)]
        torch.cuda.synchronize()
        t_plain = time.perf_counter() - t0
        t0 = time.perf_counter()
        tuned, fallback = [], 0
        for c, x in zip(qcs, xs):
            tc, info = L.learned_tune(c, x, model, min_confidence=0.5)
            tuned.append(tc)
            fallback += info["used_plain"] != 0
        streams = F.compress_batch(tuned, xs)
        torch.cuda.synchronize()
        t_learn = time.perf_counter() - t0
        worst = 0.0
        for s, x in zip(streams, xs):
            y = torch.empty_like(x)
            c2 = F.decompress_device(s, y)
            err = (y - x).abs().max().item()
            assert err <= c2.absErrorBound, (err, c2.absErrorBound)
            worst = max(worst, err / c2.absErrorBound)
        out[f"rel_{rel:g}"] = {
            "plain_qoz_one_call_per_field": {"ms": round(t_plain * 1e3, 1), "GB_s": round(nbytes / t_plain / 1e9, 3),
                                             "ratio": round(nbytes / sum(len(s) for s in plain), 4)},
            "learned_configs_batched": {"ms": round(t_learn * 1e3, 1), "GB_s": round(nbytes / t_learn / 1e9, 3),
                                        "ratio": round(nbytes / sum(len(s) for s in streams), 4),
                                        "fallback_fields": fallback},
            "speedup": round(t_plain / t_learn, 3),
            "max_err_over_bound": round(worst, 6)}
        del xs
    return out


HELD_OUT_FIELDS = 256  # held-out fields of the training distribution (seed outside the training set)


def learned_vs_sampled(x, dims, eb):
    """The learned tuner against the sampled QoZ autotune, end to end (tuning +
    compression + zstd, host clock): on this field through faz_compress_device
    (the C ABI), and on held-out synthetic fields of the training distribution
    (128^3 to 256^3, spectral slope -4..-2, anisotropy up to 8, 0-5 % noise,
    optional flat boxes, relative bounds 1e-4..1e-2; a seed outside the
    training set) through the Python API."""
    import faz_gb300 as F
    import faz_gb300.learned as L
    import torch
    if not os.path.exists(L.DEFAULT_MODEL):
        return None
    model = L.TunerModel.load()
    qc = L.qoz_conf(dims, eb)

    def c_compress(conf):
        # faz_compress_device through the C ABI; the stream stays in the
        # library's buffer (the Python wrapper would copy its 84 MB into a
        # bytes object, ~10 ms on one host core, in both arms alike)
        s = conf.to_struct()
        out, osz, tm = ctypes.c_void_p(), ctypes.c_size_t(), F.FazTimings()
        lib = F.library()
        rc = lib.faz_compress_device(ctypes.byref(s), F.FAZ_FLOAT, ctypes.c_void_p(x.data_ptr()),
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), ctypes.byref(out),
                                     ctypes.byref(osz), ctypes.byref(tm))
        if rc:
            raise F.FazError(rc, lib.faz_last_error().decode())
        lib.faz_free(out)
        return osz.value

    t_plain, n_plain = L._timed(lambda: c_compress(qc), 2)

    def learned():
        tuned, info = L.learned_tune(qc, x, model)
        return c_compress(tuned), info
    t_learn, (n_learn, info) = L._timed(learned, 3)
    # the streams themselves (untimed)
    s_plain = F.compress_device(qc, x)
    s_learn = F.compress_device(L.learned_tune(qc, x, model)[0], x)
    nbytes = x.numel() * x.element_size()
    # the network alone: features + tensor-core MLP on this field
    f = L.features(qc, x)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(10):
        model.infer(L.features(qc, x))
    torch.cuda.synchronize()
    t_net = (time.perf_counter() - t0) / 10
    _, held = L.evaluate(model, HELD_OUT_FIELDS, seed=999, reps=1)
    return {"this_field": {"sampled_ms": round(t_plain * 1e3, 2), "learned_ms": round(t_learn * 1e3, 2),
                           "speedup": round(t_plain / t_learn, 2), "ratio_sampled": round(nbytes / len(s_plain), 4),
                           "ratio_learned": round(nbytes / len(s_learn), 4), "same_stream": s_plain == s_learn,
                           "fallback": info["used_plain"], "network_ms": round(t_net * 1e3, 3)},
            "held_out": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in held.items()},
            "sampled": "QoZ tuner (QoZ = 1: per-level interpolator/direction + alpha/beta search by trial compressions)",
            "learned": "MLP 64->256->256->27 on block statistics, BF16 tcgen05 inference, plain tuner as fallback"}


def device_compress_timing(F, conf, x, stream, pay_buf, steps, warmup, launches):
    """Device-resident compression of x (CUDA events on `stream`): seconds per
    step, the per-step timings, the last payload and the resolved Config."""
    import torch
    for _ in range(warmup):
        payload, conf_out = F.compress_payload_device(conf, x, stream, out=pay_buf)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    phases = []
    ev0.record(stream)
    for _ in range(steps):
        payload, conf_out = F.compress_payload_device(conf, x, stream, out=pay_buf)
        tm = F.last_timings()
        launches[0] += tm["kernel_launches"]
        phases.append(tm)
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) / 1e3 / steps, phases, payload, conf_out


def device_decompress_timing(F, dims, conf_out, conf, x, payload, out, stream, steps, warmup, launches):
    """Device-resident decompression (pre-zstd payload for interpolation
    streams, the whole stream otherwise): seconds per step and timings."""
    import torch
    interp = conf_out.cmprAlgo == F.ALGO_INTERP
    full = None if interp else F.compress_device(conf, x, stream)

    def once():
        if interp:
            F.decompress_payload_device(len(dims), payload, out, stream)
        else:
            F.decompress_device(full, out, stream)
    for _ in range(warmup):
        once()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    phases = []
    ev0.record(stream)
    for _ in range(steps):
        once()
        tm = F.last_timings()
        launches[0] += tm["kernel_launches"]
        phases.append(tm)
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) / 1e3 / steps, phases


ALGO_NAMES = ["ALGO_LORENZO_REG", "ALGO_INTERP_LORENZO", "ALGO_INTERP", "ALGO_INTERP_BLOCKED"]


def chosen(F, c):
    d = {"cmprAlgo": ALGO_NAMES[c.cmprAlgo]}
    if c.cmprAlgo == F.ALGO_INTERP:
        d["interpAlgo"] = "cubic" if c.interpAlgo == F.INTERP_ALGO_CUBIC else "linear"
        d["interpDirection"] = c.interpDirection
    else:
        d["quantbinCnt"] = c.quantbinCnt
        d["pred_dim"] = c.pred_dim
    return d


def eb_sweep(F, dims, args, x, stream, pay_buf, out, peak, launches, rels=(1e-2, 1e-3, 1e-4, 1e-5)):
    """The same field and configuration at relative bounds 1e-2 .. 1e-5:
    device-resident compression and decompression, ratio of the whole stream,
    the tuner's choice, and the whole-path fractions of the HBM roofline."""
    nbytes = x.numel() * 4
    res = {}
    for rel in rels:
        conf = make_conf(F, dims, rel, args.interp, args.algo)
        tc, _, payload, conf_out = device_compress_timing(F, conf, x, stream, pay_buf, 3, 2, launches)
        td, _ = device_decompress_timing(F, dims, conf_out, conf, x, payload, out, stream, 3, 2, launches)
        P = len(payload)
        ratio = nbytes / len(F.compress_device(conf, x, stream))
        res[f"{rel:g}"] = {"value": round(nbytes / tc / 1e9, 3), "decompress": round(nbytes / td / 1e9, 3),
                           "unit": "GB/s", "ratio": round(ratio, 3), "payload_bytes": P,
                           "compress_frac": round((nbytes + P) / tc / 1e9 / peak, 4),
                           "decompress_frac": round((nbytes + P) / td / 1e9 / peak, 4),
                           "chosen": chosen(F, conf_out)}
    return res


def e2e_run(F, L, conf, dims, host_np, host_out, steps, warmup):
    """faz_compress / faz_decompress (the C ABI with host buffers) timed on
    the host clock: median seconds per compression and decompression, the
    per-call parts, payload bytes and stream length."""
    import ctypes
    cs = conf.to_struct()
    tmc = F.FazTimings()

    def c_compress():
        o, osz = ctypes.c_void_p(), ctypes.c_size_t()
        F.api._check(L.faz_compress(ctypes.byref(cs), F.FAZ_FLOAT, host_np.ctypes.data, ctypes.byref(o),
                                    ctypes.byref(osz), ctypes.byref(tmc)))
        return o, osz.value

    def c_decompress(buf, size):
        ds = F.FazConfigStruct()
        ds.num = host_out.size
        ptr = ctypes.c_void_p(host_out.ctypes.data)
        F.api._check(L.faz_decompress(ctypes.byref(ds), F.FAZ_FLOAT, buf, size, ctypes.byref(ptr),
                                      ctypes.byref(tmc)))
    for _ in range(warmup):
        o, n_o = c_compress()
        c_decompress(o, n_o)
        L.faz_free(o)
    tc, td, zc, zd, parts = [], [], [], [], []
    d2h = n_stream = 0
    for _ in range(steps):
        t0 = time.perf_counter()
        o, n_o = c_compress()
        tc.append(time.perf_counter() - t0)
        zc.append(tmc.zstd_ms)
        parts.append({"h2d_ms": tmc.h2d_ms, "gpu_ms": tmc.gpu_ms, "zstd_ms": tmc.zstd_ms, "call_ms": tmc.total_ms})
        d2h = tmc.payload_bytes
        n_stream = n_o
        t0 = time.perf_counter()
        c_decompress(o, n_o)
        td.append(time.perf_counter() - t0)
        zd.append(tmc.zstd_ms)
        L.faz_free(o)
    med = statistics.median
    return {"tc": med(tc), "td": med(td), "zc": med(zc), "zd": med(zd), "d2h": d2h, "stream": n_stream,
            "parts": {k: round(med(p[k] for p in parts), 3) for k in ("h2d_ms", "gpu_ms", "zstd_ms", "call_ms")}}


class _env:
    """Environment variables set for the duration of a block."""

    def __init__(self, **kv):
        self.kv = kv
        self.old = {}

    def __enter__(self):
        for k, v in self.kv.items():
            self.old[k] = os.environ.get(k)
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v

    def __exit__(self, *a):
        for k, v in self.old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def main():
    args = parse()
    dims = tuple(int(d) for d in args.dims.split(","))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(reference_arm(args, dims)), flush=True)
        return

    import numpy as np
    import torch
    import faz_gb300 as F
    from faz_gb300 import build as B
    B.build()

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    conf = make_conf(F, dims, args.eb, args.interp, args.algo)
    x_np = bench_field(dims, 1000 + rank)
    x = torch.from_numpy(x_np).to("cuda")
    nbytes = x.numel() * x.element_size()
    stream = torch.cuda.Stream()
    out = torch.empty_like(x)
    pay_buf = torch.empty(nbytes + (4 << 20), dtype=torch.uint8, pin_memory=True)
    peak, peak_kind = peaks()
    launches = [0]

    # ---- device-resident compress (value) and decompress
    barrier()
    with Clocks(local) as clk:
        barrier()
        t_comp, phases, payload, conf_out = device_compress_timing(F, conf, x, stream, pay_buf, args.steps,
                                                                   args.warmup, launches)
        barrier()
        t_dec, dphases = device_decompress_timing(F, dims, conf_out, conf, x, payload, out, stream, args.steps,
                                                  args.warmup, launches)
        barrier()
        # the plain interpolation compressor alone (ALGO_INTERP cubic), for reference
        t_plain = None
        if args.algo == "auto":
            pconf = make_conf(F, dims, args.eb, "cubic", "interp")
            t_plain, _, _, _ = device_compress_timing(F, pconf, x, stream, pay_buf, args.steps, 2, launches)
            barrier()
    clocks = clk.summary()
    psize = len(payload)
    err = (out.double() - x.double()).abs().max().item()
    assert err <= conf_out.absErrorBound, (err, conf_out.absErrorBound)

    # ---- end to end through the C ABI with host buffers (faz_compress /
    # faz_decompress: the calls a binding of the reference's SZ_compress /
    # SZ_decompress makes), host clock
    L = F.library()
    host_in = torch.empty(dims, dtype=torch.float32, pin_memory=True)
    host_in.copy_(x.cpu())
    host_np = host_in.numpy()
    host_out = torch.empty(dims, dtype=torch.float32, pin_memory=True).numpy().reshape(-1)
    barrier()
    e2e_w = max(1, args.warmup // 2)
    with _env(FAZ_ZSTD_THREADS=None, FAZ_ZSTD_MULTIFRAME=None):
        e_one = e2e_run(F, L, conf, dims, host_np, host_out, args.steps, e2e_w)
    dec = host_out.reshape(dims)
    assert np.abs(dec.astype(np.float64) - host_np.astype(np.float64)).max() <= conf_out.absErrorBound
    with _env(FAZ_ZSTD_THREADS="0", FAZ_ZSTD_MULTIFRAME=None):
        e_st = e2e_run(F, L, conf, dims, host_np, host_out, max(2, args.steps // 4), 1)
    with _env(FAZ_ZSTD_THREADS=None, FAZ_ZSTD_MULTIFRAME="1"):
        e_mf = e2e_run(F, L, conf, dims, host_np, host_out, max(2, args.steps // 4), 1)
    ratio = nbytes / e_one["stream"]

    # ---- max over ranks
    vals = torch.tensor([t_comp, t_dec, e_one["tc"], e_one["td"]], device="cuda", dtype=torch.float64)
    if dist is not None:
        dist.all_reduce(vals, op=dist.ReduceOp.MAX)
    t_comp, t_dec, te2e_c, te2e_d = vals.tolist()
    if rank != 0:
        dist.destroy_process_group()
        return

    nvals = dims[0] * dims[1] * dims[2]
    interp_chosen = conf_out.cmprAlgo == F.ALGO_INTERP
    cubic = conf_out.interpAlgo == F.INTERP_ALGO_CUBIC
    roof = None
    if interp_chosen:
        fin = statistics.median(p["finest_level_ms"] for p in phases) / 1e3
        fin_bytes = finest_level_bytes(dims, 4)
        achieved = fin_bytes / fin / 1e9
        traffic = None
        if cubic and args.eb == 1e-3:
            traffic = int(round(FINEST_TRAFFIC_BYTES * nvals / FINEST_TRAFFIC_VALUES))
        plane = dims[0] >= 33 and dims[1] >= 33 and dims[2] >= 36 and dims[2] % 4 == 0 and \
            conf_out.interpDirection in (0, 2) and os.environ.get("FAZ_FINEST_PLANES", "1") != "0"
        kname = "k_finest<compress>" if plane else "k_interp_level<float,compress>"
        roof = {"kernel": "%s finest level (%s)" % (kname, "cubic" if cubic else "linear"),
                "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind, "bytes_per_launch": fin_bytes,
                "traffic": traffic}
    cpu = None
    if not args.no_cpu_baseline:
        slab = 64
        cc, cd, shape = cpu_oracle_single(x_np[:slab], slab, args.eb, args.interp, args.algo)
        cpu = {"value": round(cc, 4), "unit": "GB/s", "cores": 1, "kind": "port",
               "sample": f"compress of a {shape[0]}x{shape[1]}x{shape[2]} slab of the same field, one thread "
                         f"(decompress {cd:.4f} GB/s)"}
    sweep = None if args.no_sweep else eb_sweep(F, dims, args, x, stream, pay_buf, out, peak, launches)
    learned = None if args.no_learned else learned_vs_sampled(x, dims, args.eb)
    batch = None if args.no_batch else batched_fields(args.batch_fields, args.eb)
    combined = None if args.no_combined else combined_f64(args.combined_fields)
    med = lambda k, ph: round(statistics.median(p[k] for p in ph), 4)  # noqa: E731

    def e2e_block(e, how):
        return {"value": round(world * nbytes / e["tc"] / 1e9, 3), "unit": "GB/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": int(e["d2h"]), "ms_per_step": round(e["tc"] * 1e3, 3),
                "decompress": round(world * nbytes / e["td"] / 1e9, 3),
                "zstd_ms_compress": round(e["zc"], 3), "zstd_ms_decompress": round(e["zd"], 3),
                "ratio": round(nbytes / e["stream"], 4), "zstd_body": how, "compress_parts_ms": e["parts"]}
    e2e = e2e_block(e_one, "one level-3 zstd frame written by zstd's worker threads (the reference's format)")
    e2e["value"] = round(world * nbytes / te2e_c / 1e9, 3)
    e2e["decompress"] = round(world * nbytes / te2e_d / 1e9, 3)
    e2e["api"] = "faz_compress / faz_decompress (C ABI, host buffers in pinned memory)"
    line = {
        "metric": METRIC,
        "value": round(world * nbytes / t_comp / 1e9, 3),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(t_comp * 1e3, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": DATA,
        "config": bench_config(dims, args),
        "parallelism": f"replicas x{world} (one field per GPU)",
        "abs_eb": conf_out.absErrorBound,
        "chosen": chosen(F, conf_out),
        "ratio": round(ratio, 3),
        "compress_frac": round((nbytes + psize) / t_comp / 1e9 / peak, 4),
        "decompress_frac": round((nbytes + psize) / t_dec / 1e9 / peak, 4),
        "payload_bytes": psize,
        "decompress": {"value": round(world * nbytes / t_dec / 1e9, 3), "unit": "GB/s",
                       "ms_per_step": round(t_dec * 1e3, 3)},
        "e2e": e2e,
        "e2e_zstd_single_thread": e2e_block(e_st, "one level-3 frame by ZSTD_compress on one thread "
                                                  "(the reference's call, byte for byte)"),
        "e2e_multiframe": e2e_block(e_mf, "independent level-3 frames of 4 MiB+ slices (format extension; "
                                          "ZSTD_decompress reads it)"),
        "roofline": roof,
        "phases_ms": {"compress": {k: med(k, phases) for k in ("tune_ms", "predict_ms", "finest_level_ms",
                                                               "huffman_ms", "host_ms", "gpu_ms")},
                      "decompress": {k: med(k, dphases) for k in ("huffman_ms", "predict_ms", "finest_level_ms",
                                                                  "gpu_ms")}},
        "plain_interp_cubic": None if t_plain is None else {
            "value": round(world * nbytes / t_plain / 1e9, 3), "unit": "GB/s", "ms_per_step": round(t_plain * 1e3, 3)},
        "eb_sweep": sweep,
        "gpu_launches": launches[0],
        "clocks": clocks,
        "cpu_baseline": cpu,
        "learned_tuner": learned,
        "batch": batch,
        "combined_f64": combined,
        "max_abs_err": err,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
