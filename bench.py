#!/usr/bin/env python
"""FAZ interpolation compress/decompress benchmark on GB300.

Workload: one 512x512x512 float32 spectral field (k^-3.5, anisotropic
correlation lengths 1:2:4, 1% noise, seeded, synthetic), relative error bound
1e-3, cubic interpolation (ALGO_INTERP).  A step is one compression of the
field; decompression is timed the same way and reported beside it.

  value       compress GB/s (input bytes / time) with the field resident in
              HBM, through the GPU path up to the pre-zstd payload in host
              memory (CUDA events on the call's stream).
  e2e         compress GB/s through faz_compress, the C ABI (host input in pinned
              memory, host->device copy, GPU path, payload copy back, host
              zstd, trailer), host clock.
  roofline    the finest interpolation level kernel (the dominant kernel):
              algorithmic bytes per launch / CUDA-event duration vs the
              measured HBM copy bandwidth.
  cpu_baseline  the CPU oracle (a restatement of the reference) on a slab
              of the same field, one thread.

--impl reference times the CPU restatement of the reference on all host
cores (one slab per worker process) on the same metric.
Under torchrun every rank compresses its own field (independent replicas,
weak scaling); rank 0 prints the line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

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
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-vs-sampled autotune comparison")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched uneven-fields measurement")
    ap.add_argument("--no-combined", action="store_true", help="skip the combined f64 learned + batched workload")
    ap.add_argument("--combined-fields", type=int, default=8,
                    help="float64 256x384x384 fields per bound in the combined workload")
    ap.add_argument("--batch-fields", type=int, default=32,
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


# DRAM traffic of one finest-level compress launch, measured with ncu
# (dram__bytes_read.sum + dram__bytes_write.sum = 342.43 MB + 100.42 MB) on a
# 256x512x512 float32 field, cubic, rel eb 1e-3; traffic grows with the number
# of values, so it is scaled to the benchmarked field by its value count.
FINEST_TRAFFIC_BYTES = 442849280
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


# ------------------------------------------------------------- CPU oracle
def _cpu_slab_job(args):
    path, shape, offset, eb, interp, algo, reps = args
    import numpy as np
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    import faz_gb300.config as C
    x = np.fromfile(path, dtype=np.float32, count=int(np.prod(shape)), offset=offset).reshape(shape)
    conf = C.Config(*shape)
    if algo == "interp":
        conf.cmprAlgo = C.ALGO_INTERP
        conf.interpAlgo = C.INTERP_ALGO_CUBIC if interp == "cubic" else C.INTERP_ALGO_LINEAR
    conf.errorBoundMode = C.EB_REL
    conf.relErrorBound = eb
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


def reference_arm(args, dims):
    """CPU restatement of the reference on all host cores: one slab per worker."""
    import multiprocessing as mp
    import numpy as np
    from faz_gb300.fields import spectral_field
    cores = os.cpu_count() or 1
    slab = max(8, min(64, dims[0] // max(1, cores)))
    nslab = min(cores, dims[0] // slab)
    sdims = (slab * nslab,) + tuple(dims[1:])
    x = spectral_field(sdims, slope=-3.5, aniso=(1, 2, 4), noise=0.01, seed=2024)
    with tempfile.NamedTemporaryFile(suffix=".f32", delete=False, dir="/dev/shm" if os.path.isdir("/dev/shm") else None) as f:
        x.tofile(f)
        path = f.name
    plane = int(np.prod(dims[1:])) * 4
    jobs = [(path, (slab,) + tuple(dims[1:]), i * slab * plane, args.eb, args.interp, args.algo, 1)
            for i in range(nslab)]
    ctx = mp.get_context("spawn")
    times_c, times_d, sizes = [], [], []
    try:
        with ctx.Pool(nslab) as pool:
            for step in range(args.warmup + args.steps):
                t0 = time.perf_counter()
                res = pool.map(_cpu_slab_job, jobs)
                wall = time.perf_counter() - t0
                if step >= args.warmup:
                    # workers run compress then decompress; split the wall time by their ratio
                    tc = sum(r[0] for r in res)
                    td = sum(r[1] for r in res)
                    times_c.append(wall * tc / (tc + td))
                    times_d.append(wall * td / (tc + td))
                    sizes.append(sum(r[2] for r in res))
    finally:
        os.unlink(path)
    nbytes = x.nbytes
    tc = statistics.median(times_c)
    td = statistics.median(times_d)
    v = nbytes / tc / 1e9
    sample = f"{nslab} slabs of {slab}x{dims[1]}x{dims[2]} float32 ({nbytes / 1e6:.0f} MB) per step, one per process"
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "GB/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(tc * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded spectral field k^-3.5, aniso 1:2:4, 1% noise",
            "config": {"workload": workload_name(dims, args), "eb_mode": "REL", "eb": args.eb},
            "cpu_baseline": {"value": round(v, 4), "unit": "GB/s", "cores": nslab, "kind": "port", "sample": sample},
            "e2e": {"value": round(v, 4), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "decompress": {"value": round(nbytes / td / 1e9, 4), "unit": "GB/s", "ms_per_step": round(td * 1e3, 3)},
            "ratio": round(nbytes / statistics.median(sizes), 3)}
    return line


def workload_name(dims, args):
    what = ("default configuration: SZ3 sampled autotune (Lorenzo vs interpolation trials) then the chosen "
            "compressor" if args.algo == "auto" else f"ALGO_INTERP {args.interp}")
    return f"{dims[0]}x{dims[1]}x{dims[2]} float32 spectral field, rel eb {args.eb:g}, {what}"


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
    t_batch, sb = timed(lambda: F.compress_batch(confs, xs))
    tmb = F.last_timings()
    t_one, so = timed(lambda: [F.compress_device(c, x) for c, x in zip(confs, xs)])
    assert sb == so, "batched streams differ from single-field streams"
    return {"fields": nfields, "shapes": [list(d) for d in BATCH_SHAPES], "bytes": nbytes,
            "batched": {"value": round(nbytes / t_batch / 1e9, 3), "unit": "GB/s", "ms": round(t_batch * 1e3, 2),
                        "levels_ms": round(tmb["predict_ms"], 2)},
            "one_call_per_field": {"value": round(nbytes / t_one / 1e9, 3), "unit": "GB/s",
                                   "ms": round(t_one * 1e3, 2)},
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


def learned_vs_sampled(x, dims, eb):
    """The learned tuner against the sampled QoZ autotune, end to end through
    compress_device (tuning + compression + zstd, host clock): on this field
    and on held-out synthetic fields of the training distribution (128^3 to
    256^3, spectral slope -4..-2, anisotropy up to 8, 0-5 % noise, optional
    flat boxes, relative bounds 1e-4..1e-2; a seed outside the training set)."""
    import faz_gb300 as F
    import faz_gb300.learned as L
    import torch
    if not os.path.exists(L.DEFAULT_MODEL):
        return None
    model = L.TunerModel.load()
    qc = L.qoz_conf(dims, eb)
    t_plain, s_plain = L._timed(lambda: F.compress_device(qc, x), 2)

    def learned():
        tuned, info = L.learned_tune(qc, x, model)
        return F.compress_device(tuned, x), info
    t_learn, (s_learn, info) = L._timed(learned, 3)
    nbytes = x.numel() * x.element_size()
    # the network alone: features + tensor-core MLP on this field
    f = L.features(qc, x)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(10):
        model.infer(L.features(qc, x))
    torch.cuda.synchronize()
    t_net = (time.perf_counter() - t0) / 10
    _, held = L.evaluate(model, 6, seed=999, reps=2)
    return {"this_field": {"sampled_ms": round(t_plain * 1e3, 2), "learned_ms": round(t_learn * 1e3, 2),
                           "speedup": round(t_plain / t_learn, 2), "ratio_sampled": round(nbytes / len(s_plain), 4),
                           "ratio_learned": round(nbytes / len(s_learn), 4), "same_stream": s_plain == s_learn,
                           "fallback": info["used_plain"], "network_ms": round(t_net * 1e3, 3)},
            "held_out": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in held.items()},
            "sampled": "QoZ tuner (QoZ = 1: per-level interpolator/direction + alpha/beta search by trial compressions)",
            "learned": "MLP 64->256->256->27 on block statistics, BF16 tcgen05 inference, plain tuner as fallback"}


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
    from faz_gb300.fields import spectral_field
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
    x = spectral_field(dims, slope=-3.5, aniso=(1, 2, 4), noise=0.01, seed=1000 + rank, device="cuda")
    nbytes = x.numel() * x.element_size()
    stream = torch.cuda.Stream()
    out = torch.empty_like(x)
    pay_buf = torch.empty(nbytes + (4 << 20), dtype=torch.uint8, pin_memory=True)

    # ---- device-resident compress (value) and decompress
    launches = 0
    for _ in range(args.warmup):
        payload, conf_out = F.compress_payload_device(conf, x, stream, out=pay_buf)
    interp_chosen = conf_out.cmprAlgo == F.ALGO_INTERP
    full_stream = None if interp_chosen else F.compress_device(conf, x, stream)

    def decompress_once():
        if interp_chosen:
            F.decompress_payload_device(len(dims), payload, out, stream)
        else:
            F.decompress_device(full_stream, out, stream)

    for _ in range(args.warmup):
        decompress_once()
    barrier()
    t_steps, phases = [], []
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        barrier()
        ev0.record(stream)
        for _ in range(args.steps):
            payload, conf_out = F.compress_payload_device(conf, x, stream, out=pay_buf)
            tm = F.last_timings()
            launches += tm["kernel_launches"]
            phases.append(tm)
        ev1.record(stream)
        barrier()
        t_comp = ev0.elapsed_time(ev1) / 1e3 / args.steps
        dphases = []
        ev0.record(stream)
        for _ in range(args.steps):
            decompress_once()
            tm = F.last_timings()
            launches += tm["kernel_launches"]
            dphases.append(tm)
        ev1.record(stream)
        barrier()
        t_dec = ev0.elapsed_time(ev1) / 1e3 / args.steps
        # the plain interpolation compressor alone (ALGO_INTERP cubic), for reference
        t_plain = None
        if args.algo == "auto":
            pconf = make_conf(F, dims, args.eb, "cubic", "interp")
            for _ in range(2):
                F.compress_payload_device(pconf, x, stream, out=pay_buf)
            barrier()
            ev0.record(stream)
            for _ in range(args.steps):
                F.compress_payload_device(pconf, x, stream, out=pay_buf)
                launches += F.last_timings()["kernel_launches"]
            ev1.record(stream)
            barrier()
            t_plain = ev0.elapsed_time(ev1) / 1e3 / args.steps
    clocks = clk.summary()
    err = (out.double() - x.double()).abs().max().item()
    assert err <= conf_out.absErrorBound, (err, conf_out.absErrorBound)

    # ---- end to end through the C ABI with host buffers (faz_compress /
    # faz_decompress: the calls a binding of the reference's SZ_compress /
    # SZ_decompress makes), host clock
    import ctypes
    L = F.library()
    host_in = torch.empty(dims, dtype=torch.float32, pin_memory=True)
    host_in.copy_(x.cpu())
    host_np = host_in.numpy()
    host_out = torch.empty(dims, dtype=torch.float32, pin_memory=True).numpy().reshape(-1)
    cs = conf.to_struct()
    tmc = F.FazTimings()

    def c_compress():
        out, osz = ctypes.c_void_p(), ctypes.c_size_t()
        F.api._check(L.faz_compress(ctypes.byref(cs), F.FAZ_FLOAT, host_np.ctypes.data, ctypes.byref(out),
                                    ctypes.byref(osz), ctypes.byref(tmc)))
        return out, osz.value

    def c_decompress(buf, size):
        ds = F.FazConfigStruct()
        ds.num = host_out.size
        ptr = ctypes.c_void_p(host_out.ctypes.data)
        F.api._check(L.faz_decompress(ctypes.byref(ds), F.FAZ_FLOAT, buf, size, ctypes.byref(ptr),
                                      ctypes.byref(tmc)))

    for _ in range(max(1, args.warmup // 2)):
        o, n_o = c_compress()
        c_decompress(o, n_o)
        L.faz_free(o)
    barrier()
    e2e_c, e2e_d, zc, zd, d2h_bytes = [], [], [], [], 0
    e2e_parts = []
    stream_len = 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o, n_o = c_compress()
        e2e_c.append(time.perf_counter() - t0)
        zc.append(tmc.zstd_ms)
        e2e_parts.append({"h2d_ms": tmc.h2d_ms, "gpu_ms": tmc.gpu_ms, "zstd_ms": tmc.zstd_ms,
                          "call_ms": tmc.total_ms})
        d2h_bytes = tmc.payload_bytes
        stream_len = n_o
        t0 = time.perf_counter()
        c_decompress(o, n_o)
        e2e_d.append(time.perf_counter() - t0)
        zd.append(tmc.zstd_ms)
        L.faz_free(o)
    ratio = nbytes / stream_len
    dec = host_out.reshape(dims)
    assert np.abs(dec.astype(np.float64) - host_np.astype(np.float64)).max() <= conf_out.absErrorBound

    # ---- max over ranks
    vals = torch.tensor([t_comp, t_dec, statistics.median(e2e_c), statistics.median(e2e_d)], device="cuda",
                        dtype=torch.float64)
    if dist is not None:
        dist.all_reduce(vals, op=dist.ReduceOp.MAX)
    t_comp, t_dec, te2e_c, te2e_d = vals.tolist()
    if rank != 0:
        dist.destroy_process_group()
        return

    peak, peak_kind = peaks()
    nvals = dims[0] * dims[1] * dims[2]
    cubic = conf_out.interpAlgo == F.INTERP_ALGO_CUBIC
    roof = None
    if interp_chosen:
        fin = statistics.median(p["finest_level_ms"] for p in phases) / 1e3
        fin_bytes = finest_level_bytes(dims, 4)
        achieved = fin_bytes / fin / 1e9
        traffic = None
        if cubic and args.eb == 1e-3:
            traffic = int(round(FINEST_TRAFFIC_BYTES * nvals / FINEST_TRAFFIC_VALUES))
        roof = {"kernel": "k_interp_level<float,compress> finest level (%s)" % ("cubic" if cubic else "linear"),
                "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind, "bytes_per_launch": fin_bytes,
                "traffic": traffic}
    cpu = None
    if not args.no_cpu_baseline:
        slab = 64
        cc, cd, shape = cpu_oracle_single(x[:slab].cpu().numpy(), slab, args.eb, args.interp, args.algo)
        cpu = {"value": round(cc, 4), "unit": "GB/s", "cores": 1, "kind": "port",
               "sample": f"compress of a {shape[0]}x{shape[1]}x{shape[2]} slab of the same field, one thread "
                         f"(decompress {cd:.4f} GB/s)"}
    learned = None if args.no_learned else learned_vs_sampled(x, dims, args.eb)
    batch = None if args.no_batch else batched_fields(args.batch_fields, args.eb)
    combined = None if args.no_combined else combined_f64(args.combined_fields)
    med = lambda k, ph: round(statistics.median(p[k] for p in ph), 4)  # noqa: E731
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
        "data": "synthetic: seeded spectral field k^-3.5, aniso 1:2:4, 1% noise, scaled to [-50,80]",
        "config": {"workload": workload_name(dims, args) + " (one field per GPU)",
                   "eb_mode": "REL", "eb": args.eb, "abs_eb": conf_out.absErrorBound,
                   "chosen": {"cmprAlgo": ["ALGO_LORENZO_REG", "ALGO_INTERP_LORENZO", "ALGO_INTERP"][conf_out.cmprAlgo],
                              "interpAlgo": "cubic" if cubic else "linear",
                              "interpDirection": conf_out.interpDirection},
                   "l2": "inputs larger than L2 (field %.0f MB vs 129 MB L2)" % (nbytes / 1e6),
                   "parallelism": f"replicas x{world}"},
        "ratio": round(ratio, 3),
        "decompress": {"value": round(world * nbytes / t_dec / 1e9, 3), "unit": "GB/s",
                       "ms_per_step": round(t_dec * 1e3, 3),
                       "e2e": round(world * nbytes / te2e_d / 1e9, 3)},
        "e2e": {"value": round(world * nbytes / te2e_c / 1e9, 3), "unit": "GB/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": int(d2h_bytes), "ms_per_step": round(te2e_c * 1e3, 3),
                "zstd_ms_compress": round(statistics.median(zc), 3),
                "zstd_ms_decompress": round(statistics.median(zd), 3),
                "api": "faz_compress / faz_decompress (C ABI, host buffers in pinned memory)",
                "compress_parts_ms": {k: round(statistics.median(p[k] for p in e2e_parts), 3)
                                      for k in ("h2d_ms", "gpu_ms", "zstd_ms", "call_ms")}},
        "roofline": roof,
        "phases_ms": {"compress": {k: med(k, phases) for k in ("tune_ms", "predict_ms", "finest_level_ms",
                                                               "huffman_ms", "host_ms", "gpu_ms")},
                      "decompress": {k: med(k, dphases) for k in ("huffman_ms", "predict_ms", "finest_level_ms",
                                                                  "gpu_ms")}},
        "plain_interp_cubic": None if t_plain is None else {
            "value": round(world * nbytes / t_plain / 1e9, 3), "unit": "GB/s", "ms_per_step": round(t_plain * 1e3, 3)},
        "gpu_launches": launches,
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
