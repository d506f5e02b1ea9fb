"""ctypes front end of the CPU oracle (oracle/faz_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA path.  Used by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg; never by the product.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = [os.path.join(HERE, "faz_oracle.c"), os.path.join(HERE, "oracle_interp.inc"),
       os.path.join(HERE, "oracle_lorenzo.inc"), os.path.join(HERE, "oracle_general.inc"),
       os.path.join(HERE, "oracle_qoz.inc"), os.path.join(HERE, "oracle_metrics.inc"),
       os.path.join(HERE, "..", "include", "faz_gb300.h")]
REF_ZSTD = os.path.join(HERE, "_ref", "libzstd145.so")

_lib = None


def build(force=False):
    """Compile liboracle.so with gcc (no FMA contraction, IEEE semantics)."""
    stale = force or not os.path.exists(LIB) or any(
        os.path.getmtime(s) > os.path.getmtime(LIB) for s in SRC)
    if stale:
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                               "-o", LIB, SRC[0], "-ldl", "-lm"])
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        from faz_gb300.config import FazConfigStruct  # noqa: F401  (layout shared with the C ABI)
        P = ctypes.POINTER
        L.orc_compress.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, P(ctypes.c_void_p),
                                   P(ctypes.c_size_t), P(ctypes.c_void_p), P(ctypes.c_size_t)]
        L.orc_interp_compress.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, P(ctypes.c_void_p),
                                          P(ctypes.c_size_t), P(ctypes.c_void_p), P(ctypes.c_size_t),
                                          P(ctypes.c_void_p), P(ctypes.c_size_t)]
        L.orc_decompress.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, P(ctypes.c_void_p),
                                     ctypes.c_void_p]
        L.orc_read_stream.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, P(ctypes.c_void_p),
                                      P(ctypes.c_size_t)]
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_zstd_version.restype = ctypes.c_uint
        L.orc_set_zstd.argtypes = [ctypes.c_char_p]
        L.orc_free.argtypes = [ctypes.c_void_p]
        L.orc_ska_order.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
        L.orc_sz3_tune.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.orc_config_save.argtypes = [ctypes.c_void_p, P(ctypes.c_void_p), P(ctypes.c_size_t)]
        L.orc_config_load.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, P(ctypes.c_size_t)]
        _lib = L
    return _lib


def set_zstd(path=None):
    """Point the oracle at a zstd library (default: the system libzstd.so.1)."""
    lib().orc_set_zstd(path.encode() if path else None)


def zstd_version():
    return lib().orc_zstd_version()


def _dtype_code(arr):
    if arr.dtype == np.float32:
        return 0
    if arr.dtype == np.float64:
        return 1
    raise TypeError("float32 or float64 only")


def _take(ptr, n):
    if n == 0:
        lib().orc_free(ptr)
        return b""
    out = ctypes.string_at(ptr, n)
    lib().orc_free(ptr)
    return out


def compress(conf, data):
    """Full stream (payload | trailer | int32) and the pre-zstd payload (None
    for an OpenMP stream, whose slab count follows OMP_NUM_THREADS or the
    host's cores, as the reference's OpenMP runtime does)."""
    if conf.openmp:
        n = int(os.environ.get("OMP_NUM_THREADS", "0").split(",")[0] or 0) or os.cpu_count() or 1
        return compress_omp(conf, data, n), None
    return _compress_one(conf, data)


def _compress_one(conf, data):
    """SZ_compress_dispatcher + trailer of one field (openmp not acted on)."""
    data = np.ascontiguousarray(data)
    s = conf.to_struct()
    out, osz, pay, psz = ctypes.c_void_p(), ctypes.c_size_t(), ctypes.c_void_p(), ctypes.c_size_t()
    rc = lib().orc_compress(ctypes.byref(s), _dtype_code(data), data.ctypes.data, ctypes.byref(out),
                            ctypes.byref(osz), ctypes.byref(pay), ctypes.byref(psz))
    if rc:
        raise RuntimeError(f"oracle compress failed ({rc}): {lib().orc_last_error().decode()}")
    return _take(out, osz.value), _take(pay, psz.value)


def interp_codes(conf, data):
    """Quantisation codes (int32, stream order), unpredictable values and payload.

    `conf` must carry an absolute error bound (errorBoundMode ABS)."""
    data = np.ascontiguousarray(data)
    s = conf.to_struct()
    codes, nc = ctypes.c_void_p(), ctypes.c_size_t()
    unp, nu = ctypes.c_void_p(), ctypes.c_size_t()
    pay, psz = ctypes.c_void_p(), ctypes.c_size_t()
    rc = lib().orc_interp_compress(ctypes.byref(s), _dtype_code(data), data.ctypes.data, ctypes.byref(codes),
                                   ctypes.byref(nc), ctypes.byref(unp), ctypes.byref(nu), ctypes.byref(pay),
                                   ctypes.byref(psz))
    if rc:
        raise RuntimeError(f"oracle compress failed ({rc}): {lib().orc_last_error().decode()}")
    c = np.frombuffer(_take(codes, nc.value * 4), dtype=np.int32).copy()
    u = np.frombuffer(_take(unp, nu.value * data.itemsize), dtype=data.dtype).copy()
    return c, u, _take(pay, psz.value)


def decompress(stream, dtype=np.float32):
    from faz_gb300.config import Config, FazConfigStruct
    import struct
    dtype = np.dtype(dtype)
    stream = bytes(stream)
    (cs,) = struct.unpack_from("<i", stream, len(stream) - 4)
    if 0 < cs <= len(stream) - 4 and _config_of(stream[len(stream) - 4 - cs:len(stream) - 4])[0].openmp:
        return decompress_omp(stream, dtype)
    return _decompress_one(stream, dtype)


def _decompress_one(stream, dtype):
    from faz_gb300.config import Config, FazConfigStruct
    buf = ctypes.create_string_buffer(bytes(stream), len(stream))
    out = ctypes.c_void_p()
    cs = FazConfigStruct()
    rc = lib().orc_decompress(buf, len(stream), 0 if dtype == np.float32 else 1, ctypes.byref(out),
                              ctypes.byref(cs))
    if rc:
        raise RuntimeError(f"oracle decompress failed ({rc}): {lib().orc_last_error().decode()}")
    num = int(cs.num)
    arr = np.frombuffer(_take(out, num * dtype.itemsize), dtype=dtype).copy()
    conf = Config.from_struct(cs)
    return arr.reshape(conf.dims), conf


def sz3_tune(conf, data):
    """The SZ3 tuner's decisions for `data` (a Config with cmprAlgo,
    interpAlgo, interpDirection, quantbinCnt and the Lorenzo settings)."""
    from faz_gb300.config import Config
    data = np.ascontiguousarray(data)
    s = conf.to_struct()
    rc = lib().orc_sz3_tune(ctypes.byref(s), _dtype_code(data), data.ctypes.data)
    if rc:
        raise RuntimeError(f"oracle tuner failed ({rc}): {lib().orc_last_error().decode()}")
    return Config.from_struct(s)


def read_stream(stream):
    """(Config, pre-zstd payload) of a stream."""
    from faz_gb300.config import Config, FazConfigStruct
    buf = ctypes.create_string_buffer(bytes(stream), len(stream))
    cs = FazConfigStruct()
    pay, psz = ctypes.c_void_p(), ctypes.c_size_t()
    rc = lib().orc_read_stream(buf, len(stream), ctypes.byref(cs), ctypes.byref(pay), ctypes.byref(psz))
    if rc:
        raise RuntimeError(f"oracle read_stream failed ({rc}): {lib().orc_last_error().decode()}")
    return Config.from_struct(cs), _take(pay, psz.value)


def ska_order(keys):
    keys = np.ascontiguousarray(keys, dtype=np.int32)
    order = np.zeros(len(keys), dtype=np.int32)
    lib().orc_ska_order(keys.ctypes.data, len(keys), order.ctypes.data)
    return order


def trailer_firstsize_span(N):
    """Byte range of Config::firstSize inside the trailer (never initialised
    by the reference on this path)."""
    return 102 + 8 * N, 110 + 8 * N


# ------------------------------------------------------------ OpenMP streams
# SZ_compress_OMP / SZ_decompress_OMP (include/QoZ/api/impl/SZImplOMP.hpp:10-149):
# the field split into nThreads slabs along its slowest axis, rows
# [t*d0//n, (t+1)*d0//n), each compressed by the dispatcher as a field of its
# own with the whole field's absolute error bound; the stream is int32
# nThreads, the slabs' Configs, their sizes (uint64 each), their compressed
# bytes, then the field's Config and its int32 size.

def _omp_rows(d0, t, n):
    return t * d0 // n, (t + 1) * d0 // n


def compress_omp(conf, data, nthreads):
    """OpenMP stream of `data` with nthreads slabs (at most dims[0])."""
    import struct
    from faz_gb300.config import EB_ABS, EB_REL
    data = np.ascontiguousarray(data)
    c = conf.copy()
    if c.errorBoundMode not in (EB_ABS, EB_REL):
        raise RuntimeError("OpenMP streams take the ABS or REL error bound mode")
    n = min(int(nthreads), c.dims[0])
    if c.errorBoundMode == EB_REL:
        # calAbsErrorBound with the range of the slabs' minima and maxima (in T)
        rng = float(data.max() - data.min())
        c.errorBoundMode = EB_ABS
        c.rng = rng
        c.absErrorBound = c.relErrorBound * rng
    confs, parts = [], []
    for t in range(n):
        lo, hi = _omp_rows(c.dims[0], t, n)
        ct = c.copy()
        ct.setDims([hi - lo] + c.dims[1:])
        s, _ = _compress_one(ct, data[lo:hi])
        (cs,) = struct.unpack_from("<i", s, len(s) - 4)
        body = len(s) - 4 - cs
        parts.append(s[:body])
        confs.append(s[body:body + cs])
    out = struct.pack("<i", n) + b"".join(confs) + b"".join(struct.pack("<Q", len(p)) for p in parts) + b"".join(parts)
    outer = _config_bytes(c)
    return out + outer + struct.pack("<i", len(outer))


def _config_bytes(conf):
    """Config::save bytes of conf (the trailer of a stream written with it)."""
    import struct
    s = conf.to_struct()
    out, osz = ctypes.c_void_p(), ctypes.c_size_t()
    rc = lib().orc_config_save(ctypes.byref(s), ctypes.byref(out), ctypes.byref(osz))
    if rc:
        raise RuntimeError(f"oracle config save failed ({rc})")
    return _take(out, osz.value)


def read_omp(stream):
    """(field Config, [(slab Config, slab stream)]) of an OpenMP stream; each
    slab stream is the slab's bytes with its Config appended, as a stream of
    its own."""
    import struct
    from faz_gb300.config import Config, FazConfigStruct
    stream = bytes(stream)
    (cs,) = struct.unpack_from("<i", stream, len(stream) - 4)
    conf, _ = _config_of(stream[len(stream) - 4 - cs:len(stream) - 4])
    body = stream[:len(stream) - 4 - cs]
    (n,) = struct.unpack_from("<i", body, 0)
    pos = 4
    slab_confs = []
    for _ in range(n):
        ct, used = _config_of(body[pos:])
        slab_confs.append((ct, body[pos:pos + used]))
        pos += used
    sizes = struct.unpack_from(f"<{n}Q", body, pos)
    pos += 8 * n
    slabs = []
    for (ct, cb), sz in zip(slab_confs, sizes):
        slabs.append((ct, body[pos:pos + sz] + cb + struct.pack("<i", len(cb))))
        pos += sz
    return conf, slabs


def _config_of(buf):
    from faz_gb300.config import Config, FazConfigStruct
    b = ctypes.create_string_buffer(bytes(buf), len(buf))
    cs = FazConfigStruct()
    used = ctypes.c_size_t()
    rc = lib().orc_config_load(b, len(buf), ctypes.byref(cs), ctypes.byref(used))
    if rc:
        raise RuntimeError("oracle config load failed")
    return Config.from_struct(cs), used.value


def decompress_omp(stream, dtype=np.float32):
    conf, slabs = read_omp(stream)
    parts = [_decompress_one(s, np.dtype(dtype))[0] for _, s in slabs]
    return np.concatenate(parts, axis=0).reshape(conf.dims), conf
