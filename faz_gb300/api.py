"""ctypes binding of libfaz_gb300.so and the Python host API."""
import ctypes
import os
import threading

import numpy as np

from .config import Config, FazConfigStruct, FazTimings, FAZ_FLOAT, FAZ_DOUBLE

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libfaz_gb300.so")
_lib = None
_lock = threading.Lock()
_tls = threading.local()

# include/faz_gb300.h status codes
STATUS = {0: "FAZ_OK", -1: "FAZ_ERR_ARG", -2: "FAZ_ERR_UNSUPPORTED", -3: "FAZ_ERR_CUDA", -4: "FAZ_ERR_FORMAT",
          -5: "FAZ_ERR_ZSTD", -6: "FAZ_ERR_DEVICE"}

EXPORTED = ["faz_config_init", "faz_config_load_ini", "faz_compress", "faz_decompress", "faz_compress_device",
            "faz_decompress_device", "faz_compress_device_payload", "faz_decompress_payload_device",
            "faz_stream_info", "faz_resolve_eb_noalloc", "faz_tune_device", "faz_tuner_features",
            "faz_compress_batch", "faz_mlp_forward", "faz_mlp_backward", "faz_mlp_adam", "faz_tuner_model_create",
            "faz_tuner_model_destroy", "faz_tuner_infer", "faz_learned_tune",
            "faz_config_size", "faz_free", "faz_last_error", "faz_zstd_version"]


class FazError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"{STATUS.get(code, code)}: {message}")
        self.code = code


def library():
    """Load libfaz_gb300.so (it must have been built: python -m faz_gb300.build)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(_LIB_PATH):
            raise FazError(-3, f"{_LIB_PATH} is not built; run `python -m faz_gb300.build`")
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER
        vp, sz = ctypes.c_void_p, ctypes.c_size_t
        L.faz_config_init.argtypes = [vp, ctypes.c_int, vp]
        L.faz_config_load_ini.argtypes = [vp, ctypes.c_char_p]
        L.faz_compress.argtypes = [vp, ctypes.c_int, vp, P(vp), P(sz), vp]
        L.faz_compress_device.argtypes = [vp, ctypes.c_int, vp, vp, P(vp), P(sz), vp]
        L.faz_decompress.argtypes = [vp, ctypes.c_int, vp, sz, P(vp), vp]
        L.faz_decompress_device.argtypes = [vp, ctypes.c_int, vp, sz, vp, vp, vp]
        L.faz_free.argtypes = [vp]
        L.faz_last_error.restype = ctypes.c_char_p
        L.faz_zstd_version.restype = ctypes.c_uint
        L.faz_config_size.restype = ctypes.c_size_t
        L.faz_compress_device_payload.argtypes = [vp, ctypes.c_int, vp, vp, vp, sz, P(sz), vp, vp]
        L.faz_stream_info.argtypes = [vp, sz, vp]
        L.faz_resolve_eb_noalloc.argtypes = [vp, ctypes.c_int, vp, vp]
        L.faz_decompress_payload_device.argtypes = [ctypes.c_int, ctypes.c_int, vp, sz, vp, ctypes.c_uint64, vp, vp]
        i32, i64, f32, f64 = ctypes.c_int, ctypes.c_int64, ctypes.c_float, ctypes.c_double
        L.faz_tune_device.argtypes = [vp, i32, vp, vp, vp]
        L.faz_compress_batch.argtypes = [i32, vp, i32, vp, vp, vp, vp, i32, vp]
        L.faz_tuner_features.argtypes = [vp, i32, vp, vp, vp]
        L.faz_mlp_forward.argtypes = [vp, vp, i32, vp, vp, vp, vp]
        L.faz_mlp_backward.argtypes = [vp, vp, vp, i32, vp, vp, vp, vp, vp, vp]
        L.faz_mlp_adam.argtypes = [vp, vp, vp, vp, i64, f32, f32, f32, f32, i32, f32, vp]
        L.faz_tuner_model_create.argtypes = [vp, vp, vp]
        L.faz_tuner_model_create.restype = vp
        L.faz_tuner_model_destroy.argtypes = [vp]
        L.faz_tuner_infer.argtypes = [vp, vp, i32, vp, vp]
        L.faz_learned_tune.argtypes = [vp, i32, vp, vp, vp, f64, vp]
        _lib = L
        return L


def _check(rc):
    if rc != 0:
        raise FazError(rc, library().faz_last_error().decode(errors="replace"))


def _dtype_code(dt):
    dt = np.dtype(dt)
    if dt == np.float32:
        return FAZ_FLOAT
    if dt == np.float64:
        return FAZ_DOUBLE
    raise TypeError("FAZ compresses float32 or float64 data")


def last_timings():
    """faz_timings of the last call on this thread, as a dict."""
    t = getattr(_tls, "timings", None)
    return t.as_dict() if t is not None else None


def zstd_version():
    return library().faz_zstd_version()


def load_ini(conf, path):
    """QoZ::Config::loadcfg: apply an INI file's settings to `conf`."""
    s = conf.to_struct()
    _check(library().faz_config_load_ini(ctypes.byref(s), os.fsencode(path)))
    lists = (conf.interpAlgo_list, conf.interpDirection_list)
    new = Config.from_struct(s)
    new.interpAlgo_list, new.interpDirection_list = lists
    return new


def _take_bytes(ptr, n):
    try:
        return ctypes.string_at(ptr, n)
    finally:
        library().faz_free(ptr)


def _is_torch_cuda(x):
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


def SZ_compress(conf, data):
    """Compress `data` (numpy array in host memory, or CUDA torch tensor) to a
    FAZ stream (bytes).  `conf` is not modified (the reference compresses a copy)."""
    if conf.num != (data.numel() if _is_torch_cuda(data) else np.asarray(data).size):
        raise ValueError("data size does not match conf.dims")
    if _is_torch_cuda(data):
        return compress_device(conf, data)
    arr = np.ascontiguousarray(data)
    s = conf.to_struct()
    out, osz, tm = ctypes.c_void_p(), ctypes.c_size_t(), FazTimings()
    _check(library().faz_compress(ctypes.byref(s), _dtype_code(arr.dtype), arr.ctypes.data, ctypes.byref(out),
                                  ctypes.byref(osz), ctypes.byref(tm)))
    _tls.timings = tm
    return _take_bytes(out, osz.value)


def compress_device(conf, tensor, stream=None):
    """Compress a contiguous CUDA tensor; work is issued on `stream`
    (a torch.cuda.Stream, default the current stream)."""
    import torch
    t = tensor.contiguous()
    dt = {torch.float32: FAZ_FLOAT, torch.float64: FAZ_DOUBLE}.get(t.dtype)
    if dt is None:
        raise TypeError("FAZ compresses float32 or float64 data")
    st = (stream or torch.cuda.current_stream(t.device)).cuda_stream
    s = conf.to_struct()
    out, osz, tm = ctypes.c_void_p(), ctypes.c_size_t(), FazTimings()
    with torch.cuda.device(t.device):
        _check(library().faz_compress_device(ctypes.byref(s), dt, ctypes.c_void_p(t.data_ptr()),
                                             ctypes.c_void_p(st), ctypes.byref(out), ctypes.byref(osz),
                                             ctypes.byref(tm)))
    _tls.timings = tm
    return _take_bytes(out, osz.value)


def compress_batch(confs, tensors, stream=None, threads=0):
    """Compress several CUDA tensors (fields of uneven shapes) in one batched
    call: returns the list of streams, each equal to compress_device's for
    that field.  All tensors share one dtype and device."""
    import torch
    if len(confs) != len(tensors) or not confs:
        raise ValueError("one configuration per field")
    ts = [t.contiguous() for t in tensors]
    dt = {torch.float32: FAZ_FLOAT, torch.float64: FAZ_DOUBLE}.get(ts[0].dtype)
    if dt is None or any(t.dtype != ts[0].dtype for t in ts):
        raise TypeError("fields must all be float32 or all float64")
    for c, t in zip(confs, ts):
        if c.num != t.numel():
            raise ValueError("data size does not match conf.dims")
    n = len(ts)
    arr = (FazConfigStruct * n)(*[c.to_struct() for c in confs])
    ptrs = (ctypes.c_void_p * n)(*[t.data_ptr() for t in ts])
    outs = (ctypes.c_void_p * n)()
    sizes = (ctypes.c_size_t * n)()
    st = (stream or torch.cuda.current_stream(ts[0].device)).cuda_stream
    tm = FazTimings()
    with torch.cuda.device(ts[0].device):
        _check(library().faz_compress_batch(n, arr, dt, ptrs, ctypes.c_void_p(st), outs, sizes, int(threads),
                                            ctypes.byref(tm)))
    _tls.timings = tm
    return [_take_bytes(outs[i], sizes[i]) for i in range(n)]


def tune_device(conf, tensor, stream=None):
    """Run the sampled autotune `conf` selects (QoZ = 1: the QoZ tuner;
    ALGO_INTERP_LORENZO: the SZ3 tuner) on a CUDA tensor without compressing.
    Returns the tuned Config (the decisions, error bound resolved to ABS)."""
    import torch
    t = tensor.contiguous()
    dt = {torch.float32: FAZ_FLOAT, torch.float64: FAZ_DOUBLE}.get(t.dtype)
    if dt is None:
        raise TypeError("FAZ compresses float32 or float64 data")
    st = (stream or torch.cuda.current_stream(t.device)).cuda_stream
    s, tm = conf.to_struct(), FazTimings()
    with torch.cuda.device(t.device):
        _check(library().faz_tune_device(ctypes.byref(s), dt, ctypes.c_void_p(t.data_ptr()), ctypes.c_void_p(st),
                                         ctypes.byref(tm)))
    _tls.timings = tm
    return Config.from_struct(s)


def stream_info(stream_bytes):
    """Config stored in a stream's trailer (dims, error bound, algorithm)."""
    s = FazConfigStruct()
    _check(library().faz_stream_info(bytes(stream_bytes), len(stream_bytes), ctypes.byref(s)))
    return Config.from_struct(s)


def SZ_decompress(conf, stream_bytes, dtype=np.float32, out=None):
    """Decompress a FAZ stream.  Writes into `out` (a contiguous numpy array
    of the stream's size, e.g. in pinned memory) or a new array.  Returns
    (array shaped by the stream's dims, Config loaded from the trailer)."""
    buf = bytes(stream_bytes)
    dtype = np.dtype(dtype)
    info = stream_info(buf)
    if out is None:
        out = np.empty(info.num, dtype=dtype)
    if out.dtype != dtype or not out.flags.c_contiguous or out.size < info.num:
        raise ValueError("output array must be contiguous, of the stream's dtype and size")
    s = FazConfigStruct()
    s.num = out.size
    ptr, tm = ctypes.c_void_p(out.ctypes.data), FazTimings()
    _check(library().faz_decompress(ctypes.byref(s), _dtype_code(dtype), buf, len(buf), ctypes.byref(ptr),
                                    ctypes.byref(tm)))
    _tls.timings = tm
    c = Config.from_struct(s)
    return out[:c.num].reshape(c.dims), c


def decompress_device(stream_bytes, out_tensor, stream=None):
    """Decompress into a preallocated contiguous CUDA tensor; returns the Config."""
    import torch
    dt = {torch.float32: FAZ_FLOAT, torch.float64: FAZ_DOUBLE}.get(out_tensor.dtype)
    if dt is None or not out_tensor.is_contiguous():
        raise TypeError("output must be a contiguous float32/float64 CUDA tensor")
    buf = bytes(stream_bytes)
    s = FazConfigStruct()
    s.num = out_tensor.numel()  # capacity of the output
    tm = FazTimings()
    st = (stream or torch.cuda.current_stream(out_tensor.device)).cuda_stream
    with torch.cuda.device(out_tensor.device):
        _check(library().faz_decompress_device(ctypes.byref(s), dt, buf, len(buf),
                                               ctypes.c_void_p(out_tensor.data_ptr()), ctypes.c_void_p(st),
                                               ctypes.byref(tm)))
    _tls.timings = tm
    c = Config.from_struct(s)
    if c.num != out_tensor.numel():
        raise ValueError("output tensor size differs from the stream's field")
    return c


def compress_payload_device(conf, tensor, stream=None, out=None):
    """GPU path without the host zstd stage, for measurement and custom
    lossless stages.  Writes the pre-zstd payload into `out` (a host uint8
    buffer: numpy array or pinned torch tensor; a pinned buffer of the
    input's size is allocated when None).  Returns (memoryview of the payload,
    Config the trailer would hold)."""
    import torch
    t = tensor.contiguous()
    dt = {torch.float32: FAZ_FLOAT, torch.float64: FAZ_DOUBLE}.get(t.dtype)
    if dt is None:
        raise TypeError("FAZ compresses float32 or float64 data")
    st = (stream or torch.cuda.current_stream(t.device)).cuda_stream
    s = conf.to_struct()
    co = FazConfigStruct()
    osz, tm = ctypes.c_size_t(), FazTimings()
    for _ in range(2):
        if out is None:
            out = torch.empty(t.numel() * t.element_size() + (1 << 20), dtype=torch.uint8, pin_memory=True)
        if isinstance(out, torch.Tensor):
            ptr, cap = out.data_ptr(), out.numel()
            view = out.numpy()
        else:
            ptr, cap = out.ctypes.data, out.nbytes
            view = out
        with torch.cuda.device(t.device):
            rc = library().faz_compress_device_payload(ctypes.byref(s), dt, ctypes.c_void_p(t.data_ptr()),
                                                       ctypes.c_void_p(st), ctypes.c_void_p(ptr), cap,
                                                       ctypes.byref(osz), ctypes.byref(co), ctypes.byref(tm))
        if rc == -1 and osz.value > cap:
            out = torch.empty(osz.value, dtype=torch.uint8, pin_memory=True)
            continue
        _check(rc)
        break
    _tls.timings = tm
    return memoryview(view)[:osz.value], Config.from_struct(co)


def decompress_payload_device(N, payload, out_tensor, stream=None):
    """Decode a pre-zstd payload (bytes-like, ideally a view of pinned memory)
    into a preallocated contiguous CUDA tensor."""
    import torch
    dt = {torch.float32: FAZ_FLOAT, torch.float64: FAZ_DOUBLE}.get(out_tensor.dtype)
    if dt is None or not out_tensor.is_contiguous():
        raise TypeError("output must be a contiguous float32/float64 CUDA tensor")
    st = (stream or torch.cuda.current_stream(out_tensor.device)).cuda_stream
    tm = FazTimings()
    if isinstance(payload, memoryview):
        arr = np.frombuffer(payload, dtype=np.uint8)
        pptr = ctypes.c_void_p(arr.ctypes.data)
    else:
        pptr = bytes(payload)
    with torch.cuda.device(out_tensor.device):
        _check(library().faz_decompress_payload_device(int(N), dt, pptr, len(payload),
                                                       ctypes.c_void_p(out_tensor.data_ptr()), out_tensor.numel(),
                                                       ctypes.c_void_p(st), ctypes.byref(tm)))
    _tls.timings = tm
