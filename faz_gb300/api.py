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
        L.faz_compress_device_payload.argtypes = [vp, ctypes.c_int, vp, vp, P(vp), P(sz), vp, vp]
        L.faz_decompress_payload_device.argtypes = [ctypes.c_int, ctypes.c_int, vp, sz, vp, ctypes.c_uint64, vp, vp]
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


def SZ_decompress(conf, stream_bytes, dtype=np.float32):
    """Decompress a FAZ stream into a new numpy array shaped by the stream's
    dims.  Returns (array, Config loaded from the stream's trailer)."""
    buf = bytes(stream_bytes)
    s = FazConfigStruct()
    out, tm = ctypes.c_void_p(), FazTimings()
    _check(library().faz_decompress(ctypes.byref(s), _dtype_code(dtype), buf, len(buf), ctypes.byref(out),
                                    ctypes.byref(tm)))
    _tls.timings = tm
    c = Config.from_struct(s)
    n = c.num * np.dtype(dtype).itemsize
    arr = np.frombuffer(_take_bytes(out, n), dtype=dtype).copy()
    return arr.reshape(c.dims), c


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


def compress_payload_device(conf, tensor, stream=None):
    """GPU path without the host zstd stage: (pre-zstd payload bytes, Config
    the trailer would hold).  For measurement and custom lossless stages."""
    import torch
    t = tensor.contiguous()
    dt = {torch.float32: FAZ_FLOAT, torch.float64: FAZ_DOUBLE}.get(t.dtype)
    if dt is None:
        raise TypeError("FAZ compresses float32 or float64 data")
    st = (stream or torch.cuda.current_stream(t.device)).cuda_stream
    s = conf.to_struct()
    co = FazConfigStruct()
    out, osz, tm = ctypes.c_void_p(), ctypes.c_size_t(), FazTimings()
    with torch.cuda.device(t.device):
        _check(library().faz_compress_device_payload(ctypes.byref(s), dt, ctypes.c_void_p(t.data_ptr()),
                                                     ctypes.c_void_p(st), ctypes.byref(out), ctypes.byref(osz),
                                                     ctypes.byref(co), ctypes.byref(tm)))
    _tls.timings = tm
    return _take_bytes(out, osz.value), Config.from_struct(co)


def decompress_payload_device(N, payload, out_tensor, stream=None):
    """Decode a pre-zstd payload into a preallocated contiguous CUDA tensor."""
    import torch
    dt = {torch.float32: FAZ_FLOAT, torch.float64: FAZ_DOUBLE}.get(out_tensor.dtype)
    if dt is None or not out_tensor.is_contiguous():
        raise TypeError("output must be a contiguous float32/float64 CUDA tensor")
    st = (stream or torch.cuda.current_stream(out_tensor.device)).cuda_stream
    tm = FazTimings()
    with torch.cuda.device(out_tensor.device):
        _check(library().faz_decompress_payload_device(int(N), dt, payload, len(payload),
                                                       ctypes.c_void_p(out_tensor.data_ptr()), out_tensor.numel(),
                                                       ctypes.c_void_p(st), ctypes.byref(tm)))
    _tls.timings = tm
