"""QoZ::Config mirror shared by the Python host API and the C ABI.

`FazConfigStruct` is the ctypes image of `faz_config` in include/faz_gb300.h;
`Config` is the Python-facing class with the field names and defaults of the
reference's QoZ::Config (include/QoZ/utils/Config.hpp:62-508).
"""
import ctypes

MAX_LEVELS = 64

# QoZ enums (include/QoZ/utils/Config.hpp:18-42)
EB_ABS, EB_REL, EB_PSNR, EB_L2NORM, EB_ABS_AND_REL, EB_ABS_OR_REL = range(6)
EB_STR = ["ABS", "REL", "PSNR", "NORM", "ABS_AND_REL", "ABS_OR_REL"]
ALGO_LORENZO_REG, ALGO_INTERP_LORENZO, ALGO_INTERP, ALGO_INTERP_BLOCKED = range(4)
ALGO_STR = ["ALGO_LORENZO_REG", "ALGO_INTERP_LORENZO", "ALGO_INTERP", "ALGO_INTERP_BLOCKED"]
INTERP_ALGO_LINEAR, INTERP_ALGO_CUBIC = range(2)
INTERP_ALGO_STR = ["INTERP_ALGO_LINEAR", "INTERP_ALGO_CUBIC"]
TUNING_TARGET_RD, TUNING_TARGET_CR, TUNING_TARGET_SSIM, TUNING_TARGET_AC = range(4)
TUNING_TARGET_STR = ["TUNING_TARGET_RD", "TUNING_TARGET_CR", "TUNING_TARGET_SSIM", "TUNING_TARGET_AC"]

FAZ_FLOAT, FAZ_DOUBLE = 0, 1

_u8, _i32, _u64, _f64 = ctypes.c_uint8, ctypes.c_int32, ctypes.c_uint64, ctypes.c_double


class FazConfigStruct(ctypes.Structure):
    _fields_ = [
        ("N", _i32),
        ("dims", _u64 * 4),
        ("num", _u64),
        ("cmprAlgo", _u8),
        ("errorBoundMode", _u8),
        ("tuningTarget", _u8),
        ("absErrorBound", _f64),
        ("relErrorBound", _f64),
        ("psnrErrorBound", _f64),
        ("l2normErrorBound", _f64),
        ("rng", _f64),
        ("alpha", _f64),
        ("beta", _f64),
        ("autoTuningRate", _f64),
        ("predictorTuningRate", _f64),
        ("lorenzo", _u8),
        ("lorenzo2", _u8),
        ("regression", _u8),
        ("regression2", _u8),
        ("openmp", _u8),
        ("lossless", _u8),
        ("encoder", _u8),
        ("interpAlgo", _u8),
        ("interpDirection", _u8),
        ("levelwisePredictionSelection", _i32),
        ("interp_list_len", _i32),
        ("interpAlgo_list", _u8 * MAX_LEVELS),
        ("interpDirection_list", _u8 * MAX_LEVELS),
        ("maxStep", _u64),
        ("interpBlockSize", _i32),
        ("quantbinCnt", _i32),
        ("blockSize", _i32),
        ("testLorenzo", _i32),
        ("sampleBlockSize", _i32),
        ("blockwiseTuning", _u8),
        ("stride", _i32),
        ("pred_dim", _i32),
        ("profiling", _i32),
        ("SSIMBlockSize", _i32),
        ("fixBlockSize", _i32),
        ("blockwiseSampleBlockSize", _i32),
        ("verbose", _u8),
        ("QoZ", _u8),
        ("FZ", _u8),
        ("abList", _i32),
        ("crossBlock", _i32),
        ("sampleBlockSampleBlockSize", _i32),
        ("peTracking", _u8),
        ("wavelet", _i32),
        ("coeffs_num", _u64),
        ("coeffs_dims_len", _i32),
        ("coeffs_dims", _u64 * 4),
        ("wavelet_rel_coeff", _f64),
        ("firstSize", _u64),
        ("pid", _i32),
        ("offsetPredictor", _i32),
        ("trimToZero", _i32),
        ("preTrim", _f64),
        ("blockOrder", _i32),
        ("sperr", _i32),
        ("sperrWithoutWave", _u8),
        ("pyBind", _u8),
        ("conditioning", _i32),
        ("meta", _u8 * 17),
        ("pybind_activated", _u8),
        ("var_first", _i32),
    ]


class FazTimings(ctypes.Structure):
    _fields_ = [
        ("total_ms", _f64),
        ("h2d_ms", _f64),
        ("gpu_ms", _f64),
        ("d2h_ms", _f64),
        ("zstd_ms", _f64),
        ("host_ms", _f64),
        ("predict_ms", _f64),
        ("finest_level_ms", _f64),
        ("huffman_ms", _f64),
        ("payload_bytes", _u64),
        ("unpred_count", _u64),
        ("kernel_launches", _u64),
        ("tune_ms", _f64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_SCALARS = [name for name, typ in FazConfigStruct._fields_
            if name not in ("dims", "interpAlgo_list", "interpDirection_list", "coeffs_dims", "meta", "N", "num")]


class Config:
    """QoZ::Config with the reference's field names and defaults.

    `Config(100, 200, 300)` gives dims {100, 200, 300}, 300 the fastest
    dimension, as `QoZ::Config(Dims...)` (Config.hpp:64-74).  Level-wise
    interpolator lists are the Python lists `interpAlgo_list` and
    `interpDirection_list`.
    """

    def __init__(self, *dims):
        s = FazConfigStruct()
        object.__setattr__(self, "_s", s)
        object.__setattr__(self, "interpAlgo_list", [])
        object.__setattr__(self, "interpDirection_list", [])
        s.cmprAlgo = ALGO_INTERP_LORENZO
        s.errorBoundMode = EB_ABS
        s.tuningTarget = TUNING_TARGET_RD
        s.relErrorBound = -1.0
        s.rng = -1.0
        s.alpha = -1.0
        s.beta = -1.0
        s.lorenzo = 1
        s.regression = 1
        s.lossless = 1
        s.encoder = 1
        s.interpAlgo = INTERP_ALGO_CUBIC
        s.interpBlockSize = 32
        s.quantbinCnt = 65536
        s.SSIMBlockSize = 8
        s.verbose = 1
        s.wavelet_rel_coeff = 0.75
        s.sperr = -1
        s.pyBind = 1
        if len(dims) == 1 and isinstance(dims[0], (list, tuple)):
            dims = tuple(dims[0])
        if dims:
            self.setDims(dims)

    # Config::setDims / constructor defaults (Config.hpp:64-89, 394-499)
    def setDims(self, dims):
        dims = [int(d) for d in dims]
        if not 1 <= len(dims) <= 4:
            raise ValueError("FAZ supports 1 to 4 dimensions")
        s = self._s
        s.N = len(dims)
        num = 1
        for i, d in enumerate(dims):
            s.dims[i] = d
            s.coeffs_dims[i] = d
            num *= d
        for i in range(len(dims), 4):
            s.dims[i] = 0
            s.coeffs_dims[i] = 0
        s.num = num
        s.coeffs_num = num
        s.coeffs_dims_len = len(dims)
        s.blockSize = 128 if len(dims) == 1 else (16 if len(dims) == 2 else 6)
        s.pred_dim = len(dims)
        s.stride = s.blockSize
        return num

    @property
    def dims(self):
        return [int(self._s.dims[i]) for i in range(self._s.N)]

    @property
    def N(self):
        return int(self._s.N)

    @property
    def num(self):
        return int(self._s.num)

    def __getattr__(self, name):
        s = object.__getattribute__(self, "_s")
        if name in _SCALARS:
            return getattr(s, name)
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in ("interpAlgo_list", "interpDirection_list"):
            object.__setattr__(self, name, [int(v) for v in value])
            return
        if name in _SCALARS:
            setattr(self._s, name, value)
            return
        raise AttributeError(f"QoZ::Config has no field {name!r}")

    def to_struct(self):
        """ctypes image with the level-wise lists copied in."""
        if len(self.interpAlgo_list) != len(self.interpDirection_list):
            raise ValueError("interpAlgo_list and interpDirection_list differ in length")
        if len(self.interpAlgo_list) > MAX_LEVELS:
            raise ValueError("too many level-wise entries")
        s = FazConfigStruct()
        ctypes.memmove(ctypes.byref(s), ctypes.byref(self._s), ctypes.sizeof(s))
        s.interp_list_len = len(self.interpAlgo_list)
        for i, (a, d) in enumerate(zip(self.interpAlgo_list, self.interpDirection_list)):
            s.interpAlgo_list[i] = a
            s.interpDirection_list[i] = d
        return s

    @classmethod
    def from_struct(cls, s):
        c = cls()
        ctypes.memmove(ctypes.byref(c._s), ctypes.byref(s), ctypes.sizeof(s))
        n = int(s.interp_list_len)
        object.__setattr__(c, "interpAlgo_list", [int(s.interpAlgo_list[i]) for i in range(n)])
        object.__setattr__(c, "interpDirection_list", [int(s.interpDirection_list[i]) for i in range(n)])
        return c

    def copy(self):
        return Config.from_struct(self.to_struct())

    def __repr__(self):
        return (f"Config(dims={self.dims}, cmprAlgo={ALGO_STR[self.cmprAlgo]}, "
                f"eb_mode={EB_STR[self.errorBoundMode]}, abs={self.absErrorBound}, rel={self.relErrorBound})")


def ctype_size_check():
    """sizeof(faz_config) as ctypes computes it (compared against the C library in tests)."""
    return ctypes.sizeof(FazConfigStruct)
