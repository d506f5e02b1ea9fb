"""GB300-native FAZ interpolation compressor: Python host API.

Mirrors the reference's entry points (include/QoZ/api/sz.hpp):

    SZ_compress(conf, data)          -> bytes          (sz.hpp:54-108)
    SZ_decompress(conf, stream, T)   -> numpy.ndarray  (sz.hpp:159-225)

`conf` is a faz_gb300.Config (QoZ::Config fields and defaults).  `data` may
be a numpy array (host memory) or a CUDA torch tensor (device memory).  The
work runs in libfaz_gb300.so (hand-written sm_103a kernels behind the C ABI of
include/faz_gb300.h); there is no CPU fallback.
"""
import os as _os

# The default autotune runs its trials on separate CUDA streams beside the
# compression it starts early; with the driver's default of 8 hardware work
# queues, a trial's kernels can land in the queue of the long Lorenzo
# wavefront kernel and wait for it to end.  32 queues keep them apart.  The
# variable is read when the process creates its CUDA context, so it only takes
# effect when this package is imported before CUDA is first used.
_os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from .config import (Config, FazConfigStruct, FazTimings, ALGO_INTERP, ALGO_INTERP_LORENZO, ALGO_LORENZO_REG,
                     ALGO_INTERP_BLOCKED, EB_ABS, EB_REL, EB_PSNR, EB_L2NORM, EB_ABS_AND_REL, EB_ABS_OR_REL,
                     INTERP_ALGO_LINEAR, INTERP_ALGO_CUBIC, FAZ_FLOAT, FAZ_DOUBLE)
from .api import (FazError, SZ_compress, SZ_decompress, compress_device, decompress_device, library,
                  last_timings, zstd_version, load_ini, compress_payload_device, decompress_payload_device,
                  stream_info, tune_device, compress_batch)

__all__ = ["Config", "FazConfigStruct", "FazTimings", "FazError", "SZ_compress", "SZ_decompress",
           "compress_device", "decompress_device", "compress_payload_device", "decompress_payload_device", "stream_info", "tune_device", "compress_batch",
           "library", "last_timings", "zstd_version", "load_ini",
           "ALGO_INTERP", "ALGO_INTERP_LORENZO", "ALGO_LORENZO_REG", "ALGO_INTERP_BLOCKED", "EB_ABS", "EB_REL",
           "EB_PSNR", "EB_L2NORM", "EB_ABS_AND_REL", "EB_ABS_OR_REL", "INTERP_ALGO_LINEAR", "INTERP_ALGO_CUBIC",
           "FAZ_FLOAT", "FAZ_DOUBLE"]
