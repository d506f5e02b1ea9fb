// noalloc.cu - error-bound resolution that allocates no memory.
//
// Some callers cannot allocate GPU memory at the point where they need the
// absolute error bound: code that runs under an allocation ban (real-time or
// safety-certified pipelines that allocate only at start-up), code that owns
// all device memory through its own arena, or a host thread that must not
// take the allocator's locks.  faz_resolve_eb_noalloc serves them: it computes
// the same absolute error bound as faz_compress (value range reduction, then
// the error-bound mode's formula) with its scratch - the per-block partial
// minima and maxima of the range reduction - in a fixed array compiled into
// this library instead of memory obtained from an allocator.
//
// The array is a file-scope __device__ array of kNoAllocScratchBytes (64 KiB
// plus 256 bytes): every GPU that loads this library keeps it until the
// process exits.  It holds one partial minimum and maximum for each of at most
// kNoAllocBlocks blocks, each block reducing a tile of kNoAllocTile values, so
// a field may have at most kNoAllocBlocks * kNoAllocTile = 2^28 values; larger
// fields are rejected.  A second one-block kernel folds the partials into the
// final minimum and maximum at the end of the array, and only those two values
// travel to the host.  All calls share the array and it keeps the last call's
// values; nothing in it needs to start at zero, because every call writes each
// entry it later reads.  Calls whose device work overlaps (on different
// streams, or from different host threads at once) race on the array.
//
// Host code cannot use the array's name as a device address: the array's
// address is looked up with cudaGetSymbolAddress on the first call on each
// device, with that device current, and cached for the life of the process.
// The cache assumes the device's primary context lives as long as the
// process: after cudaDeviceReset the cached address is stale, so this entry
// point must not be used after a reset.  Every call copies the two final
// values to the host and synchronizes `stream`, so no call may be made while
// `stream` is being captured (such calls are refused).
//
// The arguments are checked as faz_compress checks them (1 <= N <= 4, no zero
// extent, num equal to the product of the extents), and a resolved bound that
// is not positive and finite (a constant field, NaN values) is refused as
// faz_compress refuses it; on any failure conf is left unchanged.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "internal.h"

namespace faz {
namespace {

constexpr int kNoAllocBlocks = 4096;
constexpr uint64_t kNoAllocTile = 65536;
constexpr uint64_t kNoAllocMaxValues = (uint64_t)kNoAllocBlocks * kNoAllocTile;  // 2^28
constexpr size_t kNoAllocPartialBytes = (size_t)2 * kNoAllocBlocks * sizeof(double);  // 64 KiB
constexpr size_t kNoAllocScratchBytes = kNoAllocPartialBytes + 256;

// Partial minima at byte 0, maxima at byte kNoAllocBlocks * 8 (element type T
// either way); the final minimum and maximum at byte kNoAllocPartialBytes.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Fold nb partial minima/maxima into out[0] (minimum) and out[1] (maximum);
// one block of 1024 threads.
template <typename T>
__global__ void __launch_bounds__(1024) k_fold_minmax(const T *pmin, const T *pmax, int nb, T *out) {
    T mn = pmin[0], mx = pmax[0];
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        T a = pmin[i], b = pmax[i];
        mn = a < mn ? a : mn;
        mx = b > mx ? b : mx;
    }
    for (int o = 16; o > 0; o >>= 1) {
        T a = __shfl_down_sync(0xffffffffu, mn, o);
        T b = __shfl_down_sync(0xffffffffu, mx, o);
        mn = a < mn ? a : mn;
        mx = b > mx ? b : mx;
    }
    __shared__ T smn[32], smx[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { smn[wid] = mn; smx[wid] = mx; }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        mn = lane < nw ? smn[lane] : smn[0];
        mx = lane < nw ? smx[lane] : smx[0];
        for (int o = 16; o > 0; o >>= 1) {
            T a = __shfl_down_sync(0xffffffffu, mn, o);
            T b = __shfl_down_sync(0xffffffffu, mx, o);
            mn = a < mn ? a : mn;
            mx = b > mx ? b : mx;
        }
        if (lane == 0) { out[0] = mn; out[1] = mx; }
    }
}

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_ptr[kMaxDevices];

// Device address of the scratch array on the current device (looked up once).
int scratch_address(void **out, std::string &err) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
        return FAZ_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        err = "device index beyond the no-allocation table";
        return FAZ_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
            return FAZ_ERR_CUDA;
        }
        g_ptr[dev] = p;
    }
    *out = g_ptr[dev];
    return FAZ_OK;
}

template <typename T>
int resolve(faz_config *c, const T *d_data, cudaStream_t st, std::string &err) {
    if (c->errorBoundMode == FAZ_EB_ABS) return FAZ_OK;
    double rng = 0;
    if (c->errorBoundMode != FAZ_EB_L2NORM) {
        void *scratch = nullptr;
        int rc = scratch_address(&scratch, err);
        if (rc) return rc;
        const int nb = (int)((c->num + kNoAllocTile - 1) / kNoAllocTile);
        unsigned char *base = static_cast<unsigned char *>(scratch);
        T *pmin = reinterpret_cast<T *>(base);
        T *pmax = reinterpret_cast<T *>(base + kNoAllocBlocks * sizeof(double));
        T *fin = reinterpret_cast<T *>(base + kNoAllocPartialBytes);
        cudaError_t e = launch_minmax<T>(d_data, c->num, pmin, pmax, nb, st);
        if (e == cudaSuccess) {
            k_fold_minmax<T><<<1, 1024, 0, st>>>(pmin, pmax, nb, fin);
            e = cudaGetLastError();
        }
        T h[2];  // final minimum and maximum
        if (e == cudaSuccess) e = cudaMemcpyAsync(h, fin, sizeof(h), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            err = std::string("range reduction: ") + cudaGetErrorString(e);
            return FAZ_ERR_CUDA;
        }
        T r = h[1] - h[0];  // data_range: max - min in the element type
        rng = (double)r;
    }
    // calAbsErrorBound (include/QoZ/utils/Statistic.hpp:34-66)
    switch (c->errorBoundMode) {
    case FAZ_EB_REL:
        c->absErrorBound = c->relErrorBound * rng;
        break;
    case FAZ_EB_PSNR: {
        double v1 = c->psnrErrorBound + 10 * std::log10(1 - 2.0 / 3.0 * 0.99);
        double v3 = std::pow(10, v1 / (-20));
        c->absErrorBound = rng * v3;
        c->relErrorBound = c->absErrorBound / rng;
        break;
    }
    case FAZ_EB_L2NORM:
        c->absErrorBound = std::sqrt(3.0 / (double)c->num) * c->l2normErrorBound;
        break;
    case FAZ_EB_ABS_AND_REL:
        c->absErrorBound = c->absErrorBound < c->relErrorBound * rng ? c->absErrorBound : c->relErrorBound * rng;
        break;
    case FAZ_EB_ABS_OR_REL:
        c->absErrorBound = c->absErrorBound > c->relErrorBound * rng ? c->absErrorBound : c->relErrorBound * rng;
        break;
    default:
        err = "error bound mode not supported";
        return FAZ_ERR_ARG;
    }
    if (c->errorBoundMode != FAZ_EB_L2NORM) c->rng = rng;
    c->errorBoundMode = FAZ_EB_ABS;
    return FAZ_OK;
}

}  // namespace
}  // namespace faz

namespace faz {
namespace {

// The shape checks of faz_compress: 1 <= N <= 4, no zero extent, num equal to
// the product of the extents.
bool shape_ok(const faz_config &c, std::string &err) {
    if (c.N < 1 || c.N > 4) {
        err = "N must be 1..4";
        return false;
    }
    uint64_t num = 1;
    for (int i = 0; i < c.N; i++) {
        if (c.dims[i] == 0) {
            err = "zero dimension";
            return false;
        }
        num *= c.dims[i];
    }
    if (num != c.num) {
        err = "num does not match dims";
        return false;
    }
    return true;
}

}  // namespace
}  // namespace faz

extern "C" int faz_resolve_eb_noalloc(faz_config *conf, int dtype, const void *d_data, void *stream) {
    std::string err;
    int rc = FAZ_OK;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (!conf || !d_data) {
        err = "null argument";
        rc = FAZ_ERR_ARG;
    } else if (!faz::shape_ok(*conf, err)) {
        rc = FAZ_ERR_ARG;
    } else if (conf->num > faz::kNoAllocMaxValues) {
        err = "field of " + std::to_string(conf->num) + " values exceeds the no-allocation limit of " +
              std::to_string(faz::kNoAllocMaxValues) + " values";
        rc = FAZ_ERR_ARG;
    } else if (dtype != FAZ_FLOAT && dtype != FAZ_DOUBLE) {
        err = "dtype must be FAZ_FLOAT or FAZ_DOUBLE";
        rc = FAZ_ERR_ARG;
    } else if (cudaStreamIsCapturing((cudaStream_t)stream, &cap) != cudaSuccess ||
               cap != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        err = "the stream is being captured (this call synchronizes its stream)";
        rc = FAZ_ERR_ARG;
    } else {
        faz_config c = *conf;
        rc = dtype == FAZ_FLOAT ? faz::resolve<float>(&c, (const float *)d_data, (cudaStream_t)stream, err)
                                : faz::resolve<double>(&c, (const double *)d_data, (cudaStream_t)stream, err);
        if (rc == FAZ_OK && (!(c.absErrorBound > 0) || !std::isfinite(c.absErrorBound))) {
            err = "error bound must be positive and finite";
            rc = FAZ_ERR_ARG;
        }
        if (rc == FAZ_OK) *conf = c;
    }
    if (rc) faz::set_error("faz_resolve_eb_noalloc: " + err);
    return rc;
}
