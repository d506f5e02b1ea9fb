// lorenzo.cu - the Lorenzo fast frontend for 3-D fields on the GPU
// (SZFastFrontend, include/QoZ/frontend/SZFastFrontend.hpp:170-437, with
// MetaLorenzoPredictor.hpp) and its stream section (save/load, lines 48-128).
//
// The reference walks blocks of bs^3 points in row-major order and predicts
// every point from reconstructed neighbours (one- or two-layer Lorenzo, chosen
// per block from the original data), keeping the reconstruction in a slab
// buffer padded with zeros.  That is the same as predicting from a full
// reconstructed field that reads as zero before the first plane, row and
// column, so a block depends only on blocks with smaller or equal block
// coordinates.  Blocks on one diagonal bi + bj + bk = d are therefore
// independent: one launch per diagonal, one warp per block.  Inside a block
// the warp walks the point diagonals i + j + k = s in a shared-memory tile
// that holds the block and its two-deep halo.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "host.h"
#include "internal.h"
#include "quant.cuh"

namespace faz {

namespace {

constexpr int kLorWarps = 8;     // blocks (warps) per CTA
constexpr int kLorMaxBs = 8;     // largest block edge on the GPU path
constexpr int kLorBatch = 8;     // tile loads in flight per lane
constexpr int kLorMaxRadius = 65536;  // quantbinCnt up to 131072 (32-bit codes above 65536 bins)

struct LorArgs {
    int64_t d1, d2, d3;   // field dims, slowest first
    int64_t nx, ny, nz;   // blocks per dim
    int bs;               // block edge
    int pd;               // prediction dimension (1, 2, 3)
    int lo, lo2;          // one- / two-layer Lorenzo allowed
    int reg;              // linear regression allowed
    const float *rp;      // per block: the 4 reconstructed regression coefficients
    LevelArgs q;          // quantiser (eb, 1/eb, radius, float split)
};

// MetaLorenzoPredictor.hpp:8-73 on a tile with strides (tx, ty, 1)
template <typename T>
__device__ __forceinline__ T lor_pred(const T *p, int tx, int ty, int pd, bool two) {
    if (two) {
        if (pd == 3)
            return (T)2 * p[-1] - p[-2] + (T)2 * p[-ty] - (T)4 * p[-ty - 1] + (T)2 * p[-ty - 2] - p[-2 * ty] +
                   (T)2 * p[-2 * ty - 1] - p[-2 * ty - 2] + (T)2 * p[-tx] - (T)4 * p[-tx - 1] + (T)2 * p[-tx - 2] -
                   (T)4 * p[-tx - ty] + (T)8 * p[-tx - ty - 1] - (T)4 * p[-tx - ty - 2] + (T)2 * p[-tx - 2 * ty] -
                   (T)4 * p[-tx - 2 * ty - 1] + (T)2 * p[-tx - 2 * ty - 2] - p[-2 * tx] + (T)2 * p[-2 * tx - 1] -
                   p[-2 * tx - 2] + (T)2 * p[-2 * tx - ty] - (T)4 * p[-2 * tx - ty - 1] + (T)2 * p[-2 * tx - ty - 2] -
                   p[-2 * tx - 2 * ty] + (T)2 * p[-2 * tx - 2 * ty - 1] - p[-2 * tx - 2 * ty - 2];
        if (pd == 2)
            return (T)2 * p[-tx] - p[-2 * tx] + (T)2 * p[-1] - (T)4 * p[-1 - tx] + (T)2 * p[-1 - 2 * tx] - p[-2] +
                   (T)2 * p[-2 - tx] - p[-2 - 2 * tx];
        return (T)2 * p[-1] - p[-2];
    }
    if (pd == 3) return p[-1] + p[-ty] + p[-tx] - p[-ty - 1] - p[-tx - 1] - p[-tx - ty] + p[-tx - ty - 1];
    if (pd == 2) return p[-1] + p[-tx] - p[-1 - tx];
    return p[-1];
}

// The same predictors on the original field (strides d0, d1, 1), returned in T
template <typename T>
__device__ __forceinline__ T lor_pred_g(const T *p, int64_t d0, int64_t d1, int pd, bool two) {
    if (two) {
        if (pd == 3)
            return (T)2 * p[-1] - p[-2] + (T)2 * p[-d1] - (T)4 * p[-d1 - 1] + (T)2 * p[-d1 - 2] - p[-2 * d1] +
                   (T)2 * p[-2 * d1 - 1] - p[-2 * d1 - 2] + (T)2 * p[-d0] - (T)4 * p[-d0 - 1] + (T)2 * p[-d0 - 2] -
                   (T)4 * p[-d0 - d1] + (T)8 * p[-d0 - d1 - 1] - (T)4 * p[-d0 - d1 - 2] + (T)2 * p[-d0 - 2 * d1] -
                   (T)4 * p[-d0 - 2 * d1 - 1] + (T)2 * p[-d0 - 2 * d1 - 2] - p[-2 * d0] + (T)2 * p[-2 * d0 - 1] -
                   p[-2 * d0 - 2] + (T)2 * p[-2 * d0 - d1] - (T)4 * p[-2 * d0 - d1 - 1] + (T)2 * p[-2 * d0 - d1 - 2] -
                   p[-2 * d0 - 2 * d1] + (T)2 * p[-2 * d0 - 2 * d1 - 1] - p[-2 * d0 - 2 * d1 - 2];
        if (pd == 2)
            return (T)2 * p[-d0] - p[-2 * d0] + (T)2 * p[-1] - (T)4 * p[-1 - d0] + (T)2 * p[-1 - 2 * d0] - p[-2] +
                   (T)2 * p[-2 - d0] - p[-2 - 2 * d0];
        return (T)2 * p[-1] - p[-2];
    }
    if (pd == 3) return p[-1] + p[-d1] + p[-d0] - p[-d1 - 1] - p[-d0 - 1] - p[-d0 - d1] + p[-d0 - d1 - 1];
    if (pd == 2) return p[-1] + p[-d0] - p[-1 - d0];
    return p[-1];
}

// meta_block_error_estimation_3d for one point (SZFastFrontend.hpp:440-495),
// regression off.  Noise constants from include/QoZ/utils/MetaDef.hpp:24-29.
template <typename T>
__device__ __forceinline__ void meta_est(const T *c, int64_t d0, int64_t d1, T prec, int pd, int lo, int lo2,
                                         double &el, double &el2) {
    const T cd = *c;
    double lp = 0, lp2 = 0;
    T noise = 0, noise2 = 0;
    const double n1 = pd == 3 ? 1.22 : (pd == 2 ? 0.81 : 0.5);
    const double n2 = pd == 3 ? 6.8 : (pd == 2 ? 2.76 : 1.08);
    if (lo2) {
        lp2 = (double)lor_pred_g(c, d0, d1, pd, true);
        noise2 = (T)(n2 * (double)prec);
    }
    if (lo) {
        lp = (double)lor_pred_g(c, d0, d1, pd, false);
        noise = (T)(n1 * (double)prec);
    }
    el += fabs((double)cd - lp) + (double)noise;
    el2 += fabs((double)cd - lp2) + (double)noise2;
}

// compute_regression_coeffcients_3d (MetaRegressionPredictor.hpp:104-139),
// float sums in the reference's loop order.
template <typename T>
__device__ void reg_coeffs(const T *d, int sx, int sy, int sz, int64_t d0, int64_t d1, float *rp) {
    const T *cur = d;
    float fx = 0.0f, fy = 0.0f, fz = 0.0f, f = 0;
    for (int i = 0; i < sx; i++) {
        float sum_x = 0;
        for (int j = 0; j < sy; j++) {
            float sum_y = 0;
            for (int k = 0; k < sz; k++) {
                const T cd = *cur;
                sum_y = (float)(sum_y + cd);
                fz = (float)(fz + (T)(cd * (T)k));
                cur++;
            }
            fy += sum_y * (float)j;
            sum_x += sum_y;
            cur += (d1 - sz);
        }
        fx += sum_x * (float)i;
        f += sum_x;
        cur += (d0 - sy * d1);
    }
    const float coeff = (float)(1.0 / (sx * sy * sz));
    rp[0] = (2 * fx / (float)(sx - 1) - f) * 6 * coeff / (float)(sx + 1);
    rp[1] = (2 * fy / (float)(sy - 1) - f) * 6 * coeff / (float)(sy + 1);
    rp[2] = (2 * fz / (float)(sz - 1) - f) * 6 * coeff / (float)(sz + 1);
    rp[3] = f * coeff - ((float)(sx - 1) * rp[0] / 2 + (float)(sy - 1) * rp[1] / 2 + (float)(sz - 1) * rp[2] / 2);
}

// meta_blockwise_selection_3d (SZFastFrontend.hpp:498-540), one thread per
// block: 0 Lorenzo, 1 regression, 2 two-layer Lorenzo.  The block's raw
// regression coefficients go to raw[4b..4b+3].
template <typename T>
__global__ void k_lor_select(LorArgs a, const T *__restrict__ X, uint16_t *__restrict__ ind, float *__restrict__ raw) {
    const int64_t nb = a.nx * a.ny * a.nz;
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int64_t bk = b % a.nz, bj = (b / a.nz) % a.ny, bi = b / (a.nz * a.ny);
    const int bs = a.bs;
    const int sx = (bi + 1) * bs < a.d1 ? bs : (int)(a.d1 - bi * bs);
    const int sy = (bj + 1) * bs < a.d2 ? bs : (int)(a.d2 - bj * bs);
    const int sz = (bk + 1) * bs < a.d3 ? bs : (int)(a.d3 - bk * bs);
    int ms = sx < sy ? sx : sy;
    ms = ms < sz ? ms : sz;
    const int64_t d0 = a.d2 * a.d3, d1 = a.d3;
    const T *dp = X + bi * bs * d0 + bj * bs * d1 + bk * bs;
    const T prec = (T)a.q.eb;
    const bool ereg = a.reg && ms >= 2;
    float rp[4] = {0, 0, 0, 0};
    if (ereg) reg_coeffs(dp, sx, sy, sz, d0, d1, rp);
    double el = 0, el2 = 0, er = 0;
    auto est = [&](int x, int y, int z) {
        const T *c = dp + x * d0 + y * d1 + z;
        if (ereg) {
            // regression_predict_3d<T> (MetaRegressionPredictor.hpp:142-146)
            const T pr = (T)(rp[0] * (float)x + rp[1] * (float)y + rp[2] * (float)z + rp[3]);
            const T df = *c - pr;
            er += (double)(df < 0 ? -df : df);
        }
        meta_est(c, d0, d1, prec, a.pd, a.lo, a.lo2, el, el2);
    };
    for (int i = 2; i < ms - 1; i++) {
        const int m = ms - i;
        est(i, i, i);
        est(i, i, m);
        est(i, m, i);
        est(i, m, m);
    }
    if (ms > 3) est(ms - 1, ms - 1, ms - 1);
    int sel;
    if (ereg && (!a.lo || er <= el) && (!a.lo2 || er < el2)) sel = 1;
    else if (a.lo2 && (!a.lo || el2 <= el) && (!ereg || el2 <= er)) sel = 2;
    else sel = 0;
    ind[b] = (uint16_t)sel;
    if (raw) {
        for (int c = 0; c < 4; c++) raw[4 * b + c] = rp[c];
    }
}

// Loads with the L2 as the point of coherence: the wavefront reads blocks
// that other SMs wrote during the same launch, and L1 is not coherent.
template <typename T>
__device__ __forceinline__ T ld_coherent(const T *p) {
    return __ldcg(p);
}

__device__ __forceinline__ void lor_st_release(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned lor_ld_relaxed(const unsigned *p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// with a relaxed load that saw a release store before it, an acquire pattern
__device__ __forceinline__ void lor_fence_acq_rel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// The original values of block (bi, bj, bk) into the warp's tile (after its
// (bs + 2)^3 halo part); they depend on no other block, so the persistent
// kernel loads them before it waits for the block's neighbours.
template <typename T>
__device__ __forceinline__ void lor_load_x(const LorArgs &a, int64_t bi, int64_t bj, int64_t bk, T *t,
                                           const T *__restrict__ X) {
    const int lane = threadIdx.x & 31;
    const int bs = a.bs;
    const int sx = (bi + 1) * bs < a.d1 ? bs : (int)(a.d1 - bi * bs);
    const int sy = (bj + 1) * bs < a.d2 ? bs : (int)(a.d2 - bj * bs);
    const int sz = (bk + 1) * bs < a.d3 ? bs : (int)(a.d3 - bk * bs);
    const int64_t x0 = bi * bs, y0 = bj * bs, z0 = bk * bs;
    const int64_t d0 = a.d2 * a.d3, dd1 = a.d3;
    T *xs = t + (bs + 2) * (bs + 2) * (bs + 2);
    const int nv = sx * sy * sz;
    for (int e0 = lane; e0 < nv; e0 += 32 * kLorBatch) {
        T v[kLorBatch];
#pragma unroll
        for (int u = 0; u < kLorBatch; u++) {
            const int e = e0 + 32 * u;
            const int i = e / (sy * sz), r = e - i * sy * sz, j = r / sz, k = r - j * sz;
            v[u] = e < nv ? X[(x0 + i) * d0 + (y0 + j) * dd1 + (z0 + k)] : (T)0;
        }
#pragma unroll
        for (int u = 0; u < kLorBatch; u++)
            if (e0 + 32 * u < nv) xs[e0 + 32 * u] = v[u];
    }
}

// One block (bi, bj, bk), one warp: the (bs + 2)^3 tile with its two-deep
// halo of reconstructed values, then the point diagonals i + j + k = s in
// order, each point predicted from its reconstructed neighbours (in
// compression the block's original values are already in the tile:
// lor_load_x).
template <typename T, bool DECOMP, int QM, typename C>
__device__ __forceinline__ void lor_block(const LorArgs &a, int64_t bi, int64_t bj, int64_t bk, T *t, int sel,
                                          const float (&rp)[4], const uint32_t *halo, T *__restrict__ R,
                                          C *__restrict__ codes, T *__restrict__ scratch,
                                          const uint64_t *__restrict__ zpos, uint64_t nzp,
                                          const T *__restrict__ unpred) {
    const int lane = threadIdx.x & 31;
    const int bs = a.bs;
    const int sx = (bi + 1) * bs < a.d1 ? bs : (int)(a.d1 - bi * bs);
    const int sy = (bj + 1) * bs < a.d2 ? bs : (int)(a.d2 - bj * bs);
    const int sz = (bk + 1) * bs < a.d3 ? bs : (int)(a.d3 - bk * bs);
    const int64_t x0 = bi * bs, y0 = bj * bs, z0 = bk * bs;
    const int64_t d0 = a.d2 * a.d3, dd1 = a.d3;
    // tile strides: (tx, ty, 1) over (sx + 2) x (sy + 2) x (sz + 2)
    const int tz = sz + 2, ty = tz, tx = (sy + 2) * tz;
    T *xs = t + (bs + 2) * (bs + 2) * (bs + 2);
    const int tn = (sx + 2) * (sy + 2) * tz;
    // loads in batches of kLorBatch per lane, all issued before any is used
    if (sx == bs && sy == bs && sz == bs) {
        // a full block: the halo positions come from the CTA's table
        const int nh = tn - bs * bs * bs;
        for (int h0 = lane; h0 < nh; h0 += 32 * kLorBatch) {
            T v[kLorBatch];
#pragma unroll
            for (int u = 0; u < kLorBatch; u++) {
                const int h = h0 + 32 * u;
                const uint32_t p = h < nh ? halo[h] : 0u;
                const int64_t gx = x0 + (int)(p & 15u) - 2, gy = y0 + (int)((p >> 4) & 15u) - 2,
                              gz = z0 + (int)((p >> 8) & 15u) - 2;
                v[u] = (h < nh && gx >= 0 && gy >= 0 && gz >= 0) ? ld_coherent(R + (gx * d0 + gy * dd1 + gz)) : (T)0;
            }
#pragma unroll
            for (int u = 0; u < kLorBatch; u++) {
                const int h = h0 + 32 * u;
                if (h < nh) t[halo[h] >> 12] = v[u];
            }
        }
    } else
    for (int e0 = lane; e0 < tn; e0 += 32 * kLorBatch) {
        T v[kLorBatch];
#pragma unroll
        for (int u = 0; u < kLorBatch; u++) {
            const int e = e0 + 32 * u;
            const int i = e / tx, r = e - i * tx, j = r / tz, k = r - j * tz;
            const int64_t gx = x0 + i - 2, gy = y0 + j - 2, gz = z0 + k - 2;
            const bool inside = i >= 2 && j >= 2 && k >= 2;
            v[u] = (e < tn && !inside && gx >= 0 && gy >= 0 && gz >= 0) ? ld_coherent(R + (gx * d0 + gy * dd1 + gz))
                                                                       : (T)0;
        }
#pragma unroll
        for (int u = 0; u < kLorBatch; u++)
            if (e0 + 32 * u < tn) t[e0 + 32 * u] = v[u];
    }
    __syncwarp();
    const bool two = sel == 2;
    const uint64_t boff = (uint64_t)(bi * bs) * (uint64_t)d0 + (uint64_t)(bj * bs) * (uint64_t)(sx * a.d3) +
                          (uint64_t)(bk * bs) * (uint64_t)(sx * sy);
    const int nsteps = sx + sy + sz - 2;
    const int npairs = sx * sy;
    // a lane's (i, j) pairs: lane, lane + 32, ... (one pair for edges up to 5)
    const int i0 = lane / sy, j0 = lane - i0 * sy;
    for (int s = 0; s < nsteps; s++) {
        int i = i0, j = j0;
        for (int pr = lane; pr < npairs; pr += 32) {
            if (pr != lane) {
                i = pr / sy;
                j = pr - i * sy;
            }
            const int k = s - i - j;
            if (k < 0 || k >= sz) continue;
            T *c = t + (i + 2) * tx + (j + 2) * ty + (k + 2);
            T pred;
            if (sel == 1) {
                // regression_predict_quantize_3d (MetaRegressionPredictor.hpp:148-189)
                pred = (T)(rp[0] * (float)i + rp[1] * (float)j + rp[2] * (float)k + rp[3]);
            } else {
                pred = lor_pred(c, tx, ty, a.pd, two);
            }
            const uint64_t pos = boff + (uint64_t)((i * sy + j) * sz + k);
            T v;
            if (!DECOMP) {
                v = xs[(i * sy + j) * sz + k];
                T uval;
                const int code = quant_point<T, QM>(v, pred, a.q, uval);
                codes[pos] = (C)code;
                if (code == 0) scratch[pos] = uval;
            } else {
                v = recover_point<T, QM>(pred, (int)codes[pos], pos, a.q, zpos, nzp, unpred);
            }
            *c = v;
            R[(x0 + i) * d0 + (y0 + j) * dd1 + (z0 + k)] = v;
        }
        __syncwarp();
    }
}

constexpr unsigned kLorWaitLimit = 1u << 22;  // polls (with back-off) of a block's neighbours before giving up

// The whole wavefront in one launch of persistent CTAs.  A warp takes a
// ticket, and with it the block order[ticket]: blocks come diagonal by
// diagonal (bi + bj + bk ascending), so the blocks a block reads - its face
// neighbours (bi-1, bj, bk), (bi, bj-1, bk), (bi, bj, bk-1), which in turn
// waited for theirs - hold smaller tickets, taken by warps already running,
// and every wait ends.  Each wait is bounded all the same (error flag, then
// the block runs).  A finished block publishes done[b] = 1 with release
// semantics after its reconstruction is written.
template <typename T, bool DECOMP, int QM, typename C>
__global__ void __launch_bounds__(kLorWarps * 32)
    k_lor_persist(LorArgs a, const uint32_t *__restrict__ order, uint32_t nblocks, unsigned *counter,
                  unsigned *done, int *err, const T *__restrict__ X, T *__restrict__ R,
                  C *__restrict__ codes, T *__restrict__ scratch, const uint16_t *__restrict__ ind,
                  const uint64_t *__restrict__ zpos, uint64_t nzp, const T *__restrict__ unpred) {
    extern __shared__ __align__(16) unsigned char lor_smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int bs = a.bs;
    const int tstride = (bs + 2) * (bs + 2) * (bs + 2) + (DECOMP ? 0 : bs * bs * bs);
    T *t = reinterpret_cast<T *>(lor_smem) + (size_t)w * (size_t)tstride;
    // The halo positions of a full block's tile (i < 2, j < 2 or k < 2 in the
    // (bs + 2)^3 tile), packed i | j << 4 | k << 8 | tile index << 12, in tile
    // order: entry = tile index - interior points before it.
    uint32_t *halo = reinterpret_cast<uint32_t *>(lor_smem + (size_t)kLorWarps * (size_t)tstride * sizeof(T));
    {
        const int te = bs + 2, tn = te * te * te;
        for (int e = threadIdx.x; e < tn; e += blockDim.x) {
            const int i = e / (te * te), j = (e / te) % te, k = e % te;
            if (i >= 2 && j >= 2 && k >= 2) continue;
            int before = (i > 2 ? i - 2 : 0) * bs * bs;
            if (i >= 2) before += (j > 2 ? j - 2 : 0) * bs;
            if (i >= 2 && j >= 2) before += k > 2 ? k - 2 : 0;
            halo[e - before] = (uint32_t)i | ((uint32_t)j << 4) | ((uint32_t)k << 8) | ((uint32_t)e << 12);
        }
        __syncthreads();
    }
    const int64_t plane = a.ny * a.nz;
    // A warp takes its next ticket as it starts a block, so that the atomic's
    // round trip overlaps the block.  The smallest unfinished ticket is then
    // always some warp's current block (a warp's next ticket is larger than
    // its current one), whose neighbours hold smaller tickets: waits still end.
    unsigned nxt = 0;
    if (lane == 0) nxt = atomicAdd(counter, 1u);
    for (;;) {
        const unsigned tk = __shfl_sync(0xffffffffu, nxt, 0);
        if (tk >= nblocks) break;
        if (lane == 0) nxt = atomicAdd(counter, 1u);
        const int64_t b = order[tk];
        const int64_t bk = b % a.nz, bj = (b / a.nz) % a.ny, bi = b / plane;
        const unsigned *deps[3] = {bi > 0 ? done + (b - plane) : nullptr, bj > 0 ? done + (b - a.nz) : nullptr,
                                   bk > 0 ? done + (b - 1) : nullptr};
        // the block's own values, its predictor selection and regression
        // coefficients need no neighbour: their loads overlap the wait
        if (!DECOMP) lor_load_x<T>(a, bi, bj, bk, t, X);
        int sel = ind[b];
        float rp[4] = {0, 0, 0, 0};
        if (sel == 1) {
            if (a.rp == nullptr) sel = 0;  // a stream without coefficients
            else
                for (int c = 0; c < 4; c++) rp[c] = a.rp[4 * b + c];
        }
        // every lane polls the (up to three) neighbours' flags together with
        // relaxed loads; the fence after all are seen set orders the halo
        // loads after the neighbours' writes
        {
            unsigned it = 0;
            for (;;) {
                const unsigned f0 = deps[0] ? lor_ld_relaxed(deps[0]) : 1u;
                const unsigned f1 = deps[1] ? lor_ld_relaxed(deps[1]) : 1u;
                const unsigned f2 = deps[2] ? lor_ld_relaxed(deps[2]) : 1u;
                if (__all_sync(0xffffffffu, f0 != 0u && f1 != 0u && f2 != 0u)) break;
                if (++it > kLorWaitLimit) {
                    if (lane == 0) atomicExch(err, 1);
                    break;
                }
                __nanosleep(32);
            }
            lor_fence_acq_rel();
        }
        lor_block<T, DECOMP, QM, C>(a, bi, bj, bk, t, sel, rp, halo, R, codes, scratch, zpos, nzp, unpred);
        // each lane's reconstruction writes are released before the warp's flag
        lor_fence_acq_rel();
        __syncwarp();
        if (lane == 0) lor_st_release(done + b, 1u);
    }
}

template <typename T>
LorArgs make_args(const uint64_t *dims, int bs, int pd, int lo, int lo2, double eb, int radius, int reg = 0) {
    LorArgs a;
    std::memset(&a, 0, sizeof(a));
    a.d1 = (int64_t)dims[0];
    a.d2 = (int64_t)dims[1];
    a.d3 = (int64_t)dims[2];
    a.bs = bs;
    a.nx = (a.d1 - 1) / bs + 1;
    a.ny = (a.d2 - 1) / bs + 1;
    a.nz = (a.d3 - 1) / bs + 1;
    a.pd = pd;
    a.lo = lo;
    a.lo2 = lo2;
    a.reg = reg;
    a.rp = nullptr;
    a.q.eb = eb;
    a.q.recip = 1.0 / eb;
    a.q.radius = radius;
    a.q.trim = 0;
    set_fast_path<T>(a.q);
    return a;
}

// Launches the wavefront on `st`; its error flag comes back to the returned
// pinned word, to be read (check_wavefront) once `st` is synchronised.
// C: uint16_t codes, or uint32_t for more than 65536 quantisation bins.
template <typename T, typename C>
const int *launch_wavefront(const LorArgs &a, bool decomp, const T *X, T *R, C *codes, T *scratch,
                            const uint16_t *ind, const uint64_t *zpos, uint64_t nz, const T *unpred, cudaStream_t st,
                            Counter &launches) {
    const bool straight = sizeof(T) == 4 && a.q.fast;
    // the warps' tiles, then the halo table (4 bytes per halo position)
    const size_t smem = (size_t)kLorWarps *
                            (size_t)((a.bs + 2) * (a.bs + 2) * (a.bs + 2) + (decomp ? 0 : a.bs * a.bs * a.bs)) *
                            sizeof(T) +
                        (size_t)((a.bs + 2) * (a.bs + 2) * (a.bs + 2) - a.bs * a.bs * a.bs) * 4;
    void (*k)(LorArgs, const uint32_t *, uint32_t, unsigned *, unsigned *, int *, const T *, T *, C *, T *,
              const uint16_t *, const uint64_t *, uint64_t, const T *);
    if (!decomp) k = straight ? k_lor_persist<T, false, 1, C> : k_lor_persist<T, false, 0, C>;
    else k = straight ? k_lor_persist<T, true, 1, C> : k_lor_persist<T, true, 0, C>;
    CK(allow_dynamic_smem((const void *)k));
    const uint64_t nb64 = (uint64_t)(a.nx * a.ny * a.nz);
    if (nb64 >= (1ull << 32)) throw Fail{FAZ_ERR_UNSUPPORTED, "too many Lorenzo blocks"};
    const uint32_t nb = (uint32_t)nb64;
    // blocks in diagonal order (bi + bj + bk ascending, then bi, then bj)
    std::vector<uint32_t> order;
    order.reserve(nb);
    const int64_t last = (a.nx - 1) + (a.ny - 1) + (a.nz - 1);
    size_t widest = 0;  // blocks on the longest diagonal: the most that are ever ready at once
    for (int64_t d = 0; d <= last; d++) {
        const size_t before = order.size();
        const int64_t bi_lo = std::max<int64_t>(0, d - (a.ny - 1) - (a.nz - 1));
        const int64_t bi_hi = std::min<int64_t>(a.nx - 1, d);
        for (int64_t bi = bi_lo; bi <= bi_hi; bi++) {
            const int64_t r = d - bi;
            const int64_t bj_lo = std::max<int64_t>(0, r - (a.nz - 1)), bj_hi = std::min<int64_t>(a.ny - 1, r);
            for (int64_t bj = bj_lo; bj <= bj_hi; bj++)
                order.push_back((uint32_t)((bi * a.ny + bj) * a.nz + (r - bj)));
        }
        widest = std::max(widest, order.size() - before);
    }
    if (order.size() != nb) throw Fail{FAZ_ERR_DEVICE, "Lorenzo block order does not cover the blocks"};
    DevMem m(st);
    uint32_t *dorder = m.alloc<uint32_t>(nb);
    unsigned *sync = m.alloc<unsigned>((size_t)nb + 2);  // counter, done[nb]
    int *derr = m.alloc<int>(1);
    CK(cudaMemcpyAsync(dorder, order.data(), (size_t)nb * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(sync, 0, ((size_t)nb + 2) * 4, st));
    CK(cudaMemsetAsync(derr, 0, 4, st));
    int dev = 0, sms = 0, per_sm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kLorWarps * 32, smem));
    if (per_sm < 1) throw Fail{FAZ_ERR_UNSUPPORTED, "Lorenzo block does not fit on an SM"};
    // never more CTAs than stay resident (waits rely on it), nor more warps than
    // blocks on the widest diagonal: more would only wait, and hold SMs that
    // concurrent work (the tuner's other trials) needs
    const uint64_t want = (widest + kLorWarps - 1) / kLorWarps;
    const int grid = (int)std::min<uint64_t>((uint64_t)sms * (uint64_t)per_sm, want);
    k<<<grid, kLorWarps * 32, smem, st>>>(a, dorder, nb, sync, sync + 1, derr, X, R, codes, scratch, ind, zpos, nz,
                                          unpred);
    launches(cudaGetLastError());
    // the flag comes back through pinned memory: a copy to pageable memory
    // would hold the driver's pageable staging path while this kernel runs,
    // stalling concurrent pageable copies (the tuner's other trials)
    int *herr = (int *)t_pin_flag.get(64);
    CK(cudaMemcpyAsync(herr, derr, 4, cudaMemcpyDeviceToHost, st));
    return herr;
}

void check_wavefront(const int *herr) {
    if (*herr) throw Fail{FAZ_ERR_DEVICE, "Lorenzo wavefront: a block waited too long for its neighbours"};
}

template <typename T, typename C>
void run_wavefront(const LorArgs &a, bool decomp, const T *X, T *R, C *codes, T *scratch, const uint16_t *ind,
                   const uint64_t *zpos, uint64_t nz, const T *unpred, cudaStream_t st, Counter &launches) {
    const int *herr = launch_wavefront<T, C>(a, decomp, X, R, codes, scratch, ind, zpos, nz, unpred, st, launches);
    CK(cudaStreamSynchronize(st));
    check_wavefront(herr);
}

// meta_params as written by write(params, c) (include/QoZ/utils/MetaDef.hpp:33-60):
// 44 bytes, the reference's uninitialised padding written as zeros.
void put_meta_params(std::vector<uint8_t> &o, int bs, int pd, int lo, int lo2, int reg, double eb) {
    uint8_t m[44];
    std::memset(m, 0, sizeof m);
    const float prec = (float)eb;
    const float eb_lin = 1.0f * prec / 4 / (float)bs;
    const float eb_ind = (float)bs * eb_lin;
    int32_t v = bs;
    std::memcpy(m + 0, &v, 4);
    v = pd;
    std::memcpy(m + 4, &v, 4);
    m[8] = (uint8_t)(lo != 0);
    m[9] = (uint8_t)(lo2 != 0);
    m[10] = (uint8_t)(reg != 0);
    v = 2;  // lorenzo_padding_layer
    std::memcpy(m + 12, &v, 4);
    std::memcpy(m + 20, &eb_ind, 4);
    std::memcpy(m + 24, &eb_lin, 4);
    float f = 1.0f;  // reg_eb_base
    std::memcpy(m + 28, &f, 4);
    f = (float)bs;   // reg_eb_1
    std::memcpy(m + 32, &f, 4);
    f = 1.0f;        // sample_ratio
    std::memcpy(m + 36, &f, 4);
    m[40] = 1;       // lossless
    o.insert(o.end(), m, m + sizeof m);
}

// Regression coefficient precisions (MetaDef.hpp:54-59 and
// SZFastFrontend.hpp:229-235), in the element type T.
template <typename T>
void reg_precisions(int bs, double eb, T prec[4], T rprec[4]) {
    const float fprec = (float)eb;
    const float eb_lin = 1.0f * fprec / 4 / (float)bs;
    const float eb_ind = (float)bs * eb_lin;
    for (int i = 0; i < 3; i++) prec[i] = (T)eb_lin;
    prec[3] = (T)eb_ind;
    for (int i = 0; i < 4; i++) rprec[i] = (T)(1.0 / prec[i]);
}

// compress_regression_coefficient_3d over the regression blocks in block
// order (MetaRegressionPredictor.hpp:10-40): each coefficient is predicted by
// the previous regression block's reconstructed one, a serial chain; rec
// receives the reconstructed coefficients of every regression block.
template <typename T>
void reg_chain_compress(const std::vector<uint16_t> &ind, const std::vector<float> &raw, int bs, double eb,
                        std::vector<float> &rec, std::vector<uint16_t> &types, std::vector<float> &unp) {
    T prec[4], rprec[4];
    reg_precisions<T>(bs, eb, prec, rprec);
    float prev[4] = {0, 0, 0, 0};
    rec.assign(raw.size(), 0.0f);
    for (size_t b = 0; b < ind.size(); b++) {
        if (ind[b] != 1) continue;
        for (int c = 0; c < 4; c++) {
            const float pred = prev[c], cur = raw[4 * b + c];
            const double p = (double)prec[c], rp = (double)rprec[c];
            const double diff = (double)(float)(cur - pred);
            double qd = std::fabs(diff) * rp + 1;
            int code = 0;
            float dec = cur;
            if (qd < 65536) {
                qd = diff > 0 ? qd : -qd;
                const int qi = (int)(qd / 2) + 32768;
                const float dd = (float)((double)pred + (double)(2 * (qi - 32768)) * p);
                dec = dd;
                if (std::fabs((double)(float)(dd - cur)) <= p) code = qi;
                else dec = cur;
            }
            if (code == 0) unp.push_back(cur);
            types.push_back((uint16_t)code);
            rec[4 * b + c] = dec;
            prev[c] = dec;
        }
    }
}

// decode_regression_coefficients (MetaRegressionPredictor.hpp:42-80)
template <typename T>
void reg_chain_decompress(const std::vector<uint16_t> &ind, const std::vector<uint16_t> &types, const float *unp,
                          uint64_t nunp, float eb_lin, float eb_ind, std::vector<float> &rec) {
    T prec[4];
    for (int i = 0; i < 3; i++) prec[i] = (T)eb_lin;
    prec[3] = (T)eb_ind;
    float prev[4] = {0, 0, 0, 0};
    rec.assign(4 * ind.size(), 0.0f);
    size_t ti = 0;
    uint64_t ui = 0;
    for (size_t b = 0; b < ind.size(); b++) {
        if (ind[b] != 1) continue;
        for (int c = 0; c < 4; c++) {
            if (ti >= types.size()) throw Fail{FAZ_ERR_FORMAT, "regression coefficient stream too short"};
            const int tv = types[ti++];
            float v;
            if (tv == 0) {
                if (ui >= nunp) throw Fail{FAZ_ERR_FORMAT, "regression coefficient unpredictables exhausted"};
                std::memcpy(&v, unp + ui, 4);
                ui++;
            } else {
                v = (float)((double)prev[c] + (double)(2 * (tv - 32768)) * (double)prec[c]);
            }
            rec[4 * b + c] = v;
            prev[c] = v;
        }
    }
}

}  // namespace

void check_lorenzo3(const uint64_t *dims, int bs, int pd, int lo, int lo2, int reg, int radius) {
    if (!lo && !lo2 && !reg) throw Fail{FAZ_ERR_ARG, "all Lorenzo and regression predictors are disabled"};
    if (bs < 1 || bs > kLorMaxBs) throw Fail{FAZ_ERR_UNSUPPORTED, "Lorenzo block size must be 1..8 on the GPU path"};
    if (pd < 1 || pd > 3) throw Fail{FAZ_ERR_ARG, "pred_dim must be 1..3"};
    if (radius < 1 || radius > kLorMaxRadius)
        throw Fail{FAZ_ERR_UNSUPPORTED, "quantbinCnt above 131072 is not implemented on the GPU path"};
    for (int i = 0; i < 3; i++)
        if (dims[i] == 0) throw Fail{FAZ_ERR_ARG, "zero dimension"};
}

// SZ_compress_LorenzoReg for 3-D data (include/QoZ/api/impl/SZLorenzoReg.hpp:94-114):
// SZFastFrontend::compress_3d + save, then the general compressor's Huffman
// stage (SZGeneralCompressor.hpp:30-70).  Returns the pre-zstd payload in
// `out` (host).
template <typename T>
void lorenzo3_compress_payload(const uint64_t *dims, int bs, int pd, int lo, int lo2, int reg, double eb, int radius,
                               const T *dX, cudaStream_t st, Counter &launches, faz_timings &tm,
                               std::vector<uint8_t> &out) {
    check_lorenzo3(dims, bs, pd, lo, lo2, reg, radius);
    LorArgs a = make_args<T>(dims, bs, pd, lo, lo2, eb, radius, reg);
    const uint64_t n = dims[0] * dims[1] * dims[2];
    const uint64_t nb = (uint64_t)(a.nx * a.ny * a.nz);
    DevMem m(st);
    T *R = m.alloc<T>(n);
    T *scratch = m.alloc<T>(n);
    // 16-bit codes, or 32-bit ones for more than 65536 quantisation bins
    const bool wide = radius > 32768;
    uint16_t *codes16 = wide ? nullptr : m.alloc<uint16_t>(n);
    uint32_t *codes32 = wide ? m.alloc<uint32_t>(n) : nullptr;
    uint16_t *ind = m.alloc<uint16_t>(nb);
    unsigned long long *vcount = nullptr;
    if (verify_fast_path()) {
        vcount = m.alloc<unsigned long long>(1);
        CK(cudaMemsetAsync(vcount, 0, 8, st));
        a.q.verify = vcount;
    }
    Events ev_pred, ev_huff;
    CK(cudaEventRecord(ev_pred.a, st));
    float *raw = reg ? m.alloc<float>(4 * nb) : nullptr;
    k_lor_select<T><<<(unsigned)((nb + 255) / 256), 256, 0, st>>>(a, dX, ind, raw);
    launches(cudaGetLastError());
    // regression coefficients: the serial chain on the host, then the
    // reconstructed coefficients back to the device for the wavefront
    std::vector<uint16_t> rtypes;
    std::vector<float> runp;
    uint64_t reg_count = 0;
    uint16_t *drtypes = nullptr;
    if (reg) {
        std::vector<uint16_t> hind(nb);
        std::vector<float> hraw(4 * nb), rec;
        CK(cudaMemcpyAsync(hind.data(), ind, nb * 2, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(hraw.data(), raw, nb * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        auto th = clk::now();
        reg_chain_compress<T>(hind, hraw, bs, eb, rec, rtypes, runp);
        reg_count = rtypes.size() / 4;
        tm.host_ms += ms_since(th);
        float *drec = m.alloc<float>(4 * nb);
        CK(cudaMemcpyAsync(drec, rec.data(), nb * 16, cudaMemcpyHostToDevice, st));
        a.rp = drec;
        if (reg_count) {
            drtypes = m.alloc<uint16_t>(rtypes.size());
            CK(cudaMemcpyAsync(drtypes, rtypes.data(), rtypes.size() * 2, cudaMemcpyHostToDevice, st));
        }
        CK(cudaStreamSynchronize(st));  // host vectors leave scope
    }
    // the predictor selections (and regression types) are final before the
    // wavefront: their Huffman stages run on a second stream meanwhile
    Events ev_sel, ev_side;
    CK(cudaEventRecord(ev_sel.a, st));
    StreamGuard side(nullptr, true);
    CK(cudaStreamWaitEvent(side.st, ev_sel.a, 0));
    DevMem m2(side.st);
    trace_step("lorenzo wavefront queued");
    const int *herr =
        wide ? launch_wavefront<T>(a, false, dX, R, codes32, scratch, ind, nullptr, 0, nullptr, st, launches)
             : launch_wavefront<T>(a, false, dX, R, codes16, scratch, ind, nullptr, 0, nullptr, st, launches);
    CK(cudaEventRecord(ev_pred.b, st));
    HuffEncoded hi, hc, hr;
    huffman_encode_device(ind, nb, 0, m2, side.st, launches, hi, tm);
    if (reg_count) huffman_encode_device(drtypes, rtypes.size(), 32768, m2, side.st, launches, hr, tm);
    CK(cudaEventRecord(ev_side.a, side.st));
    CK(cudaStreamWaitEvent(st, ev_side.a, 0));
    CK(cudaStreamSynchronize(st));
    check_wavefront(herr);
    trace_step("lorenzo wavefront done");
    CK(cudaEventRecord(ev_huff.a, st));
    if (wide) huffman_encode_device(codes32, n, radius, m, st, launches, hc, tm);
    else huffman_encode_device(codes16, n, radius, m, st, launches, hc, tm);
    if (vcount) {
        unsigned long long vc = 0;
        CK(cudaMemcpy(&vc, vcount, 8, cudaMemcpyDeviceToHost));
        if (vc) throw Fail{FAZ_ERR_DEVICE, "float fast path disagreed with the double path at " + std::to_string(vc) + " points"};
    }
    const uint64_t nunpred = hc.nzero;
    T *unp = m.alloc<T>(nunpred ? nunpred : 1);
    if (nunpred && wide) launches(launch_compact_zeros<T>(codes32, n, hc.zc, hc.zoff, nullptr, scratch, unp, st));
    if (nunpred && !wide) launches(launch_compact_zeros<T>(codes16, n, hc.zc, hc.zoff, nullptr, scratch, unp, st));
    CK(cudaEventRecord(ev_huff.b, st));
    trace_step("lorenzo codebooks built");
    // SZFastFrontend::save: params, precision, meanInfo<T>{false, 0}, reg_count,
    // indicator tree + bits; LinearQuantizer::save; then the code tree + bits
    std::vector<uint8_t> h0;
    put_meta_params(h0, bs, pd, lo, lo2, reg, eb);
    put<double>(h0, eb);
    for (size_t i = 0; i < 2 * sizeof(T); i++) h0.push_back(0);
    put<uint64_t>(h0, reg_count);
    append_tree(h0, hi.cb, hi.nbytes);
    // encode_regression_coefficients (MetaRegressionPredictor.hpp:82-95)
    std::vector<uint8_t> hreg;
    if (reg_count) {
        put<uint64_t>(hreg, runp.size());
        const uint8_t *u = reinterpret_cast<const uint8_t *>(runp.data());
        hreg.insert(hreg.end(), u, u + runp.size() * 4);
        append_tree(hreg, hr.cb, hr.nbytes);
    }
    std::vector<uint8_t> h1;
    put<uint8_t>(h1, 2);
    put<double>(h1, eb);
    put<int32_t>(h1, radius);
    put<uint64_t>(h1, nunpred);
    std::vector<uint8_t> h2;
    append_tree(h2, hc.cb, hc.nbytes);
    const size_t rbits = reg_count ? hr.nbytes : 0;
    const size_t total =
        h0.size() + hi.nbytes + hreg.size() + rbits + h1.size() + nunpred * sizeof(T) + h2.size() + hc.nbytes;
    // device parts come back through the thread's pinned staging buffer
    // (copies to pageable memory serialise with other threads' copies)
    uint8_t *pin = t_pin_payload.get(total + 8);
    uint8_t *p = pin;
    std::memcpy(p, h0.data(), h0.size());
    p += h0.size();
    if (hi.nbytes) CK(cudaMemcpyAsync(p, hi.bits, hi.nbytes, cudaMemcpyDeviceToHost, st));
    p += hi.nbytes;
    if (!hreg.empty()) std::memcpy(p, hreg.data(), hreg.size());
    p += hreg.size();
    if (rbits) CK(cudaMemcpyAsync(p, hr.bits, rbits, cudaMemcpyDeviceToHost, st));
    p += rbits;
    std::memcpy(p, h1.data(), h1.size());
    p += h1.size();
    if (nunpred) CK(cudaMemcpyAsync(p, unp, nunpred * sizeof(T), cudaMemcpyDeviceToHost, st));
    p += nunpred * sizeof(T);
    std::memcpy(p, h2.data(), h2.size());
    p += h2.size();
    if (hc.nbytes) CK(cudaMemcpyAsync(p, hc.bits, hc.nbytes, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    emit_payload(out, pin, total);
    tm.unpred_count = nunpred;
    tm.payload_bytes = total;
    tm.predict_ms += ev_pred.ms();
    tm.huffman_ms += ev_huff.ms();
}

// SZ_decompress_LorenzoReg for 3-D data (SZLorenzoReg.hpp:117-135):
// SZFastFrontend::load + decompress_3d into dOut (device, dims[0]*dims[1]*dims[2] values).
template <typename T>
void lorenzo3_decompress(const uint8_t *pl, size_t psize, const uint64_t *dims, T *dOut, cudaStream_t st,
                         Counter &launches, faz_timings &tm) {
    const uint8_t *p = pl, *end = pl + psize;
    auto need = [&](size_t k) {
        if ((size_t)(end - p) < k) throw Fail{FAZ_ERR_FORMAT, "truncated Lorenzo stream"};
    };
    need(44);
    int32_t bs, pd;
    std::memcpy(&bs, p, 4);
    std::memcpy(&pd, p + 4, 4);
    const int lo = p[8], lo2 = p[9], reg = p[10];
    float eb_ind, eb_lin;  // meta_params regression_param_eb_independent / _linear
    std::memcpy(&eb_ind, p + 20, 4);
    std::memcpy(&eb_lin, p + 24, 4);
    p += 44;
    need(8 + 2 * sizeof(T) + 8);
    p += 8;  // precision
    p += 2 * sizeof(T);  // meanInfo<T>
    uint64_t reg_count;
    std::memcpy(&reg_count, p, 8);
    p += 8;
    if (bs < 1 || bs > kLorMaxBs) throw Fail{FAZ_ERR_UNSUPPORTED, "Lorenzo block size must be 1..8 on the GPU path"};
    if (pd < 1 || pd > 3) throw Fail{FAZ_ERR_FORMAT, "bad pred_dim"};
    (void)lo;
    (void)lo2;
    (void)reg;
    const uint64_t n = dims[0] * dims[1] * dims[2];
    DevMem m(st);
    LorArgs a0 = make_args<T>(dims, bs, pd, 1, 1, 1.0, 1);
    const uint64_t nb = (uint64_t)(a0.nx * a0.ny * a0.nz);
    uint16_t *ind = m.alloc<uint16_t>(nb);
    Events ev_dec, ev_pred;
    CK(cudaEventRecord(ev_dec.a, st));
    huffman_decode_device(p, end, nb, ind, m, st, launches);
    if (reg_count > nb) throw Fail{FAZ_ERR_FORMAT, "bad regression block count"};
    float *drec = nullptr;
    if (reg_count) {
        // decode_regression_coefficients (MetaRegressionPredictor.hpp:42-80)
        need(8);
        uint64_t nrunp;
        std::memcpy(&nrunp, p, 8);
        p += 8;
        if ((size_t)(end - p) / 4 < nrunp) throw Fail{FAZ_ERR_FORMAT, "truncated regression coefficients"};
        const float *runp = reinterpret_cast<const float *>(p);
        p += nrunp * 4;
        uint16_t *dtypes = m.alloc<uint16_t>(4 * reg_count);
        huffman_decode_device(p, end, 4 * reg_count, dtypes, m, st, launches);
        std::vector<uint16_t> hind(nb), htypes(4 * reg_count);
        CK(cudaMemcpyAsync(hind.data(), ind, nb * 2, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(htypes.data(), dtypes, htypes.size() * 2, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        uint64_t nreg = 0;
        for (uint16_t v : hind) nreg += v == 1;
        if (nreg != reg_count) throw Fail{FAZ_ERR_FORMAT, "regression block count does not match the indicators"};
        std::vector<float> rec;
        reg_chain_decompress<T>(hind, htypes, runp, nrunp, eb_lin, eb_ind, rec);
        drec = m.alloc<float>(4 * nb);
        CK(cudaMemcpyAsync(drec, rec.data(), nb * 16, cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));
    }
    need(1 + 8 + 4 + 8);
    p += 1;
    double eb;
    std::memcpy(&eb, p, 8);
    p += 8;
    int32_t radius;
    std::memcpy(&radius, p, 4);
    p += 4;
    uint64_t nunpred;
    std::memcpy(&nunpred, p, 8);
    p += 8;
    if (!(eb > 0)) throw Fail{FAZ_ERR_FORMAT, "bad error bound"};
    if (radius < 1 || radius > kLorMaxRadius)
        throw Fail{FAZ_ERR_UNSUPPORTED, "quantbinCnt above 131072 is not implemented on the GPU path"};
    if ((size_t)(end - p) / sizeof(T) < nunpred) throw Fail{FAZ_ERR_FORMAT, "truncated unpredictable values"};
    T *dunp = m.alloc<T>(nunpred ? nunpred : 1);
    if (nunpred) CK(cudaMemcpyAsync(dunp, p, nunpred * sizeof(T), cudaMemcpyHostToDevice, st));
    p += nunpred * sizeof(T);
    const bool wide = radius > 32768;  // 32-bit codes for more than 65536 bins
    uint16_t *codes16 = wide ? nullptr : m.alloc<uint16_t>(n);
    uint32_t *codes32 = wide ? m.alloc<uint32_t>(n) : nullptr;
    uint64_t *zpos = nullptr;
    uint64_t nz;
    if (wide) {
        huffman_decode_device(p, end, n, codes32, m, st, launches);
        nz = zero_positions(codes32, n, m, st, launches, zpos);
    } else {
        huffman_decode_device(p, end, n, codes16, m, st, launches);
        nz = zero_positions(codes16, n, m, st, launches, zpos);
    }
    if (nz != nunpred) throw Fail{FAZ_ERR_FORMAT, "unpredictable count does not match the zero codes"};
    CK(cudaEventRecord(ev_dec.b, st));
    LorArgs a = make_args<T>(dims, bs, pd, 1, 1, eb, radius);
    a.rp = drec;
    unsigned long long *vcount = nullptr;
    if (verify_fast_path()) {
        vcount = m.alloc<unsigned long long>(1);
        CK(cudaMemsetAsync(vcount, 0, 8, st));
        a.q.verify = vcount;
    }
    CK(cudaEventRecord(ev_pred.a, st));
    if (wide) run_wavefront<T>(a, true, nullptr, dOut, codes32, nullptr, ind, zpos, nz, dunp, st, launches);
    else run_wavefront<T>(a, true, nullptr, dOut, codes16, nullptr, ind, zpos, nz, dunp, st, launches);
    CK(cudaEventRecord(ev_pred.b, st));
    CK(cudaStreamSynchronize(st));
    if (vcount) {
        unsigned long long vc = 0;
        CK(cudaMemcpy(&vc, vcount, 8, cudaMemcpyDeviceToHost));
        if (vc) throw Fail{FAZ_ERR_DEVICE, "float fast path disagreed with the double path at " + std::to_string(vc) + " points"};
    }
    tm.huffman_ms += ev_dec.ms();
    tm.predict_ms += ev_pred.ms();
}

template void lorenzo3_compress_payload<float>(const uint64_t *, int, int, int, int, int, double, int, const float *,
                                               cudaStream_t, Counter &, faz_timings &, std::vector<uint8_t> &);
template void lorenzo3_compress_payload<double>(const uint64_t *, int, int, int, int, int, double, int,
                                                const double *, cudaStream_t, Counter &, faz_timings &,
                                                std::vector<uint8_t> &);
template void lorenzo3_decompress<float>(const uint8_t *, size_t, const uint64_t *, float *, cudaStream_t, Counter &,
                                         faz_timings &);
template void lorenzo3_decompress<double>(const uint8_t *, size_t, const uint64_t *, double *, cudaStream_t,
                                          Counter &, faz_timings &);

}  // namespace faz
