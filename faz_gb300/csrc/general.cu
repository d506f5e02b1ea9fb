// general.cu - the general frontend for 1-D and 2-D fields
// (SZ_compress_LorenzoReg / SZ_decompress_LorenzoReg with N < 3,
// include/QoZ/api/impl/SZLorenzoReg.hpp:28-135): SZGeneralFrontend
// (include/QoZ/frontend/SZGeneralFrontend.hpp:19-150) with the one- and
// two-layer Lorenzo predictors (include/QoZ/predictor/LorenzoPredictor.hpp)
// and the linear-regression predictor
// (include/QoZ/predictor/RegressionPredictor.hpp), combined by
// ComposedPredictor (include/QoZ/predictor/ComposedPredictor.hpp) when more
// than one is enabled.
//
// The reference walks blocks in row-major order and, inside a block, points
// in row-major order; each point is predicted from reconstructed values
// (zero outside the field) and overwritten by its reconstruction.  A block's
// predictor is chosen from estimates taken on the current data: original
// values inside the block, reconstructed ones before it.
//
// Without regression, a 2-D block only reads the blocks above, to the left and
// above-left, so blocks on one anti-diagonal are independent: one launch per
// block diagonal, one warp per block, a shared-memory tile with a 2-deep halo
// of reconstructed values; inside a block the points of one anti-diagonal are
// independent as well.  In 1-D every point depends on the one before it; one
// thread walks the field.
//
// Regression adds a chain in block order: each regression block's
// coefficients are quantised against the previous regression block's
// reconstructed ones, and the reconstruction they give feeds the neighbours'
// Lorenzo estimates, so which block is the previous regression block depends
// on every selection before it in row-major order.  Compression with
// regression therefore walks the 2-D blocks in row-major order in one warp
// (tile halo from the previous tile and a two-row band of the block row
// above); the least-squares fits and regression estimates, which read only
// original values, run beforehand for all blocks at once.  Decompression
// knows every selection from the stream: one thread replays the coefficient
// chain, then the anti-diagonal wavefront reconstructs.
#include <cuda_runtime.h>

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

constexpr int kGenWarps = 8;   // blocks (warps) per CTA in 2-D
constexpr int kGenMaxBs = 64;  // largest 2-D block edge on the GPU path
constexpr int kCoefRadius = 32768;  // RegressionPredictor's LinearQuantizer radius

struct GenArgs {
    int64_t d0, d1;    // field extents (1-D: d1 = 1)
    int64_t nb0, nb1;  // blocks per axis
    int N;
    int bs;
    int np;            // predictors in the list
    int kinds[3];      // list order: 1 Lorenzo, 2 two-layer Lorenzo, 3 regression
    double noise1, noise2;  // LorenzoPredictor(eb) noise for L = 1, 2
    double eb_ind, eb_lin;  // coefficient quantisers: eb / (N + 1), eb / (N + 1) / blockSize
    int cradius_ind, cradius_lin;  // their radii
    LevelArgs q;       // quantiser
};

// T-typed arithmetic, each operation rounded on its own
template <typename T> __device__ __forceinline__ T t_add(T a, T b) {
    if constexpr (sizeof(T) == 4) return __fadd_rn(a, b); else return __dadd_rn(a, b);
}
template <typename T> __device__ __forceinline__ T t_sub(T a, T b) {
    if constexpr (sizeof(T) == 4) return __fsub_rn(a, b); else return __dsub_rn(a, b);
}
template <typename T> __device__ __forceinline__ T t_mul(T a, T b) {
    if constexpr (sizeof(T) == 4) return __fmul_rn(a, b); else return __dmul_rn(a, b);
}

// RegressionPredictor::predict (RegressionPredictor.hpp:94-101) at the
// block-local index (li, lj): 0 + li*c0 (+ lj*c1) + cN, in T
template <typename T>
__device__ __forceinline__ T reg_pred(const T *c, int N, int li, int lj) {
    T p = t_add<T>((T)0, t_mul<T>((T)li, c[0]));
    if (N == 2) p = t_add<T>(p, t_mul<T>((T)lj, c[1]));
    return t_add<T>(p, c[N]);
}

// RegressionPredictor::precompress_block (RegressionPredictor.hpp:48-87): the
// least-squares plane of the block (rows i0.., columns j0.. of a field with
// row length d1), sums in double in the reference's order; false for a block
// with an extent of 1.
template <typename T>
__device__ bool reg_fit(const T *X, int64_t d1, int N, int64_t i0, int64_t j0, int sx, int sy, T *c) {
    if (sx <= 1 || (N == 2 && sy <= 1)) return false;
    const int64_t num = N == 2 ? (int64_t)sx * sy : sx;
    const T recip = (T)(1.0 / (double)num);
    double sum[3] = {0, 0, 0};
    if (N == 1) {
        double cum = 0;
        for (int t = 0; t < sx; t++) {
            const double v = (double)X[i0 + t];
            cum = __dadd_rn(cum, v);
            sum[0] = __dadd_rn(sum[0], __dmul_rn((double)t, v));
        }
        sum[1] = __dadd_rn(sum[1], cum);
    } else {
        for (int r = 0; r < sx; r++) {
            const T *row = X + (i0 + r) * d1 + j0;
            double cum = 0;
            for (int t = 0; t < sy; t++) {
                const double v = (double)row[t];
                cum = __dadd_rn(cum, v);
                sum[1] = __dadd_rn(sum[1], __dmul_rn((double)t, v));
            }
            sum[0] = __dadd_rn(sum[0], __dmul_rn(cum, (double)r));
            sum[2] = __dadd_rn(sum[2], cum);
        }
    }
    c[N] = (T)__dmul_rn(sum[N], (double)recip);
    for (int i = 0; i < N; i++) {
        const int di = i == 0 ? sx : sy;
        double v = __ddiv_rn(__dmul_rn(2.0, sum[i]), (double)(di - 1));
        v = __dmul_rn(__dsub_rn(v, sum[N]), 6.0);
        v = __ddiv_rn(__dmul_rn(v, (double)recip), (double)(di + 1));
        c[i] = (T)v;
        // cN -= (di - 1) * ci / 2, in T
        c[N] = t_sub<T>(c[N], t_mul<T>(t_mul<T>((T)(di - 1), c[i]), (T)0.5));
    }
    if (N == 1) c[2] = 0;
    return true;
}

// Fits of every block at once (they read original values only): the
// coefficients, whether the block admits regression, and for 2-D the
// regression predictor's selection estimate (no noise term) along the block's
// two diagonals (ComposedPredictor.hpp:204-218).
template <typename T>
__global__ void k_gen_fit(GenArgs a, const T *__restrict__ X, T *__restrict__ fit, uint8_t *__restrict__ fit_ok,
                          double *__restrict__ ereg) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= a.nb0 * a.nb1) return;
    const int64_t bi = b / a.nb1, bj = b - bi * a.nb1;
    const int64_t i0 = bi * a.bs, j0 = bj * a.bs;
    const int sx = i0 + a.bs < a.d0 ? a.bs : (int)(a.d0 - i0);
    const int sy = a.N == 2 ? (j0 + a.bs < a.d1 ? a.bs : (int)(a.d1 - j0)) : 1;
    T c[3] = {0, 0, 0};
    const bool ok = reg_fit<T>(X, a.d1, a.N, i0, j0, sx, sy, c);
    for (int i = 0; i < 3; i++) fit[3 * b + i] = c[i];
    fit_ok[b] = ok ? 1 : 0;
    if (a.N == 2 && ereg) {
        const int m = sx < sy ? sx : sy;
        double e = 0;
        for (int t = 0; t + 2 < m; t++) {
            const T v1 = X[(i0 + t) * a.d1 + j0 + t], v2 = X[(i0 + t) * a.d1 + j0 + (m - 1 - t)];
            e = __dadd_rn(e, (double)fabs((double)t_sub<T>(v1, reg_pred<T>(c, 2, t, t))));
            e = __dadd_rn(e, (double)fabs((double)t_sub<T>(v2, reg_pred<T>(c, 2, t, m - 1 - t))));
        }
        ereg[b] = e;
    }
}

// LorenzoPredictor<T, 2, L>::do_predict on a tile with row stride ty
template <typename T>
__device__ __forceinline__ T gen2_pred(const T *p, int ty, int L) {
    if (L == 1) return p[-1] + p[-ty] - p[-ty - 1];
    return 2 * p[-1] - p[-2] + 2 * p[-ty] - 4 * p[-ty - 1] + 2 * p[-ty - 2] - p[-2 * ty] + 2 * p[-2 * ty - 1] -
           p[-2 * ty - 2];
}

// estimate_error: fabs(*iter - predict(iter)) + noise, as T
template <typename T>
__device__ __forceinline__ T gen2_est(const T *p, int ty, int L, T noise) {
    const T d = *p - gen2_pred(p, ty, L);
    return (T)(fabs((double)d) + (double)noise);
}

// Sweep of one block's anti-diagonals with Lorenzo predictor L (one warp);
// t points at the tile, whose interior starts at row 2, column 2.
template <typename T, bool DECOMP, int QM>
__device__ __forceinline__ void gen2_sweep(const GenArgs &a, T *t, int ty, int sx, int sy, int L, uint64_t boff,
                                           int lane, uint16_t *codes, T *scratch, const uint64_t *zpos, uint64_t nzp,
                                           const T *unpred) {
    for (int s = 0; s < sx + sy - 1; s++) {
        for (int i = lane; i < sx; i += 32) {
            const int j = s - i;
            if (j < 0 || j >= sy) continue;
            T *c = t + (i + 2) * ty + (j + 2);
            const T pred = gen2_pred(c, ty, L);
            const uint64_t pos = boff + (uint64_t)(i * sy + j);
            if (!DECOMP) {
                T v = *c, uval;
                const int code = quant_point<T, QM>(v, pred, a.q, uval);
                codes[pos] = (uint16_t)code;
                if (code == 0) scratch[pos] = uval;
                *c = v;
            } else {
                *c = recover_point<T, QM>(pred, (int)codes[pos], pos, a.q, zpos, nzp, unpred);
            }
        }
        __syncwarp();
    }
}

// One regression block: every point independent of the others.
template <typename T, bool DECOMP, int QM>
__device__ __forceinline__ void gen2_reg_block(const GenArgs &a, T *t, int ty, int sx, int sy, const T *coef,
                                               uint64_t boff, int lane, uint16_t *codes, T *scratch,
                                               const uint64_t *zpos, uint64_t nzp, const T *unpred) {
    for (int e = lane; e < sx * sy; e += 32) {
        const int i = e / sy, j = e - i * sy;
        T *c = t + (i + 2) * ty + (j + 2);
        const T pred = reg_pred<T>(coef, 2, i, j);
        const uint64_t pos = boff + (uint64_t)e;
        if (!DECOMP) {
            T v = *c, uval;
            const int code = quant_point<T, QM>(v, pred, a.q, uval);
            codes[pos] = (uint16_t)code;
            if (code == 0) scratch[pos] = uval;
            *c = v;
        } else {
            *c = recover_point<T, QM>(pred, (int)codes[pos], pos, a.q, zpos, nzp, unpred);
        }
    }
    __syncwarp();
}

// One block diagonal bi + bj = d; one warp per block.  Compressing (Lorenzo
// predictors only), the warp chooses the block's predictor; decompressing,
// kind / coef hold every block's predictor and reconstructed coefficients.
template <typename T, bool DECOMP, int QM>
__global__ void __launch_bounds__(kGenWarps * 32)
    k_gen2_diag(GenArgs a, int64_t d, int64_t bi_lo, const T *__restrict__ X, T *__restrict__ R,
                uint16_t *__restrict__ codes, T *__restrict__ scratch, uint16_t *__restrict__ sel,
                const uint8_t *__restrict__ kind, const T *__restrict__ coef, const uint64_t *__restrict__ zpos,
                uint64_t nzp, const T *__restrict__ unpred) {
    extern __shared__ __align__(16) unsigned char gen_smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t bi = bi_lo + (int64_t)blockIdx.x * kGenWarps + w;
    const int64_t bj = d - bi;
    if (bi >= a.nb0 || bj < 0 || bj >= a.nb1) return;
    const int bs = a.bs;
    const int sx = (bi + 1) * bs < a.d0 ? bs : (int)(a.d0 - bi * bs);
    const int sy = (bj + 1) * bs < a.d1 ? bs : (int)(a.d1 - bj * bs);
    const int64_t i0 = bi * bs, j0 = bj * bs;
    const int ty = sy + 2;
    T *t = reinterpret_cast<T *>(gen_smem) + (size_t)w * (size_t)((bs + 2) * (bs + 2));
    const int tn = (sx + 2) * ty;
    // tile: reconstructed halo (zero outside the field) and, compressing, the
    // block's original values
    for (int e = lane; e < tn; e += 32) {
        const int i = e / ty, j = e - i * ty;
        const int64_t gi = i0 + i - 2, gj = j0 + j - 2;
        T v = 0;
        if (i >= 2 && j >= 2) {
            if (!DECOMP) v = X[gi * a.d1 + gj];
        } else if (gi >= 0 && gj >= 0) {
            v = R[gi * a.d1 + gj];
        }
        t[e] = v;
    }
    __syncwarp();
    const int64_t b = bi * a.nb1 + bj;
    const uint64_t boff = (uint64_t)i0 * (uint64_t)a.d1 + (uint64_t)j0 * (uint64_t)sx;
    int L;
    if (DECOMP) {
        L = kind[b];
    } else if (a.np == 2) {
        // ComposedPredictor::precompress_block: estimates along the two
        // diagonals of the block's leading square, summed in order
        int s = 0;
        if (lane == 0) {
            const int m = sx < sy ? sx : sy;
            const T n1 = (T)a.noise1, n2 = (T)a.noise2;
            double e1 = 0, e2 = 0;
            for (int k = 0; k + 2 < m; k++) {
                const T *p1 = t + (k + 2) * ty + (k + 2);
                const T *p2 = t + (k + 2) * ty + (m - 1 - k + 2);
                e1 += (double)gen2_est(p1, ty, 1, n1);
                e1 += (double)gen2_est(p2, ty, 1, n1);
                e2 += (double)gen2_est(p1, ty, 2, n2);
                e2 += (double)gen2_est(p2, ty, 2, n2);
            }
            s = e2 < e1 ? 1 : 0;
            sel[b] = (uint16_t)s;
        }
        L = __shfl_sync(0xffffffffu, s, 0) + 1;
    } else {
        L = a.kinds[0];
    }
    if (DECOMP && L == 3)
        gen2_reg_block<T, DECOMP, QM>(a, t, ty, sx, sy, coef + 3 * b, boff, lane, codes, scratch, zpos, nzp, unpred);
    else
        gen2_sweep<T, DECOMP, QM>(a, t, ty, sx, sy, L, boff, lane, codes, scratch, zpos, nzp, unpred);
    for (int e = lane; e < sx * sy; e += 32) {
        const int i = e / sy, j = e - i * sy;
        R[(i0 + i) * a.d1 + (j0 + j)] = t[(i + 2) * ty + (j + 2)];
    }
}

// Coefficient chain of one committed regression block, compressing
// (pred_and_quantize_coefficients, RegressionPredictor.hpp:225-231): the N
// linear terms, then the independent term, each predicted by the previous
// committed block's; prev receives the reconstruction.  Codes and
// unpredictable values are appended in commit order.
template <typename T>
__device__ void reg_commit(const GenArgs &a, const T *fit, T *prev, uint16_t *ccodes, uint64_t &ncc, T *cunp_lin,
                           uint64_t &nul, T *cunp_ind, uint64_t &nui) {
    for (int i = 0; i <= a.N; i++) {
        const bool lin = i < a.N;
        const double eb = lin ? a.eb_lin : a.eb_ind;
        T v = fit[i], uval;
        const int code = quantize<T>(v, prev[i], eb, 1.0 / eb, lin ? a.cradius_lin : a.cradius_ind, 0, uval);
        ccodes[ncc++] = (uint16_t)code;
        if (code == 0) {
            if (lin) cunp_lin[nul++] = uval;
            else cunp_ind[nui++] = uval;
        }
        prev[i] = v;
    }
}

// pred_and_recover_coefficients (RegressionPredictor.hpp:233-243); false when
// the stream runs out of codes or unpredictable values.
template <typename T>
__device__ bool reg_recover(const GenArgs &a, T *cur, const uint16_t *ccodes, uint64_t ncc, uint64_t &ic,
                            const T *cunp_lin, uint64_t nul, uint64_t &iul, const T *cunp_ind, uint64_t nui,
                            uint64_t &iui) {
    if (ic + a.N + 1 > ncc) return false;
    for (int i = 0; i <= a.N; i++) {
        const bool lin = i < a.N;
        const int code = ccodes[ic++];
        if (code == 0) {
            if (lin ? iul >= nul : iui >= nui) return false;
            cur[i] = lin ? cunp_lin[iul++] : cunp_ind[iui++];
        } else {
            const double eb = lin ? a.eb_lin : a.eb_ind;
            const int r = lin ? a.cradius_lin : a.cradius_ind;
            cur[i] = (T)((double)cur[i] + (double)(2 * (code - r)) * eb);
        }
    }
    return true;
}

// Compression of a 2-D field with regression in the list: one warp walks
// the blocks in row-major order.  The tile's left halo comes from the
// previous tile (same block row), its top halo from a band holding the last
// two reconstructed rows of the block row above (two bands, alternating).
// counts: selections, coefficient codes, linear / independent unpredictables.
template <typename T, int QM>
__global__ void __launch_bounds__(32, 1)
    k_gen2_seq(GenArgs a, const T *__restrict__ X, T *__restrict__ band, uint16_t *__restrict__ codes,
               T *__restrict__ scratch, uint16_t *__restrict__ sel, const T *__restrict__ fit,
               const uint8_t *__restrict__ fit_ok, const double *__restrict__ ereg, uint16_t *__restrict__ ccodes,
               T *__restrict__ cunp_lin, T *__restrict__ cunp_ind, unsigned long long *__restrict__ counts) {
    extern __shared__ __align__(16) unsigned char gen_smem[];
    const int lane = threadIdx.x & 31;
    const int bs = a.bs, tile = (bs + 2) * (bs + 2);
    T *tiles = reinterpret_cast<T *>(gen_smem);
    double *est = reinterpret_cast<double *>(gen_smem + (((size_t)2 * tile * sizeof(T) + 15) & ~(size_t)15));
    __shared__ T s_coef[3];
    __shared__ int s_kind;
    const bool composed = a.np > 1;
    const int nterm_max = 2 * (bs - 2);
    // lane 0's state: the previous committed coefficients and the counts
    T prev[3] = {0, 0, 0};
    uint64_t ns = 0, ncc = 0, nul = 0, nui = 0;
    int cur = 0, prev_sy = 0;
    for (int64_t bi = 0; bi < a.nb0; bi++) {
        const int sx = (bi + 1) * bs < a.d0 ? bs : (int)(a.d0 - bi * bs);
        const int64_t i0 = bi * bs;
        const T *bup = band + (size_t)((bi - 1) & 1) * 2 * (size_t)a.d1;
        for (int64_t bj = 0; bj < a.nb1; bj++) {
            const int sy = (bj + 1) * bs < a.d1 ? bs : (int)(a.d1 - bj * bs);
            const int64_t j0 = bj * bs, b = bi * a.nb1 + bj;
            const int ty = sy + 2, tn = (sx + 2) * ty;
            T *t = tiles + (size_t)cur * tile;
            const T *tp = tiles + (size_t)(cur ^ 1) * tile;
            const int typ = prev_sy + 2;
            for (int e = lane; e < tn; e += 32) {
                const int i = e / ty, j = e - i * ty;
                const int64_t gi = i0 + i - 2, gj = j0 + j - 2;
                T v = 0;
                if (i >= 2 && j >= 2) v = X[gi * a.d1 + gj];
                else if (gi < 0 || gj < 0) v = 0;
                else if (i < 2) v = bup[(size_t)i * a.d1 + gj];
                else v = tp[i * typ + prev_sy + j];
                t[e] = v;
            }
            __syncwarp();
            const uint64_t boff = (uint64_t)i0 * (uint64_t)a.d1 + (uint64_t)j0 * (uint64_t)sx;
            // ComposedPredictor::precompress_block: each Lorenzo predictor's
            // estimates along the two diagonals of the leading square, summed
            // in order; regression's from the fits
            int sid = 0;
            if (composed) {
                const int m = sx < sy ? sx : sy, nt = m - 2;
                const T n1 = (T)a.noise1, n2 = (T)a.noise2;
                for (int k = lane; k < nt; k += 32) {
                    const T *p1 = t + (k + 2) * ty + (k + 2);
                    const T *p2 = t + (k + 2) * ty + (m - 1 - k + 2);
                    for (int p = 0; p < a.np; p++) {
                        const int L = a.kinds[p];
                        if (L == 3) continue;
                        est[p * nterm_max + 2 * k] = (double)gen2_est(p1, ty, L, L == 1 ? n1 : n2);
                        est[p * nterm_max + 2 * k + 1] = (double)gen2_est(p2, ty, L, L == 1 ? n1 : n2);
                    }
                }
                __syncwarp();
                double e = 0;
                if (lane < a.np) {
                    if (a.kinds[lane] == 3) {
                        e = ereg[b];
                    } else {
                        for (int u = 0; u < 2 * nt; u++) e += est[lane * nterm_max + u];
                    }
                }
                double best = __shfl_sync(0xffffffffu, e, 0);
                for (int p = 1; p < a.np; p++) {
                    const double ep = __shfl_sync(0xffffffffu, e, p);
                    if (ep < best) {
                        best = ep;
                        sid = p;
                    }
                }
            }
            if (lane == 0) {
                int kind = a.kinds[sid];
                if (kind == 3 && !fit_ok[b]) {
                    kind = 1;  // SZGeneralFrontend's fallback LorenzoPredictor<T, N, 1>
                } else {
                    if (composed) sel[ns++] = (uint16_t)sid;
                    if (kind == 3) {
                        reg_commit<T>(a, fit + 3 * b, prev, ccodes, ncc, cunp_lin, nul, cunp_ind, nui);
                        for (int i = 0; i < 3; i++) s_coef[i] = prev[i];
                    }
                }
                s_kind = kind;
            }
            __syncwarp();
            const int kind = s_kind;
            if (kind == 3)
                gen2_reg_block<T, false, QM>(a, t, ty, sx, sy, s_coef, boff, lane, codes, scratch, nullptr, 0,
                                             nullptr);
            else
                gen2_sweep<T, false, QM>(a, t, ty, sx, sy, kind, boff, lane, codes, scratch, nullptr, 0, nullptr);
            // the block's last two rows for the block row below
            if (bi + 1 < a.nb0) {
                T *bdn = band + (size_t)(bi & 1) * 2 * (size_t)a.d1;
                for (int e = lane; e < 2 * sy; e += 32) {
                    const int r = e / sy, j = e - r * sy;
                    bdn[(size_t)r * a.d1 + j0 + j] = t[(sx + r) * ty + (j + 2)];
                }
            }
            __syncwarp();
            cur ^= 1;
            prev_sy = sy;
        }
    }
    if (lane == 0) {
        counts[0] = ns;
        counts[1] = ncc;
        counts[2] = nul;
        counts[3] = nui;
    }
}

// Decompression's coefficient chain for 2-D: each block's predictor (the
// composed predictor's selection, or the single predictor; regression's
// one-extent blocks and blocks past the end of the selections take the
// fallback) and each regression block's reconstructed coefficients.
template <typename T>
__global__ void k_gen_chain(GenArgs a, const uint16_t *__restrict__ sel, uint64_t ns,
                            const uint16_t *__restrict__ ccodes, uint64_t ncc, const T *__restrict__ cunp_lin,
                            uint64_t nul, const T *__restrict__ cunp_ind, uint64_t nui, uint8_t *__restrict__ kind,
                            T *__restrict__ coef, int *__restrict__ err) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    T cur[3] = {0, 0, 0};
    uint64_t is = 0, ic = 0, iul = 0, iui = 0;
    for (int64_t bi = 0; bi < a.nb0; bi++) {
        const int sx = (bi + 1) * a.bs < a.d0 ? a.bs : (int)(a.d0 - bi * a.bs);
        for (int64_t bj = 0; bj < a.nb1; bj++) {
            const int sy = (bj + 1) * a.bs < a.d1 ? a.bs : (int)(a.d1 - bj * a.bs);
            const int64_t b = bi * a.nb1 + bj;
            int k = a.kinds[0];
            if (a.np > 1) {
                if (is < ns) {
                    const int s = sel[is++];
                    if (s >= a.np) {
                        *err = 1;
                        return;
                    }
                    k = a.kinds[s];
                } else {
                    k = 1;
                }
            }
            if (k == 3 && (sx <= 1 || sy <= 1)) k = 1;
            if (k == 3 && !reg_recover<T>(a, cur, ccodes, ncc, ic, cunp_lin, nul, iul, cunp_ind, nui, iui)) {
                *err = 2;
                return;
            }
            kind[b] = (uint8_t)k;
            for (int i = 0; i < 3; i++) coef[3 * b + i] = k == 3 ? cur[i] : (T)0;
        }
    }
}

// 1-D: one thread walks the blocks and their points in order.  Compressing,
// it chooses each block's predictor and runs the coefficient chain;
// decompressing, it reads the selections and replays the chain.
template <typename T, bool DECOMP, int QM>
__global__ void k_gen1(GenArgs a, const T *__restrict__ X, T *__restrict__ R, uint16_t *__restrict__ codes,
                       T *__restrict__ scratch, uint16_t *__restrict__ sel, const T *__restrict__ fit,
                       const uint8_t *__restrict__ fit_ok, uint16_t *__restrict__ ccodes, T *__restrict__ cunp_lin,
                       T *__restrict__ cunp_ind, unsigned long long *__restrict__ counts,
                       const uint64_t *__restrict__ zpos, uint64_t nzp, const T *__restrict__ unpred,
                       int *__restrict__ err) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const int64_t n = a.d0;
    const T n1 = (T)a.noise1, n2 = (T)a.noise2;
    const bool composed = a.np > 1;
    T r1 = 0, r2 = 0;  // reconstructed values at i - 1, i - 2
    T cur[3] = {0, 0, 0}, prev[3] = {0, 0, 0};  // regression's current / last committed coefficients
    // compressing: counts produced; decompressing: counts given
    uint64_t ns = 0, ncc = 0, nul = 0, nui = 0;
    uint64_t is = 0, ic = 0, iul = 0, iui = 0;
    if (DECOMP) {
        ns = counts[0];
        ncc = counts[1];
        nul = counts[2];
        nui = counts[3];
    }
    for (int64_t bi = 0; bi < a.nb0; bi++) {
        const int64_t i0 = bi * a.bs;
        const int sx = (int)(i0 + a.bs < n ? a.bs : n - i0);
        int kind = a.kinds[0];
        if (!DECOMP) {
            bool reg_ok = true;
            if (a.kinds[a.np - 1] == 3) {
                reg_ok = fit_ok[bi] != 0;
                if (reg_ok)
                    for (int i = 0; i < 3; i++) cur[i] = fit[3 * bi + i];
            }
            int sid = 0;
            if (composed) {
                // estimates at the block's first and last point on the current
                // data (ComposedPredictor.hpp:192-202)
                auto at = [&](int64_t p) -> T {  // current value at p (p <= i0 + sx - 1)
                    if (p < 0) return (T)0;
                    if (p >= i0) return X[p];
                    return p == i0 - 1 ? r1 : (p == i0 - 2 ? r2 : R[p]);
                };
                const int64_t pa = i0, pb = i0 + sx - 1;
                double e[3];
                for (int p = 0; p < a.np; p++) {
                    const int L = a.kinds[p];
                    T ea, eb;
                    if (L == 1) {
                        ea = (T)(fabs((double)(at(pa) - at(pa - 1))) + (double)n1);
                        eb = (T)(fabs((double)(at(pb) - at(pb - 1))) + (double)n1);
                    } else if (L == 2) {
                        ea = (T)(fabs((double)(at(pa) - (2 * at(pa - 1) - at(pa - 2)))) + (double)n2);
                        eb = (T)(fabs((double)(at(pb) - (2 * at(pb - 1) - at(pb - 2)))) + (double)n2);
                    } else {
                        ea = (T)fabs((double)t_sub<T>(X[pa], reg_pred<T>(cur, 1, 0, 0)));
                        eb = (T)fabs((double)t_sub<T>(X[pb], reg_pred<T>(cur, 1, sx - 1, 0)));
                    }
                    e[p] = 0;
                    e[p] += (double)ea;
                    e[p] += (double)eb;
                }
                for (int p = 1; p < a.np; p++)
                    if (e[p] < e[sid]) sid = p;
            }
            kind = a.kinds[sid];
            if (kind == 3 && !reg_ok) {
                kind = 1;  // fallback LorenzoPredictor<T, 1, 1>; nothing recorded
            } else {
                if (composed) sel[ns++] = (uint16_t)sid;
                if (kind == 3) {
                    reg_commit<T>(a, cur, prev, ccodes, ncc, cunp_lin, nul, cunp_ind, nui);
                    for (int i = 0; i < 3; i++) cur[i] = prev[i];
                }
            }
        } else {
            if (composed) {
                if (is < ns) {
                    const int s = sel[is++];
                    if (s >= a.np) {
                        *err = 1;
                        return;
                    }
                    kind = a.kinds[s];
                } else {
                    kind = 1;
                }
            }
            if (kind == 3 && sx <= 1) kind = 1;
            if (kind == 3 && !reg_recover<T>(a, cur, ccodes, ncc, ic, cunp_lin, nul, iul, cunp_ind, nui, iui)) {
                *err = 2;
                return;
            }
        }
        for (int64_t i = i0; i < i0 + sx; i++) {
            const T pred = kind == 3 ? reg_pred<T>(cur, 1, (int)(i - i0), 0) : (kind == 1 ? r1 : 2 * r1 - r2);
            T v;
            if (!DECOMP) {
                v = X[i];
                T uval;
                const int code = quant_point<T, QM>(v, pred, a.q, uval);
                codes[i] = (uint16_t)code;
                if (code == 0) scratch[i] = uval;
            } else {
                v = recover_point<T, QM>(pred, (int)codes[i], (uint64_t)i, a.q, zpos, nzp, unpred);
            }
            R[i] = v;
            r2 = r1;
            r1 = v;
        }
    }
    if (!DECOMP) {
        counts[0] = ns;
        counts[1] = ncc;
        counts[2] = nul;
        counts[3] = nui;
    }
}

template <typename T>
GenArgs make_gen_args(int N, const uint64_t *dims, int bs, int lo, int lo2, int reg, double eb, int radius) {
    GenArgs a;
    std::memset(&a, 0, sizeof(a));
    a.N = N;
    a.d0 = (int64_t)dims[0];
    a.d1 = N == 2 ? (int64_t)dims[1] : 1;
    a.bs = bs;
    a.nb0 = (a.d0 - 1) / bs + 1;
    a.nb1 = N == 2 ? (a.d1 - 1) / bs + 1 : 1;
    a.np = 0;
    if (lo) a.kinds[a.np++] = 1;
    if (lo2) a.kinds[a.np++] = 2;
    if (reg) a.kinds[a.np++] = 3;
    a.noise1 = (N == 1 ? 0.5 : 0.81) * eb;
    a.noise2 = (N == 1 ? 1.08 : 2.76) * eb;
    // RegressionPredictor(block_size, eb) (RegressionPredictor.hpp:23-26)
    a.eb_ind = eb / (N + 1);
    a.eb_lin = eb / (N + 1) / bs;
    a.cradius_ind = a.cradius_lin = kCoefRadius;
    a.q.eb = eb;
    a.q.recip = 1.0 / eb;
    a.q.radius = radius;
    a.q.trim = 0;
    set_fast_path<T>(a.q);
    return a;
}

void check_gen(int N, int bs, int lo, int lo2, int reg, int radius) {
    if (N != 1 && N != 2) throw Fail{FAZ_ERR_ARG, "the general frontend here covers 1-D and 2-D data"};
    if (bs < 2) throw Fail{FAZ_ERR_UNSUPPORTED, "Lorenzo block size must be at least 2 on the GPU path"};
    if (N == 2 && bs > kGenMaxBs) throw Fail{FAZ_ERR_UNSUPPORTED, "2-D Lorenzo block size above 64 is not implemented"};
    if (!lo && !lo2 && !reg) throw Fail{FAZ_ERR_ARG, "all Lorenzo and regression methods are disabled"};
    if (radius < 1 || radius > 32768)
        throw Fail{FAZ_ERR_UNSUPPORTED, "quantbinCnt above 65536 is not implemented on the GPU path"};
}

// LinearQuantizer::save (IntegerQuantizer.hpp:185-205) header; the values follow
void put_quantizer_header(std::vector<uint8_t> &o, double eb, int radius, uint64_t nunpred) {
    put<uint8_t>(o, 2);
    put<double>(o, eb);
    put<int32_t>(o, radius);
    put<uint64_t>(o, nunpred);
}

}  // namespace

// SZGeneralFrontend::compress + save and the Huffman stage of the general
// compressor: the pre-zstd payload of a 1-D / 2-D field.
template <typename T>
void gen_compress_payload(int N, const uint64_t *dims, int bs, int lo, int lo2, int reg, double eb, int radius,
                          const T *dX, cudaStream_t st, Counter &launches, faz_timings &tm, std::vector<uint8_t> &out) {
    check_gen(N, bs, lo, lo2, reg, radius);
    const GenArgs a = make_gen_args<T>(N, dims, bs, lo, lo2, reg, eb, radius);
    const uint64_t n = (uint64_t)(a.d0 * a.d1), nb = (uint64_t)(a.nb0 * a.nb1);
    const bool composed = a.np > 1;
    const bool straight = sizeof(T) == 4 && a.q.fast;
    DevMem m(st);
    T *R = m.alloc<T>(n), *scratch = m.alloc<T>(n);
    uint16_t *codes = m.alloc<uint16_t>(n), *sel = m.alloc<uint16_t>(nb);
    // regression: fits, coefficient codes and unpredictables, counts
    T *fit = nullptr, *cunp = nullptr;
    uint8_t *fit_ok = nullptr;
    double *ereg = nullptr;
    uint16_t *ccodes = nullptr;
    unsigned long long *dcounts = m.alloc<unsigned long long>(4);
    CK(cudaMemsetAsync(dcounts, 0, 32, st));
    Events ev_pred, ev_huff;
    CK(cudaEventRecord(ev_pred.a, st));
    if (reg || N == 1) {
        fit = m.alloc<T>(3 * nb);
        fit_ok = m.alloc<uint8_t>(nb);
        ccodes = m.alloc<uint16_t>(3 * nb);
        cunp = m.alloc<T>(3 * nb);
    }
    if (reg) {
        if (N == 2) ereg = m.alloc<double>(nb);
        k_gen_fit<T><<<(unsigned)((nb + 127) / 128), 128, 0, st>>>(a, dX, fit, fit_ok, ereg);
        launches(cudaGetLastError());
    }
    if (N == 1) {
        auto k = straight ? k_gen1<T, false, 1> : k_gen1<T, false, 0>;
        k<<<1, 32, 0, st>>>(a, dX, R, codes, scratch, sel, fit, fit_ok, ccodes, cunp, cunp + 2 * nb, dcounts, nullptr,
                            0, nullptr, nullptr);
        launches(cudaGetLastError());
    } else if (reg) {
        auto k = straight ? k_gen2_seq<T, 1> : k_gen2_seq<T, 0>;
        const size_t tiles = ((size_t)2 * (bs + 2) * (bs + 2) * sizeof(T) + 15) & ~(size_t)15;
        const size_t smem = tiles + (size_t)3 * 2 * (bs - 2) * sizeof(double) + 16;
        CK(allow_dynamic_smem((const void *)k));
        T *band = m.alloc<T>(4 * (uint64_t)a.d1);
        k<<<1, 32, smem, st>>>(a, dX, band, codes, scratch, sel, fit, fit_ok, ereg, ccodes, cunp, cunp + 2 * nb,
                               dcounts);
        launches(cudaGetLastError());
    } else {
        const size_t smem = (size_t)kGenWarps * (size_t)((bs + 2) * (bs + 2)) * sizeof(T);
        auto k = straight ? k_gen2_diag<T, false, 1> : k_gen2_diag<T, false, 0>;
        CK(allow_dynamic_smem((const void *)k));
        for (int64_t d = 0; d <= (a.nb0 - 1) + (a.nb1 - 1); d++) {
            const int64_t bi_lo = std::max<int64_t>(0, d - (a.nb1 - 1));
            const int64_t bi_hi = std::min<int64_t>(a.nb0 - 1, d);
            const int64_t cnt = bi_hi - bi_lo + 1;
            k<<<(unsigned)((cnt + kGenWarps - 1) / kGenWarps), kGenWarps * 32, smem, st>>>(
                a, d, bi_lo, dX, R, codes, scratch, sel, nullptr, nullptr, nullptr, 0, nullptr);
            launches(cudaGetLastError());
        }
    }
    CK(cudaEventRecord(ev_pred.b, st));
    // selections and coefficient counts
    uint64_t cnt[4] = {composed ? nb : 0, 0, 0, 0};
    if (N == 1 || reg) {
        unsigned long long hc4[4];
        CK(cudaMemcpyAsync(hc4, dcounts, 32, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int i = 0; i < 4; i++) cnt[i] = hc4[i];
    }
    const uint64_t ns = cnt[0], ncc = cnt[1], nul = cnt[2], nui = cnt[3];
    CK(cudaEventRecord(ev_huff.a, st));
    HuffEncoded hs, hr, hc;
    if (composed && ns) huffman_encode_device(sel, ns, 0, m, st, launches, hs, tm);
    if (ncc) huffman_encode_device(ccodes, ncc, kCoefRadius, m, st, launches, hr, tm);
    huffman_encode_device(codes, n, radius, m, st, launches, hc, tm);
    const uint64_t nunpred = hc.nzero;
    T *unp = m.alloc<T>(nunpred ? nunpred : 1);
    if (nunpred) launches(launch_compact_zeros<T>(codes, n, hc.zc, hc.zoff, nullptr, scratch, unp, st));
    CK(cudaEventRecord(ev_huff.b, st));
    // SZGeneralFrontend::save: dims, block size, each predictor's save in
    // list order (Lorenzo: its id; regression: id, coefficient count, the two
    // coefficient quantizers, the coefficient codes), the composed
    // predictor's selections, LinearQuantizer::save; then the codes
    struct Part {
        std::vector<uint8_t> host;
        const void *dev;
        size_t dev_bytes;
    };
    std::vector<Part> parts;
    auto host_part = [&](std::vector<uint8_t> v) { parts.push_back(Part{std::move(v), nullptr, 0}); };
    auto dev_part = [&](const void *p, size_t nbytes) {
        if (nbytes) parts.push_back(Part{{}, p, nbytes});
    };
    {
        std::vector<uint8_t> h;
        for (int i = 0; i < N; i++) put<uint64_t>(h, dims[i]);
        put<uint32_t>(h, (uint32_t)bs);
        host_part(std::move(h));
    }
    for (int p = 0; p < a.np; p++) {
        std::vector<uint8_t> h;
        if (a.kinds[p] != 3) {
            put<uint8_t>(h, 1);  // LorenzoPredictor predictor_id
            host_part(std::move(h));
            continue;
        }
        put<uint8_t>(h, 2);  // RegressionPredictor::save (RegressionPredictor.hpp:103-120)
        put<uint64_t>(h, ncc);
        if (!ncc) {
            host_part(std::move(h));
            continue;
        }
        put_quantizer_header(h, a.eb_ind, a.cradius_ind, nui);
        host_part(std::move(h));
        dev_part(cunp + 2 * nb, nui * sizeof(T));
        std::vector<uint8_t> h2;
        put_quantizer_header(h2, a.eb_lin, a.cradius_lin, nul);
        host_part(std::move(h2));
        dev_part(cunp, nul * sizeof(T));
        std::vector<uint8_t> h3;
        append_tree(h3, hr.cb, hr.nbytes);
        host_part(std::move(h3));
        dev_part(hr.bits, hr.nbytes);
    }
    if (composed) {
        std::vector<uint8_t> h;
        put<uint64_t>(h, ns);
        if (ns) append_tree(h, hs.cb, hs.nbytes);
        host_part(std::move(h));
        if (ns) dev_part(hs.bits, hs.nbytes);
    }
    {
        std::vector<uint8_t> h;
        put_quantizer_header(h, eb, radius, nunpred);
        host_part(std::move(h));
        dev_part(unp, nunpred * sizeof(T));
        std::vector<uint8_t> h2;
        append_tree(h2, hc.cb, hc.nbytes);
        host_part(std::move(h2));
        dev_part(hc.bits, hc.nbytes);
    }
    size_t total = 0;
    for (const Part &pt : parts) total += pt.dev ? pt.dev_bytes : pt.host.size();
    // device parts come back through the thread's pinned staging buffer
    uint8_t *pin = t_pin_payload.get(total + 8);
    uint8_t *o = pin;
    for (const Part &pt : parts) {
        if (pt.dev) {
            CK(cudaMemcpyAsync(o, pt.dev, pt.dev_bytes, cudaMemcpyDeviceToHost, st));
            o += pt.dev_bytes;
        } else {
            std::memcpy(o, pt.host.data(), pt.host.size());
            o += pt.host.size();
        }
    }
    CK(cudaStreamSynchronize(st));
    emit_payload(out, pin, total);
    tm.unpred_count = nunpred;
    tm.payload_bytes = total;
    tm.predict_ms += ev_pred.ms();
    tm.huffman_ms += ev_huff.ms();
}

// SZGeneralFrontend::load + decompress into dOut (device); lo / lo2 / reg come
// from the stream's Config and fix the predictor list.  A composed stream
// holds one selection per block whose chosen predictor committed; blocks past
// the end of the selections (a 1-D final block of one point that fell back
// to the one-layer Lorenzo predictor, where the reference's own decoder reads
// past its list) take that fallback.
template <typename T>
void gen_decompress(int N, const uint8_t *pl, size_t psize, const uint64_t *dims, int lo, int lo2, int reg, T *dOut,
                    cudaStream_t st, Counter &launches, faz_timings &tm) {
    const uint8_t *p = pl, *end = pl + psize;
    auto need = [&](size_t k) {
        if ((size_t)(end - p) < k) throw Fail{FAZ_ERR_FORMAT, "truncated Lorenzo stream"};
    };
    need((size_t)N * 8 + 4);
    for (int i = 0; i < N; i++) {
        uint64_t v;
        std::memcpy(&v, p, 8);
        p += 8;
        if (v != dims[i]) throw Fail{FAZ_ERR_FORMAT, "payload dims differ from the trailer"};
    }
    uint32_t bs;
    std::memcpy(&bs, p, 4);
    p += 4;
    check_gen(N, (int)bs, lo, lo2, reg, 1);
    GenArgs a = make_gen_args<T>(N, dims, (int)bs, lo, lo2, reg, 1.0, 1);
    const uint64_t n = (uint64_t)(a.d0 * a.d1), nb = (uint64_t)(a.nb0 * a.nb1);
    const bool composed = a.np > 1;
    DevMem m(st);
    Events ev_dec, ev_pred;
    CK(cudaEventRecord(ev_dec.a, st));
    // LinearQuantizer::load header
    auto get_quantizer = [&](double &eb, int32_t &radius, uint64_t &nun) {
        need(1 + 8 + 4 + 8);
        p += 1;
        std::memcpy(&eb, p, 8);
        p += 8;
        std::memcpy(&radius, p, 4);
        p += 4;
        std::memcpy(&nun, p, 8);
        p += 8;
        if ((size_t)(end - p) / sizeof(T) < nun) throw Fail{FAZ_ERR_FORMAT, "truncated unpredictable values"};
    };
    uint64_t ncc = 0, nui = 0, nul = 0, ns = 0;
    uint16_t *ccodes = m.alloc<uint16_t>(3 * nb);
    T *cunp = m.alloc<T>(3 * nb);
    for (int k = 0; k < a.np; k++) {
        need(1);
        p += 1;  // predictor id
        if (a.kinds[k] != 3) continue;
        need(8);
        std::memcpy(&ncc, p, 8);
        p += 8;
        if (!ncc) continue;
        if (ncc > (uint64_t)(N + 1) * nb) throw Fail{FAZ_ERR_FORMAT, "bad regression coefficient count"};
        double eb_ind, eb_lin;
        int32_t r_ind, r_lin;
        get_quantizer(eb_ind, r_ind, nui);
        if (nui > nb) throw Fail{FAZ_ERR_FORMAT, "bad regression coefficient count"};
        if (nui) CK(cudaMemcpyAsync(cunp + 2 * nb, p, nui * sizeof(T), cudaMemcpyHostToDevice, st));
        p += nui * sizeof(T);
        get_quantizer(eb_lin, r_lin, nul);
        if (nul > 2 * nb) throw Fail{FAZ_ERR_FORMAT, "bad regression coefficient count"};
        if (nul) CK(cudaMemcpyAsync(cunp, p, nul * sizeof(T), cudaMemcpyHostToDevice, st));
        p += nul * sizeof(T);
        if (!(eb_ind > 0) || !(eb_lin > 0) || r_ind < 1 || r_ind > 32768 || r_lin < 1 || r_lin > 32768)
            throw Fail{FAZ_ERR_FORMAT, "bad regression coefficient quantizer"};
        a.eb_ind = eb_ind;
        a.eb_lin = eb_lin;
        a.cradius_ind = r_ind;
        a.cradius_lin = r_lin;
        huffman_decode_device(p, end, ncc, ccodes, m, st, launches);
    }
    uint16_t *sel = m.alloc<uint16_t>(nb);
    if (composed) {
        need(8);
        std::memcpy(&ns, p, 8);
        p += 8;
        if (ns > nb) throw Fail{FAZ_ERR_FORMAT, "selection count exceeds the block count"};
        if (ns) huffman_decode_device(p, end, ns, sel, m, st, launches);
    }
    double eb;
    int32_t radius;
    uint64_t nunpred;
    get_quantizer(eb, radius, nunpred);
    if (!(eb > 0)) throw Fail{FAZ_ERR_FORMAT, "bad error bound"};
    check_gen(N, (int)bs, lo, lo2, reg, radius);
    T *dunp = m.alloc<T>(nunpred ? nunpred : 1);
    if (nunpred) CK(cudaMemcpyAsync(dunp, p, nunpred * sizeof(T), cudaMemcpyHostToDevice, st));
    p += nunpred * sizeof(T);
    uint16_t *codes = m.alloc<uint16_t>(n);
    huffman_decode_device(p, end, n, codes, m, st, launches);
    uint64_t *zpos = nullptr;
    const uint64_t nz = zero_positions(codes, n, m, st, launches, zpos);
    if (nz != nunpred) throw Fail{FAZ_ERR_FORMAT, "unpredictable count does not match the zero codes"};
    CK(cudaEventRecord(ev_dec.b, st));
    {
        const GenArgs ac = a;
        a = make_gen_args<T>(N, dims, (int)bs, lo, lo2, reg, eb, radius);
        a.eb_ind = ac.eb_ind;
        a.eb_lin = ac.eb_lin;
        a.cradius_ind = ac.cradius_ind;
        a.cradius_lin = ac.cradius_lin;
    }
    const bool straight = sizeof(T) == 4 && a.q.fast;
    int *derr = m.alloc<int>(1);
    CK(cudaMemsetAsync(derr, 0, 4, st));
    CK(cudaEventRecord(ev_pred.a, st));
    if (N == 1) {
        unsigned long long hc4[4] = {ns, ncc, nul, nui};
        unsigned long long *dcounts = m.alloc<unsigned long long>(4);
        CK(cudaMemcpyAsync(dcounts, hc4, 32, cudaMemcpyHostToDevice, st));
        auto k = straight ? k_gen1<T, true, 1> : k_gen1<T, true, 0>;
        k<<<1, 32, 0, st>>>(a, nullptr, dOut, codes, nullptr, sel, nullptr, nullptr, ccodes, cunp, cunp + 2 * nb,
                            dcounts, zpos, nz, dunp, derr);
        launches(cudaGetLastError());
        CK(cudaStreamSynchronize(st));  // hc4 leaves scope
    } else {
        uint8_t *kind = m.alloc<uint8_t>(nb);
        T *coef = m.alloc<T>(3 * nb);
        k_gen_chain<T><<<1, 32, 0, st>>>(a, sel, ns, ccodes, ncc, cunp, nul, cunp + 2 * nb, nui, kind, coef, derr);
        launches(cudaGetLastError());
        const size_t smem = (size_t)kGenWarps * (size_t)((bs + 2) * (bs + 2)) * sizeof(T);
        auto k = straight ? k_gen2_diag<T, true, 1> : k_gen2_diag<T, true, 0>;
        CK(allow_dynamic_smem((const void *)k));
        for (int64_t d = 0; d <= (a.nb0 - 1) + (a.nb1 - 1); d++) {
            const int64_t bi_lo = std::max<int64_t>(0, d - (a.nb1 - 1));
            const int64_t bi_hi = std::min<int64_t>(a.nb0 - 1, d);
            const int64_t cnt = bi_hi - bi_lo + 1;
            k<<<(unsigned)((cnt + kGenWarps - 1) / kGenWarps), kGenWarps * 32, smem, st>>>(
                a, d, bi_lo, nullptr, dOut, codes, nullptr, nullptr, kind, coef, zpos, nz, dunp);
            launches(cudaGetLastError());
        }
    }
    CK(cudaEventRecord(ev_pred.b, st));
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (herr == 1) throw Fail{FAZ_ERR_FORMAT, "bad predictor selection"};
    if (herr) throw Fail{FAZ_ERR_FORMAT, "regression coefficients exhausted"};
    tm.huffman_ms += ev_dec.ms();
    tm.predict_ms += ev_pred.ms();
}

template void gen_compress_payload<float>(int, const uint64_t *, int, int, int, int, double, int, const float *,
                                          cudaStream_t, Counter &, faz_timings &, std::vector<uint8_t> &);
template void gen_compress_payload<double>(int, const uint64_t *, int, int, int, int, double, int, const double *,
                                           cudaStream_t, Counter &, faz_timings &, std::vector<uint8_t> &);
template void gen_decompress<float>(int, const uint8_t *, size_t, const uint64_t *, int, int, int, float *,
                                    cudaStream_t, Counter &, faz_timings &);
template void gen_decompress<double>(int, const uint8_t *, size_t, const uint64_t *, int, int, int, double *,
                                     cudaStream_t, Counter &, faz_timings &);

}  // namespace faz
