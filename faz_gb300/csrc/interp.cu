// interp.cu - multilevel interpolation predictor + linear quantiser kernels.
//
// One CTA per interpolation block and level (SZInterpolationCompressor.hpp
// 384-461 compress, 106-196 decompress).  The block's lattice points with an
// even index along the last sweep axis live in shared memory; sweep 1 and 2
// targets are computed there, sweep 3 targets stream from global memory.
// Lines on the block's first planes, which the reference assigns to the
// previous block, are recomputed (never emitted) so that every block of a
// level runs independently.  Codes of a sweep are staged in shared memory and
// written to their stream positions in one coalesced pass.
//
// Arithmetic follows the reference's types and operation order (compiled with
// -fmad=false): stencils in T (include/QoZ/utils/Interpolators.hpp:9-36),
// quantiser in the T/double mix of include/QoZ/quantizer/IntegerQuantizer.hpp:69-179.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdlib>
#include <cfloat>
#include <type_traits>
#include "common.cuh"
#include "fastq.cuh"
#include "internal.h"
#include "quant.cuh"
#include "stencil.cuh"

namespace faz {

// Move cnt codes between global codes[0..cnt) and shared stg[sh..sh+cnt),
// where sh = (global position & 7): the body moves 8 codes per 16-byte
// access on both sides.
template <bool TO_GLOBAL>
__device__ __forceinline__ void move_codes(uint16_t *g, uint16_t *stg, int64_t cnt, int sh) {
    const int64_t a0 = (8 - sh) & 7;
    const int64_t nbody = cnt > a0 ? (cnt - a0) >> 3 : 0;
    const int64_t tail0 = a0 + (nbody << 3);
    for (int64_t i = threadIdx.x; i < cnt; i += blockDim.x) {
        if (i < a0 || i >= tail0) {
            if (TO_GLOBAL) g[i] = stg[sh + i];
            else stg[sh + i] = g[i];
        }
    }
    for (int64_t j = threadIdx.x; j < nbody; j += blockDim.x) {
        const int64_t i = a0 + (j << 3);
        if (TO_GLOBAL) *reinterpret_cast<uint4 *>(g + i) = *reinterpret_cast<const uint4 *>(stg + sh + i);
        else *reinterpret_cast<uint4 *>(stg + sh + i) = *reinterpret_cast<const uint4 *>(g + i);
    }
}

// --------------------------------------------------------- level kernel
// One CTA per block.  Each half-warp takes one line at a time; lane t of the
// half-warp owns target 2t+1 of the line.  Shared-memory strides along every
// sweep axis are odd multiples of the lane step, so the half-warps read
// distinct banks.  Lanes past the line's targets run the same code on a valid
// target and store nothing.
// WIDE selects 64-bit element offsets; fields below 2^31 elements use 32-bit
// offsets from the block's first element.  QM selects the quantiser path
// (1: straight-line float path, 0: general).
// COH: coarse values come from W through L2 (ld.global.cg) instead of
// cp.async (which may hit L1): in the batched launch other SMs write W during
// the launch, and L1 is not coherent.
template <typename T, bool DECOMP, bool WIDE, int QM, bool COH, int CUB>
__device__ __forceinline__ void level_block(const LevelArgs &a, const int64_t bid, const T *__restrict__ X,
                                            T *__restrict__ W, uint16_t *__restrict__ codes,
                                            T *__restrict__ scratch, const uint64_t *__restrict__ zpos, uint64_t nz,
                                            const T *__restrict__ unpred, unsigned char *smem_raw) {
    using Off = typename std::conditional<WIDE, int64_t, int32_t>::type;
    T *V = reinterpret_cast<T *>(smem_raw);
    uint16_t *stg = reinterpret_cast<uint16_t *>(smem_raw + (((size_t)a.vwords * sizeof(T) + 15) & ~(size_t)15));
    int64_t bc[3];
    block_coords(a, bid, bc);
    BlockGeom g;
    block_geom(a, bc, g);
    const int P0 = a.perm[0], P1 = a.perm[1], P2 = a.perm[2];
    const int n0 = g.n0, n1 = g.n1, n2 = g.n2, h2 = g.h2;
    const int k0 = g.k0, k1 = g.k1, k2 = g.k2;
    const Off G0 = (Off)(a.s * pick3(P0, a.offs[0], a.offs[1], a.offs[2]));
    const Off G1 = (Off)(a.s * pick3(P1, a.offs[0], a.offs[1], a.offs[2]));
    const Off G2 = (Off)(a.s * pick3(P2, a.offs[0], a.offs[1], a.offs[2]));
    {
        const int64_t gbase = g.beg[0] * a.offs[0] + g.beg[1] * a.offs[1] + g.beg[2] * a.offs[2];
        X += DECOMP ? 0 : gbase;
        W += gbase;
    }
    const uint64_t base = a.block_off[bid];
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
    const int t = tid & 15, hw = tid >> 4, nhw = nt >> 4;
    const int cubic = a.cubic;
    const bool wb = a.write_back;

    // phase 0: lattice points with an even index along P2, one warp per row,
    // copied asynchronously
    {
        const int rows = n0 * n1;
        int m0 = warp / n1, m1 = warp - m0 * n1;
        for (int r = warp; r < rows; r += nwarps, m1 += nwarps) {
            while (m1 >= n1) {
                m1 -= n1;
                m0++;
            }
            const bool coarse = !(m0 & 1) && !(m1 & 1);
            if (DECOMP && !coarse) continue;
            const T *src = coarse ? W : X;
            const Off rb = m0 * G0 + m1 * G1;
            T *dst = V + r * h2;
            if (COH && coarse) {
                for (int e = lane; e < h2; e += 32) dst[e] = __ldcg(src + rb + (Off)(2 * e) * G2);
            } else {
                for (int e = lane; e < h2; e += 32) cp_async<sizeof(T)>(dst + e, src + rb + (Off)(2 * e) * G2);
            }
        }
        cp_async_wait_all();
    }
    __syncthreads();

    // sweep 1: lines along P0 at even (m1, m2), first planes included
    if (g.t0 > 0) {
        const int64_t cnt = g.c1;
        const int sh = (int)(base & 7);
        uint16_t *sg = stg + sh;
        if (DECOMP) {
            move_codes<false>(codes + base, stg, cnt, sh);
            __syncthreads();
        }
        const int st = n1 * h2;
        const int lines = ((n1 + 1) / 2) * h2;
        const bool act = t < g.t0;
        const int m0 = act ? 2 * t + 1 : 1;
        const Stencil<T> S = make_stencil<T>(m0, n0, cubic, st, 0);
        const int rk = line_rank(m0, n0, cubic);
        const Off gl = (Off)m0 * G0;
        LineCursor lc;
        lc.init(hw, nhw, h2);  // outer = e1, inner = e2
        for (int l = hw; l < lines; l += nhw, lc.next()) {
            const int e1 = lc.outer, e2 = lc.inner;
            const int col = 2 * e1 * h2 + e2;
            const bool emit = act && e1 >= k1 && e2 >= k2;
            const int rank = ((e1 - k1) * g.ne2 + (e2 - k2)) * g.t0 + rk;
            const T pred = eval_stencil<CUB>(S, V + col);
            const int idx = m0 * st + col;
            const Off gi = gl + (Off)(2 * e1) * G1 + (Off)(2 * e2) * G2;
            if (!DECOMP) {
                T v = V[idx], uv;
                const int code = quant_point<T, QM>(v, pred, a, uv);
                if (act) V[idx] = v;
                if (emit) {
                    sg[rank] = (uint16_t)code;
                    if (code == 0) scratch[base + rank] = uv;
                    if (wb) W[gi] = v;
                }
            } else if (act) {
                uint64_t pos;
                int code;
                if (emit) {
                    pos = base + rank;
                    code = sg[rank];
                } else {
                    pos = owner_pos_sweep1(a, g, bc, P1, P2, e1, e2, n2) + rk;
                    if (pos >= a.ncodes) {
                        atomicExch(a.err, 1);
                        pos = 0;
                    }
                    code = codes[pos];
                }
                const T v = recover_point<T, QM>(pred, code, pos, a, zpos, nz, unpred);
                V[idx] = v;
                if (emit) W[gi] = v;
            }
        }
        __syncthreads();
        if (!DECOMP) {
            move_codes<true>(codes + base, stg, cnt, sh);
            __syncthreads();
        }
    }

    // sweep 2: lines along P1 at (m0 any, m2 even); the m0 = 0 plane of a
    // non-first block is not needed by sweep 3 and is skipped.
    if (g.t1 > 0 && n0 - k0 > 0) {
        const int64_t cnt = g.c2;
        const uint64_t sbase = base + g.c1;
        const int sh = (int)(sbase & 7);
        uint16_t *sg = stg + sh;
        if (DECOMP) {
            move_codes<false>(codes + sbase, stg, cnt, sh);
            __syncthreads();
        }
        const int lines = (n0 - k0) * h2;
        const bool act = t < g.t1;
        const int m1 = act ? 2 * t + 1 : 1;
        const Stencil<T> S = make_stencil<T>(m1, n1, cubic, h2, 0);
        const int rk = line_rank(m1, n1, cubic);
        const Off gl = (Off)m1 * G1;
        LineCursor lc;
        lc.init(hw, nhw, h2);  // outer = m0 - k0, inner = e2
        for (int l = hw; l < lines; l += nhw, lc.next()) {
            const int q = lc.outer, e2 = lc.inner;
            const int m0 = k0 + q;
            const int col = m0 * n1 * h2 + e2;
            const bool emit = act && e2 >= k2;
            const int rank = (q * g.ne2 + (e2 - k2)) * g.t1 + rk;
            const T pred = eval_stencil<CUB>(S, V + col);
            const int idx = col + m1 * h2;
            const Off gi = (Off)m0 * G0 + gl + (Off)(2 * e2) * G2;
            if (!DECOMP) {
                T v = V[idx], uv;
                const int code = quant_point<T, QM>(v, pred, a, uv);
                if (act) V[idx] = v;
                if (emit) {
                    sg[rank] = (uint16_t)code;
                    if (code == 0) scratch[sbase + rank] = uv;
                    if (wb) W[gi] = v;
                }
            } else if (act) {
                uint64_t pos;
                int code;
                if (emit) {
                    pos = sbase + rank;
                    code = sg[rank];
                } else {
                    pos = owner_pos_sweep2(a, g, bc, P2, q) + rk;
                    if (pos >= a.ncodes) {
                        atomicExch(a.err, 1);
                        pos = 0;
                    }
                    code = codes[pos];
                }
                const T v = recover_point<T, QM>(pred, code, pos, a, zpos, nz, unpred);
                V[idx] = v;
                if (emit) W[gi] = v;
            }
        }
        __syncthreads();
        if (!DECOMP) {
            move_codes<true>(codes + sbase, stg, cnt, sh);
            __syncthreads();
        }
    }

    // sweep 3: lines along P2 at (m0, m1), emitted lines only.  Compression
    // reads the targets from global memory; the loads run two lines ahead.
    // A block that begins on the last element of an axis has no sweep-3
    // lines (n - k = 0).
    if (g.t2 > 0 && n0 - k0 > 0 && n1 - k1 > 0) {
        const int64_t cnt = g.c3;
        const uint64_t sbase = base + g.c1 + g.c2;
        const int sh = (int)(sbase & 7);
        uint16_t *sg = stg + sh;
        if (DECOMP) {
            move_codes<false>(codes + sbase, stg, cnt, sh);
            __syncthreads();
        }
        const int w1 = n1 - k1;
        const int lines = (n0 - k0) * w1;
        const bool act = t < g.t2;
        const int m2 = act ? 2 * t + 1 : 1;
        const Stencil<T> S = make_stencil<T>(m2, n2, cubic, 1, 1);
        const int rk = line_rank(m2, n2, cubic);
        const Off gl = (Off)m2 * G2 + (Off)k0 * G0 + (Off)k1 * G1;
        LineCursor lc, lp;  // line being computed / being loaded
        lc.init(hw, nhw, w1);
        lp = lc;
        T xa = 0, xb = 0;
        int lpi = hw;
        if (!DECOMP) {
            if (lpi < lines) xa = X[gl + (Off)lp.outer * G0 + (Off)lp.inner * G1];
            lpi += nhw;
            lp.next();
        }
        for (int l = hw; l < lines; l += nhw, lc.next()) {
            if (!DECOMP) {
                xb = lpi < lines ? X[gl + (Off)lp.outer * G0 + (Off)lp.inner * G1] : (T)0;
                lpi += nhw;
                lp.next();
            }
            const int q0 = lc.outer, q1 = lc.inner;
            const T *row = V + ((k0 + q0) * n1 + (k1 + q1)) * h2;
            const T pred = eval_stencil<CUB>(S, row);
            const int rank = l * g.t2 + rk;
            const Off gi = gl + (Off)q0 * G0 + (Off)q1 * G1;
            if (!DECOMP) {
                T v = xa, uv;
                const int code = quant_point<T, QM>(v, pred, a, uv);
                if (act) {
                    sg[rank] = (uint16_t)code;
                    if (code == 0) scratch[sbase + rank] = uv;
                    if (wb) W[gi] = v;
                }
                xa = xb;
            } else if (act) {
                W[gi] = recover_point<T, QM>(pred, (int)sg[rank], sbase + rank, a, zpos, nz, unpred);
            }
        }
        __syncthreads();
        if (!DECOMP) move_codes<true>(codes + sbase, stg, cnt, sh);
    }
}

template <typename T, bool DECOMP, bool WIDE, int QM, int CUB>
__global__ void __launch_bounds__(512, 2) k_interp_level(LevelArgs a, const T *__restrict__ X, T *__restrict__ W,
                                                      uint16_t *__restrict__ codes, T *__restrict__ scratch,
                                                      const uint64_t *__restrict__ zpos, uint64_t nz,
                                                      const T *__restrict__ unpred) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    level_block<T, DECOMP, WIDE, QM, false, CUB>(a, blockIdx.x, X, W, codes, scratch, zpos, nz, unpred, smem_raw);
}

// ------------------------------------------------------ coarse levels
// Levels with lattice stride s >= 2 hold 1/8 of the field or less, in few
// blocks (64 at the third level of a 512^3 field, one at the last): one CTA
// per block leaves most SMs idle while each block's sweeps run one after
// another.  Instead, each sweep of the level is one launch over every block,
// one thread per emitted target in stream order (so code stores are
// contiguous), neighbours read from the reconstruction W (coarse points and
// the earlier sweeps' targets, written before this launch began), targets
// written back to W.  Every line is computed once, by the block that emits it.
// CTA c takes chunk c % chunks of block c / chunks.
template <typename T, bool DECOMP, int QM, int CUB>
__global__ void __launch_bounds__(256) k_level_sweep(LevelArgs a, int sw, int64_t chunks, const T *__restrict__ X,
                                                    T *__restrict__ W, uint16_t *__restrict__ codes,
                                                    T *__restrict__ scratch, const uint64_t *__restrict__ zpos,
                                                    uint64_t nz, const T *__restrict__ unpred) {
    __shared__ BlockGeom sgeo;
    __shared__ int64_t sbc[3];
    const int64_t bid = (int64_t)blockIdx.x / chunks;
    const int64_t x = ((int64_t)blockIdx.x - bid * chunks) * blockDim.x + threadIdx.x;
    if (threadIdx.x == 0) {
        block_coords(a, bid, sbc);
        block_geom(a, sbc, sgeo);
    }
    __syncthreads();
    const BlockGeom &g = sgeo;
    const int64_t cnt = sw == 1 ? g.c1 : (sw == 2 ? g.c2 : g.c3);
    if (x >= cnt) return;
    const int tl = sw == 1 ? g.t0 : (sw == 2 ? g.t1 : g.t2);  // targets per line
    const int n = sw == 1 ? g.n0 : (sw == 2 ? g.n1 : g.n2);   // lattice points per line
    const int64_t L = x / tl;
    const int r = (int)(x - L * tl);
    // target of stream rank r in its line (inverse of line_rank)
    int m;
    if (!a.cubic || n < 5) {
        m = 2 * r + 1;
    } else {
        const int ia = (n & 1) ? n - 2 : n - 3;
        const int cint = (ia - 3) >> 1;
        m = r < cint ? 2 * r + 3 : (r == cint ? 1 : (r == cint + 1 ? ia : n - 1));
    }
    // lattice coordinates along P0, P1, P2 of the line's origin
    int64_t c0, c1, c2;
    if (sw == 1) {
        c0 = 0;
        c1 = 2 * (L / g.ne2 + g.k1);
        c2 = 2 * (L % g.ne2 + g.k2);
    } else if (sw == 2) {
        c0 = g.k0 + L / g.ne2;
        c1 = 0;
        c2 = 2 * (L % g.ne2 + g.k2);
    } else {
        const int64_t w1 = g.n1 - g.k1;
        c0 = g.k0 + L / w1;
        c1 = g.k1 + L % w1;
        c2 = 0;
    }
    const int P0 = a.perm[0], P1 = a.perm[1], P2 = a.perm[2];
    const int64_t o0 = pick3(P0, a.offs[0], a.offs[1], a.offs[2]), o1 = pick3(P1, a.offs[0], a.offs[1], a.offs[2]),
                  o2 = pick3(P2, a.offs[0], a.offs[1], a.offs[2]);
    const int64_t b0 = pick3(P0, g.beg[0], g.beg[1], g.beg[2]), b1 = pick3(P1, g.beg[0], g.beg[1], g.beg[2]),
                  b2 = pick3(P2, g.beg[0], g.beg[1], g.beg[2]);
    const int64_t origin = (b0 + c0 * a.s) * o0 + (b1 + c1 * a.s) * o1 + (b2 + c2 * a.s) * o2;
    const int64_t st = a.s * (sw == 1 ? o0 : (sw == 2 ? o1 : o2));
    const Stencil<T> S = make_stencil<T>(m, n, a.cubic, (int)st, 0);
    const T pred = eval_stencil<CUB>(S, W + origin);
    const int64_t gi = origin + (int64_t)m * st;
    const uint64_t pos = a.block_off[bid] + (uint64_t)(sw == 1 ? 0 : (sw == 2 ? g.c1 : g.c1 + g.c2)) + (uint64_t)x;
    if (!DECOMP) {
        T v = X[gi], uv;
        const int code = quant_point<T, QM>(v, pred, a, uv);
        codes[pos] = (uint16_t)code;
        if (code == 0) scratch[pos] = uv;
        W[gi] = v;
    } else {
        W[gi] = recover_point<T, QM>(pred, (int)codes[pos], pos, a, zpos, nz, unpred);
    }
}

// ------------------------------------------------------ batched launch
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

constexpr unsigned kBatchWaitLimit = 1u << 22;  // polls (with back-off) of a dependency before giving up

// Every field's first point / anchor grid and interpolation levels, in one
// launch of persistent CTAs.  Tickets are work items in queue order: groups
// (a field's first point, anchor chunk or level) come round by round, the
// first points and anchors first, then every field's coarsest level, and so
// on.  A CTA takes a ticket, waits until every item of the group it depends on
// (the same field's previous level) is done, runs it and counts it done.  The
// groups waited for hold smaller tickets, taken by CTAs already running, so
// every wait ends; each is bounded all the same (error flag, then the item
// runs).  Coarse values written in this launch are read through L2.
template <typename T, bool WIDE>
__global__ void __launch_bounds__(512, 2)
    k_interp_batch(const BatchGroup *__restrict__ groups, int ngroups, const BatchField *__restrict__ fields,
                   const LevelArgs *__restrict__ largs, uint64_t total, unsigned long long *counter, unsigned *done,
                   int *err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ unsigned long long s_t;
    __shared__ int s_g;
    __shared__ int64_t s_local;
    __shared__ LevelArgs s_a;
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned long long t = atomicAdd(counter, 1ull);
            s_t = t;
            if (t < total) {
                int lo = 0, hi = ngroups - 1;  // last group with item0 <= t
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if ((unsigned long long)groups[mid].item0 <= t) lo = mid;
                    else hi = mid - 1;
                }
                s_g = lo;
                s_local = (int64_t)(t - (unsigned long long)groups[lo].item0);
                const int dep = groups[lo].dep;
                if (dep >= 0) {
                    const unsigned need = (unsigned)groups[dep].nitems;
                    unsigned it = 0;
                    while (ld_acquire_u32(done + dep) < need) {
                        if (++it > kBatchWaitLimit) {
                            atomicExch(err, 1);
                            break;
                        }
                        __nanosleep(128);
                    }
                }
                if (groups[lo].kind == 2) s_a = largs[groups[lo].args];
            }
        }
        __syncthreads();
        if (s_t >= total) return;
        const BatchGroup g = groups[s_g];
        const BatchField &f = fields[g.field];
        const T *X = (const T *)f.X;
        T *W = (T *)f.W;
        T *scratch = (T *)f.scratch;
        if (g.kind == 0) {
            if (threadIdx.x == 0) {
                T v = X[0], uv;
                const int code = quantize(v, (T)0, f.eb, f.recip, f.radius, f.trim, uv);
                f.codes[0] = (uint16_t)code;
                if (code == 0) scratch[0] = uv;
                W[0] = v;
            }
        } else if (g.kind == 1) {
            const int64_t i = s_local * blockDim.x + threadIdx.x;
            const int64_t nan = f.na[0] * f.na[1] * f.na[2];
            if (i < nan) {
                const int64_t z = i % f.na[2], r = i / f.na[2];
                const int64_t y = r % f.na[1], x = r / f.na[1];
                const int64_t gi = x * f.step[0] * f.offs[0] + y * f.step[1] * f.offs[1] + z * f.step[2] * f.offs[2];
                const T v = X[gi];
                f.codes[i] = 0;
                scratch[i] = v;
                W[gi] = v;
            }
        } else {
            const bool straight = sizeof(T) == 4 && s_a.fast && s_a.trim == 0;
            if (straight && s_a.cubic)
                level_block<T, false, WIDE, 1, true, 1>(s_a, s_local, X, W, f.codes, scratch, nullptr, 0, nullptr,
                                                        smem_raw);
            else if (straight)
                level_block<T, false, WIDE, 1, true, 0>(s_a, s_local, X, W, f.codes, scratch, nullptr, 0, nullptr,
                                                        smem_raw);
            else if (s_a.cubic)
                level_block<T, false, WIDE, 0, true, 1>(s_a, s_local, X, W, f.codes, scratch, nullptr, 0, nullptr,
                                                        smem_raw);
            else
                level_block<T, false, WIDE, 0, true, 0>(s_a, s_local, X, W, f.codes, scratch, nullptr, 0, nullptr,
                                                        smem_raw);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(done + s_g, 1u);
        }
    }
}

template <typename T>
cudaError_t launch_interp_batch(const BatchGroup *groups, int ngroups, const BatchField *fields, const LevelArgs *largs,
                                uint64_t total, unsigned long long *counter, unsigned *done, int *err, bool wide,
                                int grid, int threads, size_t smem, cudaStream_t st) {
    const void *k = wide ? (const void *)k_interp_batch<T, true> : (const void *)k_interp_batch<T, false>;
    cudaError_t e = allow_dynamic_smem(k);
    if (e != cudaSuccess) return e;
    if (wide)
        k_interp_batch<T, true><<<grid, threads, smem, st>>>(groups, ngroups, fields, largs, total, counter, done, err);
    else
        k_interp_batch<T, false><<<grid, threads, smem, st>>>(groups, ngroups, fields, largs, total, counter, done,
                                                               err);
    return cudaGetLastError();
}

template <typename T, bool WIDE>
int batch_occupancy(int threads, size_t smem) {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_interp_batch<T, WIDE>, threads, smem);
    return n;
}

// ------------------------------------------------- first point / anchors
// First point quantised against prediction 0 with the base bound
// (SZInterpolationCompressor.hpp:372-374), or the anchor grid of build_grid
// (854-900) as unpredictable values with code 0.
template <typename T>
__global__ void k_first_point(const T *X, T *W, uint16_t *codes, T *scratch, double eb, double recip, int radius,
                              int trim) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        T v = X[0], uv;
        int code = quantize(v, (T)0, eb, recip, radius, trim, uv);
        codes[0] = (uint16_t)code;
        if (code == 0) scratch[0] = uv;
        W[0] = v;
    }
}

template <typename T>
__global__ void k_first_point_dec(const uint16_t *codes, T *W, double eb, int radius, int trim,
                                  const uint64_t *zpos, uint64_t nz, const T *unpred) {
    if (threadIdx.x == 0 && blockIdx.x == 0) W[0] = recover((T)0, (int)codes[0], 0, eb, radius, trim, zpos, nz, unpred);
}

// anchors at multiples of maxStep on axes 0..2 (3-D view); na0..na2 anchors per axis
template <typename T, bool DECOMP>
__global__ void k_anchors(const T *X, T *W, uint16_t *codes, T *scratch, const T *unpred, int64_t na0, int64_t na1,
                          int64_t na2, int64_t step0, int64_t step1, int64_t step2, int64_t o0, int64_t o1,
                          int64_t o2) {
    int64_t total = na0 * na1 * na2;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t z = i % na2, r = i / na2;
        int64_t y = r % na1, x = r / na1;
        int64_t gi = x * step0 * o0 + y * step1 * o1 + z * step2 * o2;
        if (!DECOMP) {
            T v = X[gi];
            codes[i] = 0;
            scratch[i] = v;
            W[gi] = v;
        } else {
            W[gi] = unpred[i];
        }
    }
}

// ------------------------------------------------------------- min / max
// 16-byte loads over the aligned body, scalar loads for the ends.
template <typename T>
__device__ __forceinline__ void minmax_body(const T *__restrict__ X, uint64_t n, unsigned bid, unsigned nblocks,
                                            T *pmin, T *pmax) {
    T mn = X[0], mx = X[0];
    constexpr int V = 16 / sizeof(T);
    const uint64_t head = ((16 - ((uintptr_t)X & 15)) & 15) / sizeof(T);
    const uint64_t h = head < n ? head : n;
    const uint64_t nvec = (n - h) / V;
    const uint64_t tid = bid * (uint64_t)blockDim.x + threadIdx.x, nth = (uint64_t)nblocks * blockDim.x;
    const uint4 *xv = reinterpret_cast<const uint4 *>(X + h);
    for (uint64_t i = tid; i < nvec; i += nth) {
        uint4 q = __ldg(xv + i);
        const T *e = reinterpret_cast<const T *>(&q);
#pragma unroll
        for (int k = 0; k < V; k++) {
            T v = e[k];
            mn = v < mn ? v : mn;
            mx = v > mx ? v : mx;
        }
    }
    for (uint64_t i = tid; i < h; i += nth) {
        T v = X[i];
        mn = v < mn ? v : mn;
        mx = v > mx ? v : mx;
    }
    for (uint64_t i = h + nvec * V + tid; i < n; i += nth) {
        T v = X[i];
        mn = v < mn ? v : mn;
        mx = v > mx ? v : mx;
    }
    __shared__ T smn[32], smx[32];
    for (int o = 16; o > 0; o >>= 1) {
        T a = __shfl_down_sync(0xffffffffu, mn, o);
        T b = __shfl_down_sync(0xffffffffu, mx, o);
        mn = a < mn ? a : mn;
        mx = b > mx ? b : mx;
    }
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { smn[wid] = mn; smx[wid] = mx; }
    __syncthreads();
    if (wid == 0) {
        int nw = blockDim.x >> 5;
        mn = lane < nw ? smn[lane] : smn[0];
        mx = lane < nw ? smx[lane] : smx[0];
        for (int o = 16; o > 0; o >>= 1) {
            T a = __shfl_down_sync(0xffffffffu, mn, o);
            T b = __shfl_down_sync(0xffffffffu, mx, o);
            mn = a < mn ? a : mn;
            mx = b > mx ? b : mx;
        }
        if (lane == 0) { pmin[bid] = mn; pmax[bid] = mx; }
    }
}

template <typename T>
__global__ void k_minmax(const T *__restrict__ X, uint64_t n, T *pmin, T *pmax) {
    minmax_body(X, n, blockIdx.x, gridDim.x, pmin, pmax);
}

// min / max of every field of a batch: CTA (b, f) takes slice b of field f
template <typename T>
__global__ void k_minmax_batch(const T *const *__restrict__ X, const uint64_t *__restrict__ n, T *pmin, T *pmax) {
    const unsigned f = blockIdx.y;
    minmax_body(X[f], n[f], blockIdx.x, gridDim.x, pmin + (size_t)f * gridDim.x, pmax + (size_t)f * gridDim.x);
}

template <typename T>
cudaError_t launch_minmax_batch(const T *const *X, const uint64_t *n, int nfields, T *pmin, T *pmax, int nblocks,
                                cudaStream_t st) {
    k_minmax_batch<T><<<dim3(nblocks, nfields), 512, 0, st>>>(X, n, pmin, pmax);
    return cudaGetLastError();
}

// ------------------------------------------------------------ launchers

template <typename T>
cudaError_t launch_minmax(const T *X, uint64_t n, T *pmin, T *pmax, int nblocks, cudaStream_t st) {
    k_minmax<T><<<nblocks, 512, 0, st>>>(X, n, pmin, pmax);
    return cudaGetLastError();
}

template <typename T>
size_t level_smem_bytes(const LevelArgs &a) {
    size_t vb = ((size_t)a.vwords * sizeof(T) + 15) / 16 * 16;
    return vb + (size_t)a.stage_cap * sizeof(uint16_t);
}

// Coarse levels (stride >= 2) with few blocks, of fields below 2^31 values:
// the three sweep launches of k_level_sweep instead of one CTA per block.
template <typename T>
cudaError_t launch_level_sweeps(const LevelArgs &a, int64_t nblocks, bool decomp, const T *X, T *W, uint16_t *codes,
                                T *scratch, const uint64_t *zpos, uint64_t nz, const T *unpred, cudaStream_t st,
                                int *nlaunch) {
    const bool straight = sizeof(T) == 4 && a.fast && a.trim == 0;
    void (*k)(LevelArgs, int, int64_t, const T *, T *, uint16_t *, T *, const uint64_t *, uint64_t, const T *);
    if (a.cubic) {
        if (straight) k = decomp ? k_level_sweep<T, true, 1, 1> : k_level_sweep<T, false, 1, 1>;
        else k = decomp ? k_level_sweep<T, true, 0, 1> : k_level_sweep<T, false, 0, 1>;
    } else {
        if (straight) k = decomp ? k_level_sweep<T, true, 1, 0> : k_level_sweep<T, false, 1, 0>;
        else k = decomp ? k_level_sweep<T, true, 0, 0> : k_level_sweep<T, false, 0, 0>;
    }
    // the first block has the most targets in every sweep (no first planes
    // skipped, full extent)
    int64_t bc0[3] = {0, 0, 0};
    BlockGeom g0;
    block_geom(a, bc0, g0);
    const int64_t cmax[3] = {g0.c1, g0.c2, g0.c3};
    for (int sw = 1; sw <= 3; sw++) {
        if (cmax[sw - 1] <= 0) continue;
        const int64_t chunks = (cmax[sw - 1] + 255) / 256;
        k<<<(unsigned)(nblocks * chunks), 256, 0, st>>>(a, sw, chunks, X, W, codes, scratch, zpos, nz, unpred);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        ++*nlaunch;
    }
    return cudaSuccess;
}

template <typename T>
cudaError_t launch_level(const LevelArgs &a, int64_t nblocks, bool decomp, const T *X, T *W, uint16_t *codes,
                         T *scratch, const uint64_t *zpos, uint64_t nz, const T *unpred, cudaStream_t st,
                         int *nlaunch) {
    size_t sm = level_smem_bytes<T>(a);
    // half-warps take lines: enough threads for the lines of a block
    int64_t vol = (int64_t)a.vwords * 2;
    int threads = vol >= 8192 ? 512 : (vol >= 1024 ? 256 : (vol >= 256 ? 128 : 64));
    const bool wide = a.dims[0] * a.dims[1] * a.dims[2] >= ((int64_t)1 << 31);
    const bool straight = sizeof(T) == 4 && a.fast && a.trim == 0;
    // levels with fewer blocks than two per SM (the block kernel would leave
    // SMs idle) take the sweep launches
    static const int sms = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 1;
    }();
    const int64_t per_block = (a.bs / a.s + 1) * (a.bs / a.s + 1) * (a.bs / a.s + 1) / 256 + 1;
    if (a.s >= 2 && !wide && nblocks < 2 * sms && nblocks * per_block < (1ll << 31))
        return launch_level_sweeps<T>(a, nblocks, decomp, X, W, codes, scratch, zpos, nz, unpred, st, nlaunch);
    // the finest level of a 3-D float field: plane-parallel kernel (finest.cu).
    // It compresses faster than the block kernel below but decompresses
    // slower (0.95 vs 0.86 ms on 512^3), so decompression keeps the block
    // kernel.  FAZ_FINEST_PLANES (read per call, for comparisons): 0 = block
    // kernel for both, 2 = plane kernel for both.
    const char *plane_env = std::getenv("FAZ_FINEST_PLANES");
    const int plane_mode = plane_env && plane_env[0] == '0' ? 0 : (plane_env && plane_env[0] == '2' ? 2 : 1);
    if constexpr (sizeof(T) == 4) {
        if ((decomp ? plane_mode == 2 : plane_mode >= 1) && finest_eligible(a, decomp, X, sizeof(T))) {
            ++*nlaunch;
            return launch_finest(a, nblocks, decomp, reinterpret_cast<const float *>(X), reinterpret_cast<float *>(W),
                                 codes, reinterpret_cast<float *>(scratch), zpos, nz,
                                 reinterpret_cast<const float *>(unpred), st);
        }
    }
    ++*nlaunch;
    void (*k)(LevelArgs, const T *, T *, uint16_t *, T *, const uint64_t *, uint64_t, const T *);
#define FAZ_PICK(CUB)                                                                                            \
    if (straight) {                                                                                              \
        if (!decomp) k = wide ? k_interp_level<T, false, true, 1, CUB> : k_interp_level<T, false, false, 1, CUB>; \
        else k = wide ? k_interp_level<T, true, true, 1, CUB> : k_interp_level<T, true, false, 1, CUB>;          \
    } else {                                                                                                     \
        if (!decomp) k = wide ? k_interp_level<T, false, true, 0, CUB> : k_interp_level<T, false, false, 0, CUB>; \
        else k = wide ? k_interp_level<T, true, true, 0, CUB> : k_interp_level<T, true, false, 0, CUB>;          \
    }
    if (a.cubic) {
        FAZ_PICK(1)
    } else {
        FAZ_PICK(0)
    }
#undef FAZ_PICK
    cudaError_t e = allow_dynamic_smem((const void *)k);
    if (e != cudaSuccess) return e;
    k<<<(unsigned)nblocks, threads, sm, st>>>(a, X, W, codes, scratch, zpos, nz, unpred);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_first_point(bool decomp, const T *X, T *W, uint16_t *codes, T *scratch, double eb, int radius,
                               int trim, const uint64_t *zpos, uint64_t nz, const T *unpred, cudaStream_t st) {
    if (!decomp) k_first_point<T><<<1, 32, 0, st>>>(X, W, codes, scratch, eb, 1.0 / eb, radius, trim);
    else k_first_point_dec<T><<<1, 32, 0, st>>>(codes, W, eb, radius, trim, zpos, nz, unpred);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_anchors(bool decomp, const T *X, T *W, uint16_t *codes, T *scratch, const T *unpred,
                           const int64_t *na, const int64_t *step, const int64_t *offs, cudaStream_t st) {
    int64_t total = na[0] * na[1] * na[2];
    int blocks = (int)((total + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    if (blocks < 1) blocks = 1;
    if (!decomp)
        k_anchors<T, false><<<blocks, 256, 0, st>>>(X, W, codes, scratch, unpred, na[0], na[1], na[2], step[0], step[1],
                                                     step[2], offs[0], offs[1], offs[2]);
    else
        k_anchors<T, true><<<blocks, 256, 0, st>>>(X, W, codes, scratch, unpred, na[0], na[1], na[2], step[0], step[1],
                                                    step[2], offs[0], offs[1], offs[2]);
    return cudaGetLastError();
}

#define INST(T)                                                                                                  \
    template cudaError_t launch_minmax<T>(const T *, uint64_t, T *, T *, int, cudaStream_t);                     \
    template size_t level_smem_bytes<T>(const LevelArgs &);                                                      \
    template cudaError_t launch_level<T>(const LevelArgs &, int64_t, bool, const T *, T *, uint16_t *, T *,      \
                                         const uint64_t *, uint64_t, const T *, cudaStream_t, int *);            \
    template cudaError_t launch_first_point<T>(bool, const T *, T *, uint16_t *, T *, double, int, int,          \
                                               const uint64_t *, uint64_t, const T *, cudaStream_t);             \
    template cudaError_t launch_anchors<T>(bool, const T *, T *, uint16_t *, T *, const T *, const int64_t *,   \
                                           const int64_t *, const int64_t *, cudaStream_t);                      \
    template cudaError_t launch_interp_batch<T>(const BatchGroup *, int, const BatchField *, const LevelArgs *,   \
                                                uint64_t, unsigned long long *, unsigned *, int *, bool, int, int,\
                                                size_t, cudaStream_t);                                           \
    template int batch_occupancy<T, false>(int, size_t);                                                         \
    template cudaError_t launch_minmax_batch<T>(const T *const *, const uint64_t *, int, T *, T *, int,           \
                                                cudaStream_t);                                                   \
    template int batch_occupancy<T, true>(int, size_t);
INST(float)
INST(double)
#undef INST

}  // namespace faz
