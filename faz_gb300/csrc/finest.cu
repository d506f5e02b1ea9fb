// finest.cu - the finest interpolation level (lattice stride 1) of 3-D float
// fields, plane by plane.
//
// At stride 1 a block's lattice points split by the parity of their
// coordinates in sweep order (P0, P1, P2), SZInterpolationCompressor.hpp
// 3143-3360: all even = coarse (reconstructed by the previous level); odd
// along P0, even along P1 and P2 = sweep-1 targets, predicted along P0 from
// coarse points only; odd along P1, even along P2 = sweep-2 targets,
// predicted along P1 inside their P0-plane; odd along P2 = sweep-3 targets,
// predicted along P2 inside their row.  Once the block's coarse points are in
// shared memory every P0-plane is therefore independent of the others: one
// warp takes one plane, a TMA tiled copy (cp.async.bulk.tensor) brings the
// plane's original values into shared memory, and the warp runs the three
// sweeps of that plane.  The general level kernel (interp.cu) instead stages
// the block's whole even-P2 lattice and walks lines with per-line bookkeeping.
//
// Stream positions are the ones of interp.cu (closed form from level, block,
// sweep, line and index; common.cuh): sweep-1 codes of a block interleave all
// planes, so they are staged in shared memory and written once per block;
// sweep-2 and sweep-3 codes of a plane are contiguous and go straight to
// global memory, 32 bytes per half-warp.
//
// Requirements (finest_eligible): float data on the exact float quantiser
// path, P2 the contiguous axis, a block edge that is a multiple of 4 up to 32
// (block begins along P2 are TMA x coordinates, 16-byte multiples), a 3-D
// field below 2^31 values whose rows are 16-byte multiples (the tensor map's
// strides).  The compression uses this kernel; the decompression variant
// (codes in, the plane written back row by row) is correct but slower than
// the block kernel and runs only with FAZ_FINEST_PLANES=2 (interp.cu).
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <cstring>

#include "common.cuh"
#include "internal.h"
#include "quant.cuh"
#include "stencil.cuh"

namespace faz {

namespace {

constexpr int FW = 16;                 // warps per CTA
constexpr int FX = 36;                 // plane row pitch in floats (TMA box inner extent: 144 bytes)
constexpr int FROWS = 33;              // plane rows (block edge + 1)
constexpr int FC = 17;                 // coarse points per axis
constexpr uint32_t FPLANE_BYTES = FX * FROWS * 4;
constexpr int FXS_BYTES = (FPLANE_BYTES + 127) / 128 * 128;
constexpr int FC_BYTES = (FC * FC * FC * 4 + 127) / 128 * 128;
constexpr int FSTAGE = FC * FC * 16 + 16;  // sweep-1 codes of a block + alignment shift
constexpr int FSTAGE_BYTES = (FSTAGE * 2 + 127) / 128 * 128;
constexpr int FSMEM = FC_BYTES + FSTAGE_BYTES + FW * FXS_BYTES + 128;
constexpr uint32_t FWAIT_LIMIT = 1u << 24;  // try_wait polls before a TMA wait gives up

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tma_plane(float *dst, const CUtensorMap *tm, int x, int y, int z, uint64_t *bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(FPLANE_BYTES)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(saddr(dst)),
        "l"(tm), "r"(x), "r"(y), "r"(z), "r"(saddr(bar))
        : "memory");
}

// Bounded wait for phase `phase` of the plane barrier; false when it gave up.
__device__ __forceinline__ bool tma_wait(uint64_t *bar, uint32_t phase) {
    uint32_t done = 0;
    for (uint32_t it = 0; it < FWAIT_LIMIT && !done; it++) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(saddr(bar)), "r"(phase)
            : "memory");
    }
    return __all_sync(0xffffffffu, done) != 0;
}

// One quantisation of the exact float path and its bookkeeping: the code goes
// to *dst, an unpredictable value to *udst.
__device__ __forceinline__ float finest_point(float v, float pred, const LevelArgs &a, bool emit, uint16_t *dst,
                                              float *udst) {
    float uv;
    const int code = quant_point<float, 1>(v, pred, a, uv);
    if (emit) {
        *dst = (uint16_t)code;
        if (code == 0) *udst = uv;
    }
    return v;
}

// Compression (DECOMP = 0): X through the tensor map, codes and unpredictable
// values out.  Decompression (DECOMP = 1): codes in, every reconstructed
// target of the block into W.  Either way the plane buffer Xs ends up holding
// the plane's reconstruction at even P2 indices (each value written where its
// original was read, once the original is no longer needed) and, in
// decompression, at odd ones too; decompression then writes the plane's rows
// back.  W holds the coarse points (earlier levels) in both directions.
template <bool DECOMP, int CUB>
__global__ void __launch_bounds__(FW * 32, 2)
    k_finest(LevelArgs a, const __grid_constant__ CUtensorMap tm, float *__restrict__ W, uint16_t *__restrict__ codes,
             float *__restrict__ scratch, const uint64_t *__restrict__ zpos, uint64_t nz,
             const float *__restrict__ unpred) {
    extern __shared__ __align__(128) unsigned char smem[];
    float *C = reinterpret_cast<float *>(smem);
    uint16_t *stage = reinterpret_cast<uint16_t *>(smem + FC_BYTES);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float *Xs = reinterpret_cast<float *>(smem + FC_BYTES + FSTAGE_BYTES + warp * FXS_BYTES);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + FC_BYTES + FSTAGE_BYTES + FW * FXS_BYTES) + warp;

    int64_t bc[3];
    block_coords(a, blockIdx.x, bc);
    BlockGeom g;
    block_geom(a, bc, g);
    const int P0 = a.perm[0], P1 = a.perm[1];
    const int n0 = g.n0, n1 = g.n1, n2 = g.n2;
    const int k0 = g.k0, k1 = g.k1, k2 = g.k2;
    const int hh1 = (n1 + 1) / 2, h2 = g.h2;
    const int64_t G0 = pick3(P0, a.offs[0], a.offs[1], a.offs[2]);
    const int64_t G1 = pick3(P1, a.offs[0], a.offs[1], a.offs[2]);
    float *wb = W + g.beg[0] * a.offs[0] + g.beg[1] * a.offs[1] + g.beg[2] * a.offs[2];
    const uint64_t base = a.block_off[blockIdx.x];
    uint16_t *cb = codes + base;                  // the block's codes
    float *ub = DECOMP ? nullptr : scratch + base;  // their unpredictable values
    const int cubic = a.cubic;
    const int sh1 = (int)(base & 7);

    if (!DECOMP && lane == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(bar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // coarse points of the block: C[c0][c1][c2] = W at (2c0, 2c1, 2c2)
    {
        const int rows = ((n0 + 1) / 2) * hh1;
        for (int r = warp; r < rows; r += FW) {
            const int c0 = r / hh1, c1 = r - c0 * hh1;
            const float *src = wb + 2 * c0 * G0 + 2 * c1 * G1;
            if (lane < h2) cp_async<4>(C + (c0 * FC + c1) * FC + lane, src + 2 * lane);
        }
        cp_async_wait_all();
    }
    if (DECOMP) {
        // the block's sweep-1 codes (they interleave all planes)
        const int cnt = (int)g.c1;
        const int a0 = (8 - sh1) & 7;
        const int nbody = cnt > a0 ? (cnt - a0) >> 3 : 0;
        const int tail0 = a0 + (nbody << 3);
        for (int i = tid; i < cnt; i += blockDim.x)
            if (i < a0 || i >= tail0) stage[sh1 + i] = cb[i];
        for (int j = tid; j < nbody; j += blockDim.x) {
            const int i = a0 + (j << 3);
            *reinterpret_cast<uint4 *>(stage + sh1 + i) = *reinterpret_cast<const uint4 *>(cb + i);
        }
    }
    __syncthreads();

    const int t = lane & 15, half = lane >> 4;
    const int np = n0 - k0;   // planes with emitted codes
    const int w1 = n1 - k1;   // emitted rows (sweep 3)
    const int w2 = n2 - k2;   // emitted columns
    uint32_t phase = 0;
    bool ok = true;
    // planes in pairs (an odd and an even P0 index) per warp, so that warps
    // get the same work
    for (int pp = warp; 2 * pp < np && ok; pp += FW) {
        for (int s = 0; s < 2; s++) {
            const int m0 = k0 + 2 * pp + s;
            if (m0 >= n0) break;
            // the previous plane's reads and in-place writes of Xs come before
            // the copy engine's writes of the next plane
            if (!DECOMP) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (!DECOMP && lane == 0) {
                const int x = (int)g.beg[2];
                const int y = (int)g.beg[1] + (P0 == 1 ? m0 : 0);
                const int z = (int)g.beg[0] + (P0 == 0 ? m0 : 0);
                tma_plane(Xs, &tm, x, y, z, bar);
            }
            if (!DECOMP) {
                if (!tma_wait(bar, phase)) {
                    // the call fails; wait (bounded again) for the copy in flight
                    // before the warp leaves, so that it does not land in shared
                    // memory that another CTA may own by then
                    if (lane == 0 && a.err) atomicExch(a.err, 1);
                    (void)tma_wait(bar, phase);
                    ok = false;
                    break;
                }
                phase ^= 1;
            }
            if (!(m0 & 1)) {
                // even plane: its even-P1 / even-P2 points are coarse
                const float *cp = C + (m0 >> 1) * FC * FC;
                LineCursor lc;
                lc.init(lane, 32, h2);  // outer = e1, inner = e2
                for (int i = lane; i < hh1 * h2; i += 32, lc.next())
                    Xs[2 * lc.outer * FX + 2 * lc.inner] = cp[lc.outer * FC + lc.inner];
            } else {
                // sweep 1: targets (m0, 2e1, 2e2) from the coarse planes; first
                // the lines this block emits (stream rank = flat index x t0 +
                // rank in the line), then those on its first planes, which the
                // previous blocks emit (recomputed in compression, decoded from
                // their owners' streams in decompression)
                const Stencil<float> S1 = make_stencil<float>(m0, n0, cubic, FC * FC, 1);
                const int rk0 = line_rank(m0, n0, cubic);
                const int ne = g.ne1 * g.ne2;
                LineCursor lc;
                if (ne > 0) lc.init(lane, 32, g.ne2);
                for (int i0 = 0; i0 < ne; i0 += 32, lc.next()) {
                    const int i = i0 + lane;
                    const bool in = i < ne;
                    const int e1 = k1 + (in ? lc.outer : 0), e2 = k2 + (in ? lc.inner : 0);
                    const float pred = eval_stencil<CUB>(S1, C + e1 * FC + e2);
                    const int rank = (in ? i : 0) * g.t0 + rk0;
                    float *xp = Xs + 2 * e1 * FX + 2 * e2;
                    float v;
                    if (!DECOMP) v = finest_point(*xp, pred, a, in, stage + sh1 + rank, ub + rank);
                    else v = recover_point<float, 1>(pred, (int)stage[sh1 + rank], base + rank, a, zpos, nz, unpred);
                    if (in) *xp = v;
                }
                const int nfirst = k1 * h2 + k2 * (hh1 - k1);
                for (int j0 = 0; j0 < nfirst; j0 += 32) {
                    const int j = j0 + lane;
                    const bool in = j < nfirst;
                    int e1 = 0, e2 = 0;
                    if (in) {
                        if (j < k1 * h2) e2 = j;
                        else e1 = k1 + (j - k1 * h2);
                    }
                    const float pred = eval_stencil<CUB>(S1, C + e1 * FC + e2);
                    float *xp = Xs + 2 * e1 * FX + 2 * e2;
                    float v;
                    if (!DECOMP) {
                        v = finest_point(*xp, pred, a, false, nullptr, nullptr);
                    } else {
                        uint64_t pos = owner_pos_sweep1(a, g, bc, P1, a.perm[2], e1, e2, n2) + rk0;
                        if (pos >= a.ncodes) {
                            atomicExch(a.err, 1);
                            pos = 0;
                        }
                        v = recover_point<float, 1>(pred, (int)codes[pos], pos, a, zpos, nz, unpred);
                    }
                    if (in) *xp = v;
                }
            }
            __syncwarp();
            // sweep 2: targets (m0, 2t+1, 2e2), lines along P1
            if (g.t1 > 0) {
                const bool act = t < g.t1;
                const int m1 = act ? 2 * t + 1 : 1;
                const Stencil<float> S2 = make_stencil<float>(m1, n1, cubic, FX, 0);
                const int rk1 = line_rank(m1, n1, cubic);
                const int pb = (int)g.c1 + (m0 - k0) * g.ne2 * g.t1 + rk1 - k2 * g.t1;
                // decompression: stream position of column e2 (for the first-plane
                // column, its owner's: the previous block along P2), and its code
                // loaded one column ahead
                uint64_t own = 0;
                if (DECOMP && k2) {
                    own = owner_pos_sweep2(a, g, bc, a.perm[2], m0 - k0) + rk1;
                    if (own >= a.ncodes) {
                        atomicExch(a.err, 1);
                        own = 0;
                    }
                }
                auto dpos = [&](int e2) -> uint64_t {
                    const int ec = e2 < h2 ? e2 : h2 - 1;
                    return ec >= k2 ? base + (uint64_t)(pb + ec * g.t1) : own;
                };
                uint64_t npos = 0;
                int ncode = a.radius;
                if (DECOMP) {
                    npos = dpos(half);
                    if (act) ncode = codes[npos];
                }
                for (int e2b = 0; e2b < h2; e2b += 2) {
                    const int e2 = e2b + half;
                    const bool in = act && e2 < h2;
                    const int ec = e2 < h2 ? e2 : h2 - 1;
                    const float pred = eval_stencil<CUB>(S2, Xs + 2 * ec);
                    const int off = pb + ec * g.t1;
                    float *xp = Xs + m1 * FX + 2 * ec;
                    float v;
                    if (!DECOMP) {
                        v = finest_point(*xp, pred, a, in && ec >= k2, cb + off, ub + off);
                    } else {
                        const uint64_t pos = npos;
                        const int code = ncode;
                        if (e2b + 2 < h2) {
                            npos = dpos(e2 + 2);
                            if (act) ncode = codes[npos];
                        }
                        v = recover_point<float, 1>(pred, code, pos, a, zpos, nz, unpred);
                    }
                    if (in) *xp = v;
                }
            }
            __syncwarp();
            // sweep 3: targets (m0, m1, 2t+1) of the emitted rows, lines along P2
            if (g.t2 > 0) {
                const bool act = t < g.t2;
                const int m2 = act ? 2 * t + 1 : 1;
                const Stencil<float> S3 = make_stencil<float>(m2, n2, cubic, 1, 0);
                const int rk2 = line_rank(m2, n2, cubic);
                const int hr = (w1 + 1) >> 1;  // rows per half-warp
                const int pb = (int)(g.c1 + g.c2) + (m0 - k0) * w1 * g.t2 + rk2;
                // decompression: each code loaded one row ahead
                int ncode = a.radius;
                if (DECOMP && act && hr > 0) ncode = cb[pb + min(half * hr, w1 - 1) * g.t2];
                for (int it = 0; it < hr; it++) {
                    const int rho = it + half * hr;
                    const bool in = act && rho < w1;
                    const int rc = rho < w1 ? rho : w1 - 1;
                    const float *row = Xs + (k1 + rc) * FX;
                    const float pred = eval_stencil<CUB>(S3, row);
                    const int off = pb + rc * g.t2;
                    if (!DECOMP) {
                        finest_point(row[m2], pred, a, in, cb + off, ub + off);
                    } else {
                        const int code = ncode;
                        if (act && it + 1 < hr) ncode = cb[pb + min(rho + 1, w1 - 1) * g.t2];
                        const float v = recover_point<float, 1>(pred, code, base + off, a, zpos, nz, unpred);
                        if (in) Xs[(k1 + rc) * FX + m2] = v;
                    }
                }
            }
            if (DECOMP && w2 > 0) {
                // the plane's emitted rows and columns back to W, coarse points
                // (written by earlier levels) left alone
                __syncwarp();
                float *dst = wb + (int64_t)m0 * G0;
                for (int m1 = k1; m1 < n1; m1++) {
                    float *drow = dst + (int64_t)m1 * G1;
                    const float *srow = Xs + m1 * FX;
                    const bool odd_row = (m0 | m1) & 1;  // no coarse point in the row
                    for (int m2 = k2 + lane; m2 < n2; m2 += 32)
                        if (odd_row || (m2 & 1)) drow[m2] = srow[m2];
                }
            }
        }
    }
    if (DECOMP) return;
    __syncthreads();
    // sweep-1 codes of the block, 16 bytes per store where aligned
    const int cnt = (int)g.c1;
    const int a0 = (8 - sh1) & 7;
    const int nbody = cnt > a0 ? (cnt - a0) >> 3 : 0;
    const int tail0 = a0 + (nbody << 3);
    for (int i = tid; i < cnt; i += blockDim.x)
        if (i < a0 || i >= tail0) cb[i] = stage[sh1 + i];
    for (int j = tid; j < nbody; j += blockDim.x) {
        const int i = a0 + (j << 3);
        *reinterpret_cast<uint4 *>(cb + i) = *reinterpret_cast<const uint4 *>(stage + sh1 + i);
    }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return (EncodeTiledFn) nullptr;
        return (EncodeTiledFn)p;
    }();
    return fn;
}

}  // namespace

bool finest_eligible(const LevelArgs &a, bool decomp, const void *X, size_t elem) {
    // block begins along the contiguous axis are TMA x coordinates: 16-byte
    // multiples, so the block edge is a multiple of 4 values
    if (elem != 4 || a.s != 1 || a.bs > 32 || (a.bs & 3) || a.write_back || !a.fast || a.trim != 0) return false;
    if (a.perm[2] != 2 || a.perm[0] > 1 || a.perm[1] > 1) return false;
    if (a.dims[0] < FROWS || a.dims[1] < FROWS || a.dims[2] < FX || (a.dims[2] & 3)) return false;
    if (a.dims[0] * a.dims[1] * a.dims[2] >= ((int64_t)1 << 31)) return false;
    if (decomp) return true;
    if (((uintptr_t)X & 15) != 0) return false;
    return encode_tiled() != nullptr;
}

cudaError_t launch_finest(const LevelArgs &a, int64_t nblocks, bool decomp, const float *X, float *W,
                          uint16_t *codes, float *scratch, const uint64_t *zpos, uint64_t nz, const float *unpred,
                          cudaStream_t st) {
    CUtensorMap tm;
    std::memset(&tm, 0, sizeof(tm));
    if (!decomp) {
        const cuuint64_t gdim[3] = {(cuuint64_t)a.dims[2], (cuuint64_t)a.dims[1], (cuuint64_t)a.dims[0]};
        const cuuint64_t gstride[2] = {(cuuint64_t)a.dims[2] * 4, (cuuint64_t)(a.dims[1] * a.dims[2]) * 4};
        // the plane of P0 index m0: rows along P1, FX values along axis 2
        const cuuint32_t box[3] = {(cuuint32_t)FX, a.perm[0] == 0 ? (cuuint32_t)FROWS : 1u,
                                   a.perm[0] == 0 ? 1u : (cuuint32_t)FROWS};
        const cuuint32_t estride[3] = {1, 1, 1};
        CUresult r = encode_tiled()(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(X), gdim, gstride,
                                    box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
    }
    void (*k)(LevelArgs, const CUtensorMap, float *, uint16_t *, float *, const uint64_t *, uint64_t, const float *);
    if (decomp) k = a.cubic ? k_finest<true, 1> : k_finest<true, 0>;
    else k = a.cubic ? k_finest<false, 1> : k_finest<false, 0>;
    cudaError_t e = allow_dynamic_smem((const void *)k);
    if (e != cudaSuccess) return e;
    k<<<(unsigned)nblocks, FW * 32, FSMEM, st>>>(a, tm, W, codes, scratch, zpos, nz, unpred);
    return cudaGetLastError();
}

}  // namespace faz
