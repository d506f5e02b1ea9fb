// blocked.cu - ALGO_INTERP_BLOCKED (SZ_compress_Interp_blocked,
// include/QoZ/api/impl/SZInterp.hpp:3021-3500) and the streams it writes:
// SZInterpolationCompressor::compress_block / decompress_block
// (include/QoZ/compressor/SZInterpolationCompressor.hpp:533-781, 201-323)
// for 3-D fields; and ::compress / ::decompress (lines 324-470, 42-199) with
// a fixBlockSize that leaves the coarse lattice (not a multiple of 2^levels),
// where the same block loop runs with the level's interpolator and direction
// for every block (1-D and 2-D fields embedded as 3-D with leading axes of
// extent 1).
//
// Every level is cut into blocks of interpBlockSize points (not scaled by
// the level stride).  Compressing, each block first runs every candidate of
// {linear, cubic} x {direction 0, direction N!-1} on its sample region in
// tuning mode 2 (summed |value - prediction|, reconstruction written, no codes
// kept), restores the region, and compresses itself with the candidate of the
// first smallest loss; the stream records one interpolator and direction per
// block.  The interpolation of a block is block_interpolation's three sweeps
// (block_interpolation_block3d with crossBlock 0 is the same loop nest).
//
// Dependencies.  A block writes the targets of its box less its first planes
// (its lines start one step past them) and reads its whole box, so it reads
// what the blocks one lower on some axes wrote on the shared faces at the same
// level, with candidates of their own.  The blocks of a level therefore run
// as a wavefront over block anti-diagonals bx + by + bz (every writer a block
// reads from lies on an earlier one): one launch per diagonal, one CTA per
// block.  At the level whose stride equals the block edge this carries a
// chain of corner points across blocks; above it every line of a block holds
// a single point, nothing is coded, and every block records the first
// candidate.
//
// A CTA works on the field in global memory: threads take the lines of a
// sweep, each line walked in the reference's point order; a trial's loss is
// summed per line by its thread and then over the lines in loop-nest order by
// one thread, the nesting of the reference's sums (block_interpolation_1d's
// own total, added up by block_interpolation), so the choices are the
// reference's.  Targets take their original values from X and the values
// they are predicted from from W (the reconstruction), so a trial's writes to
// W are never read by another trial or by the compression that follows.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
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

constexpr int kBlkThreads = 256;
constexpr int kBlkMaxEdge = 64;  // largest interpBlockSize on the GPU path

// One level of the block-wise compressor.
struct BlkLevel {
    int64_t dims[3], offs[3];
    int64_t s;        // lattice stride of the level
    int64_t B;        // block edge (interpBlockSize)
    int64_t sbs;      // trial sample edge
    int64_t nb[3];    // blocks per axis
    int perm[6][3];   // direction permutations (lexicographic)
    int ndir;         // N! = 6
    LevelArgs q;      // the level's quantiser (eb, radius, trimToZero, float fast path)
    const uint64_t *block_off;  // first code position of each block at this level
    uint8_t *ops, *dirs;        // per block: chosen (compressing) or given (decompressing)
    int *err;                   // set when a decoded choice is out of range
};

// block_interpolation_1d (SZInterpolationCompressor.hpp:1306-1417) over one
// line: first point at W / X offset o0, n points stride st.  MODE 0
// compresses (codes from pos), 1 is tuning mode 2 (returns the line's summed
// |value - prediction|), 2 decompresses.
template <typename T, int MODE>
__device__ double blk_line(const BlkLevel &a, const T *__restrict__ X, T *__restrict__ W, int64_t o0, int64_t st,
                           int64_t n, bool cubic, uint64_t pos, uint16_t *__restrict__ codes, T *__restrict__ scratch,
                           const uint64_t *__restrict__ zpos, uint64_t nz, const T *__restrict__ unpred) {
    double e = 0;
    if (n <= 1) return e;
    auto put = [&](int64_t i, T pred) {
        const int64_t o = o0 + i * st;
        if (MODE == 2) {
            W[o] = recover_point<T, 0>(pred, (int)codes[pos], pos, a.q, zpos, nz, unpred);
            pos++;
            return;
        }
        T v = X[o], uval;
        if (MODE == 1) e += (double)(T)fabs((double)(T)(v - pred));
        const int code = quant_point<T, 0>(v, pred, a.q, uval);
        if (MODE == 0) {
            codes[pos] = (uint16_t)code;
            if (code == 0) scratch[pos] = uval;
            pos++;
        }
        W[o] = v;
    };
    auto w = [&](int64_t i) -> T { return W[o0 + i * st]; };
    if (!cubic || n < 5) {
        for (int64_t i = 1; i + 1 < n; i += 2) put(i, i_linear<T>(w(i - 1), w(i + 1)));
        if (n % 2 == 0) {
            const int64_t i = n - 1;
            if (n < 4) put(i, w(i - 1));
            else put(i, linear1_any<T>(w(i - 3), w(i - 1)));
        }
    } else {
        int64_t i;
        for (i = 3; i + 3 < n; i += 2) put(i, i_cubic<T>(w(i - 3), w(i - 1), w(i + 1), w(i + 3)));
        put(1, i_quad1<T>(w(0), w(2), w(4)));
        put(i, i_quad2<T>(w(i - 3), w(i - 1), w(i + 1)));
        if (n % 2 == 0) put(n - 1, i_quad3<T>(w(n - 6), w(n - 4), w(n - 2)));
    }
    return e;
}

// block_interpolation for 3-D (SZInterpolationCompressor.hpp:3143-3360) on the
// block [b, e] with permutation perm, all threads of the CTA.  Trial mode
// leaves each line's loss in lsum (loop-nest order) and returns the number
// of lines.
template <typename T, int MODE>
__device__ int64_t blk_pass(const BlkLevel &a, const T *__restrict__ X, T *__restrict__ W, const int64_t *b,
                            const int64_t *e, const int *perm, bool cubic, uint64_t pos0, uint16_t *__restrict__ codes,
                            T *__restrict__ scratch, const uint64_t *__restrict__ zpos, uint64_t nz,
                            const T *__restrict__ unpred, double *lsum) {
    const int64_t s = a.s;
    int64_t line_base = 0;
    uint64_t code_base = pos0;
    for (int d = 0; d < 3; d++) {
        const int ad = perm[d];
        int oax[2], k = 0;
        int64_t step[2];
        for (int p = 0; p < 3; p++) {
            if (p == d) continue;
            oax[k] = perm[p];
            step[k] = p < d ? s : 2 * s;
            k++;
        }
        int64_t start[2], cnt[2];
        for (int j = 0; j < 2; j++) {
            const int ax = oax[j];
            start[j] = b[ax] ? b[ax] + step[j] : 0;
            cnt[j] = start[j] > e[ax] ? 0 : (e[ax] - start[j]) / step[j] + 1;
        }
        const int64_t n = (e[ad] - b[ad]) / s + 1;
        const int64_t tpl = n / 2;
        const int64_t nlines = cnt[0] * cnt[1];
        for (int64_t l = threadIdx.x; l < nlines; l += blockDim.x) {
            const int64_t c0 = start[0] + (l / cnt[1]) * step[0], c1 = start[1] + (l % cnt[1]) * step[1];
            const int64_t o0 = b[ad] * a.offs[ad] + c0 * a.offs[oax[0]] + c1 * a.offs[oax[1]];
            const double le = blk_line<T, MODE>(a, X, W, o0, s * a.offs[ad], n, cubic,
                                                code_base + (uint64_t)(l * tpl), codes, scratch, zpos, nz, unpred);
            if (MODE == 1) lsum[line_base + l] = le;
        }
        code_base += (uint64_t)(nlines * tpl);
        line_base += nlines;
        __syncthreads();
    }
    return line_base;
}

// One block of a level.  KIND 0: trials, then compression with the chosen
// candidate; 1: compression with the candidate in ops / dirs; 2:
// decompression with it.
template <typename T, int KIND>
__device__ void blk_block(const BlkLevel &a, int64_t blk, const T *__restrict__ X, T *__restrict__ W,
                          uint16_t *__restrict__ codes, T *__restrict__ scratch, const uint64_t *__restrict__ zpos,
                          uint64_t nz, const T *__restrict__ unpred, double *lsum) {
    __shared__ int s_choice[2];
    const int64_t bz = blk % a.nb[2], by = (blk / a.nb[2]) % a.nb[1], bx = blk / (a.nb[2] * a.nb[1]);
    const int64_t bidx[3] = {bx, by, bz};
    int64_t b[3], e[3];
    for (int i = 0; i < 3; i++) {
        b[i] = bidx[i] * a.B;
        e[i] = std::min<int64_t>(b[i] + a.B, a.dims[i] - 1);
    }
    int op, dir;
    if (KIND != 0) {
        op = a.ops[blk];
        dir = a.dirs[blk];
        if (op > 1 || dir >= a.ndir) {
            if (threadIdx.x == 0) *a.err = 1;
            return;
        }
    } else {
        int64_t se[3];
        for (int i = 0; i < 3; i++) se[i] = std::min<int64_t>(b[i] + a.sbs, a.dims[i] - 1);
        // candidates in the reference's order; the first smallest loss wins,
        // cubic with direction 0 when no loss is below DBL_MAX
        double best = DBL_MAX;
        int bop = 1, bdir = 0;
        for (int c = 0; c < 4; c++) {
            const int cop = c / 2, cdir = (c & 1) ? a.ndir - 1 : 0;
            const int64_t nl = blk_pass<T, 1>(a, X, W, b, se, a.perm[cdir], cop == 1, 0, nullptr, nullptr, nullptr,
                                              0, nullptr, lsum);
            if (threadIdx.x == 0) {
                double loss = 0;
                for (int64_t l = 0; l < nl; l++) loss += lsum[l];
                if (loss < best) {
                    best = loss;
                    bop = cop;
                    bdir = cdir;
                }
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            s_choice[0] = bop;
            s_choice[1] = bdir;
            a.ops[blk] = (uint8_t)bop;
            a.dirs[blk] = (uint8_t)bdir;
        }
        __syncthreads();
        op = s_choice[0];
        dir = s_choice[1];
    }
    if (KIND == 2)
        blk_pass<T, 2>(a, X, W, b, e, a.perm[dir], op == 1, a.block_off[blk], codes, scratch, zpos, nz, unpred, lsum);
    else
        blk_pass<T, 0>(a, X, W, b, e, a.perm[dir], op == 1, a.block_off[blk], codes, scratch, zpos, nz, unpred, lsum);
    __syncthreads();
}

// The blocks of one anti-diagonal: block list[first + blockIdx.x].
template <typename T, int KIND>
__global__ void __launch_bounds__(kBlkThreads)
    k_blk_level(BlkLevel a, const int64_t *__restrict__ list, int64_t first, const T *__restrict__ X,
                T *__restrict__ W, uint16_t *__restrict__ codes, T *__restrict__ scratch,
                const uint64_t *__restrict__ zpos, uint64_t nz, const T *__restrict__ unpred) {
    extern __shared__ __align__(16) unsigned char blk_smem[];
    double *lsum = reinterpret_cast<double *>(blk_smem);
    blk_block<T, KIND>(a, list[first + blockIdx.x], X, W, codes, scratch, zpos, nz, unpred, lsum);
}

// Host plan of the block-wise levels.
struct BlkPlan {
    uint64_t num = 0;
    int levels = 0, top = 0;
    bool anchor = false;
    int64_t na[3] = {1, 1, 1};
    uint64_t nanchor = 1;
    int64_t nb[3] = {1, 1, 1};
    uint64_t nblocks = 0;
    std::vector<uint64_t> block_off;    // levels top..1, blocks in order
    std::vector<int64_t> diag_list;     // block ids sorted by anti-diagonal
    std::vector<int64_t> diag_first;    // first index of each diagonal (+ end)
};

// Codes one block holds at stride s (block_interpolation's loop counts).
uint64_t block_codes(const int64_t *b, const int64_t *e, int64_t s, const int *perm) {
    uint64_t total = 0;
    for (int d = 0; d < 3; d++) {
        const int ad = perm[d];
        uint64_t lines = 1;
        for (int p = 0; p < 3; p++) {
            if (p == d) continue;
            const int ax = perm[p];
            const int64_t step = p < d ? s : 2 * s;
            const int64_t start = b[ax] ? b[ax] + step : 0;
            lines *= start > e[ax] ? 0 : (uint64_t)((e[ax] - start) / step + 1);
        }
        total += lines * (uint64_t)(((e[ad] - b[ad]) / s + 1) / 2);
    }
    return total;
}

BlkPlan make_blk_plan(const uint64_t *dims, uint64_t maxStep, int B) {
    BlkPlan p;
    p.num = dims[0] * dims[1] * dims[2];
    for (int i = 0; i < 3; i++) p.levels = std::max(p.levels, ceil_log2(dims[i]));
    if (maxStep > 0) {
        // SZInterpolationCompressor::init (lines 820-852) with an anchor grid
        if (maxStep & (maxStep - 1)) throw Fail{FAZ_ERR_UNSUPPORTED, "maxStep must be a power of two on the GPU path"};
        p.anchor = true;
        p.levels += 1;
        int lm = 0;
        while (((uint64_t)1 << (lm + 1)) <= maxStep) lm++;
        lm += 1;
        if (lm <= p.levels) p.levels = lm;
        p.nanchor = 1;
        for (int i = 0; i < 3; i++) {
            p.na[i] = (int64_t)((dims[i] - 1) / maxStep + 1);
            p.nanchor *= (uint64_t)p.na[i];
        }
    }
    p.top = p.anchor ? p.levels - 1 : p.levels;
    p.nblocks = 1;
    for (int i = 0; i < 3; i++) {
        p.nb[i] = (int64_t)((dims[i] - 1) / (uint64_t)B + 1);
        p.nblocks *= (uint64_t)p.nb[i];
    }
    // every direction visits the same points; direction 0 counts them
    const int perm0[3] = {0, 1, 2};
    uint64_t pos = p.nanchor;
    for (int level = p.top; level > 0; level--) {
        const int64_t s = (int64_t)1 << (level - 1);
        for (uint64_t blk = 0; blk < p.nblocks; blk++) {
            const int64_t bz = (int64_t)blk % p.nb[2], by = ((int64_t)blk / p.nb[2]) % p.nb[1],
                          bx = (int64_t)blk / (p.nb[2] * p.nb[1]);
            const int64_t bi[3] = {bx, by, bz};
            int64_t b[3], e[3];
            for (int i = 0; i < 3; i++) {
                b[i] = bi[i] * B;
                e[i] = std::min<int64_t>(b[i] + B, (int64_t)dims[i] - 1);
            }
            p.block_off.push_back(pos);
            pos += block_codes(b, e, s, perm0);
        }
    }
    // With an anchor grid and blocks smaller than maxStep, the level whose
    // stride equals the block edge codes the anchor points a second time, so
    // the stream holds more codes than points, and the reference's decoder
    // decodes only as many codes as points (its last points then read past
    // its list); such streams are not produced here.
    if (pos != p.num)
        throw Fail{FAZ_ERR_UNSUPPORTED, "blocks smaller than maxStep code the anchor points twice, which the "
                                        "reference cannot decode; not implemented"};
    // anti-diagonals bx + by + bz
    const int64_t nd = p.nb[0] + p.nb[1] + p.nb[2] - 2;
    std::vector<std::vector<int64_t>> by_d((size_t)nd);
    for (uint64_t blk = 0; blk < p.nblocks; blk++) {
        const int64_t bz = (int64_t)blk % p.nb[2], by = ((int64_t)blk / p.nb[2]) % p.nb[1],
                      bx = (int64_t)blk / (p.nb[2] * p.nb[1]);
        by_d[(size_t)(bx + by + bz)].push_back((int64_t)blk);
    }
    for (auto &v : by_d) {
        p.diag_first.push_back((int64_t)p.diag_list.size());
        p.diag_list.insert(p.diag_list.end(), v.begin(), v.end());
    }
    p.diag_first.push_back((int64_t)p.diag_list.size());
    return p;
}

template <typename T>
BlkLevel level_args(const BlkPlan &p, const uint64_t *dims, int B, int bwsbs, int level, double eb, double alpha,
                    double beta, int radius, int trim) {
    BlkLevel a;
    std::memset(&a, 0, sizeof(a));
    for (int i = 0; i < 3; i++) {
        a.dims[i] = (int64_t)dims[i];
        a.nb[i] = p.nb[i];
    }
    a.offs[2] = 1;
    a.offs[1] = a.dims[2];
    a.offs[0] = a.dims[1] * a.dims[2];
    a.s = (int64_t)1 << (level - 1);
    a.B = B;
    // blockwiseSampleBlockSize at the two finest levels, the block above
    // (compress_block, SZInterpolationCompressor.hpp:616-618)
    a.sbs = level <= 2 ? bwsbs : B;
    if (a.sbs > B) a.sbs = B;
    const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    std::memcpy(a.perm, perms, sizeof(perms));
    a.ndir = 6;
    a.q.eb = level_eb(eb, alpha, beta, level);
    a.q.recip = 1.0 / a.q.eb;
    a.q.radius = radius;
    a.q.trim = trim;
    set_fast_path<T>(a.q);
    return a;
}

// Every level after the first point / anchors.  ops / dirs: one entry per
// block per level (device), written by KIND 0, read by KIND 1 and 2.
template <typename T, int KIND>
void blk_levels(const BlkPlan &p, const uint64_t *dims3, int B, int bwsbs, double eb, double alpha, double beta,
                int radius, int trim, const T *X, T *W, uint16_t *codes, T *scratch, const uint64_t *zpos, uint64_t nz,
                const T *unpred, uint8_t *ops, uint8_t *dirs, int *derr, DevMem &m, cudaStream_t st,
                Counter &launches) {
    uint64_t *boff = m.alloc<uint64_t>(p.block_off.size());
    CK(cudaMemcpyAsync(boff, p.block_off.data(), p.block_off.size() * 8, cudaMemcpyHostToDevice, st));
    int64_t *dlist = m.alloc<int64_t>(p.diag_list.size());
    CK(cudaMemcpyAsync(dlist, p.diag_list.data(), p.diag_list.size() * 8, cudaMemcpyHostToDevice, st));
    auto k = k_blk_level<T, KIND>;
    // trial line sums: at most 3 (B + 1)^2 lines per block
    const size_t smem = KIND == 0 ? (size_t)3 * (B + 1) * (B + 1) * sizeof(double) : 16;
    CK(allow_dynamic_smem((const void *)k));
    int li = 0;
    for (int level = p.top; level > 0; level--, li++) {
        BlkLevel a = level_args<T>(p, dims3, B, bwsbs, level, eb, alpha, beta, radius, trim);
        a.block_off = boff + (size_t)li * p.nblocks;
        a.ops = ops + (size_t)li * p.nblocks;
        a.dirs = dirs + (size_t)li * p.nblocks;
        a.err = derr;
        if (a.s > B) {
            // every line of a block holds one point: no codes, every trial's
            // loss 0, so the first candidate (linear, direction 0) is recorded
            if (KIND == 0) {
                CK(cudaMemsetAsync(a.ops, 0, p.nblocks, st));
                CK(cudaMemsetAsync(a.dirs, 0, p.nblocks, st));
            }
            continue;
        }
        for (size_t d = 0; d + 1 < p.diag_first.size(); d++) {
            const int64_t f = p.diag_first[d], cnt = p.diag_first[d + 1] - f;
            if (cnt <= 0) continue;
            k<<<(unsigned)cnt, kBlkThreads, smem, st>>>(a, dlist, f, X, W, codes, scratch, zpos, nz, unpred);
            launches(cudaGetLastError());
        }
    }
}

void check_blocked(int N, int B, int bwsbs, int cross, int border) {
    if (N != 3) throw Fail{FAZ_ERR_UNSUPPORTED, "ALGO_INTERP_BLOCKED is defined for 3-D data"};
    if (B < 2 || B > kBlkMaxEdge || (B & (B - 1)))
        throw Fail{FAZ_ERR_UNSUPPORTED, "block-wise interpolation needs interpBlockSize a power of two in [2, 64] on "
                                        "the GPU path"};
    if (bwsbs < 1) throw Fail{FAZ_ERR_ARG, "bad blockwiseSampleBlockSize"};
    if (cross) throw Fail{FAZ_ERR_UNSUPPORTED, "crossBlock is not implemented"};
    if (border) throw Fail{FAZ_ERR_UNSUPPORTED, "block orders other than 0 are not implemented"};
}

// 1-D / 2-D fields embedded as 3-D with leading axes of extent 1, their
// directions as the 3-D permutations that keep those axes first
void embed(int N, const uint64_t *dims, uint64_t *dims3) {
    const int e = 3 - N;
    for (int i = 0; i < 3; i++) dims3[i] = 1;
    for (int i = 0; i < N; i++) dims3[e + i] = dims[i];
}

int embed_dir(int N, int dir) {
    if (N == 3) return dir;
    if (N == 2) return dir == 0 ? 0 : 1;  // (0, 1, 2) and (0, 2, 1)
    return 0;
}

void anchor_launch_args(const BlkPlan &p, const uint64_t *dims3, uint64_t maxStep, int N, int64_t *step,
                        int64_t *offs) {
    const int e = 3 - N;
    for (int i = 0; i < 3; i++) step[i] = i < e ? 1 : (int64_t)maxStep;
    offs[0] = (int64_t)(dims3[1] * dims3[2]);
    offs[1] = (int64_t)dims3[2];
    offs[2] = 1;
    (void)p;
}

}  // namespace

// SZ_compress_Interp_blocked up to compress_block: the Config it leaves
// (ALGO_INTERP with block-wise tuning, blocks of interpBlockSize).  The
// alpha/beta search it runs for autoTuningRate > 0 is not implemented.
void blocked_prepare(faz_config &c) {
    if (c.N != 3) throw Fail{FAZ_ERR_UNSUPPORTED, "ALGO_INTERP_BLOCKED is defined for 3-D data"};
    if (c.autoTuningRate > 0)
        throw Fail{FAZ_ERR_UNSUPPORTED, "ALGO_INTERP_BLOCKED with autoTuningRate > 0 is not implemented"};
    c.cmprAlgo = FAZ_ALGO_INTERP;
    if (c.interpBlockSize <= 0) c.interpBlockSize = 32;
    int max_level = (int)std::log2((double)c.interpBlockSize) + 1;
    if (c.maxStep > 0) {
        const int t = (int)std::log2((double)c.maxStep);
        if (t < max_level) max_level = t;
    }
    if (c.levelwisePredictionSelection > max_level) c.levelwisePredictionSelection = max_level;
    if (c.blockwiseSampleBlockSize == 0) c.blockwiseSampleBlockSize = c.interpBlockSize;
    if (c.blockwiseSampleBlockSize < 4) c.blockwiseSampleBlockSize = 4;
    c.fixBlockSize = c.interpBlockSize;
    c.blockwiseTuning = 1;
    check_blocked(c.N, c.interpBlockSize, c.blockwiseSampleBlockSize, c.crossBlock, c.blockOrder);
}

// Whether a fixBlockSize keeps every level's blocks on the coarse lattice
// (fixBlockSize a multiple of 2^top), the case the level kernels cover.
bool fixbs_aligned(int N, const uint64_t *dims, uint64_t maxStep, int fixbs) {
    uint64_t dims3[3];
    embed(N, dims, dims3);
    int levels = 0;
    for (int i = 0; i < 3; i++) levels = std::max(levels, ceil_log2(dims3[i]));
    if (maxStep > 0) {
        levels += 1;
        int lm = 0;
        while (((uint64_t)1 << (lm + 1)) <= maxStep) lm++;
        lm += 1;
        if (lm <= levels) levels = lm;
        levels -= 1;
    }
    return levels <= 0 || fixbs % (1 << std::min(levels, 30)) == 0;
}

// compress_block up to its codes: first point / anchors, then every level
// block by block.  codes / scratch hold the codes in stream order and the
// unpredictable values at their code positions; ops / dirs (host) receive
// the per-block choices, levels coarse to fine.
template <typename T>
void blocked_codes(const faz_config &c, const T *dX, T *W, uint16_t *codes, T *scratch, DevMem &m, cudaStream_t st,
                   Counter &launches, std::vector<uint8_t> &ops, std::vector<uint8_t> &dirs) {
    check_blocked(c.N, c.interpBlockSize, c.blockwiseSampleBlockSize, c.crossBlock, c.blockOrder);
    const BlkPlan p = make_blk_plan(c.dims, c.maxStep, c.interpBlockSize);
    const double eb = c.absErrorBound;
    const int radius = c.quantbinCnt / 2;
    if (!p.anchor) {
        launches(launch_first_point<T>(false, dX, W, codes, scratch, eb, radius, c.trimToZero, nullptr, 0, nullptr, st));
    } else {
        int64_t step[3], offs[3];
        anchor_launch_args(p, c.dims, c.maxStep, 3, step, offs);
        launches(launch_anchors<T>(false, dX, W, codes, scratch, nullptr, p.na, step, offs, st));
    }
    const size_t nops = (size_t)p.top * p.nblocks;
    uint8_t *dops = m.alloc<uint8_t>(2 * nops);
    int *derr = m.alloc<int>(1);
    CK(cudaMemsetAsync(derr, 0, 4, st));
    blk_levels<T, 0>(p, c.dims, c.interpBlockSize, c.blockwiseSampleBlockSize, eb, c.alpha, c.beta, radius,
                     c.trimToZero, dX, W, codes, scratch, nullptr, 0, nullptr, dops, dops + nops, derr, m, st,
                     launches);
    ops.resize(nops);
    dirs.resize(nops);
    uint8_t *hb = t_pin_small.get(2 * nops + 8);
    if (nops) CK(cudaMemcpyAsync(hb, dops, 2 * nops, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::memcpy(ops.data(), hb, nops);
    std::memcpy(dirs.data(), hb + nops, nops);
}

namespace {

// Device choice lists of a fixed-block stream: every block of a level takes
// the level's interpolator and direction (the level lists, or interpAlgo /
// interpDirection).
uint8_t *level_choices(const BlkPlan &p, int N, int interp, int dir, const std::vector<uint8_t> &il,
                       const std::vector<uint8_t> &dl, DevMem &m, cudaStream_t st) {
    const size_t nops = (size_t)p.top * p.nblocks;
    std::vector<uint8_t> h(2 * nops + 1);
    int li = 0;
    for (int level = p.top; level > 0; level--, li++) {
        int op = interp, d = dir;
        if (!il.empty()) {
            const size_t k = (size_t)(level - 1) < il.size() ? (size_t)(level - 1) : il.size() - 1;
            op = il[k];
            d = dl[k];
        }
        const int nd = N == 3 ? 6 : (N == 2 ? 2 : 1);
        if (d < 0 || d >= nd) throw Fail{FAZ_ERR_ARG, "interpolation direction out of range"};
        std::memset(h.data() + (size_t)li * p.nblocks, op == FAZ_INTERP_ALGO_CUBIC ? 1 : 0, p.nblocks);
        std::memset(h.data() + nops + (size_t)li * p.nblocks, embed_dir(N, d), p.nblocks);
    }
    uint8_t *dops = m.alloc<uint8_t>(2 * nops + 1);
    CK(cudaMemcpyAsync(dops, h.data(), 2 * nops, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));  // h leaves scope
    return dops;
}

void check_fixed(int N, int fixbs) {
    if (N < 1 || N > 3) throw Fail{FAZ_ERR_UNSUPPORTED, "fixBlockSize is implemented for 1-D to 3-D data"};
    if (fixbs < 2 || fixbs > kBlkMaxEdge || (fixbs & (fixbs - 1)))
        throw Fail{FAZ_ERR_UNSUPPORTED, "a fixBlockSize that is not a multiple of 2^levels must be a power of two in "
                                        "[2, 64] on the GPU path"};
}

}  // namespace

// SZInterpolationCompressor::compress (lines 324-470) with a fixBlockSize
// that leaves the coarse lattice: blocks of fixBlockSize at every level, the
// level's interpolator and direction for every block.
template <typename T>
void fixed_block_codes(const faz_config &c, const std::vector<uint8_t> &il, const std::vector<uint8_t> &dl,
                       const T *dX, T *W, uint16_t *codes, T *scratch, DevMem &m, cudaStream_t st, Counter &launches) {
    check_fixed(c.N, c.fixBlockSize);
    if (c.crossBlock || c.blockOrder)
        throw Fail{FAZ_ERR_UNSUPPORTED, "crossBlock and other block orders are not implemented"};
    uint64_t dims3[3];
    embed(c.N, c.dims, dims3);
    if (c.maxStep > 0 && c.N < 2) throw Fail{FAZ_ERR_UNSUPPORTED, "an anchor grid needs 2-D or 3-D data"};
    const BlkPlan p = make_blk_plan(dims3, c.maxStep, c.fixBlockSize);
    const double eb = c.absErrorBound;
    const int radius = c.quantbinCnt / 2;
    if (!p.anchor) {
        launches(launch_first_point<T>(false, dX, W, codes, scratch, eb, radius, c.trimToZero, nullptr, 0, nullptr, st));
    } else {
        int64_t step[3], offs[3];
        anchor_launch_args(p, dims3, c.maxStep, c.N, step, offs);
        launches(launch_anchors<T>(false, dX, W, codes, scratch, nullptr, p.na, step, offs, st));
    }
    const size_t nops = (size_t)p.top * p.nblocks;
    uint8_t *dops = level_choices(p, c.N, c.interpAlgo, c.interpDirection, il, dl, m, st);
    int *derr = m.alloc<int>(1);
    CK(cudaMemsetAsync(derr, 0, 4, st));
    blk_levels<T, 1>(p, dims3, c.fixBlockSize, c.fixBlockSize, eb, c.alpha, c.beta, radius, c.trimToZero, dX, W, codes,
                     scratch, nullptr, 0, nullptr, dops, dops + nops, derr, m, st, launches);
}

// decompress_block, or decompress with a fixBlockSize off the coarse
// lattice, after the codes are decoded: first point / anchors, then every
// level with the per-block choices (block-wise streams) or the level's
// interpolator and direction (ops empty).
template <typename T>
void blocked_decompress_levels(int N, const uint64_t *dims, uint64_t maxStep, int B, double eb, double alpha,
                               double beta, int radius, int trim, int interp, int dir,
                               const std::vector<uint8_t> &il, const std::vector<uint8_t> &dl,
                               const std::vector<uint8_t> &ops, const std::vector<uint8_t> &dirs, bool blockwise,
                               const uint16_t *codes, const uint64_t *zpos, uint64_t nz, const T *unpred, T *dOut,
                               DevMem &m, cudaStream_t st, Counter &launches) {
    if (blockwise) check_blocked(N, B, 1, 0, 0);
    else check_fixed(N, B);
    uint64_t dims3[3];
    embed(N, dims, dims3);
    if (maxStep > 0 && N < 2) throw Fail{FAZ_ERR_UNSUPPORTED, "an anchor grid needs 2-D or 3-D data"};
    const BlkPlan p = make_blk_plan(dims3, maxStep, B);
    const size_t nops = (size_t)p.top * p.nblocks;
    uint16_t *cw = const_cast<uint16_t *>(codes);
    if (!p.anchor) {
        launches(launch_first_point<T>(true, nullptr, dOut, cw, nullptr, eb, radius, trim, zpos, nz, unpred, st));
    } else {
        int64_t step[3], offs[3];
        anchor_launch_args(p, dims3, maxStep, N, step, offs);
        launches(launch_anchors<T>(true, nullptr, dOut, cw, nullptr, unpred, p.na, step, offs, st));
    }
    uint8_t *dops;
    if (blockwise) {
        if (ops.size() != nops || dirs.size() != nops)
            throw Fail{FAZ_ERR_FORMAT, "block-wise choice list does not match the blocks"};
        dops = m.alloc<uint8_t>(2 * nops + 1);
        if (nops) {
            CK(cudaMemcpyAsync(dops, ops.data(), nops, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(dops + nops, dirs.data(), nops, cudaMemcpyHostToDevice, st));
        }
    } else {
        dops = level_choices(p, N, interp, dir, il, dl, m, st);
    }
    int *derr = m.alloc<int>(1);
    CK(cudaMemsetAsync(derr, 0, 4, st));
    blk_levels<T, 2>(p, dims3, B, B, eb, alpha, beta, radius, trim, nullptr, dOut, cw, nullptr, zpos, nz, unpred, dops,
                     dops + nops, derr, m, st, launches);
    int *he = (int *)t_pin_small.get(64);
    CK(cudaMemcpyAsync(he, derr, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));  // host lists leave scope
    if (*he) throw Fail{FAZ_ERR_FORMAT, "block-wise choice out of range"};
}

template void blocked_codes<float>(const faz_config &, const float *, float *, uint16_t *, float *, DevMem &,
                                   cudaStream_t, Counter &, std::vector<uint8_t> &, std::vector<uint8_t> &);
template void blocked_codes<double>(const faz_config &, const double *, double *, uint16_t *, double *, DevMem &,
                                    cudaStream_t, Counter &, std::vector<uint8_t> &, std::vector<uint8_t> &);
template void fixed_block_codes<float>(const faz_config &, const std::vector<uint8_t> &, const std::vector<uint8_t> &,
                                       const float *, float *, uint16_t *, float *, DevMem &, cudaStream_t, Counter &);
template void fixed_block_codes<double>(const faz_config &, const std::vector<uint8_t> &, const std::vector<uint8_t> &,
                                        const double *, double *, uint16_t *, double *, DevMem &, cudaStream_t,
                                        Counter &);
template void blocked_decompress_levels<float>(int, const uint64_t *, uint64_t, int, double, double, double, int, int,
                                               int, int, const std::vector<uint8_t> &, const std::vector<uint8_t> &,
                                               const std::vector<uint8_t> &, const std::vector<uint8_t> &, bool,
                                               const uint16_t *, const uint64_t *, uint64_t, const float *, float *,
                                               DevMem &, cudaStream_t, Counter &);
template void blocked_decompress_levels<double>(int, const uint64_t *, uint64_t, int, double, double, double, int, int,
                                                int, int, const std::vector<uint8_t> &, const std::vector<uint8_t> &,
                                                const std::vector<uint8_t> &, const std::vector<uint8_t> &, bool,
                                                const uint16_t *, const uint64_t *, uint64_t, const double *, double *,
                                                DevMem &, cudaStream_t, Counter &);

}  // namespace faz
