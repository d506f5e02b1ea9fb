// qoz.cu - the QoZ tuner (QoZ = 1, the faz tool's -q) on the GPU.
//
// Reference: Tuning with conf.QoZ (include/QoZ/api/impl/SZInterp.hpp:1588-2557),
// sampleBlocks (992-1127), CompressTest (1130-1392), setABwithRelBound
// (1394-1420), init_alphalist / init_betalist (868-933), and
// SZInterpolationCompressor::compress in its tuning modes
// (include/QoZ/compressor/SZInterpolationCompressor.hpp:324-470, 924-978).
//
// The tuner compresses a few sampled (sbs+1)^N blocks many times: with every
// candidate interpolator and direction per level (tuning mode 2: summed
// absolute prediction loss), then with every alpha/beta candidate (tuning
// mode 1: codes, bit rate after Huffman + zstd, PSNR from summed squared
// errors).  On the GPU one launch per level and sweep covers every sampled
// block (one thread per target); each target's error lands at its stream
// position and k_qz_sum adds the errors in the reference's nesting (per line,
// then per level block, then a running total), so the sums and therefore
// the decisions are those of the reference.  The decision logic is the
// reference's, on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <future>
#include <memory>
#include <exception>
#include <string>
#include <vector>

#include "common.cuh"
#include "host.h"
#include "internal.h"
#include "quant.cuh"
#include "tuning_metrics.h"

namespace faz {

size_t zstd_framed_size_host(const uint8_t *p, size_t n);

namespace {

// One level sweep over all sampled blocks.
struct QzSweep {
    int64_t offs[3];       // strides inside a block field (3-D embedding)
    int64_t cpb;           // stream slots per block
    int axis;              // sweep axis
    int oth[2];            // the other axes, outer loop first
    int64_t g[2], cnt[2];  // their grid steps and counts
    int64_t s, n, tpl;     // stride along the axis, points and targets per line
    int64_t seg_off;       // first stream slot of this sweep inside a block
    int cubic;
    int64_t per;           // values per block
};

// target index of rank r in a line of n points (inverse of line_rank)
__device__ __forceinline__ int64_t target_of_rank(int64_t r, int64_t n, int cubic) {
    if (!cubic || n < 5) return 2 * r + 1;
    const int64_t ia = (n & 1) ? n - 2 : n - 3;
    const int64_t cint = (ia - 3) >> 1;
    if (r < cint) return 3 + 2 * r;
    if (r == cint) return 1;
    if (r == cint + 1) return ia;
    return n - 1;
}

// MODE 1: quantise, store code / unpredictable value / squared error;
// MODE 2: store |d - pred|, quantise without keeping anything.
template <typename T, int MODE, int QM>
__global__ void k_qz_sweep(QzSweep w, LevelArgs q, T *__restrict__ data, uint16_t *__restrict__ codes,
                           T *__restrict__ scratch, double *__restrict__ err, uint64_t total) {
    const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const uint64_t lines = (uint64_t)(w.cnt[0] * w.cnt[1]);
    const int64_t r = (int64_t)(idx % (uint64_t)w.tpl);
    const uint64_t L = (idx / (uint64_t)w.tpl) % lines;
    const uint64_t k = idx / ((uint64_t)w.tpl * lines);
    // offsets as scalars: arrays indexed by the sweep's axes (a local one, or
    // the parameter struct's) would be kept in local memory
    auto off = [&](int ax) { return ax == 0 ? w.offs[0] : (ax == 1 ? w.offs[1] : w.offs[2]); };
    const int64_t i = target_of_rank(r, w.n, w.cubic);
    T *d = data + k * (uint64_t)w.per + (int64_t)(L / (uint64_t)w.cnt[1]) * w.g[0] * off(w.oth[0]) +
           (int64_t)(L % (uint64_t)w.cnt[1]) * w.g[1] * off(w.oth[1]) + i * w.s * off(w.axis);
    const int64_t st = w.s * off(w.axis);
    const int64_t n = w.n;
    T pred;
    if (!w.cubic || n < 5) {
        if (i + 1 < n) pred = i_linear(d[-st], d[st]);
        else if (n < 4) pred = d[-st];
        else pred = linear1_any<T>(d[-3 * st], d[-st]);
    } else {
        if (i == 1) pred = i_quad1(d[-st], d[st], d[3 * st]);
        else if (i + 3 < n) pred = i_cubic(d[-3 * st], d[-st], d[st], d[3 * st]);
        else if ((n & 1) == 0 && i == n - 1) pred = i_quad3(d[-5 * st], d[-3 * st], d[-st]);
        else pred = i_quad2(d[-3 * st], d[-st], d[st]);
    }
    const uint64_t pos = k * (uint64_t)w.cpb + (uint64_t)w.seg_off + L * (uint64_t)w.tpl + (uint64_t)r;
    const T orig = *d;
    T v = orig, uval;
    const int code = quant_point<T, QM>(v, pred, q, uval);
    if (MODE == 1) {
        codes[pos] = (uint16_t)code;
        if (code == 0) scratch[pos] = uval;
        const T df = v - orig;
        err[pos] = (double)(T)(df * df);
    } else {
        const T df = orig - pred;
        err[pos] = (double)(df < 0 ? -df : df);
    }
    *d = v;
}

// build_grid in tuning mode 1 (SZInterpolationCompressor.hpp:854-900): the
// maxStep grid from maxStep on, code 0, the value unpredictable.  Axes below
// `e` are the 3-D embedding's leading ones.
template <typename T>
__global__ void k_qz_anchor(const T *__restrict__ data, int64_t per, int64_t cpb, int64_t nax, int64_t nay, int64_t naz,
                            int64_t ms, int e, int64_t o0, int64_t o1, uint16_t *__restrict__ codes,
                            T *__restrict__ scratch, uint64_t total) {
    const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const uint64_t na = (uint64_t)(nax * nay * naz);
    const uint64_t k = idx / na, a = idx % na;
    const int64_t z = (int64_t)(a % (uint64_t)naz), y = (int64_t)((a / (uint64_t)naz) % (uint64_t)nay),
                  x = (int64_t)(a / ((uint64_t)naz * (uint64_t)nay));
    const int64_t cx = e > 0 ? 0 : (x + 1) * ms, cy = e > 1 ? 0 : (y + 1) * ms, cz = (z + 1) * ms;
    const T v = data[k * (uint64_t)per + cx * o0 + cy * o1 + cz];
    codes[k * (uint64_t)cpb + a] = 0;
    scratch[k * (uint64_t)cpb + a] = v;
}

// The first point against prediction 0 (no anchor grid).
template <typename T, int MODE>
__global__ void k_qz_first(LevelArgs q, T *__restrict__ data, int64_t per, int64_t cpb, uint16_t *__restrict__ codes,
                           T *__restrict__ scratch, uint64_t nblk) {
    const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nblk) return;
    T v = data[k * (uint64_t)per], uval;
    const int code = quantize<T>(v, (T)0, q.eb, q.recip, q.radius, q.trim, uval);
    if (MODE == 1) {
        codes[k * (uint64_t)cpb] = (uint16_t)code;
        if (code == 0) scratch[k * (uint64_t)cpb] = uval;
    }
    data[k * (uint64_t)per] = v;
}

struct SumSeg {
    int64_t off;    // first slot
    int64_t lines;  // lines of this sweep
    int64_t tpl;    // targets per line
    int level_end;  // 1 when this is the level's last sweep
};
constexpr int kMaxSegs = 64;
struct SumPlan {
    int nseg;
    int64_t cpb;
    SumSeg seg[kMaxSegs];
};

// Per block: sum of line sums per level block, running total over levels
// (block_interpolation_1d / block_interpolation / compress accumulation).
__global__ void k_qz_sum(SumPlan p, const double *__restrict__ err, double *__restrict__ out, uint64_t nblk) {
    const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nblk) return;
    const double *e = err + k * (uint64_t)p.cpb;
    double total = 0, blk = 0;
    for (int sgi = 0; sgi < p.nseg; sgi++) {
        const SumSeg sg = p.seg[sgi];
        const double *x = e + sg.off;
        for (int64_t l = 0; l < sg.lines; l++) {
            double ls = 0;
            for (int64_t t = 0; t < sg.tpl; t++) ls += x[t];
            blk += ls;
            x += sg.tpl;
        }
        if (sg.level_end) {
            total += blk;
            blk = 0;
        }
    }
    out[k] = total;
}

// q_bins of CompressTest: for each level range, every block's codes of it.
__global__ void k_qz_regroup(const uint16_t *__restrict__ codes, int64_t cpb, const int64_t *__restrict__ rlo,
                             const int64_t *__restrict__ rlen, const int64_t *__restrict__ rout, int nr, uint64_t nblk,
                             uint16_t *__restrict__ out, uint64_t total) {
    const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    // find the range (few of them)
    int g = 0;
    while (g + 1 < nr && idx >= (uint64_t)rout[g + 1]) g++;
    const uint64_t o = idx - (uint64_t)rout[g];
    const uint64_t k = o / (uint64_t)rlen[g], m = o % (uint64_t)rlen[g];
    out[idx] = codes[k * (uint64_t)cpb + (uint64_t)rlo[g] + m];
}

template <typename T>
__global__ void k_qz_gather(const T *__restrict__ X, const int64_t *__restrict__ starts, int64_t d1, int64_t d2,
                            int64_t bsz, int N, T *__restrict__ out, uint64_t total) {
    const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const uint64_t per = N == 3 ? (uint64_t)(bsz * bsz * bsz) : (uint64_t)(bsz * bsz);
    const uint64_t k = idx / per, o = idx % per;
    const int64_t *s = starts + 3 * k;
    uint64_t src;
    if (N == 3) {
        const int64_t z = (int64_t)(o % (uint64_t)bsz), y = (int64_t)((o / (uint64_t)bsz) % (uint64_t)bsz),
                      x = (int64_t)(o / ((uint64_t)bsz * (uint64_t)bsz));
        src = (uint64_t)(x + s[0]) * (uint64_t)(d1 * d2) + (uint64_t)(y + s[1]) * (uint64_t)d2 + (uint64_t)(z + s[2]);
    } else {
        const int64_t y = (int64_t)(o % (uint64_t)bsz), x = (int64_t)(o / (uint64_t)bsz);
        src = (uint64_t)(x + s[0]) * (uint64_t)d2 + (uint64_t)(y + s[1]);
    }
    out[idx] = X[src];
}

// Geometry of a sampled block as an N-D field for the interpolation
// compressor (one interpolation block per level: interpBlockSize >= sbs).
struct QzGeom {
    int N, e;              // dims and 3-D embedding offset
    int64_t bsz, per;
    int64_t offs[3];
    int levels;            // interpolation_level after init()
    bool anchor;
    int64_t ms;
    int64_t na[3];         // anchors per axis in tuning mode 1
    int64_t nanchor;
    int64_t cpb;           // stream slots per block (full run, mode 1)
};

QzGeom make_geom(int N, int64_t bsz, int64_t maxStep) {
    QzGeom g;
    std::memset(&g, 0, sizeof(g));
    g.N = N;
    g.e = 3 - N;
    g.bsz = bsz;
    g.per = 1;
    for (int i = 0; i < N; i++) g.per *= bsz;
    int64_t d3[3] = {1, 1, 1};
    for (int i = 0; i < N; i++) d3[g.e + i] = bsz;
    g.offs[2] = 1;
    g.offs[1] = d3[2];
    g.offs[0] = d3[1] * d3[2];
    g.levels = ceil_log2((uint64_t)bsz);
    g.ms = maxStep;
    if (maxStep > 0) {
        g.anchor = true;
        g.levels += 1;
        int lm = 0;
        while (((uint64_t)1 << (lm + 1)) <= (uint64_t)maxStep) lm++;
        lm += 1;
        if (lm <= g.levels) g.levels = lm;
        for (int i = 0; i < 3; i++) g.na[i] = 1;
        g.nanchor = 1;
        for (int i = 0; i < N; i++) {
            // x = maxStep, 2 maxStep, ... < bsz
            g.na[g.e + i] = bsz > maxStep ? (bsz - 1) / maxStep : 0;
            g.nanchor *= g.na[g.e + i];
        }
    }
    return g;
}

const int P3[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};

// One tuning run over levels [start, end+1] of every sampled block.
struct QzRun {
    int mode;                   // 1 or 2
    int start_level, end_level; // after the reference's clamping
    double eb, alpha, beta;
    int trim;
    int interp, dir;            // when no level list
    const std::vector<uint8_t> *il, *dl;
};

template <typename T>
void qz_run(const QzGeom &g, const QzRun &R, T *work, uint16_t *codes, T *scratch, double *err, uint64_t nblk,
            SumPlan &sp, std::vector<std::pair<int64_t, int64_t>> *level_ranges, cudaStream_t st, Counter &launches) {
    sp.nseg = 0;
    sp.cpb = g.cpb;
    int64_t pos = 0;
    int start = R.start_level;
    if (!g.anchor) {
        LevelArgs q;
        std::memset(&q, 0, sizeof(q));
        q.eb = R.eb;
        q.recip = 1.0 / R.eb;
        q.radius = 32768;
        q.trim = R.trim;
        if (R.mode == 1)
            k_qz_first<T, 1><<<(unsigned)((nblk + 127) / 128), 128, 0, st>>>(q, work, g.per, g.cpb, codes, scratch, nblk);
        else
            k_qz_first<T, 2><<<(unsigned)((nblk + 127) / 128), 128, 0, st>>>(q, work, g.per, g.cpb, codes, scratch, nblk);
        launches(cudaGetLastError());
        pos = 1;
    } else if (start == g.levels) {
        if (R.mode == 1 && g.nanchor > 0) {
            const uint64_t total = (uint64_t)g.nanchor * nblk;
            // axis strides of the embedded field for the anchor coordinates
            k_qz_anchor<T><<<(unsigned)((total + 127) / 128), 128, 0, st>>>(
                work, g.per, g.cpb, g.na[0], g.na[1], g.na[2], g.ms, g.e, g.offs[0], g.offs[1], codes, scratch, total);
            launches(cudaGetLastError());
        }
        pos = R.mode == 1 ? g.nanchor : 0;
        start--;
    }
    if (level_ranges) level_ranges->clear();
    int64_t range_lo = 0;
    // stream slots of levels above `start` (full-run layout) for mode 2
    // runs that begin below the top
    {
        int64_t p0 = g.anchor ? g.nanchor : 1;
        for (int level = g.levels - (g.anchor ? 1 : 0); level > start; level--) {
            const int64_t s = (int64_t)1 << (level - 1);
            int64_t lvl = 0;
            for (int sw = 0; sw < g.N; sw++) {
                int64_t lines = 1;
                // line counts do not depend on the direction's axis order
                for (int u = 0; u < g.N; u++)
                    if (u != sw) lines *= (g.bsz - 1) / (u < sw ? s : 2 * s) + 1;
                lvl += lines * (((g.bsz - 1) / s + 1) / 2);
            }
            p0 += lvl;
        }
        if (R.mode == 2) pos = p0;
    }
    for (int level = start; level > R.end_level; level--) {
        LevelArgs q;
        std::memset(&q, 0, sizeof(q));
        q.eb = level_eb(R.eb, R.alpha, R.beta, level);
        q.recip = 1.0 / q.eb;
        q.radius = 32768;
        q.trim = R.trim;
        set_fast_path<T>(q);
        const bool straight = sizeof(T) == 4 && q.fast && q.trim == 0;
        int interp = R.interp, dir = R.dir;
        if (R.il && !R.il->empty()) {
            const size_t li = (size_t)(level - 1) < R.il->size() ? (size_t)(level - 1) : R.il->size() - 1;
            interp = (*R.il)[li];
            dir = (*R.dl)[li];
        }
        int perm[3] = {0, 1, 2};
        if (g.N == 2) {
            if (dir != 0) {
                perm[0] = 1;
                perm[1] = 0;
            }
        } else if (g.N == 3) {
            if (dir < 0 || dir > 5) throw Fail{FAZ_ERR_ARG, "interpolation direction out of range"};
            for (int i = 0; i < 3; i++) perm[i] = P3[dir][i];
        }
        const int64_t s = (int64_t)1 << (level - 1);
        for (int d = 0; d < g.N; d++) {
            QzSweep w;
            std::memset(&w, 0, sizeof(w));
            for (int i = 0; i < 3; i++) w.offs[i] = g.offs[i];
            w.cpb = g.cpb;
            w.per = g.per;
            w.axis = g.e + perm[d];
            int no = 0;
            w.g[0] = w.g[1] = 1;
            w.cnt[0] = w.cnt[1] = 1;
            w.oth[0] = w.oth[1] = 0;
            for (int ee = 0; ee < g.N; ee++) {
                if (ee == d) continue;
                w.oth[no] = g.e + perm[ee];
                w.g[no] = ee < d ? s : 2 * s;
                w.cnt[no] = (g.bsz - 1) / w.g[no] + 1;
                no++;
            }
            if (g.N == 2) {  // the missing axis: the embedding's leading one
                w.oth[1] = w.oth[0];
                w.g[1] = w.g[0];
                w.cnt[1] = w.cnt[0];
                w.oth[0] = 0;
                w.g[0] = 1;
                w.cnt[0] = 1;
            } else if (g.N == 1) {
                w.oth[0] = 0;
                w.oth[1] = 1;
            }
            w.s = s;
            w.n = (g.bsz - 1) / s + 1;
            w.tpl = w.n / 2;
            w.cubic = interp == FAZ_INTERP_ALGO_CUBIC;
            w.seg_off = pos;
            const int64_t lines = w.cnt[0] * w.cnt[1];
            const uint64_t total = (uint64_t)(lines * w.tpl) * nblk;
            if (total) {
                const unsigned grid = (unsigned)((total + 255) / 256);
                if (R.mode == 1) {
                    if (straight) k_qz_sweep<T, 1, 1><<<grid, 256, 0, st>>>(w, q, work, codes, scratch, err, total);
                    else k_qz_sweep<T, 1, 0><<<grid, 256, 0, st>>>(w, q, work, codes, scratch, err, total);
                } else {
                    if (straight) k_qz_sweep<T, 2, 1><<<grid, 256, 0, st>>>(w, q, work, codes, scratch, err, total);
                    else k_qz_sweep<T, 2, 0><<<grid, 256, 0, st>>>(w, q, work, codes, scratch, err, total);
                }
                launches(cudaGetLastError());
            }
            if (sp.nseg >= kMaxSegs) throw Fail{FAZ_ERR_UNSUPPORTED, "too many tuning levels"};
            sp.seg[sp.nseg++] = SumSeg{pos, lines, w.tpl, d == g.N - 1 ? 1 : 0};
            pos += lines * w.tpl;
        }
        if (level_ranges) {
            level_ranges->push_back({range_lo, pos});
            range_lo = pos;
        }
    }
}

// Codes per block of a full tuning-1 run.
int64_t full_run_slots(const QzGeom &g) {
    int64_t p = g.anchor ? g.nanchor : 1;
    for (int level = g.levels - (g.anchor ? 1 : 0); level > 0; level--) {
        const int64_t s = (int64_t)1 << (level - 1);
        for (int sw = 0; sw < g.N; sw++) {
            int64_t lines = 1;
            for (int u = 0; u < g.N; u++)
                if (u != sw) lines *= (g.bsz - 1) / (u < sw ? s : 2 * s) + 1;
            p += lines * (((g.bsz - 1) / s + 1) / 2);
        }
    }
    return p;
}

// profiling_block_2d / profiling_block_3d (include/QoZ/utils/Sample.hpp:13-67,
// 143-180): one thread per candidate block start (multiples of sbs); flag[b]
// = 1 when the range of the block's points at multiples of `stride` (the
// reference's loop order and comparisons) exceeds abseb.
template <typename T>
__global__ void k_qz_profile(const T *__restrict__ X, int64_t d1, int64_t d2, int64_t nby, int64_t nbz, int64_t sbs,
                             int64_t stride, int N, double abseb, uint8_t *flag, uint64_t nb) {
    const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int64_t bz = (int64_t)(b % (uint64_t)nbz), by = (int64_t)((b / (uint64_t)nbz) % (uint64_t)nby);
    const int64_t bx = (int64_t)(b / ((uint64_t)nbz * (uint64_t)nby));
    const int64_t dyz = d1 * d2;
    const T *s0 = X + bx * sbs * dyz + by * sbs * d2 + bz * sbs;
    T mn = s0[0], mx = s0[0];
    for (int64_t ii = 0; ii <= sbs; ii += stride)
        for (int64_t jj = 0; jj <= sbs; jj += stride)
            for (int64_t kk = 0; N == 2 ? kk == 0 : kk <= sbs; kk += (N == 3 ? stride : 1)) {
                const T v = s0[ii * dyz + jj * d2 + kk];
                if (v < mn) mn = v;
                else if (v > mx) mx = v;
            }
    flag[b] = (double)(T)(mx - mn) > abseb ? 1 : 0;
}

// blockwise_profiling's variance (include/QoZ/utils/Metrics.hpp:24-100) of
// the blocks of bs points per axis at the given starts: one thread per block,
// the reference's sequential double sums.
template <typename T>
__global__ void k_qz_sigma2(const T *__restrict__ X, const int64_t *__restrict__ starts, uint64_t n, int64_t d1,
                            int64_t d2, int64_t bs, int N, double *out) {
    const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const int64_t x = starts[3 * b], y = starts[3 * b + 1], z = starts[3 * b + 2];
    const int64_t dyz = d1 * d2, zn = N == 3 ? bs : 1;
    const double ne = (double)(N == 3 ? bs * bs * bs : bs * bs);
    double sum = 0, sigma2 = 0;
    for (int64_t i = x; i < x + bs; i++)
        for (int64_t j = y; j < y + bs; j++)
            for (int64_t k = z; k < z + zn; k++) {
                const T value = X[i * dyz + j * d2 + k];
                sum += value;
            }
    const double mean = sum / ne;
    for (int64_t i = x; i < x + bs; i++)
        for (int64_t j = y; j < y + bs; j++)
            for (int64_t k = z; k < z + zn; k++) {
                const T value = X[i * dyz + j * d2 + k];
                sigma2 += (value - mean) * (value - mean);
            }
    sigma2 /= ne;
    out[b] = sigma2;
}

}  // namespace

// QoZ defaults and the settings derived from the field before any trial
// (SZInterp.hpp:1588-1625, 1660-1690, 1800-1812); returns max_interp_level.
template <typename T>
int qoz_prepare(faz_config &c, const T *dX, cudaStream_t st, Counter &launches) {
    const int N = c.N;
    if (N != 2 && N != 3) throw Fail{FAZ_ERR_UNSUPPORTED, "QoZ tuning is implemented for 2-D and 3-D data"};
    if (c.tuningTarget > 3) throw Fail{FAZ_ERR_ARG, "tuningTarget must be RD, CR, SSIM or AC"};
    if (c.rng < 0) c.rng = device_range<T>(dX, c.num, st, launches);
    if (c.relErrorBound <= 0) c.relErrorBound = c.absErrorBound / c.rng;
    // waveAutoFix (default 1, not a Config field here) turns the Lorenzo
    // trial off above a relative bound of 1e-3 and under the SSIM target
    // (SZInterp.hpp:1592-1594)
    if (c.relErrorBound > 1e-3 || c.tuningTarget == 2) c.testLorenzo = 0;
    if (c.QoZ) {
        // QoZ defaults (SZInterp.hpp:1597-1625)
        if (c.autoTuningRate <= 0) c.autoTuningRate = N == 2 ? 0.01 : 0.005;
        if (c.predictorTuningRate <= 0) c.predictorTuningRate = N == 2 ? 0.01 : 0.005;
        if (c.maxStep <= 0) c.maxStep = N == 2 ? 64 : 32;
        if (c.levelwisePredictionSelection <= 0) c.levelwisePredictionSelection = N == 2 ? 6 : 4;
        if (c.sampleBlockSize <= 0) c.sampleBlockSize = N == 2 ? 64 : 32;
        c.profiling = 0;
        c.testLorenzo = 0;
        c.sperr = -1;
        c.conditioning = 0;
        c.pyBind = 0;
        c.sperrWithoutWave = 0;
    }
    // without QoZ the tuner runs from the configuration's own rates
    // (predictorTuningRate in (0, 1)); these variants are not implemented
    if (c.autoTuningRate < 0) throw Fail{FAZ_ERR_UNSUPPORTED, "a negative autoTuningRate is not implemented"};
    int max_interp_level = -1;
    for (int i = 0; i < N; i++) {
        const int l = (int)std::ceil(std::log2((double)c.dims[i]));
        if (max_interp_level < l) max_interp_level = l;
    }
    if (c.maxStep > 0) {
        const int t = (int)(unsigned)std::log2((double)c.maxStep);
        if (t <= max_interp_level) max_interp_level = t;
        if (c.levelwisePredictionSelection > max_interp_level) c.levelwisePredictionSelection = max_interp_level;
    }
    uint64_t shortest = c.dims[0];
    for (int i = 0; i < N; i++) shortest = std::min<uint64_t>(shortest, c.dims[i]);
    if (c.sampleBlockSize <= 0) c.sampleBlockSize = N == 2 ? 64 : 32;  // SZInterp.hpp:1783-1786
    const int minimum_sbs = 16;
    if (c.sampleBlockSize < minimum_sbs) c.sampleBlockSize = minimum_sbs;
    while ((uint64_t)c.sampleBlockSize >= shortest) c.sampleBlockSize /= 2;
    while (c.autoTuningRate > 0 && c.sampleBlockSize >= 2 * minimum_sbs &&
           (std::pow(c.sampleBlockSize, N) / (double)c.num) > 1.5 * c.autoTuningRate)
        c.sampleBlockSize /= 2;
    if (!(c.predictorTuningRate > 0 && c.predictorTuningRate < 1))
        throw Fail{FAZ_ERR_UNSUPPORTED, "QoZ tuning needs predictorTuningRate in (0, 1)"};
    const int64_t sbs = c.sampleBlockSize;
    if (c.fixBlockSize > 0 || c.interpBlockSize < sbs)
        throw Fail{FAZ_ERR_UNSUPPORTED, "QoZ tuning needs interpBlockSize >= sampleBlockSize and no fixBlockSize"};
    if (c.blockwiseTuning) throw Fail{FAZ_ERR_UNSUPPORTED, "blockwiseTuning is not implemented"};
    return max_interp_level;
}
template int qoz_prepare<float>(faz_config &, const float *, cudaStream_t, Counter &);
template int qoz_prepare<double>(faz_config &, const double *, cudaStream_t, Counter &);

// QoZ Tuning for the RD target on 2-D / 3-D data; on return c holds the
// decisions (per-level lists, alpha, beta, maxStep, ...).
template <typename T>
void qoz_tune_device(faz_config &c, const T *dX, cudaStream_t st, Counter &launches, faz_timings &tm) {
    const int N = c.N;
    // FAZ_TUNE_TRACE=1: the tuner's timeline on stderr
    const char *trace_env = std::getenv("FAZ_TUNE_TRACE");
    const bool trace = trace_env && trace_env[0] == '1';
    const auto t_start = clk::now();
    auto mark = [&](const char *what, double a = 0, double b = 0) {
        if (trace) std::fprintf(stderr, "qoz %9.3f ms  %s %g %g\n", ms_since(t_start), what, a, b);
    };
    const int max_interp_level = qoz_prepare<T>(c, dX, st, launches);
    mark("prepared");
    const double rel_bound = c.relErrorBound > 0 ? c.relErrorBound : c.absErrorBound / (double)(T)c.rng;
    const int64_t sbs = c.sampleBlockSize, bsz = sbs + 1;
    const uint64_t d0 = c.dims[0], d1 = c.dims[1], d2 = N == 3 ? c.dims[2] : 1;
    // candidate blocks: starts at multiples of sbs (sampleBlocks' loops)
    const uint64_t nbx = (d0 - 1) / sbs, nby = (d1 - 1) / sbs, nbz = N == 3 ? (d2 - 1) / sbs : 1;
    const uint64_t totalblock_num = nbx * nby * (N == 3 ? nbz : 1);
    auto start_of = [&](uint64_t b, std::vector<int64_t> &out) {
        out.push_back((int64_t)(b / (nbz * nby)) * sbs);
        out.push_back((int64_t)((b / nbz) % nby) * sbs);
        out.push_back(N == 3 ? (int64_t)(b % nbz) * sbs : 0);
    };
    // sampleBlocks without profiling (var_first 0): every (size_t)(1/rate)-th block
    auto plain_starts = [&](double rate) {
        uint64_t stride = (uint64_t)(1.0 / rate);
        if (stride <= 0) stride = 1;
        std::vector<int64_t> st;
        for (uint64_t b = 0; b < totalblock_num; b += stride) start_of(b, st);
        return st;
    };
    DevMem m(st);
    // profiling (SZInterp.hpp:1820-1842): the blocks whose subsampled range
    // exceeds the bound; profiling_coeff scales the B-M CompressTests
    double pcoeff = 1;
    std::vector<int64_t> starts;
    std::vector<uint64_t> filt;  // the profiled blocks
    if (c.profiling) {
        uint8_t *dflag = m.alloc<uint8_t>(totalblock_num + 1);
        int64_t pstride = sbs / 4;
        if (pstride == 0) pstride = sbs;
        k_qz_profile<T><<<(unsigned)((totalblock_num + 255) / 256), 256, 0, st>>>(
            dX, (int64_t)d1, (int64_t)d2, (int64_t)nby, (int64_t)nbz, sbs, pstride, N, c.absErrorBound, dflag,
            totalblock_num);
        launches(cudaGetLastError());
        std::vector<uint8_t> hflag(totalblock_num);
        CK(cudaMemcpyAsync(hflag.data(), dflag, totalblock_num, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (uint64_t b = 0; b < totalblock_num; b++)
            if (hflag[b]) filt.push_back(b);
        const uint64_t npst = filt.size();
        if (npst <= (uint64_t)(int)(0.3 * c.predictorTuningRate)) c.profiling = 0;
        if (c.profiling) {
            pcoeff = (double)npst / totalblock_num;
            // sampleBlocks with profiling: every sample_stride-th filtered block
            uint64_t sstride = (uint64_t)(npst / (totalblock_num * c.predictorTuningRate));
            if (sstride <= 0) sstride = 1;
            for (uint64_t t = 0; t < npst; t += sstride) start_of(filt[t], starts);
        }
    }
    if (c.var_first) {
        // sampleBlocks with var_first (SZInterp.hpp:1020-1037, 1086-1124): the
        // candidates of largest block variance, largest first (the order a
        // max-heap of (sigma2, starts) hands them out)
        if (!c.profiling && N != 3)
            throw Fail{FAZ_ERR_UNSUPPORTED, "var_first sampling without profiling covers 3-D data"};
        std::vector<int64_t> cand;
        if (c.profiling)
            for (uint64_t b : filt) start_of(b, cand);
        else
            for (uint64_t b = 0; b < totalblock_num; b++) start_of(b, cand);
        const uint64_t nc = cand.size() / 3;
        int64_t *dc = m.alloc<int64_t>(cand.size());
        double *ds2 = m.alloc<double>(nc);
        CK(cudaMemcpyAsync(dc, cand.data(), cand.size() * 8, cudaMemcpyHostToDevice, st));
        k_qz_sigma2<T><<<(unsigned)((nc + 127) / 128), 128, 0, st>>>(dX, dc, nc, (int64_t)d1, (int64_t)d2, bsz, N, ds2);
        launches(cudaGetLastError());
        std::vector<double> s2(nc);
        CK(cudaMemcpyAsync(s2.data(), ds2, nc * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        std::vector<uint64_t> ord(nc);
        for (uint64_t t = 0; t < nc; t++) ord[t] = t;
        std::sort(ord.begin(), ord.end(), [&](uint64_t a, uint64_t b) {
            if (s2[a] != s2[b]) return s2[a] > s2[b];
            for (int q = 0; q < 3; q++)
                if (cand[3 * a + q] != cand[3 * b + q]) return cand[3 * a + q] > cand[3 * b + q];
            return false;
        });
        uint64_t k = (uint64_t)(totalblock_num * c.predictorTuningRate);
        if (c.profiling && k > nc) k = nc;
        if (k == 0) k = 1;
        if (k > nc) k = nc;
        starts.clear();
        for (uint64_t t = 0; t < k; t++)
            for (int q = 0; q < 3; q++) starts.push_back(cand[3 * ord[t] + q]);
    } else if (!c.profiling) {
        starts = plain_starts(c.predictorTuningRate);
    }
    QzGeom g = make_geom(N, bsz, (int64_t)c.maxStep);
    g.cpb = full_run_slots(g);
    uint64_t nblk = 0, nv = 0, ns = 0;
    T *blocks = nullptr, *work = nullptr, *scratch = nullptr;
    uint16_t *codes = nullptr;
    double *err = nullptr, *bsum = nullptr;
    std::vector<double> hsum;
    // the sampled blocks and the buffers sized by their count
    auto gather = [&](const std::vector<int64_t> &sts) {
        nblk = sts.size() / 3;
        if (nblk == 0) throw Fail{FAZ_ERR_UNSUPPORTED, "no block to sample for QoZ tuning"};
        nv = nblk * (uint64_t)g.per;
        ns = nblk * (uint64_t)g.cpb;
        blocks = m.alloc<T>(nv);
        work = m.alloc<T>(nv);
        scratch = m.alloc<T>(ns);
        codes = m.alloc<uint16_t>(ns);
        err = m.alloc<double>(ns);
        bsum = m.alloc<double>(nblk);
        hsum.assign(nblk, 0.0);
        int64_t *dstarts = m.alloc<int64_t>(sts.size());
        CK(cudaMemcpyAsync(dstarts, sts.data(), sts.size() * 8, cudaMemcpyHostToDevice, st));
        k_qz_gather<T><<<(unsigned)((nv + 255) / 256), 256, 0, st>>>(dX, dstarts, (int64_t)c.dims[1],
                                                                      N == 3 ? (int64_t)c.dims[2] : (int64_t)c.dims[1],
                                                                      bsz, N, blocks, nv);
        launches(cudaGetLastError());
    };
    gather(starts);
    mark("sampled blocks", (double)nblk, (double)nv);
    auto block_sums = [&](const SumPlan &sp) -> double {
        k_qz_sum<<<(unsigned)((nblk + 63) / 64), 64, 0, st>>>(sp, err, bsum, nblk);
        launches(cudaGetLastError());
        CK(cudaMemcpyAsync(hsum.data(), bsum, nblk * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        double s = 0;
        for (uint64_t k = 0; k < nblk; k++) s += hsum[k];
        return s;
    };
    const double o_alpha = c.alpha, o_beta = c.beta;
    if (c.autoTuningRate > 0) {
        // setABwithRelBound(rel_bound, 0) (SZInterp.hpp:1394-1420)
        double a, b;
        if (rel_bound >= 0.01) a = 2, b = 2;
        else if (rel_bound >= 0.007) a = 1.75, b = 2;
        else if (rel_bound >= 0.004) a = 1.5, b = 2;
        else if (rel_bound > 0.001) a = 1.25, b = 1.5;
        else a = 1, b = 1;
        c.alpha = a;
        c.beta = b;
    }
    const int Lsel = c.levelwisePredictionSelection;
    std::vector<uint8_t> il(Lsel > 0 ? Lsel : 0), dl(Lsel > 0 ? Lsel : 0);
    const int dirs[2] = {0, N == 3 ? 5 : 1};
    SumPlan sp;
    // One CompressTest (SZInterp.hpp:1130-1392) of every sampled block: bit
    // rate after Huffman + zstd, PSNR from the summed squared errors.  Its
    // device buffers and bookkeeping live in a context, so that several tests
    // can run at once, each on its own stream and host thread.
    struct CtCtx {
        DevMem m;
        T *work, *scratch;
        uint16_t *codes;
        double *err, *bsum;
        std::vector<double> hsum;
        SumPlan sp;
        std::vector<std::pair<int64_t, int64_t>> ranges;
        Counter launches;
        faz_timings tm;
        CtCtx(cudaStream_t s, uint64_t nv_, uint64_t ns_, uint64_t nblk_) : m(s), hsum(nblk_, 0.0) {
            work = m.alloc<T>(nv_);
            scratch = m.alloc<T>(ns_);
            codes = m.alloc<uint16_t>(ns_);
            err = m.alloc<double>(ns_);
            bsum = m.alloc<double>(nblk_);
            std::memset(&tm, 0, sizeof(tm));
        }
    };
    // The SSIM and autocorrelation targets score the alpha/beta search's
    // tests by the sampled blocks' reconstructions (tuning_metrics.h): set
    // once the search's sample is in, with the original blocks on the host.
    int metric_target = 0;
    std::vector<T> horig;
    SsimCubes cubes;
    auto target_metric = [&](const std::vector<T> &cur) -> double {
        if (metric_target == 2) return ssim_metric<T>(cubes, horig.data(), cur.data(), nblk);
        return 1.0 - autocorrelation_of<T>(horig.data(), cur.data(), horig.size());
    };
    auto compress_test_on = [&](CtCtx &x, cudaStream_t s, int op, int dir, double alpha, double beta, double eb,
                                double &bitrate, double &psnr, bool lists, double pc) {
        CK(cudaMemcpyAsync(x.work, blocks, nv * sizeof(T), cudaMemcpyDeviceToDevice, s));
        QzRun R{1, g.levels, 0, eb, alpha, beta, c.trimToZero, op, dir, lists ? &il : nullptr, lists ? &dl : nullptr};
        qz_run<T>(g, R, x.work, x.codes, x.scratch, x.err, nblk, x.sp, &x.ranges, s, x.launches);
        k_qz_sum<<<(unsigned)((nblk + 63) / 64), 64, 0, s>>>(x.sp, x.err, x.bsum, nblk);
        x.launches(cudaGetLastError());
        CK(cudaMemcpyAsync(x.hsum.data(), x.bsum, nblk * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        double se = 0;
        for (uint64_t k = 0; k < nblk; k++) se += x.hsum[k];
        // q_bins: level ranges from the coarsest, each across all blocks
        // (the anchors travel with the first interpolated level)
        std::vector<int64_t> rlo, rlen, rout;
        int64_t o = 0;
        for (size_t i = 0; i < x.ranges.size(); i++) {
            const int64_t lo = i == 0 ? 0 : x.ranges[i].first, hi = x.ranges[i].second;
            if (hi <= lo) continue;
            rlo.push_back(lo);
            rlen.push_back(hi - lo);
            rout.push_back(o);
            o += (hi - lo) * (int64_t)nblk;
        }
        if (o != (int64_t)ns) throw Fail{FAZ_ERR_DEVICE, "tuning codes do not cover the sampled blocks"};
        int64_t *dr = x.m.alloc<int64_t>(3 * rlo.size() + 3);
        std::vector<int64_t> hr;
        hr.insert(hr.end(), rlo.begin(), rlo.end());
        hr.insert(hr.end(), rlen.begin(), rlen.end());
        hr.insert(hr.end(), rout.begin(), rout.end());
        CK(cudaMemcpyAsync(dr, hr.data(), hr.size() * 8, cudaMemcpyHostToDevice, s));
        uint16_t *qb = x.m.alloc<uint16_t>(ns);
        const int nr = (int)rlo.size();
        k_qz_regroup<<<(unsigned)((ns + 255) / 256), 256, 0, s>>>(x.codes, g.cpb, dr, dr + nr, dr + 2 * nr, nr, nblk,
                                                                  qb, ns);
        x.launches(cudaGetLastError());
        HuffEncoded h;
        huffman_encode_device(qb, ns, 32768, x.m, s, x.launches, h, x.tm);
        // unpredictable values in the order the quantiser kept them
        // (block by block, stream order): zeros of the block-major codes
        const uint64_t nsub = hist_subchunks(ns);
        unsigned long long *zc = x.m.alloc<unsigned long long>(nsub + 1), *zoff = x.m.alloc<unsigned long long>(nsub + 1);
        unsigned long long *ztmp = x.m.alloc<unsigned long long>(scan_temp_words(nsub) + 1);
        x.launches(launch_count_zeros(x.codes, ns, zc, s));
        x.launches(launch_scan_u64(zc, zoff, nsub, ztmp, s));
        const uint64_t nunp = h.nzero;
        T *unp = x.m.alloc<T>(nunp ? nunp : 1);
        if (nunp) x.launches(launch_compact_zeros<T>(x.codes, ns, zc, zoff, nullptr, x.scratch, unp, s));
        std::vector<uint8_t> head;
        put<uint8_t>(head, 2);
        put<double>(head, eb);
        put<int32_t>(head, 32768);
        put<uint64_t>(head, nunp);
        std::vector<uint8_t> tree;
        append_tree(tree, h.cb, h.nbytes);
        // the payload through the thread's pinned staging buffer
        const size_t plen = head.size() + nunp * sizeof(T) + tree.size() + h.nbytes;
        uint8_t *pl = t_pin_payload.get(plen + 8);
        std::memcpy(pl, head.data(), head.size());
        if (nunp) CK(cudaMemcpyAsync(pl + head.size(), unp, nunp * sizeof(T), cudaMemcpyDeviceToHost, s));
        std::memcpy(pl + head.size() + nunp * sizeof(T), tree.data(), tree.size());
        if (h.nbytes)
            CK(cudaMemcpyAsync(pl + head.size() + nunp * sizeof(T) + tree.size(), h.bits, h.nbytes,
                               cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        // profiling_coeff scales both (SZInterp.hpp:1364-1370)
        const double ele = (double)nv;
        mark("  compress test payload", (double)plen, alpha);
        bitrate = 8 * (double)zstd_framed_size_host(pl, plen) / ele;
        mark("  compress test zstd", beta, eb);
        bitrate *= pc;
        double mse = se / ele;
        mse *= pc;
        psnr = 20 * std::log10(c.rng) - 10 * std::log10(mse);
        if (metric_target >= 2) {
            // the reconstructions are left in the working copy
            std::vector<T> cur(nv);
            CK(cudaMemcpyAsync(cur.data(), x.work, nv * sizeof(T), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            psnr = target_metric(cur);
        }
    };
    // tests on the tuner's own stream
    std::unique_ptr<CtCtx> main_ctx;
    auto compress_test = [&](int op, int dir, double alpha, double beta, double eb, double &bitrate, double &psnr,
                             bool lists = true, double pc = 1.0) {
        if (!main_ctx || main_ctx->hsum.size() != nblk) main_ctx.reset(new CtCtx(st, nv, ns, nblk));
        compress_test_on(*main_ctx, st, op, dir, alpha, beta, eb, bitrate, psnr, lists, pc);
        launches.n += main_ctx->launches.n;
        main_ctx->launches.n = 0;
        tm.host_ms += main_ctx->tm.host_ms;
        main_ctx->tm.host_ms = 0;
    };
    // without the alpha/beta search (autoTuningRate = 0) the decisions
    // compare compression ratios of CompressTests (TUNING_TARGET_CR)
    const bool cr_tests = c.autoTuningRate == 0;
    double best_lorenzo_ratio = 0, best_interp_cr = 0;
    if (c.testLorenzo && cr_tests) {
        // SZInterp.hpp:1925-1932
        double br, mm;
        lorenzo_compress_test<T>(N, blocks, nblk, bsz, c.absErrorBound, c.rng, 1.0, st, launches, br, mm);
        best_lorenzo_ratio = sizeof(T) * 8.0 / br;
    }
    if (Lsel > 0) {
        // per-level selection by summed prediction loss (tuning mode 2)
        for (int level = Lsel; level > 0; level--) {
            int start_level = level == Lsel ? 9999 : level, end_level = level - 1;
            if (start_level <= 0 || start_level > g.levels) start_level = g.levels;
            if (end_level >= start_level || end_level < 0) end_level = 0;
            int best_op = 1, best_dir = 0;
            double best = DBL_MAX;
            for (int op = 0; op < 2; op++)
                for (int di = 0; di < 2; di++) {
                    CK(cudaMemcpyAsync(work, blocks, nv * sizeof(T), cudaMemcpyDeviceToDevice, st));
                    QzRun R{2, start_level, end_level, c.absErrorBound, c.alpha, c.beta, c.trimToZero, op, dirs[di],
                            nullptr, nullptr};
                    qz_run<T>(g, R, work, codes, scratch, err, nblk, sp, nullptr, st, launches);
                    const double cur = block_sums(sp);
                    if (cur < best) {
                        best = cur;
                        best_op = op;
                        best_dir = dirs[di];
                    }
                }
            il[level - 1] = (uint8_t)best_op;
            dl[level - 1] = (uint8_t)best_dir;
            mark("level selected", level, best_op * 10 + best_dir);
        }
        // the candidate loop leaves its last candidate in the configuration
        c.interpAlgo = FAZ_INTERP_ALGO_CUBIC;
        c.interpDirection = (uint8_t)dirs[1];
        if (cr_tests) {
            // CompressTest of the Config as the loop leaves it: its last
            // candidate on every level, the lists not yet in the Config
            // (SZInterp.hpp:2020-2032)
            double br, mm;
            compress_test(FAZ_INTERP_ALGO_CUBIC, dirs[1], c.alpha, c.beta, c.absErrorBound, br, mm, false);
            best_interp_cr = sizeof(T) * 8.0 / br;
        }
    } else {
        // one interpolator and direction for every level, by the compression
        // ratio of a CompressTest per candidate (SZInterp.hpp:2036-2076)
        int best_op = FAZ_INTERP_ALGO_CUBIC, best_dir = 0;
        double best_cr = 0;
        for (int op = 0; op < 2; op++)
            for (int di = 0; di < 2; di++) {
                double br, mm;
                compress_test(op, dirs[di], c.alpha, c.beta, c.absErrorBound, br, mm);
                const double cr = sizeof(T) * 8.0 / br;
                if (cr > best_cr) {
                    best_cr = cr;
                    best_op = op;
                    best_dir = dirs[di];
                }
            }
        c.interpAlgo = best_op;
        c.interpDirection = (uint8_t)best_dir;
        if (cr_tests) best_interp_cr = best_cr;
    }
    c.alpha = o_alpha;
    c.beta = o_beta;
    // SZInterp.hpp:2083
    bool use_interp = best_interp_cr >= best_lorenzo_ratio || best_lorenzo_ratio >= 80 || best_interp_cr >= 80;
    if (c.autoTuningRate > 0 && use_interp && c.autoTuningRate != c.predictorTuningRate)
        gather(plain_starts(c.autoTuningRate));  // its own sample, no profiling (SZInterp.hpp:2199-2202)
    if (c.autoTuningRate > 0) {
        // B-M tuning (SZInterp.hpp:2187-2515): CompressTest per alpha/beta
        double bestalpha = 1, bestbeta = 1, bestb = 9999, bestm = 0;
        // init_alphalist / init_betalist (SZInterp.hpp:868-933); the CR target
        // compares bit rates alone (its CompressTest metric is 0)
        const bool cr = c.tuningTarget == 1;
        // abList 0, 1, 2: alpha up to 2, 2.5, 3
        static const std::vector<double> alist0{1, 1.25, 1.5, 1.75, 2}, alist1{1, 1.25, 1.5, 1.75, 2, 2.25, 2.5},
            alist2{1, 1.25, 1.5, 1.75, 2, 2.25, 2.5, 2.75, 3}, blist_rd{1.5, 2, 3, 4};
        static const std::vector<double> alist_cr{-1, 1, 1.25, 1.5, 1.75, 2}, blist_cr{-1, 1.5, 2, 3};
        const std::vector<double> &alist =
            cr ? alist_cr : (c.abList == 0 ? alist0 : (c.abList == 1 ? alist1 : alist2));
        const std::vector<double> &blist = cr ? blist_cr : blist_rd;
        const double oriabseb = c.absErrorBound;
        auto stop_here = [&](double alpha, double beta) {
            return (alpha >= 1 && std::pow(alpha, max_interp_level - 1) <= beta) ||
                   (alpha < 1 && alpha * (max_interp_level - 1) <= beta);
        };
        // The grid's CompressTests at the bound itself are independent of
        // one another: all of them run at once, each with its own stream,
        // buffers and host thread.  The search below reads their results in
        // the reference's order (a test it never reaches is simply unused)
        // and runs the tests it derives on the way - a bound scaled by a ratio
        // found so far - one by one.
        struct GridRes {
            double br = 0, mm = 0;
            uint64_t launches = 0;
            double host_ms = 0;
        };
        std::vector<std::pair<double, double>> grid;
        for (double alpha : alist)
            for (double beta : blist)
                if (!((alpha >= 1 && alpha > beta) || (alpha < 0 && beta != -1))) grid.emplace_back(alpha, beta);
        CK(cudaStreamSynchronize(st));  // the sampled blocks are gathered
        if (c.tuningTarget >= 2) {
            horig.resize(nv);
            CK(cudaMemcpyAsync(horig.data(), blocks, nv * sizeof(T), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            if (c.tuningTarget == 2)
                cubes = ssim_cubes<T>(horig.data(), nblk, N, (size_t)bsz, (size_t)c.SSIMBlockSize);
            metric_target = c.tuningTarget;
        }
        const int op0 = c.interpAlgo, dir0 = c.interpDirection;
        std::vector<std::future<GridRes>> futs;
        for (const auto &ab : grid) {
            const double alpha = ab.first, beta = ab.second;
            futs.push_back(TaskThreads::get().submit<GridRes>([&, alpha, beta]() {
                StreamGuard sg(nullptr);
                CtCtx x(sg.st, nv, ns, nblk);
                GridRes r;
                compress_test_on(x, sg.st, op0, dir0, alpha, beta, oriabseb, r.br, r.mm, true, pcoeff);
                CK(cudaStreamSynchronize(sg.st));
                r.launches = x.launches.n;
                r.host_ms = x.tm.host_ms;
                return r;
            }));
        }
        std::vector<GridRes> gres(grid.size());
        {
            std::exception_ptr first;
            for (size_t i = 0; i < futs.size(); i++) {
                try {
                    gres[i] = futs[i].get();
                    launches.n += gres[i].launches;
                    tm.host_ms += gres[i].host_ms;
                } catch (...) {
                    if (!first) first = std::current_exception();
                }
            }
            if (first) std::rethrow_exception(first);
        }
        mark("grid tests", (double)grid.size());
        auto grid_result = [&](double alpha, double beta, double &br, double &mm) {
            for (size_t i = 0; i < grid.size(); i++)
                if (grid[i].first == alpha && grid[i].second == beta) {
                    br = gres[i].br;
                    mm = gres[i].mm;
                    return;
                }
            throw Fail{FAZ_ERR_DEVICE, "alpha/beta test missing from the grid"};
        };
        // The tests the search derives (at the bound scaled by a point's bit
        // rate over the best one) follow from the grid's results as long as
        // no derived test moves the best point, which is rare: walk the
        // search under that assumption, run the derived tests it meets at
        // once, and let the search below take a result only where its bound
        // is the one the search asks for (else that test runs again).
        struct Derived {
            double alpha, beta, eb;
            GridRes r;
        };
        std::vector<Derived> derived;
        {
            double bb = 9999, bm = 0;
            for (double alpha : alist) {
                for (double beta : blist) {
                    if ((alpha >= 1 && alpha > beta) || (alpha < 0 && beta != -1)) continue;
                    double br, mm;
                    grid_result(alpha, beta, br, mm);
                    if (cr) mm = 0;
                    if ((!cr && mm >= bm && br <= bb) || (cr && br <= bb)) {
                        bb = br;
                        bm = mm;
                    } else if ((!cr && mm <= bm && br >= bb) || (cr && br > bb)) {
                        if (stop_here(alpha, beta)) break;
                        continue;
                    } else {
                        derived.push_back({alpha, beta, oriabseb * (br / bb), GridRes{}});
                    }
                    if (stop_here(alpha, beta)) break;
                }
            }
            std::vector<std::future<GridRes>> dfut;
            for (const Derived &dv : derived) {
                const double alpha = dv.alpha, beta = dv.beta, ebd = dv.eb;
                dfut.push_back(TaskThreads::get().submit<GridRes>([&, alpha, beta, ebd]() {
                    StreamGuard sg(nullptr);
                    CtCtx x(sg.st, nv, ns, nblk);
                    GridRes r;
                    compress_test_on(x, sg.st, op0, dir0, alpha, beta, ebd, r.br, r.mm, true, pcoeff);
                    CK(cudaStreamSynchronize(sg.st));
                    r.launches = x.launches.n;
                    r.host_ms = x.tm.host_ms;
                    return r;
                }));
            }
            std::exception_ptr first;
            for (size_t i = 0; i < dfut.size(); i++) {
                try {
                    derived[i].r = dfut[i].get();
                    launches.n += derived[i].r.launches;
                    tm.host_ms += derived[i].r.host_ms;
                } catch (...) {
                    if (!first) first = std::current_exception();
                }
            }
            if (first) std::rethrow_exception(first);
        }
        mark("derived tests", (double)derived.size());
        auto derived_test = [&](double alpha, double beta, double ebd, double &br, double &mm) {
            for (const Derived &dv : derived)
                if (dv.alpha == alpha && dv.beta == beta && dv.eb == ebd) {
                    br = dv.r.br;
                    mm = dv.r.mm;
                    return;
                }
            compress_test(op0, dir0, alpha, beta, ebd, br, mm, true, pcoeff);
        };
        for (double alpha : alist) {
            for (double beta : blist) {
                if ((alpha >= 1 && alpha > beta) || (alpha < 0 && beta != -1)) continue;
                double br, mm;
                grid_result(alpha, beta, br, mm);
                if (trace) std::fprintf(stderr, "qoz ab %g %g bitrate %.17g metric %.17g\n", alpha, beta, br, mm);
                if (cr) mm = 0;
                if ((!cr && mm >= bestm && br <= bestb) || (cr && br <= bestb)) {
                    bestalpha = alpha;
                    bestbeta = beta;
                    bestb = br;
                    bestm = mm;
                } else if ((!cr && mm <= bestm && br >= bestb) || (cr && br > bestb)) {
                    if (stop_here(alpha, beta)) break;
                    continue;
                } else {
                    const double fix = br / bestb;
                    double br2, m2;
                    derived_test(alpha, beta, oriabseb * fix, br2, m2);
                    if (cr) m2 = 0;
                    const double a = (mm - m2) / (br - br2);
                    const double b = mm - a * br;
                    const double reg = a * bestb + b;
                    if (reg > bestm) {
                        bestalpha = alpha;
                        bestbeta = beta;
                        bestb = br;
                        bestm = mm;
                    }
                }
                if (stop_here(alpha, beta)) break;
            }
        }
        c.absErrorBound = oriabseb;
        if (c.testLorenzo) {
            // the Lorenzo candidate: CompressTest with ALGO_LORENZO_REG
            // against the best alpha/beta point (SZInterp.hpp:2428-2486)
            double br, mm;
            std::vector<T> rec;
            lorenzo_compress_test<T>(N, blocks, nblk, bsz, oriabseb, c.rng, pcoeff, st, launches, br, mm,
                                     metric_target >= 2 ? &rec : nullptr);
            if (metric_target >= 2) mm = target_metric(rec);
            if (cr) mm = 0;
            if ((!cr && mm >= bestm && br <= bestb) || (cr && br <= bestb)) {
                bestb = br;
                bestm = mm;
                bestalpha = bestbeta = -1;
                use_interp = false;
            } else if ((!cr && mm <= bestm && br >= bestb) || (cr && br > bestb)) {
                use_interp = true;
            } else {
                const double fix = br / bestb;
                double br2, m2;
                lorenzo_compress_test<T>(N, blocks, nblk, bsz, oriabseb * fix, c.rng, pcoeff, st, launches, br2, m2,
                                         metric_target >= 2 ? &rec : nullptr);
                if (metric_target >= 2) m2 = target_metric(rec);
                if (cr) m2 = 0;
                const double a = (mm - m2) / (br - br2);
                if (a > 0) {
                    const double b = mm - a * br;
                    const double reg = a * bestb + b;
                    if (reg > bestm) {
                        bestb = br;
                        bestm = mm;
                        bestalpha = bestbeta = -1;
                        use_interp = false;
                    }
                }
            }
        }
        c.alpha = bestalpha;
        c.beta = bestbeta;
        c.wavelet_rel_coeff = 1;
        c.wavelet = 0;
    }
    mark("tuned", c.alpha, c.beta);
    if (!use_interp) {
        // Lorenzo: its own settings (the caller then runs the Lorenzo compressor)
        c.cmprAlgo = FAZ_ALGO_LORENZO_REG;
        qoz_lorenzo_followup<T>(c, dX, st, launches, tm);
        return;
    }
    if (Lsel > 0) {
        c.interp_list_len = Lsel;
        for (int i = 0; i < Lsel; i++) {
            c.interpAlgo_list[i] = il[i];
            c.interpDirection_list[i] = dl[i];
        }
    }
    c.cmprAlgo = FAZ_ALGO_INTERP;
}

template void qoz_tune_device<float>(faz_config &, const float *, cudaStream_t, Counter &, faz_timings &);
template void qoz_tune_device<double>(faz_config &, const double *, cudaStream_t, Counter &, faz_timings &);

}  // namespace faz
