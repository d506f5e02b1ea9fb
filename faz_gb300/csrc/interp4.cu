// interp4.cu - multilevel interpolation of 4-D fields, compress and decompress.
//
// block_interpolation for N = 4 (SZInterpolationCompressor.hpp:3363-3442)
// sweeps a block four times, along the axes of the direction's permutation
// (dims[0..3]); sweep d interpolates lines along dims[d] at every lattice index
// of the axes swept before it and at even indices of the axes swept after it,
// each axis starting past its first plane when the block does not begin at 0
// (that plane's lines belong to the previous block).  Lines run in row-major
// order of the other axes (sweep order), targets inside a line in the order of
// block_interpolation_1d (line_rank, common.cuh); blocks in row-major order.
//
// Every line reads only points with an even index along its own axis, which
// earlier sweeps or levels produced, so each sweep of a level is one launch
// over all blocks of the level, one thread per target in stream order, with
// neighbours read from the reconstruction W (as the coarse-level sweep kernel
// of interp.cu does for 1-D to 3-D).  Every line is computed once, by the block
// that emits it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "common.cuh"
#include "host.h"
#include "internal.h"
#include "quant.cuh"
#include "stencil.cuh"

namespace faz {

namespace {

struct Level4 {
    LevelArgs q;       // quantiser settings (eb, 1/eb, radius, exact float path)
    int64_t dims[4], offs[4], nb[4];
    int perm[4];
    int64_t s, bs;
    int cubic;
    const uint64_t *block_off;
};

struct Geom4 {
    int64_t beg[4];
    int n[4], k[4];  // lattice points per axis, 1 if the block begins past 0 (axis order)
    int64_t c[4];    // codes of sweeps 1..4
};

__host__ __device__ inline int64_t sweep_lines(const Level4 &a, const Geom4 &g, int d, int j) {
    const int ax = a.perm[j];
    return j < d ? (int64_t)(g.n[ax] - g.k[ax]) : (int64_t)((g.n[ax] + 1) / 2 - g.k[ax]);
}

__host__ __device__ inline void geom4(const Level4 &a, int64_t bid, Geom4 &g) {
    int64_t bc[4];
    for (int i = 3; i >= 0; i--) {
        bc[i] = bid % a.nb[i];
        bid /= a.nb[i];
    }
    for (int i = 0; i < 4; i++) {
        const int64_t b = bc[i] * a.bs;
        int64_t e = b + a.bs;
        if (e > a.dims[i] - 1) e = a.dims[i] - 1;
        g.beg[i] = b;
        g.n[i] = (int)((e - b) / a.s + 1);
        g.k[i] = b != 0;
    }
    for (int d = 0; d < 4; d++) {
        int64_t lines = 1;
        for (int j = 0; j < 4; j++)
            if (j != d) lines *= sweep_lines(a, g, d, j);
        g.c[d] = lines * (g.n[a.perm[d]] / 2);
    }
}

template <typename T, bool DECOMP, int QM, int CUB>
__global__ void __launch_bounds__(256) k_level4_sweep(Level4 a, int d, int64_t chunks, const T *__restrict__ X,
                                                     T *__restrict__ W, uint16_t *__restrict__ codes,
                                                     T *__restrict__ scratch, const uint64_t *__restrict__ zpos,
                                                     uint64_t nz, const T *__restrict__ unpred) {
    __shared__ Geom4 sg;
    const int64_t bid = (int64_t)blockIdx.x / chunks;
    const int64_t x = ((int64_t)blockIdx.x - bid * chunks) * blockDim.x + threadIdx.x;
    if (threadIdx.x == 0) geom4(a, bid, sg);
    __syncthreads();
    const Geom4 &g = sg;
    if (x >= g.c[d]) return;
    const int Pd = a.perm[d];
    const int n = g.n[Pd];
    const int tl = n / 2;  // targets per line
    int64_t L = x / tl;
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
    // the line's origin: the other axes' indices, row-major in sweep order
    int64_t origin = 0;
    for (int j = 3; j >= 0; j--) {
        const int ax = a.perm[j];
        int64_t c = 0;
        if (j != d) {
            const int64_t cnt = sweep_lines(a, g, d, j);
            const int64_t idx = L % cnt;
            L /= cnt;
            c = j < d ? g.k[ax] + idx : 2 * (g.k[ax] + idx);
        }
        origin += (g.beg[ax] + c * a.s) * a.offs[ax];
    }
    const int64_t st = a.s * a.offs[Pd];
    const Stencil<T> S = make_stencil<T>(m, n, a.cubic, (int)st, 0);
    const T pred = eval_stencil<CUB>(S, W + origin);
    const int64_t gi = origin + (int64_t)m * st;
    int64_t soff = 0;
    for (int j = 0; j < d; j++) soff += g.c[j];
    const uint64_t pos = a.block_off[bid] + (uint64_t)(soff + x);
    if (!DECOMP) {
        T v = X[gi], uv;
        const int code = quant_point<T, QM>(v, pred, a.q, uv);
        codes[pos] = (uint16_t)code;
        if (code == 0) scratch[pos] = uv;
        W[gi] = v;
    } else {
        W[gi] = recover_point<T, QM>(pred, (int)codes[pos], pos, a.q, zpos, nz, unpred);
    }
}

struct Plan4Level {
    Level4 a;
    int64_t nblocks;
    size_t off_index;
    int64_t cmax[4];  // codes per sweep of the first block (the largest)
};

struct Plan4 {
    std::vector<Plan4Level> lv;
    std::vector<uint64_t> block_off;
};

std::vector<std::vector<int>> perms4() {
    std::vector<int> p = {0, 1, 2, 3};
    std::vector<std::vector<int>> out;
    do out.push_back(p);
    while (std::next_permutation(p.begin(), p.end()));
    return out;
}

template <typename T>
Plan4 make_plan4(const uint64_t *dims, uint64_t maxStep, int blocksize, int fixbs, int interp, int dir,
                 const std::vector<uint8_t> &ilist, const std::vector<uint8_t> &dlist, double eb, double alpha,
                 double beta, int radius, int trim) {
    if (maxStep > 0) throw Fail{FAZ_ERR_UNSUPPORTED, "an anchor grid needs 2-D or 3-D data"};
    if (blocksize <= 0 || (blocksize & 1)) throw Fail{FAZ_ERR_UNSUPPORTED, "interpBlockSize must be a positive even number"};
    uint64_t num = 1;
    int levels = 0;
    for (int i = 0; i < 4; i++) {
        num *= dims[i];
        levels = std::max(levels, ceil_log2(dims[i]));
    }
    if (num >= ((uint64_t)1 << 31)) throw Fail{FAZ_ERR_UNSUPPORTED, "4-D fields of 2^31 values or more are not implemented"};
    if (fixbs > 0 && levels > 0 && (fixbs % (1 << levels)) != 0)
        throw Fail{FAZ_ERR_UNSUPPORTED, "fixBlockSize must be a multiple of 2^levels on the GPU path"};
    const auto perms = perms4();
    Plan4 p;
    uint64_t pos = 1;  // the first point
    for (int level = levels; level > 0; level--) {
        Plan4Level L;
        Level4 &a = L.a;
        std::memset(&a, 0, sizeof(a));
        int cur_interp = interp, cur_dir = dir;
        if (!ilist.empty()) {
            const size_t li = (size_t)(level - 1) < ilist.size() ? (size_t)(level - 1) : ilist.size() - 1;
            cur_interp = ilist[li];
            cur_dir = dlist[li];
        }
        if (cur_dir < 0 || cur_dir >= (int)perms.size()) throw Fail{FAZ_ERR_ARG, "interpolation direction out of range"};
        a.offs[3] = 1;
        for (int i = 2; i >= 0; i--) a.offs[i] = a.offs[i + 1] * (int64_t)dims[i + 1];
        for (int i = 0; i < 4; i++) {
            a.dims[i] = (int64_t)dims[i];
            a.perm[i] = perms[cur_dir][i];
        }
        a.s = (int64_t)1 << (level - 1);
        a.bs = fixbs > 0 ? fixbs : (int64_t)blocksize * a.s;
        a.cubic = cur_interp == FAZ_INTERP_ALGO_CUBIC;
        a.q.radius = radius;
        a.q.trim = trim;
        a.q.eb = level_eb(eb, alpha, beta, level);
        a.q.recip = 1.0 / a.q.eb;
        a.q.cubic = a.cubic;
        set_fast_path<T>(a.q);
        L.nblocks = 1;
        for (int i = 0; i < 4; i++) {
            a.nb[i] = (a.dims[i] - 1) / a.bs + 1;
            L.nblocks *= a.nb[i];
        }
        L.off_index = p.block_off.size();
        for (int64_t b = 0; b < L.nblocks; b++) {
            Geom4 g;
            geom4(a, b, g);
            if (b == 0)
                for (int d = 0; d < 4; d++) L.cmax[d] = g.c[d];
            p.block_off.push_back(pos);
            pos += (uint64_t)(g.c[0] + g.c[1] + g.c[2] + g.c[3]);
        }
        p.lv.push_back(L);
    }
    if (pos != num) throw Fail{FAZ_ERR_UNSUPPORTED, "block decomposition does not cover the field exactly"};
    return p;
}

template <typename T>
void run_levels4(Plan4 &p, bool decomp, const T *X, T *W, uint16_t *codes, T *scratch, const uint64_t *zpos,
                 uint64_t nz, const T *unpred, unsigned long long *verify, uint64_t ncodes, DevMem &m, cudaStream_t st,
                 Counter &launches) {
    uint64_t *boff = m.alloc<uint64_t>(std::max<size_t>(p.block_off.size(), 1));
    if (!p.block_off.empty())
        CK(cudaMemcpyAsync(boff, p.block_off.data(), p.block_off.size() * 8, cudaMemcpyHostToDevice, st));
    for (Plan4Level &L : p.lv) {
        Level4 a = L.a;
        a.block_off = boff + L.off_index;
        a.q.ncodes = ncodes;
        a.q.verify = verify;
        const bool straight = sizeof(T) == 4 && a.q.fast && a.q.trim == 0;
        void (*k)(Level4, int, int64_t, const T *, T *, uint16_t *, T *, const uint64_t *, uint64_t, const T *);
        if (a.cubic) {
            if (straight) k = decomp ? k_level4_sweep<T, true, 1, 1> : k_level4_sweep<T, false, 1, 1>;
            else k = decomp ? k_level4_sweep<T, true, 0, 1> : k_level4_sweep<T, false, 0, 1>;
        } else {
            if (straight) k = decomp ? k_level4_sweep<T, true, 1, 0> : k_level4_sweep<T, false, 1, 0>;
            else k = decomp ? k_level4_sweep<T, true, 0, 0> : k_level4_sweep<T, false, 0, 0>;
        }
        for (int d = 0; d < 4; d++) {
            if (L.cmax[d] <= 0) continue;
            const int64_t chunks = (L.cmax[d] + 255) / 256;
            if (L.nblocks * chunks >= ((int64_t)1 << 31)) throw Fail{FAZ_ERR_UNSUPPORTED, "4-D level too large"};
            k<<<(unsigned)(L.nblocks * chunks), 256, 0, st>>>(a, d, chunks, X, W, codes, scratch, zpos, nz, unpred);
            launches(cudaGetLastError());
        }
    }
}

}  // namespace

template <typename T>
void interp4_codes(const faz_config &c, double eb, int radius, const std::vector<uint8_t> &il,
                   const std::vector<uint8_t> &dl, const T *dX, T *W, uint16_t *codes, T *scratch,
                   unsigned long long *verify, DevMem &m, cudaStream_t st, Counter &launches) {
    Plan4 p = make_plan4<T>(c.dims, c.maxStep, c.interpBlockSize, c.fixBlockSize, c.interpAlgo, c.interpDirection, il,
                            dl, eb, c.alpha, c.beta, radius, c.trimToZero);
    launches(launch_first_point<T>(false, dX, W, codes, scratch, eb, radius, c.trimToZero, nullptr, 0, nullptr, st));
    run_levels4<T>(p, false, dX, W, codes, scratch, nullptr, 0, nullptr, verify, c.num, m, st, launches);
}

template <typename T>
void interp4_decompress(const uint64_t *dims, uint64_t maxStep, int blocksize, int fixbs, int interp, int dir,
                        const std::vector<uint8_t> &il, const std::vector<uint8_t> &dl, double eb, double alpha,
                        double beta, int radius, int trim, const uint16_t *codes, const uint64_t *zpos, uint64_t nz,
                        const T *unpred, T *dOut, unsigned long long *verify, DevMem &m, cudaStream_t st,
                        Counter &launches) {
    Plan4 p = make_plan4<T>(dims, maxStep, blocksize, fixbs, interp, dir, il, dl, eb, alpha, beta, radius, trim);
    uint64_t num = 1;
    for (int i = 0; i < 4; i++) num *= dims[i];
    launches(launch_first_point<T>(true, nullptr, dOut, const_cast<uint16_t *>(codes), nullptr, eb, radius, trim, zpos,
                                   nz, unpred, st));
    run_levels4<T>(p, true, nullptr, dOut, const_cast<uint16_t *>(codes), nullptr, zpos, nz, unpred, verify, num, m, st,
                   launches);
}

#define INST(T)                                                                                                     \
    template void interp4_codes<T>(const faz_config &, double, int, const std::vector<uint8_t> &,                   \
                                   const std::vector<uint8_t> &, const T *, T *, uint16_t *, T *,                   \
                                   unsigned long long *, DevMem &, cudaStream_t, Counter &);                        \
    template void interp4_decompress<T>(const uint64_t *, uint64_t, int, int, int, int, const std::vector<uint8_t> &, \
                                        const std::vector<uint8_t> &, double, double, double, int, int,             \
                                        const uint16_t *, const uint64_t *, uint64_t, const T *, T *,               \
                                        unsigned long long *, DevMem &, cudaStream_t, Counter &);
INST(float)
INST(double)
#undef INST

}  // namespace faz
