// lorenzo_candidate.cu - the Lorenzo candidate of the QoZ tuner on the GPU.
//
// Reference: CompressTest with ALGO_LORENZO_REG and the RD target
// (include/QoZ/api/impl/SZInterp.hpp:1131-1392, called from 2428-2486).  One
// general compressor - SZGeneralFrontend with ComposedPredictor over
// LorenzoPredictor<T,N,1> and LorenzoPredictor<T,N,2> (block size 5), a
// LinearQuantizer with radius 65536, HuffmanEncoder<int>, Lossless_zstd
// (make_lorenzo_regression_compressor, include/QoZ/api/impl/SZLorenzoReg.hpp:
// 28-90) - compresses every sampled block of (sbs+1)^N points in turn with
// tuning = 1, so its codes, block selections and unpredictable values
// accumulate across the blocks; encoding_lossless then writes one payload
// (include/QoZ/compressor/SZGeneralCompressor.hpp:45-91) whose zstd-framed
// size gives the bit rate, and the blocks' reconstructions give the PSNR.
//
// On the GPU a sub-block reads only sub-blocks with smaller or equal indices
// on every axis, so the sub-blocks of one diagonal bi + bj + bk = d are
// independent: one launch per diagonal covers every sampled block (grid.y),
// one warp per sub-block, with a shared-memory tile holding a 2-deep halo of
// reconstructed values; inside a sub-block the points of one plane
// i + j + k = s are independent.  Codes are 32-bit (the radius is 65536) and
// go through a small 32-bit Huffman path here: warp-aggregated histogram,
// the reference codebook built on the host, bit offsets from a scan, and the
// codes OR-ed into the bit string.
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

size_t zstd_framed_size_host(const uint8_t *p, size_t n);

namespace {

constexpr int kBs = 5;                // CompressTest's block size
constexpr int kTe = kBs + 2;          // tile edge (2-deep halo)
constexpr int kTile = kTe * kTe * kTe;
constexpr int kWarps = 8;             // sub-blocks per CTA
constexpr int kRadius = 65536;        // quantbinCnt 131072 / 2

struct TestArgs {
    int64_t D;      // sampled block edge (sbs + 1)
    int64_t nb;     // sub-blocks per axis
    int64_t per;    // points per sampled block
    double eb, recip;
    double noise1, noise2;  // LorenzoPredictor<T,3,L>(eb) noise
};

// LorenzoPredictor<T,3,L>::do_predict (include/QoZ/predictor/LorenzoPredictor.hpp:
// 146-152, 217-229) on a tile, terms in the reference's order
template <typename T>
__device__ __forceinline__ T pred3(const T *p, int L) {
#define Q(a, b, c) p[-((a) * kTe * kTe + (b) * kTe + (c))]
    if (L == 1) return Q(0, 0, 1) + Q(0, 1, 0) + Q(1, 0, 0) - Q(0, 1, 1) - Q(1, 0, 1) - Q(1, 1, 0) + Q(1, 1, 1);
    return 2 * Q(0, 0, 1) - Q(0, 0, 2) + 2 * Q(0, 1, 0) - 4 * Q(0, 1, 1) + 2 * Q(0, 1, 2) - Q(0, 2, 0) +
           2 * Q(0, 2, 1) - Q(0, 2, 2) + 2 * Q(1, 0, 0) - 4 * Q(1, 0, 1) + 2 * Q(1, 0, 2) - 4 * Q(1, 1, 0) +
           8 * Q(1, 1, 1) - 4 * Q(1, 1, 2) + 2 * Q(1, 2, 0) - 4 * Q(1, 2, 1) + 2 * Q(1, 2, 2) - Q(2, 0, 0) +
           2 * Q(2, 0, 1) - Q(2, 0, 2) + 2 * Q(2, 1, 0) - 4 * Q(2, 1, 1) + 2 * Q(2, 1, 2) - Q(2, 2, 0) +
           2 * Q(2, 2, 1) - Q(2, 2, 2);
#undef Q
}

// estimate_error: fabs(*iter - predict(iter)) + noise, as T
template <typename T>
__device__ __forceinline__ T est3(const T *p, int L, T noise) {
    const T d = *p - pred3(p, L);
    return (T)(fabs((double)d) + (double)noise);
}

// One sub-block diagonal of every sampled block (blockIdx.y).  X: sampled
// blocks (original values), R: their reconstructions, codes / scratch at
// stream positions, sel per sub-block, sq the squared reconstruction error
// of every point at its position in its sampled block.
template <typename T>
__global__ void __launch_bounds__(kWarps * 32)
    k_lor_test_diag(TestArgs a, int64_t d, const T *__restrict__ X, T *__restrict__ R, int *__restrict__ codes,
                    T *__restrict__ scratch, int *__restrict__ sel, T *__restrict__ sq) {
    __shared__ T tiles[kWarps][kTile];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t pair = (int64_t)blockIdx.x * kWarps + w;
    if (pair >= a.nb * a.nb) return;
    const int64_t bi = pair / a.nb, bj = pair - bi * a.nb, bk = d - bi - bj;
    if (bk < 0 || bk >= a.nb) return;
    const int64_t D = a.D, blk = blockIdx.y;
    const int64_t i0 = bi * kBs, j0 = bj * kBs, k0 = bk * kBs;
    const int sx = i0 + kBs < D ? kBs : (int)(D - i0);
    const int sy = j0 + kBs < D ? kBs : (int)(D - j0);
    const int sz = k0 + kBs < D ? kBs : (int)(D - k0);
    const T *Xb = X + blk * a.per;
    T *Rb = R + blk * a.per;
    T *t = tiles[w];
    // tile: reconstructed halo (zero outside the block), original interior
    for (int e = lane; e < kTile; e += 32) {
        const int i = e / (kTe * kTe), r = e - i * kTe * kTe, j = r / kTe, k = r - j * kTe;
        T v = 0;
        if (i < sx + 2 && j < sy + 2 && k < sz + 2) {
            const int64_t gi = i0 + i - 2, gj = j0 + j - 2, gk = k0 + k - 2;
            const int64_t g = (gi * D + gj) * D + gk;
            if (i >= 2 && j >= 2 && k >= 2) v = Xb[g];
            else if (gi >= 0 && gj >= 0 && gk >= 0) v = Rb[g];
        }
        t[e] = v;
    }
    __syncwarp();
    // ComposedPredictor::precompress_block: estimates along the four
    // diagonals of the sub-block's leading cube, summed in order
    int s1 = 0;
    if (lane == 0) {
        int m = sx < sy ? sx : sy;
        m = sz < m ? sz : m;
        const T n1 = (T)a.noise1, n2 = (T)a.noise2;
        double e1 = 0, e2 = 0;
        for (int q = 0; q + 2 < m; q++) {
            const int u = m - 1 - q;
            const T *p1 = t + ((q + 2) * kTe + (q + 2)) * kTe + (q + 2);
            const T *p2 = t + ((q + 2) * kTe + (q + 2)) * kTe + (u + 2);
            const T *p3 = t + ((q + 2) * kTe + (u + 2)) * kTe + (q + 2);
            const T *p4 = t + ((q + 2) * kTe + (u + 2)) * kTe + (u + 2);
            e1 += (double)est3(p1, 1, n1);
            e1 += (double)est3(p2, 1, n1);
            e1 += (double)est3(p3, 1, n1);
            e1 += (double)est3(p4, 1, n1);
            e2 += (double)est3(p1, 2, n2);
            e2 += (double)est3(p2, 2, n2);
            e2 += (double)est3(p3, 2, n2);
            e2 += (double)est3(p4, 2, n2);
        }
        s1 = e2 < e1 ? 1 : 0;
        sel[(blk * a.nb + bi) * a.nb * a.nb + bj * a.nb + bk] = s1;
    }
    const int L = __shfl_sync(0xffffffffu, s1, 0) + 1;
    // points in row-major order inside the sub-block; a plane at a time
    const uint64_t boff = (uint64_t)(blk * a.per + i0 * D * D + j0 * sx * D + k0 * sx * sy);
    for (int s = 0; s < sx + sy + sz - 2; s++) {
        for (int e = lane; e < sx * sy; e += 32) {
            const int i = e / sy, j = e - i * sy, k = s - i - j;
            if (k < 0 || k >= sz) continue;
            T *c = t + ((i + 2) * kTe + (j + 2)) * kTe + (k + 2);
            const T pred = pred3(c, L);
            const T orig = *c;
            T v = orig, uval;
            const int code = quantize<T>(v, pred, a.eb, a.recip, kRadius, 0, uval);
            const uint64_t pos = boff + (uint64_t)((i * sy + j) * sz + k);
            codes[pos] = code;
            if (code == 0) scratch[pos] = uval;
            *c = v;
            const T diff = orig - v;
            sq[blk * a.per + ((i0 + i) * D + (j0 + j)) * D + (k0 + k)] = diff * diff;
        }
        __syncwarp();
    }
    for (int e = lane; e < sx * sy * sz; e += 32) {
        const int i = e / (sy * sz), r = e - i * sy * sz, j = r / sz, k = r - j * sz;
        Rb[((i0 + i) * D + (j0 + j)) * D + (k0 + k)] = t[((i + 2) * kTe + (j + 2)) * kTe + (k + 2)];
    }
}

// LorenzoPredictor<T,2,L>::do_predict (LorenzoPredictor.hpp:123-128, 189-195)
// on a 2-D tile of row stride kTe
template <typename T>
__device__ __forceinline__ T pred2(const T *p, int L) {
#define Q(a, b) p[-((a) * kTe + (b))]
    if (L == 1) return Q(0, 1) + Q(1, 0) - Q(1, 1);
    return 2 * Q(0, 1) - Q(0, 2) + 2 * Q(1, 0) - 4 * Q(1, 1) + 2 * Q(1, 2) - Q(2, 0) + 2 * Q(2, 1) - Q(2, 2);
#undef Q
}

template <typename T>
__device__ __forceinline__ T est2(const T *p, int L, T noise) {
    const T d = *p - pred2(p, L);
    return (T)(fabs((double)d) + (double)noise);
}

// The 2-D form: one sub-block diagonal bi + bj = d of every sampled block
// (blockIdx.y), a warp per 5 x 5 sub-block, anti-diagonals of points inside.
template <typename T>
__global__ void __launch_bounds__(kWarps * 32)
    k_lor_test_diag2(TestArgs a, int64_t d, const T *__restrict__ X, T *__restrict__ R, int *__restrict__ codes,
                     T *__restrict__ scratch, int *__restrict__ sel, T *__restrict__ sq) {
    __shared__ T tiles[kWarps][kTe * kTe];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t bi = (int64_t)blockIdx.x * kWarps + w, bj = d - bi;
    if (bi >= a.nb || bj < 0 || bj >= a.nb) return;
    const int64_t D = a.D, blk = blockIdx.y;
    const int64_t i0 = bi * kBs, j0 = bj * kBs;
    const int sx = i0 + kBs < D ? kBs : (int)(D - i0);
    const int sy = j0 + kBs < D ? kBs : (int)(D - j0);
    const T *Xb = X + blk * a.per;
    T *Rb = R + blk * a.per;
    T *t = tiles[w];
    for (int e = lane; e < kTe * kTe; e += 32) {
        const int i = e / kTe, j = e - i * kTe;
        T v = 0;
        if (i < sx + 2 && j < sy + 2) {
            const int64_t gi = i0 + i - 2, gj = j0 + j - 2;
            if (i >= 2 && j >= 2) v = Xb[gi * D + gj];
            else if (gi >= 0 && gj >= 0) v = Rb[gi * D + gj];
        }
        t[e] = v;
    }
    __syncwarp();
    // ComposedPredictor::precompress_block: the two diagonals of the leading square
    int s1 = 0;
    if (lane == 0) {
        const int m = sx < sy ? sx : sy;
        const T n1 = (T)a.noise1, n2 = (T)a.noise2;
        double e1 = 0, e2 = 0;
        for (int q = 0; q + 2 < m; q++) {
            const T *p1 = t + (q + 2) * kTe + (q + 2);
            const T *p2 = t + (q + 2) * kTe + (m - 1 - q + 2);
            e1 += (double)est2(p1, 1, n1);
            e1 += (double)est2(p2, 1, n1);
            e2 += (double)est2(p1, 2, n2);
            e2 += (double)est2(p2, 2, n2);
        }
        s1 = e2 < e1 ? 1 : 0;
        sel[(blk * a.nb + bi) * a.nb + bj] = s1;
    }
    const int L = __shfl_sync(0xffffffffu, s1, 0) + 1;
    const uint64_t boff = (uint64_t)(blk * a.per + i0 * D + j0 * sx);
    for (int s = 0; s < sx + sy - 1; s++) {
        for (int i = lane; i < sx; i += 32) {
            const int j = s - i;
            if (j < 0 || j >= sy) continue;
            T *c = t + (i + 2) * kTe + (j + 2);
            const T pred = pred2(c, L);
            const T orig = *c;
            T v = orig, uval;
            const int code = quantize<T>(v, pred, a.eb, a.recip, kRadius, 0, uval);
            const uint64_t pos = boff + (uint64_t)(i * sy + j);
            codes[pos] = code;
            if (code == 0) scratch[pos] = uval;
            *c = v;
            const T diff = orig - v;
            sq[blk * a.per + (i0 + i) * D + (j0 + j)] = diff * diff;
        }
        __syncwarp();
    }
    for (int e = lane; e < sx * sy; e += 32) {
        const int i = e / sy, j = e - i * sy;
        Rb[(i0 + i) * D + (j0 + j)] = t[(i + 2) * kTe + (j + 2)];
    }
}

// ---------------------------------------------------- 32-bit Huffman codes
// Symbol counts and first positions; lanes holding the same symbol combine
// (the lowest lane has the smallest position).
__global__ void k_hist_i32(const int *__restrict__ codes, uint64_t n, int nsym, unsigned long long *cnt,
                           unsigned long long *first, int *bad) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint64_t i = base + threadIdx.x;
        const bool in = i < n;
        int c = in ? codes[i] : -1;
        if (in && (c < 0 || c >= nsym)) {
            atomicExch(bad, 1);
            c = -1;
        }
        const unsigned grp = __match_any_sync(0xffffffffu, c);
        const int leader = __ffs(grp) - 1;
        if (c >= 0 && (int)(threadIdx.x & 31) == leader) {
            atomicAdd(&cnt[c], (unsigned long long)__popc(grp));
            atomicMin(&first[c], (unsigned long long)i);
        }
    }
}

__global__ void k_len_i32(const int *__restrict__ codes, uint64_t n, int offset, const uint8_t *__restrict__ len,
                          unsigned long long *bits, unsigned long long *zero) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = codes[i];
    bits[i] = len[c - offset];
    zero[i] = c == 0;
}

// codes MSB-first into 32-bit words (bit b of the string is bit 31 - b % 32
// of word b / 32), words shared by neighbours combined with atomicOr
__global__ void k_put_i32(const int *__restrict__ codes, uint64_t n, int offset,
                          const unsigned long long *__restrict__ code64, const uint8_t *__restrict__ len,
                          const unsigned long long *__restrict__ off, uint32_t *words) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = codes[i] - offset;
    int l = len[s];
    unsigned long long c = code64[s];
    uint64_t b = off[i];
    while (l > 0) {
        const int sh = (int)(b & 31);
        const int take = 32 - sh < l ? 32 - sh : l;
        const uint32_t piece = (uint32_t)(c >> (64 - take)) << (32 - sh - take);
        atomicOr(&words[b >> 5], piece);
        c <<= take;
        b += (uint64_t)take;
        l -= take;
    }
}

// byte order of the bit string: the first byte holds bits 0..7
__global__ void k_bswap_words(uint32_t *words, uint64_t n) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) words[i] = __byte_perm(words[i], 0, 0x0123);
}

template <typename T>
__global__ void k_scatter_unpred(const int *__restrict__ codes, uint64_t n, const unsigned long long *__restrict__ zoff,
                                 const T *__restrict__ scratch, T *__restrict__ unp) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && codes[i] == 0) unp[zoff[i]] = scratch[i];
}

unsigned grid_of(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

struct Huff32 {
    Codebook cb;
    uint32_t *bits = nullptr;
    uint64_t nbytes = 0, nzero = 0;
    unsigned long long *zoff = nullptr;  // exclusive scan of code == 0
};

// HuffmanEncoder<int>::preprocess_encode + encode (include/QoZ/encoder/
// HuffmanEncoder.hpp:93-116, 150-227, 529-566) of n 32-bit codes in [0, nsym)
void huffman_i32(const int *codes, uint64_t n, int nsym, DevMem &m, cudaStream_t st, Counter &launches, Huff32 &h) {
    unsigned long long *cnt = m.alloc<unsigned long long>(nsym), *first = m.alloc<unsigned long long>(nsym);
    int *bad = m.alloc<int>(1);
    CK(cudaMemsetAsync(cnt, 0, (size_t)nsym * 8, st));
    CK(cudaMemsetAsync(first, 0xff, (size_t)nsym * 8, st));
    CK(cudaMemsetAsync(bad, 0, 4, st));
    unsigned g = grid_of(n, 256);
    if (g > 1024) g = 1024;
    if (g == 0) g = 1;
    k_hist_i32<<<g, 256, 0, st>>>(codes, n, nsym, cnt, first, bad);
    launches(cudaGetLastError());
    std::vector<unsigned long long> hc(nsym), hf(nsym);
    int hbad = 0;
    CK(cudaMemcpyAsync(hc.data(), cnt, (size_t)nsym * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hf.data(), first, (size_t)nsym * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&hbad, bad, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (hbad) throw Fail{FAZ_ERR_DEVICE, "Lorenzo trial code outside the quantiser's range"};
    std::vector<int> syms;
    std::vector<uint64_t> cnts, firsts;
    for (int s = 0; s < nsym; s++)
        if (hc[s]) {
            syms.push_back(s);
            cnts.push_back(hc[s]);
            firsts.push_back(hf[s]);
        }
    h.nzero = hc[0];
    std::string err;
    const int rc = build_codebook(syms, cnts, firsts, h.cb, err);
    if (rc) throw Fail{rc, err};
    const Codebook &cb = h.cb;
    uint64_t total_bits = 0;
    for (size_t i = 0; i < syms.size(); i++) total_bits += cnts[i] * (uint64_t)cb.len[syms[i] - cb.offset];
    h.nbytes = (total_bits + 7) / 8;
    unsigned long long *dcode = m.alloc<unsigned long long>(cb.stateNum);
    uint8_t *dlen = m.alloc<uint8_t>(cb.stateNum);
    CK(cudaMemcpyAsync(dcode, cb.code.data(), (size_t)cb.stateNum * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dlen, cb.len.data(), (size_t)cb.stateNum, cudaMemcpyHostToDevice, st));
    unsigned long long *bits = m.alloc<unsigned long long>(n + 1), *off = m.alloc<unsigned long long>(n + 1);
    unsigned long long *zero = m.alloc<unsigned long long>(n + 1);
    h.zoff = m.alloc<unsigned long long>(n + 1);
    unsigned long long *tmp = m.alloc<unsigned long long>(scan_temp_words(n) + 1);
    k_len_i32<<<grid_of(n, 256), 256, 0, st>>>(codes, n, cb.offset, dlen, bits, zero);
    launches(cudaGetLastError());
    launches(launch_scan_u64(bits, off, n, tmp, st));
    launches(launch_scan_u64(zero, h.zoff, n, tmp, st));
    const uint64_t nwords = (total_bits + 31) / 32 + 1;
    h.bits = m.alloc<uint32_t>(nwords);
    CK(cudaMemsetAsync(h.bits, 0, nwords * 4, st));
    k_put_i32<<<grid_of(n, 256), 256, 0, st>>>(codes, n, cb.offset, dcode, dlen, off, h.bits);
    launches(cudaGetLastError());
    k_bswap_words<<<grid_of(nwords, 256), 256, 0, st>>>(h.bits, nwords);
    launches(cudaGetLastError());
}

}  // namespace

// CompressTest(ALGO_LORENZO_REG, TUNING_TARGET_RD) on nblk sampled blocks of
// bsz^N points (N = 2 or 3) (dBlocks, block after block, row-major): bit rate of the one
// payload the general compressor writes and PSNR of the reconstructions (which
// `recon`, when given, receives for the SSIM and autocorrelation targets).
template <typename T>
void lorenzo_compress_test(int N, const T *dBlocks, uint64_t nblk, int64_t bsz, double eb, double rng,
                           double pcoeff, cudaStream_t st, Counter &launches, double &bitrate, double &psnr,
                           std::vector<T> *recon) {
    if (N != 2 && N != 3) throw Fail{FAZ_ERR_UNSUPPORTED, "the Lorenzo candidate covers 2-D and 3-D data"};
    TestArgs a;
    a.D = bsz;
    a.nb = (bsz - 1) / kBs + 1;
    a.per = N == 3 ? bsz * bsz * bsz : bsz * bsz;
    a.eb = eb;
    a.recip = 1.0 / eb;
    a.noise1 = (N == 3 ? 1.22 : 0.81) * eb;
    a.noise2 = (N == 3 ? 6.8 : 2.76) * eb;
    if (nblk > 65535) throw Fail{FAZ_ERR_UNSUPPORTED, "too many sampled blocks for the Lorenzo trial"};
    const uint64_t nsub = N == 3 ? (uint64_t)(a.nb * a.nb * a.nb) : (uint64_t)(a.nb * a.nb);
    const uint64_t n = nblk * (uint64_t)a.per, nsel = nblk * nsub;
    DevMem m(st);
    T *R = m.alloc<T>(n), *scratch = m.alloc<T>(n), *sq = m.alloc<T>(n);
    int *codes = m.alloc<int>(n), *sel = m.alloc<int>(nsel);
    if (N == 3) {
        const dim3 grid((unsigned)((a.nb * a.nb + kWarps - 1) / kWarps), (unsigned)nblk);
        for (int64_t d = 0; d <= 3 * (a.nb - 1); d++) {
            k_lor_test_diag<T><<<grid, kWarps * 32, 0, st>>>(a, d, dBlocks, R, codes, scratch, sel, sq);
            launches(cudaGetLastError());
        }
    } else {
        const dim3 grid((unsigned)((a.nb + kWarps - 1) / kWarps), (unsigned)nblk);
        for (int64_t d = 0; d <= 2 * (a.nb - 1); d++) {
            k_lor_test_diag2<T><<<grid, kWarps * 32, 0, st>>>(a, d, dBlocks, R, codes, scratch, sel, sq);
            launches(cudaGetLastError());
        }
    }
    Huff32 hs, hc;
    huffman_i32(sel, nsel, 2, m, st, launches, hs);
    huffman_i32(codes, n, 2 * kRadius, m, st, launches, hc);
    const uint64_t nunp = hc.nzero;
    T *unp = m.alloc<T>(nunp ? nunp : 1);
    if (nunp) {
        k_scatter_unpred<T><<<grid_of(n, 256), 256, 0, st>>>(codes, n, hc.zoff, scratch, unp);
        launches(cudaGetLastError());
    }
    // SZGeneralFrontend::save (dims, block size, predictors with the
    // selections, LinearQuantizer::save), then the codes
    std::vector<uint8_t> h0;
    for (int i = 0; i < N; i++) put<uint64_t>(h0, (uint64_t)bsz);
    put<uint32_t>(h0, (uint32_t)kBs);
    put<uint8_t>(h0, 1);
    put<uint8_t>(h0, 1);
    put<uint64_t>(h0, nsel);
    append_tree(h0, hs.cb, hs.nbytes);
    std::vector<uint8_t> h1;
    put<uint8_t>(h1, 2);
    put<double>(h1, eb);
    put<int32_t>(h1, kRadius);
    put<uint64_t>(h1, nunp);
    std::vector<uint8_t> h2;
    append_tree(h2, hc.cb, hc.nbytes);
    const size_t total = h0.size() + hs.nbytes + h1.size() + nunp * sizeof(T) + h2.size() + hc.nbytes;
    std::vector<uint8_t> pl(total);
    std::vector<T> hsq(n);
    uint8_t *p = pl.data();
    std::memcpy(p, h0.data(), h0.size());
    p += h0.size();
    if (hs.nbytes) CK(cudaMemcpyAsync(p, hs.bits, hs.nbytes, cudaMemcpyDeviceToHost, st));
    p += hs.nbytes;
    std::memcpy(p, h1.data(), h1.size());
    p += h1.size();
    if (nunp) CK(cudaMemcpyAsync(p, unp, nunp * sizeof(T), cudaMemcpyDeviceToHost, st));
    p += nunp * sizeof(T);
    std::memcpy(p, h2.data(), h2.size());
    p += h2.size();
    if (hc.nbytes) CK(cudaMemcpyAsync(p, hc.bits, hc.nbytes, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hsq.data(), sq, n * sizeof(T), cudaMemcpyDeviceToHost, st));
    if (recon) {
        recon->resize(n);
        CK(cudaMemcpyAsync(recon->data(), R, n * sizeof(T), cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
    // the squared errors summed block by block, point by point (the
    // reference's loop order), in double
    double se = 0;
    for (uint64_t i = 0; i < n; i++) se += hsq[i];
    // profiling_coeff scales both (SZInterp.hpp:1364-1370)
    const double ele = (double)n;
    bitrate = 8 * (double)zstd_framed_size_host(pl.data(), pl.size()) / ele;
    bitrate *= pcoeff;
    double mse = se / ele;
    mse *= pcoeff;
    psnr = 20 * std::log10(rng) - 10 * std::log10(mse);
}

template void lorenzo_compress_test<float>(int, const float *, uint64_t, int64_t, double, double, double,
                                           cudaStream_t, Counter &, double &, double &, std::vector<float> *);
template void lorenzo_compress_test<double>(int, const double *, uint64_t, int64_t, double, double, double,
                                            cudaStream_t, Counter &, double &, double &, std::vector<double> *);

}  // namespace faz
