// huffman.cu - Huffman histogram, encode and decode kernels.
//
// Stream format (include/QoZ/encoder/HuffmanEncoder.hpp:150-268): the codes
// of all symbols concatenated, most significant bit first, zero padded to a
// byte.  Encoding is a two-pass bit-offset scan; decoding of unmodified
// streams splits the bit string into fixed-size units, decodes each unit
// speculatively from its nominal start and repeats for units whose true start
// (the end of the previous unit's decode) differs, until every unit starts on
// a codeword boundary (Huffman codes self-synchronise within a few codewords).
#include <cuda_runtime.h>
#include <cstdint>
#include "internal.h"

namespace faz {

// --------------------------------------------------------------- histogram
// A CTA takes a chunk of HCHUNK codes; warp w of the CTA takes the contiguous
// sub-chunk [w*HSUB, (w+1)*HSUB) of it, so that zero codes can later be
// compacted per warp with one running offset and no block barriers.
// Counts of every symbol, the stream position of its first occurrence, and
// the number of zero codes per warp sub-chunk.  Symbols within +-HWIN/2 of
// `center` are counted in shared memory.
static constexpr int HWIN = 4096;
static constexpr int HWARPS = 32;
static constexpr uint64_t HSUB = 8192;
static constexpr uint64_t HCHUNK = HSUB * HWARPS;

// C: the code type, uint16_t, or uint32_t for quantisers of more than 65536
// bins (16-byte loads for 16-bit codes, plain loads otherwise).
template <typename C>
__global__ void __launch_bounds__(1024) k_histogram(const C *__restrict__ codes, uint64_t n, int center,
                                                    unsigned long long *hist, unsigned long long *first,
                                                    unsigned long long *zcount) {
    __shared__ unsigned int scnt[HWIN];
    __shared__ unsigned int sfirst[HWIN];
    for (int i = threadIdx.x; i < HWIN; i += blockDim.x) {
        scnt[i] = 0;
        sfirst[i] = 0xffffffffu;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint64_t c0 = (uint64_t)blockIdx.x * HCHUNK;
    const uint64_t s0 = c0 + (uint64_t)w * HSUB;
    uint64_t s1 = s0 + HSUB;
    if (s1 > n) s1 = n;
    const int lo = center - HWIN / 2;
    unsigned int zc = 0;
    // lanes take 8 consecutive codes (one 16-byte load); the first-position
    // atomic runs only when the position beats the recorded one
    auto count = [&](int v, uint64_t i) {
        if (v == 0) zc++;
        int b = v - lo;
        if (b >= 0 && b < HWIN) {
            atomicAdd(&scnt[b], 1u);
            const unsigned int off = (unsigned int)(i - c0);
            if (off < sfirst[b]) atomicMin(&sfirst[b], off);
        } else {
            atomicAdd(&hist[v], 1ull);
            atomicMin(&first[v], (unsigned long long)i);
        }
    };
    if (sizeof(C) == 2 && s1 - s0 == HSUB) {
        const uint4 *cv = reinterpret_cast<const uint4 *>(codes + s0);
        for (int it = 0; it < (int)(HSUB / 256); it++) {
            uint4 q = cv[it * 32 + lane];
            const uint16_t *e = reinterpret_cast<const uint16_t *>(&q);
            const uint64_t i0 = s0 + (uint64_t)(it * 32 + lane) * 8;
#pragma unroll
            for (int k = 0; k < 8; k++) count(e[k], i0 + k);
        }
    } else {
        for (uint64_t i = s0 + lane; i < s1; i += 32) count((int)codes[i], i);
    }
    for (int o = 16; o > 0; o >>= 1) zc += __shfl_down_sync(0xffffffffu, zc, o);
    if (lane == 0) zcount[(uint64_t)blockIdx.x * HWARPS + w] = zc;
    __syncthreads();
    for (int b = threadIdx.x; b < HWIN; b += blockDim.x) {
        if (scnt[b]) {
            atomicAdd(&hist[lo + b], (unsigned long long)scnt[b]);
            atomicMin(&first[lo + b], (unsigned long long)(c0 + sfirst[b]));
        }
    }
}

// The symbols of non-zero count, compacted in no particular order:
// list[3k], list[3k+1], list[3k+2] = symbol, count, first position;
// *nlist = their number.
__global__ void __launch_bounds__(256) k_hist_compact(const unsigned long long *__restrict__ hist,
                                                     const unsigned long long *__restrict__ first, int nsym,
                                                     unsigned long long *list, unsigned int *nlist) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const bool nz = s < nsym && hist[s] != 0;
    const unsigned int m = __ballot_sync(0xffffffffu, nz);
    if (m == 0) return;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    unsigned int base = 0;
    if (lane == leader) base = atomicAdd(nlist, (unsigned int)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (nz) {
        const unsigned int k = base + (unsigned int)__popc(m & ((1u << lane) - 1u));
        list[3 * (size_t)k] = (unsigned long long)s;
        list[3 * (size_t)k + 1] = hist[s];
        list[3 * (size_t)k + 2] = first[s];
    }
}

// Zero-code count per warp sub-chunk (decompress side).
template <typename C>
__global__ void __launch_bounds__(1024) k_count_zeros(const C *__restrict__ codes, uint64_t n,
                                                      unsigned long long *zcount) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint64_t s0 = (uint64_t)blockIdx.x * HCHUNK + (uint64_t)w * HSUB;
    uint64_t s1 = s0 + HSUB;
    if (s1 > n) s1 = n;
    unsigned int zc = 0;
    for (uint64_t i = s0 + lane; i < s1; i += 32) zc += codes[i] == 0;
    for (int o = 16; o > 0; o >>= 1) zc += __shfl_down_sync(0xffffffffu, zc, o);
    if (lane == 0) zcount[(uint64_t)blockIdx.x * HWARPS + w] = zc;
}

// Compaction of the zero codes of each warp sub-chunk, in stream order,
// starting at zoff[sub-chunk]: positions (zpos) and/or the values recorded at
// those positions (vals from scratch).
template <typename T, typename C>
__global__ void __launch_bounds__(1024) k_compact_zeros(const C *__restrict__ codes, uint64_t n,
                                                        const unsigned long long *zcount,
                                                        const unsigned long long *zoff, uint64_t *zpos,
                                                        const T *scratch, T *vals) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint64_t sub = (uint64_t)blockIdx.x * HWARPS + w;
    if (zcount[sub] == 0) return;
    const uint64_t s0 = sub * HSUB;
    uint64_t s1 = s0 + HSUB;
    if (s1 > n) s1 = n;
    unsigned long long run = zoff[sub];
    // 256 codes per warp step: lane L reads codes [b + 8L, b + 8L + 8) with one
    // 16-byte load (s0 is a multiple of 8192 and codes is 256-byte aligned),
    // so the zeros of a step come in stream order lane by lane
    uint64_t b = s0;
    for (; sizeof(C) == 2 && b + 256 <= s1; b += 256) {
        const uint4 q = *reinterpret_cast<const uint4 *>(codes + b + 8 * lane);
        const uint32_t wd[4] = {q.x, q.y, q.z, q.w};
        unsigned int m = 0;  // bit k: code b + 8 lane + k is zero
#pragma unroll
        for (int k = 0; k < 4; k++) {
            m |= (wd[k] & 0xffffu) == 0 ? 1u << (2 * k) : 0u;
            m |= (wd[k] >> 16) == 0 ? 1u << (2 * k + 1) : 0u;
        }
        const int c = __popc(m);
        int x = c;  // inclusive scan of the counts across lanes
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        const int total = __shfl_sync(0xffffffffu, x, 31);
        unsigned long long o = run + (unsigned long long)(x - c);
        while (m) {
            const int k = __ffs(m) - 1;
            m &= m - 1;
            const uint64_t i = b + 8 * lane + k;
            if (zpos) zpos[o] = i;
            if (vals) vals[o] = scratch[i];
            o++;
        }
        run += (unsigned long long)total;
    }
    for (; b < s1; b += 32) {
        const uint64_t i = b + lane;
        const bool z = i < s1 && codes[i] == 0;
        const unsigned int bal = __ballot_sync(0xffffffffu, z);
        if (z) {
            const unsigned long long o = run + __popc(bal & ((1u << lane) - 1));
            if (zpos) zpos[o] = i;
            if (vals) vals[o] = scratch[i];
        }
        run += __popc(bal);
    }
}

// ------------------------------------------------------------------- scan
// Exclusive scan of n 64-bit values (out[n] = total): per-block totals,
// one-block scan of the totals, per-block scan with the block's offset.
static constexpr int SCAN_T = 512;
static constexpr int SCAN_E = 8;
static constexpr int SCAN_B = SCAN_T * SCAN_E;

__device__ __forceinline__ unsigned long long block_excl_scan(unsigned long long v, unsigned long long *sh,
                                                              unsigned long long &total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        unsigned long long y = lane < nw ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long z = __shfl_up_sync(0xffffffffu, y, o);
            if (lane >= o) y += z;
        }
        sh[lane] = y;
    }
    __syncthreads();
    total = sh[nw - 1];
    unsigned long long wbase = w ? sh[w - 1] : 0;
    __syncthreads();
    return wbase + x - v;
}

__global__ void __launch_bounds__(SCAN_T) k_scan_reduce(const unsigned long long *in, uint64_t n,
                                                       unsigned long long *bsum) {
    __shared__ unsigned long long sh[32];
    uint64_t b0 = (uint64_t)blockIdx.x * SCAN_B;
    unsigned long long s = 0;
    for (int k = 0; k < SCAN_E; k++) {
        uint64_t i = b0 + (uint64_t)threadIdx.x * SCAN_E + k;
        if (i < n) s += in[i];
    }
    unsigned long long tot;
    block_excl_scan(s, sh, tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

// one block: exclusive scan of nb block totals in place (nb <= any), total in bsum[nb]
__global__ void __launch_bounds__(1024) k_scan_top(unsigned long long *bsum, uint64_t nb) {
    __shared__ unsigned long long sh[32];
    unsigned long long carry = 0;
    for (uint64_t c = 0; c < nb; c += blockDim.x) {
        uint64_t i = c + threadIdx.x;
        unsigned long long v = i < nb ? bsum[i] : 0;
        unsigned long long tot;
        unsigned long long e = block_excl_scan(v, sh, tot);
        if (i < nb) bsum[i] = carry + e;
        carry += tot;
    }
    if (threadIdx.x == 0) bsum[nb] = carry;
}

__global__ void __launch_bounds__(SCAN_T) k_scan_down(const unsigned long long *in, uint64_t n,
                                                     const unsigned long long *bsum, unsigned long long *out,
                                                     uint64_t nb) {
    __shared__ unsigned long long sh[32];
    uint64_t b0 = (uint64_t)blockIdx.x * SCAN_B;
    unsigned long long v[SCAN_E];
    unsigned long long s = 0;
    for (int k = 0; k < SCAN_E; k++) {
        uint64_t i = b0 + (uint64_t)threadIdx.x * SCAN_E + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    unsigned long long tot;
    unsigned long long e = block_excl_scan(s, sh, tot) + bsum[blockIdx.x];
    for (int k = 0; k < SCAN_E; k++) {
        uint64_t i = b0 + (uint64_t)threadIdx.x * SCAN_E + k;
        if (i < n) out[i] = e;
        e += v[k];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = bsum[nb];
}

// ------------------------------------------------------------------ encode
// Symbol tables indexed by (code - offset): MSB-aligned code, bit length.
static constexpr int ENC_PER_THREAD = 16;
static constexpr int ENC_THREADS = 256;
static constexpr int ENC_CHUNK = ENC_PER_THREAD * ENC_THREADS;

template <typename C>
__global__ void __launch_bounds__(ENC_THREADS) k_encode_bits(const C *__restrict__ codes, uint64_t n, int offset,
                                                            const uint8_t *__restrict__ len,
                                                            unsigned long long *chunkbits) {
    __shared__ unsigned long long ws[ENC_THREADS / 32];
    const uint64_t c0 = (uint64_t)blockIdx.x * ENC_CHUNK;
    unsigned long long s = 0;
    for (int k = 0; k < ENC_PER_THREAD; k++) {
        uint64_t i = c0 + (uint64_t)k * ENC_THREADS + threadIdx.x;
        if (i < n) s += len[(int)codes[i] - offset];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < ENC_THREADS / 32; w++) t += ws[w];
        chunkbits[blockIdx.x] = t;
    }
}

__device__ __forceinline__ uint32_t bswap32(uint32_t x) { return __byte_perm(x, 0, 0x0123); }

// Pack one chunk: each thread owns ENC_PER_THREAD consecutive symbols.
// Words in shared memory follow the global 32-bit word grid of the output.
// packed[state] = (len << 32) | code right-aligned (codes up to 32 bits);
// longer codes are read from code64 (MSB-aligned).
template <typename C>
__global__ void __launch_bounds__(ENC_THREADS) k_encode_pack(const C *__restrict__ codes, uint64_t n, int offset,
                                                            const unsigned long long *__restrict__ code64,
                                                            const unsigned long long *__restrict__ packed,
                                                            const uint8_t *__restrict__ len,
                                                            const unsigned long long *__restrict__ chunkoff,
                                                            uint32_t *out, int smem_words) {
    extern __shared__ uint32_t sw[];
    __shared__ unsigned long long wtot[ENC_THREADS / 32];
    const uint64_t c0 = (uint64_t)blockIdx.x * ENC_CHUNK;
    const uint64_t gbit = chunkoff[blockIdx.x];
    const uint64_t gend = chunkoff[blockIdx.x + 1];
    if (gend == gbit) return;
    const uint64_t w0 = gbit >> 5;
    const uint64_t wl = (gend - 1) >> 5;
    const int nwords = (int)(wl - w0 + 1);
    for (int i = threadIdx.x; i < nwords && i < smem_words; i += blockDim.x) sw[i] = 0;
    C sym[ENC_PER_THREAD];
    unsigned int mybits = 0;
    const uint64_t t0 = c0 + (uint64_t)threadIdx.x * ENC_PER_THREAD;
    // symbols of this thread (every 16-bit value is a valid symbol)
    const int nvalid = t0 >= n ? 0 : (n - t0 >= ENC_PER_THREAD ? ENC_PER_THREAD : (int)(n - t0));
    if (sizeof(C) == 2 && nvalid == ENC_PER_THREAD) {
        // 16 codes = two 16-byte loads (codes is 256-byte aligned, t0 a multiple of 16)
        const uint4 *cv = reinterpret_cast<const uint4 *>(codes + t0);
        uint4 qa = cv[0], qb = cv[1];
        const uint16_t *pa = reinterpret_cast<const uint16_t *>(&qa);
        const uint16_t *pb = reinterpret_cast<const uint16_t *>(&qb);
#pragma unroll
        for (int k = 0; k < 8; k++) {
            sym[k] = (C)(pa[k] - offset);
            sym[k + 8] = (C)(pb[k] - offset);
        }
#pragma unroll
        for (int k = 0; k < ENC_PER_THREAD; k++) mybits += len[sym[k]];
    } else {
#pragma unroll
        for (int k = 0; k < ENC_PER_THREAD; k++) {
            uint64_t i = t0 + k;
            sym[k] = i < n ? (C)((int)codes[i] - offset) : (C)0;
            if (i < n) mybits += len[sym[k]];
        }
    }
    // exclusive scan of the threads' bit counts (warp shuffles + warp totals)
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned long long x = mybits;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wtot[wid] = x;
    __syncthreads();
    unsigned long long wbase = 0;
    for (int w = 0; w < wid; w++) wbase += wtot[w];
    // bit position relative to word w0
    const uint64_t pos = (gbit & 31) + wbase + x - mybits;
    // bits accumulate right-aligned in acc (nacc valid bits, the first word
    // starting with `fill` zero bits owned by the previous thread); whole
    // words are stored, the thread's first (shared) and last words are ORed
    uint32_t wi = (uint32_t)(pos >> 5);
    const int fill = (int)(pos & 31);
    unsigned long long acc = 0;
    int nacc = fill;
    bool first_word = true;
    auto push = [&](uint32_t bits, int l) {  // l <= 32
        acc = (acc << l) | bits;
        nacc += l;
        if (nacc >= 32) {
            nacc -= 32;
            const uint32_t word = (uint32_t)(acc >> nacc);
            if (first_word && fill) atomicOr(&sw[wi], word);
            else sw[wi] = word;
            first_word = false;
            wi++;
        }
    };
    // a fixed trip count keeps sym[] in registers (a loop bounded by nvalid
    // would index it dynamically, from local memory)
#pragma unroll
    for (int k = 0; k < ENC_PER_THREAD; k++) {
        if (k >= nvalid) break;
        const unsigned long long e = packed[sym[k]];
        const int l = (int)((e >> 32) & 0xff);
        if (l <= 32) {
            push((uint32_t)e, l);
        } else {
            // codes longer than 32 bits: right-align the MSB-aligned code
            const unsigned long long c = l == 64 ? code64[sym[k]] : code64[sym[k]] >> (64 - l);
            push((uint32_t)(c >> 32), l - 32);
            push((uint32_t)c, 32);
        }
    }
    if (nacc > 0) {
        const uint32_t word = (uint32_t)(acc << (32 - nacc));
        if (word) atomicOr(&sw[wi], word);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nwords; i += blockDim.x) {
        uint32_t v = bswap32(sw[i]);
        if (i == 0 || i == nwords - 1) {
            if (v) atomicOr(&out[w0 + i], v);
        } else {
            out[w0 + i] = v;
        }
    }
}

// ------------------------------------------------------------------ decode
// A CTA decodes DEC_T consecutive units of DEC_UNIT bits from a copy of its
// segment of the bit string (plus a halo) in shared memory, with the
// 2^LUT_BITS-entry table beside it.  DEC_UNIT is an odd number of 32-bit
// words so that the units of a warp start in different banks.
struct DecTables {
    const uint32_t *lut;     // 2^LUT_BITS entries: (len << 24) | state, or DEC_NODE | node
    const uint32_t *left, *right;
    const int32_t *sym;      // state of a leaf
    const uint8_t *leaf;
};
static constexpr int LUT_BITS = 12;
static constexpr uint32_t DEC_NODE = 0x80000000u;
static constexpr int DEC_T = 256;
static constexpr int DEC_WORDS = 17;                 // words per unit (17: fastest of 9, 13, 17, 33 on GB300)
static constexpr uint64_t DEC_UNIT = DEC_WORDS * 32; // bits per unit
static constexpr int DEC_HALO = 8;                   // words past the last unit
static constexpr int DEC_SEG = DEC_T * DEC_WORDS + DEC_HALO;
static constexpr int DEC_NB = 16;                    // boundaries recorded per unit

// bits [p, p+64) of the segment (word-grid relative), MSB first
__device__ __forceinline__ uint64_t seg_peek(const uint32_t *sw, uint32_t p) {
    uint32_t w = p >> 5, b = p & 31;
    uint64_t hi = ((uint64_t)sw[w] << 32) | sw[w + 1];
    if (!b) return hi;
    return (hi << b) | (sw[w + 2] >> (32 - b));
}

// one symbol at segment bit p: returns its state (or -1 on a damaged tree)
// and advances p.  Codes are at most 64 bits long.
__device__ __forceinline__ int dec_sym(const DecTables &t, const uint32_t *slut, const uint32_t *sw, uint32_t &p) {
    uint64_t win = seg_peek(sw, p);
    uint32_t e = slut[win >> (64 - LUT_BITS)];
    if (!(e & DEC_NODE)) {
        p += e >> 24;
        return (int)(e & 0xffffff);
    }
    uint32_t node = e & 0xffffff;
    for (int b = LUT_BITS; b < 64; b++) {
        int bit = (int)((win >> (63 - b)) & 1);
        node = bit ? t.right[node] : t.left[node];
        if (t.leaf[node]) {
            p += b + 1;
            return t.sym[node];
        }
    }
    return -1;
}

__device__ __forceinline__ uint32_t bswap_w(uint32_t x) { return __byte_perm(x, 0, 0x0123); }

// Stage the CTA's segment (as big-endian words) and the lookup table.
__device__ __forceinline__ void dec_stage(const DecTables &t, const uint32_t *__restrict__ w32, uint64_t nwords,
                                          uint32_t *slut, uint32_t *sw, uint64_t wbase) {
    for (int i = threadIdx.x; i < (1 << LUT_BITS); i += blockDim.x) slut[i] = t.lut[i];
    for (int i = threadIdx.x; i < DEC_SEG; i += blockDim.x) {
        uint64_t gi = wbase + i;
        sw[i] = gi < nwords ? bswap_w(w32[gi]) : 0u;
    }
    __syncthreads();
}

// Speculative pass: unit u decodes from its nominal start u*DEC_UNIT to the
// first codeword end at or past the unit's end; records the end, the symbol
// count, and the first DEC_NB codeword boundaries (offsets from the start).
__global__ void __launch_bounds__(DEC_T) k_decode_spec(DecTables t, const uint32_t *__restrict__ w32, uint64_t nwords,
                                                      uint64_t nbits, uint64_t nunits, uint64_t ubase,
                                                      uint64_t *end, unsigned int *cnt, uint16_t *bnd, int *err) {
    __shared__ uint32_t slut[1 << LUT_BITS];
    __shared__ uint32_t sw[DEC_SEG];
    const uint64_t u0 = ubase + (uint64_t)blockIdx.x * DEC_T;
    dec_stage(t, w32, nwords, slut, sw, u0 * DEC_WORDS);
    const uint64_t u = u0 + threadIdx.x;
    if (u >= nunits) return;
    const uint64_t g0 = u0 * DEC_UNIT;
    uint64_t lim = (u + 1) * DEC_UNIT;
    if (lim > nbits) lim = nbits;
    const uint32_t start = (uint32_t)(u * DEC_UNIT - g0);
    const uint32_t stop = (uint32_t)(lim - g0);
    uint32_t p = start;
    unsigned int c = 0;
    uint16_t *b = bnd + u * DEC_NB;
    while (p < stop) {
        if (c < DEC_NB) b[c] = (uint16_t)(p - start);
        if (dec_sym(t, slut, sw, p) < 0) {
            atomicExch(err, 1);
            break;
        }
        c++;
    }
    for (unsigned int k = c; k < DEC_NB; k++) b[k] = 0xffff;
    end[u] = g0 + p;
    cnt[u] = c;
}

// Synchronisation pass: unit u restarts at the true end of unit u-1 (given
// in `start_in`, a copy of the previous pass's ends) and decodes until its
// position meets a boundary of its speculative decode; from there the two
// decodes coincide.  Units that do not meet one within the recorded window
// decode to the end.  Sets *changed when any end moved.
__global__ void __launch_bounds__(DEC_T) k_decode_resync(DecTables t, const uint32_t *__restrict__ w32,
                                                        uint64_t nwords, uint64_t nbits, uint64_t nunits,
                                                        const uint64_t *end_in, uint64_t *end_out,
                                                        unsigned int *cnt, const uint16_t *bnd, uint64_t *start,
                                                        int *changed) {
    __shared__ uint32_t slut[1 << LUT_BITS];
    __shared__ uint32_t sw[DEC_SEG];
    const uint64_t u0 = (uint64_t)blockIdx.x * DEC_T;
    dec_stage(t, w32, nwords, slut, sw, u0 * DEC_WORDS);
    const uint64_t u = u0 + threadIdx.x;
    if (u >= nunits) return;
    const uint64_t g0 = u0 * DEC_UNIT;
    const uint64_t s_true = u == 0 ? 0 : end_in[u - 1];
    if (s_true == start[u]) {
        end_out[u] = end_in[u];
        return;
    }
    uint64_t lim = (u + 1) * DEC_UNIT;
    if (lim > nbits) lim = nbits;
    const uint32_t nominal = (uint32_t)(u * DEC_UNIT - g0);
    const uint32_t stop = (uint32_t)(lim - g0);
    if (s_true < g0 || s_true - g0 > stop + 64) {
        atomicExch(changed, -1);
        return;
    }
    uint32_t p = (uint32_t)(s_true - g0);
    const bool first_pass = start[u] == u * DEC_UNIT;
    // the speculative boundaries, ascending (unused entries are 0xffff)
    uint32_t bw[DEC_NB / 2];
    const uint32_t *b32 = reinterpret_cast<const uint32_t *>(bnd + u * DEC_NB);
#pragma unroll
    for (int k = 0; k < DEC_NB / 2; k++) bw[k] = first_pass ? b32[k] : 0xffffffffu;
    unsigned int c = 0;
    bool synced = false;
    int j = 0;  // first speculative boundary not yet passed
    while (p < stop) {
        const uint32_t off = p - nominal;
        while (j < DEC_NB) {
            uint32_t bj = (bw[j >> 1] >> ((j & 1) * 16)) & 0xffffu;
            if (bj >= off) break;
            j++;
        }
        if (j < DEC_NB && ((bw[j >> 1] >> ((j & 1) * 16)) & 0xffffu) == off) {
            c += cnt[u] - j;
            synced = true;
            break;
        }
        if (dec_sym(t, slut, sw, p) < 0) {
            atomicExch(changed, -1);
            return;
        }
        c++;
    }
    const uint64_t e = synced ? end_in[u] : g0 + p;
    start[u] = s_true;
    cnt[u] = c;
    end_out[u] = e;
    if (e != end_in[u]) atomicCAS(changed, 0, 1);
}

// Final pass: decode unit u from its true start into out[off[u]...].
template <typename C>
__global__ void __launch_bounds__(DEC_T) k_decode_write(DecTables t, const uint32_t *__restrict__ w32, uint64_t nwords,
                                                       uint64_t nbits, uint64_t nunits, const uint64_t *start,
                                                       const unsigned long long *off, uint64_t nout, int offset,
                                                       C *out) {
    __shared__ uint32_t slut[1 << LUT_BITS];
    __shared__ uint32_t sw[DEC_SEG];
    const uint64_t u0 = (uint64_t)blockIdx.x * DEC_T;
    dec_stage(t, w32, nwords, slut, sw, u0 * DEC_WORDS);
    const uint64_t u = u0 + threadIdx.x;
    if (u >= nunits) return;
    const uint64_t g0 = u0 * DEC_UNIT;
    uint64_t lim = (u + 1) * DEC_UNIT;
    if (lim > nbits) lim = nbits;
    uint32_t p = (uint32_t)(start[u] - g0);
    const uint32_t stop = (uint32_t)(lim - g0);
    uint64_t o = off[u];
    if constexpr (sizeof(C) != 2) {  // wide codes: one store per symbol
        while (p < stop && o < nout) {
            int s = dec_sym(t, slut, sw, p);
            if (s < 0) return;
            out[o++] = (C)(s + offset);
        }
    } else {
    // 2-byte stores up to a 16-byte boundary, then 8 symbols per store
    while (p < stop && o < nout && (o & 7)) {
        int s = dec_sym(t, slut, sw, p);
        if (s < 0) return;
        out[o++] = (C)(s + offset);
    }
    uint32_t pk[4];
    int k = 0;
    while (p < stop && o + k < nout) {
        int s = dec_sym(t, slut, sw, p);
        if (s < 0) break;
        uint32_t v = (uint32_t)(uint16_t)(s + offset);
        if (k & 1) pk[k >> 1] |= v << 16;
        else pk[k >> 1] = v;
        if (++k == 8) {
            *reinterpret_cast<uint4 *>((uint16_t *)out + o) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            o += 8;
            k = 0;
        }
    }
    for (int i = 0; i < k; i++) out[o + i] = (C)(uint16_t)(pk[i >> 1] >> ((i & 1) * 16));
    }
}

template <typename C>
__global__ void k_fill_u16(C *out, uint64_t n, C v) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = v;
}

__global__ void k_widen_counts(const unsigned int *cnt, unsigned long long *out, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = cnt[i];
}

// ------------------------------------------------------------ launchers

static inline unsigned grid_for(uint64_t n, uint64_t per) { return (unsigned)((n + per - 1) / per); }

uint64_t hist_subchunks(uint64_t n) { return ((n + HCHUNK - 1) / HCHUNK) * HWARPS; }

cudaError_t launch_hist_compact(const unsigned long long *hist, const unsigned long long *first, int nsym,
                                unsigned long long *list, unsigned int *nlist, cudaStream_t st) {
    k_hist_compact<<<(unsigned)((nsym + 255) / 256), 256, 0, st>>>(hist, first, nsym, list, nlist);
    return cudaGetLastError();
}

cudaError_t launch_histogram(const uint16_t *codes, uint64_t n, int center, unsigned long long *hist,
                             unsigned long long *first, unsigned long long *zcount, cudaStream_t st) {
    k_histogram<uint16_t><<<grid_for(n, HCHUNK), 1024, 0, st>>>(codes, n, center, hist, first, zcount);
    return cudaGetLastError();
}
cudaError_t launch_histogram(const uint32_t *codes, uint64_t n, int center, unsigned long long *hist,
                             unsigned long long *first, unsigned long long *zcount, cudaStream_t st) {
    k_histogram<uint32_t><<<grid_for(n, HCHUNK), 1024, 0, st>>>(codes, n, center, hist, first, zcount);
    return cudaGetLastError();
}

cudaError_t launch_count_zeros(const uint16_t *codes, uint64_t n, unsigned long long *zcount, cudaStream_t st) {
    k_count_zeros<uint16_t><<<grid_for(n, HCHUNK), 1024, 0, st>>>(codes, n, zcount);
    return cudaGetLastError();
}
cudaError_t launch_count_zeros(const uint32_t *codes, uint64_t n, unsigned long long *zcount, cudaStream_t st) {
    k_count_zeros<uint32_t><<<grid_for(n, HCHUNK), 1024, 0, st>>>(codes, n, zcount);
    return cudaGetLastError();
}

template <typename T, typename C>
cudaError_t launch_compact_zeros(const C *codes, uint64_t n, const unsigned long long *zcount,
                                 const unsigned long long *zoff, uint64_t *zpos, const T *scratch, T *vals,
                                 cudaStream_t st) {
    k_compact_zeros<T, C><<<grid_for(n, HCHUNK), 1024, 0, st>>>(codes, n, zcount, zoff, zpos, scratch, vals);
    return cudaGetLastError();
}
#define FAZ_INST_COMPACT(T, C)                                                                               \
    template cudaError_t launch_compact_zeros<T, C>(const C *, uint64_t, const unsigned long long *,       \
                                                    const unsigned long long *, uint64_t *, const T *, T *, \
                                                    cudaStream_t);
FAZ_INST_COMPACT(float, uint16_t)
FAZ_INST_COMPACT(double, uint16_t)
FAZ_INST_COMPACT(float, uint32_t)
FAZ_INST_COMPACT(double, uint32_t)
#undef FAZ_INST_COMPACT

uint64_t scan_temp_words(uint64_t n) { return (n + SCAN_B - 1) / SCAN_B + 1; }

cudaError_t launch_scan_u64(const unsigned long long *in, unsigned long long *out, uint64_t n,
                            unsigned long long *temp, cudaStream_t st) {
    uint64_t nb = (n + SCAN_B - 1) / SCAN_B;
    if (nb == 0) nb = 1;
    k_scan_reduce<<<(unsigned)nb, SCAN_T, 0, st>>>(in, n, temp);
    k_scan_top<<<1, 1024, 0, st>>>(temp, nb);
    k_scan_down<<<(unsigned)nb, SCAN_T, 0, st>>>(in, n, temp, out, nb);
    return cudaGetLastError();
}

uint64_t encode_chunks(uint64_t n) { return (n + ENC_CHUNK - 1) / ENC_CHUNK; }

template <typename C>
cudaError_t encode_bits_impl(const C *codes, uint64_t n, int offset, const uint8_t *len,
                             unsigned long long *chunkbits, cudaStream_t st) {
    k_encode_bits<C><<<grid_for(n, ENC_CHUNK), ENC_THREADS, 0, st>>>(codes, n, offset, len, chunkbits);
    return cudaGetLastError();
}
cudaError_t launch_encode_bits(const uint16_t *codes, uint64_t n, int offset, const uint8_t *len,
                               unsigned long long *chunkbits, cudaStream_t st) {
    return encode_bits_impl(codes, n, offset, len, chunkbits, st);
}
cudaError_t launch_encode_bits(const uint32_t *codes, uint64_t n, int offset, const uint8_t *len,
                               unsigned long long *chunkbits, cudaStream_t st) {
    return encode_bits_impl(codes, n, offset, len, chunkbits, st);
}

template <typename C>
cudaError_t encode_pack_impl(const C *codes, uint64_t n, int offset, const unsigned long long *code64,
                             const unsigned long long *packed, const uint8_t *len, const unsigned long long *chunkoff,
                             uint32_t *out, int maxlen, cudaStream_t st) {
    int words = (int)(((uint64_t)ENC_CHUNK * (uint64_t)maxlen + 31) / 32 + 2);
    size_t sm = (size_t)words * 4;
    cudaError_t e = allow_dynamic_smem((const void *)k_encode_pack<C>);
    if (e != cudaSuccess) return e;
    k_encode_pack<C><<<grid_for(n, ENC_CHUNK), ENC_THREADS, sm, st>>>(codes, n, offset, code64, packed, len,
                                                                       chunkoff, out, words);
    return cudaGetLastError();
}
cudaError_t launch_encode_pack(const uint16_t *codes, uint64_t n, int offset, const unsigned long long *code64,
                               const unsigned long long *packed, const uint8_t *len,
                               const unsigned long long *chunkoff, uint32_t *out, int maxlen, cudaStream_t st) {
    return encode_pack_impl(codes, n, offset, code64, packed, len, chunkoff, out, maxlen, st);
}
cudaError_t launch_encode_pack(const uint32_t *codes, uint64_t n, int offset, const unsigned long long *code64,
                               const unsigned long long *packed, const uint8_t *len,
                               const unsigned long long *chunkoff, uint32_t *out, int maxlen, cudaStream_t st) {
    return encode_pack_impl(codes, n, offset, code64, packed, len, chunkoff, out, maxlen, st);
}

uint64_t decode_units(uint64_t nbits) { return (nbits + DEC_UNIT - 1) / DEC_UNIT; }
uint64_t decode_unit_bits() { return DEC_UNIT; }
int decode_boundaries() { return DEC_NB; }

uint64_t decode_cta_units() { return DEC_T; }

cudaError_t launch_decode_spec(const DecodeTablesDev &td, const uint32_t *w32, uint64_t nwords, uint64_t nbits,
                               uint64_t nunits, uint64_t ubase, uint64_t uend, uint64_t *end, unsigned int *cnt,
                               uint16_t *bnd, int *err, cudaStream_t st) {
    DecTables t{td.lut, td.left, td.right, td.sym, td.leaf};
    if (uend > nunits) uend = nunits;
    if (uend <= ubase) return cudaSuccess;
    k_decode_spec<<<grid_for(uend - ubase, DEC_T), DEC_T, 0, st>>>(t, w32, nwords, nbits, uend, ubase, end, cnt, bnd,
                                                                    err);
    return cudaGetLastError();
}

cudaError_t launch_decode_resync(const DecodeTablesDev &td, const uint32_t *w32, uint64_t nwords, uint64_t nbits,
                                 uint64_t nunits, const uint64_t *end_in, uint64_t *end_out, unsigned int *cnt,
                                 const uint16_t *bnd, uint64_t *start, int *changed, cudaStream_t st) {
    DecTables t{td.lut, td.left, td.right, td.sym, td.leaf};
    k_decode_resync<<<grid_for(nunits, DEC_T), DEC_T, 0, st>>>(t, w32, nwords, nbits, nunits, end_in, end_out, cnt,
                                                                bnd, start, changed);
    return cudaGetLastError();
}

template <typename C>
cudaError_t decode_write_impl(const DecodeTablesDev &td, const uint32_t *w32, uint64_t nwords, uint64_t nbits,
                              uint64_t nunits, const uint64_t *start, const unsigned long long *off, uint64_t nout,
                              int offset, C *out, cudaStream_t st) {
    DecTables t{td.lut, td.left, td.right, td.sym, td.leaf};
    k_decode_write<C><<<grid_for(nunits, DEC_T), DEC_T, 0, st>>>(t, w32, nwords, nbits, nunits, start, off, nout,
                                                                  offset, out);
    return cudaGetLastError();
}
cudaError_t launch_decode_write(const DecodeTablesDev &td, const uint32_t *w32, uint64_t nwords, uint64_t nbits,
                                uint64_t nunits, const uint64_t *start, const unsigned long long *off, uint64_t nout,
                                int offset, uint16_t *out, cudaStream_t st) {
    return decode_write_impl(td, w32, nwords, nbits, nunits, start, off, nout, offset, out, st);
}
cudaError_t launch_decode_write(const DecodeTablesDev &td, const uint32_t *w32, uint64_t nwords, uint64_t nbits,
                                uint64_t nunits, const uint64_t *start, const unsigned long long *off, uint64_t nout,
                                int offset, uint32_t *out, cudaStream_t st) {
    return decode_write_impl(td, w32, nwords, nbits, nunits, start, off, nout, offset, out, st);
}

__global__ void k_init_starts(uint64_t *start, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        start[i] = i * DEC_UNIT;
}
cudaError_t launch_init_starts(uint64_t *start, uint64_t n, cudaStream_t st) {
    unsigned g = grid_for(n, 1024);
    if (g > 4096) g = 4096;
    if (g == 0) g = 1;
    k_init_starts<<<g, 1024, 0, st>>>(start, n);
    return cudaGetLastError();
}

cudaError_t launch_fill_u16(uint16_t *out, uint64_t n, uint16_t v, cudaStream_t st) {
    unsigned g = grid_for(n, 1024);
    if (g > 4096) g = 4096;
    if (g == 0) g = 1;
    k_fill_u16<uint16_t><<<g, 1024, 0, st>>>(out, n, v);
    return cudaGetLastError();
}
cudaError_t launch_fill_u16(uint32_t *out, uint64_t n, uint32_t v, cudaStream_t st) {
    unsigned g = grid_for(n, 1024);
    if (g > 4096) g = 4096;
    if (g == 0) g = 1;
    k_fill_u16<uint32_t><<<g, 1024, 0, st>>>(out, n, v);
    return cudaGetLastError();
}

cudaError_t launch_widen_counts(const unsigned int *cnt, unsigned long long *out, uint64_t n, cudaStream_t st) {
    unsigned g = grid_for(n, 1024);
    if (g > 4096) g = 4096;
    if (g == 0) g = 1;
    k_widen_counts<<<g, 1024, 0, st>>>(cnt, out, n);
    return cudaGetLastError();
}

}  // namespace faz
