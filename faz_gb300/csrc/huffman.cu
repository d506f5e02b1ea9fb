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
// Counts of every symbol, the stream position of its first occurrence, and
// the number of zero codes per chunk.  Symbols within +-HWIN/2 of `center`
// are counted in shared memory.
static constexpr int HWIN = 4096;

__global__ void __launch_bounds__(1024) k_histogram(const uint16_t *__restrict__ codes, uint64_t n, uint64_t chunk,
                                                    int center, unsigned long long *hist,
                                                    unsigned long long *first, unsigned long long *zcount) {
    __shared__ unsigned int scnt[HWIN];
    __shared__ unsigned int sfirst[HWIN];
    __shared__ unsigned int szero;
    for (int i = threadIdx.x; i < HWIN; i += blockDim.x) {
        scnt[i] = 0;
        sfirst[i] = 0xffffffffu;
    }
    if (threadIdx.x == 0) szero = 0;
    __syncthreads();
    const uint64_t c0 = (uint64_t)blockIdx.x * chunk;
    uint64_t c1 = c0 + chunk;
    if (c1 > n) c1 = n;
    const int lo = center - HWIN / 2;
    unsigned int zc = 0;
    for (uint64_t i = c0 + threadIdx.x; i < c1; i += blockDim.x) {
        int v = codes[i];
        unsigned int off = (unsigned int)(i - c0);
        if (v == 0) zc++;
        int b = v - lo;
        if (b >= 0 && b < HWIN) {
            atomicAdd(&scnt[b], 1u);
            atomicMin(&sfirst[b], off);
        } else {
            atomicAdd(&hist[v], 1ull);
            atomicMin(&first[v], (unsigned long long)i);
        }
    }
    for (int o = 16; o > 0; o >>= 1) zc += __shfl_down_sync(0xffffffffu, zc, o);
    if ((threadIdx.x & 31) == 0 && zc) atomicAdd(&szero, zc);
    __syncthreads();
    for (int b = threadIdx.x; b < HWIN; b += blockDim.x) {
        if (scnt[b]) {
            atomicAdd(&hist[lo + b], (unsigned long long)scnt[b]);
            atomicMin(&first[lo + b], (unsigned long long)(c0 + sfirst[b]));
        }
    }
    if (threadIdx.x == 0) zcount[blockIdx.x] = szero;
}

// Gather the unpredictable values (stream order) from the per-position
// scratch: chunk c's zero codes go to unpred[zoff[c]...].
template <typename T>
__global__ void __launch_bounds__(1024) k_gather_unpred(const uint16_t *__restrict__ codes, uint64_t n, uint64_t chunk,
                                                        const unsigned long long *zcount,
                                                        const unsigned long long *zoff, const T *scratch, T *unpred) {
    if (zcount[blockIdx.x] == 0) return;
    __shared__ unsigned int wsum[32];
    __shared__ unsigned long long run;
    const uint64_t c0 = (uint64_t)blockIdx.x * chunk;
    uint64_t c1 = c0 + chunk;
    if (c1 > n) c1 = n;
    if (threadIdx.x == 0) run = zoff[blockIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (uint64_t b = c0; b < c1; b += blockDim.x) {
        uint64_t i = b + threadIdx.x;
        bool z = i < c1 && codes[i] == 0;
        unsigned int bal = __ballot_sync(0xffffffffu, z);
        unsigned int before = __popc(bal & ((1u << lane) - 1));
        if (lane == 0) wsum[wid] = __popc(bal);
        __syncthreads();
        unsigned long long wbase = run;
        for (int w = 0; w < wid; w++) wbase += wsum[w];
        if (z) unpred[wbase + before] = scratch[i];
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long s = 0;
            for (int w = 0; w < nw; w++) s += wsum[w];
            run += s;
        }
        __syncthreads();
    }
}

// Stream positions of the zero codes (for recovery of unpredictable values).
__global__ void __launch_bounds__(1024) k_zero_positions(const uint16_t *__restrict__ codes, uint64_t n,
                                                         uint64_t chunk, const unsigned long long *zcount,
                                                         const unsigned long long *zoff, uint64_t *zpos) {
    if (zcount[blockIdx.x] == 0) return;
    __shared__ unsigned int wsum[32];
    __shared__ unsigned long long run;
    const uint64_t c0 = (uint64_t)blockIdx.x * chunk;
    uint64_t c1 = c0 + chunk;
    if (c1 > n) c1 = n;
    if (threadIdx.x == 0) run = zoff[blockIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (uint64_t b = c0; b < c1; b += blockDim.x) {
        uint64_t i = b + threadIdx.x;
        bool z = i < c1 && codes[i] == 0;
        unsigned int bal = __ballot_sync(0xffffffffu, z);
        unsigned int before = __popc(bal & ((1u << lane) - 1));
        if (lane == 0) wsum[wid] = __popc(bal);
        __syncthreads();
        unsigned long long wbase = run;
        for (int w = 0; w < wid; w++) wbase += wsum[w];
        if (z) zpos[wbase + before] = i;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long s = 0;
            for (int w = 0; w < nw; w++) s += wsum[w];
            run += s;
        }
        __syncthreads();
    }
}

// Zero-code count per chunk (decompress side).
__global__ void __launch_bounds__(1024) k_count_zeros(const uint16_t *__restrict__ codes, uint64_t n, uint64_t chunk,
                                                      unsigned long long *zcount) {
    __shared__ unsigned int s;
    if (threadIdx.x == 0) s = 0;
    __syncthreads();
    const uint64_t c0 = (uint64_t)blockIdx.x * chunk;
    uint64_t c1 = c0 + chunk;
    if (c1 > n) c1 = n;
    unsigned int zc = 0;
    for (uint64_t i = c0 + threadIdx.x; i < c1; i += blockDim.x) zc += codes[i] == 0;
    for (int o = 16; o > 0; o >>= 1) zc += __shfl_down_sync(0xffffffffu, zc, o);
    if ((threadIdx.x & 31) == 0 && zc) atomicAdd(&s, zc);
    __syncthreads();
    if (threadIdx.x == 0) zcount[blockIdx.x] = s;
}

// Exclusive scan of n 64-bit values in one CTA; total written to out[n].
__global__ void __launch_bounds__(1024) k_scan_u64(const unsigned long long *in, unsigned long long *out, uint64_t n) {
    __shared__ unsigned long long part[1024];
    const uint64_t per = (n + blockDim.x - 1) / blockDim.x;
    const uint64_t a = threadIdx.x * per;
    uint64_t b = a + per;
    if (b > n) b = n;
    unsigned long long s = 0;
    for (uint64_t i = a; i < b; i++) s += in[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
        unsigned long long v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned long long run = threadIdx.x ? part[threadIdx.x - 1] : 0;
    for (uint64_t i = a; i < b; i++) {
        unsigned long long v = in[i];
        out[i] = run;
        run += v;
    }
    if (threadIdx.x == blockDim.x - 1) out[n] = part[threadIdx.x];
}

// ------------------------------------------------------------------ encode
// Symbol tables indexed by (code - offset): MSB-aligned code, bit length.
static constexpr int ENC_PER_THREAD = 16;
static constexpr int ENC_THREADS = 256;
static constexpr int ENC_CHUNK = ENC_PER_THREAD * ENC_THREADS;

__global__ void __launch_bounds__(ENC_THREADS) k_encode_bits(const uint16_t *__restrict__ codes, uint64_t n, int offset,
                                                            const uint8_t *__restrict__ len,
                                                            unsigned long long *chunkbits) {
    __shared__ unsigned long long ws[ENC_THREADS / 32];
    const uint64_t c0 = (uint64_t)blockIdx.x * ENC_CHUNK;
    unsigned long long s = 0;
    for (int k = 0; k < ENC_PER_THREAD; k++) {
        uint64_t i = c0 + (uint64_t)k * ENC_THREADS + threadIdx.x;
        if (i < n) s += len[codes[i] - offset];
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
__global__ void __launch_bounds__(ENC_THREADS) k_encode_pack(const uint16_t *__restrict__ codes, uint64_t n, int offset,
                                                            const unsigned long long *__restrict__ code64,
                                                            const uint8_t *__restrict__ len,
                                                            const unsigned long long *__restrict__ chunkoff,
                                                            uint32_t *out, int smem_words) {
    extern __shared__ uint32_t sw[];
    __shared__ unsigned long long tsum[ENC_THREADS];
    const uint64_t c0 = (uint64_t)blockIdx.x * ENC_CHUNK;
    const uint64_t gbit = chunkoff[blockIdx.x];
    const uint64_t gend = chunkoff[blockIdx.x + 1];
    if (gend == gbit) return;
    const uint64_t w0 = gbit >> 5;
    const uint64_t wl = (gend - 1) >> 5;
    const int nwords = (int)(wl - w0 + 1);
    for (int i = threadIdx.x; i < nwords && i < smem_words; i += blockDim.x) sw[i] = 0;
    uint16_t sym[ENC_PER_THREAD];
    unsigned long long mybits = 0;
    const uint64_t t0 = c0 + (uint64_t)threadIdx.x * ENC_PER_THREAD;
    for (int k = 0; k < ENC_PER_THREAD; k++) {
        uint64_t i = t0 + k;
        sym[k] = i < n ? (uint16_t)(codes[i] - offset) : 0xffff;
        if (i < n) mybits += len[sym[k]];
    }
    tsum[threadIdx.x] = mybits;
    __syncthreads();
    for (int o = 1; o < ENC_THREADS; o <<= 1) {
        unsigned long long v = threadIdx.x >= (unsigned)o ? tsum[threadIdx.x - o] : 0;
        __syncthreads();
        tsum[threadIdx.x] += v;
        __syncthreads();
    }
    uint64_t pos = (gbit & 31) + (tsum[threadIdx.x] - mybits);  // bit position relative to word w0
    for (int k = 0; k < ENC_PER_THREAD; k++) {
        if (sym[k] == 0xffff) break;
        int l = len[sym[k]];
        if (l == 0) continue;
        unsigned long long c = code64[sym[k]];
        int wi = (int)(pos >> 5), b = (int)(pos & 31);
        uint32_t p0 = (uint32_t)(c >> (32 + b));
        if (p0) atomicOr(&sw[wi], p0);
        if (l + b > 32) {
            uint32_t p1 = (uint32_t)((c << (32 - b)) >> 32);
            if (b == 0) p1 = (uint32_t)c;
            if (p1) atomicOr(&sw[wi + 1], p1);
        }
        if (l + b > 64) {
            uint32_t p2 = (uint32_t)(c << (32 - b));
            if (p2) atomicOr(&sw[wi + 2], p2);
        }
        pos += l;
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
struct DecTables {
    const uint32_t *lut;     // 2^LUT_BITS entries: (len << 24) | state, or DEC_NODE | node
    const uint32_t *left, *right;
    const int32_t *sym;      // state of a leaf
    const uint8_t *leaf;
};
static constexpr int LUT_BITS = 12;
static constexpr uint32_t DEC_NODE = 0x80000000u;

__device__ __forceinline__ uint64_t bswap64(uint64_t x) {
    uint32_t lo = (uint32_t)x, hi = (uint32_t)(x >> 32);
    return ((uint64_t)bswap32(lo) << 32) | bswap32(hi);
}

// 64 bits of the stream starting at bit p (the buffer is padded by 16 bytes).
__device__ __forceinline__ uint64_t peek64(const uint64_t *__restrict__ w, uint64_t p) {
    uint64_t i = p >> 6;
    int sh = (int)(p & 63);
    uint64_t a = bswap64(w[i]);
    if (!sh) return a;
    uint64_t b = bswap64(w[i + 1]);
    return (a << sh) | (b >> (64 - sh));
}

// Decode one symbol at bit p; returns its state and advances p.  Codes are
// at most 64 bits long; a walk that finds no leaf within 64 bits (a damaged
// tree) returns -1 and moves p past `stop`.
__device__ __forceinline__ int dec_one(const DecTables &t, const uint32_t *slut, const uint64_t *w, uint64_t &p,
                                       uint64_t stop) {
    uint64_t win = peek64(w, p);
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
    p = stop + 64;
    return -1;
}

// Pass over units: decode from start[u] (unit 0 from bit 0) until the bit
// position reaches the end of the unit; record the end position and count.
// With `refine`, only units whose recorded start differs from the previous
// unit's end are decoded again; `changed` is set when any end moves.
__global__ void __launch_bounds__(256) k_decode_sync(DecTables t, const uint64_t *__restrict__ w, uint64_t nbits,
                                                    uint64_t unit, uint64_t nunits, const uint64_t *end_in,
                                                    uint64_t *start, uint64_t *end_out, unsigned int *cnt,
                                                    int refine, int *changed) {
    __shared__ uint32_t slut[1 << LUT_BITS];
    for (int i = threadIdx.x; i < (1 << LUT_BITS); i += blockDim.x) slut[i] = t.lut[i];
    __syncthreads();
    uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (u >= nunits) return;
    uint64_t lim = (u + 1) * unit;
    if (lim > nbits) lim = nbits;
    uint64_t s;
    if (!refine) {
        s = u * unit;
    } else {
        s = u == 0 ? 0 : end_in[u - 1];
        if (s == start[u]) {
            end_out[u] = end_in[u];
            return;
        }
    }
    uint64_t p = s;
    unsigned int c = 0;
    while (p < lim) {
        if (dec_one(t, slut, w, p, lim) < 0) atomicExch(changed, -1);
        c++;
    }
    start[u] = s;
    end_out[u] = p;
    cnt[u] = c;
    if (refine && p != end_in[u]) atomicCAS(changed, 0, 1);
}

// Final pass: decode unit u from its true start into out[off[u]...].
__global__ void __launch_bounds__(256) k_decode_write(DecTables t, const uint64_t *__restrict__ w, uint64_t nbits,
                                                     uint64_t unit, uint64_t nunits, const uint64_t *start,
                                                     const unsigned long long *off, uint64_t nout, int offset,
                                                     uint16_t *out) {
    __shared__ uint32_t slut[1 << LUT_BITS];
    for (int i = threadIdx.x; i < (1 << LUT_BITS); i += blockDim.x) slut[i] = t.lut[i];
    __syncthreads();
    uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (u >= nunits) return;
    uint64_t lim = (u + 1) * unit;
    if (lim > nbits) lim = nbits;
    uint64_t p = start[u];
    uint64_t o = off[u];
    while (p < lim && o < nout) {
        int s = dec_one(t, slut, w, p, lim);
        if (s < 0) break;
        out[o++] = (uint16_t)(s + offset);
    }
}

__global__ void k_fill_u16(uint16_t *out, uint64_t n, uint16_t v) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = v;
}

__global__ void k_widen_counts(const unsigned int *cnt, unsigned long long *out, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = cnt[i];
}

// ------------------------------------------------------------ launchers

static inline unsigned grid_for(uint64_t n, uint64_t per) { return (unsigned)((n + per - 1) / per); }

cudaError_t launch_histogram(const uint16_t *codes, uint64_t n, uint64_t chunk, int center,
                             unsigned long long *hist, unsigned long long *first, unsigned long long *zcount,
                             cudaStream_t st) {
    k_histogram<<<grid_for(n, chunk), 1024, 0, st>>>(codes, n, chunk, center, hist, first, zcount);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_gather_unpred(const uint16_t *codes, uint64_t n, uint64_t chunk, const unsigned long long *zcount,
                                 const unsigned long long *zoff, const T *scratch, T *unpred, cudaStream_t st) {
    k_gather_unpred<T><<<grid_for(n, chunk), 1024, 0, st>>>(codes, n, chunk, zcount, zoff, scratch, unpred);
    return cudaGetLastError();
}
template cudaError_t launch_gather_unpred<float>(const uint16_t *, uint64_t, uint64_t, const unsigned long long *,
                                                 const unsigned long long *, const float *, float *, cudaStream_t);
template cudaError_t launch_gather_unpred<double>(const uint16_t *, uint64_t, uint64_t, const unsigned long long *,
                                                  const unsigned long long *, const double *, double *,
                                                  cudaStream_t);

cudaError_t launch_count_zeros(const uint16_t *codes, uint64_t n, uint64_t chunk, unsigned long long *zcount,
                               cudaStream_t st) {
    k_count_zeros<<<grid_for(n, chunk), 1024, 0, st>>>(codes, n, chunk, zcount);
    return cudaGetLastError();
}

cudaError_t launch_zero_positions(const uint16_t *codes, uint64_t n, uint64_t chunk, const unsigned long long *zcount,
                                  const unsigned long long *zoff, uint64_t *zpos, cudaStream_t st) {
    k_zero_positions<<<grid_for(n, chunk), 1024, 0, st>>>(codes, n, chunk, zcount, zoff, zpos);
    return cudaGetLastError();
}

cudaError_t launch_scan_u64(const unsigned long long *in, unsigned long long *out, uint64_t n, cudaStream_t st) {
    k_scan_u64<<<1, 1024, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

uint64_t encode_chunks(uint64_t n) { return (n + ENC_CHUNK - 1) / ENC_CHUNK; }

cudaError_t launch_encode_bits(const uint16_t *codes, uint64_t n, int offset, const uint8_t *len,
                               unsigned long long *chunkbits, cudaStream_t st) {
    k_encode_bits<<<grid_for(n, ENC_CHUNK), ENC_THREADS, 0, st>>>(codes, n, offset, len, chunkbits);
    return cudaGetLastError();
}

cudaError_t launch_encode_pack(const uint16_t *codes, uint64_t n, int offset, const unsigned long long *code64,
                               const uint8_t *len, const unsigned long long *chunkoff, uint32_t *out, int maxlen,
                               cudaStream_t st) {
    int words = (int)(((uint64_t)ENC_CHUNK * (uint64_t)maxlen + 31) / 32 + 2);
    size_t sm = (size_t)words * 4;
    cudaError_t e = cudaFuncSetAttribute(k_encode_pack, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k_encode_pack<<<grid_for(n, ENC_CHUNK), ENC_THREADS, sm, st>>>(codes, n, offset, code64, len, chunkoff, out,
                                                                    words);
    return cudaGetLastError();
}

cudaError_t launch_decode_sync(const DecodeTablesDev &td, const uint64_t *w, uint64_t nbits, uint64_t unit,
                               uint64_t nunits, const uint64_t *end_in, uint64_t *start, uint64_t *end_out,
                               unsigned int *cnt, int refine, int *changed, cudaStream_t st) {
    DecTables t{td.lut, td.left, td.right, td.sym, td.leaf};
    k_decode_sync<<<grid_for(nunits, 256), 256, 0, st>>>(t, w, nbits, unit, nunits, end_in, start, end_out, cnt,
                                                          refine, changed);
    return cudaGetLastError();
}

cudaError_t launch_decode_write(const DecodeTablesDev &td, const uint64_t *w, uint64_t nbits, uint64_t unit,
                                uint64_t nunits, const uint64_t *start, const unsigned long long *off, uint64_t nout,
                                int offset, uint16_t *out, cudaStream_t st) {
    DecTables t{td.lut, td.left, td.right, td.sym, td.leaf};
    k_decode_write<<<grid_for(nunits, 256), 256, 0, st>>>(t, w, nbits, unit, nunits, start, off, nout, offset, out);
    return cudaGetLastError();
}

cudaError_t launch_fill_u16(uint16_t *out, uint64_t n, uint16_t v, cudaStream_t st) {
    unsigned g = grid_for(n, 1024);
    if (g > 4096) g = 4096;
    if (g == 0) g = 1;
    k_fill_u16<<<g, 1024, 0, st>>>(out, n, v);
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
