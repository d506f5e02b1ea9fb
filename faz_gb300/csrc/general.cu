// general.cu - the general Lorenzo frontend for 1-D and 2-D fields
// (SZ_compress_LorenzoReg / SZ_decompress_LorenzoReg with N < 3,
// include/QoZ/api/impl/SZLorenzoReg.hpp:28-135): SZGeneralFrontend
// (include/QoZ/frontend/SZGeneralFrontend.hpp:19-150) with the one- and
// two-layer Lorenzo predictors (include/QoZ/predictor/LorenzoPredictor.hpp),
// combined by ComposedPredictor (include/QoZ/predictor/ComposedPredictor.hpp)
// when both are enabled.
//
// The reference walks blocks in row-major order and, inside a block, points
// in row-major order; each point is predicted from reconstructed values
// (zero outside the field) and overwritten by its reconstruction.  A block's
// predictor is chosen from estimates taken on the current data: original
// values inside the block, reconstructed ones before it.  In 2-D a block only
// reads the blocks above, to the left and above-left, so blocks on one
// anti-diagonal are independent: one launch per block diagonal, one warp per
// block, a shared-memory tile with a 2-deep halo of reconstructed values.
// Inside a block the points of one anti-diagonal are independent as well.
// In 1-D every point depends on the one before it; one thread walks the field.
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

struct GenArgs {
    int64_t d0, d1;    // field extents (1-D: d1 = 1)
    int64_t nb0, nb1;  // blocks per axis
    int bs;
    int lo, lo2;       // one- / two-layer Lorenzo enabled
    double noise1, noise2;  // LorenzoPredictor(eb) noise for L = 1, 2
    LevelArgs q;       // quantiser
};

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

// One block diagonal bi + bj = d; one warp per block.
template <typename T, bool DECOMP, int QM>
__global__ void __launch_bounds__(kGenWarps * 32)
    k_gen2_diag(GenArgs a, int64_t d, int64_t bi_lo, const T *__restrict__ X, T *__restrict__ R,
                uint16_t *__restrict__ codes, T *__restrict__ scratch, uint16_t *__restrict__ sel,
                const uint64_t *__restrict__ zpos, uint64_t nzp, const T *__restrict__ unpred) {
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
    int L;
    if (a.lo && a.lo2) {
        if (!DECOMP) {
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
            L = sel[b] == 1 ? 2 : 1;
        }
    } else {
        L = a.lo ? 1 : 2;
    }
    const uint64_t boff = (uint64_t)i0 * (uint64_t)a.d1 + (uint64_t)j0 * (uint64_t)sx;
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
    for (int e = lane; e < sx * sy; e += 32) {
        const int i = e / sy, j = e - i * sy;
        R[(i0 + i) * a.d1 + (j0 + j)] = t[(i + 2) * ty + (j + 2)];
    }
}

// 1-D: one thread walks the blocks and their points in order.
template <typename T, bool DECOMP, int QM>
__global__ void k_gen1(GenArgs a, const T *__restrict__ X, T *__restrict__ R, uint16_t *__restrict__ codes,
                       T *__restrict__ scratch, uint16_t *__restrict__ sel, const uint64_t *__restrict__ zpos,
                       uint64_t nzp, const T *__restrict__ unpred) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const int64_t n = a.d0;
    const T n1 = (T)a.noise1, n2 = (T)a.noise2;
    T r1 = 0, r2 = 0;  // reconstructed values at i - 1, i - 2
    for (int64_t bi = 0; bi < a.nb0; bi++) {
        const int64_t i0 = bi * a.bs;
        const int64_t sx = i0 + a.bs < n ? a.bs : n - i0;
        int L;
        if (a.lo && a.lo2) {
            if (!DECOMP) {
                // estimates at the block's first and last point on the current data
                auto at = [&](int64_t p) -> T {  // current value at p (p <= i0 + sx - 1)
                    if (p < 0) return (T)0;
                    if (p >= i0) return X[p];
                    return p == i0 - 1 ? r1 : (p == i0 - 2 ? r2 : R[p]);
                };
                const int64_t pa = i0, pb = i0 + sx - 1;
                double e1 = 0, e2 = 0;
                {
                    const T da = at(pa) - at(pa - 1), db = at(pb) - at(pb - 1);
                    e1 += (double)(T)(fabs((double)da) + (double)n1);
                    e1 += (double)(T)(fabs((double)db) + (double)n1);
                    const T ea = at(pa) - (2 * at(pa - 1) - at(pa - 2));
                    const T eb2 = at(pb) - (2 * at(pb - 1) - at(pb - 2));
                    e2 += (double)(T)(fabs((double)ea) + (double)n2);
                    e2 += (double)(T)(fabs((double)eb2) + (double)n2);
                }
                L = e2 < e1 ? 2 : 1;
                sel[bi] = (uint16_t)(L - 1);
            } else {
                L = sel[bi] == 1 ? 2 : 1;
            }
        } else {
            L = a.lo ? 1 : 2;
        }
        for (int64_t i = i0; i < i0 + sx; i++) {
            const T pred = L == 1 ? r1 : 2 * r1 - r2;
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
}

template <typename T>
GenArgs make_gen_args(int N, const uint64_t *dims, int bs, int lo, int lo2, double eb, int radius) {
    GenArgs a;
    std::memset(&a, 0, sizeof(a));
    a.d0 = (int64_t)dims[0];
    a.d1 = N == 2 ? (int64_t)dims[1] : 1;
    a.bs = bs;
    a.nb0 = (a.d0 - 1) / bs + 1;
    a.nb1 = N == 2 ? (a.d1 - 1) / bs + 1 : 1;
    a.lo = lo;
    a.lo2 = lo2;
    a.noise1 = (N == 1 ? 0.5 : 0.81) * eb;
    a.noise2 = (N == 1 ? 1.08 : 2.76) * eb;
    a.q.eb = eb;
    a.q.recip = 1.0 / eb;
    a.q.radius = radius;
    a.q.trim = 0;
    set_fast_path<T>(a.q);
    return a;
}

template <typename T>
void gen_run(int N, const GenArgs &a, bool decomp, const T *X, T *R, uint16_t *codes, T *scratch, uint16_t *sel,
             const uint64_t *zpos, uint64_t nz, const T *unpred, cudaStream_t st, Counter &launches) {
    const bool straight = sizeof(T) == 4 && a.q.fast;
    if (N == 1) {
        void (*k)(GenArgs, const T *, T *, uint16_t *, T *, uint16_t *, const uint64_t *, uint64_t, const T *);
        if (!decomp) k = straight ? k_gen1<T, false, 1> : k_gen1<T, false, 0>;
        else k = straight ? k_gen1<T, true, 1> : k_gen1<T, true, 0>;
        k<<<1, 32, 0, st>>>(a, X, R, codes, scratch, sel, zpos, nz, unpred);
        launches(cudaGetLastError());
        return;
    }
    const size_t smem = (size_t)kGenWarps * (size_t)((a.bs + 2) * (a.bs + 2)) * sizeof(T);
    void (*k)(GenArgs, int64_t, int64_t, const T *, T *, uint16_t *, T *, uint16_t *, const uint64_t *, uint64_t,
              const T *);
    if (!decomp) k = straight ? k_gen2_diag<T, false, 1> : k_gen2_diag<T, false, 0>;
    else k = straight ? k_gen2_diag<T, true, 1> : k_gen2_diag<T, true, 0>;
    CK(allow_dynamic_smem((const void *)k));
    for (int64_t d = 0; d <= (a.nb0 - 1) + (a.nb1 - 1); d++) {
        const int64_t bi_lo = std::max<int64_t>(0, d - (a.nb1 - 1));
        const int64_t bi_hi = std::min<int64_t>(a.nb0 - 1, d);
        const int64_t cnt = bi_hi - bi_lo + 1;
        k<<<(unsigned)((cnt + kGenWarps - 1) / kGenWarps), kGenWarps * 32, smem, st>>>(a, d, bi_lo, X, R, codes,
                                                                                      scratch, sel, zpos, nz, unpred);
        launches(cudaGetLastError());
    }
}

void check_gen(int N, int bs, int lo, int lo2, int radius) {
    if (N != 1 && N != 2) throw Fail{FAZ_ERR_ARG, "the general Lorenzo frontend here covers 1-D and 2-D data"};
    if (bs < 2) throw Fail{FAZ_ERR_UNSUPPORTED, "Lorenzo block size must be at least 2 on the GPU path"};
    if (N == 2 && bs > kGenMaxBs) throw Fail{FAZ_ERR_UNSUPPORTED, "2-D Lorenzo block size above 64 is not implemented"};
    if (!lo && !lo2) throw Fail{FAZ_ERR_ARG, "all Lorenzo and regression methods are disabled"};
    if (radius < 1 || radius > 32768)
        throw Fail{FAZ_ERR_UNSUPPORTED, "quantbinCnt above 65536 is not implemented on the GPU path"};
}

}  // namespace

// SZGeneralFrontend::compress + save and the Huffman stage of the general
// compressor: the pre-zstd payload of a 1-D / 2-D field (Lorenzo predictors).
template <typename T>
void gen_compress_payload(int N, const uint64_t *dims, int bs, int lo, int lo2, double eb, int radius, const T *dX,
                          cudaStream_t st, Counter &launches, faz_timings &tm, std::vector<uint8_t> &out) {
    check_gen(N, bs, lo, lo2, radius);
    const GenArgs a = make_gen_args<T>(N, dims, bs, lo, lo2, eb, radius);
    const uint64_t n = (uint64_t)(a.d0 * a.d1), nb = (uint64_t)(a.nb0 * a.nb1);
    const bool composed = lo && lo2;
    DevMem m(st);
    T *R = m.alloc<T>(n), *scratch = m.alloc<T>(n);
    uint16_t *codes = m.alloc<uint16_t>(n), *sel = m.alloc<uint16_t>(nb);
    Events ev_pred, ev_huff;
    CK(cudaEventRecord(ev_pred.a, st));
    gen_run<T>(N, a, false, dX, R, codes, scratch, sel, nullptr, 0, nullptr, st, launches);
    CK(cudaEventRecord(ev_pred.b, st));
    CK(cudaEventRecord(ev_huff.a, st));
    HuffEncoded hs, hc;
    if (composed) huffman_encode_device(sel, nb, 0, m, st, launches, hs, tm);
    huffman_encode_device(codes, n, radius, m, st, launches, hc, tm);
    const uint64_t nunpred = hc.nzero;
    T *unp = m.alloc<T>(nunpred ? nunpred : 1);
    if (nunpred) launches(launch_compact_zeros<T>(codes, n, hc.zc, hc.zoff, nullptr, scratch, unp, st));
    CK(cudaEventRecord(ev_huff.b, st));
    // SZGeneralFrontend::save: dims, block size, predictors (ids; the
    // composed predictor's selections), LinearQuantizer::save; then the codes
    std::vector<uint8_t> h0;
    for (int i = 0; i < N; i++) put<uint64_t>(h0, dims[i]);
    put<uint32_t>(h0, (uint32_t)bs);
    put<uint8_t>(h0, 1);  // LorenzoPredictor predictor_id
    if (composed) {
        put<uint8_t>(h0, 1);
        put<uint64_t>(h0, nb);
        append_tree(h0, hs.cb, hs.nbytes);
    }
    const size_t sbits = composed ? hs.nbytes : 0;
    std::vector<uint8_t> h1;
    put<uint8_t>(h1, 2);
    put<double>(h1, eb);
    put<int32_t>(h1, radius);
    put<uint64_t>(h1, nunpred);
    std::vector<uint8_t> h2;
    append_tree(h2, hc.cb, hc.nbytes);
    const size_t total = h0.size() + sbits + h1.size() + nunpred * sizeof(T) + h2.size() + hc.nbytes;
    // device parts come back through the thread's pinned staging buffer
    uint8_t *pin = t_pin_payload.get(total + 8);
    uint8_t *p = pin;
    std::memcpy(p, h0.data(), h0.size());
    p += h0.size();
    if (sbits) CK(cudaMemcpyAsync(p, hs.bits, sbits, cudaMemcpyDeviceToHost, st));
    p += sbits;
    std::memcpy(p, h1.data(), h1.size());
    p += h1.size();
    if (nunpred) CK(cudaMemcpyAsync(p, unp, nunpred * sizeof(T), cudaMemcpyDeviceToHost, st));
    p += nunpred * sizeof(T);
    std::memcpy(p, h2.data(), h2.size());
    p += h2.size();
    if (hc.nbytes) CK(cudaMemcpyAsync(p, hc.bits, hc.nbytes, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    out.assign(pin, pin + total);
    tm.unpred_count = nunpred;
    tm.payload_bytes = total;
    tm.predict_ms += ev_pred.ms();
    tm.huffman_ms += ev_huff.ms();
}

// SZGeneralFrontend::load + decompress into dOut (device); lo / lo2 come
// from the stream's Config and fix the predictor list.
template <typename T>
void gen_decompress(int N, const uint8_t *pl, size_t psize, const uint64_t *dims, int lo, int lo2, T *dOut,
                    cudaStream_t st, Counter &launches, faz_timings &tm) {
    const uint8_t *p = pl, *end = pl + psize;
    auto need = [&](size_t k) {
        if ((size_t)(end - p) < k) throw Fail{FAZ_ERR_FORMAT, "truncated Lorenzo stream"};
    };
    need((size_t)N * 8 + 4 + 1);
    for (int i = 0; i < N; i++) {
        uint64_t v;
        std::memcpy(&v, p, 8);
        p += 8;
        if (v != dims[i]) throw Fail{FAZ_ERR_FORMAT, "payload dims differ from the trailer"};
    }
    uint32_t bs;
    std::memcpy(&bs, p, 4);
    p += 4;
    p += 1;  // predictor id
    const bool composed = lo && lo2;
    check_gen(N, (int)bs, lo, lo2, 1);
    const GenArgs a0 = make_gen_args<T>(N, dims, (int)bs, lo, lo2, 1.0, 1);
    const uint64_t n = (uint64_t)(a0.d0 * a0.d1), nb = (uint64_t)(a0.nb0 * a0.nb1);
    DevMem m(st);
    uint16_t *sel = m.alloc<uint16_t>(nb);
    Events ev_dec, ev_pred;
    CK(cudaEventRecord(ev_dec.a, st));
    if (composed) {
        need(1 + 8);
        p += 1;
        uint64_t ns;
        std::memcpy(&ns, p, 8);
        p += 8;
        if (ns != nb) throw Fail{FAZ_ERR_FORMAT, "selection count differs from the block count"};
        huffman_decode_device(p, end, nb, sel, m, st, launches);
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
    check_gen(N, (int)bs, lo, lo2, radius);
    if ((size_t)(end - p) / sizeof(T) < nunpred) throw Fail{FAZ_ERR_FORMAT, "truncated unpredictable values"};
    T *dunp = m.alloc<T>(nunpred ? nunpred : 1);
    if (nunpred) CK(cudaMemcpyAsync(dunp, p, nunpred * sizeof(T), cudaMemcpyHostToDevice, st));
    p += nunpred * sizeof(T);
    uint16_t *codes = m.alloc<uint16_t>(n);
    huffman_decode_device(p, end, n, codes, m, st, launches);
    uint64_t *zpos = nullptr;
    const uint64_t nz = zero_positions(codes, n, m, st, launches, zpos);
    if (nz != nunpred) throw Fail{FAZ_ERR_FORMAT, "unpredictable count does not match the zero codes"};
    CK(cudaEventRecord(ev_dec.b, st));
    const GenArgs a = make_gen_args<T>(N, dims, (int)bs, lo, lo2, eb, radius);
    CK(cudaEventRecord(ev_pred.a, st));
    gen_run<T>(N, a, true, nullptr, dOut, codes, nullptr, sel, zpos, nz, dunp, st, launches);
    CK(cudaEventRecord(ev_pred.b, st));
    CK(cudaStreamSynchronize(st));
    tm.huffman_ms += ev_dec.ms();
    tm.predict_ms += ev_pred.ms();
}

template void gen_compress_payload<float>(int, const uint64_t *, int, int, int, double, int, const float *,
                                          cudaStream_t, Counter &, faz_timings &, std::vector<uint8_t> &);
template void gen_compress_payload<double>(int, const uint64_t *, int, int, int, double, int, const double *,
                                           cudaStream_t, Counter &, faz_timings &, std::vector<uint8_t> &);
template void gen_decompress<float>(int, const uint8_t *, size_t, const uint64_t *, int, int, float *, cudaStream_t,
                                    Counter &, faz_timings &);
template void gen_decompress<double>(int, const uint8_t *, size_t, const uint64_t *, int, int, double *, cudaStream_t,
                                     Counter &, faz_timings &);

}  // namespace faz
