// quant.cuh - device-side stencils and linear quantiser shared by the
// interpolation, block-interpolation and Lorenzo kernels.
//
// Arithmetic follows the reference's types and operation order (compiled with
// -fmad=false): stencils in T (include/QoZ/utils/Interpolators.hpp:9-36),
// quantiser in the T/double mix of include/QoZ/quantizer/IntegerQuantizer.hpp:69-179.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "common.cuh"
#include "fastq.cuh"

namespace faz {

// ---------------------------------------------------------------- stencils
// x/2^k is exact scaling, identical to the reference's division.
template <typename T> __device__ __forceinline__ T i_linear(T a, T b) { return (a + b) * (T)0.5; }
template <typename T> __device__ __forceinline__ T i_linear1(T a, T b) {
    return (T)(-0.5 * (double)a + 1.5 * (double)b);
}
template <typename T> __device__ __forceinline__ T i_quad1(T a, T b, T c) {
    return ((T)3 * a + (T)6 * b - c) * (T)0.125;
}
template <typename T> __device__ __forceinline__ T i_quad2(T a, T b, T c) {
    return (-a + (T)6 * b + (T)3 * c) * (T)0.125;
}
template <typename T> __device__ __forceinline__ T i_quad3(T a, T b, T c) {
    return ((T)3 * a - (T)10 * b + (T)15 * c) * (T)0.125;
}
template <typename T> __device__ __forceinline__ T i_cubic(T a, T b, T c, T d) {
    return (-a + (T)9 * b + (T)9 * c - d) * (T)0.0625;
}

// LinearQuantizer::quantize_and_overwrite (IntegerQuantizer.hpp:69-108).
// Returns the code; v becomes the reconstruction when predictable; uval is
// the value recorded as unpredictable when the code is 0.
template <typename T>
__device__ __forceinline__ int quantize(T &v, T pred, double eb, double recip, int radius, int trim, T &uval) {
    T orig = v;
    if (trim > 0 && fabs((double)orig) <= eb) {
        v = 0;
        uval = 0;
        return trim - 1;
    }
    T diff = orig - pred;
    double x = (double)(diff < 0 ? -diff : diff) * recip;
    uval = orig;
    if (!(x < 2147483647.0)) return 0;
    int qi = (int)x + 1;
    if (qi >= 2 * radius) return 0;
    int half = qi >> 1;
    int q2 = half << 1;
    int code;
    if (diff < 0) {
        q2 = -q2;
        code = radius - half;
    } else {
        code = radius + half;
    }
    T dec = (T)((double)pred + (double)q2 * eb);
    T err = dec - orig;
    if (fabs((double)err) > eb || (trim == 2 && code == 1)) return 0;
    v = dec;
    return code;
}

// ----------------------------------------------------- exact float path
// For float data the reference rounds through double: x = (double)|diff| *
// (1/eb) truncated to int, and dec = (float)((double)pred + (double)q2 * eb).
// GB300 runs double arithmetic at a small fraction of its float rate, so the
// float path below computes both results from float-float products (eb and
// 1/eb held as float pairs, Dekker products via fmaf) and proves each result
// equal to the double computation: floor(x) only matters where it changes
// (floor(x)+1)>>1, i.e. near odd integers, and the final float rounding only
// where the exact value lies near a midpoint between floats.  Within 2^-20
// (floor) or 2^-18 ulp (rounding) of such a boundary, on cancellation, at
// powers of two, zero or non-finite values, the double computation is used.

// Double-precision fallbacks of the float path, kept out of line: inlined,
// the compiler may evaluate them unconditionally (as selects), which on GB300's
// narrow double pipe costs more than the whole float path.
// The out-of-line part returns the code and the value as one 64-bit word:
// reference parameters to an out-of-line function would keep the caller's
// variables in local memory on every path.
static __device__ __noinline__ unsigned long long quantize_dp_f32_packed(float orig, float pred, double eb,
                                                                        double recip, int radius, int trim) {
    float v = orig, uval;
    const int code = quantize<float>(v, pred, eb, recip, radius, trim, uval);
    return ((unsigned long long)(unsigned)code << 32) | (unsigned long long)__float_as_uint(v);
}
__device__ __forceinline__ int quantize_dp_f32(float &v, float pred, double eb, double recip, int radius, int trim,
                                               float &uval) {
    const float orig = v;
    const unsigned long long r = quantize_dp_f32_packed(orig, pred, eb, recip, radius, trim);
    v = __uint_as_float((unsigned)r);
    uval = (trim > 0 && fabs((double)orig) <= eb) ? 0.0f : orig;  // quantize's unpredictable value
    return (int)(unsigned)(r >> 32);
}
static __device__ __noinline__ float dequant_dp_f32(float pred, int q2, double eb) {
    return (float)((double)pred + (double)q2 * eb);
}
static __device__ __noinline__ float linear1_dp_f32(float a, float b) { return i_linear1(a, b); }

// Float specialisation of the quantiser: fast path with the double path as
// the fallback (and, in verify mode, as the check).
__device__ __forceinline__ int quantize_fast(float &v, float pred, const LevelArgs &a, float &uval) {
    float orig = v;
    if (a.trim > 0 && !(fabsf(orig) > a.eblo)) {
        v = 0;
        uval = 0;
        return a.trim - 1;
    }
    float diff = orig - pred;
    // |diff| clearly below eb: floor(x) = 0, half = 0, code = radius, and the
    // reconstruction pred + 0*eb is pred + 0.0f; |pred - orig| = |diff| <= eb.
    if (fabsf(diff) < a.eb_half0) {
        uval = orig;
        v = pred + 0.0f;
        return a.radius;
    }
    int twor = 2 * a.radius;
    int half = half_index_f32(fabsf(diff), a.rh, a.rl, a.twor_f, twor);
    if (half == -1) return quantize_dp_f32(v, pred, a.eb, a.recip, a.radius, a.trim, uval);
    uval = orig;
    if (half == -2) return 0;
    int q2 = half << 1;
    int code;
    if (diff < 0) {
        q2 = -q2;
        code = a.radius - half;
    } else {
        code = a.radius + half;
    }
    float dec;
    if (!dequant_f32(pred, q2, a.eh, a.el, dec)) dec = dequant_dp_f32(pred, q2, a.eb);
    float err = dec - orig;
    if (fabsf(err) > a.eblo || (a.trim == 2 && code == 1)) return 0;
    v = dec;
    return code;
}

template <typename T>
__device__ __forceinline__ int quantize_any(T &v, T pred, const LevelArgs &a, T &uval) {
    if constexpr (sizeof(T) == 4) {
        if (a.fast) {
            if (a.verify) {
                float v2 = v, u2;
                int c2 = quantize<float>(v2, pred, a.eb, a.recip, a.radius, a.trim, u2);
                int c = quantize_fast(v, pred, a, uval);
                if (c != c2 || __float_as_uint(v) != __float_as_uint(v2) ||
                    (c == 0 && __float_as_uint(uval) != __float_as_uint(u2)))
                    atomicAdd(a.verify, 1ull);
                return c;
            }
            return quantize_fast(v, pred, a, uval);
        }
    }
    return quantize<T>(v, pred, a.eb, a.recip, a.radius, a.trim, uval);
}

// LinearQuantizer::recover (IntegerQuantizer.hpp:160-179); code 0 reads the
// unpredictable value of stream position pos.
template <typename T>
__device__ __forceinline__ T recover(T pred, int code, uint64_t pos, double eb, int radius, int trim,
                                     const uint64_t *zpos, uint64_t nz, const T *unpred) {
    if (trim == 2 && code == 1) return 0;
    if (code) return (T)((double)pred + (double)(2 * (code - radius)) * eb);
    uint64_t lo = 0, hi = nz;
    while (lo < hi) {
        uint64_t mid = (lo + hi) >> 1;
        if (zpos[mid] < pos) lo = mid + 1; else hi = mid;
    }
    return lo < nz ? unpred[lo] : (T)0;
}

static __device__ __noinline__ float recover_dp_f32(float pred, int code, uint64_t pos, double eb, int radius, int trim,
                                             const uint64_t *zpos, uint64_t nz, const float *unpred) {
    return recover<float>(pred, code, pos, eb, radius, trim, zpos, nz, unpred);
}

template <typename T>
__device__ __forceinline__ T recover_any(T pred, int code, uint64_t pos, const LevelArgs &a, const uint64_t *zpos,
                                         uint64_t nz, const T *unpred) {
    if constexpr (sizeof(T) == 4) {
        if (a.fast && code != 0 && !(a.trim == 2 && code == 1)) {
            float out;
            if (dequant_f32(pred, 2 * (code - a.radius), a.eh, a.el, out)) {
                if (a.verify) {
                    float ref = recover<float>(pred, code, pos, a.eb, a.radius, a.trim, zpos, nz, unpred);
                    if (__float_as_uint(ref) != __float_as_uint(out)) atomicAdd(a.verify, 1ull);
                }
                return out;
            }
        }
    }
    if constexpr (sizeof(T) == 4) return recover_dp_f32(pred, code, pos, a.eb, a.radius, a.trim, zpos, nz, unpred);
    else return recover<T>(pred, code, pos, a.eb, a.radius, a.trim, zpos, nz, unpred);
}

// ------------------------------------------------------- async copies
// Element copies global -> shared that complete asynchronously (cp.async),
// so that a CTA has its whole lattice load in flight at once.
template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem) {
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    if constexpr (BYTES == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Straight-line reconstruction pred + q2*eb (dequant_f32 without early
// exits); returns true when undecided.
__device__ __forceinline__ bool dequant_f32_straight(float pred, int q2, float eh, float el, float &out) {
    const float q = int_to_float_small(q2);
    const float p1 = q * eh;
    const float e1 = fmaf(q, eh, -p1);
    const float p2 = q * el;
    const float s = pred + p1;
    const float bb = s - pred;
    const float t = (pred - (s - bb)) + (p1 - bb);
    const float lo = t + (e1 + p2);
    const float r = s + lo;
    const float res = (s - r) + lo;
    const float ar = fabsf(r);
    const uint32_t rb = f32_bits(ar);
    const float bigv = fmaxf(fabsf(pred), fabsf(p1));
    const float u = f32_from_bits(rb & 0x7f800000u) * 0x1p-23f;
    const bool und = q2 != 0 && (!(ar >= 0x1p-100f) || ar * 256.0f < bigv || (rb & 0x7fffffu) == 0 ||
                                 rb >= 0x7f000000u || fabsf(fabsf(res) - 0.5f * u) < u * 0x1p-12f);
    out = q2 == 0 ? pred + 0.0f : r;
    return und;
}

// One quantisation: QM 1 is the straight-line float path (trimToZero 0,
// eb within the fast range) with the double computation for undecided
// points; QM 0 is the general path.  v becomes the value the field takes,
// uval the value recorded when the code is 0.
template <typename T, int QM>
__device__ __forceinline__ int quant_point(T &v, T pred, const LevelArgs &a, T &uval) {
    if constexpr (QM == 1 && sizeof(T) == 4) {
        const float orig = v;
        float out;
        bool und;
        int code = quantize_f32_straight(orig, pred, a.rh, a.rl, a.eh, a.el, a.eblo, a.twor_f, a.radius, out, und);
        if (und) {
            out = orig;
            code = quantize_dp_f32(out, pred, a.eb, a.recip, a.radius, 0, uval);
        }
        if (a.verify) {
            float v2 = orig, u2;
            int c2 = quantize<float>(v2, pred, a.eb, a.recip, a.radius, 0, u2);
            if (c2 != code || __float_as_uint(v2) != __float_as_uint(out)) atomicAdd(a.verify, 1ull);
        }
        uval = orig;
        v = out;
        return code;
    } else {
        return quantize_any(v, pred, a, uval);
    }
}

template <typename T, int QM>
__device__ __forceinline__ T recover_point(T pred, int code, uint64_t pos, const LevelArgs &a, const uint64_t *zpos,
                                           uint64_t nz, const T *unpred) {
    if constexpr (QM == 1 && sizeof(T) == 4) {
        float out;
        const bool und = dequant_f32_straight(pred, 2 * (code - a.radius), a.eh, a.el, out);
        if (code == 0 || und) out = recover_dp_f32(pred, code, pos, a.eb, a.radius, 0, zpos, nz, unpred);
        if (a.verify) {
            float ref = recover<float>(pred, code, pos, a.eb, a.radius, 0, zpos, nz, unpred);
            if (__float_as_uint(ref) != __float_as_uint(out)) atomicAdd(a.verify, 1ull);
        }
        return out;
    } else {
        return recover_any(pred, code, pos, a, zpos, nz, unpred);
    }
}

// linear1 evaluates with double constants; float data takes the out-of-line
// double path
template <typename T>
__device__ __forceinline__ T linear1_any(T a, T b) {
    if constexpr (sizeof(T) == 4) return linear1_dp_f32(a, b);
    else return i_linear1(a, b);
}

}  // namespace faz
