// fastq.cuh - exact float emulation of the reference quantiser's double steps.
//
// For float data the reference rounds through double
// (include/QoZ/quantizer/IntegerQuantizer.hpp:80-97):
//   x = (double)|data - pred| * (1.0 / eb);  qi = (int)x + 1;  half = qi >> 1
//   dec = (float)((double)pred + (double)q2 * eb),  q2 = +-2*half
// GB300 runs double arithmetic at a small fraction of its float rate.  The
// functions below compute the same integers and floats from float-float
// products (eb and 1/eb split into float pairs, exact products via fmaf) and
// report "undecided" whenever the float computation cannot prove the result:
//   - floor(x) only matters where it changes (floor(x) + 1) >> 1, i.e. near odd
//     integers; within 2^-20 of one the double path decides;
//   - the final rounding to float only matters where the exact value lies near
//     a midpoint between two floats; within 2^-12 ulp of one, on cancellation
//     (|result| < |terms| / 256), at powers of two, zero, tiny or huge values
//     the double path decides.
// Both functions are __host__ __device__ so that tests can check them on the
// CPU against the double computation.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#include "common.cuh"

namespace faz {

FAZ_HD uint32_t f32_bits(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    uint32_t u;
    std::memcpy(&u, &x, 4);
    return u;
#endif
}
FAZ_HD float f32_from_bits(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x;
    std::memcpy(&x, &u, 4);
    return x;
#endif
}

// Integer <-> float for |x| < 2^22 with one float add and integer ops
// (GB300 executes float<->int conversions and float rounding on its narrow
// double-precision pipe): adding 1.5*2^23 leaves round-to-nearest(x) in the
// low mantissa bits.
constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int32_t kMagicBits = 0x4B400000;
FAZ_HD int32_t rint_small(float x) { return (int32_t)f32_bits(x + kMagic) - kMagicBits; }
FAZ_HD float int_to_float_small(int32_t i) { return f32_from_bits((uint32_t)(i + kMagicBits)) - kMagic; }

// floor((floor(x) + 1) / 2) for x = RN_double(d * recip), recip = rh + rl.
// Returns -1 when undecided, -2 when floor(x) + 1 >= twor (unpredictable).
// twor <= 65536, so ph < twor keeps every value below 2^22.
FAZ_HD int half_index_f32(float d, float rh, float rl, float twor_f, int twor) {
    float ph = d * rh;
    if (!(ph < twor_f)) return ph != ph ? -1 : -2;
    float pl = fmaf(d, rh, -ph);
    float c = fmaf(d, rl, pl);
    // k = floor(ph): nearest integer, minus one if it lies above ph
    int32_t ki = rint_small(ph);
    float kf = int_to_float_small(ki);
    if (kf > ph) {
        ki -= 1;
        kf -= 1.0f;
    }
    float f = (ph - kf) + c;        // in (-1/256, 1 + 1/256)
    int32_t ri = rint_small(f);     // -1, 0, 1 or 2
    float fr = f - int_to_float_small(ri);  // in [-1/2, 1/2]
    int fl;
    if (fabsf(fr) > 0x1p-20f) {
        fl = ki + ri - (fr < 0.0f ? 1 : 0);
    } else {
        int B = ki + ri;
        if (B & 1) return -1;  // floor is B-1 or B, with different halves
        fl = B;                // floor is B-1 or B, same half B/2
    }
    int qi = fl + 1;
    if (qi >= twor) return -2;
    return qi >> 1;
}

// RN_float(RN_double(pred + RN_double(q2 * eb))), eb = eh + el (+ a residual
// below 2^-48 eb).  Returns false when undecided.
FAZ_HD bool dequant_f32(float pred, int q2, float eh, float el, float &out) {
    if (q2 == 0) {
        out = pred + 0.0f;
        return true;
    }
    float q = int_to_float_small(q2);  // |q2| <= 65536
    float p1 = q * eh;
    float e1 = fmaf(q, eh, -p1);
    float p2 = q * el;
    float s = pred + p1;
    float bb = s - pred;
    float t = (pred - (s - bb)) + (p1 - bb);
    float lo = t + (e1 + p2);
    float r = s + lo;
    float res = (s - r) + lo;
    float ar = fabsf(r);
    uint32_t ri = f32_bits(ar);
    float big = fmaxf(fabsf(pred), fabsf(p1));
    // Error budget in units of u = ulp(r), with cancellation C = big/|r| <= 2^8:
    // double roundings of the reference <= 2^-29 C, float-pair product and
    // the sum of the low parts <= 2^-24 C each, res itself <= 2^-25; total
    // < 2^-14.5, against a 2^-12 margin.
    if (!(ar >= 0x1p-100f) || ar * 256.0f < big || (ri & 0x7fffffu) == 0 || ri >= 0x7f000000u) return false;
    float u = f32_from_bits(ri & 0x7f800000u) * 0x1p-23f;
    if (fabsf(fabsf(res) - 0.5f * u) < u * 0x1p-12f) return false;
    out = r;
    return true;
}

// Straight-line form of the float quantiser for trimToZero = 0 (the
// reference's quantize_and_overwrite, IntegerQuantizer.hpp:69-108, with the
// double steps replaced by half_index_f32 / dequant_f32 above).  Returns the
// code and the value the field takes (reconstruction, or orig when the code
// is 0).  `undecided` is set when the float proofs do not settle the result;
// the caller then runs the double computation.
FAZ_HD int quantize_f32_straight(float orig, float pred, float rh, float rl, float eh, float el, float eblo,
                                 float twor_f, int radius, float &out, bool &undecided) {
    const float diff = orig - pred;
    const float d = fabsf(diff);
    const float ph = d * rh;
    const bool nan_in = ph != ph;
    const bool big = !(ph < twor_f) && !nan_in;
    const float phc = (ph < twor_f) ? ph : 0.0f;
    const float pl = fmaf(d, rh, -ph);
    const float c = (ph < twor_f) ? fmaf(d, rl, pl) : 0.0f;
    int32_t ki = rint_small(phc);
    float kf = int_to_float_small(ki);
    const bool over = kf > phc;
    ki -= over ? 1 : 0;
    kf -= over ? 1.0f : 0.0f;
    const float f = (phc - kf) + c;
    const int32_t ri = rint_small(f);
    const float fr = f - int_to_float_small(ri);
    const bool near = !(fabsf(fr) > 0x1p-20f);
    const int32_t B = ki + ri;
    const int32_t fl = near ? B : B - (fr < 0.0f ? 1 : 0);
    const int twor = 2 * radius;
    const int qi = fl + 1;
    const bool unpred_q = big || qi >= twor;
    const int half = qi >> 1;
    const bool neg = diff < 0;
    const int q2 = unpred_q ? 0 : (neg ? -(half << 1) : (half << 1));
    const int code = neg ? radius - half : radius + half;
    // reconstruction (dequant_f32 without branches)
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
    const bool und_d = q2 != 0 && (!(ar >= 0x1p-100f) || ar * 256.0f < bigv || (rb & 0x7fffffu) == 0 ||
                                   rb >= 0x7f000000u || fabsf(fabsf(res) - 0.5f * u) < u * 0x1p-12f);
    const float dec = q2 == 0 ? pred + 0.0f : r;
    const float err = dec - orig;
    const bool unpred = unpred_q || fabsf(err) > eblo;
    undecided = nan_in || (near && (B & 1)) || (!unpred_q && und_d);
    out = unpred ? orig : dec;
    return unpred ? 0 : code;
}

}  // namespace faz
