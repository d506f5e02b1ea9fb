// CPU check of the exact float quantiser emulation (faz_gb300/csrc/fastq.cuh)
// against the reference's double computation, on random and adversarial
// inputs.  A decided result must equal the double result bit for bit;
// "undecided" (fall back to double) is allowed and counted.
// Usage: fastq_check <cases> <seed>; prints counts; exit 1 on any mismatch.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../faz_gb300/csrc/fastq.cuh"

using namespace faz;

struct Split {
    double eb, recip;
    float eh, el, rh, rl;
};

static Split split(double eb) {
    Split s;
    s.eb = eb;
    s.recip = 1.0 / eb;
    s.eh = (float)eb;
    s.el = (float)(eb - (double)s.eh);
    s.rh = (float)s.recip;
    s.rl = (float)(s.recip - (double)s.rh);
    return s;
}

static int ref_half(float d, double recip, int twor) {
    double x = (double)d * recip;
    if (!(x < 2147483647.0)) return -2;
    int qi = (int)x + 1;
    if (qi >= twor) return -2;
    return qi >> 1;
}

// LinearQuantizer::quantize_and_overwrite for float data, trimToZero = 0,
// in the reference's float/double arithmetic
static int ref_quantize(float orig, float pred, double eb, int radius, float &out) {
    double recip = 1.0 / eb;
    float diff = orig - pred;
    double x = (double)std::fabs(diff) * recip;
    out = orig;
    if (!(x < 2147483647.0)) return 0;
    int qi = (int)x + 1;
    if (qi >= radius * 2) return 0;
    qi >>= 1;
    int half = qi;
    qi <<= 1;
    int code;
    if (diff < 0) { qi = -qi; code = radius - half; } else code = radius + half;
    float dec = (float)((double)pred + (double)qi * eb);
    float err = dec - orig;
    if (std::fabs((double)err) > eb) return 0;
    out = dec;
    return code;
}

int main(int argc, char **argv) {
    uint64_t cases = argc > 1 ? strtoull(argv[1], 0, 10) : 1000000;
    uint64_t seed = argc > 2 ? strtoull(argv[2], 0, 10) : 1;
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    uint64_t h_ok = 0, h_bad = 0, h_und = 0, d_ok = 0, d_bad = 0, d_und = 0;
    const int twor = 65536;
    for (uint64_t i = 0; i < cases; i++) {
        // error bound: wide magnitudes, decimal-looking values, powers of two
        double eb;
        int kind = (int)(rng() % 4);
        if (kind == 0) eb = std::pow(10.0, -8 + 11 * U(rng)) * (1 + U(rng));
        else if (kind == 1) eb = std::ldexp(1.0, -30 + (int)(rng() % 40));
        else if (kind == 2) eb = (double)(1 + rng() % 1000) * std::pow(10.0, -(int)(rng() % 9));
        else eb = 1e-3 * (double)(float)(130 * U(rng));
        Split s = split(eb);
        // ---- half index
        float d;
        int dk = (int)(rng() % 5);
        if (dk == 0) {
            d = (float)(U(rng) * 70000 * eb);
        } else if (dk == 1) {
            int K = 2 * (int)(rng() % 33000) + 1;  // odd boundary
            double t = ((double)K + (U(rng) - 0.5) * std::ldexp(1.0, -(int)(rng() % 40))) * eb;
            d = (float)t;
            int nudge = (int)(rng() % 5) - 2;
            for (int k = 0; k < std::abs(nudge); k++) d = std::nextafter(d, nudge > 0 ? INFINITY : 0.0f);
        } else if (dk == 2) {
            d = (float)((double)(rng() % 66000) * eb);
        } else if (dk == 3) {
            d = (float)(U(rng) * 4 * eb);
        } else {
            d = std::ldexp((float)U(rng), -(int)(rng() % 60));
        }
        d = std::fabs(d);
        int got = half_index_f32(d, s.rh, s.rl, (float)twor, twor);
        int ref = ref_half(d, s.recip, twor);
        if (got == -1) h_und++;
        else if (got == ref) h_ok++;
        else {
            if (h_bad < 10)
                printf("half mismatch: d=%a eb=%a got=%d ref=%d\n", (double)d, eb, got, ref);
            h_bad++;
        }
        // ---- dequantisation
        int half = (int)(rng() % 40000);
        if (rng() % 4 == 0) half = (int)(rng() % 4);
        int q2 = 2 * half * ((rng() & 1) ? 1 : -1);
        float pred;
        int pk = (int)(rng() % 5);
        if (pk == 0) {
            pred = (float)((U(rng) - 0.5) * 200);
        } else if (pk == 1) {
            // exact sum close to a midpoint between two floats
            float v = (float)((U(rng) - 0.5) * 200);
            double mid = (double)v + 0.5 * (double)(std::nextafter(v, INFINITY) - v);
            mid += (U(rng) - 0.5) * std::ldexp(std::fabs((double)v), -(int)(30 + rng() % 30));
            pred = (float)(mid - (double)q2 * eb);
        } else if (pk == 2) {
            pred = (float)(-(double)q2 * eb * (1 + (U(rng) - 0.5) * 1e-6));  // cancellation
        } else if (pk == 3) {
            pred = std::ldexp(1.0f, (int)(rng() % 20) - 10) * ((rng() & 1) ? 1 : -1);
        } else {
            pred = (rng() & 1) ? 0.0f : -0.0f;
        }
        float out;
        float refd = (float)((double)pred + (double)q2 * eb);
        if (!dequant_f32(pred, q2, s.eh, s.el, out)) d_und++;
        else if (f32_bits(out) == f32_bits(refd)) d_ok++;
        else {
            if (d_bad < 10)
                printf("dequant mismatch: pred=%a q2=%d eb=%a got=%a ref=%a\n", (double)pred, q2, eb, (double)out,
                       (double)refd);
            d_bad++;
        }
    }
    // ---- straight-line quantiser vs the reference arithmetic
    uint64_t q_ok = 0, q_und = 0, q_bad = 0;
    std::mt19937_64 rng2(seed * 7 + 1);
    for (uint64_t i = 0; i < cases; i++) {
        double eb;
        int kind = (int)(rng2() % 3);
        if (kind == 0) eb = std::pow(10.0, -6 + 8 * U(rng2)) * (1 + U(rng2));
        else if (kind == 1) eb = std::ldexp(1.0, -20 + (int)(rng2() % 25));
        else eb = 1e-3 * (double)(float)(130 * U(rng2));
        Split sp = split(eb);
        float eblo = (float)eb;
        if ((double)eblo > eb) eblo = std::nextafter(eblo, 0.0f);
        float pred = (float)((U(rng2) - 0.5) * 200);
        float orig;
        int ok = (int)(rng2() % 6);
        if (ok == 0) orig = pred + (float)((U(rng2) - 0.5) * 10 * eb);
        else if (ok == 1) orig = (float)((double)pred + (2.0 * (int)(rng2() % 50) - 49 + (U(rng2) - 0.5) * 1e-6) * eb);
        else if (ok == 2) orig = (float)((double)pred + (double)(int)(rng2() % 200000 - 100000) * eb);
        else if (ok == 3) orig = pred;
        else if (ok == 4) orig = std::nextafter(pred, (rng2() & 1) ? INFINITY : -INFINITY);
        else orig = (float)((U(rng2) - 0.5) * 1e-3);
        int radius = (rng2() % 8 == 0) ? 1 + (int)(rng2() % 1000) : 32768;
        float out_ref, out;
        bool und;
        int cref = ref_quantize(orig, pred, eb, radius, out_ref);
        int c = quantize_f32_straight(orig, pred, sp.rh, sp.rl, sp.eh, sp.el, eblo, (float)(2 * radius), radius, out, und);
        if (und) q_und++;
        else if (c == cref && f32_bits(out) == f32_bits(out_ref)) q_ok++;
        else {
            if (q_bad < 10)
                printf("quantize mismatch: orig=%a pred=%a eb=%a r=%d got=(%d,%a) ref=(%d,%a)\n", (double)orig,
                       (double)pred, eb, radius, c, (double)out, cref, (double)out_ref);
            q_bad++;
        }
    }
    printf("quantize: ok=%" PRIu64 " undecided=%" PRIu64 " bad=%" PRIu64 "\n", q_ok, q_und, q_bad);
    if (q_bad) return 1;
    printf("half: ok=%" PRIu64 " undecided=%" PRIu64 " bad=%" PRIu64 "\n", h_ok, h_und, h_bad);
    printf("dequant: ok=%" PRIu64 " undecided=%" PRIu64 " bad=%" PRIu64 "\n", d_ok, d_und, d_bad);
    return (h_bad || d_bad) ? 1 : 0;
}
