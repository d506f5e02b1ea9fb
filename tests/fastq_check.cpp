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
    printf("half: ok=%" PRIu64 " undecided=%" PRIu64 " bad=%" PRIu64 "\n", h_ok, h_und, h_bad);
    printf("dequant: ok=%" PRIu64 " undecided=%" PRIu64 " bad=%" PRIu64 "\n", d_ok, d_und, d_bad);
    return (h_bad || d_bad) ? 1 : 0;
}
