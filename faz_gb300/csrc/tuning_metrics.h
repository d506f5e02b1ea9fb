// tuning_metrics.h - the QoZ tuner's SSIM and autocorrelation targets (host).
//
// With TUNING_TARGET_SSIM or TUNING_TARGET_AC the alpha/beta search's
// CompressTests (include/QoZ/api/impl/SZInterp.hpp:1299-1341, 1376-1378)
// score the reconstruction of the sampled blocks instead of its PSNR:
//   - SSIM: each sampled block of (sbs+1)^N points is cut into cubes of edge
//     SSIMBlockSize, starting at 0, s, 2s, ... while start + s < sbs + 1; the
//     original's mean, variance and range per cube are computed once
//     (SZInterp.hpp:2223-2256), the reconstruction's and the covariance per
//     test, and metric += SSIM / (number of cubes), block by block, cube by
//     cube (include/QoZ/utils/Metrics.hpp:14-151);
//   - AC: 1 - the lag-one autocorrelation of original - reconstruction over
//     all sampled blocks flattened block after block (Metrics.hpp:227-260).
// The sums are sequential in double with the reference's types (values and
// differences in T, 3-D covariance products in T), so every decision that
// compares metrics is the reference's.  The GPU produces the reconstructions;
// these loops are a few passes over the sample on the host.
#pragma once
#include <cstddef>
#include <cstdint>
#include <vector>

namespace faz {

struct SsimCubes {
    int N = 3;
    size_t bsz = 0, s = 0;
    std::vector<double> mean, sigma2, range;  // the original's, per cube
};

// blockwise_profiling (Metrics.hpp:24-102)
template <typename T>
void cube_profile(const T *d, int N, size_t bsz, size_t i0, size_t j0, size_t k0, size_t s, double &mean,
                  double &sigma2, double &range) {
    double sum = 0, mx, mn, sg = 0;
    if (N == 2) {
        const size_t en = s * s;
        mx = mn = d[i0 * bsz + j0];
        for (size_t i = i0; i < i0 + s; i++)
            for (size_t j = j0; j < j0 + s; j++) {
                const T v = d[i * bsz + j];
                sum += v;
                mx = v > mx ? v : mx;
                mn = v < mn ? v : mn;
            }
        mean = sum / en;
        for (size_t i = i0; i < i0 + s; i++)
            for (size_t j = j0; j < j0 + s; j++) {
                const T v = d[i * bsz + j];
                sg += (v - mean) * (v - mean);
            }
        range = mx - mn;
        sigma2 = sg / en;
        return;
    }
    const size_t en = s * s * s, yz = bsz * bsz;
    mx = mn = d[i0 * yz + j0 * bsz + k0];
    for (size_t i = i0; i < i0 + s; i++)
        for (size_t j = j0; j < j0 + s; j++)
            for (size_t k = k0; k < k0 + s; k++) {
                const T v = d[i * yz + j * bsz + k];
                sum += v;
                mx = v > mx ? v : mx;
                mn = v < mn ? v : mn;
            }
    mean = sum / en;
    for (size_t i = i0; i < i0 + s; i++)
        for (size_t j = j0; j < j0 + s; j++)
            for (size_t k = k0; k < k0 + s; k++) {
                const T v = d[i * yz + j * bsz + k];
                sg += (v - mean) * (v - mean);
            }
    range = mx - mn;
    sigma2 = sg / en;
}

// blockwise_cov (Metrics.hpp:104-151)
template <typename T>
double cube_cov(const T *d, const T *d2, int N, size_t bsz, size_t i0, size_t j0, size_t k0, size_t s, double mean,
                double mean2) {
    double cs = 0;
    if (N == 2) {
        const size_t en = s * s;
        for (size_t i = i0; i < i0 + s; i++)
            for (size_t j = j0; j < j0 + s; j++) {
                const T v = d[i * bsz + j], v2 = d2[i * bsz + j];
                cs += (v - mean) * (v2 - mean2);
            }
        return cs / en;
    }
    const size_t en = s * s * s, yz = bsz * bsz;
    for (size_t i = i0; i < i0 + s; i++)
        for (size_t j = j0; j < j0 + s; j++)
            for (size_t k = k0; k < k0 + s; k++) {
                const T v = d[i * yz + j * bsz + k], v2 = d2[i * yz + j * bsz + k];
                const T p = v * v2;
                cs += p;
            }
    return cs / en - mean * mean2;
}

// SSIM (Metrics.hpp:14-22)
inline double ssim_of(double xr, double xm, double xv2, double ym, double yv2, double cov) {
    double c1 = 0.0001, c2 = 0.0009;
    if (xr > 0) {
        c1 *= (xr * xr);
        c2 *= xr * xr;
    }
    return (2 * xm * ym + c1) * (2 * cov + c2) / ((xm * xm + ym * ym + c1) * (xv2 + yv2 + c2));
}

// calls f(i, j, k) for every SSIM cube of a block, in the reference's order
template <typename F>
void for_cubes(int N, size_t bsz, size_t s, F f) {
    for (size_t i = 0; i + s < bsz; i += s)
        for (size_t j = 0; j + s < bsz; j += s) {
            if (N == 2) {
                f(i, j, (size_t)0);
                continue;
            }
            for (size_t k = 0; k + s < bsz; k += s) f(i, j, k);
        }
}

// the original's cube statistics (SZInterp.hpp:2223-2256)
template <typename T>
SsimCubes ssim_cubes(const T *blocks, size_t nblk, int N, size_t bsz, size_t s) {
    SsimCubes c;
    c.N = N;
    c.bsz = bsz;
    c.s = s;
    const size_t per = N == 3 ? bsz * bsz * bsz : bsz * bsz;
    for (size_t b = 0; b < nblk; b++)
        for_cubes(N, bsz, s, [&](size_t i, size_t j, size_t k) {
            double m, v, r;
            cube_profile(blocks + b * per, N, bsz, i, j, k, s, m, v, r);
            c.mean.push_back(m);
            c.sigma2.push_back(v);
            c.range.push_back(r);
        });
    return c;
}

// the SSIM target's metric of reconstructions `cur` of `orig` (both block
// after block)
template <typename T>
double ssim_metric(const SsimCubes &c, const T *orig, const T *cur, size_t nblk) {
    const size_t per = c.N == 3 ? c.bsz * c.bsz * c.bsz : c.bsz * c.bsz;
    const size_t ncube = c.mean.size();
    double metric = 0;
    size_t idx = 0;
    for (size_t b = 0; b < nblk; b++)
        for_cubes(c.N, c.bsz, c.s, [&](size_t i, size_t j, size_t k) {
            double m, v, r;
            cube_profile(cur + b * per, c.N, c.bsz, i, j, k, c.s, m, v, r);
            const double cov = cube_cov(orig + b * per, cur + b * per, c.N, c.bsz, i, j, k, c.s, c.mean[idx], m);
            metric += ssim_of(c.range[idx], c.mean[idx], c.sigma2[idx], m, v, cov) / ncube;
            idx++;
        });
    return metric;
}

// autocorrelation (Metrics.hpp:227-260) of data - data2
template <typename T>
double autocorrelation_of(const T *data, const T *data2, size_t n) {
    std::vector<T> diffs(n);
    double avg = 0;
    for (size_t i = 0; i < n; i++) {
        const T v = data[i] - data2[i];
        avg += v;
        diffs[i] = v;
    }
    avg /= n;
    double cov = 0;
    for (size_t i = 0; i < n; i++) {
        const T v = (T)(diffs[i] - avg);
        const T p = v * v;
        cov += p;
    }
    cov /= n;
    if (cov == 0) return 1.0;
    double sum = 0;
    for (size_t i = 0; i + 1 < n; i++) sum += (diffs[i] - avg) * (diffs[i + 1] - avg);
    return sum / (n - 1) / cov;
}

}  // namespace faz
