// stencil.cuh - interpolation stencils of one lattice target, a line counter
// and the stream positions of first-plane lines, shared by the level kernels
// (interp.cu, finest.cu).
//
// Arithmetic follows the reference's types and operation order (compiled with
// -fmad=false): include/QoZ/utils/Interpolators.hpp:9-36, the emission order
// and boundary stencils of SZInterpolationCompressor.hpp:1306-1417.
#pragma once
#include <cuda_runtime.h>
#include "quant.cuh"

namespace faz {

// Stencil of one target, set up once per lane and sweep: the values it reads
// (shared-memory offsets from the line origin) and the coefficients of the
// reference's formula, folded so that one expression evaluates all of them
// in the reference's operation order:
//   y = ((k1*x1 + k2*x2) + k3*x3) + k4*x4 with 2, 3 or 4 terms, times scale.
// k = +-1 multiplies are exact, so -a + 9b equals (-1)*a + 9*b bit for bit
// and x - c equals x + (-1)*c.
template <typename T>
struct Stencil {
    int i1, i2, i3, i4;  // shared-memory offsets
    T k1, k2, k3, k4, scale;
    int nt;              // 1 copy, 2..4 terms, 5 linear1 (double literals)
};

template <typename T>
__device__ __forceinline__ Stencil<T> make_stencil(int m, int n, int cubic, int st, int sh) {
    Stencil<T> S;
    int o1 = -1, o2 = 1, o3 = -1, o4 = -1;
    S.k1 = 1; S.k2 = 1; S.k3 = 0; S.k4 = 0; S.scale = (T)0.5; S.nt = 2;
    if (!cubic || n < 5) {
        if (m + 1 >= n) {
            if (n < 4) { S.nt = 1; o1 = -1; o2 = -1; }
            else { S.nt = 5; o1 = -3; o2 = -1; }
        }
    } else {
        int ia = (n & 1) ? n - 2 : n - 3;
        if (m == 1) {            // (3a + 6b - c) / 8, a=v0 b=v2 c=v4
            o1 = -1; o2 = 1; o3 = 3; S.k1 = 3; S.k2 = 6; S.k3 = -1; S.nt = 3; S.scale = (T)0.125;
        } else if (m == ia) {    // (-a + 6b + 3c) / 8
            o1 = -3; o2 = -1; o3 = 1; S.k1 = -1; S.k2 = 6; S.k3 = 3; S.nt = 3; S.scale = (T)0.125;
        } else if (m == n - 1) { // (3a - 10b + 15c) / 8
            o1 = -5; o2 = -3; o3 = -1; S.k1 = 3; S.k2 = -10; S.k3 = 15; S.nt = 3; S.scale = (T)0.125;
        } else {                 // (-a + 9b + 9c - d) / 16
            o1 = -3; o2 = -1; o3 = 1; o4 = 3; S.k1 = -1; S.k2 = 9; S.k3 = 9; S.k4 = -1; S.nt = 4;
            S.scale = (T)0.0625;
        }
    }
    S.i1 = ((m + o1) >> sh) * st;
    S.i2 = ((m + o2) >> sh) * st;
    S.i3 = ((m + o3) >> sh) * st;
    S.i4 = ((m + o4) >> sh) * st;
    return S;
}


// CUB = 0: a linear level, whose stencils are copy, (a + b) / 2 or linear1
template <int CUB, typename T>
__device__ __forceinline__ T eval_stencil(const Stencil<T> &S, const T *p) {
    T x1 = p[S.i1], x2 = p[S.i2];
    if (S.nt == 5) return linear1_any(x1, x2);
    if (!CUB) return S.nt == 1 ? x1 : (x1 + x2) * S.scale;
    T x3 = p[S.i3], x4 = p[S.i4];
    T s2 = S.k1 * x1 + S.k2 * x2;
    T s3 = s2 + S.k3 * x3;
    T s4 = s3 + S.k4 * x4;
    T y = S.nt == 4 ? s4 : (S.nt == 3 ? s3 : s2);
    return S.nt == 1 ? x1 : y * S.scale;
}

// Line counter (outer, inner) of lines enumerated row-major with `inner`
// values per outer step, advanced by a fixed stride without division.
struct LineCursor {
    int outer, inner, dout, din, width;
    __device__ __forceinline__ void init(int start, int stride, int w) {
        width = w;
        outer = start / w;
        inner = start - outer * w;
        dout = stride / w;
        din = stride - dout * w;
    }
    __device__ __forceinline__ void next() {
        inner += din;
        outer += dout;
        const bool wrap = inner >= width;
        inner -= wrap ? width : 0;
        outer += wrap ? 1 : 0;
    }
};


// Owner of a first-plane line in decompression: the stream position of the
// line's first code in the previous block that emitted it.
__device__ __forceinline__ uint64_t owner_pos_sweep1(const LevelArgs &a, const BlockGeom &g, const int64_t *bc,
                                                     int P1, int P2, int e1, int e2, int n2) {
    const bool s1 = e1 < g.k1, s2 = e2 < g.k2;
    const int64_t ob0 = bc[0] - ((s1 && P1 == 0) || (s2 && P2 == 0));
    const int64_t ob1 = bc[1] - ((s1 && P1 == 1) || (s2 && P2 == 1));
    const int64_t ob2 = bc[2] - ((s1 && P1 == 2) || (s2 && P2 == 2));
    const int nf = (int)(a.bs / a.s) + 1;
    const int on2 = s2 ? nf : n2;
    const int ok1 = pick3(P1, ob0, ob1, ob2) != 0, ok2 = pick3(P2, ob0, ob1, ob2) != 0;
    const int oe1 = s1 ? (nf - 1) / 2 : e1;
    const int oe2 = s2 ? (nf - 1) / 2 : e2;
    const int one2 = (on2 + 1) / 2 - ok2;
    const int64_t oid = (ob0 * a.nb[1] + ob1) * a.nb[2] + ob2;
    return a.block_off[oid] + (uint64_t)((oe1 - ok1) * one2 + (oe2 - ok2)) * g.t0;
}

__device__ __forceinline__ uint64_t owner_pos_sweep2(const LevelArgs &a, const BlockGeom &g, const int64_t *bc,
                                                     int P2, int q) {
    const int64_t ob0 = bc[0] - (P2 == 0), ob1 = bc[1] - (P2 == 1), ob2 = bc[2] - (P2 == 2);
    const int nf = (int)(a.bs / a.s) + 1;
    const int ok2 = pick3(P2, ob0, ob1, ob2) != 0;
    const int oe2 = (nf - 1) / 2;
    const int one2 = (nf + 1) / 2 - ok2;
    const int64_t oc1 = (int64_t)g.ne1 * one2 * g.t0;
    const int64_t oid = (ob0 * a.nb[1] + ob1) * a.nb[2] + ob2;
    return a.block_off[oid] + oc1 + (uint64_t)(q * one2 + (oe2 - ok2)) * g.t1;
}

}  // namespace faz
