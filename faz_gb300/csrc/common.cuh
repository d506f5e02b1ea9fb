// common.cuh - shared definitions of the GB300 FAZ library (device and host).
//
// Geometry of the multilevel interpolation: every field is handled as 3-D
// (1-D and 2-D fields get leading axes of extent 1).  A level with lattice
// stride s cuts the field into blocks of edge bs (interpBlockSize*s, or
// fixBlockSize), row-major (include/QoZ/utils/Iterator.hpp:143-214), block end
// clipped to dim-1 (SZInterpolationCompressor.hpp:424-437).  Inside a block,
// sweep d interpolates lines along axis perm[d] (SZInterpolationCompressor.hpp
// 3143-3360); a block whose begin along an axis is non-zero does not emit the
// lines on that first plane (they belong to the previous block).
#pragma once
#include <cstdint>
#include <cstddef>

#ifdef __CUDACC__
#define FAZ_HD __host__ __device__ __forceinline__
#else
#define FAZ_HD inline
#endif

namespace faz {

// Per-level launch description, computed on the host.
struct LevelArgs {
    int64_t dims[3];     // field extent per axis (axis 2 fastest)
    int64_t offs[3];     // element stride per axis
    int64_t s;           // lattice stride 2^(level-1)
    int64_t bs;          // block edge in elements
    int64_t nb[3];       // blocks per axis
    int perm[3];         // sweep order (axes)
    int cubic;           // 1 = cubic, 0 = linear
    int write_back;      // compress: store reconstructed targets (needed by finer levels)
    int radius;          // quantisation radius
    int trim;            // trimToZero
    double eb;           // this level's error bound
    double recip;        // 1.0 / eb (double division, as LinearQuantizer::set_eb)
    int vwords;          // shared-memory elements reserved for the block lattice
    int stage_cap;       // shared-memory code staging capacity (codes)
    const uint64_t *block_off;  // stream position of each block's first code
    uint64_t ncodes;     // codes in the whole stream (bounds every code read)
    int *err;            // set to 1 by a kernel that met an out-of-range position
    // float fast path: eb and 1/eb split into float pairs, largest float <= eb
    float eh, el, rh, rl, eblo, twor_f;
    float eb_half0;      // |diff| below this float gives half index 0 for sure
    int fast;            // 1: float data uses the exact float fast path
    unsigned long long *verify;  // non-null: count fast/double disagreements here
};

// Lattice geometry of one block.
struct BlockGeom {
    int n[3];        // lattice points per axis (in axis order)
    int sk[3];       // 1 if the block begins past 0 on that axis
    int64_t beg[3];  // first element coordinate per axis
    // in sweep order (P0, P1, P2 = perm[0..2]):
    int n0, n1, n2, k0, k1, k2;
    int h2;          // even lattice points along P2 = (n2+1)/2
    int ne1, ne2;    // emitted even lines along P1 / P2
    int t0, t1, t2;  // targets per line in sweeps 1, 2, 3
    int64_t c1, c2, c3;  // codes emitted by sweeps 1, 2, 3
};

FAZ_HD void block_coords(const LevelArgs &a, int64_t bid, int64_t *bc) {
    bc[2] = bid % a.nb[2];
    int64_t r = bid / a.nb[2];
    bc[1] = r % a.nb[1];
    bc[0] = r / a.nb[1];
}

// element i of (x0, x1, x2) without a runtime-indexed array
template <typename V>
FAZ_HD V pick3(int i, V x0, V x1, V x2) { return i == 0 ? x0 : (i == 1 ? x1 : x2); }

FAZ_HD void block_geom(const LevelArgs &a, const int64_t *bc, BlockGeom &g) {
    for (int d = 0; d < 3; d++) {
        int64_t b = bc[d] * a.bs;
        int64_t e = b + a.bs;
        if (e > a.dims[d] - 1) e = a.dims[d] - 1;
        g.beg[d] = b;
        g.n[d] = (int)((e - b) / a.s + 1);
        g.sk[d] = b != 0;
    }
    g.n0 = pick3(a.perm[0], g.n[0], g.n[1], g.n[2]);
    g.n1 = pick3(a.perm[1], g.n[0], g.n[1], g.n[2]);
    g.n2 = pick3(a.perm[2], g.n[0], g.n[1], g.n[2]);
    g.k0 = pick3(a.perm[0], g.sk[0], g.sk[1], g.sk[2]);
    g.k1 = pick3(a.perm[1], g.sk[0], g.sk[1], g.sk[2]);
    g.k2 = pick3(a.perm[2], g.sk[0], g.sk[1], g.sk[2]);
    g.h2 = (g.n2 + 1) / 2;
    g.ne1 = (g.n1 + 1) / 2 - g.k1;
    g.ne2 = (g.n2 + 1) / 2 - g.k2;
    g.t0 = g.n0 / 2;
    g.t1 = g.n1 / 2;
    g.t2 = g.n2 / 2;
    g.c1 = (int64_t)g.ne1 * g.ne2 * g.t0;
    g.c2 = (int64_t)(g.n0 - g.k0) * g.ne2 * g.t1;
    g.c3 = (int64_t)(g.n0 - g.k0) * (g.n1 - g.k1) * g.t2;
}

// Stream rank of odd lattice index m inside a line of n points
// (emission order of block_interpolation_1d, SZInterpolationCompressor.hpp:1306-1417):
// linear / short lines ascend; cubic lines emit interior points 3,5,...,
// then 1, then the first odd index past the interior, then n-1 for even n.
FAZ_HD int line_rank(int m, int n, int cubic) {
    if (!cubic || n < 5) return (m - 1) >> 1;
    int ia = (n & 1) ? n - 2 : n - 3;
    int cint = (ia - 3) >> 1;
    if (m == 1) return cint;
    if (m == ia) return cint + 1;
    if (m == n - 1) return cint + 2;
    return (m - 3) >> 1;
}

}  // namespace faz
