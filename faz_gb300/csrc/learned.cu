// learned.cu - the learned tuner: block-statistic features, a small MLP
// (64 -> 256 -> 256 -> 27 logits) trained on the GPU by the library's own
// forward / backward / Adam kernels, and BF16 inference on the 5th-generation
// tensor cores (tcgen05.mma with the accumulator in tensor memory).
//
// The network predicts what the QoZ-style sampled autotune decides
// (include/QoZ/api/impl/SZInterp.hpp:1857-2113 per-level interpolator and
// direction, 2194-2543 alpha/beta search) and whether the SZ3 sampled tuner
// (SZInterp.hpp:2115-2187) picks Lorenzo over interpolation.  It has no
// counterpart in the reference: it replaces the trial compressions, and the
// quantiser still enforces the error bound point by point, so a wrong
// prediction costs compression ratio, never accuracy.
//
// Feature statistics are reduced in a fixed order (per block tree reduction,
// then blocks in order), so features are deterministic.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "host.h"
#include "internal.h"

namespace faz {

namespace {

constexpr int FEB = 33;        // feature block edge (one 32-cell block with its far face)
constexpr int NCFG = 22;       // 12 linear + 9 cubic stencil configurations + misc
constexpr int NST = 7;         // statistics per configuration
constexpr int FT = 256;        // threads per feature block

// ------------------------------------------------------------------ features
// Statistics of one stencil configuration over one block: residuals of the
// linear (x[p-s] + x[p+s]) / 2 or cubic (-x[p-3s] + 9x[p-s] + 9x[p+s] - x[p+3s]) / 16
// prediction along one axis, for every block point whose stencil stays inside
// the block.  cfg 21 gathers value moments.
template <typename T>
__global__ void k_feat_block(const T *x, int64_t d1, int64_t d2, const int64_t *origins, double eb, double *stats) {
    const int blk = blockIdx.x, cfg = blockIdx.y;
    const int64_t o0 = origins[3 * blk], o1 = origins[3 * blk + 1], o2 = origins[3 * blk + 2];
    const T *base = x + (o0 * d1 + o1) * d2 + o2;
    const int64_t st[3] = {d1 * d2, d2, 1};
    double acc[NST];
#pragma unroll
    for (int i = 0; i < NST; i++) acc[i] = 0;
    const int npts = FEB * FEB * FEB;
    if (cfg < 21) {
        const bool cubic = cfg >= 12;
        const int c = cubic ? cfg - 12 : cfg;
        const int s = 1 << (c / 3), axis = c % 3, reach = cubic ? 3 * s : s;
        const int64_t so = st[axis] * s;
        for (int p = threadIdx.x; p < npts; p += FT) {
            const int i0 = p / (FEB * FEB), i1 = (p / FEB) % FEB, i2 = p % FEB;
            const int ia = axis == 0 ? i0 : (axis == 1 ? i1 : i2);
            if (ia - reach < 0 || ia + reach >= FEB) continue;
            const T *q = base + i0 * st[0] + i1 * st[1] + i2 * st[2];
            const double v = (double)q[0];
            double pred;
            if (cubic)
                pred = (-(double)q[-3 * so] + 9.0 * (double)q[-so] + 9.0 * (double)q[so] - (double)q[3 * so]) / 16.0;
            else
                pred = ((double)q[-so] + (double)q[so]) * 0.5;
            const double r = v - pred, ar = fabs(r), r2 = r * r;
            acc[0] += ar;
            acc[1] += ar <= eb ? 1.0 : 0.0;
            acc[2] += 1.0;
            acc[3] += r2;
            acc[4] += ar <= 0.1 * eb ? 1.0 : 0.0;
            acc[5] += ar > 16.0 * eb ? 1.0 : 0.0;
            acc[6] += r2 * r2;
        }
    } else {
        for (int p = threadIdx.x; p < npts; p += FT) {
            const int i0 = p / (FEB * FEB), i1 = (p / FEB) % FEB, i2 = p % FEB;
            const T *q = base + i0 * st[0] + i1 * st[1] + i2;
            const double v = (double)q[0];
            acc[0] += v;
            acc[1] += v * v;
            acc[2] += 1.0;
            if (i2 + 1 < FEB) acc[3] += q[1] == q[0] ? 1.0 : 0.0;
        }
    }
    __shared__ double red[FT];
    for (int k = 0; k < NST; k++) {
        red[threadIdx.x] = acc[k];
        __syncthreads();
        for (int w = FT / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) stats[((int64_t)blk * NCFG + cfg) * NST + k] = red[0];
        __syncthreads();
    }
}

__device__ __forceinline__ float lg2p(double v) { return (float)log2(1.0 + v); }

// Sums the blocks' statistics in block order and writes the FAZ_TUNER_FEATURES
// features (layout in the C header).
__global__ void k_feat_finish(const double *stats, int nblk, double eb, double rng, double rel, double d0, double d1,
                              double d2, float *out) {
    __shared__ double tot[NCFG * NST];
    for (int i = threadIdx.x; i < NCFG * NST; i += blockDim.x) {
        double s = 0;
        for (int b = 0; b < nblk; b++) s += stats[(int64_t)b * NCFG * NST + i];
        tot[i] = s;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    auto S = [&](int cfg, int k) { return tot[cfg * NST + k]; };
    auto mean_abs = [&](int cfg) { return S(cfg, 2) > 0 ? S(cfg, 0) / S(cfg, 2) : 0.0; };
    auto frac = [&](int cfg, int k) { return S(cfg, 2) > 0 ? S(cfg, k) / S(cfg, 2) : 0.0; };
    float f[64];
    for (int c = 0; c < 21; c++) f[c] = lg2p(mean_abs(c) / eb);           // 0..20
    for (int c = 0; c < 21; c++) f[21 + c] = (float)frac(c, 1);           // 21..41
    for (int a = 0; a < 3; a++) f[42 + a] = lg2p(sqrt(frac(a, 3)) / eb);  // 42..44
    for (int a = 0; a < 3; a++) f[45 + a] = lg2p(sqrt(frac(12 + a, 3)) / eb);
    for (int a = 0; a < 3; a++) f[48 + a] = (float)frac(a, 4);
    for (int a = 0; a < 3; a++) f[51 + a] = (float)frac(a, 5);
    {
        const double m2 = frac(2, 3), m4 = frac(2, 6);
        f[54] = m2 > 0 ? (float)log2(m4 / (m2 * m2) + 1e-12) : 0.0f;
    }
    const double n = S(21, 2);
    const double mean = n > 0 ? S(21, 0) / n : 0.0;
    const double var = n > 0 ? fmax(S(21, 1) / n - mean * mean, 0.0) : 0.0;
    f[55] = (float)log2(fmax(rng, 1e-300) / eb);
    f[56] = lg2p(sqrt(var) / eb);
    f[57] = (float)log2(d0);
    f[58] = (float)log2(d1);
    f[59] = (float)log2(d2);
    f[60] = (float)log10(rel);
    f[61] = n > 0 ? (float)(S(21, 3) / n) : 0.0f;
    f[62] = (float)log2((double)nblk);
    f[63] = (f[9] + f[10] + f[11] - f[0] - f[1] - f[2]) / 3.0f;
    for (int i = 0; i < 64; i++) out[i] = isfinite(f[i]) ? f[i] : 0.0f;
}

// ------------------------------------------------------------ MLP training
constexpr int IN = FAZ_TUNER_FEATURES, H = FAZ_TUNER_HIDDEN, OUT = FAZ_TUNER_LOGITS;
constexpr int64_t OFF_W1 = 0, OFF_B1 = OFF_W1 + (int64_t)H * IN, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + (int64_t)H * H,
                  OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + (int64_t)OUT * H, NPARAM = OFF_B3 + OUT;
static_assert(NPARAM == FAZ_TUNER_PARAMS, "parameter layout");

// heads over the logits: (first logit, classes)
__constant__ int c_head_lo[FAZ_TUNER_HEADS] = {0, 4, 8, 12, 16, 21, 25};
__constant__ int c_head_n[FAZ_TUNER_HEADS] = {4, 4, 4, 4, 5, 4, 2};

// C[m, n] = sum_k A(m, k) B(k, n) (+ bias[n]) (relu), strided operands; 16x16
// output tile per block, k in order (deterministic).
__global__ void k_gemm(int M, int N, int K, const float *A, int64_t sam, int64_t sak, const float *B, int64_t sbk,
                       int64_t sbn, float *C, int64_t ldc, const float *bias, int relu, int accumulate) {
    __shared__ float As[16][17], Bs[16][17];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int m = blockIdx.y * 16 + ty, n = blockIdx.x * 16 + tx;
    float acc = 0;
    for (int k0 = 0; k0 < K; k0 += 16) {
        const int ka = k0 + tx, kb = k0 + ty;
        As[ty][tx] = (m < M && ka < K) ? A[m * sam + ka * sak] : 0.0f;
        const int nb = blockIdx.x * 16 + tx;
        Bs[ty][tx] = (kb < K && nb < N) ? B[kb * sbk + nb * sbn] : 0.0f;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 16; k++) acc = fmaf(As[ty][k], Bs[k][tx], acc);
        __syncthreads();
    }
    if (m < M && n < N) {
        if (bias) acc += bias[n];
        if (relu) acc = fmaxf(acc, 0.0f);
        if (accumulate) acc += C[m * ldc + n];
        C[m * ldc + n] = acc;
    }
}

void gemm(cudaStream_t st, int M, int N, int K, const float *A, int64_t sam, int64_t sak, const float *B, int64_t sbk,
          int64_t sbn, float *C, int64_t ldc, const float *bias, bool relu) {
    dim3 blk(16, 16), grd((N + 15) / 16, (M + 15) / 16);
    k_gemm<<<grd, blk, 0, st>>>(M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, bias, relu, 0);
}

// Softmax cross-entropy of every head: dZ = (softmax - onehot) / B for
// labelled heads (label >= 0), 0 otherwise; loss[b] = summed CE of sample b.
__global__ void k_heads_loss(const float *Z, const int32_t *labels, int B, float *dZ, float *loss) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    float tot = 0;
    for (int h = 0; h < FAZ_TUNER_HEADS; h++) {
        const int lo = c_head_lo[h], n = c_head_n[h];
        const int lab = labels[b * FAZ_TUNER_LABELS + h];
        const float *z = Z + (int64_t)b * OUT + lo;
        float *dz = dZ + (int64_t)b * OUT + lo;
        if (lab < 0 || lab >= n) {
            for (int i = 0; i < n; i++) dz[i] = 0;
            continue;
        }
        float mx = z[0];
        for (int i = 1; i < n; i++) mx = fmaxf(mx, z[i]);
        float se = 0;
        for (int i = 0; i < n; i++) se += expf(z[i] - mx);
        const float lse = mx + logf(se);
        tot += lse - z[lab];
        for (int i = 0; i < n; i++) dz[i] = (expf(z[i] - lse) - (i == lab ? 1.0f : 0.0f)) / (float)B;
    }
    loss[b] = tot;
}

__global__ void k_relu_mask(float *d, const float *h, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && h[i] <= 0.0f) d[i] = 0.0f;
}

// db[n] = sum_b dY[b, n] (b in order)
__global__ void k_colsum(const float *dY, int B, int N, float *db) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0;
    for (int b = 0; b < B; b++) s += dY[(int64_t)b * N + n];
    db[n] = s;
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, int64_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2, float wd) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1 - b1) * gi, vi = b2 * v[i] + (1 - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * ((mi / c1) / (sqrtf(vi / c2) + eps) + wd * p[i]);
}

// --------------------------------------------------- tensor-core inference
// Y[M, N] = act(X[M, K] W[N, K]^T + b) with bf16 X, W and an f32 accumulator
// in tensor memory.  One CTA of 128 threads per 128-row tile: all threads
// stage X and W into shared memory in the no-swizzle K-major core-matrix
// layout (8 rows x 16 bytes per core matrix), one thread issues K/16
// tcgen05.mma (M = 128, N, K = 16) and commits them to an mbarrier, and the
// four warps read their 32 accumulator lanes back with tcgen05.ld.
constexpr int TC_M = 128;
constexpr uint32_t TC_WAIT_LIMIT = 1u << 24;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start, leading (K-direction core matrix)
// and stride (8-row group) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16: f32 accumulator, bf16 A and B, both
// K-major, N / 8 and M / 16.
__host__ __device__ constexpr uint32_t tc_idesc(int n, int m) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

template <int K, int N>
__global__ void __launch_bounds__(128, 1)
    k_dense_tc(const __nv_bfloat16 *X, int M, const __nv_bfloat16 *W, const float *bias, int relu, float *Yf,
               __nv_bfloat16 *Yb, int *err) {
    static_assert(K % 16 == 0 && K <= 256 && N % 16 == 0 && N >= 32 && N <= 256, "tile shape");
    constexpr uint32_t NCOL = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sa = smem;                           // 128 x K bf16
    uint8_t *sb = smem + TC_M * K * 2;            // N x K bf16
    uint64_t *bar = (uint64_t *)(sb + N * K * 2);  // mbarrier
    uint32_t *slot = (uint32_t *)(bar + 1);       // tensor-memory address
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t row0 = (int64_t)blockIdx.x * TC_M;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(NCOL));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    // operands into the core-matrix layout: element (r, k) of a K-major
    // operand lives at ((r / 8) * (K / 8) + k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2
    constexpr int KC = K / 8;
    for (int q = tid; q < TC_M * KC; q += 128) {
        const int r = q / KC, kc = q % KC;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (row0 + r < M) v = *(const uint4 *)(X + (row0 + r) * K + kc * 8);
        *(uint4 *)(sa + ((r >> 3) * KC + kc) * 128 + (r & 7) * 16) = v;
    }
    for (int q = tid; q < N * KC; q += 128) {
        const int r = q / KC, kc = q % KC;
        const uint4 v = *(const uint4 *)(W + (int64_t)r * K + kc * 8);
        *(uint4 *)(sb + ((r >> 3) * KC + kc) * 128 + (r & 7) * 16) = v;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *(volatile uint32_t *)slot;

    if (tid == 0) {
        constexpr uint32_t idesc = tc_idesc(N, TC_M);
        const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
#pragma unroll
        for (int kk = 0; kk < K / 16; kk++) {
            const uint64_t ad = tc_desc(a0 + kk * 256, 128, KC * 128);
            const uint64_t bd = tc_desc(b0 + kk * 256, 128, KC * 128);
            const uint32_t acc = kk > 0 ? 1u : 0u;
            asm volatile(
                "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(bar))
                     : "memory");
    }
    // bounded wait for the MMAs (phase 0 of the barrier)
    uint32_t done = 0;
    for (uint32_t it = 0; it < TC_WAIT_LIMIT && !done; it++) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(0u)
            : "memory");
    }
    done = __any_sync(0xffffffffu, done);  // the phase completed if any lane saw it
    if (!done && lane == 0) atomicExch(err, 1);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (done) {
        const int64_t r = row0 + warp * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c = 0; c < N; c += 8) {
            uint32_t v[8];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                : "r"(lane_addr + (uint32_t)c));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (r < M) {
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    float y = __uint_as_float(v[j]) + bias[c + j];
                    if (relu) y = fmaxf(y, 0.0f);
                    if (Yf) Yf[r * N + c + j] = y;
                    if (Yb) Yb[r * N + c + j] = __float2bfloat16_rn(y);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOL));
}

template <int K, int N>
size_t tc_smem() {
    return (size_t)TC_M * K * 2 + (size_t)N * K * 2 + 16;
}

template <int K, int N>
void dense_tc(cudaStream_t st, const __nv_bfloat16 *X, int M, const __nv_bfloat16 *W, const float *bias, bool relu,
              float *Yf, __nv_bfloat16 *Yb, int *err, Counter &launches) {
    const size_t sm = tc_smem<K, N>();
    CK(allow_dynamic_smem((const void *)k_dense_tc<K, N>));
    k_dense_tc<K, N><<<(unsigned)((M + TC_M - 1) / TC_M), 128, sm, st>>>(X, M, W, bias, relu ? 1 : 0, Yf, Yb, err);
    launches(cudaGetLastError());
}

// standardised features -> bf16 rows
__global__ void k_standardise(const float *F, int B, const float *mu, const float *sd, __nv_bfloat16 *X) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)B * IN) return;
    const int j = (int)(i % IN);
    X[i] = __float2bfloat16_rn((F[i] - mu[j]) / sd[j]);
}

uint16_t bf16_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;  // NaN
    u += 0x7fffu + ((u >> 16) & 1u);                      // round to nearest even
    return (uint16_t)(u >> 16);
}

}  // namespace

// ------------------------------------------------------------------ host
struct TunerModel {
    int device = -1;
    __nv_bfloat16 *w1 = nullptr, *w2 = nullptr, *w3 = nullptr;  // bf16, W3 padded to 32 rows
    float *b1 = nullptr, *b2 = nullptr, *b3 = nullptr;          // b3 padded to 32
    float *mu = nullptr, *sd = nullptr;
};

// Feature-block origins: every 32-cell block on the 32-grid that fits, then
// every ceil(count / 64)-th of them in row-major order.
std::vector<int64_t> feature_origins(const uint64_t *dims) {
    std::vector<int64_t> all;
    for (uint64_t x = 0; x + FEB <= dims[0]; x += FEB - 1)
        for (uint64_t y = 0; y + FEB <= dims[1]; y += FEB - 1)
            for (uint64_t z = 0; z + FEB <= dims[2]; z += FEB - 1) {
                all.push_back((int64_t)x);
                all.push_back((int64_t)y);
                all.push_back((int64_t)z);
            }
    const size_t n = all.size() / 3, step = (n + FAZ_TUNER_MAX_BLOCKS - 1) / FAZ_TUNER_MAX_BLOCKS;
    std::vector<int64_t> o;
    for (size_t i = 0; i < n; i += (step ? step : 1)) o.insert(o.end(), all.begin() + 3 * i, all.begin() + 3 * i + 3);
    return o;
}

template <typename T>
void tuner_features_device(const faz_config &c, const T *dX, cudaStream_t st, float *dF, Counter &launches) {
    if (c.N != 3) throw Fail{FAZ_ERR_UNSUPPORTED, "learned tuner features are defined for 3-D fields"};
    for (int i = 0; i < 3; i++)
        if (c.dims[i] < (uint64_t)FEB) throw Fail{FAZ_ERR_UNSUPPORTED, "learned tuner needs every extent >= 33"};
    if (!(c.absErrorBound > 0)) throw Fail{FAZ_ERR_ARG, "learned tuner needs a resolved positive error bound"};
    const std::vector<int64_t> org = feature_origins(c.dims);
    const int nblk = (int)(org.size() / 3);
    DevMem m(st);
    int64_t *dorg = m.alloc<int64_t>(org.size());
    double *stats = m.alloc<double>((size_t)nblk * NCFG * NST);
    CK(cudaMemcpyAsync(dorg, org.data(), org.size() * 8, cudaMemcpyHostToDevice, st));
    k_feat_block<T><<<dim3(nblk, NCFG), FT, 0, st>>>(dX, (int64_t)c.dims[1], (int64_t)c.dims[2], dorg, c.absErrorBound,
                                                     stats);
    launches(cudaGetLastError());
    const double rel = c.relErrorBound > 0 ? c.relErrorBound : c.absErrorBound / c.rng;
    k_feat_finish<<<1, 128, 0, st>>>(stats, nblk, c.absErrorBound, c.rng, rel, (double)c.dims[0], (double)c.dims[1],
                                     (double)c.dims[2], dF);
    launches(cudaGetLastError());
}
template void tuner_features_device<float>(const faz_config &, const float *, cudaStream_t, float *, Counter &);
template void tuner_features_device<double>(const faz_config &, const double *, cudaStream_t, float *, Counter &);

void mlp_forward(const float *P, const float *X, int B, float *H1, float *H2, float *Z, cudaStream_t st,
                 Counter &launches) {
    gemm(st, B, H, IN, X, IN, 1, P + OFF_W1, 1, IN, H1, H, P + OFF_B1, true);
    launches(cudaGetLastError());
    gemm(st, B, H, H, H1, H, 1, P + OFF_W2, 1, H, H2, H, P + OFF_B2, true);
    launches(cudaGetLastError());
    gemm(st, B, OUT, H, H2, H, 1, P + OFF_W3, 1, H, Z, OUT, P + OFF_B3, false);
    launches(cudaGetLastError());
}

void mlp_backward(const float *P, const float *X, const int32_t *labels, int B, const float *H1, const float *H2,
                  const float *Z, float *G, float *loss, cudaStream_t st, Counter &launches) {
    DevMem m(st);
    float *dZ = m.alloc<float>((size_t)B * OUT), *dH2 = m.alloc<float>((size_t)B * H), *dH1 = m.alloc<float>((size_t)B * H);
    k_heads_loss<<<(B + 127) / 128, 128, 0, st>>>(Z, labels, B, dZ, loss);
    launches(cudaGetLastError());
    // layer 3: dW3[o, h] = sum_b dZ[b, o] H2[b, h]; dH2 = dZ W3
    gemm(st, OUT, H, B, dZ, 1, OUT, H2, H, 1, G + OFF_W3, H, nullptr, false);
    k_colsum<<<1, 32, 0, st>>>(dZ, B, OUT, G + OFF_B3);
    gemm(st, B, H, OUT, dZ, OUT, 1, P + OFF_W3, H, 1, dH2, H, nullptr, false);
    k_relu_mask<<<(unsigned)(((int64_t)B * H + 255) / 256), 256, 0, st>>>(dH2, H2, (int64_t)B * H);
    // layer 2
    gemm(st, H, H, B, dH2, 1, H, H1, H, 1, G + OFF_W2, H, nullptr, false);
    k_colsum<<<(H + 127) / 128, 128, 0, st>>>(dH2, B, H, G + OFF_B2);
    gemm(st, B, H, H, dH2, H, 1, P + OFF_W2, H, 1, dH1, H, nullptr, false);
    k_relu_mask<<<(unsigned)(((int64_t)B * H + 255) / 256), 256, 0, st>>>(dH1, H1, (int64_t)B * H);
    // layer 1
    gemm(st, H, IN, B, dH1, 1, H, X, IN, 1, G + OFF_W1, IN, nullptr, false);
    k_colsum<<<(H + 127) / 128, 128, 0, st>>>(dH1, B, H, G + OFF_B1);
    launches(cudaGetLastError());
    launches.n += 10;
}

void mlp_adam(float *P, const float *G, float *M, float *V, int64_t n, float lr, float b1, float b2, float eps, int t,
              float wd, cudaStream_t st, Counter &launches) {
    const float c1 = 1.0f - std::pow(b1, (float)t), c2 = 1.0f - std::pow(b2, (float)t);
    k_adam<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(P, G, M, V, n, lr, b1, b2, eps, c1, c2, wd);
    launches(cudaGetLastError());
}

TunerModel *tuner_model_create(const float *P, const float *mu, const float *sd) {
    auto *t = new TunerModel;
    try {
        CK(cudaGetDevice(&t->device));
        std::vector<uint16_t> w1((size_t)H * IN), w2((size_t)H * H), w3((size_t)32 * H, 0);
        for (size_t i = 0; i < w1.size(); i++) w1[i] = bf16_bits(P[OFF_W1 + i]);
        for (size_t i = 0; i < w2.size(); i++) w2[i] = bf16_bits(P[OFF_W2 + i]);
        for (size_t i = 0; i < (size_t)OUT * H; i++) w3[i] = bf16_bits(P[OFF_W3 + i]);
        std::vector<float> b3(32, 0.0f);
        std::memcpy(b3.data(), P + OFF_B3, OUT * 4);
        CK(cudaMalloc(&t->w1, w1.size() * 2));
        CK(cudaMalloc(&t->w2, w2.size() * 2));
        CK(cudaMalloc(&t->w3, w3.size() * 2));
        CK(cudaMalloc(&t->b1, H * 4));
        CK(cudaMalloc(&t->b2, H * 4));
        CK(cudaMalloc(&t->b3, 32 * 4));
        CK(cudaMalloc(&t->mu, IN * 4));
        CK(cudaMalloc(&t->sd, IN * 4));
        CK(cudaMemcpy(t->w1, w1.data(), w1.size() * 2, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(t->w2, w2.data(), w2.size() * 2, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(t->w3, w3.data(), w3.size() * 2, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(t->b1, P + OFF_B1, H * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(t->b2, P + OFF_B2, H * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(t->b3, b3.data(), 32 * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(t->mu, mu, IN * 4, cudaMemcpyHostToDevice));
        std::vector<float> s(sd, sd + IN);
        for (float &v : s)
            if (!(v > 0)) v = 1.0f;
        CK(cudaMemcpy(t->sd, s.data(), IN * 4, cudaMemcpyHostToDevice));
    } catch (...) {
        tuner_model_destroy(t);
        throw;
    }
    return t;
}

void tuner_model_destroy(TunerModel *t) {
    if (!t) return;
    cudaFree(t->w1);
    cudaFree(t->w2);
    cudaFree(t->w3);
    cudaFree(t->b1);
    cudaFree(t->b2);
    cudaFree(t->b3);
    cudaFree(t->mu);
    cudaFree(t->sd);
    delete t;
}

// logits of B feature rows through the bf16 tensor-core path
void tuner_infer_device(const TunerModel &t, const float *dF, int B, float *dZ, cudaStream_t st, Counter &launches) {
    int dev = -1;
    CK(cudaGetDevice(&dev));
    if (dev != t.device) throw Fail{FAZ_ERR_ARG, "tuner model belongs to another device"};
    if (B <= 0) throw Fail{FAZ_ERR_ARG, "no feature rows"};
    DevMem m(st);
    __nv_bfloat16 *x = m.alloc<__nv_bfloat16>((size_t)B * IN), *h1 = m.alloc<__nv_bfloat16>((size_t)B * H),
                  *h2 = m.alloc<__nv_bfloat16>((size_t)B * H);
    float *z = m.alloc<float>((size_t)B * 32);
    int *err = m.alloc<int>(1);
    CK(cudaMemsetAsync(err, 0, 4, st));
    k_standardise<<<(unsigned)(((int64_t)B * IN + 255) / 256), 256, 0, st>>>(dF, B, t.mu, t.sd, x);
    launches(cudaGetLastError());
    dense_tc<IN, H>(st, x, B, t.w1, t.b1, true, nullptr, h1, err, launches);
    dense_tc<H, H>(st, h1, B, t.w2, t.b2, true, nullptr, h2, err, launches);
    dense_tc<H, 32>(st, h2, B, t.w3, t.b3, false, z, nullptr, err, launches);
    CK(cudaMemcpy2DAsync(dZ, OUT * 4, z, 32 * 4, OUT * 4, B, cudaMemcpyDeviceToDevice, st));
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (herr) throw Fail{FAZ_ERR_DEVICE, "tensor-core MMA did not complete in time"};
}

}  // namespace faz

namespace faz {

namespace {
const double kAlpha[5] = {1, 1.25, 1.5, 1.75, 2};
const double kBeta[4] = {1.5, 2, 3, 4};

void softmax(const float *z, int n, double *p) {
    double mx = z[0];
    for (int i = 1; i < n; i++) mx = std::max<double>(mx, z[i]);
    double s = 0;
    for (int i = 0; i < n; i++) s += (p[i] = std::exp((double)z[i] - mx));
    for (int i = 0; i < n; i++) p[i] /= s;
}
}  // namespace

// The learned replacement of the QoZ tuner (see the C header).
template <typename T>
void learned_tune_device(faz_config &c, const T *dX, cudaStream_t st, const TunerModel &model, double min_conf,
                         faz_tuner_choice &ch, Counter &launches, faz_timings &tm) {
    std::memset(&ch, 0, sizeof(ch));
    const faz_config plain = c;
    auto use_plain = [&](int why) {
        c = plain;
        qoz_tune_device<T>(c, dX, st, launches, tm);
        ch.used_plain = why;
    };
    if (!(c.cmprAlgo == FAZ_ALGO_INTERP_LORENZO && c.QoZ) || c.N != 3 || c.tuningTarget != 0) {
        if (c.cmprAlgo == FAZ_ALGO_INTERP_LORENZO && c.QoZ) use_plain(3);
        else throw Fail{FAZ_ERR_UNSUPPORTED, "the learned tuner replaces the QoZ tuner (QoZ = 1, ALGO_INTERP_LORENZO)"};
        return;
    }
    for (int i = 0; i < 3; i++)
        if (c.dims[i] < (uint64_t)FEB) return use_plain(3);
    qoz_prepare<T>(c, dX, st, launches);
    const int Lsel = c.levelwisePredictionSelection;
    // the network predicts the RD-target decisions of the default sampling
    if (Lsel < 1 || Lsel > 4 || !(c.autoTuningRate > 0) || c.tuningTarget != 0 || c.profiling || c.var_first)
        return use_plain(3);
    DevMem m(st);
    float *dF = m.alloc<float>(IN), *dZ = m.alloc<float>(OUT);
    tuner_features_device<T>(c, dX, st, dF, launches);
    tuner_infer_device(model, dF, 1, dZ, st, launches);
    CK(cudaMemcpyAsync(ch.logits, dZ, OUT * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const float *z = ch.logits;
    double conf = 1.0, p[5];
    uint8_t il[4], dl[4];
    for (int l = 0; l < Lsel; l++) {
        softmax(z + 4 * l, 4, p);
        const int k = (int)(std::max_element(p, p + 4) - p);
        conf = std::min(conf, p[k]);
        il[l] = (uint8_t)(k >> 1);
        dl[l] = (uint8_t)((k & 1) ? 5 : 0);
    }
    double pa[5], pb[4], pl[2];
    softmax(z + 16, 5, pa);
    softmax(z + 21, 4, pb);
    softmax(z + 25, 2, pl);
    // best alpha/beta pair among those the search visits (alpha <= beta)
    int ba = 0, bb = 0;
    double best = -1;
    for (int a = 0; a < 5; a++)
        for (int b = 0; b < 4; b++)
            if (kAlpha[a] <= kBeta[b] && pa[a] * pb[b] > best) {
                best = pa[a] * pb[b];
                ba = a;
                bb = b;
            }
    conf = std::min(conf, std::min(pa[ba], pb[bb]));
    ch.confidence = (float)conf;
    ch.p_lorenzo = (float)pl[1];
    if (pl[1] > 0.5) return use_plain(2);
    if (conf < min_conf) return use_plain(1);
    // the decisions the QoZ tuner leaves in the configuration
    c.interp_list_len = Lsel;
    for (int l = 0; l < Lsel; l++) {
        c.interpAlgo_list[l] = il[l];
        c.interpDirection_list[l] = dl[l];
    }
    c.interpAlgo = FAZ_INTERP_ALGO_CUBIC;
    c.interpDirection = 5;
    c.alpha = kAlpha[ba];
    c.beta = kBeta[bb];
    c.wavelet_rel_coeff = 1;
    c.wavelet = 0;
    c.cmprAlgo = FAZ_ALGO_INTERP;
}
template void learned_tune_device<float>(faz_config &, const float *, cudaStream_t, const TunerModel &, double,
                                         faz_tuner_choice &, Counter &, faz_timings &);
template void learned_tune_device<double>(faz_config &, const double *, cudaStream_t, const TunerModel &, double,
                                          faz_tuner_choice &, Counter &, faz_timings &);

}  // namespace faz
