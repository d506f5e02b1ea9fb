// tuner.cu - the SZ3 tuner of the default configuration (ALGO_INTERP_LORENZO)
// on the GPU: sampling, the Lorenzo trial, the block-interpolation trials and
// the quantisation-interval estimate, with the decision logic on the host.
//
// Reference: SZ_compress_Interp_lorenzo (include/QoZ/api/impl/SZInterp.hpp
// 2561-2880) with the SZ3 branch of Tuning (2115-2187), sampling<T,N>
// (include/QoZ/utils/Extraction.hpp:11-232), do_not_use_this_interp_compress_block_test
// (SZInterp.hpp:558-577) over SZBlockInterpolationCompressor::compress
// (include/QoZ/compressor/deprecated/SZBlockInterpolationCompressor.hpp:127-280)
// and optimize_quant_invl_3d (include/QoZ/utils/QuantOptimization.hpp:88-148).
// Every trial is a whole compression of the sample whose compressed size
// (zstd framing included) decides, so the trials run the same GPU stages as
// the real compressors and hand their payloads to the host zstd.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <future>
#include <string>
#include <vector>

#include "common.cuh"
#include "host.h"
#include "internal.h"
#include "quant.cuh"

namespace faz {

namespace {

struct Dims3 {
    int64_t v[3];
};

// sampling<T,N>: corner blocks of every dmin-cube, gathered (one thread per
// sample point).  Dims are embedded as 3-D with leading 1s.
template <typename T>
__global__ void k_sample(const T *__restrict__ X, Dims3 gd, Dims3 sd, int64_t sb, int64_t dmin, int e,
                         T *__restrict__ out, uint64_t sn) {
    const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= sn) return;
    int64_t c[3], g[3];
    c[2] = (int64_t)(idx % (uint64_t)sd.v[2]);
    c[1] = (int64_t)((idx / (uint64_t)sd.v[2]) % (uint64_t)sd.v[1]);
    c[0] = (int64_t)(idx / ((uint64_t)sd.v[2] * (uint64_t)sd.v[1]));
    for (int a = 0; a < 3; a++) {
        if (a < e) {
            g[a] = 0;
            continue;
        }
        const int64_t b = c[a] / (2 * sb), i = c[a] % (2 * sb);
        const int64_t di = i < sb ? i + sb : dmin - 3 * sb + i;
        g[a] = b * dmin + di;
    }
    out[idx] = X[(g[0] * gd.v[1] + g[1]) * gd.v[2] + g[2]];
}

// ------------------------------------------------ block interpolation trial
struct BiSweep {
    int64_t nb[3];        // blocks per dim (3-D embedding)
    int64_t bs;           // block edge (all blocks full)
    int64_t block_codes;  // codes per block
    int64_t dims[3], offs[3];
    int axis;             // sweep axis (3-D index)
    int oth[2];           // other axes, increasing
    int64_t g[2], cnt[2]; // their grid steps and point counts
    int64_t s;            // stride along the axis
    int64_t n, tpl;       // points per line, targets per line
    int64_t seg_off;      // first code of this (level, sweep) inside a block
    int cubic;
};

// block_interpolation_1d targets (SZBlockInterpolationCompressor.hpp:204-280):
// odd indices in increasing order, one thread each.  The four
// block-interpolation trials (linear / cubic, two directions) run in the same
// launches: blockIdx.y picks the trial, each with its own copy of the sample,
// codes and sweep geometry.
constexpr int kBiTrials = 4;
template <typename T>
struct BiTrials {
    BiSweep w[kBiTrials];
    T *data[kBiTrials];
    uint16_t *codes[kBiTrials];
    T *scratch[kBiTrials];
};

template <typename T, int QM>
__global__ void k_bi_sweep4(BiTrials<T> b, LevelArgs q, uint64_t total) {
    const int v = blockIdx.y;
    const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const BiSweep &w = b.w[v];
    const uint64_t lines = (uint64_t)(w.cnt[0] * w.cnt[1]);
    const int64_t r = (int64_t)(idx % (uint64_t)w.tpl);
    const uint64_t L = (idx / (uint64_t)w.tpl) % lines;
    const uint64_t t = idx / ((uint64_t)w.tpl * lines);
    int64_t bc[3];
    bc[2] = (int64_t)(t % (uint64_t)w.nb[2]);
    bc[1] = (int64_t)((t / (uint64_t)w.nb[2]) % (uint64_t)w.nb[1]);
    bc[0] = (int64_t)(t / ((uint64_t)w.nb[2] * (uint64_t)w.nb[1]));
    // coordinates as scalars (an array indexed by the sweep's axes would live
    // in local memory)
    int64_t c0 = bc[0] * w.bs, c1 = bc[1] * w.bs, c2 = bc[2] * w.bs;
    auto add = [&](int ax, int64_t v) {
        c0 += ax == 0 ? v : 0;
        c1 += ax == 1 ? v : 0;
        c2 += ax == 2 ? v : 0;
    };
    const int64_t u1 = (int64_t)(L % (uint64_t)w.cnt[1]), u0 = (int64_t)(L / (uint64_t)w.cnt[1]);
    add(w.oth[0], u0 * w.g[0]);
    add(w.oth[1], u1 * w.g[1]);
    const int64_t i = 2 * r + 1;
    add(w.axis, i * w.s);
    const int64_t pos = c0 * w.offs[0] + c1 * w.offs[1] + c2 * w.offs[2];
    const int64_t st = w.s * (w.axis == 0 ? w.offs[0] : (w.axis == 1 ? w.offs[1] : w.offs[2]));
    T *d = b.data[v] + pos;
    const int64_t n = w.n;
    T pred;
    if (!w.cubic || n < 5) {
        if (i + 1 < n) pred = i_linear(d[-st], d[st]);
        else if (n < 4) pred = d[-st];
        else pred = linear1_any<T>(d[-3 * st], d[-st]);
    } else {
        if (i == 1) pred = i_quad1(d[-st], d[st], d[3 * st]);
        else if (i + 3 < n) pred = i_cubic(d[-3 * st], d[-st], d[st], d[3 * st]);
        else if ((n & 1) == 0 && i == n - 1) pred = i_quad3(d[-5 * st], d[-3 * st], d[-st]);
        else pred = i_quad2(d[-3 * st], d[-st], d[st]);
    }
    T val = *d, uval;
    const int code = quant_point<T, QM>(val, pred, q, uval);
    const uint64_t cp = t * (uint64_t)w.block_codes + (uint64_t)w.seg_off + L * (uint64_t)w.tpl + (uint64_t)r;
    b.codes[v][cp] = (uint16_t)code;
    if (code == 0) b.scratch[v][cp] = uval;
    *d = val;
}

// Each block's corner against prediction 0.
template <typename T>
__global__ void k_bi_corner4(BiTrials<T> b, LevelArgs q, uint64_t nblocks) {
    const int v = blockIdx.y;
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nblocks) return;
    const BiSweep &w = b.w[v];
    const int64_t b2 = (int64_t)(t % (uint64_t)w.nb[2]);
    const int64_t b1 = (int64_t)((t / (uint64_t)w.nb[2]) % (uint64_t)w.nb[1]);
    const int64_t b0 = (int64_t)(t / ((uint64_t)w.nb[2] * (uint64_t)w.nb[1]));
    const int64_t pos = (b0 * w.offs[0] + b1 * w.offs[1] + b2 * w.offs[2]) * w.bs;
    T val = b.data[v][pos], uval;
    const int code = quantize<T>(val, (T)0, q.eb, q.recip, q.radius, 0, uval);
    b.codes[v][t * (uint64_t)w.block_codes] = (uint16_t)code;
    if (code == 0) b.scratch[v][t * (uint64_t)w.block_codes] = uval;
    b.data[v][pos] = val;
}

// optimize_quant_invl_3d: histogram of sampled Lorenzo prediction errors.
// Samples come as runs (first position, count) with stride 100.
template <typename T>
__global__ void k_quant_hist(const T *__restrict__ X, int64_t r23, int64_t r3, const uint64_t *__restrict__ seg_pos,
                             const uint32_t *__restrict__ seg_cnt, uint64_t nseg, double precision,
                             unsigned long long *__restrict__ hist) {
    const uint64_t sgi = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (sgi >= nseg) return;
    const uint64_t p0 = seg_pos[sgi];
    const uint32_t c = seg_cnt[sgi];
    for (uint32_t m = 0; m < c; m++) {
        const T *p = X + p0 + (uint64_t)m * 100;
        const T pv = p[-1] + p[-r3] + p[-r23] - p[-r3 - 1] - p[-r23 - 1] - p[-r23 - r3] + p[-r23 - r3 - 1];
        const T diff = pv - *p;
        const float pe = (float)(diff < 0 ? -diff : diff);
        uint64_t pi = (uint64_t)(((double)pe / precision + 1) / 2);
        if (pi >= 32768) pi = 32767;
        atomicAdd(&hist[pi], 1ull);
    }
}

size_t zstd_framed_size(const uint8_t *p, size_t n) {
    std::string err;
    const Zstd &z = zstd_lib(err);
    if (!z.ok) throw Fail{FAZ_ERR_ZSTD, err};
    size_t zs = zstd_level3_size(z, p, n);
    if (z.isError(zs)) throw Fail{FAZ_ERR_ZSTD, "ZSTD_compress failed"};
    return zs + 8;
}

// do_not_use_this_interp_compress_block_test (SZInterp.hpp:558-577):
// SZBlockInterpolationCompressor::compress on the sample (blocks of edge bs,
// which tile the sample exactly), for the four trials at once.  Each trial's
// codes (stream order) and unpredictable values (at their code positions)
// are left in its arrays.
struct BiTrialSpec {
    int cubic, dir;
};

// Buffers come from `m` (ordered on its stream); the work runs on `st`.
template <typename T>
void block_interp_sweeps(int N, const uint64_t *sdims, const T *dS, double eb, const BiTrialSpec *spec, int64_t bs,
                         DevMem &m, cudaStream_t st, Counter &launches, BiTrials<T> &b) {
    uint64_t num = 1;
    for (int i = 0; i < N; i++) {
        num *= sdims[i];
        if (sdims[i] % (uint64_t)bs) throw Fail{FAZ_ERR_UNSUPPORTED, "sample does not tile into sampling blocks"};
    }
    LevelArgs q;
    std::memset(&q, 0, sizeof(q));
    q.eb = eb;
    q.recip = 1.0 / eb;
    q.radius = 32768;
    q.trim = 0;
    set_fast_path<T>(q);
    const bool straight = sizeof(T) == 4 && q.fast;
    const int e = 3 - N;
    int perm[kBiTrials][3];
    for (int v = 0; v < kBiTrials; v++) {
        b.data[v] = m.alloc<T>(num);
        b.codes[v] = m.alloc<uint16_t>(num);
        b.scratch[v] = m.alloc<T>(num);
    }
    {
        Events ev;
        CK(cudaEventRecord(ev.a, m.st));
        CK(cudaStreamWaitEvent(st, ev.a, 0));
    }
    for (int v = 0; v < kBiTrials; v++) {
        CK(cudaMemcpyAsync(b.data[v], dS, num * sizeof(T), cudaMemcpyDeviceToDevice, st));
        BiSweep &w = b.w[v];
        std::memset(&w, 0, sizeof(w));
        for (int i = 0; i < 3; i++) {
            w.dims[i] = 1;
            w.nb[i] = 1;
        }
        for (int i = 0; i < N; i++) {
            w.dims[e + i] = (int64_t)sdims[i];
            w.nb[e + i] = (int64_t)sdims[i] / bs;
        }
        w.offs[2] = 1;
        w.offs[1] = w.dims[2];
        w.offs[0] = w.dims[1] * w.dims[2];
        w.bs = bs;
        int64_t bc = 1;
        for (int i = 0; i < N; i++) bc *= bs;
        w.block_codes = bc;
        w.cubic = spec[v].cubic;
        const int dir = spec[v].dir;
        perm[v][0] = 0;
        perm[v][1] = 1;
        perm[v][2] = 2;
        if (N == 2 && dir != 0) {
            perm[v][0] = 1;
            perm[v][1] = 0;
        }
        if (N == 3) {
            static const int P3[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
            if (dir < 0 || dir > 5) throw Fail{FAZ_ERR_ARG, "interpolation direction out of range"};
            for (int i = 0; i < 3; i++) perm[v][i] = P3[dir][i];
        }
    }
    const uint64_t nblocks = (uint64_t)(b.w[0].nb[0] * b.w[0].nb[1] * b.w[0].nb[2]);
    k_bi_corner4<T><<<dim3((unsigned)((nblocks + 255) / 256), kBiTrials), 256, 0, st>>>(b, q, nblocks);
    launches(cudaGetLastError());
    int maxl = 0;
    while (((int64_t)1 << maxl) < bs) maxl++;
    if (maxl < 1) maxl = 1;
    int64_t off = 1;  // the corner
    for (int level = maxl; level > 0; level--) {
        const int64_t s_ = (int64_t)1 << (level - 1);
        bool swept[kBiTrials][3] = {};
        for (int sw = 0; sw < N; sw++) {
            uint64_t total = 0, per_block = 0;
            for (int v = 0; v < kBiTrials; v++) {
                BiSweep &w = b.w[v];
                const int a = e + perm[v][sw];
                w.axis = a;
                int no = 0;
                for (int i = 0; i < 3; i++)
                    if (i != a) w.oth[no++] = i;
                for (int u = 0; u < 2; u++) {
                    const int ax = w.oth[u];
                    if (ax < e) {
                        w.g[u] = 1;
                        w.cnt[u] = 1;
                    } else {
                        w.g[u] = swept[v][ax] ? s_ : 2 * s_;
                        w.cnt[u] = (bs - 1) / w.g[u] + 1;
                    }
                }
                w.s = s_;
                w.n = (bs - 1) / s_ + 1;
                w.tpl = w.n / 2;
                w.seg_off = off;
                const uint64_t pb = (uint64_t)(w.cnt[0] * w.cnt[1] * w.tpl);
                // blocks are cubes, so every trial's sweep has the same size
                if (v > 0 && pb != per_block) throw Fail{FAZ_ERR_DEVICE, "trial sweeps differ in size"};
                per_block = pb;
                total = pb * nblocks;
                swept[v][a] = true;
            }
            if (total) {
                const dim3 grid((unsigned)((total + 255) / 256), kBiTrials);
                if (straight) k_bi_sweep4<T, 1><<<grid, 256, 0, st>>>(b, q, total);
                else k_bi_sweep4<T, 0><<<grid, 256, 0, st>>>(b, q, total);
                launches(cudaGetLastError());
            }
            off += (int64_t)per_block;
        }
    }
    if (off != b.w[0].block_codes) throw Fail{FAZ_ERR_DEVICE, "block interpolation did not cover its blocks"};
}

// The Huffman stage and payload of one block-interpolation trial; `report`
// gets the payload's size as soon as the codebook is built.
template <typename T>
void block_interp_tail(int N, const uint64_t *sdims, double eb, int cubic, int dir, int64_t bs, uint16_t *codes,
                       T *scratch, cudaStream_t st, Counter &launches, faz_timings &tm, std::vector<uint8_t> &pl,
                       const std::function<void(size_t)> &report = {}) {
    uint64_t num = 1;
    for (int i = 0; i < N; i++) num *= sdims[i];
    DevMem m(st);
    HuffEncoded hc;
    auto sized = [&](const HuffEncoded &e) {
        if (!report) return;
        const size_t head = (size_t)N * 8 + 4 + 4 + 4 + 1 + 8 + 4 + 8;
        const size_t tree = 4 + 4 + 4 + e.cb.tree.size() + 8;
        report(head + e.nzero * sizeof(T) + tree + e.nbytes);
    };
    huffman_encode_device(codes, num, 32768, m, st, launches, hc, tm, sized);
    trace_step("trial encode queued");
    const uint64_t nunpred = hc.nzero;
    T *unp = m.alloc<T>(nunpred ? nunpred : 1);
    if (nunpred) launches(launch_compact_zeros<T>(codes, num, hc.zc, hc.zoff, nullptr, scratch, unp, st));
    std::vector<uint8_t> h;
    for (int i = 0; i < N; i++) put<uint64_t>(h, sdims[i]);
    put<uint32_t>(h, (uint32_t)bs);
    put<int32_t>(h, cubic);
    put<int32_t>(h, dir);
    put<uint8_t>(h, 2);
    put<double>(h, eb);
    put<int32_t>(h, 32768);
    put<uint64_t>(h, nunpred);
    std::vector<uint8_t> h2;
    append_tree(h2, hc.cb, hc.nbytes);
    // device parts come back through the thread's pinned staging buffer
    // (copies to pageable memory serialise with the other trials' copies)
    const size_t total = h.size() + nunpred * sizeof(T) + h2.size() + hc.nbytes;
    uint8_t *pin = t_pin_payload.get(total + 8);
    std::memcpy(pin, h.data(), h.size());
    if (nunpred) CK(cudaMemcpyAsync(pin + h.size(), unp, nunpred * sizeof(T), cudaMemcpyDeviceToHost, st));
    std::memcpy(pin + h.size() + nunpred * sizeof(T), h2.data(), h2.size());
    if (hc.nbytes)
        CK(cudaMemcpyAsync(pin + h.size() + nunpred * sizeof(T) + h2.size(), hc.bits, hc.nbytes,
                           cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    emit_payload(pl, pin, total);
}

// One trial on its own host thread and CUDA stream: the trials are
// independent compressions of the same sample, so they overlap on the GPU and
// each thread computes its zstd size as soon as its payload is ready.
// FAZ_TUNE_TRACE=1 prints the tuner's timeline (trial payloads, zstd sizes,
// the overlapped compression) to stderr.

struct Trial {
    const char *name = "";
    clk::time_point t0;
    std::future<size_t> size;
    std::promise<size_t> raw;  // pre-zstd payload size, known before the zstd size
    std::future<size_t> raw_f = raw.get_future();
    uint64_t launches = 0;
    double host_ms = 0;
    template <typename F>
    void start(cudaEvent_t ready, F body) {
        size = TaskThreads::get().submit<size_t>([this, ready, body]() -> size_t {
            // the payload buffer stays with the (persistent) thread, so that
            // a few MB are not allocated and faulted in again for each trial
            thread_local std::vector<uint8_t> pl;
            pl.clear();
            // the payload stays in the thread's pinned staging buffer
            PayloadView view;
            struct ViewScope {
                explicit ViewScope(PayloadView *v) { t_payload_view = v; }
                ~ViewScope() { t_payload_view = nullptr; }
            } scope(&view);
            bool reported = false;
            size_t early = 0;
            auto report = [&](size_t n) {
                if (reported) return;
                reported = true;
                early = n;
                raw.set_value(n);
                if (tune_trace()) std::fprintf(stderr, "tune %8.3f ms  %s size %zu bytes\n", ms_since(t0), name, n);
            };
            try {
                // the trials gate the tuner's decision: they take SMs ahead of
                // the overlapped compression
                if (tune_trace()) std::fprintf(stderr, "tune %8.3f ms  %s starts\n", ms_since(t0), name);
                StreamGuard sg(nullptr, true);
                CK(cudaStreamWaitEvent(sg.st, ready, 0));
                Counter c;
                faz_timings t;
                std::memset(&t, 0, sizeof(t));
                body(sg.st, c, t, pl, std::function<void(size_t)>(report));
                launches = c.n;
                host_ms = t.host_ms;
            } catch (...) {
                if (!reported) raw.set_exception(std::current_exception());
                throw;
            }
            const uint8_t *pd = view.data ? view.data : pl.data();
            const size_t pn = view.data ? view.size : pl.size();
            if (reported && early != pn) throw Fail{FAZ_ERR_DEVICE, "a trial's reported size differs from its payload"};
            report(pn);
            if (tune_trace()) std::fprintf(stderr, "tune %8.3f ms  %s payload %zu bytes\n", ms_since(t0), name, pn);
            const size_t z = zstd_framed_size(pd, pn);
            if (tune_trace()) std::fprintf(stderr, "tune %8.3f ms  %s zstd %zu bytes\n", ms_since(t0), name, z);
            return z;
        });
    }
    size_t get() { return size.get(); }
    // a trial still running holds references to this object and the caller's
    // buffers: wait for it (as a std::async future would)
    ~Trial() {
        if (size.valid()) size.wait();
    }
};

template <typename T>
void lorenzo_payload(const uint64_t *sdims, const T *dS, int bs, int pd, double eb, int radius, cudaStream_t st,
                     Counter &launches, faz_timings &tm, std::vector<uint8_t> &pl) {
    faz_timings t2;
    std::memset(&t2, 0, sizeof(t2));
    lorenzo3_compress_payload<T>(sdims, bs, pd, 1, 1, 0, eb, radius, dS, st, launches, t2, pl);
    tm.host_ms += t2.host_ms;
}

// optimize_quant_invl_3d: the sample walk (QuantOptimization.hpp:97-139) on
// the host as runs of stride-100 positions, the error histogram on the GPU,
// estimate_quantization_intervals (lines 26-39) on the host.
template <typename T>
int quant_intervals(const T *dX, const uint64_t *dims, double precision, cudaStream_t st, Counter &launches) {
    const uint64_t r1 = dims[0], r2 = dims[1], r3 = dims[2];
    const uint64_t sd = 100, r23 = r2 * r3, len = r1 * r23;
    std::vector<uint64_t> spos;
    std::vector<uint32_t> scnt;
    uint64_t oc = sd - 2, pos = r23 + r3 + oc, n1 = 1, n2 = 1, sample_count = 0;
    while (pos < len) {
        if (pos < r23 + r3 + 1) throw Fail{FAZ_ERR_UNSUPPORTED, "field too small for the quantisation-interval estimate"};
        // positions pos, pos + sd, ... while the column offset stays inside the row
        uint64_t k = 1;
        if (oc < r3) k = (r3 - oc + sd - 1) / sd;
        const uint64_t kmax = (len - pos + sd - 1) / sd;
        const uint64_t take = k < kmax ? k : kmax;
        spos.push_back(pos);
        scnt.push_back((uint32_t)take);
        sample_count += take;
        if (take < k) break;
        pos += (k - 1) * sd;
        oc += (k - 1) * sd;
        oc += sd;
        n2++;
        if (n2 == r2) {
            n1++;
            n2 = 1;
            pos += r3;
        }
        const uint64_t oc2 = (n1 + n2) % sd;
        pos += (r3 + sd - oc) + (sd - oc2);
        oc = sd - oc2;
        if (oc == 0) oc++;
    }
    DevMem m(st);
    const uint64_t nseg = spos.size();
    unsigned long long *hist = m.alloc<unsigned long long>(32768);
    CK(cudaMemsetAsync(hist, 0, 32768 * 8, st));
    if (nseg) {
        uint64_t *dpos = m.alloc<uint64_t>(nseg);
        uint32_t *dcnt = m.alloc<uint32_t>(nseg);
        CK(cudaMemcpyAsync(dpos, spos.data(), nseg * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(dcnt, scnt.data(), nseg * 4, cudaMemcpyHostToDevice, st));
        k_quant_hist<T><<<(unsigned)((nseg + 255) / 256), 256, 0, st>>>(dX, (int64_t)r23, (int64_t)r3, dpos, dcnt,
                                                                       nseg, precision, hist);
        launches(cudaGetLastError());
    }
    std::vector<unsigned long long> h(32768);
    CK(cudaMemcpyAsync(h.data(), hist, 32768 * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const uint64_t target = (uint64_t)(sample_count * 0.999);
    uint64_t sum = 0, i;
    for (i = 0; i < 32768; i++) {
        sum += h[i];
        if (sum > target) break;
    }
    if (i == 32768) i = 32767;
    unsigned acc = (unsigned)(2 * (i + 1));
    unsigned b = acc - 1;
    b |= b >> 1;
    b |= b >> 2;
    b |= b >> 4;
    b |= b >> 8;
    b |= b >> 16;
    const unsigned ni = 2 * (b + 1);
    return ni > 32 ? (int)ni : 32;
}

float cal_sampling_ratio(uint64_t block, uint64_t n, uint64_t dmin, int N, const uint64_t *dims) {
    uint64_t sample_n = 1;
    for (int i = 0; i < N; i++) sample_n *= dims[i] / dmin * 2 * block;
    return (float)(sample_n * 1.0 / n);
}

void set_dims_defaults(faz_config &c) {
    c.blockSize = c.N == 1 ? 128 : (c.N == 2 ? 16 : 6);
    c.pred_dim = c.N;
    c.stride = c.blockSize;
}

}  // namespace

// SZ_compress_Interp_lorenzo's tuning for the default configuration (no QoZ
// or rate-driven tuning): on return c.cmprAlgo is ALGO_INTERP or
// ALGO_LORENZO_REG and the chosen settings are in c.
size_t zstd_framed_size_host(const uint8_t *p, size_t n) { return zstd_framed_size(p, n); }

// Sampled field of sampling<T,N> (include/QoZ/utils/Extraction.hpp:89-143):
// corner blocks of edge 2 * sb of every dmin-cube, dims sdims[0..N).
template <typename T>
struct Sample {
    uint64_t sb = 0, sn = 0;
    uint64_t sdims[3] = {1, 1, 1};
    T *dS = nullptr;
};

// false when the field is too small to sample (sampling_num == num)
template <typename T>
bool take_sample(const faz_config &c, const T *dX, DevMem &m, cudaStream_t st, Counter &launches, Sample<T> &s) {
    const int N = c.N;
    uint64_t dims[4], dmin = c.dims[0];
    for (int i = 0; i < N; i++) {
        dims[i] = c.dims[i];
        dmin = std::min<uint64_t>(dmin, dims[i]);
    }
    uint64_t sb = dmin;
    while (cal_sampling_ratio(sb, c.num, dmin, N, dims) > 0.035) sb--;
    if (sb * 2 > dmin) sb = dmin / 2;
    if (sb < 9) return false;
    if (N > 3) throw Fail{FAZ_ERR_UNSUPPORTED, "tuning a sampled 4-D field is not implemented on the GPU path"};
    // sample dims (N of them), embedded as 3-D with leading 1s for the gather
    Dims3 gd{}, sdd{};
    const int e = 3 - N;
    for (int i = 0; i < 3; i++) {
        gd.v[i] = 1;
        sdd.v[i] = 1;
    }
    uint64_t sn = 1;
    for (int i = 0; i < N; i++) {
        s.sdims[i] = dims[i] / dmin * 2 * sb;
        gd.v[e + i] = (int64_t)dims[i];
        sdd.v[e + i] = (int64_t)s.sdims[i];
        sn *= s.sdims[i];
    }
    s.sb = sb;
    s.sn = sn;
    s.dS = m.alloc<T>(sn);
    k_sample<T><<<(unsigned)((sn + 255) / 256), 256, 0, st>>>(dX, gd, sdd, (int64_t)sb, (int64_t)dmin, e, s.dS, sn);
    launches(cudaGetLastError());
    return true;
}

// Lorenzo follow-up of both tuners (SZInterp.hpp:2779-2837 and 2797-2845):
// the Lorenzo settings, the quantisation-interval estimate and the pred_dim
// and 16384-bin trials on the sample, from the Lorenzo ratio best_l.
template <typename T>
void lorenzo_followup(faz_config &c, const T *dX, const Sample<T> &smp, double best_l, cudaStream_t st,
                      Counter &launches, faz_timings &tm) {
    const int N = c.N;
    uint64_t dims[4];
    for (int i = 0; i < N; i++) dims[i] = c.dims[i];
    const uint64_t *sdims = smp.sdims;
    const T *dS = smp.dS;
    const double eb = c.absErrorBound;
    const double sbytes = smp.sn * 1.0 * sizeof(T);
    double r;
    faz_config lc = c;
    lc.cmprAlgo = FAZ_ALGO_LORENZO_REG;
    lc.lorenzo = 1;
    lc.lorenzo2 = 1;
    lc.regression = 0;
    lc.regression2 = 0;
    lc.openmp = 0;
    lc.blockSize = 5;
    set_dims_defaults(lc);  // setDims(sample dims)
    if (N == 3) {
        lc.quantbinCnt = quant_intervals<T>(dX, dims, eb, st, launches);  // up to 131072
        lc.pred_dim = 2;
        {
            std::vector<uint8_t> pl;
            lorenzo_payload<T>(sdims, dS, lc.blockSize, lc.pred_dim, eb, lc.quantbinCnt / 2, st, launches, tm, pl);
            r = sbytes / zstd_framed_size(pl.data(), pl.size());
        }
        if (r > best_l * 1.02) best_l = r;
        else lc.pred_dim = 3;
    }
    if (c.relErrorBound < 1.01e-6 && best_l > 5 && lc.quantbinCnt != 16384) {
        const int q0 = lc.quantbinCnt;
        lc.quantbinCnt = 16384;
        std::vector<uint8_t> pl;
        if (N == 3)
            lorenzo_payload<T>(sdims, dS, lc.blockSize, lc.pred_dim, eb, lc.quantbinCnt / 2, st, launches, tm, pl);
        else
            gen_compress_payload<T>(N, sdims, lc.blockSize, 1, 1, 0, eb, lc.quantbinCnt / 2, dS, st, launches, tm, pl);
        r = sbytes / zstd_framed_size(pl.data(), pl.size());
        if (r > best_l * 1.02) best_l = r;
        else lc.quantbinCnt = q0;
    }
    set_dims_defaults(lc);  // setDims(full dims)
    c = lc;
}

template <typename T>
void sz3_tune_device(faz_config &c, const T *dX, cudaStream_t st, Counter &launches, faz_timings &tm,
                     const std::function<void(const faz_config &, const faz_config *)> &speculate) {
    const int N = c.N;
    if (c.QoZ || c.autoTuningRate > 0 || c.predictorTuningRate > 0)
        throw Fail{FAZ_ERR_UNSUPPORTED, "QoZ / rate-driven tuning is not implemented on the GPU path"};
    if (c.preTrim > 0) throw Fail{FAZ_ERR_UNSUPPORTED, "preTrim is not implemented on the GPU path"};
    if (c.wavelet > 0) throw Fail{FAZ_ERR_UNSUPPORTED, "wavelet modes are not part of the interpolation path"};
    if (c.rng < 0) c.rng = device_range<T>(dX, c.num, st, launches);
    if (c.relErrorBound <= 0) c.relErrorBound = c.absErrorBound / c.rng;
    uint64_t dims[4];
    for (int i = 0; i < N; i++) dims[i] = c.dims[i];
    DevMem m(st);
    Sample<T> smp;
    if (!take_sample<T>(c, dX, m, st, launches, smp)) {
        c.cmprAlgo = FAZ_ALGO_INTERP;
        return;
    }
    const uint64_t sb = smp.sb, sn = smp.sn;
    const uint64_t *sdims = smp.sdims;
    const T *dS = smp.dS;
    const double eb = c.absErrorBound;
    const double sbytes = sn * 1.0 * sizeof(T);
    // Tuning, SZ3 branch: the Lorenzo trial (blockSize 5), linear and cubic
    // block-interpolation trials in the configured direction, and the
    // direction-5 trial of whichever wins, computed for both so that every
    // zstd size runs on its own host thread while the GPU moves on.
    const int dop = N == 3 ? 5 : (N == 2 ? 1 : 0);  // factorial(N) - 1
    Events ready;
    CK(cudaEventRecord(ready.a, st));
    Trial jl, ji[2], jd[2];
    const auto tt0 = clk::now();
    if (tune_trace()) trace_epoch() = tt0;
    jl.name = "lorenzo";
    ji[0].name = "linear";
    ji[1].name = "cubic";
    jd[0].name = "linear-dir5";
    jd[1].name = "cubic-dir5";
    for (Trial *t : {&jl, &ji[0], &ji[1], &jd[0], &jd[1]}) t->t0 = tt0;
    // The Lorenzo trial is a long, latency-bound wavefront launch (one warp
    // per block of the sample, few warps per SM): it starts first and runs
    // beside the interpolation trials and the overlapped compression (on the
    // 512^3 benchmark field the tuner then takes 4.6 ms instead of 5.0 ms
    // with the Lorenzo trial started after the interpolation trials' sizes).
    auto start_lorenzo = [&]() {
        jl.start(ready.a, [&](cudaStream_t s2, Counter &c2, faz_timings &t2, std::vector<uint8_t> &pl,
                              const std::function<void(size_t)> &) {
            if (N == 3) lorenzo_payload<T>(sdims, dS, 5, 3, eb, c.quantbinCnt / 2, s2, c2, t2, pl);
            else gen_compress_payload<T>(N, sdims, 5, 1, 1, 0, eb, c.quantbinCnt / 2, dS, s2, c2, t2, pl);
        });
    };
    start_lorenzo();
    const int dir0 = c.interpDirection;
    // the four block-interpolation trials' sweeps in shared launches on a
    // high-priority stream; each trial's Huffman stage then runs on its own
    // thread and stream
    const BiTrialSpec spec[kBiTrials] = {{0, dir0}, {1, dir0}, {0, dop}, {1, dop}};
    BiTrials<T> bt;
    StreamGuard sf(nullptr, true);
    CK(cudaStreamWaitEvent(sf.st, ready.a, 0));
    block_interp_sweeps<T>(N, sdims, dS, eb, spec, (int64_t)sb, m, sf.st, launches, bt);
    Events swept;
    CK(cudaEventRecord(swept.a, sf.st));
    for (int op = 0; op < 2; op++) {
        ji[op].start(swept.a, [&, op](cudaStream_t s2, Counter &c2, faz_timings &t2, std::vector<uint8_t> &pl,
                                      const std::function<void(size_t)> &rep) {
            block_interp_tail<T>(N, sdims, eb, op, dir0, (int64_t)sb, bt.codes[op], bt.scratch[op], s2, c2, t2, pl, rep);
        });
        jd[op].start(swept.a, [&, op](cudaStream_t s2, Counter &c2, faz_timings &t2, std::vector<uint8_t> &pl,
                                      const std::function<void(size_t)> &rep) {
            block_interp_tail<T>(N, sdims, eb, op, dop, (int64_t)sb, bt.codes[2 + op], bt.scratch[2 + op], s2, c2,
                                 t2, pl, rep);
        });
    }
    // While the Lorenzo trial and the zstd sizes are computed, compress the
    // field with the interpolation choice the pre-zstd sizes point to (the
    // caller keeps the result if the final choice agrees, which it does unless
    // Lorenzo wins or two candidates are within zstd's effect of each other).
    if (speculate) {
        bool ok = true;
        size_t ri[2] = {0, 0}, rd[2] = {0, 0};
        try {
            for (int op = 0; op < 2; op++) {
                ri[op] = ji[op].raw_f.get();
                rd[op] = jd[op].raw_f.get();
            }
        } catch (...) {
            ok = false;  // the trial's own error surfaces below
        }
        if (ok) {
            // the Lorenzo trial is not waited for: interpolation usually wins.
            // The decision rule below runs on the pre-zstd sizes; zstd moves
            // a trial's size by a few tenths of a percent at most, so choices
            // closer than kClose are called for both sides.
            constexpr double kClose = 0.003;
            auto ratio = [&](size_t raw) { return sbytes / (raw + 8); };
            auto pick_dir = [&](int op) { return ratio(rd[op]) > ratio(ri[op]) * 1.02 ? dop : dir0; };
            faz_config g = c;
            g.cmprAlgo = FAZ_ALGO_INTERP;
            g.interpAlgo = ratio(ri[1]) > ratio(ri[0]) ? 1 : 0;
            g.interpDirection = pick_dir(g.interpAlgo);
            faz_config alt = g;
            const double r0 = ratio(ri[0]), r1 = ratio(ri[1]);
            if (std::fabs(r0 - r1) < kClose * std::min(r0, r1)) {
                alt.interpAlgo = 1 - g.interpAlgo;
                alt.interpDirection = pick_dir(alt.interpAlgo);
            } else {
                const double q = ratio(rd[g.interpAlgo]) / (ratio(ri[g.interpAlgo]) * 1.02);
                if (std::fabs(q - 1.0) < kClose) alt.interpDirection = g.interpDirection == dop ? dir0 : dop;
            }
            const bool two = alt.interpAlgo != g.interpAlgo || alt.interpDirection != g.interpDirection;
            if (tune_trace())
                std::fprintf(stderr, "tune %8.3f ms  overlapped compression starts (%s)\n", ms_since(tt0),
                             two ? "two candidates" : "one candidate");
            speculate(g, two ? &alt : nullptr);
            if (tune_trace()) std::fprintf(stderr, "tune %8.3f ms  overlapped compression ends\n", ms_since(tt0));
        }
    }
    // every trial finishes (or fails) before the sample is released
    size_t zl = 0, zi[2] = {0, 0}, zd[2] = {0, 0};
    std::exception_ptr first_err;
    auto collect = [&](Trial &t, size_t &out) {
        try {
            out = t.get();
        } catch (...) {
            if (!first_err) first_err = std::current_exception();
        }
        launches.n += t.launches;
        tm.host_ms += t.host_ms;
    };
    collect(jl, zl);
    for (int op = 0; op < 2; op++) {
        collect(ji[op], zi[op]);
        collect(jd[op], zd[op]);
    }
    if (first_err) std::rethrow_exception(first_err);
    double best_l = sbytes / zl;
    double best_i = 0;
    for (int op = FAZ_INTERP_ALGO_LINEAR; op <= FAZ_INTERP_ALGO_CUBIC; op++) {
        const double r = sbytes / zi[op];
        if (r > best_i) {
            best_i = r;
            c.interpAlgo = op;
        }
    }
    const double rd_lin = sbytes / zd[0], rd_cub = sbytes / zd[1];
    double r = c.interpAlgo == FAZ_INTERP_ALGO_CUBIC ? rd_cub : rd_lin;
    if (r > best_i * 1.02) {
        best_i = r;
        c.interpDirection = dop;
    }
    const bool use_interp = !(best_l > best_i && best_l < 80 && best_i < 80);
    if (use_interp) {
        c.cmprAlgo = FAZ_ALGO_INTERP;
        return;
    }
    lorenzo_followup<T>(c, dX, smp, best_l, st, launches, tm);
}

template void sz3_tune_device<float>(faz_config &, const float *, cudaStream_t, Counter &, faz_timings &,
                                     const std::function<void(const faz_config &, const faz_config *)> &);
template void sz3_tune_device<double>(faz_config &, const double *, cudaStream_t, Counter &, faz_timings &,
                                      const std::function<void(const faz_config &, const faz_config *)> &);


// After the QoZ tuner chose Lorenzo (SZInterp.hpp:2797-2845): the sample of
// sampling<T,N>, its Lorenzo ratio under the Lorenzo settings (Config::setDims
// of the sample dims: block size 6 in 3-D, 16 in 2-D), then the follow-up.
template <typename T>
void qoz_lorenzo_followup(faz_config &c, const T *dX, cudaStream_t st, Counter &launches, faz_timings &tm) {
    const int N = c.N;
    c.lorenzo = 1;
    c.lorenzo2 = 1;
    c.regression = 0;
    c.regression2 = 0;
    c.openmp = 0;
    c.blockSize = 5;
    DevMem m(st);
    Sample<T> smp;
    if (!take_sample<T>(c, dX, m, st, launches, smp)) return;
    faz_config lc = c;
    set_dims_defaults(lc);  // setDims(sample dims)
    std::vector<uint8_t> pl;
    if (N == 3)
        lorenzo_payload<T>(smp.sdims, smp.dS, lc.blockSize, lc.pred_dim, c.absErrorBound, lc.quantbinCnt / 2, st,
                           launches, tm, pl);
    else
        gen_compress_payload<T>(N, smp.sdims, lc.blockSize, 1, 1, 0, c.absErrorBound, lc.quantbinCnt / 2, smp.dS, st,
                                launches, tm, pl);
    const double best_l = smp.sn * 1.0 * sizeof(T) / zstd_framed_size(pl.data(), pl.size());
    lorenzo_followup<T>(c, dX, smp, best_l, st, launches, tm);
}

template void qoz_lorenzo_followup<float>(faz_config &, const float *, cudaStream_t, Counter &, faz_timings &);
template void qoz_lorenzo_followup<double>(faz_config &, const double *, cudaStream_t, Counter &, faz_timings &);

}  // namespace faz
