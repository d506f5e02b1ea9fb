// capi.cu - host orchestration of the GPU compress/decompress path and the
// extern "C" entry points declared in include/faz_gb300.h.
//
// compress (SZ_compress -> SZInterpolationCompressor::compress, reference
// include/QoZ/api/sz.hpp:54-108, SZInterpolationCompressor.hpp:324-529):
//   range (for relative bounds) -> first point / anchor grid -> one kernel per
//   level -> histogram -> codebook (host) -> unpredictable gather -> Huffman
//   encode -> payload assembled in pinned memory -> host zstd -> trailer.
// decompress (sz.hpp:159-205, SZInterpolationCompressor.hpp:42-199):
//   trailer -> host zstd -> header / unpredictables / tree -> GPU Huffman
//   decode -> zero positions -> first point / anchors -> one kernel per level.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "host.h"
#include "internal.h"

namespace faz {

const char *last_error();

namespace {

// --------------------------------------------------------------- geometry
struct LevelPlan {
    LevelArgs args;
    int64_t nblocks;
    uint64_t off_index;  // first entry of this level in the block-offset table
};

struct Plan {
    int N = 0;
    int64_t dims3[3], offs3[3];
    uint64_t num = 0;
    int levels = 0;      // interpolation_level after init()
    bool anchor = false;
    uint64_t maxStep = 0;
    int64_t na[3] = {1, 1, 1};
    uint64_t nanchor = 0;  // codes before the first level
    std::vector<LevelPlan> lv;
    std::vector<uint64_t> block_off;
    uint64_t total_codes = 0;
    size_t max_smem = 0;
};

// permutations of 0..N-1 in lexicographic order (std::next_permutation)
std::vector<std::vector<int>> permutations(int N) {
    std::vector<int> s(N);
    for (int i = 0; i < N; i++) s[i] = i;
    std::vector<std::vector<int>> out;
    do {
        out.push_back(s);
    } while (std::next_permutation(s.begin(), s.end()));
    return out;
}

template <typename T>
Plan make_plan(int N, const uint64_t *dims, uint64_t maxStep, int blocksize, int fixbs, int interp, int dir,
               const std::vector<uint8_t> &ilist, const std::vector<uint8_t> &dlist, double eb, double alpha,
               double beta, int radius, int trim, size_t smem_limit) {
    Plan p;
    p.N = N;
    p.num = 1;
    int e = 3 - N;
    for (int i = 0; i < 3; i++) p.dims3[i] = 1;
    for (int i = 0; i < N; i++) {
        p.dims3[e + i] = (int64_t)dims[i];
        p.num *= dims[i];
    }
    p.offs3[2] = 1;
    p.offs3[1] = p.dims3[2];
    p.offs3[0] = p.dims3[1] * p.dims3[2];
    p.levels = 0;
    for (int i = 0; i < N; i++) p.levels = std::max(p.levels, ceil_log2(dims[i]));
    p.maxStep = maxStep;
    if (maxStep > 0) {
        p.anchor = true;
        p.levels += 1;
        int lm = 0;
        while (((uint64_t)1 << (lm + 1)) <= maxStep) lm++;
        lm += 1;
        if (lm <= p.levels) p.levels = lm;
        if (maxStep & (maxStep - 1)) throw Fail{FAZ_ERR_UNSUPPORTED, "maxStep must be a power of two on the GPU path"};
        if (N != 2 && N != 3) throw Fail{FAZ_ERR_UNSUPPORTED, "an anchor grid needs 2-D or 3-D data"};
        for (int i = 0; i < 3; i++) p.na[i] = 1;
        for (int i = 0; i < N; i++) p.na[e + i] = (int64_t)((dims[i] - 1) / maxStep + 1);
        p.nanchor = (uint64_t)(p.na[0] * p.na[1] * p.na[2]);
    } else {
        p.nanchor = 1;
    }
    if (blocksize <= 0 || (blocksize & 1)) throw Fail{FAZ_ERR_UNSUPPORTED, "interpBlockSize must be a positive even number"};
    auto perms = permutations(N);
    int top = p.anchor ? p.levels - 1 : p.levels;
    if (fixbs > 0) {
        // block begins must stay on the coarse lattice of every level
        if (top > 0 && (fixbs % (1 << top)) != 0)
            throw Fail{FAZ_ERR_UNSUPPORTED, "fixBlockSize must be a multiple of 2^levels on the GPU path"};
    }
    uint64_t pos = p.nanchor;
    for (int level = top; level > 0; level--) {
        LevelPlan L;
        LevelArgs &a = L.args;
        std::memset(&a, 0, sizeof(a));
        int cur_interp = interp, cur_dir = dir;
        if (!ilist.empty()) {
            size_t li = (size_t)(level - 1) < ilist.size() ? (size_t)(level - 1) : ilist.size() - 1;
            cur_interp = ilist[li];
            cur_dir = dlist[li];
        }
        if (cur_dir < 0 || cur_dir >= (int)perms.size()) throw Fail{FAZ_ERR_ARG, "interpolation direction out of range"};
        for (int i = 0; i < 3; i++) {
            a.dims[i] = p.dims3[i];
            a.offs[i] = p.offs3[i];
        }
        for (int i = 0; i < e; i++) a.perm[i] = i;
        for (int i = 0; i < N; i++) a.perm[e + i] = perms[cur_dir][i] + e;
        a.s = (int64_t)1 << (level - 1);
        a.bs = fixbs > 0 ? fixbs : (int64_t)blocksize * a.s;
        a.cubic = cur_interp == FAZ_INTERP_ALGO_CUBIC;
        a.radius = radius;
        a.trim = trim;
        a.eb = level_eb(eb, alpha, beta, level);
        a.recip = 1.0 / a.eb;
        set_fast_path<T>(a);
        a.write_back = level > 1;
        int64_t nmax[3];
        L.nblocks = 1;
        for (int i = 0; i < 3; i++) {
            a.nb[i] = (a.dims[i] - 1) / a.bs + 1;
            L.nblocks *= a.nb[i];
            int64_t ext = std::min<int64_t>(a.bs, a.dims[i] - 1);
            nmax[i] = ext / a.s + 1;
        }
        int64_t m0 = nmax[a.perm[0]], m1 = nmax[a.perm[1]], m2 = nmax[a.perm[2]];
        int64_t vw = m0 * m1 * ((m2 + 1) / 2);
        int64_t stage = std::max({((m1 + 1) / 2) * ((m2 + 1) / 2) * (m0 / 2), m0 * ((m2 + 1) / 2) * (m1 / 2),
                                  m0 * m1 * (m2 / 2)});
        a.vwords = (int)vw;
        a.stage_cap = (int)std::max<int64_t>(stage, 1) + 16;  // + alignment shift
        size_t sm = level_smem_bytes<T>(a);
        if (sm > smem_limit)
            throw Fail{FAZ_ERR_UNSUPPORTED, "interpolation block does not fit in shared memory (block size too large)"};
        p.max_smem = std::max(p.max_smem, sm);
        L.off_index = p.block_off.size();
        int64_t bc[3];
        for (int64_t b = 0; b < L.nblocks; b++) {
            block_coords(a, b, bc);
            BlockGeom g;
            block_geom(a, bc, g);
            p.block_off.push_back(pos);
            pos += (uint64_t)(g.c1 + g.c2 + g.c3);
        }
        p.lv.push_back(L);
    }
    p.total_codes = pos;
    if (p.total_codes != p.num && !(p.anchor && (N == 1 || N == 4)))
        throw Fail{FAZ_ERR_UNSUPPORTED, "block decomposition does not cover the field exactly"};
    return p;
}

// --------------------------------------------------------------- compress
void check_config(const faz_config &c) {
    if (c.N < 1 || c.N > 4) throw Fail{FAZ_ERR_ARG, "N must be 1..4"};
    uint64_t num = 1;
    for (int i = 0; i < c.N; i++) {
        if (c.dims[i] == 0) throw Fail{FAZ_ERR_ARG, "zero dimension"};
        num *= c.dims[i];
    }
    if (num != c.num) throw Fail{FAZ_ERR_ARG, "num does not match dims"};
    if (c.N == 4 && (c.cmprAlgo != FAZ_ALGO_INTERP || c.openmp))
        throw Fail{FAZ_ERR_UNSUPPORTED, "4-D fields are implemented for ALGO_INTERP (without openmp) on the GPU path"};
    if (c.cmprAlgo != FAZ_ALGO_INTERP && c.cmprAlgo != FAZ_ALGO_INTERP_LORENZO && c.cmprAlgo != FAZ_ALGO_LORENZO_REG &&
        c.cmprAlgo != FAZ_ALGO_INTERP_BLOCKED)
        throw Fail{FAZ_ERR_UNSUPPORTED,
                   "cmprAlgo must be ALGO_INTERP, ALGO_INTERP_LORENZO, ALGO_LORENZO_REG or ALGO_INTERP_BLOCKED"};
    if (c.cmprAlgo == FAZ_ALGO_INTERP_BLOCKED && c.N != 3)
        throw Fail{FAZ_ERR_UNSUPPORTED, "ALGO_INTERP_BLOCKED is defined for 3-D data"};
    if (c.cmprAlgo == FAZ_ALGO_INTERP_LORENZO && c.FZ && !c.QoZ)
        throw Fail{FAZ_ERR_UNSUPPORTED, "FAZ features (wavelets, SPERR, conditioning; FZ = 1) are not implemented; "
                                        "set FZ = 0 (faz -F 0)"};
    if (c.cmprAlgo == FAZ_ALGO_LORENZO_REG && c.N == 3 && c.regression2)
        throw Fail{FAZ_ERR_UNSUPPORTED, "ALGO_LORENZO_REG is implemented for 3-D data without regression2"};
    if (c.cmprAlgo == FAZ_ALGO_LORENZO_REG && c.N < 3 && c.regression2)
        throw Fail{FAZ_ERR_UNSUPPORTED, "ALGO_LORENZO_REG on 1-D / 2-D data is implemented without regression2 "
                                        "(Regression2ndOrder = NO)"};
    if (c.blockwiseTuning && c.cmprAlgo != FAZ_ALGO_INTERP_BLOCKED)
        throw Fail{FAZ_ERR_UNSUPPORTED, "blockwiseTuning is set by ALGO_INTERP_BLOCKED only"};
    if (c.wavelet != 0 || ((c.wavelet > 0 || c.sperrWithoutWave) && c.sperr >= c.wavelet))
        throw Fail{FAZ_ERR_UNSUPPORTED, "wavelet / SPERR modes are not part of the interpolation path"};
    // 32-bit codes (more than 65536 bins) are implemented for the 3-D Lorenzo
    // frontend, where the default tuner's interval estimate can ask for them
    if (c.quantbinCnt < 2 || c.quantbinCnt > 131072 ||
        (c.quantbinCnt > 65536 && !(c.cmprAlgo == FAZ_ALGO_LORENZO_REG && c.N == 3)))
        throw Fail{FAZ_ERR_UNSUPPORTED, "quantbinCnt must be in [2, 65536] on the GPU path (up to 131072 for "
                                        "ALGO_LORENZO_REG on 3-D data)"};
    if (c.interp_list_len < 0 || c.interp_list_len > FAZ_MAX_LEVELS) throw Fail{FAZ_ERR_ARG, "bad level list length"};
}

}  // namespace

// data_range<T> (include/QoZ/utils/Statistic.hpp:12-21) on the device: max - min
// in the element type.
template <typename T>
double device_range(const T *dX, uint64_t n, cudaStream_t st, Counter &launches) {
    int nb = (int)std::min<uint64_t>(152 * 4, (n + 4095) / 4096);
    if (nb < 1) nb = 1;
    DevMem m(st);
    T *pmin = m.alloc<T>(nb), *pmax = m.alloc<T>(nb);
    launches(launch_minmax<T>(dX, n, pmin, pmax, nb, st));
    std::vector<T> hmin(nb), hmax(nb);
    CK(cudaMemcpyAsync(hmin.data(), pmin, nb * sizeof(T), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hmax.data(), pmax, nb * sizeof(T), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    T mn = hmin[0], mx = hmax[0];
    for (int i = 0; i < nb; i++) {
        if (hmin[i] < mn) mn = hmin[i];
        if (hmax[i] > mx) mx = hmax[i];
    }
    T r = mx - mn;
    return (double)r;
}
template double device_range<float>(const float *, uint64_t, cudaStream_t, Counter &);
template double device_range<double>(const double *, uint64_t, cudaStream_t, Counter &);

// calAbsErrorBound (include/QoZ/utils/Statistic.hpp:34-66); `rng` computed
// on the device when the mode needs it.
// the absolute bound of a non-ABS mode from the field's range (max - min in
// the element type; unused for L2NORM)
void resolve_eb_range(faz_config &c, double rng) {
    switch (c.errorBoundMode) {
    case FAZ_EB_REL:
        c.absErrorBound = c.relErrorBound * rng;
        break;
    case FAZ_EB_PSNR: {
        double v1 = c.psnrErrorBound + 10 * std::log10(1 - 2.0 / 3.0 * 0.99);
        double v3 = std::pow(10, v1 / (-20));
        c.absErrorBound = rng * v3;
        c.relErrorBound = c.absErrorBound / rng;
        break;
    }
    case FAZ_EB_L2NORM:
        c.absErrorBound = std::sqrt(3.0 / (double)c.num) * c.l2normErrorBound;
        break;
    case FAZ_EB_ABS_AND_REL:
        c.absErrorBound = std::min(c.absErrorBound, c.relErrorBound * rng);
        break;
    case FAZ_EB_ABS_OR_REL:
        c.absErrorBound = std::max(c.absErrorBound, c.relErrorBound * rng);
        break;
    default:
        throw Fail{FAZ_ERR_ARG, "error bound mode not supported"};
    }
    if (c.errorBoundMode != FAZ_EB_L2NORM) c.rng = rng;
    c.errorBoundMode = FAZ_EB_ABS;
}

template <typename T>
void resolve_eb(faz_config &c, const T *dX, cudaStream_t st, Counter &launches) {
    if (c.errorBoundMode == FAZ_EB_ABS) return;
    double rng = 0;
    if (c.errorBoundMode != FAZ_EB_L2NORM) rng = device_range<T>(dX, c.num, st, launches);
    resolve_eb_range(c, rng);
}
template void resolve_eb<float>(faz_config &, const float *, cudaStream_t, Counter &);
template void resolve_eb<double>(faz_config &, const double *, cudaStream_t, Counter &);

namespace {

// GPU part of compression: returns the pre-zstd payload in a pinned buffer.
// Where the payload goes: a caller buffer of `cap` bytes, or (dst == nullptr)
// the thread's pinned staging buffer.
struct Sink {
    uint8_t *dst = nullptr;
    size_t cap = 0;
    bool too_small = false;
};

}  // namespace

// Histogram, codebook (host) and Huffman encoding of n codes on the device
// (HuffmanEncoder::preprocess_encode + encode, HuffmanEncoder.hpp:93-227).
// `center` is the code the histogram's shared-memory window is centred on.
template <typename C>
void huffman_encode_impl(const C *codes, uint64_t n, int center, DevMem &m, cudaStream_t st, Counter &launches,
                         HuffEncoded &h, faz_timings &tm, const std::function<void(const HuffEncoded &)> &sized) {
    const uint64_t nsub = hist_subchunks(n);
    const uint64_t nech = encode_chunks(n);
    // every value a code of this width can take
    const int nsym = sizeof(C) == 2 ? 65536 : std::max(65536, 2 * center + 1);
    // the symbols that occur come back as a compact list (the first
    // kListHead entries with the count, the rest, if any, in a second copy);
    // at most min(nsym, n) symbols occur, and the head copy reads kListHead
    constexpr size_t kListHead = 2048;
    const size_t list_cap = std::max<size_t>(std::min<uint64_t>((uint64_t)nsym, n), kListHead);
    // One allocation holds the work arrays (CUDA calls are few: the tuners
    // run several of these encodes on concurrent host threads, whose calls
    // serialise in the driver).  In 8-byte words, each part 256-byte aligned:
    // histogram + list count, first positions, zero counts and offsets, scan
    // scratch, list, codebook tables (stateNum <= nsym + 1 entries of 17
    // bytes), chunk bit counts and offsets.
    auto up = [](uint64_t w) { return (w + 31) & ~(uint64_t)31; };
    const uint64_t w_hist = up((uint64_t)nsym + 1), w_first = up((uint64_t)nsym), w_z = up(nsub + 1),
                   w_tmp = up(scan_temp_words(std::max<uint64_t>(nsub, nech)) + 1), w_list = up(3 * list_cap),
                   w_tab = up(((uint64_t)nsym + 1) * 17 / 8 + 1), w_ch = up(nech + 1);
    unsigned long long *work =
        m.alloc<unsigned long long>(w_hist + w_first + 2 * w_z + w_tmp + w_list + w_tab + 2 * w_ch);
    unsigned long long *hist = work;
    unsigned int *dnl = reinterpret_cast<unsigned int *>(hist + nsym);
    unsigned long long *first = hist + w_hist;
    h.zc = first + w_first;
    h.zoff = h.zc + w_z;
    unsigned long long *stmp = h.zoff + w_z;
    unsigned long long *dlist = stmp + w_tmp;
    uint8_t *dtab = reinterpret_cast<uint8_t *>(dlist + w_list);
    unsigned long long *cbits = dlist + w_list + w_tab;
    unsigned long long *coff = cbits + w_ch;
    CK(cudaMemsetAsync(hist, 0, ((size_t)nsym + 1) * 8, st));
    CK(cudaMemsetAsync(first, 0xff, (size_t)nsym * 8, st));
    launches(launch_histogram(codes, n, center, hist, first, h.zc, st));
    launches(launch_scan_u64(h.zc, h.zoff, nsub, stmp, st));
    launches(launch_hist_compact(hist, first, nsym, dlist, dnl, st));
    uint8_t *hb = t_pin_small.get(16 + kListHead * 24);
    CK(cudaMemcpyAsync(hb, dnl, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hb + 8, h.zoff + nsub, 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hb + 16, dlist, kListHead * 24, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (tune_trace()) {
        char msg[96];
        std::snprintf(msg, sizeof(msg), "huffman histogram of %llu codes on the host", (unsigned long long)n);
        trace_step(msg);
    }
    auto th1 = clk::now();
    unsigned int nl = 0;
    std::memcpy(&nl, hb, 4);
    std::memcpy(&h.nzero, hb + 8, 8);
    if (nl > (unsigned int)nsym || nl > list_cap)
        throw Fail{FAZ_ERR_DEVICE, "histogram list longer than the symbol range"};
    std::vector<unsigned long long> rest;
    if (nl > kListHead) {
        rest.resize(3 * (size_t)(nl - kListHead));
        CK(cudaMemcpyAsync(rest.data(), dlist + 3 * kListHead, rest.size() * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    std::vector<int> syms(nl);
    std::vector<uint64_t> cnts(nl), firsts(nl);
    const unsigned long long *head = (const unsigned long long *)(hb + 16);
    for (unsigned int k = 0; k < nl; k++) {
        const unsigned long long *e = k < kListHead ? head + 3 * (size_t)k : rest.data() + 3 * (size_t)(k - kListHead);
        syms[k] = (int)e[0];
        cnts[k] = e[1];
        firsts[k] = e[2];
    }
    trace_step("huffman symbols listed");
    std::string err;
    int rc = build_codebook(syms, cnts, firsts, h.cb, err);
    if (rc) throw Fail{rc, err};
    trace_step("huffman tree built");
    tm.host_ms += ms_since(th1);
    const Codebook &cb = h.cb;
    // The three tables (MSB-aligned codes, packed length|code, lengths) go
    // up in one copy from the thread's pinned staging: pageable copies from
    // several threads serialise in the driver.  The staging is refilled once
    // the thread's previous upload from it has completed.
    const size_t S = (size_t)cb.stateNum;
    if (S > (size_t)nsym + 1) throw Fail{FAZ_ERR_DEVICE, "Huffman codebook larger than the symbol range"};
    TableStage &ts = t_table_stage;
    uint8_t *htab = ts.acquire(S * 17);
    unsigned long long *hcode = reinterpret_cast<unsigned long long *>(htab);
    unsigned long long *hpacked = hcode + S;
    std::memcpy(hcode, cb.code.data(), S * 8);
    for (size_t i = 0; i < S; i++) {
        const int l = cb.len[i];
        hpacked[i] = ((unsigned long long)l << 32) | (l >= 1 && l <= 32 ? (cb.code[i] >> (64 - l)) : 0ull);
    }
    std::memcpy(htab + S * 16, cb.len.data(), S);
    CK(cudaMemcpyAsync(dtab, htab, S * 17, cudaMemcpyHostToDevice, st));
    ts.release(st);
    unsigned long long *dcode = reinterpret_cast<unsigned long long *>(dtab);
    unsigned long long *dpacked = dcode + S;
    uint8_t *dlen = dtab + S * 16;
    trace_step("huffman tables uploaded");
    // the encoded size from the counts and code lengths (what the device's
    // chunk scan adds up)
    uint64_t total_bits = 0;
    for (size_t i = 0; i < syms.size(); i++) total_bits += cnts[i] * (uint64_t)cb.len[syms[i] - cb.offset];
    h.nbytes = (total_bits + 7) / 8;
    if (tune_trace()) {
        char msg[96];
        std::snprintf(msg, sizeof(msg), "huffman codebook of %llu codes built", (unsigned long long)n);
        trace_step(msg);
    }
    if (sized) sized(h);
    launches(launch_encode_bits(codes, n, cb.offset, dlen, cbits, st));
    launches(launch_scan_u64(cbits, coff, nech, stmp, st));
    const uint64_t nwords = (total_bits + 31) / 32 + 1;
    h.bits = m.alloc<uint32_t>(nwords);
    CK(cudaMemsetAsync(h.bits, 0, nwords * 4, st));
    if (total_bits)
        launches(launch_encode_pack(codes, n, cb.offset, dcode, dpacked, dlen, coff, h.bits, std::max(cb.maxlen, 1), st));
}

void huffman_encode_device(const uint16_t *codes, uint64_t n, int center, DevMem &m, cudaStream_t st,
                           Counter &launches, HuffEncoded &h, faz_timings &tm,
                           const std::function<void(const HuffEncoded &)> &sized) {
    huffman_encode_impl(codes, n, center, m, st, launches, h, tm, sized);
}
void huffman_encode_device(const uint32_t *codes, uint64_t n, int center, DevMem &m, cudaStream_t st,
                           Counter &launches, HuffEncoded &h, faz_timings &tm,
                           const std::function<void(const HuffEncoded &)> &sized) {
    if (center < 0 || center > (1 << 20)) throw Fail{FAZ_ERR_UNSUPPORTED, "quantisation radius too large"};
    huffman_encode_impl(codes, n, center, m, st, launches, h, tm, sized);
}

// HuffmanEncoder::save header + tree, then the encoded size (HuffmanEncoder.hpp:119-137, 150-227)
void append_tree(std::vector<uint8_t> &o, const Codebook &cb, uint64_t nbytes) {
    put<int32_t>(o, cb.offset);
    put_be32(o, cb.nodeCount);
    put_be32(o, cb.stateNum / 2);
    o.insert(o.end(), cb.tree.begin(), cb.tree.end());
    put<uint64_t>(o, nbytes);
}

namespace {

// The Huffman stage of an interpolation compression whose codes (stream order)
// and unpredictable values (at their code positions in scratch) are on the
// device: the bit string, and the unpredictable values in stream order.
template <typename T>
struct InterpEncoded {
    HuffEncoded he;
    T *unpred = nullptr;
};

template <typename T>
void interp_encode(uint64_t n, int radius, uint16_t *codes, T *scratch, unsigned long long *vcount, const int *lerr,
                   DevMem &m, cudaStream_t st, Counter &launches, faz_timings &tm, InterpEncoded<T> &e) {
    huffman_encode_device(codes, n, radius, m, st, launches, e.he, tm);
    if (lerr) {
        int le = 0;
        CK(cudaMemcpy(&le, lerr, sizeof(int), cudaMemcpyDeviceToHost));
        if (le) throw Fail{FAZ_ERR_DEVICE, "an interpolation level kernel gave up waiting for its plane copies"};
    }
    if (vcount) {
        unsigned long long vc = 0;
        CK(cudaMemcpy(&vc, vcount, 8, cudaMemcpyDeviceToHost));
        if (vc) throw Fail{FAZ_ERR_DEVICE, "float fast path disagreed with the double path at " + std::to_string(vc) + " points"};
    }
    const uint64_t nunpred = e.he.nzero;
    e.unpred = m.alloc<T>(nunpred ? nunpred : 1);
    if (nunpred) launches(launch_compact_zeros<T>(codes, n, e.he.zc, e.he.zoff, nullptr, scratch, e.unpred, st));
}

// The payload of an encoded interpolation compression: the bytes
// SZInterpolationCompressor::compress hands to zstd (SZInterpolationCompressor.hpp:
// 485-512, IntegerQuantizer.hpp:185-201, HuffmanEncoder.hpp:119-137 and 150-227).
template <typename T>
void interp_emit(const faz_config &c, const std::vector<uint8_t> &il, const std::vector<uint8_t> &dl, double eb,
                 int radius, const InterpEncoded<T> &e, cudaStream_t st, faz_timings &tm, Sink *sink,
                 uint8_t *&payload, size_t &psize) {
    const uint64_t nunpred = e.he.nzero;
    const Codebook &cb = e.he.cb;
    const uint64_t nbytes = e.he.nbytes;
    auto th2 = clk::now();
    std::vector<uint8_t> head;
    for (int i = 0; i < c.N; i++) put<uint64_t>(head, c.dims[i]);
    put<uint32_t>(head, (uint32_t)c.interpBlockSize);
    put<int32_t>(head, (int32_t)c.interpAlgo);
    put<int32_t>(head, (int32_t)c.interpDirection);
    put<double>(head, c.alpha);
    put<double>(head, c.beta);
    put<uint64_t>(head, c.maxStep);
    put<int32_t>(head, c.interp_list_len);
    put<uint8_t>(head, c.blockwiseTuning);
    put<int32_t>(head, c.fixBlockSize);
    put<uint64_t>(head, (uint64_t)(int64_t)c.crossBlock);
    put<int32_t>(head, c.trimToZero);
    put<int32_t>(head, c.blockOrder);
    head.insert(head.end(), il.begin(), il.end());
    head.insert(head.end(), dl.begin(), dl.end());
    put<uint8_t>(head, 2);
    put<double>(head, eb);
    put<int32_t>(head, radius);
    put<uint64_t>(head, nunpred);
    std::vector<uint8_t> tree;
    append_tree(tree, cb, nbytes);
    psize = head.size() + nunpred * sizeof(T) + tree.size() + nbytes;
    if (sink && sink->dst) {
        if (psize > sink->cap) {
            sink->too_small = true;
            throw Fail{FAZ_ERR_ARG, "payload buffer too small: need " + std::to_string(psize) + " bytes"};
        }
        payload = sink->dst;
    } else {
        payload = t_pin_payload.get(psize + 8);
    }
    std::memcpy(payload, head.data(), head.size());
    size_t o = head.size();
    tm.host_ms += ms_since(th2);
    if (nunpred) CK(cudaMemcpyAsync(payload + o, e.unpred, nunpred * sizeof(T), cudaMemcpyDeviceToHost, st));
    o += nunpred * sizeof(T);
    std::memcpy(payload + o, tree.data(), tree.size());
    o += tree.size();
    if (nbytes) CK(cudaMemcpyAsync(payload + o, e.he.bits, nbytes, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    tm.unpred_count = nunpred;
    tm.payload_bytes = psize;
}

// Both stages: the Huffman stage and the payload.
template <typename T>
void interp_payload_tail(const faz_config &c, const std::vector<uint8_t> &il, const std::vector<uint8_t> &dl,
                         double eb, int radius, uint64_t n, uint16_t *codes, T *scratch, unsigned long long *vcount,
                         DevMem &m, cudaStream_t st, Counter &launches, faz_timings &tm, Sink *sink,
                         uint8_t *&payload, size_t &psize, cudaEvent_t huff_end = nullptr, const int *lerr = nullptr) {
    InterpEncoded<T> e;
    interp_encode<T>(n, radius, codes, scratch, vcount, lerr, m, st, launches, tm, e);
    if (huff_end) CK(cudaEventRecord(huff_end, st));
    interp_emit<T>(c, il, dl, eb, radius, e, st, tm, sink, payload, psize);
}

// The device part of an interpolation compression up to the quantisation
// codes (stream order) and the unpredictable values at their code positions;
// interp_finish adds the Huffman stage and the payload.
template <typename T>
struct InterpCodes {
    faz_config c;  // error bound resolved
    double eb = 0;
    int radius = 0;
    std::vector<uint8_t> il, dl;
    uint64_t n = 0;
    bool have_levels = false;
    DevMem m;
    T *scratch = nullptr;
    uint16_t *codes = nullptr;
    unsigned long long *vcount = nullptr;
    int *lerr = nullptr;  // set by a level kernel whose bounded wait gave up
    Events ev_pred, ev_fin, ev_huff;
    InterpEncoded<T> enc;  // the Huffman stage, once interp_encode_codes ran
    bool encoded = false;
    explicit InterpCodes(cudaStream_t st) : m(st) {}
};

// First point / anchor grid and every level (SZInterpolationCompressor.hpp:
// 324-461); resolves the error bound of c.
template <typename T>
void interp_levels(InterpCodes<T> &r, faz_config &c, const T *dX, cudaStream_t st, Counter &launches) {
    resolve_eb<T>(c, dX, st, launches);
    const double eb = c.absErrorBound;
    if (!(eb > 0) || !std::isfinite(eb)) throw Fail{FAZ_ERR_ARG, "error bound must be positive and finite"};
    const int radius = c.quantbinCnt / 2;
    if (radius > 32768) throw Fail{FAZ_ERR_UNSUPPORTED, "interpolation with more than 65536 bins is not implemented"};
    r.il.assign(c.interpAlgo_list, c.interpAlgo_list + c.interp_list_len);
    r.dl.assign(c.interpDirection_list, c.interpDirection_list + c.interp_list_len);
    if (c.N == 4) {
        // 4-D: one launch per level and sweep (interp4.cu)
        DevMem &m = r.m;
        T *W = m.alloc<T>(c.num);
        r.scratch = m.alloc<T>(c.num);
        r.codes = m.alloc<uint16_t>(c.num);
        unsigned long long *vcount = nullptr;
        if (verify_fast_path()) {
            vcount = m.alloc<unsigned long long>(1);
            CK(cudaMemsetAsync(vcount, 0, 8, st));
        }
        CK(cudaEventRecord(r.ev_pred.a, st));
        interp4_codes<T>(c, eb, radius, r.il, r.dl, dX, W, r.codes, r.scratch, vcount, m, st, launches);
        CK(cudaEventRecord(r.ev_pred.b, st));
        r.c = c;
        r.eb = eb;
        r.radius = radius;
        r.n = c.num;
        r.vcount = vcount;
        r.have_levels = false;
        return;
    }
    if (c.fixBlockSize > 0 && !fixbs_aligned(c.N, c.dims, c.maxStep, c.fixBlockSize)) {
        // blocks of fixBlockSize that leave the coarse lattice: the block
        // wavefront of blocked.cu with the level's interpolator and direction
        DevMem &m = r.m;
        T *W = m.alloc<T>(c.num);
        r.scratch = m.alloc<T>(c.num);
        r.codes = m.alloc<uint16_t>(c.num);
        CK(cudaEventRecord(r.ev_pred.a, st));
        fixed_block_codes<T>(c, r.il, r.dl, dX, W, r.codes, r.scratch, m, st, launches);
        CK(cudaEventRecord(r.ev_pred.b, st));
        r.c = c;
        r.eb = eb;
        r.radius = radius;
        r.n = c.num;
        r.vcount = nullptr;
        r.have_levels = false;
        return;
    }
    Plan p = make_plan<T>(c.N, c.dims, c.maxStep, c.interpBlockSize, c.fixBlockSize, c.interpAlgo, c.interpDirection,
                          r.il, r.dl, eb, c.alpha, c.beta, radius, c.trimToZero, smem_limit());
    const uint64_t n = p.num;
    DevMem &m = r.m;
    T *W = m.alloc<T>(n);
    T *scratch = m.alloc<T>(n);
    uint16_t *codes = m.alloc<uint16_t>(n);
    uint64_t *boff = m.alloc<uint64_t>(p.block_off.size());
    CK(cudaMemcpyAsync(boff, p.block_off.data(), p.block_off.size() * 8, cudaMemcpyHostToDevice, st));
    // first point / anchors
    if (!p.anchor) {
        launches(launch_first_point<T>(false, dX, W, codes, scratch, eb, radius, c.trimToZero, nullptr, 0, nullptr, st));
    } else {
        int64_t step[3] = {1, 1, 1};
        int e = 3 - p.N;
        for (int i = 0; i < p.N; i++) step[e + i] = (int64_t)p.maxStep;
        launches(launch_anchors<T>(false, dX, W, codes, scratch, nullptr, p.na, step, p.offs3, st));
    }
    unsigned long long *vcount = nullptr;
    if (verify_fast_path()) {
        vcount = m.alloc<unsigned long long>(1);
        CK(cudaMemsetAsync(vcount, 0, 8, st));
    }
    int *lerr = m.alloc<int>(1);
    CK(cudaMemsetAsync(lerr, 0, sizeof(int), st));
    CK(cudaEventRecord(r.ev_pred.a, st));
    for (size_t li = 0; li < p.lv.size(); li++) {
        const LevelPlan &L = p.lv[li];
        LevelArgs a = L.args;
        a.block_off = boff + L.off_index;
        a.ncodes = n;
        a.err = lerr;
        a.verify = vcount;
        if (li + 1 == p.lv.size()) CK(cudaEventRecord(r.ev_fin.a, st));
        int nl = 0;
        CK(launch_level<T>(a, L.nblocks, false, dX, W, codes, scratch, nullptr, 0, nullptr, st, &nl));
        launches.n += nl;
    }
    CK(cudaEventRecord(r.ev_fin.b, st));
    CK(cudaEventRecord(r.ev_pred.b, st));
    r.c = c;
    r.eb = eb;
    r.radius = radius;
    r.n = n;
    r.scratch = scratch;
    r.codes = codes;
    r.vcount = vcount;
    r.lerr = lerr;
    r.have_levels = !p.lv.empty();
}

// The Huffman stage of interp_levels' codes (the speculative compressions of
// the SZ3 tuner run it before the tuner's decision).
template <typename T>
void interp_encode_codes(InterpCodes<T> &r, cudaStream_t st, faz_timings &tm, Counter &launches) {
    CK(cudaEventRecord(r.ev_huff.a, st));
    interp_encode<T>(r.n, r.radius, r.codes, r.scratch, r.vcount, r.lerr, r.m, st, launches, tm, r.enc);
    CK(cudaEventRecord(r.ev_huff.b, st));
    r.encoded = true;
}

// The Huffman stage (unless it ran already) and the payload of
// interp_levels' codes.
template <typename T>
void interp_finish(InterpCodes<T> &r, cudaStream_t st, uint8_t *&payload, size_t &psize, faz_timings &tm,
                   Counter &launches, Sink *sink) {
    if (!r.encoded) interp_encode_codes<T>(r, st, tm, launches);
    interp_emit<T>(r.c, r.il, r.dl, r.eb, r.radius, r.enc, st, tm, sink, payload, psize);
    tm.predict_ms = r.ev_pred.ms();
    tm.finest_level_ms = r.have_levels ? r.ev_fin.ms() : 0.0;
    tm.huffman_ms = r.ev_huff.ms();
}

template <typename T>
void compress_payload(faz_config &c, const T *dX, cudaStream_t st, uint8_t *&payload, size_t &psize,
                      faz_timings &tm, Counter &launches, Sink *sink = nullptr) {
    InterpCodes<T> r(st);
    interp_levels<T>(r, c, dX, st, launches);
    interp_finish<T>(r, st, payload, psize, tm, launches, sink);
}

// ALGO_INTERP_BLOCKED (SZInterp.hpp:3021-3500, compress_block
// SZInterpolationCompressor.hpp:533-781): the Config becomes ALGO_INTERP with
// block-wise tuning; the payload is the interpolation payload with the
// per-block choices after the header.
template <typename T>
void blocked_payload(faz_config &c, const T *dX, cudaStream_t st, uint8_t *&payload, size_t &psize, faz_timings &tm,
                     Counter &launches, Sink *sink) {
    blocked_prepare(c);
    const int radius = c.quantbinCnt / 2;
    if (radius > 32768) throw Fail{FAZ_ERR_UNSUPPORTED, "interpolation with more than 65536 bins is not implemented"};
    const uint64_t n = c.num;
    DevMem m(st);
    T *W = m.alloc<T>(n), *scratch = m.alloc<T>(n);
    uint16_t *codes = m.alloc<uint16_t>(n);
    Events ev_pred, ev_huff;
    CK(cudaEventRecord(ev_pred.a, st));
    std::vector<uint8_t> ops, dirs;
    blocked_codes<T>(c, dX, W, codes, scratch, m, st, launches, ops, dirs);
    CK(cudaEventRecord(ev_pred.b, st));
    // compress_block (lines 753-757): choice count, interpolators, directions
    std::vector<uint8_t> il;
    put<uint64_t>(il, (uint64_t)ops.size());
    il.insert(il.end(), ops.begin(), ops.end());
    CK(cudaEventRecord(ev_huff.a, st));
    interp_payload_tail<T>(c, il, dirs, c.absErrorBound, radius, n, codes, scratch, nullptr, m, st, launches, tm, sink,
                           payload, psize, ev_huff.b);
    tm.predict_ms = ev_pred.ms();
    tm.huffman_ms = ev_huff.ms();
}

// SZ_compress_dispatcher (include/QoZ/api/impl/SZDispatcher.hpp:12-36): error
// bound, the default configuration's tuner, then the chosen compressor.
template <typename T>
void compress_dispatch(faz_config &c, const T *dX, cudaStream_t st, uint8_t *&payload, size_t &psize,
                       faz_timings &tm, Counter &launches, Sink *sink = nullptr) {
    resolve_eb<T>(c, dX, st, launches);
    if (!(c.absErrorBound > 0) || !std::isfinite(c.absErrorBound))
        throw Fail{FAZ_ERR_ARG, "error bound must be positive and finite"};
    if (c.cmprAlgo == FAZ_ALGO_INTERP_LORENZO && qoz_tuned(c)) {
        // QoZ tuning (the faz tool's -q, or a predictorTuningRate in (0, 1)),
        // then the interpolation compressor
        auto tt = clk::now();
        qoz_tune_device<T>(c, dX, st, launches, tm);
        tm.tune_ms = ms_since(tt);
    }
    if (c.cmprAlgo == FAZ_ALGO_INTERP_LORENZO) {
        auto tt = clk::now();
        faz_timings tt_tm;
        std::memset(&tt_tm, 0, sizeof(tt_tm));
        // While the trials' zstd sizes are computed, the interpolation
        // compression that the pre-zstd sizes point to runs; it is kept when
        // the final choice is the same.  When the best two candidates are too
        // close for the pre-zstd sizes to tell, the codes of both are computed
        // and the Huffman stage of the winner follows the decision.
        bool have = false;
        faz_config guess;
        std::memset(&guess, 0, sizeof(guess));
        std::unique_ptr<InterpCodes<T>> both[2];
        faz_config both_conf[2];
        auto speculate = [&](const faz_config &g, const faz_config *alt) {
            if (!alt) {
                guess = g;
                compress_payload<T>(guess, dX, st, payload, psize, tm, launches, sink);
                have = true;
                return;
            }
            for (int k = 0; k < 2; k++) {
                both_conf[k] = k ? *alt : g;
                both[k].reset(new InterpCodes<T>(st));
                interp_levels<T>(*both[k], both_conf[k], dX, st, launches);
            }
        };
        sz3_tune_device<T>(c, dX, st, launches, tt_tm, speculate);
        tm.tune_ms = ms_since(tt);
        if (c.cmprAlgo == FAZ_ALGO_INTERP) {
            if (have && c.interpAlgo == guess.interpAlgo && c.interpDirection == guess.interpDirection) return;
            for (int k = 0; k < 2; k++) {
                if (both[k] && c.interpAlgo == both_conf[k].interpAlgo &&
                    c.interpDirection == both_conf[k].interpDirection) {
                    interp_finish<T>(*both[k], st, payload, psize, tm, launches, sink);
                    return;
                }
            }
        }
    }
    if (c.cmprAlgo == FAZ_ALGO_INTERP) {
        compress_payload<T>(c, dX, st, payload, psize, tm, launches, sink);
        return;
    }
    if (c.cmprAlgo == FAZ_ALGO_INTERP_BLOCKED) {
        blocked_payload<T>(c, dX, st, payload, psize, tm, launches, sink);
        return;
    }
    std::vector<uint8_t> pl;
    if (c.N < 3) {
        if (c.regression2)
            throw Fail{FAZ_ERR_UNSUPPORTED, "ALGO_LORENZO_REG on 1-D / 2-D data is implemented without regression2"};
        gen_compress_payload<T>(c.N, c.dims, c.blockSize, c.lorenzo, c.lorenzo2, c.regression, c.absErrorBound,
                                c.quantbinCnt / 2, dX, st, launches, tm, pl);
    } else {
        if (c.N != 3 || c.regression2)
            throw Fail{FAZ_ERR_UNSUPPORTED, "ALGO_LORENZO_REG is implemented for 3-D data without regression2"};
        lorenzo3_compress_payload<T>(c.dims, c.blockSize, c.pred_dim, c.lorenzo, c.lorenzo2, c.regression,
                                     c.absErrorBound, c.quantbinCnt / 2, dX, st, launches, tm, pl);
    }
    psize = pl.size();
    if (sink && sink->dst) {
        if (psize > sink->cap) {
            sink->too_small = true;
            throw Fail{FAZ_ERR_ARG, "payload buffer too small: need " + std::to_string(psize) + " bytes"};
        }
        payload = sink->dst;
    } else {
        payload = t_pin_payload.get(psize + 8);
    }
    std::memcpy(payload, pl.data(), psize);
}

// Lossless_zstd::compress framing (include/QoZ/lossless/Lossless_zstd.hpp:22-32),
// then Config::save + int32 trailer size (include/QoZ/api/sz.hpp:77-91).
void finish_stream(const faz_config &c, const uint8_t *payload, size_t psize, char **out, size_t *out_size,
                   faz_timings &tm, bool parallel_frames = true) {
    std::string err;
    const Zstd &z = zstd_lib(err);
    if (!z.ok) throw Fail{FAZ_ERR_ZSTD, err};
    auto t0 = clk::now();
    std::vector<uint8_t> trailer;
    config_save(c, trailer);
    // one level-3 frame, by zstd's worker threads (FAZ_ZSTD_THREADS, default
    // the host's cores up to 16) or, with FAZ_ZSTD_THREADS=0, by ZSTD_compress
    // itself as the reference calls it; FAZ_ZSTD_MULTIFRAME=1 writes
    // independent frames instead
    const ZstdPlan plan = zstd_plan(psize);
    size_t bound = zstd_body_bound(z, psize, plan);
    size_t cap = 8 + bound + trailer.size() + 4;
    char *buf = (char *)std::malloc(cap);
    if (!buf) throw Fail{FAZ_ERR_ARG, "out of host memory"};
    uint64_t raw = psize;
    std::memcpy(buf, &raw, 8);
    size_t zs = zstd_compress_body(z, (uint8_t *)buf + 8, bound, payload, psize, plan, parallel_frames);
    if (z.isError(zs)) {
        std::free(buf);
        throw Fail{FAZ_ERR_ZSTD, "ZSTD_compress failed"};
    }
    tm.zstd_ms += ms_since(t0);
    size_t pos = 8 + zs;
    std::memcpy(buf + pos, trailer.data(), trailer.size());
    pos += trailer.size();
    int32_t ts = (int32_t)trailer.size();
    std::memcpy(buf + pos, &ts, 4);
    pos += 4;
    *out = buf;
    *out_size = pos;
}

template <typename T>
int compress_payload_impl(const faz_config *conf_in, const void *d_data, void *user_stream, char *out, size_t cap,
                          size_t *out_size, faz_config *conf_out, faz_timings *tmo) {
    faz_timings tm;
    std::memset(&tm, 0, sizeof(tm));
    auto t0 = clk::now();
    Sink sink;
    sink.dst = (uint8_t *)out;
    sink.cap = cap;
    try {
        if (!conf_in || !d_data || !out || !out_size) throw Fail{FAZ_ERR_ARG, "null argument"};
        faz_config c = *conf_in;
        check_config(c);
        init_pool_once();
        StreamGuard sg(user_stream, false, NullStream::Default);
        Counter launches;
        Events ev_gpu;
        uint8_t *payload;
        size_t psize;
        CK(cudaEventRecord(ev_gpu.a, sg.st));
        try {
            compress_dispatch<T>(c, (const T *)d_data, sg.st, payload, psize, tm, launches, &sink);
        } catch (const Fail &f) {
            if (sink.too_small) *out_size = psize;
            throw;
        }
        CK(cudaEventRecord(ev_gpu.b, sg.st));
        CK(cudaStreamSynchronize(sg.st));
        tm.gpu_ms = ev_gpu.ms();
        *out_size = psize;
        if (conf_out) *conf_out = c;
        tm.kernel_launches = launches.n;
    } catch (const Fail &f) {
        set_error(f.msg);
        return f.code;
    } catch (const std::exception &e) {
        set_error(e.what());
        return FAZ_ERR_ARG;
    }
    tm.total_ms = ms_since(t0);
    if (tmo) *tmo = tm;
    return FAZ_OK;
}

// Batched compression of device-resident fields: one launch resolves every
// field's range, one persistent launch runs every ALGO_INTERP field's first
// point / anchors and all of its levels from a work queue, then the Huffman
// stage, payload and zstd frame of each field run on a pool of host threads
// (each with its own stream).  Fields with another algorithm (a tuner, Lorenzo)
// are compressed one by one afterwards.  Every stream equals the one
// faz_compress_device writes for the same field and configuration.
template <typename T>
int compress_batch_impl(int nf, const faz_config *confs, const void *const *d_data, void *user_stream, char **outs,
                        size_t *out_sizes, int threads_hint, faz_timings *tmo) {
    faz_timings tm;
    std::memset(&tm, 0, sizeof(tm));
    auto t0 = clk::now();
    try {
        if (nf <= 0 || !confs || !d_data || !outs || !out_sizes) throw Fail{FAZ_ERR_ARG, "null argument"};
        for (int i = 0; i < nf; i++) {
            outs[i] = nullptr;
            out_sizes[i] = 0;
            if (!d_data[i]) throw Fail{FAZ_ERR_ARG, "null field pointer"};
        }
        init_pool_once();
        StreamGuard sg(user_stream, false, NullStream::Default);
        cudaStream_t st = sg.st;
        Counter launches;
        std::vector<faz_config> cs(confs, confs + nf);
        for (auto &c : cs) check_config(c);
        DevMem m(st);
        // ranges of every field that needs one, in one launch
        {
            std::vector<const T *> ptr;
            std::vector<uint64_t> num;
            std::vector<int> which;
            for (int i = 0; i < nf; i++)
                if (cs[i].errorBoundMode != FAZ_EB_ABS && cs[i].errorBoundMode != FAZ_EB_L2NORM) {
                    which.push_back(i);
                    ptr.push_back((const T *)d_data[i]);
                    num.push_back(cs[i].num);
                }
            std::vector<double> rng(nf, 0.0);
            if (!which.empty()) {
                const int nb = 64, k = (int)which.size();
                const T **dptr = m.alloc<const T *>(k);
                uint64_t *dnum = m.alloc<uint64_t>(k);
                T *pmin = m.alloc<T>((size_t)k * nb), *pmax = m.alloc<T>((size_t)k * nb);
                CK(cudaMemcpyAsync(dptr, ptr.data(), k * sizeof(T *), cudaMemcpyHostToDevice, st));
                CK(cudaMemcpyAsync(dnum, num.data(), k * 8, cudaMemcpyHostToDevice, st));
                launches(launch_minmax_batch<T>(dptr, dnum, k, pmin, pmax, nb, st));
                std::vector<T> hmin((size_t)k * nb), hmax((size_t)k * nb);
                CK(cudaMemcpyAsync(hmin.data(), pmin, hmin.size() * sizeof(T), cudaMemcpyDeviceToHost, st));
                CK(cudaMemcpyAsync(hmax.data(), pmax, hmax.size() * sizeof(T), cudaMemcpyDeviceToHost, st));
                CK(cudaStreamSynchronize(st));
                for (int j = 0; j < k; j++) {
                    T mn = hmin[(size_t)j * nb], mx = hmax[(size_t)j * nb];
                    for (int b = 0; b < nb; b++) {
                        mn = std::min(mn, hmin[(size_t)j * nb + b]);
                        mx = std::max(mx, hmax[(size_t)j * nb + b]);
                    }
                    const T r = mx - mn;
                    rng[which[j]] = (double)r;
                }
            }
            for (int i = 0; i < nf; i++)
                if (cs[i].errorBoundMode != FAZ_EB_ABS) resolve_eb_range(cs[i], rng[i]);
        }
        for (auto &c : cs)
            if (!(c.absErrorBound > 0) || !std::isfinite(c.absErrorBound))
                throw Fail{FAZ_ERR_ARG, "error bound must be positive and finite"};
        // plans and work queue of the ALGO_INTERP fields
        struct FieldWork {
            int idx;
            Plan p;
            std::vector<uint8_t> il, dl;
            uint16_t *codes;
            T *W, *scratch;
        };
        std::vector<FieldWork> fw;
        std::vector<int> rest;
        const int threads = threads_hint == 256 || threads_hint == 128 ? threads_hint : 512;
        for (int i = 0; i < nf; i++) {
            const faz_config &c = cs[i];
            if (c.cmprAlgo != FAZ_ALGO_INTERP || c.N == 4 ||
                (c.fixBlockSize > 0 && !fixbs_aligned(c.N, c.dims, c.maxStep, c.fixBlockSize))) {
                rest.push_back(i);
                continue;
            }
            FieldWork w;
            w.idx = i;
            w.il.assign(c.interpAlgo_list, c.interpAlgo_list + c.interp_list_len);
            w.dl.assign(c.interpDirection_list, c.interpDirection_list + c.interp_list_len);
            w.p = make_plan<T>(c.N, c.dims, c.maxStep, c.interpBlockSize, c.fixBlockSize, c.interpAlgo,
                               c.interpDirection, w.il, w.dl, c.absErrorBound, c.alpha, c.beta, c.quantbinCnt / 2,
                               c.trimToZero, smem_limit());
            w.W = m.alloc<T>(w.p.num);
            w.scratch = m.alloc<T>(w.p.num);
            w.codes = m.alloc<uint16_t>(w.p.num);
            fw.push_back(std::move(w));
        }
        Events ev_pred;
        CK(cudaEventRecord(ev_pred.a, st));
        if (!fw.empty()) {
            std::vector<uint64_t> boff;
            std::vector<BatchField> bf(fw.size());
            std::vector<LevelArgs> la;
            std::vector<BatchGroup> groups;
            std::vector<size_t> boff_base(fw.size());
            bool wide = false;
            size_t smem = 16;
            for (size_t k = 0; k < fw.size(); k++) {
                boff_base[k] = boff.size();
                boff.insert(boff.end(), fw[k].p.block_off.begin(), fw[k].p.block_off.end());
                wide = wide || (int64_t)fw[k].p.num >= ((int64_t)1 << 31);
            }
            uint64_t *dboff = m.alloc<uint64_t>(boff.size() + 1);
            CK(cudaMemcpyAsync(dboff, boff.data(), boff.size() * 8, cudaMemcpyHostToDevice, st));
            std::vector<int> first_la(fw.size());
            for (size_t k = 0; k < fw.size(); k++) {
                const faz_config &c = cs[fw[k].idx];
                const Plan &p = fw[k].p;
                BatchField &f = bf[k];
                std::memset(&f, 0, sizeof(f));
                f.X = d_data[fw[k].idx];
                f.W = fw[k].W;
                f.codes = fw[k].codes;
                f.scratch = fw[k].scratch;
                f.eb = c.absErrorBound;
                f.recip = 1.0 / c.absErrorBound;
                f.radius = c.quantbinCnt / 2;
                f.trim = c.trimToZero;
                f.anchor = p.anchor ? 1 : 0;
                for (int a = 0; a < 3; a++) {
                    f.na[a] = p.na[a];
                    f.offs[a] = p.offs3[a];
                    f.step[a] = 1;
                }
                for (int a = 0; a < p.N; a++) f.step[3 - p.N + a] = (int64_t)p.maxStep;
                first_la[k] = (int)la.size();
                for (const LevelPlan &L : p.lv) {
                    LevelArgs a = L.args;
                    a.block_off = dboff + boff_base[k] + L.off_index;
                    a.ncodes = p.num;
                    a.err = nullptr;
                    a.verify = nullptr;
                    la.push_back(a);
                    smem = std::max(smem, level_smem_bytes<T>(a));
                }
            }
            // groups round by round: first points / anchors, then the coarsest
            // level of every field, the next level, ...
            std::vector<int> last(fw.size(), -1);
            size_t rounds = 0;
            for (auto &w : fw) rounds = std::max(rounds, w.p.lv.size());
            int64_t item = 0;
            for (size_t r = 0; r <= rounds; r++) {
                for (size_t k = 0; k < fw.size(); k++) {
                    BatchGroup g;
                    g.field = (int)k;
                    g.dep = last[k];
                    g.item0 = item;
                    if (r == 0) {
                        g.args = -1;
                        if (bf[k].anchor) {
                            const int64_t nan = bf[k].na[0] * bf[k].na[1] * bf[k].na[2];
                            g.kind = 1;
                            g.nitems = (nan + threads - 1) / threads;
                        } else {
                            g.kind = 0;
                            g.nitems = 1;
                        }
                    } else {
                        if (r - 1 >= fw[k].p.lv.size()) continue;
                        g.kind = 2;
                        g.args = first_la[k] + (int)(r - 1);
                        g.nitems = fw[k].p.lv[r - 1].nblocks;
                    }
                    if (g.nitems <= 0) continue;
                    if (g.nitems >= ((int64_t)1 << 31)) throw Fail{FAZ_ERR_UNSUPPORTED, "too many blocks in one level"};
                    last[k] = (int)groups.size();
                    groups.push_back(g);
                    item += g.nitems;
                }
            }
            BatchGroup *dg = m.alloc<BatchGroup>(groups.size());
            BatchField *dbf = m.alloc<BatchField>(bf.size());
            LevelArgs *dla = m.alloc<LevelArgs>(la.size() + 1);
            unsigned *done = m.alloc<unsigned>(groups.size());
            unsigned long long *counter = m.alloc<unsigned long long>(1);
            int *err = m.alloc<int>(1);
            CK(cudaMemcpyAsync(dg, groups.data(), groups.size() * sizeof(BatchGroup), cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(dbf, bf.data(), bf.size() * sizeof(BatchField), cudaMemcpyHostToDevice, st));
            if (!la.empty())
                CK(cudaMemcpyAsync(dla, la.data(), la.size() * sizeof(LevelArgs), cudaMemcpyHostToDevice, st));
            CK(cudaMemsetAsync(done, 0, groups.size() * 4, st));
            CK(cudaMemsetAsync(counter, 0, 8, st));
            CK(cudaMemsetAsync(err, 0, 4, st));
            int dev = 0, sms = 0;
            CK(cudaGetDevice(&dev));
            CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            const int occ = std::max(1, wide ? batch_occupancy<T, true>(threads, smem) : batch_occupancy<T, false>(threads, smem));
            const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(item, (int64_t)sms * occ));
            launches(launch_interp_batch<T>(dg, (int)groups.size(), dbf, dla, (uint64_t)item, counter, done, err, wide,
                                            (int)grid, threads, smem, st));
            int herr = 0;
            CK(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            if (herr) throw Fail{FAZ_ERR_DEVICE, "batched levels: an item waited too long for its previous level"};
        }
        CK(cudaEventRecord(ev_pred.b, st));
        CK(cudaStreamSynchronize(st));
        tm.predict_ms = ev_pred.ms();
        // Huffman, payload and zstd of each field on a pool of host threads
        std::atomic<size_t> next{0};
        std::vector<std::string> errs(fw.size());
        std::vector<int> codes_rc(fw.size(), 0);
        std::vector<faz_timings> tms(fw.size());
        std::vector<uint64_t> nl(fw.size(), 0);
        auto worker = [&]() {
            {
                const size_t k = next.fetch_add(1);
                if (k >= fw.size()) return;
                try {
                    std::memset(&tms[k], 0, sizeof(faz_timings));
                    StreamGuard s2(nullptr);
                    DevMem m2(s2.st);
                    Counter c2;
                    faz_config c = cs[fw[k].idx];
                    uint8_t *payload;
                    size_t psize;
                    interp_payload_tail<T>(c, fw[k].il, fw[k].dl, c.absErrorBound, c.quantbinCnt / 2, fw[k].p.num,
                                           fw[k].codes, fw[k].scratch, nullptr, m2, s2.st, c2, tms[k], nullptr,
                                           payload, psize);
                    // the same frames as a single-field call, compressed on this thread
                    finish_stream(c, payload, psize, &outs[fw[k].idx], &out_sizes[fw[k].idx], tms[k], false);
                    nl[k] = c2.n;
                } catch (const Fail &f) {
                    codes_rc[k] = f.code;
                    errs[k] = f.msg;
                } catch (const std::exception &e) {
                    codes_rc[k] = FAZ_ERR_ARG;
                    errs[k] = e.what();
                }
            }
        };
        {
            std::vector<std::function<void()>> tasks(fw.size(), worker);
            HostPool::get().run(tasks);
        }
        for (size_t k = 0; k < fw.size(); k++) {
            if (codes_rc[k]) throw Fail{codes_rc[k], errs[k]};
            launches.n += nl[k];
            tm.zstd_ms += tms[k].zstd_ms;
            tm.huffman_ms += tms[k].huffman_ms;
            tm.payload_bytes += tms[k].payload_bytes;
            tm.unpred_count += tms[k].unpred_count;
        }
        // the other fields, one by one
        for (int i : rest) {
            faz_config c = cs[i];
            uint8_t *payload;
            size_t psize;
            faz_timings t1;
            std::memset(&t1, 0, sizeof(t1));
            compress_dispatch<T>(c, (const T *)d_data[i], st, payload, psize, t1, launches);
            finish_stream(c, payload, psize, &outs[i], &out_sizes[i], t1);
            tm.zstd_ms += t1.zstd_ms;
            tm.payload_bytes += t1.payload_bytes;
        }
        tm.kernel_launches = launches.n;
    } catch (const Fail &f) {
        for (int i = 0; i < nf && outs; i++) {
            std::free(outs[i]);
            outs[i] = nullptr;
        }
        set_error(f.msg);
        return f.code;
    } catch (const std::exception &e) {
        for (int i = 0; i < nf && outs; i++) {
            std::free(outs[i]);
            outs[i] = nullptr;
        }
        set_error(e.what());
        return FAZ_ERR_ARG;
    }
    tm.total_ms = ms_since(t0);
    if (tmo) *tmo = tm;
    return FAZ_OK;
}

template <typename T>
void compress_omp(faz_config &c, const T *dX, cudaStream_t st, char **out, size_t *out_size, faz_timings &tm);

// slab: compress one slab of an OpenMP stream (its openmp flag is not acted on)
template <typename T>
int compress_impl(const faz_config *conf_in, const void *data, bool on_device, void *user_stream, char **out,
                  size_t *out_size, faz_timings *tmo, bool slab = false) {
    faz_timings tm;
    std::memset(&tm, 0, sizeof(tm));
    auto t0 = clk::now();
    try {
        if (!conf_in || !data || !out || !out_size) throw Fail{FAZ_ERR_ARG, "null argument"};
        faz_config c = *conf_in;
        check_config(c);
        init_pool_once();
        StreamGuard sg(user_stream, false, on_device ? NullStream::Default : NullStream::Library);
        cudaStream_t st = sg.st;
        Counter launches;
        Events ev_h2d, ev_gpu;
        const T *dX;
        DevMem m(st);
        if (!on_device) {
            T *tmp = m.alloc<T>(c.num);
            CK(cudaEventRecord(ev_h2d.a, st));
            CK(cudaMemcpyAsync(tmp, data, c.num * sizeof(T), cudaMemcpyHostToDevice, st));
            CK(cudaEventRecord(ev_h2d.b, st));
            dX = tmp;
        } else {
            dX = (const T *)data;
        }
        if (c.openmp && !slab) {
            CK(cudaStreamSynchronize(st));
            if (!on_device) tm.h2d_ms = ev_h2d.ms();
            compress_omp<T>(c, dX, st, out, out_size, tm);
        } else {
            uint8_t *payload;
            size_t psize;
            CK(cudaEventRecord(ev_gpu.a, st));
            compress_dispatch<T>(c, dX, st, payload, psize, tm, launches);
            CK(cudaEventRecord(ev_gpu.b, st));
            CK(cudaStreamSynchronize(st));
            if (!on_device) tm.h2d_ms = ev_h2d.ms();
            tm.gpu_ms = ev_gpu.ms();
            finish_stream(c, payload, psize, out, out_size, tm);
            tm.kernel_launches = launches.n;
        }
    } catch (const Fail &f) {
        set_error(f.msg);
        return f.code;
    } catch (const std::exception &e) {
        set_error(e.what());
        return FAZ_ERR_ARG;
    }
    tm.total_ms = ms_since(t0);
    if (tmo) *tmo = tm;
    return FAZ_OK;
}

// Slabs of an OpenMP stream: the reference runs one slab per OpenMP thread
// (omp_get_num_threads), so the count follows OMP_NUM_THREADS when it is set
// and the host's hardware threads otherwise, at most dims[0].
int omp_slab_count(uint64_t d0) {
    long n = 0;
    if (const char *e = std::getenv("OMP_NUM_THREADS")) n = std::strtol(e, nullptr, 10);
    if (n <= 0) n = (long)std::max(1u, std::thread::hardware_concurrency());
    if ((uint64_t)n > d0) n = (long)d0;
    return (int)n;
}

// slab t of nt along the slowest axis: rows [lo, hi) (SZImplOMP.hpp:44-46)
void omp_slab_rows(uint64_t d0, int t, int nt, uint64_t &lo, uint64_t &hi) {
    lo = (uint64_t)t * d0 / (uint64_t)nt;
    hi = (uint64_t)(t + 1) * d0 / (uint64_t)nt;
}

// the slab's Config: the field's, with Config::setDims of the slab's extents
// (include/QoZ/utils/Config.hpp:77-89)
faz_config omp_slab_config(const faz_config &c, uint64_t rows) {
    faz_config ct = c;
    ct.dims[0] = rows;
    ct.num = rows;
    for (int i = 1; i < c.N; i++) ct.num *= c.dims[i];
    ct.coeffs_num = ct.num;
    ct.coeffs_dims_len = c.N;
    for (int i = 0; i < c.N; i++) ct.coeffs_dims[i] = ct.dims[i];
    ct.blockSize = c.N == 1 ? 128 : (c.N == 2 ? 16 : 6);
    ct.pred_dim = c.N;
    ct.stride = ct.blockSize;
    return ct;
}

// SZ_compress_OMP (include/QoZ/api/impl/SZImplOMP.hpp:10-95): the error
// bound from the whole field's range, then every slab compressed as a field
// of its own; the stream is int nThreads, the slabs' Configs, their sizes
// (size_t each) and their compressed bytes, then the field's Config.
template <typename T>
void compress_omp(faz_config &c, const T *dX, cudaStream_t st, char **out, size_t *out_size, faz_timings &tm) {
    if (c.errorBoundMode != FAZ_EB_ABS && c.errorBoundMode != FAZ_EB_REL)
        throw Fail{FAZ_ERR_UNSUPPORTED, "OpenMP streams take the ABS or REL error bound mode"};
    Counter launches;
    if (c.errorBoundMode != FAZ_EB_ABS) resolve_eb<T>(c, dX, st, launches);
    const int nt = omp_slab_count(c.dims[0]);
    uint64_t base = 1;
    for (int i = 1; i < c.N; i++) base *= c.dims[i];
    std::vector<std::vector<uint8_t>> confs(nt), parts(nt);
    for (int t = 0; t < nt; t++) {
        uint64_t lo, hi;
        omp_slab_rows(c.dims[0], t, nt, lo, hi);
        const faz_config ct = omp_slab_config(c, hi - lo);
        char *so = nullptr;
        size_t ss = 0;
        faz_timings t2;
        std::memset(&t2, 0, sizeof(t2));
        const int rc = compress_impl<T>(&ct, dX + lo * base, true, st, &so, &ss, &t2, true);
        if (rc) throw Fail{rc, std::string("slab ") + std::to_string(t) + ": " + last_error()};
        int32_t cs;
        std::memcpy(&cs, so + ss - 4, 4);
        const size_t body = ss - 4 - (size_t)cs;
        parts[t].assign((const uint8_t *)so, (const uint8_t *)so + body);
        confs[t].assign((const uint8_t *)so + body, (const uint8_t *)so + body + cs);
        std::free(so);
        tm.gpu_ms += t2.gpu_ms;
        tm.zstd_ms += t2.zstd_ms;
        tm.host_ms += t2.host_ms;
        tm.payload_bytes += t2.payload_bytes;
        tm.unpred_count += t2.unpred_count;
        tm.kernel_launches += t2.kernel_launches;
    }
    std::vector<uint8_t> trailer;
    config_save(c, trailer);
    size_t total = 4 + 4 + trailer.size();
    for (int t = 0; t < nt; t++) total += confs[t].size() + 8 + parts[t].size();
    uint8_t *buf = (uint8_t *)std::malloc(total);
    if (!buf) throw Fail{FAZ_ERR_ARG, "out of host memory"};
    uint8_t *p = buf;
    const int32_t n32 = nt;
    std::memcpy(p, &n32, 4);
    p += 4;
    for (int t = 0; t < nt; t++) {
        std::memcpy(p, confs[t].data(), confs[t].size());
        p += confs[t].size();
    }
    for (int t = 0; t < nt; t++) {
        const uint64_t sz = parts[t].size();
        std::memcpy(p, &sz, 8);
        p += 8;
    }
    for (int t = 0; t < nt; t++) {
        std::memcpy(p, parts[t].data(), parts[t].size());
        p += parts[t].size();
    }
    std::memcpy(p, trailer.data(), trailer.size());
    p += trailer.size();
    const int32_t ts = (int32_t)trailer.size();
    std::memcpy(p, &ts, 4);
    p += 4;
    *out = (char *)buf;
    *out_size = (size_t)(p - buf);
    tm.kernel_launches += launches.n;
}

// -------------------------------------------------------------- decompress
struct Parsed {
    faz_config conf;
    int N;
    uint64_t dims[4];
    uint32_t blocksize;
    int32_t interp, dir, nlist, fixbs, trim, border;
    double alpha, beta, eb;
    uint64_t maxStep, cross;
    uint8_t bwt;
    std::vector<uint8_t> il, dl;
    int32_t radius;
    uint64_t nunpred;
    const uint8_t *unpred;
    DecodeTablesHost tables;
    uint64_t nbytes;
    const uint8_t *bits;
};

template <typename V>
V rd(const uint8_t *&p, const uint8_t *end) {
    if ((size_t)(end - p) < sizeof(V)) throw Fail{FAZ_ERR_FORMAT, "truncated stream header"};
    V v;
    std::memcpy(&v, p, sizeof(V));
    p += sizeof(V);
    return v;
}

// SZInterpolationCompressor::decompress header reads (lines 53-88),
// LinearQuantizer::load (IntegerQuantizer.hpp:203-226), HuffmanEncoder::load.
void parse_payload(const uint8_t *pl, size_t n, int N, Parsed &P) {
    const uint8_t *p = pl, *end = pl + n;
    P.N = N;
    for (int i = 0; i < N; i++) P.dims[i] = rd<uint64_t>(p, end);
    P.blocksize = rd<uint32_t>(p, end);
    P.interp = rd<int32_t>(p, end);
    P.dir = rd<int32_t>(p, end);
    P.alpha = rd<double>(p, end);
    P.beta = rd<double>(p, end);
    P.maxStep = rd<uint64_t>(p, end);
    P.nlist = rd<int32_t>(p, end);
    P.bwt = rd<uint8_t>(p, end);
    P.fixbs = rd<int32_t>(p, end);
    P.cross = rd<uint64_t>(p, end);
    P.trim = rd<int32_t>(p, end);
    P.border = rd<int32_t>(p, end);
    if (P.bwt) {
        // decompress_block (lines 233-239): one interpolator and direction per
        // block and level; the level lists are not read
        const uint64_t nops = rd<uint64_t>(p, end);
        if ((size_t)(end - p) / 2 < nops) throw Fail{FAZ_ERR_FORMAT, "truncated block-wise choices"};
        P.il.assign(p, p + nops);
        p += nops;
        P.dl.assign(p, p + nops);
        p += nops;
        P.nlist = 0;
    } else {
        if (P.nlist < 0 || P.nlist > FAZ_MAX_LEVELS) throw Fail{FAZ_ERR_FORMAT, "bad level list length"};
        if ((size_t)(end - p) < (size_t)2 * P.nlist) throw Fail{FAZ_ERR_FORMAT, "truncated level lists"};
        P.il.assign(p, p + P.nlist);
        p += P.nlist;
        P.dl.assign(p, p + P.nlist);
        p += P.nlist;
    }
    rd<uint8_t>(p, end);
    P.eb = rd<double>(p, end);
    P.radius = rd<int32_t>(p, end);
    P.nunpred = rd<uint64_t>(p, end);
    P.unpred = p;
}

}  // namespace

// HuffmanEncoder::load + decode (HuffmanEncoder.hpp:236-296) on the device:
// reads the tree and bit string at p (advancing it) and writes num codes.
template <typename C>
void huffman_decode_impl(const uint8_t *&p, const uint8_t *end, uint64_t num, C *codes, DevMem &m, cudaStream_t st,
                         Counter &launches) {
    DecodeTablesHost t;
    std::string err;
    int rc = parse_tree(p, end, t, err);
    if (rc) throw Fail{rc, err};
    if ((size_t)(end - p) < 8) throw Fail{FAZ_ERR_FORMAT, "truncated stream header"};
    uint64_t nbytes;
    std::memcpy(&nbytes, p, 8);
    p += 8;
    if ((size_t)(end - p) < nbytes) throw Fail{FAZ_ERR_FORMAT, "truncated Huffman bits"};
    const uint8_t *hbits = p;
    p += nbytes;
    if (t.constant || nbytes == 0) {
        int v = t.constant_state + t.offset;
        if (v < 0 || (sizeof(C) == 2 && v > 65535)) throw Fail{FAZ_ERR_FORMAT, "Huffman symbol out of range"};
        launches(launch_fill_u16(codes, num, (C)v, st));
        return;
    }
    const uint64_t nwords = (nbytes + 3) / 4;
    uint32_t *dbits = m.alloc<uint32_t>(nwords + 16);
    CK(cudaMemsetAsync(dbits, 0, (nwords + 16) * 4, st));
    uint32_t *lut = m.alloc<uint32_t>(t.lut.size());
    uint32_t *dl = m.alloc<uint32_t>(t.nodeCount), *dr = m.alloc<uint32_t>(t.nodeCount);
    int32_t *ds = m.alloc<int32_t>(t.nodeCount);
    uint8_t *dleaf = m.alloc<uint8_t>(t.nodeCount);
    CK(cudaMemcpyAsync(lut, t.lut.data(), t.lut.size() * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dl, t.left.data(), t.nodeCount * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dr, t.right.data(), t.nodeCount * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ds, t.sym.data(), t.nodeCount * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dleaf, t.leaf.data(), t.nodeCount, cudaMemcpyHostToDevice, st));
    DecodeTablesDev td{lut, dl, dr, ds, dleaf};
    const uint64_t nbits = nbytes * 8;
    const uint64_t nunits = decode_units(nbits);
    uint64_t *start = m.alloc<uint64_t>(nunits);
    uint64_t *ea = m.alloc<uint64_t>(nunits), *eb2 = m.alloc<uint64_t>(nunits);
    unsigned int *cnt = m.alloc<unsigned int>(nunits);
    uint16_t *bnd = m.alloc<uint16_t>(nunits * decode_boundaries());
    unsigned long long *cnt64 = m.alloc<unsigned long long>(nunits + 1);
    unsigned long long *off = m.alloc<unsigned long long>(nunits + 1);
    unsigned long long *dtmp = m.alloc<unsigned long long>(scan_temp_words(nunits) + 1);
    int *flags = m.alloc<int>(2);  // [0] changed, [1] damaged tree
    CK(cudaMemsetAsync(flags, 0, 8, st));
    launches(launch_init_starts(start, nunits, st));
    // The bit string comes over in slices on a copy stream while the
    // speculative decode of the slices already in runs (a unit reads up to 8
    // words past its CTA's units: each slice's copy carries the next slice's
    // first 128 bytes).
    {
        const uint64_t cta = decode_cta_units();
        const uint64_t unit_bytes = decode_unit_bits() / 8;
        // four slices of a bit string of 16 MB or more: each decode launch
        // still fills the GPU, three quarters of the copy overlap decoding
        const uint64_t nslices0 = nbytes >= (16u << 20) ? 4 : 1;
        const uint64_t slice_units = ((nunits + nslices0 - 1) / nslices0 + cta - 1) / cta * cta;
        const uint64_t nslices = (nunits + slice_units - 1) / slice_units;
        if (nslices <= 1) {
            CK(cudaMemcpyAsync(dbits, hbits, nbytes, cudaMemcpyHostToDevice, st));
            launches(launch_decode_spec(td, dbits, nwords, nbits, nunits, 0, nunits, ea, cnt, bnd, flags + 1, st));
        } else {
            StreamGuard cs(nullptr);
            Events ready;
            CK(cudaEventRecord(ready.a, st));  // dbits cleared
            CK(cudaStreamWaitEvent(cs.st, ready.a, 0));
            std::vector<cudaEvent_t> done(nslices, nullptr);
            try {
                for (uint64_t k = 0; k < nslices; k++) {
                    CK(cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming));
                    const uint64_t b0 = k * slice_units * unit_bytes;
                    const uint64_t b1 = std::min<uint64_t>(nbytes, (k + 1) * slice_units * unit_bytes + 128);
                    CK(cudaMemcpyAsync((uint8_t *)dbits + b0, hbits + b0, b1 - b0, cudaMemcpyHostToDevice, cs.st));
                    CK(cudaEventRecord(done[k], cs.st));
                    CK(cudaStreamWaitEvent(st, done[k], 0));
                    launches(launch_decode_spec(td, dbits, nwords, nbits, nunits, k * slice_units,
                                                (k + 1) * slice_units, ea, cnt, bnd, flags + 1, st));
                }
            } catch (...) {
                cudaStreamSynchronize(cs.st);
                for (cudaEvent_t e : done)
                    if (e) cudaEventDestroy(e);
                throw;
            }
            // the copy stream's work is ordered before st's next launch; the
            // events go once it has finished
            CK(cudaStreamSynchronize(cs.st));
            for (cudaEvent_t e : done) cudaEventDestroy(e);
        }
    }
    int *hflag = (int *)t_pin_small.get(64);
    bool converged = false;
    for (int it = 0; it < 1024; it++) {
        CK(cudaMemsetAsync(flags, 0, 4, st));
        launches(launch_decode_resync(td, dbits, nwords, nbits, nunits, ea, eb2, cnt, bnd, start, flags, st));
        CK(cudaMemcpyAsync(hflag, flags, 8, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        std::swap(ea, eb2);
        if (hflag[0] < 0 || hflag[1]) throw Fail{FAZ_ERR_FORMAT, "Huffman stream decodes outside the tree"};
        if (hflag[0] == 0) {
            converged = true;
            break;
        }
    }
    if (!converged) throw Fail{FAZ_ERR_UNSUPPORTED, "Huffman stream did not synchronise within 1024 passes"};
    launches(launch_widen_counts(cnt, cnt64, nunits, st));
    launches(launch_scan_u64(cnt64, off, nunits, dtmp, st));
    uint64_t total;
    CK(cudaMemcpyAsync(hflag, off + nunits, 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::memcpy(&total, hflag, 8);
    if (total < num) throw Fail{FAZ_ERR_FORMAT, "Huffman stream holds fewer symbols than the field"};
    launches(launch_decode_write(td, dbits, nwords, nbits, nunits, start, off, num, t.offset, codes, st));
}

void huffman_decode_device(const uint8_t *&p, const uint8_t *end, uint64_t num, uint16_t *codes, DevMem &m,
                           cudaStream_t st, Counter &launches) {
    huffman_decode_impl(p, end, num, codes, m, st, launches);
}
void huffman_decode_device(const uint8_t *&p, const uint8_t *end, uint64_t num, uint32_t *codes, DevMem &m,
                           cudaStream_t st, Counter &launches) {
    huffman_decode_impl(p, end, num, codes, m, st, launches);
}

// Sorted positions of the zero codes (the unpredictable points); returns
// their count.
template <typename C>
uint64_t zero_positions_impl(const C *codes, uint64_t num, DevMem &m, cudaStream_t st, Counter &launches,
                             uint64_t *&zpos) {
    const uint64_t nsub = hist_subchunks(num);
    unsigned long long *zc = m.alloc<unsigned long long>(nsub + 1);
    unsigned long long *zoff = m.alloc<unsigned long long>(nsub + 1);
    unsigned long long *ztmp = m.alloc<unsigned long long>(scan_temp_words(nsub) + 1);
    launches(launch_count_zeros(codes, num, zc, st));
    launches(launch_scan_u64(zc, zoff, nsub, ztmp, st));
    uint64_t *hz = (uint64_t *)t_pin_small.get(64);
    CK(cudaMemcpyAsync(hz, zoff + nsub, 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const uint64_t nz = *hz;
    zpos = m.alloc<uint64_t>(nz ? nz : 1);
    if (nz) launches(launch_compact_zeros<float>(codes, num, zc, zoff, zpos, nullptr, nullptr, st));
    return nz;
}
uint64_t zero_positions(const uint16_t *codes, uint64_t num, DevMem &m, cudaStream_t st, Counter &launches,
                        uint64_t *&zpos) {
    return zero_positions_impl(codes, num, m, st, launches, zpos);
}
uint64_t zero_positions(const uint32_t *codes, uint64_t num, DevMem &m, cudaStream_t st, Counter &launches,
                        uint64_t *&zpos) {
    return zero_positions_impl(codes, num, m, st, launches, zpos);
}

namespace {

template <typename T>
void decompress_device(const uint8_t *pl, size_t n, Parsed &P, T *dOut, cudaStream_t st, faz_timings &tm,
                       Counter &launches) {
    const uint8_t *end = pl + n;
    const uint8_t *p = P.unpred;
    if ((size_t)(end - p) / sizeof(T) < P.nunpred) throw Fail{FAZ_ERR_FORMAT, "truncated unpredictable values"};
    p += P.nunpred * sizeof(T);
    if (!(P.eb > 0)) throw Fail{FAZ_ERR_FORMAT, "bad error bound"};
    if (P.bwt || (P.fixbs > 0 && P.N <= 3 && !fixbs_aligned(P.N, P.dims, P.maxStep, P.fixbs))) {
        // decompress_block, or blocks of fixBlockSize off the coarse lattice
        if (P.bwt && P.N != 3) throw Fail{FAZ_ERR_UNSUPPORTED, "block-wise tuned streams are implemented for 3-D data"};
        if (P.cross || P.border)
            throw Fail{FAZ_ERR_UNSUPPORTED, "streams with crossBlock or another block order are not implemented"};
        uint64_t num = 1;
        for (int i = 0; i < P.N; i++) num *= P.dims[i];
        DevMem m(st);
        uint16_t *codes = m.alloc<uint16_t>(num);
        T *dunpred = m.alloc<T>(P.nunpred ? P.nunpred : 1);
        if (P.nunpred) CK(cudaMemcpyAsync(dunpred, P.unpred, P.nunpred * sizeof(T), cudaMemcpyHostToDevice, st));
        Events ev_dec, ev_pred;
        CK(cudaEventRecord(ev_dec.a, st));
        huffman_decode_device(p, end, num, codes, m, st, launches);
        uint64_t *zpos = nullptr;
        const uint64_t nz = zero_positions(codes, num, m, st, launches, zpos);
        if (nz != P.nunpred) throw Fail{FAZ_ERR_FORMAT, "unpredictable count does not match the zero codes"};
        CK(cudaEventRecord(ev_dec.b, st));
        CK(cudaEventRecord(ev_pred.a, st));
        static const std::vector<uint8_t> none;
        blocked_decompress_levels<T>(P.N, P.dims, P.maxStep, P.bwt ? (int)P.blocksize : P.fixbs, P.eb, P.alpha, P.beta,
                                     P.radius, P.trim, P.interp, P.dir, P.bwt ? none : P.il, P.bwt ? none : P.dl,
                                     P.bwt ? P.il : none, P.bwt ? P.dl : none, P.bwt != 0, codes, zpos, nz, dunpred,
                                     dOut, m, st, launches);
        CK(cudaEventRecord(ev_pred.b, st));
        tm.huffman_ms = ev_dec.ms();
        tm.predict_ms = ev_pred.ms();
        return;
    }
    if (P.N == 4) {
        if (P.cross || P.border)
            throw Fail{FAZ_ERR_UNSUPPORTED, "streams with crossBlock or another block order are not implemented"};
        uint64_t num = 1;
        for (int i = 0; i < 4; i++) num *= P.dims[i];
        DevMem m(st);
        uint16_t *codes = m.alloc<uint16_t>(num);
        T *dunpred = m.alloc<T>(P.nunpred ? P.nunpred : 1);
        if (P.nunpred) CK(cudaMemcpyAsync(dunpred, P.unpred, P.nunpred * sizeof(T), cudaMemcpyHostToDevice, st));
        Events ev_dec, ev_pred;
        CK(cudaEventRecord(ev_dec.a, st));
        huffman_decode_device(p, end, num, codes, m, st, launches);
        uint64_t *zpos = nullptr;
        const uint64_t nz = zero_positions(codes, num, m, st, launches, zpos);
        if (nz != P.nunpred) throw Fail{FAZ_ERR_FORMAT, "unpredictable count does not match the zero codes"};
        CK(cudaEventRecord(ev_dec.b, st));
        unsigned long long *vcount = nullptr;
        if (verify_fast_path()) {
            vcount = m.alloc<unsigned long long>(1);
            CK(cudaMemsetAsync(vcount, 0, 8, st));
        }
        CK(cudaEventRecord(ev_pred.a, st));
        interp4_decompress<T>(P.dims, P.maxStep, (int)P.blocksize, P.fixbs, P.interp, P.dir, P.il, P.dl, P.eb, P.alpha,
                              P.beta, P.radius, P.trim, codes, zpos, nz, dunpred, dOut, vcount, m, st, launches);
        CK(cudaEventRecord(ev_pred.b, st));
        CK(cudaStreamSynchronize(st));
        if (vcount) {
            unsigned long long vc = 0;
            CK(cudaMemcpy(&vc, vcount, 8, cudaMemcpyDeviceToHost));
            if (vc) throw Fail{FAZ_ERR_DEVICE, "float fast path disagreed with the double path at " + std::to_string(vc) + " points"};
        }
        tm.huffman_ms = ev_dec.ms();
        tm.predict_ms = ev_pred.ms();
        return;
    }
    Plan pl_ = make_plan<T>(P.N, P.dims, P.maxStep, (int)P.blocksize, P.fixbs, P.interp, P.dir, P.il, P.dl, P.eb, P.alpha,
                            P.beta, P.radius, P.trim, smem_limit());
    const uint64_t num = pl_.num;
    DevMem m(st);
    uint16_t *codes = m.alloc<uint16_t>(num);
    T *dunpred = m.alloc<T>(P.nunpred ? P.nunpred : 1);
    if (P.nunpred) CK(cudaMemcpyAsync(dunpred, P.unpred, P.nunpred * sizeof(T), cudaMemcpyHostToDevice, st));
    Events ev_dec, ev_pred, ev_fin;
    CK(cudaEventRecord(ev_dec.a, st));
    huffman_decode_device(p, end, num, codes, m, st, launches);
    CK(cudaEventRecord(ev_dec.b, st));
    // zero positions for the unpredictable values
    uint64_t *zpos = nullptr;
    const uint64_t nz = zero_positions(codes, num, m, st, launches, zpos);
    if (nz != P.nunpred)
        throw Fail{FAZ_ERR_FORMAT, "unpredictable count does not match the zero codes"};
    if (!pl_.anchor) {
        launches(launch_first_point<T>(true, nullptr, dOut, codes, nullptr, P.eb, P.radius, P.trim, zpos, nz, dunpred, st));
    } else {
        int64_t step[3] = {1, 1, 1};
        int e = 3 - pl_.N;
        for (int i = 0; i < pl_.N; i++) step[e + i] = (int64_t)pl_.maxStep;
        launches(launch_anchors<T>(true, nullptr, dOut, codes, nullptr, dunpred, pl_.na, step, pl_.offs3, st));
    }
    uint64_t *boff = m.alloc<uint64_t>(pl_.block_off.size());
    CK(cudaMemcpyAsync(boff, pl_.block_off.data(), pl_.block_off.size() * 8, cudaMemcpyHostToDevice, st));
    int *kerr = m.alloc<int>(1);
    CK(cudaMemsetAsync(kerr, 0, 4, st));
    unsigned long long *vcount = nullptr;
    if (verify_fast_path()) {
        vcount = m.alloc<unsigned long long>(1);
        CK(cudaMemsetAsync(vcount, 0, 8, st));
    }
    CK(cudaEventRecord(ev_pred.a, st));
    for (size_t li = 0; li < pl_.lv.size(); li++) {
        const LevelPlan &L = pl_.lv[li];
        LevelArgs a = L.args;
        a.block_off = boff + L.off_index;
        a.ncodes = num;
        a.err = kerr;
        a.verify = vcount;
        if (li + 1 == pl_.lv.size()) CK(cudaEventRecord(ev_fin.a, st));
        int nl = 0;
        CK(launch_level<T>(a, L.nblocks, true, nullptr, dOut, codes, nullptr, zpos, nz, dunpred, st, &nl));
        launches.n += nl;
    }
    CK(cudaEventRecord(ev_fin.b, st));
    CK(cudaEventRecord(ev_pred.b, st));
    int *hk = (int *)t_pin_small.get(64);
    CK(cudaMemcpyAsync(hk, kerr, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (*hk) throw Fail{FAZ_ERR_DEVICE, "level kernel met an out-of-range stream position"};
    if (vcount) {
        unsigned long long vc = 0;
        CK(cudaMemcpy(&vc, vcount, 8, cudaMemcpyDeviceToHost));
        if (vc) throw Fail{FAZ_ERR_DEVICE, "float fast path disagreed with the double path at " + std::to_string(vc) + " points"};
    }
    tm.huffman_ms = ev_dec.ms();
    tm.predict_ms = ev_pred.ms();
    tm.finest_level_ms = pl_.lv.empty() ? 0.0 : ev_fin.ms();
}

// Split a stream into trailer config and zstd-decompressed payload (pinned).
void open_stream(const char *cmp, size_t cmp_size, faz_config &conf, uint8_t *&payload, size_t &psize,
                 faz_timings &tm) {
    if (!cmp || cmp_size < 4) throw Fail{FAZ_ERR_FORMAT, "stream too short"};
    int32_t cs;
    std::memcpy(&cs, cmp + cmp_size - 4, 4);
    if (cs <= 0 || (size_t)cs + 4 > cmp_size) throw Fail{FAZ_ERR_FORMAT, "bad trailer size"};
    int rc = config_load(conf, (const uint8_t *)cmp + cmp_size - 4 - cs, (size_t)cs);
    if (rc) throw Fail{rc, "bad stream trailer"};
    size_t body = cmp_size - 4 - cs;
    if (body < 8) throw Fail{FAZ_ERR_FORMAT, "stream too short"};
    uint64_t raw;
    std::memcpy(&raw, cmp, 8);
    std::string err;
    const Zstd &z = zstd_lib(err);
    if (!z.ok) throw Fail{FAZ_ERR_ZSTD, err};
    if (raw > ((uint64_t)1 << 46)) throw Fail{FAZ_ERR_FORMAT, "implausible payload size"};
    payload = t_pin_payload.get(raw + 64);
    auto t0 = clk::now();
    size_t got = zstd_decompress_frames(z, payload, raw, (const uint8_t *)cmp + 8, body - 8, zstd_threads());
    tm.zstd_ms += ms_since(t0);
    if (z.isError(got) || got != raw) throw Fail{FAZ_ERR_ZSTD, "ZSTD_decompress failed"};
    psize = raw;
}

template <typename T>
void decompress_omp(const faz_config &c, const char *cmp, size_t cmp_size, T *dOut, cudaStream_t st,
                    faz_timings &tm);

// slab: decompress one slab of an OpenMP stream (its openmp flag is not acted on)
template <typename T>
int decompress_impl(faz_config *conf_io, const char *cmp, size_t cmp_size, void **out, bool on_device, void *dOutUser,
                    void *user_stream, faz_timings *tmo, bool slab = false) {
    faz_timings tm;
    std::memset(&tm, 0, sizeof(tm));
    auto t0 = clk::now();
    try {
        if (!conf_io) throw Fail{FAZ_ERR_ARG, "null config"};
        if (!slab) {
            // an OpenMP stream (SZ_decompress_OMP, include/QoZ/api/impl/SZImplOMP.hpp:97-149)
            faz_config oc;
            if (!cmp || cmp_size < 4) throw Fail{FAZ_ERR_FORMAT, "stream too short"};
            int32_t cs;
            std::memcpy(&cs, cmp + cmp_size - 4, 4);
            if (cs <= 0 || (size_t)cs + 4 > cmp_size) throw Fail{FAZ_ERR_FORMAT, "bad trailer size"};
            if (config_load(oc, (const uint8_t *)cmp + cmp_size - 4 - cs, (size_t)cs)) throw Fail{FAZ_ERR_FORMAT, "bad stream trailer"};
            if (oc.openmp) {
                if (oc.N == 4) throw Fail{FAZ_ERR_UNSUPPORTED, "4-D fields are not implemented on the GPU path"};
                const bool caller_buffer = on_device || (out && *out);
                if (caller_buffer && conf_io->num < oc.num)
                    throw Fail{FAZ_ERR_ARG, "output buffer holds fewer values than the stream's field"};
                init_pool_once();
                StreamGuard sg(user_stream, false, on_device ? NullStream::Default : NullStream::Library);
                DevMem m(sg.st);
                T *dOut = on_device ? (T *)dOutUser : m.alloc<T>(oc.num);
                if (!dOut) throw Fail{FAZ_ERR_ARG, "null output"};
                decompress_omp<T>(oc, cmp, cmp_size - 4 - (size_t)cs, dOut, sg.st, tm);
                if (!on_device) {
                    if (!out) throw Fail{FAZ_ERR_ARG, "null output"};
                    const bool alloc = *out == nullptr;
                    T *h = alloc ? (T *)std::malloc(oc.num * sizeof(T)) : (T *)*out;
                    if (!h) throw Fail{FAZ_ERR_ARG, "out of host memory"};
                    Events ev_d2h;
                    CK(cudaEventRecord(ev_d2h.a, sg.st));
                    cudaError_t e = cudaMemcpyAsync(h, dOut, oc.num * sizeof(T), cudaMemcpyDeviceToHost, sg.st);
                    if (e == cudaSuccess) e = cudaEventRecord(ev_d2h.b, sg.st);
                    if (e == cudaSuccess) e = cudaStreamSynchronize(sg.st);
                    if (e != cudaSuccess) {
                        if (alloc) std::free(h);
                        throw Fail{FAZ_ERR_CUDA, std::string("device to host copy: ") + cudaGetErrorString(e)};
                    }
                    tm.d2h_ms = ev_d2h.ms();
                    *out = h;
                } else {
                    CK(cudaStreamSynchronize(sg.st));
                }
                *conf_io = oc;
                tm.total_ms = ms_since(t0);
                if (tmo) *tmo = tm;
                return FAZ_OK;
            }
        }
        // a caller-provided output holds conf->num values
        const uint64_t cap = conf_io->num;
        const bool caller_buffer = on_device || (out && *out);
        faz_config c;
        uint8_t *payload;
        size_t psize;
        open_stream(cmp, cmp_size, c, payload, psize, tm);
        // SZ_decompress_dispatcher (include/QoZ/api/impl/SZDispatcher.hpp:41-52)
        const bool lor = c.cmprAlgo == FAZ_ALGO_LORENZO_REG;
        if (!lor && c.cmprAlgo != FAZ_ALGO_INTERP)
            throw Fail{FAZ_ERR_UNSUPPORTED, "stream algorithm is neither ALGO_INTERP nor ALGO_LORENZO_REG"};
        if (lor && (c.regression2 || c.N > 3))
            throw Fail{FAZ_ERR_UNSUPPORTED, "ALGO_LORENZO_REG streams are implemented for 1-D, 2-D and 3-D data "
                                            "without regression2"};
        if (c.wavelet != 0) throw Fail{FAZ_ERR_UNSUPPORTED, "wavelet streams are not part of the interpolation path"};
        if (caller_buffer && cap < c.num)
            throw Fail{FAZ_ERR_ARG, "output buffer holds fewer values than the stream's field"};
        Parsed P;
        P.conf = c;
        P.nlist = 0;
        P.nunpred = 0;
        if (!lor) {
            parse_payload(payload, psize, c.N, P);
            for (int i = 0; i < c.N; i++)
                if (P.dims[i] != c.dims[i]) throw Fail{FAZ_ERR_FORMAT, "header dims differ from trailer dims"};
        }
        init_pool_once();
        StreamGuard sg(user_stream, false, on_device ? NullStream::Default : NullStream::Library);
        cudaStream_t st = sg.st;
        Counter launches;
        Events ev_gpu, ev_d2h;
        DevMem m(st);
        T *dOut;
        if (on_device) {
            if (!dOutUser) throw Fail{FAZ_ERR_ARG, "null output"};
            dOut = (T *)dOutUser;
        } else {
            if (!out) throw Fail{FAZ_ERR_ARG, "null output"};
            dOut = m.alloc<T>(c.num);
        }
        CK(cudaEventRecord(ev_gpu.a, st));
        if (lor && c.N < 3)
            gen_decompress<T>(c.N, payload, psize, c.dims, c.lorenzo, c.lorenzo2, c.regression, dOut, st, launches, tm);
        else if (lor) lorenzo3_decompress<T>(payload, psize, c.dims, dOut, st, launches, tm);
        else decompress_device<T>(payload, psize, P, dOut, st, tm, launches);
        CK(cudaEventRecord(ev_gpu.b, st));
        if (!on_device) {
            bool alloc = *out == nullptr;
            T *h = alloc ? (T *)std::malloc(c.num * sizeof(T)) : (T *)*out;
            if (!h) throw Fail{FAZ_ERR_ARG, "out of host memory"};
            CK(cudaEventRecord(ev_d2h.a, st));
            cudaError_t e = cudaMemcpyAsync(h, dOut, c.num * sizeof(T), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaEventRecord(ev_d2h.b, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) {
                if (alloc) std::free(h);
                throw Fail{FAZ_ERR_CUDA, std::string("device to host copy: ") + cudaGetErrorString(e)};
            }
            tm.d2h_ms = ev_d2h.ms();
            *out = h;
        } else {
            CK(cudaStreamSynchronize(st));
        }
        tm.gpu_ms = ev_gpu.ms();
        tm.payload_bytes = psize;
        tm.unpred_count = P.nunpred;
        tm.kernel_launches = launches.n;
        *conf_io = c;
        if (!lor) conf_io->interp_list_len = P.nlist;
        for (int i = 0; i < P.nlist; i++) {
            conf_io->interpAlgo_list[i] = P.il[i];
            conf_io->interpDirection_list[i] = P.dl[i];
        }
    } catch (const Fail &f) {
        set_error(f.msg);
        return f.code;
    } catch (const std::exception &e) {
        set_error(e.what());
        return FAZ_ERR_ARG;
    }
    tm.total_ms = ms_since(t0);
    if (tmo) *tmo = tm;
    return FAZ_OK;
}

// SZ_decompress_OMP: nThreads, the slabs' Configs and sizes, then every slab
// decompressed as a field of its own into its rows of dOut.  body: the
// stream's bytes before the field's Config.
template <typename T>
void decompress_omp(const faz_config &c, const char *cmp, size_t body, T *dOut, cudaStream_t st, faz_timings &tm) {
    const uint8_t *p = (const uint8_t *)cmp, *end = p + body;
    if (body < 4) throw Fail{FAZ_ERR_FORMAT, "truncated OpenMP stream"};
    int32_t nt;
    std::memcpy(&nt, p, 4);
    p += 4;
    if (nt < 1 || (uint64_t)nt > c.dims[0]) throw Fail{FAZ_ERR_FORMAT, "bad OpenMP slab count"};
    std::vector<const uint8_t *> cp(nt);
    std::vector<size_t> cl(nt);
    for (int t = 0; t < nt; t++) {
        faz_config ct;
        size_t used = 0;
        if (config_load(ct, p, (size_t)(end - p), &used)) throw Fail{FAZ_ERR_FORMAT, "bad slab Config"};
        cp[t] = p;
        cl[t] = used;
        p += used;
    }
    if ((size_t)(end - p) < (size_t)nt * 8) throw Fail{FAZ_ERR_FORMAT, "truncated OpenMP stream"};
    std::vector<uint64_t> sz(nt);
    for (int t = 0; t < nt; t++) {
        std::memcpy(&sz[t], p, 8);
        p += 8;
    }
    uint64_t base = 1;
    for (int i = 1; i < c.N; i++) base *= c.dims[i];
    std::vector<uint8_t> one;
    for (int t = 0; t < nt; t++) {
        if ((uint64_t)(end - p) < sz[t]) throw Fail{FAZ_ERR_FORMAT, "truncated OpenMP slab"};
        uint64_t lo, hi;
        omp_slab_rows(c.dims[0], t, nt, lo, hi);
        // the slab as a stream of its own: its bytes, its Config, the Config's size
        one.assign(p, p + sz[t]);
        one.insert(one.end(), cp[t], cp[t] + cl[t]);
        const int32_t cs = (int32_t)cl[t];
        one.insert(one.end(), (const uint8_t *)&cs, (const uint8_t *)&cs + 4);
        p += sz[t];
        faz_config ct;
        std::memset(&ct, 0, sizeof(ct));
        ct.num = (hi - lo) * base;
        faz_timings t2;
        std::memset(&t2, 0, sizeof(t2));
        const int rc = decompress_impl<T>(&ct, (const char *)one.data(), one.size(), nullptr, true, dOut + lo * base, st,
                                          &t2, true);
        if (rc) throw Fail{rc, std::string("slab ") + std::to_string(t) + ": " + last_error()};
        if (ct.num != (hi - lo) * base) throw Fail{FAZ_ERR_FORMAT, "slab extents differ from the field's split"};
        tm.gpu_ms += t2.gpu_ms;
        tm.zstd_ms += t2.zstd_ms;
        tm.payload_bytes += t2.payload_bytes;
        tm.unpred_count += t2.unpred_count;
        tm.kernel_launches += t2.kernel_launches;
    }
}

template <typename T>
int decompress_payload_impl(int N, const char *payload, size_t psize, void *d_out, uint64_t cap, void *user_stream,
                            faz_timings *tmo) {
    faz_timings tm;
    std::memset(&tm, 0, sizeof(tm));
    auto t0 = clk::now();
    try {
        if (N < 1 || N > 4) throw Fail{FAZ_ERR_ARG, "N must be 1..4"};
        if (!payload || !d_out) throw Fail{FAZ_ERR_ARG, "null argument"};
        Parsed P;
        std::memset(&P.conf, 0, sizeof(P.conf));
        parse_payload((const uint8_t *)payload, psize, N, P);
        uint64_t num = 1;
        for (int i = 0; i < N; i++) num *= P.dims[i];
        if (cap < num) throw Fail{FAZ_ERR_ARG, "output buffer holds fewer values than the payload's field"};
        init_pool_once();
        StreamGuard sg(user_stream, false, NullStream::Default);
        Counter launches;
        Events ev_gpu;
        CK(cudaEventRecord(ev_gpu.a, sg.st));
        decompress_device<T>((const uint8_t *)payload, psize, P, (T *)d_out, sg.st, tm, launches);
        CK(cudaEventRecord(ev_gpu.b, sg.st));
        CK(cudaStreamSynchronize(sg.st));
        tm.gpu_ms = ev_gpu.ms();
        tm.payload_bytes = psize;
        tm.unpred_count = P.nunpred;
        tm.kernel_launches = launches.n;
    } catch (const Fail &f) {
        set_error(f.msg);
        return f.code;
    } catch (const std::exception &e) {
        set_error(e.what());
        return FAZ_ERR_ARG;
    }
    tm.total_ms = ms_since(t0);
    if (tmo) *tmo = tm;
    return FAZ_OK;
}

template <typename T>
int tune_impl(faz_config *conf, const void *d_data, void *user_stream, faz_timings *tmo) {
    faz_timings tm;
    std::memset(&tm, 0, sizeof(tm));
    auto t0 = clk::now();
    try {
        if (!conf || !d_data) throw Fail{FAZ_ERR_ARG, "null argument"};
        faz_config c = *conf;
        check_config(c);
        init_pool_once();
        StreamGuard sg(user_stream, false, NullStream::Default);
        Counter launches;
        const T *dX = (const T *)d_data;
        resolve_eb<T>(c, dX, sg.st, launches);
        if (!(c.absErrorBound > 0) || !std::isfinite(c.absErrorBound))
            throw Fail{FAZ_ERR_ARG, "error bound must be positive and finite"};
        auto tt = clk::now();
        if (c.cmprAlgo == FAZ_ALGO_INTERP_LORENZO && qoz_tuned(c)) {
            qoz_tune_device<T>(c, dX, sg.st, launches, tm);
        } else if (c.cmprAlgo == FAZ_ALGO_INTERP_LORENZO) {
            faz_timings t2;
            std::memset(&t2, 0, sizeof(t2));
            sz3_tune_device<T>(c, dX, sg.st, launches, t2, {});
        }
        CK(cudaStreamSynchronize(sg.st));
        tm.tune_ms = ms_since(tt);
        tm.kernel_launches = launches.n;
        *conf = c;
    } catch (const Fail &f) {
        set_error(f.msg);
        return f.code;
    } catch (const std::exception &e) {
        set_error(e.what());
        return FAZ_ERR_ARG;
    }
    tm.total_ms = ms_since(t0);
    if (tmo) *tmo = tm;
    return FAZ_OK;
}

template <typename T>
int features_impl(const faz_config *conf, const void *d_data, void *user_stream, float *dF) {
    try {
        if (!conf || !d_data || !dF) throw Fail{FAZ_ERR_ARG, "null argument"};
        faz_config c = *conf;
        check_config(c);
        init_pool_once();
        StreamGuard sg(user_stream, false, NullStream::Default);
        Counter launches;
        if (c.rng < 0 && c.errorBoundMode == FAZ_EB_ABS) c.rng = device_range<T>((const T *)d_data, c.num, sg.st, launches);
        resolve_eb<T>(c, (const T *)d_data, sg.st, launches);
        if (c.rng < 0) c.rng = device_range<T>((const T *)d_data, c.num, sg.st, launches);
        tuner_features_device<T>(c, (const T *)d_data, sg.st, dF, launches);
        CK(cudaStreamSynchronize(sg.st));
    } catch (const Fail &f) {
        set_error(f.msg);
        return f.code;
    } catch (const std::exception &e) {
        set_error(e.what());
        return FAZ_ERR_ARG;
    }
    return FAZ_OK;
}

template <typename T>
int learned_impl(faz_config *conf, const void *d_data, void *user_stream, const TunerModel *model, double min_conf,
                 faz_tuner_choice *choice) {
    auto t0 = clk::now();
    try {
        if (!conf || !d_data || !model) throw Fail{FAZ_ERR_ARG, "null argument"};
        faz_config c = *conf;
        check_config(c);
        init_pool_once();
        StreamGuard sg(user_stream, false, NullStream::Default);
        Counter launches;
        faz_timings tm;
        std::memset(&tm, 0, sizeof(tm));
        const T *dX = (const T *)d_data;
        resolve_eb<T>(c, dX, sg.st, launches);
        if (!(c.absErrorBound > 0) || !std::isfinite(c.absErrorBound))
            throw Fail{FAZ_ERR_ARG, "error bound must be positive and finite"};
        if (c.rng < 0) c.rng = device_range<T>(dX, c.num, sg.st, launches);
        faz_tuner_choice ch;
        learned_tune_device<T>(c, dX, sg.st, *model, min_conf, ch, launches, tm);
        CK(cudaStreamSynchronize(sg.st));
        ch.tune_ms = ms_since(t0);
        if (choice) *choice = ch;
        *conf = c;
    } catch (const Fail &f) {
        set_error(f.msg);
        return f.code;
    } catch (const std::exception &e) {
        set_error(e.what());
        return FAZ_ERR_ARG;
    }
    return FAZ_OK;
}

}  // namespace
}  // namespace faz

// ================================================================= C ABI
extern "C" {

int faz_config_init(faz_config *conf, int N, const uint64_t *dims) {
    int rc = faz::config_init(conf, N, dims);
    if (rc) faz::set_error("faz_config_init: N must be 1..4");
    return rc;
}

int faz_config_load_ini(faz_config *conf, const char *path) {
    if (!conf) return FAZ_ERR_ARG;
    std::string err;
    int rc = faz::config_load_ini(conf, path, err);
    if (rc) faz::set_error(err);
    return rc;
}

int faz_compress(const faz_config *conf, int dtype, const void *data, char **out, size_t *out_size,
                 faz_timings *timings) {
    if (dtype == FAZ_FLOAT) return faz::compress_impl<float>(conf, data, false, nullptr, out, out_size, timings);
    if (dtype == FAZ_DOUBLE) return faz::compress_impl<double>(conf, data, false, nullptr, out, out_size, timings);
    faz::set_error("dtype must be FAZ_FLOAT or FAZ_DOUBLE");
    return FAZ_ERR_ARG;
}

int faz_compress_device(const faz_config *conf, int dtype, const void *d_data, void *stream, char **out,
                        size_t *out_size, faz_timings *timings) {
    if (dtype == FAZ_FLOAT) return faz::compress_impl<float>(conf, d_data, true, stream, out, out_size, timings);
    if (dtype == FAZ_DOUBLE) return faz::compress_impl<double>(conf, d_data, true, stream, out, out_size, timings);
    faz::set_error("dtype must be FAZ_FLOAT or FAZ_DOUBLE");
    return FAZ_ERR_ARG;
}

int faz_decompress(faz_config *conf, int dtype, const char *cmp, size_t cmp_size, void **out, faz_timings *timings) {
    if (dtype == FAZ_FLOAT) return faz::decompress_impl<float>(conf, cmp, cmp_size, out, false, nullptr, nullptr, timings);
    if (dtype == FAZ_DOUBLE)
        return faz::decompress_impl<double>(conf, cmp, cmp_size, out, false, nullptr, nullptr, timings);
    faz::set_error("dtype must be FAZ_FLOAT or FAZ_DOUBLE");
    return FAZ_ERR_ARG;
}

int faz_decompress_device(faz_config *conf, int dtype, const char *cmp, size_t cmp_size, void *d_out, void *stream,
                          faz_timings *timings) {
    if (dtype == FAZ_FLOAT)
        return faz::decompress_impl<float>(conf, cmp, cmp_size, nullptr, true, d_out, stream, timings);
    if (dtype == FAZ_DOUBLE)
        return faz::decompress_impl<double>(conf, cmp, cmp_size, nullptr, true, d_out, stream, timings);
    faz::set_error("dtype must be FAZ_FLOAT or FAZ_DOUBLE");
    return FAZ_ERR_ARG;
}

int faz_compress_device_payload(const faz_config *conf, int dtype, const void *d_data, void *stream, char *out,
                                size_t capacity, size_t *out_size, faz_config *conf_out, faz_timings *timings) {
    if (dtype == FAZ_FLOAT)
        return faz::compress_payload_impl<float>(conf, d_data, stream, out, capacity, out_size, conf_out, timings);
    if (dtype == FAZ_DOUBLE)
        return faz::compress_payload_impl<double>(conf, d_data, stream, out, capacity, out_size, conf_out, timings);
    faz::set_error("dtype must be FAZ_FLOAT or FAZ_DOUBLE");
    return FAZ_ERR_ARG;
}

int faz_decompress_payload_device(int N, int dtype, const char *payload, size_t size, void *d_out, uint64_t capacity,
                                  void *stream, faz_timings *timings) {
    if (dtype == FAZ_FLOAT)
        return faz::decompress_payload_impl<float>(N, payload, size, d_out, capacity, stream, timings);
    if (dtype == FAZ_DOUBLE)
        return faz::decompress_payload_impl<double>(N, payload, size, d_out, capacity, stream, timings);
    faz::set_error("dtype must be FAZ_FLOAT or FAZ_DOUBLE");
    return FAZ_ERR_ARG;
}

int faz_stream_info(const char *cmp, size_t cmp_size, faz_config *conf) {
    if (!cmp || !conf || cmp_size < 4) {
        faz::set_error("faz_stream_info: stream too short");
        return FAZ_ERR_FORMAT;
    }
    int32_t cs;
    std::memcpy(&cs, cmp + cmp_size - 4, 4);
    if (cs <= 0 || (size_t)cs + 4 > cmp_size) {
        faz::set_error("faz_stream_info: bad trailer size");
        return FAZ_ERR_FORMAT;
    }
    int rc = faz::config_load(*conf, (const uint8_t *)cmp + cmp_size - 4 - cs, (size_t)cs);
    if (rc) faz::set_error("faz_stream_info: bad trailer");
    return rc;
}

size_t faz_config_size(void) { return sizeof(faz_config); }

void faz_free(void *p) { std::free(p); }

const char *faz_last_error(void) { return faz::last_error(); }

unsigned faz_zstd_version(void) {
    std::string err;
    const faz::Zstd &z = faz::zstd_lib(err);
    return z.ok ? z.version : 0;
}


int faz_compress_batch(int n, const faz_config *confs, int dtype, const void *const *d_data, void *stream, char **outs,
                       size_t *out_sizes, int threads, faz_timings *timings) {
    if (dtype == FAZ_FLOAT) return faz::compress_batch_impl<float>(n, confs, d_data, stream, outs, out_sizes, threads, timings);
    if (dtype == FAZ_DOUBLE)
        return faz::compress_batch_impl<double>(n, confs, d_data, stream, outs, out_sizes, threads, timings);
    faz::set_error("dtype must be FAZ_FLOAT or FAZ_DOUBLE");
    return FAZ_ERR_ARG;
}

int faz_tune_device(faz_config *conf, int dtype, const void *d_data, void *stream, faz_timings *timings) {
    if (dtype == FAZ_FLOAT) return faz::tune_impl<float>(conf, d_data, stream, timings);
    if (dtype == FAZ_DOUBLE) return faz::tune_impl<double>(conf, d_data, stream, timings);
    faz::set_error("dtype must be FAZ_FLOAT or FAZ_DOUBLE");
    return FAZ_ERR_ARG;
}

int faz_tuner_features(const faz_config *conf, int dtype, const void *d_data, void *stream, float *d_features) {
    if (dtype == FAZ_FLOAT) return faz::features_impl<float>(conf, d_data, stream, d_features);
    if (dtype == FAZ_DOUBLE) return faz::features_impl<double>(conf, d_data, stream, d_features);
    faz::set_error("dtype must be FAZ_FLOAT or FAZ_DOUBLE");
    return FAZ_ERR_ARG;
}

#define FAZ_GUARD(...)                           \
    try {                                        \
        __VA_ARGS__;                             \
    } catch (const faz::Fail &f) {               \
        faz::set_error(f.msg);                   \
        return f.code;                           \
    } catch (const std::exception &e) {          \
        faz::set_error(e.what());                \
        return FAZ_ERR_ARG;                      \
    }                                            \
    return FAZ_OK;

int faz_mlp_forward(const float *d_params, const float *d_x, int batch, float *d_h1, float *d_h2, float *d_logits,
                    void *stream) {
    FAZ_GUARD({
        if (!d_params || !d_x || !d_h1 || !d_h2 || !d_logits || batch <= 0) throw faz::Fail{FAZ_ERR_ARG, "bad argument"};
        faz::Counter launches;
        faz::mlp_forward(d_params, d_x, batch, d_h1, d_h2, d_logits, (cudaStream_t)stream, launches);
    })
}

int faz_mlp_backward(const float *d_params, const float *d_x, const int32_t *d_labels, int batch, const float *d_h1,
                     const float *d_h2, const float *d_logits, float *d_grads, float *d_loss, void *stream) {
    FAZ_GUARD({
        if (!d_params || !d_x || !d_labels || !d_h1 || !d_h2 || !d_logits || !d_grads || !d_loss || batch <= 0)
            throw faz::Fail{FAZ_ERR_ARG, "bad argument"};
        faz::Counter launches;
        faz::mlp_backward(d_params, d_x, d_labels, batch, d_h1, d_h2, d_logits, d_grads, d_loss, (cudaStream_t)stream,
                          launches);
    })
}

int faz_mlp_adam(float *d_params, const float *d_grads, float *d_m, float *d_v, int64_t n, float lr, float beta1,
                 float beta2, float eps, int step, float weight_decay, void *stream) {
    FAZ_GUARD({
        if (!d_params || !d_grads || !d_m || !d_v || n <= 0 || step < 1) throw faz::Fail{FAZ_ERR_ARG, "bad argument"};
        faz::Counter launches;
        faz::mlp_adam(d_params, d_grads, d_m, d_v, n, lr, beta1, beta2, eps, step, weight_decay, (cudaStream_t)stream,
                      launches);
    })
}

faz_tuner_model *faz_tuner_model_create(const float *h_params, const float *h_mean, const float *h_std) {
    if (!h_params || !h_mean || !h_std) {
        faz::set_error("null argument");
        return nullptr;
    }
    try {
        return (faz_tuner_model *)faz::tuner_model_create(h_params, h_mean, h_std);
    } catch (const faz::Fail &f) {
        faz::set_error(f.msg);
    }
    return nullptr;
}

void faz_tuner_model_destroy(faz_tuner_model *model) { faz::tuner_model_destroy((faz::TunerModel *)model); }

int faz_tuner_infer(const faz_tuner_model *model, const float *d_features, int batch, float *d_logits, void *stream) {
    FAZ_GUARD({
        if (!model || !d_features || !d_logits) throw faz::Fail{FAZ_ERR_ARG, "null argument"};
        faz::init_pool_once();
        faz::StreamGuard sg(stream, false, faz::NullStream::Default);
        faz::Counter launches;
        faz::tuner_infer_device(*(const faz::TunerModel *)model, d_features, batch, d_logits, sg.st, launches);
    })
}

int faz_learned_tune(faz_config *conf, int dtype, const void *d_data, void *stream, const faz_tuner_model *model,
                     double min_confidence, faz_tuner_choice *choice) {
    const auto *m = (const faz::TunerModel *)model;
    if (dtype == FAZ_FLOAT) return faz::learned_impl<float>(conf, d_data, stream, m, min_confidence, choice);
    if (dtype == FAZ_DOUBLE) return faz::learned_impl<double>(conf, d_data, stream, m, min_confidence, choice);
    faz::set_error("dtype must be FAZ_FLOAT or FAZ_DOUBLE");
    return FAZ_ERR_ARG;
}

}  // extern "C"
