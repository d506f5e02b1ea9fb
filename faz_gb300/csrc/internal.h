// internal.h - host-side declarations shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <mutex>
#include <set>
#include <string>
#include <utility>
#include <vector>

#include "../../include/faz_gb300.h"
#include "common.cuh"

namespace faz {

// Let a kernel take up to the device's opt-in shared memory per block, once
// per (device, kernel).  Setting the limit to each launch's own need instead
// races: host threads launching the same kernel concurrently (the tuner's
// trials) can lower it between another thread's set and launch.
// smallest l with 2^l >= d (ceil(log2(d)) for d >= 1)
inline int ceil_log2(uint64_t d) {
    int l = 0;
    while (((uint64_t)1 << l) < d) l++;
    return l;
}

// Level error bound (SZInterpolationCompressor.hpp:386-406, eb_ratio 0.5)
inline double level_eb(double eb, double alpha, double beta, int level) {
    if (alpha < 0) return level >= 3 ? eb * 0.5 : eb;
    if (alpha >= 1) {
        double cr = std::pow(alpha, level - 1);
        if (cr > beta) cr = beta;
        return eb / cr;
    }
    double cr = 1 - (level - 1) * alpha;
    if (cr < beta) cr = beta;
    return eb * cr;
}

inline cudaError_t allow_dynamic_smem(const void *func) {
    static std::mutex mu;
    static std::set<std::pair<int, const void *>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(mu);
    if (done.count({dev, func})) return cudaSuccess;
    int optin = 0;
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return e;
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, func);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    if (e == cudaSuccess) done.insert({dev, func});
    return e;
}

// ---------------------------------------------------------------- kernels
template <typename T>
cudaError_t launch_minmax(const T *X, uint64_t n, T *pmin, T *pmax, int nblocks, cudaStream_t st);
template <typename T>
size_t level_smem_bytes(const LevelArgs &a);
// One interpolation level; *nlaunch grows by the kernel launches it made.
template <typename T>
cudaError_t launch_level(const LevelArgs &a, int64_t nblocks, bool decomp, const T *X, T *W, uint16_t *codes,
                         T *scratch, const uint64_t *zpos, uint64_t nz, const T *unpred, cudaStream_t st,
                         int *nlaunch);
// The finest level of a 3-D float field, plane by plane with TMA-staged
// planes (finest.cu): whether a level qualifies, and its launch.
bool finest_eligible(const LevelArgs &a, bool decomp, const void *X, size_t elem);
cudaError_t launch_finest(const LevelArgs &a, int64_t nblocks, bool decomp, const float *X, float *W,
                          uint16_t *codes, float *scratch, const uint64_t *zpos, uint64_t nz, const float *unpred,
                          cudaStream_t st);
template <typename T>
cudaError_t launch_first_point(bool decomp, const T *X, T *W, uint16_t *codes, T *scratch, double eb, int radius,
                               int trim, const uint64_t *zpos, uint64_t nz, const T *unpred, cudaStream_t st);
template <typename T>
cudaError_t launch_anchors(bool decomp, const T *X, T *W, uint16_t *codes, T *scratch, const T *unpred,
                           const int64_t *na, const int64_t *step, const int64_t *offs, cudaStream_t st);

// Batched compression: every field's first point / anchors and levels in one
// persistent launch from a device work queue (interp.cu).
struct BatchField {
    const void *X;
    void *W;
    uint16_t *codes;
    void *scratch;
    double eb, recip;  // base error bound (first point)
    int radius, trim;
    int anchor;        // 1: anchor grid (na, step, offs), 0: first point
    int64_t na[3], step[3], offs[3];
};
struct BatchGroup {
    int field;
    int kind;        // 0 first point, 1 anchors, 2 level
    int args;        // level: index into the LevelArgs table
    int dep;         // group whose items must all be done first (-1: none)
    int64_t nitems;  // work items (blocks; anchor chunks of `threads` anchors; 1)
    int64_t item0;   // first ticket of the group
};
template <typename T>
cudaError_t launch_interp_batch(const BatchGroup *groups, int ngroups, const BatchField *fields, const LevelArgs *largs,
                                uint64_t total, unsigned long long *counter, unsigned *done, int *err, bool wide,
                                int grid, int threads, size_t smem, cudaStream_t st);

template <typename T>
cudaError_t launch_minmax_batch(const T *const *X, const uint64_t *n, int nfields, T *pmin, T *pmax, int nblocks,
                                cudaStream_t st);
template <typename T, bool WIDE>
int batch_occupancy(int threads, size_t smem);

uint64_t hist_subchunks(uint64_t n);
// the symbols of non-zero count: list[3k..3k+2] = symbol, count, first
// position, in no particular order; *nlist (zeroed by the caller) their number
cudaError_t launch_hist_compact(const unsigned long long *hist, const unsigned long long *first, int nsym,
                                unsigned long long *list, unsigned int *nlist, cudaStream_t st);
// Huffman stage kernels; the uint32_t overloads serve quantisers of more than
// 65536 bins.
cudaError_t launch_histogram(const uint16_t *codes, uint64_t n, int center, unsigned long long *hist,
                             unsigned long long *first, unsigned long long *zcount, cudaStream_t st);
cudaError_t launch_histogram(const uint32_t *codes, uint64_t n, int center, unsigned long long *hist,
                             unsigned long long *first, unsigned long long *zcount, cudaStream_t st);
cudaError_t launch_count_zeros(const uint16_t *codes, uint64_t n, unsigned long long *zcount, cudaStream_t st);
cudaError_t launch_count_zeros(const uint32_t *codes, uint64_t n, unsigned long long *zcount, cudaStream_t st);
template <typename T, typename C>
cudaError_t launch_compact_zeros(const C *codes, uint64_t n, const unsigned long long *zcount,
                                 const unsigned long long *zoff, uint64_t *zpos, const T *scratch, T *vals,
                                 cudaStream_t st);
uint64_t scan_temp_words(uint64_t n);
cudaError_t launch_scan_u64(const unsigned long long *in, unsigned long long *out, uint64_t n,
                            unsigned long long *temp, cudaStream_t st);
uint64_t encode_chunks(uint64_t n);
cudaError_t launch_encode_bits(const uint16_t *codes, uint64_t n, int offset, const uint8_t *len,
                               unsigned long long *chunkbits, cudaStream_t st);
cudaError_t launch_encode_bits(const uint32_t *codes, uint64_t n, int offset, const uint8_t *len,
                               unsigned long long *chunkbits, cudaStream_t st);
cudaError_t launch_encode_pack(const uint16_t *codes, uint64_t n, int offset, const unsigned long long *code64,
                               const unsigned long long *packed, const uint8_t *len,
                               const unsigned long long *chunkoff, uint32_t *out, int maxlen, cudaStream_t st);
cudaError_t launch_encode_pack(const uint32_t *codes, uint64_t n, int offset, const unsigned long long *code64,
                               const unsigned long long *packed, const uint8_t *len,
                               const unsigned long long *chunkoff, uint32_t *out, int maxlen, cudaStream_t st);

struct DecodeTablesDev {
    const uint32_t *lut;
    const uint32_t *left, *right;
    const int32_t *sym;
    const uint8_t *leaf;
};
uint64_t decode_units(uint64_t nbits);
uint64_t decode_unit_bits();
int decode_boundaries();
cudaError_t launch_init_starts(uint64_t *start, uint64_t n, cudaStream_t st);
// speculative decode of units [ubase, min(uend, nunits)); ubase a multiple of
// decode_cta_units()
uint64_t decode_cta_units();
cudaError_t launch_decode_spec(const DecodeTablesDev &t, const uint32_t *w32, uint64_t nwords, uint64_t nbits,
                               uint64_t nunits, uint64_t ubase, uint64_t uend, uint64_t *end, unsigned int *cnt,
                               uint16_t *bnd, int *err, cudaStream_t st);
cudaError_t launch_decode_resync(const DecodeTablesDev &t, const uint32_t *w32, uint64_t nwords, uint64_t nbits,
                                 uint64_t nunits, const uint64_t *end_in, uint64_t *end_out, unsigned int *cnt,
                                 const uint16_t *bnd, uint64_t *start, int *changed, cudaStream_t st);
cudaError_t launch_decode_write(const DecodeTablesDev &t, const uint32_t *w32, uint64_t nwords, uint64_t nbits,
                                uint64_t nunits, const uint64_t *start, const unsigned long long *off, uint64_t nout,
                                int offset, uint16_t *out, cudaStream_t st);
cudaError_t launch_decode_write(const DecodeTablesDev &t, const uint32_t *w32, uint64_t nwords, uint64_t nbits,
                                uint64_t nunits, const uint64_t *start, const unsigned long long *off, uint64_t nout,
                                int offset, uint32_t *out, cudaStream_t st);
cudaError_t launch_fill_u16(uint16_t *out, uint64_t n, uint16_t v, cudaStream_t st);
cudaError_t launch_fill_u16(uint32_t *out, uint64_t n, uint32_t v, cudaStream_t st);
cudaError_t launch_widen_counts(const unsigned int *cnt, unsigned long long *out, uint64_t n, cudaStream_t st);

// ------------------------------------------------------------ Huffman host
struct Codebook {
    int offset = 0;          // smallest symbol
    int stateNum = 0;        // max - min + 2
    int nodeCount = 0;       // 2 * distinct - 1
    int maxlen = 0;
    std::vector<uint64_t> code;  // per state, MSB-aligned
    std::vector<uint8_t> len;    // per state
    std::vector<uint8_t> tree;   // serialised tree (HuffmanEncoder::save body after the two ints)
};
// Build the reference codebook from symbol counts and first-occurrence
// positions (symbols with count 0 are absent).
int build_codebook(const std::vector<int> &syms, const std::vector<uint64_t> &counts,
                   const std::vector<uint64_t> &first, Codebook &cb, std::string &err);

struct DecodeTablesHost {
    int offset = 0;
    int nodeCount = 0;
    bool constant = false;       // single-symbol stream
    int constant_state = 0;
    std::vector<uint32_t> lut, left, right;
    std::vector<int32_t> sym;
    std::vector<uint8_t> leaf;
};
// Parse HuffmanEncoder::save output at p (advances p); builds decode tables.
int parse_tree(const uint8_t *&p, const uint8_t *end, DecodeTablesHost &t, std::string &err);
constexpr int kLutBits = 12;

// -------------------------------------------------------------- stream/io
void config_save(const faz_config &c, std::vector<uint8_t> &out);
// used (optional): bytes the Config occupies
int config_load(faz_config &c, const uint8_t *p, size_t n, size_t *used = nullptr);
int config_init(faz_config *c, int N, const uint64_t *dims);
int config_load_ini(faz_config *c, const char *path, std::string &err);

struct Zstd {
    bool ok = false;
    unsigned version = 0;
    size_t (*compress)(void *, size_t, const void *, size_t, int) = nullptr;
    size_t (*decompress)(void *, size_t, const void *, size_t) = nullptr;
    unsigned (*isError)(size_t) = nullptr;
    size_t (*bound)(size_t) = nullptr;
    unsigned long long (*frameContentSize)(const void *, size_t) = nullptr;
    size_t (*findFrameCompressedSize)(const void *, size_t) = nullptr;
    unsigned long long (*getFrameContentSize)(const void *, size_t) = nullptr;
    // advanced API (one frame compressed by worker threads); null if absent
    void *(*createCCtx)() = nullptr;
    size_t (*freeCCtx)(void *) = nullptr;
    size_t (*setParameter)(void *, int, int) = nullptr;
    size_t (*compress2)(void *, void *, size_t, const void *, size_t) = nullptr;
    // ZSTD_compress on a caller's context (the same frame); null if absent
    size_t (*compressCCtx)(void *, void *, size_t, const void *, size_t, int) = nullptr;
};
// ZSTD_compress at level 3 with this thread's reused context and output
// buffer (no allocation per call); returns the frame size
size_t zstd_level3_size(const Zstd &z, const void *src, size_t n);

// How the body of a Lossless_zstd stream (one level-3 frame in the reference,
// include/QoZ/lossless/Lossless_zstd.hpp:22-32) is written:
//   Single  - ZSTD_compress on the calling thread: the reference's own call,
//             byte for byte (FAZ_ZSTD_THREADS=0);
//   Workers - one level-3 frame compressed by zstd's worker threads in jobs of
//             a size fixed by the payload length, so the bytes do not depend
//             on the worker count (the default, FAZ_ZSTD_THREADS workers);
//   Frames  - independent level-3 frames of consecutive slices, compressed and
//             decompressed in parallel (FAZ_ZSTD_MULTIFRAME=1): a format
//             extension that ZSTD_decompress still reads.
enum class ZstdMode { Single, Workers, Frames };
struct ZstdPlan {
    ZstdMode mode = ZstdMode::Single;
    int threads = 0;   // workers (Workers) or host threads (Frames)
    int nframes = 1;   // Frames only
    int job = 0;       // Workers only: job size in bytes
};
ZstdPlan zstd_plan(size_t n);
size_t zstd_body_bound(const Zstd &z, size_t n, const ZstdPlan &p);
// `parallel` false compresses on the calling thread alone (one worker for
// Workers, frames one after another for Frames): the same bytes.
size_t zstd_compress_body(const Zstd &z, uint8_t *dst, size_t cap, const uint8_t *src, size_t n, const ZstdPlan &p,
                          bool parallel = true);
// Decodes one or more concatenated frames (independent frames in parallel).
size_t zstd_decompress_frames(const Zstd &z, uint8_t *dst, size_t raw, const uint8_t *src, size_t n, int threads);
int zstd_threads();  // FAZ_ZSTD_THREADS, default the host's cores up to 16
const Zstd &zstd_lib(std::string &err);

// ------------------------------------------------------------------ errors
void set_error(const std::string &msg);

}  // namespace faz
