// host.h - host-side utilities shared by the library's orchestration files:
// error type, device memory from the stream-ordered pool, cached pinned
// staging, stream/event guards, launch counting, byte packing and the float
// quantiser's parameter split.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <future>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace faz {

using clk = std::chrono::steady_clock;
inline double ms_since(clk::time_point t) { return std::chrono::duration<double, std::milli>(clk::now() - t).count(); }

// FAZ_TUNE_TRACE=1 prints the tuner's timeline to stderr: milliseconds since
// the current tuning call began (trace_epoch), from whichever thread runs the
// step.
inline bool tune_trace() {
    static const bool on = [] {
        const char *e = std::getenv("FAZ_TUNE_TRACE");
        return e && e[0] == '1';
    }();
    return on;
}
inline clk::time_point &trace_epoch() {
    static clk::time_point t0 = clk::now();
    return t0;
}
inline void trace_step(const char *what) {
    if (tune_trace()) std::fprintf(stderr, "tune %8.3f ms  %s\n", ms_since(trace_epoch()), what);
}

struct Fail {
    int code;
    std::string msg;
};

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t _e = (call);                                                              \
        if (_e != cudaSuccess) throw Fail{FAZ_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)}; \
    } while (0)

// ----------------------------------------------------- memory management
// Device memory comes from the stream-ordered pool (cached across calls);
// pinned host staging is cached per thread and grows on demand.
struct DevMem {
    cudaStream_t st;
    std::vector<void *> ptrs;
    explicit DevMem(cudaStream_t s) : st(s) {}
    template <typename T>
    T *alloc(size_t count) {
        void *p = nullptr;
        size_t bytes = count * sizeof(T);
        if (bytes == 0) bytes = 16;
        CK(cudaMallocAsync(&p, bytes, st));
        ptrs.push_back(p);
        return (T *)p;
    }
    ~DevMem() {
        for (void *p : ptrs) cudaFreeAsync(p, st);
    }
};

inline void init_pool_once() {
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t thr = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
    });
}

struct Pinned {
    uint8_t *p = nullptr;
    size_t cap = 0;
    uint8_t *get(size_t n) {
        if (n > cap) {
            if (p) cudaFreeHost(p);
            p = nullptr;
            cap = 0;
            size_t c = std::max<size_t>(n + n / 4, 1 << 20);
            if (cudaHostAlloc((void **)&p, c, cudaHostAllocDefault) != cudaSuccess)
                throw Fail{FAZ_ERR_CUDA, "cudaHostAlloc failed"};
            cap = c;
        }
        return p;
    }
    ~Pinned() {
        if (p) cudaFreeHost(p);
    }
};
inline thread_local Pinned t_pin_payload;
inline thread_local Pinned t_pin_small;
inline thread_local Pinned t_pin_flag;  // device status words read after a later synchronisation

// Pinned staging for host-to-device uploads whose copies complete after the
// call returns: acquire() waits for the thread's previous upload from it,
// release(st) marks the new one (an event recorded on st).
struct TableStage {
    Pinned buf;
    cudaEvent_t ev = nullptr;
    int dev = -1;
    bool pending = false;
    uint8_t *acquire(size_t n) {
        if (pending) CK(cudaEventSynchronize(ev));
        pending = false;
        return buf.get(n);
    }
    void release(cudaStream_t st) {
        int d = 0;
        CK(cudaGetDevice(&d));
        if (ev && d != dev) {
            cudaEventDestroy(ev);
            ev = nullptr;
        }
        if (!ev) {
            CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            dev = d;
        }
        CK(cudaEventRecord(ev, st));
        pending = true;
    }
    ~TableStage() {
        if (ev) cudaEventDestroy(ev);
    }
};
inline thread_local TableStage t_table_stage;

// Payload producers assemble their bytes in the thread's pinned staging
// buffer and end with emit_payload: the bytes are copied into `out`, or, while
// the thread has a view installed (t_payload_view), left where they are, the
// view pointing at them until the thread assembles its next payload (a
// tuning trial only measures its payload's zstd size).
struct PayloadView {
    const uint8_t *data = nullptr;
    size_t size = 0;
};
inline thread_local PayloadView *t_payload_view = nullptr;
inline void emit_payload(std::vector<uint8_t> &out, const uint8_t *pin, size_t n) {
    if (t_payload_view) {
        t_payload_view->data = pin;
        t_payload_view->size = n;
        out.clear();
        return;
    }
    out.assign(pin, pin + n);
}

// How a call on device buffers reads a NULL stream: the legacy default
// stream, so that the call is ordered after the caller's default-stream work
// (the data it reads may still be being written there).
enum class NullStream { Library, Default };

struct StreamGuard {
    cudaStream_t st = nullptr;
    bool own = false;
    // user stream, or (NULL) the legacy default stream or a library stream
    // (at the device's highest priority when `high` is set)
    explicit StreamGuard(void *user, bool high = false, NullStream ns = NullStream::Library) {
        if (user) {
            st = (cudaStream_t)user;
        } else if (ns == NullStream::Default) {
            st = cudaStreamLegacy;
        } else if (high) {
            int least = 0, greatest = 0;
            CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
            CK(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, greatest));
            own = true;
        } else {
            CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
            own = true;
        }
    }
    ~StreamGuard() {
        if (own) cudaStreamDestroy(st);
    }
};

// Host threads that live for the process, so that their thread-local pinned
// staging buffers are reused from call to call.  run() executes the tasks on
// the pool (the caller waits) and is safe to call from several threads.
class HostPool {
  public:
    static HostPool &get() {
        static HostPool pool;
        return pool;
    }
    void run(std::vector<std::function<void()>> &tasks) {
        if (tasks.empty()) return;
        struct Batch {
            std::mutex mu;
            std::condition_variable cv;
            size_t left;
        } b;
        b.left = tasks.size();
        {
            std::lock_guard<std::mutex> g(mu_);
            for (auto &t : tasks)
                q_.push_back([&b, &t] {
                    t();
                    std::lock_guard<std::mutex> g2(b.mu);
                    if (--b.left == 0) b.cv.notify_all();
                });
        }
        cv_.notify_all();
        std::unique_lock<std::mutex> lk(b.mu);
        b.cv.wait(lk, [&] { return b.left == 0; });
    }
    ~HostPool() {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : th_) t.join();
    }

  private:
    HostPool() {
        const unsigned n = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        for (unsigned i = 0; i < n; i++)
            th_.emplace_back([this] {
                for (;;) {
                    std::function<void()> job;
                    {
                        std::unique_lock<std::mutex> lk(mu_);
                        cv_.wait(lk, [this] { return stop_ || !q_.empty(); });
                        if (stop_ && q_.empty()) return;
                        job = std::move(q_.front());
                        q_.pop_front();
                    }
                    job();
                }
            });
    }
    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<std::function<void()>> q_;
    std::vector<std::thread> th_;
    bool stop_ = false;
};

// Persistent host threads for the tuner's concurrent trials.  A trial on a
// fresh thread would allocate its thread-local pinned staging buffers anew
// (and free them when the thread ends, which synchronises the device); these
// threads keep them for the process.  A task runs with the submitting
// thread's device current.  (Each trial still creates its own stream: a
// stream kept by the worker from call to call measured slower.)
class TaskThreads {
  public:
    static TaskThreads &get() {
        static TaskThreads pool;
        return pool;
    }
    template <typename R>
    std::future<R> submit(std::function<R()> f) {
        int dev = 0;
        cudaGetDevice(&dev);
        auto task = std::make_shared<std::packaged_task<R()>>(std::move(f));
        std::future<R> fut = task->get_future();
        {
            std::lock_guard<std::mutex> g(mu_);
            q_.push_back(Job{dev, [task] { (*task)(); }});
        }
        cv_.notify_one();
        return fut;
    }
    ~TaskThreads() {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : th_) t.join();
    }

  private:
    struct Job {
        int dev;
        std::function<void()> fn;
    };
    // one thread per host core, 8 to 32 of them (the tuners' trials and the
    // QoZ tuner's alpha/beta tests run here concurrently)
    static int thread_count() {
        const unsigned hw = std::thread::hardware_concurrency();
        return (int)std::min(32u, std::max(8u, hw));
    }
    TaskThreads() {
        const int n = thread_count();
        for (int i = 0; i < n; i++)
            th_.emplace_back([this] {
                for (;;) {
                    Job job;
                    {
                        std::unique_lock<std::mutex> lk(mu_);
                        cv_.wait(lk, [this] { return stop_ || !q_.empty(); });
                        if (stop_ && q_.empty()) return;
                        job = std::move(q_.front());
                        q_.pop_front();
                    }
                    cudaSetDevice(job.dev);
                    job.fn();
                }
            });
    }
    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<Job> q_;
    std::vector<std::thread> th_;
    bool stop_ = false;
};

struct Events {
    cudaEvent_t a = nullptr, b = nullptr;
    Events() {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
    }
    ~Events() {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    float ms() {
        float t = 0;
        cudaEventElapsedTime(&t, a, b);
        return t;
    }
};

template <typename V>
void put(std::vector<uint8_t> &o, V v) {
    uint8_t b[sizeof(V)];
    std::memcpy(b, &v, sizeof(V));
    o.insert(o.end(), b, b + sizeof(V));
}
inline void put_be32(std::vector<uint8_t> &o, int32_t v) {
    o.push_back((uint8_t)(v >> 24));
    o.push_back((uint8_t)(v >> 16));
    o.push_back((uint8_t)(v >> 8));
    o.push_back((uint8_t)v);
}

struct Counter {
    uint64_t n = 0;
    void operator()(cudaError_t e) {
        if (e != cudaSuccess) throw Fail{FAZ_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e)};
        n++;
    }
};

// Float-pair split of eb and 1/eb for the exact float quantiser (interp.cu).
// Enabled for float data with eb within [2^-60, 2^60]; FAZ_FASTPATH=0 turns it off.
template <typename T>
void set_fast_path(LevelArgs &a) {
    a.fast = 0;
    if (sizeof(T) != 4) return;
    const char *env = std::getenv("FAZ_FASTPATH");
    if (env && env[0] == '0') return;
    if (!(a.eb >= 0x1p-60 && a.eb <= 0x1p60)) return;
    a.eh = (float)a.eb;
    a.el = (float)(a.eb - (double)a.eh);
    a.rh = (float)a.recip;
    a.rl = (float)(a.recip - (double)a.rh);
    float lo = (float)a.eb;
    if ((double)lo > a.eb) lo = std::nextafter(lo, 0.0f);
    a.eblo = lo;
    a.twor_f = (float)(2 * a.radius);
    // d < eb * (1 - 2^-20) gives d * (1/eb) < 1 - 2^-20 + 2^-52, so floor(x) = 0
    a.eb_half0 = (float)(a.eb * (1.0 - 0x1p-20));
    if ((double)a.eb_half0 > a.eb * (1.0 - 0x1p-20)) a.eb_half0 = std::nextafter(a.eb_half0, 0.0f);
    if (a.radius == 1) a.eb_half0 = 0.0f;  // code 1 may be unpredictable under trimToZero 2
    a.fast = 1;
}

inline bool verify_fast_path() {
    const char *env = std::getenv("FAZ_VERIFY_FASTPATH");
    return env && env[0] == '1';
}

inline size_t smem_limit() {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return (size_t)v;
}

// Lorenzo fast frontend (lorenzo.cu) and the default configuration's tuner (tuner.cu)
template <typename T>
void lorenzo3_compress_payload(const uint64_t *dims, int bs, int pd, int lo, int lo2, int reg, double eb, int radius,
                               const T *dX, cudaStream_t st, Counter &launches, faz_timings &tm,
                               std::vector<uint8_t> &out);
template <typename T>
void lorenzo3_decompress(const uint8_t *pl, size_t psize, const uint64_t *dims, T *dOut, cudaStream_t st,
                         Counter &launches, faz_timings &tm);
// The SZ3 tuner of the default configuration.  `speculate` (optional) is
// called once the pre-zstd sizes of the interpolation trials are known, with
// the candidate they point to and - when the best two are too close for those
// sizes to tell - the runner-up (else null).
template <typename T>
void sz3_tune_device(faz_config &c, const T *dX, cudaStream_t st, Counter &launches, faz_timings &tm,
                     const std::function<void(const faz_config &, const faz_config *)> &speculate);

template <typename T>
void qoz_tune_device(faz_config &c, const T *dX, cudaStream_t st, Counter &launches, faz_timings &tm);
template <typename T>
int qoz_prepare(faz_config &c, const T *dX, cudaStream_t st, Counter &launches);
// The QoZ tuner's Lorenzo candidate: CompressTest(ALGO_LORENZO_REG) of nblk
// sampled 2-D / 3-D blocks of bsz^N points (bit rate, PSNR); with `recon`
// the blocks' reconstructions also come back to the host.
template <typename T>
void lorenzo_compress_test(int N, const T *dBlocks, uint64_t nblk, int64_t bsz, double eb, double rng,
                           double pcoeff, cudaStream_t st, Counter &launches, double &bitrate, double &psnr,
                           std::vector<T> *recon = nullptr);
// Lorenzo settings once the QoZ tuner has chosen Lorenzo (sampling, the
// quantisation-interval estimate, pred_dim and 16384-bin trials).
template <typename T>
void qoz_lorenzo_followup(faz_config &c, const T *dX, cudaStream_t st, Counter &launches, faz_timings &tm);
// Tuning runs its QoZ branch (SZInterp.hpp:1857) for QoZ = 1 and for any
// predictorTuningRate in (0, 1)
inline bool qoz_tuned(const faz_config &c) {
    return c.QoZ || (c.predictorTuningRate > 0 && c.predictorTuningRate < 1);
}
// general frontend for 1-D / 2-D fields: Lorenzo, two-layer Lorenzo and
// linear-regression predictors as enabled (general.cu)
template <typename T>
void gen_compress_payload(int N, const uint64_t *dims, int bs, int lo, int lo2, int reg, double eb, int radius,
                          const T *dX, cudaStream_t st, Counter &launches, faz_timings &tm, std::vector<uint8_t> &out);
template <typename T>
void gen_decompress(int N, const uint8_t *pl, size_t psize, const uint64_t *dims, int lo, int lo2, int reg, T *dOut,
                    cudaStream_t st, Counter &launches, faz_timings &tm);
// ALGO_INTERP_BLOCKED and fixBlockSize off the coarse lattice (blocked.cu):
// the Config SZ_compress_Interp_blocked leaves, the codes of both kinds of
// stream, and their decoder
void blocked_prepare(faz_config &c);
bool fixbs_aligned(int N, const uint64_t *dims, uint64_t maxStep, int fixbs);
template <typename T>
void blocked_codes(const faz_config &c, const T *dX, T *W, uint16_t *codes, T *scratch, DevMem &m, cudaStream_t st,
                   Counter &launches, std::vector<uint8_t> &ops, std::vector<uint8_t> &dirs);
template <typename T>
void fixed_block_codes(const faz_config &c, const std::vector<uint8_t> &il, const std::vector<uint8_t> &dl,
                       const T *dX, T *W, uint16_t *codes, T *scratch, DevMem &m, cudaStream_t st, Counter &launches);
// 4-D fields (interp4.cu): codes and unpredictable values of every level, and
// the inverse
template <typename T>
void interp4_codes(const faz_config &c, double eb, int radius, const std::vector<uint8_t> &il,
                   const std::vector<uint8_t> &dl, const T *dX, T *W, uint16_t *codes, T *scratch,
                   unsigned long long *verify, DevMem &m, cudaStream_t st, Counter &launches);
template <typename T>
void interp4_decompress(const uint64_t *dims, uint64_t maxStep, int blocksize, int fixbs, int interp, int dir,
                        const std::vector<uint8_t> &il, const std::vector<uint8_t> &dl, double eb, double alpha,
                        double beta, int radius, int trim, const uint16_t *codes, const uint64_t *zpos, uint64_t nz,
                        const T *unpred, T *dOut, unsigned long long *verify, DevMem &m, cudaStream_t st,
                        Counter &launches);
template <typename T>
void blocked_decompress_levels(int N, const uint64_t *dims, uint64_t maxStep, int B, double eb, double alpha,
                               double beta, int radius, int trim, int interp, int dir,
                               const std::vector<uint8_t> &il, const std::vector<uint8_t> &dl,
                               const std::vector<uint8_t> &ops, const std::vector<uint8_t> &dirs, bool blockwise,
                               const uint16_t *codes, const uint64_t *zpos, uint64_t nz, const T *unpred, T *dOut,
                               DevMem &m, cudaStream_t st, Counter &launches);
// calAbsErrorBound on the device (capi.cu)
template <typename T>
void resolve_eb(faz_config &c, const T *dX, cudaStream_t st, Counter &launches);
// learned tuner (learned.cu)
struct TunerModel;
template <typename T>
void tuner_features_device(const faz_config &c, const T *dX, cudaStream_t st, float *dF, Counter &launches);
void mlp_forward(const float *P, const float *X, int B, float *H1, float *H2, float *Z, cudaStream_t st,
                 Counter &launches);
void mlp_backward(const float *P, const float *X, const int32_t *labels, int B, const float *H1, const float *H2,
                  const float *Z, float *G, float *loss, cudaStream_t st, Counter &launches);
void mlp_adam(float *P, const float *G, float *M, float *V, int64_t n, float lr, float b1, float b2, float eps, int t,
              float wd, cudaStream_t st, Counter &launches);
TunerModel *tuner_model_create(const float *P, const float *mu, const float *sd);
void tuner_model_destroy(TunerModel *t);
void tuner_infer_device(const TunerModel &t, const float *dF, int B, float *dZ, cudaStream_t st, Counter &launches);
template <typename T>
void learned_tune_device(faz_config &c, const T *dX, cudaStream_t st, const TunerModel &model, double min_conf,
                         faz_tuner_choice &ch, Counter &launches, faz_timings &tm);

template <typename T>
double device_range(const T *dX, uint64_t n, cudaStream_t st, Counter &launches);

// ------------------------------------------------------- Huffman stages
struct HuffEncoded {
    Codebook cb;
    uint32_t *bits = nullptr;  // device: the MSB-first bit string
    uint64_t nbytes = 0;
    uint64_t nzero = 0;        // codes equal to 0 (unpredictable points)
    unsigned long long *zc = nullptr, *zoff = nullptr;  // zero counts per sub-chunk and their exclusive scan
};
// `sized`, when given, runs as soon as the codebook, the zero count and the
// encoded size are known on the host (before the encoding kernels finish).
// The uint32_t overloads serve quantisers of more than 65536 bins.
void huffman_encode_device(const uint16_t *codes, uint64_t n, int center, DevMem &m, cudaStream_t st,
                           Counter &launches, HuffEncoded &h, faz_timings &tm,
                           const std::function<void(const HuffEncoded &)> &sized = {});
void huffman_encode_device(const uint32_t *codes, uint64_t n, int center, DevMem &m, cudaStream_t st,
                           Counter &launches, HuffEncoded &h, faz_timings &tm,
                           const std::function<void(const HuffEncoded &)> &sized = {});
void append_tree(std::vector<uint8_t> &o, const Codebook &cb, uint64_t nbytes);
void huffman_decode_device(const uint8_t *&p, const uint8_t *end, uint64_t num, uint16_t *codes, DevMem &m,
                           cudaStream_t st, Counter &launches);
void huffman_decode_device(const uint8_t *&p, const uint8_t *end, uint64_t num, uint32_t *codes, DevMem &m,
                           cudaStream_t st, Counter &launches);
uint64_t zero_positions(const uint16_t *codes, uint64_t num, DevMem &m, cudaStream_t st, Counter &launches,
                        uint64_t *&zpos);
uint64_t zero_positions(const uint32_t *codes, uint64_t num, DevMem &m, cudaStream_t st, Counter &launches,
                        uint64_t *&zpos);

}  // namespace faz
