// stream.cpp - QoZ::Config mirror (defaults, INI loader, stream trailer) and
// the host zstd binding.
#include <dlfcn.h>

#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <new>
#include <mutex>
#include <sstream>
#include <thread>
#include <vector>

#include "internal.h"

namespace faz {

// ------------------------------------------------------------------ errors
static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }
const char *last_error() { return g_last_error.c_str(); }

// ------------------------------------------------------------------ config
// QoZ::Config::Config(Dims...) and member defaults (include/QoZ/utils/Config.hpp:64-74, 394-499)
int config_init(faz_config *c, int N, const uint64_t *dims) {
    if (!c || N < 1 || N > 4 || !dims) return FAZ_ERR_ARG;
    std::memset(c, 0, sizeof(*c));
    c->N = N;
    c->num = 1;
    for (int i = 0; i < N; i++) {
        c->dims[i] = dims[i];
        c->coeffs_dims[i] = dims[i];
        c->num *= dims[i];
    }
    c->coeffs_dims_len = N;
    c->coeffs_num = c->num;
    c->cmprAlgo = FAZ_ALGO_INTERP_LORENZO;
    c->errorBoundMode = FAZ_EB_ABS;
    c->relErrorBound = -1.0;
    c->rng = -1.0;
    c->alpha = -1.0;
    c->beta = -1.0;
    c->lorenzo = 1;
    c->regression = 1;
    c->lossless = 1;
    c->encoder = 1;
    c->interpAlgo = FAZ_INTERP_ALGO_CUBIC;
    c->interpBlockSize = 32;
    c->quantbinCnt = 65536;
    c->blockSize = N == 1 ? 128 : (N == 2 ? 16 : 6);
    c->pred_dim = N;
    c->stride = c->blockSize;
    c->SSIMBlockSize = 8;
    c->verbose = 1;
    c->wavelet_rel_coeff = 0.75;
    c->sperr = -1;
    c->pyBind = 1;
    return FAZ_OK;
}

namespace {

// Minimal INI reader with the conventions of the reference's inih: sections
// in brackets, "name = value" or "name : value", ';'/'#' comment lines, ';'
// inline comments after whitespace, case-insensitive section and key names.
struct Ini {
    std::map<std::string, std::string> kv;
    static std::string lower(std::string s) {
        std::transform(s.begin(), s.end(), s.begin(), [](unsigned char ch) { return (char)std::tolower(ch); });
        return s;
    }
    static std::string trim(const std::string &s) {
        size_t a = 0, b = s.size();
        while (a < b && std::isspace((unsigned char)s[a])) a++;
        while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
        return s.substr(a, b - a);
    }
    bool load(const char *path) {
        std::ifstream f(path);
        if (!f) return false;
        std::string line, section;
        while (std::getline(f, line)) {
            std::string t = trim(line);
            if (t.empty() || t[0] == ';' || t[0] == '#') continue;
            if (t[0] == '[') {
                size_t e = t.find(']');
                if (e == std::string::npos) return false;
                section = trim(t.substr(1, e - 1));
                continue;
            }
            size_t eq = t.find_first_of("=:");
            if (eq == std::string::npos) return false;
            std::string name = trim(t.substr(0, eq));
            std::string value = t.substr(eq + 1);
            for (size_t i = 1; i < value.size(); i++) {
                if (value[i] == ';' && std::isspace((unsigned char)value[i - 1])) {
                    value = value.substr(0, i);
                    break;
                }
            }
            kv[lower(section) + "=" + lower(name)] = trim(value);
        }
        return true;
    }
    bool has(const char *s, const char *k) const { return kv.count(lower(s) + "=" + lower(k)) > 0; }
    std::string get(const char *s, const char *k) const {
        auto it = kv.find(lower(s) + "=" + lower(k));
        return it == kv.end() ? std::string() : it->second;
    }
    long integer(const char *s, const char *k, long dflt) const {
        if (!has(s, k)) return dflt;
        std::string v = get(s, k);
        char *end;
        long n = std::strtol(v.c_str(), &end, 0);
        return end > v.c_str() ? n : dflt;
    }
    double real(const char *s, const char *k, double dflt) const {
        if (!has(s, k)) return dflt;
        std::string v = get(s, k);
        char *end;
        double n = std::strtod(v.c_str(), &end);
        return end > v.c_str() ? n : dflt;
    }
    bool boolean(const char *s, const char *k, bool dflt) const {
        if (!has(s, k)) return dflt;
        std::string v = lower(get(s, k));
        if (v == "true" || v == "yes" || v == "on" || v == "1") return true;
        if (v == "false" || v == "no" || v == "off" || v == "0") return false;
        return dflt;
    }
};

}  // namespace

// QoZ::Config::loadcfg (include/QoZ/utils/Config.hpp:91-233), the keys this
// library's configuration carries.
int config_load_ini(faz_config *c, const char *path, std::string &err) {
    Ini ini;
    if (!path || !ini.load(path)) {
        err = std::string("Can't load cfg file ") + (path ? path : "(null)");
        return FAZ_ERR_ARG;
    }
    const char *G = "GlobalSettings", *A = "AlgoSettings";
    static const char *algo[] = {"ALGO_LORENZO_REG", "ALGO_INTERP_LORENZO", "ALGO_INTERP", "ALGO_INTERP_BLOCKED"};
    std::string s = ini.get(G, "CmprAlgo");
    for (int i = 0; i < 4; i++)
        if (s == algo[i]) c->cmprAlgo = (uint8_t)i;
    static const char *ebs[] = {"ABS", "REL", "PSNR", "NORM", "ABS_AND_REL", "ABS_OR_REL"};
    s = ini.get(G, "ErrorBoundMode");
    for (int i = 0; i < 6; i++)
        if (s == ebs[i]) c->errorBoundMode = (uint8_t)i;
    static const char *tts[] = {"TUNING_TARGET_RD", "TUNING_TARGET_CR", "TUNING_TARGET_SSIM", "TUNING_TARGET_AC"};
    s = ini.get(G, "tuningTarget");
    for (int i = 0; i < 4; i++)
        if (s == tts[i]) c->tuningTarget = (uint8_t)i;
    c->absErrorBound = ini.real(G, "AbsErrorBound", c->absErrorBound);
    c->relErrorBound = ini.real(G, "RelErrorBound", c->relErrorBound);
    c->psnrErrorBound = ini.real(G, "PSNRErrorBound", c->psnrErrorBound);
    c->l2normErrorBound = ini.real(G, "L2NormErrorBound", c->l2normErrorBound);
    c->alpha = ini.real(A, "alpha", c->alpha);
    c->beta = ini.real(A, "beta", c->beta);
    c->autoTuningRate = ini.real(A, "autoTuningRate", c->autoTuningRate);
    c->predictorTuningRate = ini.real(A, "predictorTuningRate", c->predictorTuningRate);
    c->wavelet_rel_coeff = ini.real(A, "wavelet_rel_coeff", c->wavelet_rel_coeff);
    c->preTrim = ini.real(A, "preTrim", c->preTrim);
    c->openmp = ini.boolean(G, "OpenMP", c->openmp);
    c->lorenzo = ini.boolean(A, "Lorenzo", c->lorenzo);
    c->lorenzo2 = ini.boolean(A, "Lorenzo2ndOrder", c->lorenzo2);
    c->regression = ini.boolean(A, "Regression", c->regression);
    c->regression2 = ini.boolean(A, "Regression2ndOrder", c->regression2);
    s = ini.get(A, "InterpolationAlgo");
    if (s == "INTERP_ALGO_LINEAR") c->interpAlgo = FAZ_INTERP_ALGO_LINEAR;
    else if (s == "INTERP_ALGO_CUBIC") c->interpAlgo = FAZ_INTERP_ALGO_CUBIC;
    c->interpDirection = (uint8_t)ini.integer(A, "InterpDirection", c->interpDirection);
    c->interpBlockSize = (int32_t)ini.integer(A, "InterpBlockSize", c->interpBlockSize);
    c->blockSize = (int32_t)ini.integer(A, "BlockSize", c->blockSize);
    c->quantbinCnt = (int32_t)ini.integer(A, "QuantizationBinTotal", c->quantbinCnt);
    c->maxStep = (uint64_t)ini.integer(A, "maxStep", (long)c->maxStep);
    c->sampleBlockSize = (int32_t)ini.integer(A, "sampleBlockSize", c->sampleBlockSize);
    c->levelwisePredictionSelection =
        (int32_t)ini.integer(A, "levelwisePredictionSelection", c->levelwisePredictionSelection);
    c->testLorenzo = (int32_t)ini.integer(A, "testLorenzo", c->testLorenzo);
    c->profiling = (int32_t)ini.integer(A, "profiling", c->profiling);
    c->var_first = (int32_t)ini.integer(A, "var_first", c->var_first);
    c->abList = (int32_t)ini.integer(A, "abList", c->abList);
    c->SSIMBlockSize = (int32_t)ini.integer(A, "SSIMBlockSize", c->SSIMBlockSize);
    c->fixBlockSize = (int32_t)ini.integer(A, "fixBlockSize", c->fixBlockSize);
    c->verbose = ini.boolean(A, "verbose", c->verbose);
    c->QoZ = ini.boolean(A, "QoZ", c->QoZ);
    c->FZ = ini.boolean(A, "FZ", c->FZ);
    c->sperrWithoutWave = ini.boolean(A, "sperrWithoutWave", c->sperrWithoutWave);
    c->pyBind = ini.boolean(A, "pyBind", c->pyBind);
    c->blockwiseSampleBlockSize = (int32_t)ini.integer(A, "blockwiseSampleBlockSize", c->blockwiseSampleBlockSize);
    c->crossBlock = (int32_t)ini.integer(A, "crossBlock", c->crossBlock);
    c->sampleBlockSampleBlockSize =
        (int32_t)ini.integer(A, "sampleBlockSampleBlockSize", c->sampleBlockSampleBlockSize);
    c->peTracking = ini.boolean(A, "peTracking", c->peTracking);
    c->wavelet = (int32_t)ini.integer(A, "wavelet", c->wavelet);
    c->offsetPredictor = (int32_t)ini.integer(A, "offsetPredictor", c->offsetPredictor);
    c->trimToZero = (int32_t)ini.integer(A, "trimToZero", c->trimToZero);
    c->pid = (int32_t)ini.integer(A, "pid", c->pid);
    c->blockOrder = (int32_t)ini.integer(A, "blockOrder", c->blockOrder);
    c->sperr = (int32_t)ini.integer(A, "sperr", c->sperr);
    c->conditioning = (int32_t)ini.integer(A, "conditioning", c->conditioning);
    return FAZ_OK;
}

namespace {
template <typename V>
void put(std::vector<uint8_t> &o, V v) {
    uint8_t b[sizeof(V)];
    std::memcpy(b, &v, sizeof(V));
    o.insert(o.end(), b, b + sizeof(V));
}
struct Reader {
    const uint8_t *p;
    size_t n, pos = 0;
    bool bad = false;
    template <typename V>
    V get() {
        V v{};
        if (pos + sizeof(V) > n) {
            bad = true;
            return v;
        }
        std::memcpy(&v, p + pos, sizeof(V));
        pos += sizeof(V);
        return v;
    }
};
}  // namespace

// QoZ::Config::save (include/QoZ/utils/Config.hpp:240-309).  firstSize is
// never assigned on this path in the reference; it is written as 0 here.
void config_save(const faz_config &c, std::vector<uint8_t> &o) {
    put<char>(o, (char)c.N);
    for (int i = 0; i < c.N; i++) put<uint64_t>(o, c.dims[i]);
    put<uint64_t>(o, c.num);
    put<uint8_t>(o, c.cmprAlgo);
    put<uint8_t>(o, c.errorBoundMode);
    put<uint8_t>(o, c.tuningTarget);
    put<double>(o, c.absErrorBound);
    put<double>(o, c.relErrorBound);
    put<double>(o, c.alpha);
    put<double>(o, c.beta);
    put<uint8_t>(o, c.lorenzo);
    put<uint8_t>(o, c.lorenzo2);
    put<uint8_t>(o, c.regression);
    put<uint8_t>(o, c.regression2);
    put<uint8_t>(o, c.interpAlgo);
    put<uint8_t>(o, c.interpDirection);
    put<int32_t>(o, c.interpBlockSize);
    put<uint8_t>(o, c.lossless);
    put<uint8_t>(o, c.encoder);
    put<int32_t>(o, c.quantbinCnt);
    put<int32_t>(o, c.blockSize);
    put<int32_t>(o, c.levelwisePredictionSelection);
    put<uint8_t>(o, c.blockwiseTuning);
    put<int32_t>(o, c.stride);
    put<uint64_t>(o, c.maxStep);
    put<int32_t>(o, c.pred_dim);
    put<uint8_t>(o, c.openmp);
    put<int32_t>(o, c.fixBlockSize);
    put<int32_t>(o, c.blockwiseSampleBlockSize);
    put<int32_t>(o, c.crossBlock);
    put<int32_t>(o, c.wavelet);
    put<uint64_t>(o, 0);  // firstSize
    put<int32_t>(o, c.offsetPredictor);
    put<uint64_t>(o, c.coeffs_num);
    if (c.coeffs_num > 0) {
        put<uint64_t>(o, (uint64_t)c.coeffs_dims_len);
        for (int i = 0; i < c.coeffs_dims_len; i++) put<uint64_t>(o, c.coeffs_dims[i]);
    }
    put<int32_t>(o, c.pid);
    put<int32_t>(o, c.blockOrder);
    put<int32_t>(o, c.sperr);
    put<uint8_t>(o, c.sperrWithoutWave);
    put<uint8_t>(o, c.pyBind);
    if (c.pyBind) put<uint64_t>(o, 0);  // metadata string (empty)
    put<int32_t>(o, c.conditioning);
    if (c.conditioning > 0) o.insert(o.end(), c.meta, c.meta + 17);
}

// QoZ::Config::load (include/QoZ/utils/Config.hpp:311-388)
int config_load(faz_config &c, const uint8_t *p, size_t n, size_t *used) {
    Reader r{p, n};
    faz_config t;
    std::memset(&t, 0, sizeof(t));
    t.N = r.get<char>();
    if (t.N < 1 || t.N > 4) return FAZ_ERR_FORMAT;
    for (int i = 0; i < t.N; i++) t.dims[i] = r.get<uint64_t>();
    t.num = r.get<uint64_t>();
    t.cmprAlgo = r.get<uint8_t>();
    t.errorBoundMode = r.get<uint8_t>();
    t.tuningTarget = r.get<uint8_t>();
    t.absErrorBound = r.get<double>();
    t.relErrorBound = r.get<double>();
    t.alpha = r.get<double>();
    t.beta = r.get<double>();
    t.lorenzo = r.get<uint8_t>();
    t.lorenzo2 = r.get<uint8_t>();
    t.regression = r.get<uint8_t>();
    t.regression2 = r.get<uint8_t>();
    t.interpAlgo = r.get<uint8_t>();
    t.interpDirection = r.get<uint8_t>();
    t.interpBlockSize = r.get<int32_t>();
    t.lossless = r.get<uint8_t>();
    t.encoder = r.get<uint8_t>();
    t.quantbinCnt = r.get<int32_t>();
    t.blockSize = r.get<int32_t>();
    t.levelwisePredictionSelection = r.get<int32_t>();
    t.blockwiseTuning = r.get<uint8_t>();
    t.stride = r.get<int32_t>();
    t.maxStep = r.get<uint64_t>();
    t.pred_dim = r.get<int32_t>();
    t.openmp = r.get<uint8_t>();
    t.fixBlockSize = r.get<int32_t>();
    t.blockwiseSampleBlockSize = r.get<int32_t>();
    t.crossBlock = r.get<int32_t>();
    t.wavelet = r.get<int32_t>();
    t.firstSize = r.get<uint64_t>();
    t.offsetPredictor = r.get<int32_t>();
    t.coeffs_num = r.get<uint64_t>();
    if (t.coeffs_num > 0) {
        uint64_t len = r.get<uint64_t>();
        if (len > 4) return FAZ_ERR_FORMAT;
        t.coeffs_dims_len = (int32_t)len;
        for (uint64_t i = 0; i < len; i++) t.coeffs_dims[i] = r.get<uint64_t>();
    }
    t.pid = r.get<int32_t>();
    t.blockOrder = r.get<int32_t>();
    t.sperr = r.get<int32_t>();
    t.sperrWithoutWave = r.get<uint8_t>();
    t.pyBind = r.get<uint8_t>();
    if (t.pyBind) {
        uint64_t ms = r.get<uint64_t>();
        if (ms > n) return FAZ_ERR_FORMAT;
        r.pos += ms;
    }
    t.conditioning = r.get<int32_t>();
    if (t.conditioning > 0) {
        for (int i = 0; i < 17; i++) t.meta[i] = r.get<uint8_t>();
    }
    if (r.bad) return FAZ_ERR_FORMAT;
    uint64_t num = 1;
    for (int i = 0; i < t.N; i++) num *= t.dims[i];
    if (num != t.num) return FAZ_ERR_FORMAT;
    // fields the trailer does not carry keep their defaults
    t.rng = -1;
    t.SSIMBlockSize = 8;
    t.verbose = 1;
    t.wavelet_rel_coeff = 0.75;
    c = t;
    if (used) *used = r.pos;
    return FAZ_OK;
}

// ------------------------------------------------------------------- zstd
// The reference links zstd (its bundled 1.4.5 when no system copy is found)
// and calls ZSTD_compress at level 3 (include/QoZ/lossless/Lossless_zstd.hpp:22-54).
// This library loads the host's libzstd at run time (FAZ_ZSTD_LIBRARY
// overrides the default libzstd.so.1).
const Zstd &zstd_lib(std::string &err) {
    static Zstd z;
    static std::once_flag once;
    static std::string load_err;
    std::call_once(once, [] {
        const char *path = std::getenv("FAZ_ZSTD_LIBRARY");
        if (!path || !*path) path = "libzstd.so.1";
        void *h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
        if (!h) {
            load_err = std::string("cannot load zstd library ") + path;
            return;
        }
        z.compress = (size_t(*)(void *, size_t, const void *, size_t, int))dlsym(h, "ZSTD_compress");
        z.decompress = (size_t(*)(void *, size_t, const void *, size_t))dlsym(h, "ZSTD_decompress");
        z.isError = (unsigned (*)(size_t))dlsym(h, "ZSTD_isError");
        z.bound = (size_t(*)(size_t))dlsym(h, "ZSTD_compressBound");
        auto ver = (unsigned (*)(void))dlsym(h, "ZSTD_versionNumber");
        if (!z.compress || !z.decompress || !z.isError || !z.bound || !ver) {
            load_err = "zstd library lacks ZSTD_compress/ZSTD_decompress";
            return;
        }
        z.version = ver();
        z.findFrameCompressedSize = (size_t(*)(const void *, size_t))dlsym(h, "ZSTD_findFrameCompressedSize");
        z.getFrameContentSize = (unsigned long long (*)(const void *, size_t))dlsym(h, "ZSTD_getFrameContentSize");
        z.createCCtx = (void *(*)())dlsym(h, "ZSTD_createCCtx");
        z.freeCCtx = (size_t(*)(void *))dlsym(h, "ZSTD_freeCCtx");
        z.setParameter = (size_t(*)(void *, int, int))dlsym(h, "ZSTD_CCtx_setParameter");
        z.compress2 = (size_t(*)(void *, void *, size_t, const void *, size_t))dlsym(h, "ZSTD_compress2");
        z.compressCCtx = (size_t(*)(void *, void *, size_t, const void *, size_t, int))dlsym(h, "ZSTD_compressCCtx");
        z.ok = true;
    });
    if (!z.ok) err = load_err;
    return z;
}

// The tuner's trials need the size of the frame ZSTD_compress writes for
// each trial payload; ZSTD_compressCCtx writes the same frame with a context
// that this thread keeps, and the output goes to a buffer it keeps too (a
// fresh context and a zero-filled buffer per call cost more than the
// compression of a small payload).
size_t zstd_level3_size(const Zstd &z, const void *src, size_t n) {
    struct Scratch {
        const Zstd *z = nullptr;
        void *cctx = nullptr;
        std::unique_ptr<uint8_t[]> buf;
        size_t cap = 0;
        ~Scratch() {
            if (cctx && z && z->freeCCtx) z->freeCCtx(cctx);
        }
    };
    thread_local Scratch s;
    const size_t need = z.bound(n) + 1;
    if (need > s.cap) {
        s.buf.reset(new uint8_t[need]);
        s.cap = need;
    }
    if (z.compressCCtx && z.createCCtx && z.freeCCtx) {
        if (!s.cctx) {
            s.cctx = z.createCCtx();
            s.z = &z;
        }
        if (s.cctx) return z.compressCCtx(s.cctx, s.buf.get(), s.cap, src, n, 3);
    }
    return z.compress(s.buf.get(), s.cap, src, n, 3);
}

int zstd_threads() {
    int t = (int)std::min<unsigned>(16u, std::max(1u, std::thread::hardware_concurrency()));
    if (const char *env = std::getenv("FAZ_ZSTD_THREADS")) t = std::atoi(env);
    return t < 0 ? 0 : t;
}

namespace {

int zstd_frame_count(size_t n, int threads) {
    if (threads <= 0) return 1;
    const size_t kMinFrame = (size_t)4 << 20;  // slices of at least 4 MiB
    size_t nf = n / kMinFrame;
    if (nf > (size_t)(2 * threads)) nf = (size_t)(2 * threads);
    return nf < 1 ? 1 : (int)nf;
}

// Stable parameter ids of zstd's advanced API (zstd.h, ZSTD_cParameter).
constexpr int kZstdLevel = 100, kZstdWorkers = 400, kZstdJobSize = 401, kZstdOverlapLog = 402;

// Compression context of the calling thread, kept between calls (its worker
// pool and buffers survive).
struct CCtxHolder {
    const Zstd *z = nullptr;
    void *cctx = nullptr;
    ~CCtxHolder() {
        if (cctx && z) z->freeCCtx(cctx);
    }
};

size_t compress_workers(const Zstd &z, uint8_t *dst, size_t cap, const uint8_t *src, size_t n, int workers, int job) {
    thread_local CCtxHolder h;
    if (!h.cctx) {
        h.z = &z;
        h.cctx = z.createCCtx();
        if (!h.cctx) return (size_t)-1;
    }
    if (z.isError(z.setParameter(h.cctx, kZstdLevel, 3)) || z.isError(z.setParameter(h.cctx, kZstdWorkers, workers)) ||
        z.isError(z.setParameter(h.cctx, kZstdJobSize, job)) || z.isError(z.setParameter(h.cctx, kZstdOverlapLog, 0)))
        return (size_t)-1;
    return z.compress2(h.cctx, dst, cap, src, n);
}

size_t compress_frames(const Zstd &z, uint8_t *dst, size_t cap, const uint8_t *src, size_t n, int nframes,
                       bool parallel) {
    if (nframes <= 1) return z.compress(dst, cap, src, n, 3);
    const size_t slice = (n + nframes - 1) / nframes;
    struct Part {
        size_t lo, len, size = 0, off = 0;
        std::unique_ptr<uint8_t[]> buf;
    };
    std::vector<Part> parts(nframes);
    for (int i = 0; i < nframes; i++) {
        parts[i].lo = std::min(n, slice * i);
        parts[i].len = std::min(n, parts[i].lo + slice) - parts[i].lo;
    }
    auto each = [&](auto &&fn) {
        if (!parallel) {
            for (int i = 0; i < nframes; i++) fn(i);
            return;
        }
        std::vector<std::thread> pool;
        for (int i = 0; i < nframes; i++) pool.emplace_back(fn, i);
        for (auto &t : pool) t.join();
    };
    each([&](int i) {
        Part &p = parts[i];
        const size_t b = z.bound(p.len);
        p.buf.reset(new (std::nothrow) uint8_t[b]);
        p.size = p.buf ? z.compress(p.buf.get(), b, src + p.lo, p.len, 3) : (size_t)-1;
    });
    size_t o = 0;
    for (auto &p : parts) {
        if (z.isError(p.size)) return p.size;
        p.off = o;
        o += p.size;
    }
    if (o > cap) return (size_t)-1;
    each([&](int i) { std::memcpy(dst + parts[i].off, parts[i].buf.get(), parts[i].size); });
    return o;
}

}  // namespace

ZstdPlan zstd_plan(size_t n) {
    std::string err;
    const Zstd &z = zstd_lib(err);
    ZstdPlan p;
    p.threads = zstd_threads();
    if (p.threads <= 0) return p;  // Single
    const char *mf = std::getenv("FAZ_ZSTD_MULTIFRAME");
    if (mf && mf[0] == '1') {
        p.mode = ZstdMode::Frames;
        p.nframes = zstd_frame_count(n, p.threads);
        if (p.nframes <= 1) p.mode = ZstdMode::Single;
        return p;
    }
    const size_t kJobMin = (size_t)1 << 20, kJobMax = (size_t)8 << 20;
    if (!z.ok || !z.createCCtx || !z.setParameter || !z.compress2 || n < 2 * kJobMin) return p;  // Single
    // jobs of a size that depends on n alone (about 64 of them), so that the
    // frame is the same for any worker count
    size_t job = std::min(kJobMax, std::max(kJobMin, n / 64));
    p.mode = ZstdMode::Workers;
    p.job = (int)job;
    return p;
}

size_t zstd_body_bound(const Zstd &z, size_t n, const ZstdPlan &p) {
    if (p.mode != ZstdMode::Frames || p.nframes <= 1) return z.bound(n);
    size_t b = 0;
    const size_t slice = (n + p.nframes - 1) / p.nframes;
    for (int i = 0; i < p.nframes; i++) {
        const size_t lo = std::min(n, slice * i), hi = std::min(n, lo + slice);
        b += z.bound(hi - lo);
    }
    return b;
}

size_t zstd_compress_body(const Zstd &z, uint8_t *dst, size_t cap, const uint8_t *src, size_t n, const ZstdPlan &p,
                          bool parallel) {
    switch (p.mode) {
    case ZstdMode::Workers:
        return compress_workers(z, dst, cap, src, n, parallel ? p.threads : 1, p.job);
    case ZstdMode::Frames:
        return compress_frames(z, dst, cap, src, n, p.nframes, parallel);
    default:
        return z.compress(dst, cap, src, n, 3);
    }
}

size_t zstd_decompress_frames(const Zstd &z, uint8_t *dst, size_t raw, const uint8_t *src, size_t n, int threads) {
    struct Frame {
        size_t off, csize, out, dsize;
    };
    std::vector<Frame> fr;
    if (z.findFrameCompressedSize && z.getFrameContentSize && threads > 0) {
        size_t off = 0, out = 0;
        while (off < n) {
            const size_t fs = z.findFrameCompressedSize(src + off, n - off);
            if (z.isError(fs) || fs == 0) {
                fr.clear();
                break;
            }
            const unsigned long long ds = z.getFrameContentSize(src + off, fs);
            if (ds >= (1ull << 62)) {  // unknown or error: decode the whole body in one call
                fr.clear();
                break;
            }
            fr.push_back({off, fs, out, (size_t)ds});
            off += fs;
            out += (size_t)ds;
        }
        if (out != raw) fr.clear();
    }
    if (fr.size() <= 1) return z.decompress(dst, raw, src, n);
    std::vector<size_t> got(fr.size(), 0);
    std::vector<std::thread> pool;
    const size_t nt = std::min<size_t>(fr.size(), (size_t)threads);
    for (size_t t = 0; t < nt; t++) {
        pool.emplace_back([&, t] {
            for (size_t i = t; i < fr.size(); i += nt)
                got[i] = z.decompress(dst + fr[i].out, fr[i].dsize, src + fr[i].off, fr[i].csize);
        });
    }
    for (auto &t : pool) t.join();
    for (size_t i = 0; i < fr.size(); i++)
        if (z.isError(got[i]) || got[i] != fr[i].dsize) return (size_t)-1;
    return raw;
}

}  // namespace faz
