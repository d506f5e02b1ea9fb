/*
 * faz_gb300.hpp - the reference's C++ API (namespace QoZ, SZ_compress /
 * SZ_decompress templates) over the C ABI of faz_gb300.h, so that code
 * written against include/QoZ/api/sz.hpp compiles unchanged:
 *
 *   QoZ::Config conf(100, 200, 300);          // 300 is the fastest dimension
 *   conf.errorBoundMode = QoZ::EB_REL;
 *   conf.relErrorBound = 1e-3;
 *   size_t outSize;
 *   char *cmp = SZ_compress(conf, data, outSize);   // release with delete[]
 *   float *dec = SZ_decompress<float>(conf, cmp, outSize);  // delete[]
 *
 * Config mirrors QoZ::Config (include/QoZ/utils/Config.hpp:61-499): the same
 * member names, meaning and defaults for every field the compressor reads
 * or writes to the stream trailer.  Errors that the reference answers with
 * exit(0) throw QoZ::Error here.
 */
#ifndef FAZ_GB300_HPP
#define FAZ_GB300_HPP

#include <array>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "faz_gb300.h"

namespace QoZ {

enum EB { EB_ABS, EB_REL, EB_PSNR, EB_L2NORM, EB_ABS_AND_REL, EB_ABS_OR_REL };
constexpr const char *EB_STR[] = {"ABS", "REL", "PSNR", "NORM", "ABS_AND_REL", "ABS_OR_REL"};
enum ALGO { ALGO_LORENZO_REG, ALGO_INTERP_LORENZO, ALGO_INTERP, ALGO_INTERP_BLOCKED };
constexpr const char *ALGO_STR[] = {"ALGO_LORENZO_REG", "ALGO_INTERP_LORENZO", "ALGO_INTERP", "ALGO_INTERP_BLOCKED"};
enum INTERP_ALGO { INTERP_ALGO_LINEAR, INTERP_ALGO_CUBIC };
constexpr const char *INTERP_ALGO_STR[] = {"INTERP_ALGO_LINEAR", "INTERP_ALGO_CUBIC"};
enum TUNING_TARGET { TUNING_TARGET_RD, TUNING_TARGET_CR, TUNING_TARGET_SSIM, TUNING_TARGET_AC };
constexpr const char *TUNING_TARGET_STR[] = {"TUNING_TARGET_RD", "TUNING_TARGET_CR", "TUNING_TARGET_SSIM",
                                             "TUNING_TARGET_AC"};

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
    if (rc != FAZ_OK) throw Error(rc, faz_last_error());
}

class Config {
  public:
    char N = 0;
    std::vector<size_t> dims;
    size_t num = 0;
    uint8_t cmprAlgo = ALGO_INTERP_LORENZO;
    uint8_t errorBoundMode = EB_ABS;
    uint8_t tuningTarget = TUNING_TARGET_RD;
    double absErrorBound = 0;
    double relErrorBound = -1.0;
    double psnrErrorBound = 0;
    double l2normErrorBound = 0;
    double rng = -1;
    double alpha = -1;
    double beta = -1;
    double autoTuningRate = 0.0;
    double predictorTuningRate = 0.0;
    bool lorenzo = true;
    bool lorenzo2 = false;
    bool regression = true;
    bool regression2 = false;
    bool openmp = false;
    uint8_t lossless = 1;
    uint8_t encoder = 1;
    uint8_t interpAlgo = INTERP_ALGO_CUBIC;
    uint8_t interpDirection = 0;
    int levelwisePredictionSelection = 0;
    std::vector<uint8_t> interpAlgo_list;
    std::vector<uint8_t> interpDirection_list;
    size_t maxStep = 0;
    int interpBlockSize = 32;
    int quantbinCnt = 65536;
    int blockSize = 0;
    int testLorenzo = 0;
    int sampleBlockSize = 0;
    bool blockwiseTuning = 0;
    int stride = 0;
    int pred_dim = 0;
    int profiling = 0;
    int var_first = 0;
    int SSIMBlockSize = 8;
    int fixBlockSize = 0;
    int blockwiseSampleBlockSize = 0;
    bool verbose = 1;
    bool QoZ = 0;
    int abList = 0;
    int crossBlock = 0;
    int sampleBlockSampleBlockSize = 0;
    bool peTracking = 0;
    int wavelet = 0;
    std::vector<size_t> coeffs_dims;
    size_t coeffs_num = 0;
    double wavelet_rel_coeff = 0.75;
    size_t firstSize = 0;
    int pid = 0;
    int offsetPredictor = 0;
    int trimToZero = 0;
    double preTrim = 0.0;
    int blockOrder = 0;
    int sperr = -1;
    int conditioning = 0;
    std::array<uint8_t, 17> meta{};
    bool sperrWithoutWave = false;
    bool pyBind = true;
    bool pybind_activated = false;
    bool FZ = false;

    Config() = default;

    // Config(Dims...) - Config.hpp:64-74; dims[0] is the slowest dimension
    template <class... Dims, typename = typename std::enable_if<(sizeof...(Dims) >= 1)>::type>
    explicit Config(Dims... args) {
        std::vector<size_t> d{static_cast<size_t>(args)...};
        init(d);
    }

    // Config::setDims (Config.hpp:77-89)
    template <class Iter>
    size_t setDims(Iter begin, Iter end) {
        dims = std::vector<size_t>(begin, end);
        coeffs_dims = dims;
        N = (char)dims.size();
        num = 1;
        for (size_t d : dims) num *= d;
        coeffs_num = num;
        blockSize = (N == 1 ? 128 : (N == 2 ? 16 : 6));
        pred_dim = N;
        stride = blockSize;
        return num;
    }

    // Config::loadcfg (Config.hpp:91-233)
    void loadcfg(const std::string &path) {
        faz_config c = to_c();
        check(faz_config_load_ini(&c, path.c_str()));
        from_c(c);
    }

    faz_config to_c() const {
        faz_config c;
        std::memset(&c, 0, sizeof(c));
        if (dims.empty() || dims.size() > 4) throw Error(FAZ_ERR_ARG, "Config needs 1 to 4 dimensions");
        c.N = (int32_t)N;
        for (size_t i = 0; i < dims.size(); i++) c.dims[i] = dims[i];
        c.num = num;
        c.cmprAlgo = cmprAlgo;
        c.errorBoundMode = errorBoundMode;
        c.tuningTarget = tuningTarget;
        c.absErrorBound = absErrorBound;
        c.relErrorBound = relErrorBound;
        c.psnrErrorBound = psnrErrorBound;
        c.l2normErrorBound = l2normErrorBound;
        c.rng = rng;
        c.alpha = alpha;
        c.beta = beta;
        c.autoTuningRate = autoTuningRate;
        c.predictorTuningRate = predictorTuningRate;
        c.lorenzo = lorenzo;
        c.lorenzo2 = lorenzo2;
        c.regression = regression;
        c.regression2 = regression2;
        c.openmp = openmp;
        c.lossless = lossless;
        c.encoder = encoder;
        c.interpAlgo = interpAlgo;
        c.interpDirection = interpDirection;
        c.levelwisePredictionSelection = levelwisePredictionSelection;
        if (interpAlgo_list.size() != interpDirection_list.size() || interpAlgo_list.size() > FAZ_MAX_LEVELS)
            throw Error(FAZ_ERR_ARG, "interpAlgo_list and interpDirection_list must have equal length <= 64");
        c.interp_list_len = (int32_t)interpAlgo_list.size();
        for (size_t i = 0; i < interpAlgo_list.size(); i++) {
            c.interpAlgo_list[i] = interpAlgo_list[i];
            c.interpDirection_list[i] = interpDirection_list[i];
        }
        c.maxStep = maxStep;
        c.interpBlockSize = interpBlockSize;
        c.quantbinCnt = quantbinCnt;
        c.blockSize = blockSize;
        c.testLorenzo = testLorenzo;
        c.sampleBlockSize = sampleBlockSize;
        c.blockwiseTuning = blockwiseTuning;
        c.stride = stride;
        c.pred_dim = pred_dim;
        c.profiling = profiling;
        c.var_first = var_first;
        c.SSIMBlockSize = SSIMBlockSize;
        c.fixBlockSize = fixBlockSize;
        c.blockwiseSampleBlockSize = blockwiseSampleBlockSize;
        c.verbose = verbose;
        c.QoZ = QoZ;
        c.FZ = FZ;
        c.abList = abList;
        c.crossBlock = crossBlock;
        c.sampleBlockSampleBlockSize = sampleBlockSampleBlockSize;
        c.peTracking = peTracking;
        c.wavelet = wavelet;
        c.coeffs_num = coeffs_num;
        c.coeffs_dims_len = (int32_t)coeffs_dims.size();
        for (size_t i = 0; i < coeffs_dims.size() && i < 4; i++) c.coeffs_dims[i] = coeffs_dims[i];
        c.wavelet_rel_coeff = wavelet_rel_coeff;
        c.firstSize = firstSize;
        c.pid = pid;
        c.offsetPredictor = offsetPredictor;
        c.trimToZero = trimToZero;
        c.preTrim = preTrim;
        c.blockOrder = blockOrder;
        c.sperr = sperr;
        c.sperrWithoutWave = sperrWithoutWave;
        c.pyBind = pyBind;
        c.conditioning = conditioning;
        std::memcpy(c.meta, meta.data(), 17);
        c.pybind_activated = pybind_activated;
        return c;
    }

    void from_c(const faz_config &c) {
        N = (char)c.N;
        dims.assign(c.dims, c.dims + c.N);
        num = c.num;
        cmprAlgo = c.cmprAlgo;
        errorBoundMode = c.errorBoundMode;
        tuningTarget = c.tuningTarget;
        absErrorBound = c.absErrorBound;
        relErrorBound = c.relErrorBound;
        psnrErrorBound = c.psnrErrorBound;
        l2normErrorBound = c.l2normErrorBound;
        rng = c.rng;
        alpha = c.alpha;
        beta = c.beta;
        autoTuningRate = c.autoTuningRate;
        predictorTuningRate = c.predictorTuningRate;
        lorenzo = c.lorenzo;
        lorenzo2 = c.lorenzo2;
        regression = c.regression;
        regression2 = c.regression2;
        openmp = c.openmp;
        lossless = c.lossless;
        encoder = c.encoder;
        interpAlgo = c.interpAlgo;
        interpDirection = c.interpDirection;
        levelwisePredictionSelection = c.levelwisePredictionSelection;
        interpAlgo_list.assign(c.interpAlgo_list, c.interpAlgo_list + c.interp_list_len);
        interpDirection_list.assign(c.interpDirection_list, c.interpDirection_list + c.interp_list_len);
        maxStep = c.maxStep;
        interpBlockSize = c.interpBlockSize;
        quantbinCnt = c.quantbinCnt;
        blockSize = c.blockSize;
        testLorenzo = c.testLorenzo;
        sampleBlockSize = c.sampleBlockSize;
        blockwiseTuning = c.blockwiseTuning;
        stride = c.stride;
        pred_dim = c.pred_dim;
        profiling = c.profiling;
        var_first = c.var_first;
        SSIMBlockSize = c.SSIMBlockSize;
        fixBlockSize = c.fixBlockSize;
        blockwiseSampleBlockSize = c.blockwiseSampleBlockSize;
        verbose = c.verbose;
        QoZ = c.QoZ;
        FZ = c.FZ;
        abList = c.abList;
        crossBlock = c.crossBlock;
        sampleBlockSampleBlockSize = c.sampleBlockSampleBlockSize;
        peTracking = c.peTracking;
        wavelet = c.wavelet;
        coeffs_num = c.coeffs_num;
        coeffs_dims.assign(c.coeffs_dims, c.coeffs_dims + (c.coeffs_dims_len > 4 ? 4 : c.coeffs_dims_len));
        wavelet_rel_coeff = c.wavelet_rel_coeff;
        firstSize = c.firstSize;
        pid = c.pid;
        offsetPredictor = c.offsetPredictor;
        trimToZero = c.trimToZero;
        preTrim = c.preTrim;
        blockOrder = c.blockOrder;
        sperr = c.sperr;
        sperrWithoutWave = c.sperrWithoutWave;
        pyBind = c.pyBind;
        conditioning = c.conditioning;
        std::memcpy(meta.data(), c.meta, 17);
        pybind_activated = c.pybind_activated;
    }

  private:
    void init(const std::vector<size_t> &d) {
        if (d.empty() || d.size() > 4) throw Error(FAZ_ERR_ARG, "Config needs 1 to 4 dimensions");
        uint64_t dd[4] = {0, 0, 0, 0};
        for (size_t i = 0; i < d.size(); i++) dd[i] = d[i];
        faz_config c;
        check(faz_config_init(&c, (int)d.size(), dd));
        from_c(c);
    }
};

template <class T>
constexpr int dtype_of() {
    static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value,
                  "FAZ compresses float or double data");
    return std::is_same<T, float>::value ? FAZ_FLOAT : FAZ_DOUBLE;
}

}  // namespace QoZ

// SZ_compress<T> (include/QoZ/api/sz.hpp:54-108): the stream in a new[]
// buffer (release with delete[]); config.pybind_activated is the only field
// written back, as in the reference.
template <class T>
char *SZ_compress(QoZ::Config &config, const T *data, size_t &outSize) {
    faz_config c = config.to_c();
    char *out = nullptr;
    QoZ::check(faz_compress(&c, QoZ::dtype_of<T>(), data, &out, &outSize, nullptr));
    char *r = new char[outSize];
    std::memcpy(r, out, outSize);
    faz_free(out);
    return r;
}

// SZ_decompress<T> (sz.hpp:159-205): conf receives the stream's
// configuration; decData is allocated with new[] when it is nullptr, and
// must otherwise hold the stream's field.
template <class T>
void SZ_decompress(QoZ::Config &conf, char *cmpData, size_t cmpSize, T *&decData) {
    faz_config c;
    QoZ::check(faz_stream_info(cmpData, cmpSize, &c));
    const uint64_t num = c.num;
    bool alloc = decData == nullptr;
    if (alloc) decData = new T[num];
    void *out = decData;
    c.num = num;  // capacity of the output
    int rc = faz_decompress(&c, QoZ::dtype_of<T>(), cmpData, cmpSize, &out, nullptr);
    if (rc != FAZ_OK) {
        if (alloc) {
            delete[] decData;
            decData = nullptr;
        }
        QoZ::check(rc);
    }
    conf.from_c(c);
}

// SZ_decompress<T> (sz.hpp:220-225): a new[] array of the stream's field.
template <class T>
T *SZ_decompress(QoZ::Config &conf, char *cmpData, size_t cmpSize) {
    T *decData = nullptr;
    SZ_decompress<T>(conf, cmpData, cmpSize, decData);
    return decData;
}

#endif  // FAZ_GB300_HPP
