/*
 * faz_gb300.h - C ABI of the GB300-native FAZ interpolation compressor.
 *
 * The entry points below are what a foreign-function binding of FAZ's
 * compress/decompress path attaches to.  They replace the C++ template
 * entry points of the reference:
 *
 *   template<class T> char *SZ_compress(QoZ::Config&, const T*, size_t&)
 *       include/QoZ/api/sz.hpp:54-108           -> faz_compress()
 *   template<class T> void SZ_decompress(QoZ::Config&, char*, size_t, T*&)
 *       include/QoZ/api/sz.hpp:159-205          -> faz_decompress()
 *   template<class T> T *SZ_decompress(QoZ::Config&, char*, size_t)
 *       include/QoZ/api/sz.hpp:220-225          -> faz_decompress() with *out == NULL
 *   QoZ::Config::Config(Dims...)  include/QoZ/utils/Config.hpp:64-74  -> faz_config_init()
 *   QoZ::Config::loadcfg(path)    include/QoZ/utils/Config.hpp:91-233 -> faz_config_load_ini()
 *   QoZ::calAbsErrorBound         include/QoZ/utils/Statistic.hpp:34-66 (run inside faz_compress)
 *
 * Plain C types only: pointers, sizes and a POD configuration struct whose
 * fields carry the names, meaning and defaults of QoZ::Config.
 *
 * Ownership: buffers returned through `char **out` / `void **out` are
 * allocated by the library and released with faz_free().
 * Errors: every call returns FAZ_OK (0) or a negative status; the message of
 * the last failure on the calling thread is available from faz_last_error().
 * The reference terminates the process on bad input (e.g.
 * include/QoZ/api/impl/SZDispatcher.hpp:49-50); this library returns instead.
 * Threading: calls on different threads are independent.  Calls on host
 * buffers use their own CUDA stream on the current device.  Calls on device
 * buffers take a `stream` (a cudaStream_t) that orders their work after the
 * caller's; NULL is the legacy default stream, as everywhere in CUDA.
 */
#ifndef FAZ_GB300_H
#define FAZ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FAZ_OK 0
#define FAZ_ERR_ARG (-1)        /* invalid argument or configuration */
#define FAZ_ERR_UNSUPPORTED (-2) /* configuration outside the implemented path */
#define FAZ_ERR_CUDA (-3)       /* CUDA runtime failure */
#define FAZ_ERR_FORMAT (-4)     /* malformed or truncated stream */
#define FAZ_ERR_ZSTD (-5)       /* host zstd library missing or failed */
#define FAZ_ERR_DEVICE (-6)     /* a kernel reported an error status */

/* data types, as the reference CLI numbers them (test/faz.cpp:10-11) */
#define FAZ_FLOAT 0
#define FAZ_DOUBLE 1

/* QoZ::ALGO (include/QoZ/utils/Config.hpp:24-26) */
#define FAZ_ALGO_LORENZO_REG 0
#define FAZ_ALGO_INTERP_LORENZO 1
#define FAZ_ALGO_INTERP 2
#define FAZ_ALGO_INTERP_BLOCKED 3
/* QoZ::EB (Config.hpp:18-20) */
#define FAZ_EB_ABS 0
#define FAZ_EB_REL 1
#define FAZ_EB_PSNR 2
#define FAZ_EB_L2NORM 3
#define FAZ_EB_ABS_AND_REL 4
#define FAZ_EB_ABS_OR_REL 5
/* QoZ::INTERP_ALGO (Config.hpp:30-31) */
#define FAZ_INTERP_ALGO_LINEAR 0
#define FAZ_INTERP_ALGO_CUBIC 1

#define FAZ_MAX_LEVELS 64

/*
 * Mirror of QoZ::Config (include/QoZ/utils/Config.hpp:394-499): the fields
 * written to the stream trailer by Config::save (Config.hpp:240-309) plus the
 * knobs the interpolation path reads.  faz_config_init() sets the reference
 * defaults.  Booleans are uint8_t (0/1).
 */
typedef struct faz_config {
    int32_t N;                      /* char N */
    uint64_t dims[4];               /* dims[0] is the slowest dimension */
    uint64_t num;
    uint8_t cmprAlgo;               /* default ALGO_INTERP_LORENZO */
    uint8_t errorBoundMode;         /* default EB_ABS */
    uint8_t tuningTarget;           /* default TUNING_TARGET_RD */
    double absErrorBound;
    double relErrorBound;           /* default -1 */
    double psnrErrorBound;
    double l2normErrorBound;
    double rng;                     /* default -1 */
    double alpha;                   /* default -1 */
    double beta;                    /* default -1 */
    double autoTuningRate;          /* default 0 */
    double predictorTuningRate;     /* default 0 */
    uint8_t lorenzo;                /* default 1 */
    uint8_t lorenzo2;               /* default 0 */
    uint8_t regression;             /* default 1 */
    uint8_t regression2;            /* default 0 */
    uint8_t openmp;                 /* default 0 */
    uint8_t lossless;               /* default 1 */
    uint8_t encoder;                /* default 1 */
    uint8_t interpAlgo;             /* default INTERP_ALGO_CUBIC */
    uint8_t interpDirection;        /* default 0 */
    int32_t levelwisePredictionSelection;
    int32_t interp_list_len;        /* size of interpAlgo_list / interpDirection_list */
    uint8_t interpAlgo_list[FAZ_MAX_LEVELS];
    uint8_t interpDirection_list[FAZ_MAX_LEVELS];
    uint64_t maxStep;               /* default 0 (no anchor grid) */
    int32_t interpBlockSize;        /* default 32 */
    int32_t quantbinCnt;            /* default 65536 */
    int32_t blockSize;              /* 128 (1D) / 16 (2D) / 6 (3D, 4D) */
    int32_t testLorenzo;
    int32_t sampleBlockSize;
    uint8_t blockwiseTuning;
    int32_t stride;                 /* = blockSize */
    int32_t pred_dim;               /* = N */
    int32_t profiling;
    int32_t SSIMBlockSize;          /* default 8 */
    int32_t fixBlockSize;
    int32_t blockwiseSampleBlockSize;
    uint8_t verbose;                /* default 1 */
    uint8_t QoZ;
    uint8_t FZ;
    int32_t abList;
    int32_t crossBlock;
    int32_t sampleBlockSampleBlockSize;
    uint8_t peTracking;
    int32_t wavelet;
    uint64_t coeffs_num;            /* = num */
    int32_t coeffs_dims_len;        /* = N */
    uint64_t coeffs_dims[4];        /* = dims */
    double wavelet_rel_coeff;       /* default 0.75 */
    uint64_t firstSize;             /* never set on this path; written as 0 */
    int32_t pid;
    int32_t offsetPredictor;
    int32_t trimToZero;
    double preTrim;
    int32_t blockOrder;
    int32_t sperr;                  /* default -1 */
    uint8_t sperrWithoutWave;
    uint8_t pyBind;                 /* default 1; metadata string is empty */
    int32_t conditioning;
    uint8_t meta[17];
    uint8_t pybind_activated;
    int32_t var_first;              /* QoZ-branch sampling by block variance (default 0) */
} faz_config;

/* Per-call timings in milliseconds, filled when a non-NULL pointer is given. */
typedef struct faz_timings {
    double total_ms;       /* whole call, host clock */
    double h2d_ms;         /* host -> device copy of the input / payload */
    double gpu_ms;         /* device work between the copies (CUDA events) */
    double d2h_ms;         /* device -> host copy of the result */
    double zstd_ms;        /* host zstd stage */
    double host_ms;        /* host codebook / stream assembly */
    double predict_ms;     /* interpolation level kernels (CUDA events) */
    double finest_level_ms;    /* the finest (last) level kernel alone */
    double huffman_ms;     /* histogram + codebook + encode, or decode */
    uint64_t payload_bytes;    /* pre-zstd payload */
    uint64_t unpred_count;
    uint64_t kernel_launches;  /* kernels this library launched in the call */
    double tune_ms;        /* the default configuration's tuner (trials included) */
} faz_timings;

/* QoZ::Config::Config(dims...) - Config.hpp:64-74.  dims[0] slowest. */
int faz_config_init(faz_config *conf, int N, const uint64_t *dims);

/* QoZ::Config::loadcfg - Config.hpp:91-233 ([GlobalSettings]/[AlgoSettings]). */
int faz_config_load_ini(faz_config *conf, const char *path);

/* SZ_compress<T> - sz.hpp:54-108.  `data` is host memory holding conf->num
 * values of `dtype`.  On success *out is a library-allocated stream of
 * *out_size bytes: payload | Config trailer | int32 trailer size.  conf is
 * read, not modified, as in the reference (which compresses a copy). */
int faz_compress(const faz_config *conf, int dtype, const void *data,
                 char **out, size_t *out_size, faz_timings *timings);

/* SZ_decompress<T> - sz.hpp:159-205.  Decodes the stream and returns its
 * trailer configuration in *conf.  If *out is NULL the library allocates the
 * output (release with faz_free); otherwise *out must hold conf->num values
 * (conf->num on entry is the capacity; a larger field is rejected).  Unlike
 * the reference, no side file is written. */
int faz_decompress(faz_config *conf, int dtype, const char *cmp, size_t cmp_size,
                   void **out, faz_timings *timings);

/* Read a stream's trailer (Config::load, include/QoZ/utils/Config.hpp:311-388)
 * into *conf without decoding, e.g. to size the output of faz_decompress. */
int faz_stream_info(const char *cmp, size_t cmp_size, faz_config *conf);

/* Same as faz_compress with the input already in device memory (d_data) and
 * work issued on `stream` (a cudaStream_t; NULL = the legacy default stream). */
int faz_compress_device(const faz_config *conf, int dtype, const void *d_data,
                        void *stream, char **out, size_t *out_size,
                        faz_timings *timings);

/* Same as faz_decompress writing into device memory d_out, which holds
 * conf->num values on entry (a stream with a larger field is rejected). */
int faz_decompress_device(faz_config *conf, int dtype, const char *cmp,
                          size_t cmp_size, void *d_out, void *stream,
                          faz_timings *timings);

/* The GPU path without the host zstd stage, for callers that run their own
 * lossless stage and for measuring the device work: compress device data to
 * the pre-zstd payload (the bytes the reference hands to ZSTD_compress in
 * SZInterpolationCompressor::compress, SZInterpolationCompressor.hpp:485-517),
 * written to the caller's host buffer `out` of `capacity` bytes (pinned memory
 * copies fastest).  *out_size receives the payload size; if it exceeds
 * `capacity` the call returns FAZ_ERR_ARG with *out_size set and writes
 * nothing.  *conf_out (may be NULL) receives the configuration the trailer
 * would hold. */
int faz_compress_device_payload(const faz_config *conf, int dtype, const void *d_data,
                                void *stream, char *out, size_t capacity, size_t *out_size,
                                faz_config *conf_out, faz_timings *timings);

/* Decode a pre-zstd payload of an N-dimensional field into device memory
 * d_out holding `capacity` values. */
int faz_decompress_payload_device(int N, int dtype, const char *payload, size_t size,
                                  void *d_out, uint64_t capacity, void *stream,
                                  faz_timings *timings);

/* Resolve the absolute error bound of conf for the field d_data (conf->num
 * values of `dtype` in device memory, work issued on `stream`) without
 * allocating any memory.  This has no counterpart in the reference.  It is
 * for callers that cannot allocate when they need the bound: code under an
 * allocation ban (pipelines that allocate only at start-up), code that owns
 * all device memory through its own arena, or threads that must not take the
 * allocator's locks.  It computes what faz_compress derives before
 * compressing (value range, then the mode's formula): conf->absErrorBound and
 * conf->rng are set and conf->errorBoundMode becomes FAZ_EB_ABS.  Its scratch
 * is a 64 KiB array inside this library that every GPU loading the library
 * keeps until exit; fields above 2^28 values are rejected with FAZ_ERR_ARG.
 * All calls share that array: calls whose device work overlaps race.  The
 * first call on each device looks the array's address up and caches it for
 * the life of the process (the device's primary context must not be reset
 * afterwards).  Every call synchronizes `stream`, so none may be made while
 * `stream` is being captured; such a call returns FAZ_ERR_ARG.  Shapes are
 * checked as faz_compress checks them (1 <= N <= 4, num equal to the product
 * of dims), a resolved bound that is not positive and finite (constant field,
 * NaN values) is refused with FAZ_ERR_ARG as faz_compress refuses it, and on
 * any failure conf is left unchanged. */
int faz_resolve_eb_noalloc(faz_config *conf, int dtype, const void *d_data, void *stream);

/* Batched compression of n device-resident fields of uneven shapes (no
 * counterpart in the reference, which compresses one field per call).  Field
 * i has configuration confs[i] and data d_data[i] (confs[i].num values of
 * `dtype`); its stream goes to outs[i] (release each with faz_free) with size
 * out_sizes[i], byte for byte the stream faz_compress_device writes for it.
 * One launch resolves every field's error bound; one persistent launch of
 * `threads` threads per CTA (512, 256 or 128; 0 = 512) runs the first point /
 * anchor grid and every interpolation level of every ALGO_INTERP field from a
 * device work queue, a level starting once the field's previous level is
 * done; Huffman coding, payload and zstd run per field on host threads.
 * Fields with another cmprAlgo are compressed one by one afterwards.  On
 * failure no output is returned. */
int faz_compress_batch(int n, const faz_config *confs, int dtype, const void *const *d_data, void *stream, char **outs,
                       size_t *out_sizes, int threads, faz_timings *timings);

/* Run the sampled autotune that `conf` selects and stop before compressing:
 * QoZ = 1 runs the QoZ tuner (Tuning, include/QoZ/api/impl/SZInterp.hpp:
 * 1588-2557), cmprAlgo ALGO_INTERP_LORENZO without QoZ the SZ3 tuner
 * (SZInterp.hpp:2561-2880).  On return `conf` holds the decisions (cmprAlgo,
 * interpAlgo / interpDirection, per-level lists, alpha, beta, Lorenzo
 * settings) with the error bound resolved to ABS; compressing that
 * configuration writes the stream the tuned compression writes.  No
 * counterpart in the reference, where tuning happens inside SZ_compress. */
int faz_tune_device(faz_config *conf, int dtype, const void *d_data, void *stream, faz_timings *timings);

/* ---------------------------------------------------------------------------
 * Learned tuner (no counterpart in the reference).  A multilayer perceptron
 * FAZ_TUNER_FEATURES -> FAZ_TUNER_HIDDEN -> FAZ_TUNER_HIDDEN -> FAZ_TUNER_LOGITS
 * (ReLU hidden layers) predicts, from block statistics of a 3-D field, what the
 * QoZ tuner decides: per level 1..4 the interpolator and direction (4 classes:
 * linear dir 0, linear dir 5, cubic dir 0, cubic dir 5), alpha (1, 1.25, 1.5,
 * 1.75, 2), beta (1.5, 2, 3, 4), and whether the SZ3 tuner picks Lorenzo
 * (2 classes).  Heads, in logit order: level 1..4 (4 each), alpha (5), beta
 * (4), Lorenzo (2).  Parameters are one float array: W1[H][F], b1[H],
 * W2[H][H], b2[H], W3[L][H], b3[L] (row-major, y = W x + b).
 * ------------------------------------------------------------------------- */
#define FAZ_TUNER_FEATURES 64
#define FAZ_TUNER_HIDDEN 256
#define FAZ_TUNER_LOGITS 27
#define FAZ_TUNER_HEADS 7
#define FAZ_TUNER_LABELS 8 /* int32 labels per sample: one per head (-1 = none), 1 unused */
#define FAZ_TUNER_PARAMS 89371
#define FAZ_TUNER_MAX_BLOCKS 64 /* feature blocks (33^3 values each) per field */

typedef struct faz_tuner_model faz_tuner_model;

typedef struct faz_tuner_choice {
    int used_plain;       /* 0: the network decided; 1: low confidence, the plain tuner
                             decided; 2: Lorenzo predicted, the plain tuner decided;
                             3: configuration outside the network's scope */
    float confidence;     /* smallest top-class probability over the heads used */
    float p_lorenzo;      /* predicted probability that the SZ3 tuner picks Lorenzo */
    float logits[FAZ_TUNER_LOGITS];
    double tune_ms;       /* host wall time of the whole decision */
} faz_tuner_choice;

/* The FAZ_TUNER_FEATURES features of a 3-D field (every extent >= 33) into
 * d_features (device, float).  The error bound is resolved as for
 * compression.  Features come from up to FAZ_TUNER_MAX_BLOCKS 33^3 blocks on
 * the 32-grid: for strides 1, 2, 4, 8 (linear) and 1, 2, 4 (cubic) along each
 * axis, log2(1 + mean |residual| / eb) and the fraction of residuals within
 * eb; residual RMS, tails, kurtosis; log2(range / eb), log2(std / eb),
 * log2 extents, log10 relative bound, flat-neighbour fraction, block count. */
int faz_tuner_features(const faz_config *conf, int dtype, const void *d_data, void *stream, float *d_features);

/* Training kernels (FP32).  Device pointers; `batch` rows.  forward writes
 * the hidden activations and logits; backward writes the gradient of the mean
 * (over rows) summed softmax cross-entropy of the labelled heads into d_grads
 * (FAZ_TUNER_PARAMS floats) and each row's summed cross-entropy into d_loss;
 * adam applies one AdamW step (step counts from 1). */
int faz_mlp_forward(const float *d_params, const float *d_x, int batch, float *d_h1, float *d_h2, float *d_logits,
                    void *stream);
int faz_mlp_backward(const float *d_params, const float *d_x, const int32_t *d_labels, int batch, const float *d_h1,
                     const float *d_h2, const float *d_logits, float *d_grads, float *d_loss, void *stream);
int faz_mlp_adam(float *d_params, const float *d_grads, float *d_m, float *d_v, int64_t n, float lr, float beta1,
                 float beta2, float eps, int step, float weight_decay, void *stream);

/* Inference model on the current device: BF16 copies of the weights for the
 * tensor cores, plus the feature standardisation (x - mean) / std. */
faz_tuner_model *faz_tuner_model_create(const float *h_params, const float *h_mean, const float *h_std);
void faz_tuner_model_destroy(faz_tuner_model *model);

/* Logits of `batch` feature rows (device), BF16 operands with FP32
 * accumulation on the tensor cores (tcgen05.mma). */
int faz_tuner_infer(const faz_tuner_model *model, const float *d_features, int batch, float *d_logits, void *stream);

/* The learned replacement of the QoZ tuner: for a configuration with QoZ = 1
 * on a 3-D field, sets the decisions the QoZ tuner would set (per-level lists,
 * alpha, beta, cmprAlgo = ALGO_INTERP) from the network's prediction.  The
 * plain QoZ tuner decides instead when the prediction's confidence is below
 * `min_confidence`, when Lorenzo is predicted, or when the configuration is
 * outside the network's scope (choice->used_plain says which). */
int faz_learned_tune(faz_config *conf, int dtype, const void *d_data, void *stream, const faz_tuner_model *model,
                     double min_confidence, faz_tuner_choice *choice);

/* sizeof(faz_config) as this library was compiled, for bindings that
 * mirror the struct (ctypes, cgo, JNI) to check their layout. */
size_t faz_config_size(void);

/* Release a buffer returned by this library. */
void faz_free(void *p);

/* Message of the last failed call on this thread ("" if none). */
const char *faz_last_error(void);

/* Host zstd library in use: its ZSTD_versionNumber(), or 0 if none loaded.
 * The library is found as libzstd.so.1 unless FAZ_ZSTD_LIBRARY names a path. */
unsigned faz_zstd_version(void);

#ifdef __cplusplus
}
#endif
#endif /* FAZ_GB300_H */
