// faz - command-line front end with the reference tool's flags and output
// (test/faz.cpp:21-640), compressing and decompressing on the GPU through
// the C++ API of include/faz_gb300.hpp.
//
// Differences from the reference tool: -F takes an integer without
// overwriting neighbouring options; with -F 1 (the default) the FAZ
// wavelet / SPERR features are requested, which this library does not
// implement, so compression with the default ALGO_INTERP_LORENZO
// configuration needs -F 0; errors end the program with a non-zero status.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <fstream>
#include <iostream>
#include <memory>
#include <vector>

#include "../../include/faz_gb300.hpp"

namespace {

constexpr int kFloat = 0, kDouble = 1;

void usage() {
    printf("Usage: faz <options>\n");
    printf("Options:\n");
    printf("* general options:\n");
    printf("\t-h: print the help information\n");
    printf("\t-v: print the version number\n");
    printf("\t-a : print compression results such as distortions\n");
    printf("* input and output:\n");
    printf("\t-i <path> : original binary input file\n");
    printf("\t-o <path> : compressed output file, default in binary format\n");
    printf("\t-z <path> : compressed output (w -i) or input (w/o -i) file\n");
    printf("\t-t : store compressed output file in text format\n");
    printf("* data type:\n");
    printf("\t-f: single precision (float type)\n");
    printf("\t-d: double precision (double type)\n");
    printf("* configuration file: \n");
    printf("\t-c <configuration file> : configuration file faz.config\n");
    printf("* error control: (the error control parameters here will overwrite the setting in sz.config)\n");
    printf("\t-M <error control mode> <error bound (optional)> \n");
    printf("\terror control mode as follows: \n");
    printf("\t\tABS (absolute error bound)\n");
    printf("\t\tREL (value range based error bound, so a.k.a., VR_REL)\n");
    printf("\t\tPSNR (peak signal-to-noise ratio)\n");
    printf("\t\tNORM (norm2 error : sqrt(sum(xi-xi')^2)\n");
    printf("\t\tABS_AND_REL (using min{ABS, REL})\n");
    printf("\t\tABS_OR_REL (using max{ABS, REL})\n");
    printf("\terror bound can be set directly after the error control mode, or separately with the following options:\n");
    printf("\t\t-A <absolute error bound>: specifying absolute error bound\n");
    printf("\t\t-R <value_range based relative error bound>: specifying relative error bound\n");
    printf("\t\t-S <PSNR>: specifying PSNR\n");
    printf("\t\t-N <normErr>: specifying normErr\n");
    printf("    -q: use QoZ mode (deactivated in default)\n");
    printf("    -F <1/0>: activate FAZ features or not (activated in default)\n");
    printf("    -T <tuning target> \n");
    printf("    -C <anchor stride> : stride of anchor points.\n");
    printf("    -B <sampling block size> : block size of sampled data block for auto-tuning.\n");
    printf("* dimensions: \n");
    printf("\t-1 <nx> : dimension for 1D data such as data[nx]\n");
    printf("\t-2 <nx> <ny> : dimensions for 2D data such as data[ny][nx]\n");
    printf("\t-3 <nx> <ny> <nz> : dimensions for 3D data such as data[nz][ny][nx] \n");
    printf("\t-4 <nx> <ny> <nz> <np>: dimensions for 4D data such as data[np][nz][ny][nx] \n");
    printf("* examples: \n");
    printf("\tfaz -f -i test.dat    -z test.dat.faz     -3 8 8 128 -M ABS 1e-3 \n");
    printf("\tfaz -f -z test.dat.faz -o test.dat.faz.out -3 8 8 128 -M REL 1e-3 -a \n");
    exit(0);
}

[[noreturn]] void fail(const std::string &msg) {
    fprintf(stderr, "Error: %s\n", msg.c_str());
    exit(1);
}

std::vector<char> read_bytes(const char *path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        std::cout << " Error, Couldn't find the file: " << path << "\n";
        exit(1);
    }
    f.seekg(0, std::ios::end);
    const size_t n = (size_t)f.tellg();
    f.seekg(0, std::ios::beg);
    std::vector<char> b(n);
    f.read(b.data(), (std::streamsize)n);
    return b;
}

void write_bytes(const char *path, const void *p, size_t n) {
    std::ofstream f(path, std::ios::binary);
    if (!f) fail(std::string("unable to open file for output: ") + path);
    f.write((const char *)p, (std::streamsize)n);
}

double seconds_since(std::chrono::steady_clock::time_point t) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t).count();
}

// QoZ::verify (include/QoZ/utils/Statistic.hpp:118-180): the distortion report
template <class T>
void verify(const T *ori, const T *dec, size_t n) {
    double Max = ori[0], Min = ori[0];
    double diffMax = std::fabs((double)(T)(dec[0] - ori[0]));
    double maxpw = 0, sum1 = 0, sum2 = 0, l2sum = 0;
    for (size_t i = 0; i < n; i++) {
        sum1 += ori[i];
        sum2 += dec[i];
        l2sum += (double)(T)(dec[i] * dec[i]);
    }
    const double mean1 = sum1 / n, mean2 = sum2 / n;
    double sum3 = 0, sum4 = 0, sum = 0, prod = 0;
    for (size_t i = 0; i < n; i++) {
        if (Max < ori[i]) Max = ori[i];
        if (Min > ori[i]) Min = ori[i];
        const double err = std::fabs((double)(T)(dec[i] - ori[i]));
        if (ori[i] != 0) {
            const double rel = err / std::fabs((double)ori[i]);
            if (maxpw < rel) maxpw = rel;
        }
        if (diffMax < err) diffMax = err;
        prod += (ori[i] - mean1) * (dec[i] - mean2);
        sum3 += (ori[i] - mean1) * (ori[i] - mean1);
        sum4 += (dec[i] - mean2) * (dec[i] - mean2);
        sum += err * err;
    }
    const double std1 = std::sqrt(sum3 / n), std2 = std::sqrt(sum4 / n);
    const double ac = prod / n / std1 / std2;
    const double mse = sum / n, range = Max - Min;
    const double psnr = 20 * std::log10(range) - 10 * std::log10(mse);
    const double nrmse = std::sqrt(mse) / range;
    const double normErr = std::sqrt(sum), normErrNorm = normErr / std::sqrt(l2sum);
    printf("Min=%.20G, Max=%.20G, range=%.20G\n", Min, Max, range);
    printf("Max absolute error = %.2G\n", diffMax);
    printf("Max relative error = %.2G\n", diffMax / (Max - Min));
    printf("Max pw relative error = %.2G\n", maxpw);
    printf("PSNR = %f, NRMSE= %.10G\n", psnr, nrmse);
    printf("normError = %f, normErr_norm = %f\n", normErr, normErrNorm);
    printf("acEff=%f\n", ac);
}

template <class T>
void compress(const char *inPath, const char *cmpPath, QoZ::Config &conf) {
    std::vector<char> raw = read_bytes(inPath);
    if (raw.size() / sizeof(T) != conf.num) fail("File size is not equals to the input setting");
    size_t outSize;
    auto t0 = std::chrono::steady_clock::now();
    char *bytes = SZ_compress<T>(conf, reinterpret_cast<const T *>(raw.data()), outSize);
    const double t = seconds_since(t0);
    std::string out = cmpPath ? std::string(cmpPath) : std::string(inPath) + ".faz";
    write_bytes(out.c_str(), bytes, outSize);
    printf("compression ratio = %.2f \n", conf.num * 1.0 * sizeof(T) / outSize);
    printf("compression time = %f\n", t);
    printf("compressed data file = %s\n", out.c_str());
    delete[] bytes;
}

template <class T>
void decompress(const char *inPath, const char *cmpPath, const char *decPath, QoZ::Config &conf, bool binary,
                bool report) {
    std::vector<char> cmp = read_bytes(cmpPath);
    auto t0 = std::chrono::steady_clock::now();
    T *dec = SZ_decompress<T>(conf, cmp.data(), cmp.size());
    const double t = seconds_since(t0);
    std::string out = decPath ? std::string(decPath) : std::string(cmpPath) + ".out";
    if (binary) {
        write_bytes(out.c_str(), dec, conf.num * sizeof(T));
    } else {
        std::ofstream f(out);
        if (!f) fail("unable to open file for output: " + out);
        for (size_t i = 0; i < conf.num; i++) f << dec[i] << std::endl;
    }
    if (report) {
        std::vector<char> ori = read_bytes(inPath);
        if (ori.size() / sizeof(T) != conf.num) fail("original file size does not match the stream");
        verify<T>(reinterpret_cast<const T *>(ori.data()), dec, conf.num);
    }
    delete[] dec;
    printf("compression ratio = %f\n", conf.num * sizeof(T) * 1.0 / cmp.size());
    printf("decompression time = %f seconds.\n", t);
    printf("decompressed file = %s\n", out.c_str());
}

int parse_int(const char *s) {
    int v;
    if (sscanf(s, "%d", &v) != 1) usage();
    return v;
}

size_t parse_size(const char *s) {
    size_t v;
    if (sscanf(s, "%zu", &v) != 1) usage();
    return v;
}

}  // namespace

int main(int argc, char *argv[]) {
    bool binaryOutput = true, report = false, compression = false, decompression = false, sz2mode = false;
    int dataType = kFloat;
    char *inPath = nullptr, *cmpPath = nullptr, *conPath = nullptr, *decPath = nullptr;
    char *errBoundMode = nullptr, *errBound = nullptr, *absEB = nullptr, *relEB = nullptr, *psnrEB = nullptr,
         *normEB = nullptr, *tuningTarget = nullptr;
    int maxStep = 0, sampleBlockSize = 0, faz = 1;
    bool qoz = false, testLorenzo = false, delCmpPath = false;
    size_t r1 = 0, r2 = 0, r3 = 0, r4 = 0;
    if (argc == 1) usage();
    for (int i = 1; i < argc; i++) {
        if (argv[i][0] != '-' || argv[i][1] == 0 || argv[i][2]) usage();
        auto next = [&]() -> char * {
            if (++i == argc) usage();
            return argv[i];
        };
        switch (argv[i][1]) {
        case 'h': usage(); break;
        case 'v': printf("version: %s\n", "0.1.0.0"); return 0;
        case 'b': binaryOutput = true; break;
        case 't': binaryOutput = false; break;
        case 'a': report = true; break;
        case 'z':
            compression = true;
            if (i + 1 < argc) {
                cmpPath = argv[i + 1];
                if (cmpPath[0] != '-') i++;
                else cmpPath = nullptr;
            }
            break;
        case 'x':
            sz2mode = true;
            decompression = true;
            if (i + 1 < argc) {
                decPath = argv[i + 1];
                if (decPath[0] != '-') i++;
                else decPath = nullptr;
            }
            break;
        case 'f': dataType = kFloat; break;
        case 'd': dataType = kDouble; break;
        case 'i': inPath = next(); break;
        case 'q': qoz = true; break;
        case 'F': faz = parse_int(next()); break;
        case 'l': testLorenzo = true; break;
        case 'o': decPath = next(); break;
        case 's': sz2mode = true; cmpPath = next(); break;
        case 'c': conPath = next(); break;
        case '1': r1 = parse_size(next()); break;
        case '2': r1 = parse_size(next()); r2 = parse_size(next()); break;
        case '3': r1 = parse_size(next()); r2 = parse_size(next()); r3 = parse_size(next()); break;
        case '4':
            r1 = parse_size(next());
            r2 = parse_size(next());
            r3 = parse_size(next());
            r4 = parse_size(next());
            break;
        case 'M':
            errBoundMode = next();
            if (i + 1 < argc && argv[i + 1][0] != '-') errBound = argv[++i];
            break;
        case 'A': absEB = next(); break;
        case 'R': relEB = next(); break;
        case 'N': normEB = next(); break;
        case 'S': psnrEB = next(); break;
        case 'T': tuningTarget = next(); break;
        case 'C': maxStep = parse_int(next()); break;
        case 'B': sampleBlockSize = parse_int(next()); break;
        default: usage();
        }
    }
    if (inPath == nullptr && cmpPath == nullptr) {
        printf("Error: you need to specify either a raw binary data file or a compressed data file as input\n");
        usage();
    }
    if (!sz2mode && inPath != nullptr && cmpPath != nullptr) compression = true;
    if (cmpPath != nullptr && decPath != nullptr) decompression = true;
    std::string tmpCmp;
    if (inPath != nullptr && cmpPath == nullptr && decPath != nullptr) {
        compression = true;
        decompression = true;
        tmpCmp = std::string(inPath) + ".faz.tmp";
        cmpPath = &tmpCmp[0];
        delCmpPath = true;
    }
    if (inPath == nullptr || errBoundMode == nullptr) compression = false;
    if (!compression && !decompression) usage();

    try {
        QoZ::Config conf;
        if (r2 == 0) conf = QoZ::Config(r1);
        else if (r3 == 0) conf = QoZ::Config(r2, r1);
        else if (r4 == 0) conf = QoZ::Config(r3, r2, r1);
        else conf = QoZ::Config(r4, r3, r2, r1);
        if (qoz) conf.QoZ = 1;
        if (faz) conf.FZ = 1;
        if (testLorenzo) conf.testLorenzo = 1;
        if (maxStep > 0) conf.maxStep = maxStep;
        if (sampleBlockSize > 0) conf.sampleBlockSize = sampleBlockSize;
        if (compression && conPath != nullptr) conf.loadcfg(conPath);
        if (errBoundMode != nullptr) {
            if (relEB) conf.relErrorBound = atof(relEB);
            if (absEB) conf.absErrorBound = atof(absEB);
            if (psnrEB) conf.psnrErrorBound = atof(psnrEB);
            if (normEB) conf.l2normErrorBound = atof(normEB);
            if (strcmp(errBoundMode, "ABS") == 0) {
                conf.errorBoundMode = QoZ::EB_ABS;
                if (errBound) conf.absErrorBound = atof(errBound);
            } else if (strcmp(errBoundMode, "REL") == 0 || strcmp(errBoundMode, "VR_REL") == 0) {
                conf.errorBoundMode = QoZ::EB_REL;
                if (errBound) conf.relErrorBound = atof(errBound);
            } else if (strcmp(errBoundMode, "PSNR") == 0) {
                conf.errorBoundMode = QoZ::EB_PSNR;
                if (errBound) conf.psnrErrorBound = atof(errBound);
            } else if (strcmp(errBoundMode, "NORM") == 0) {
                conf.errorBoundMode = QoZ::EB_L2NORM;
                if (errBound) conf.l2normErrorBound = atof(errBound);
            } else if (strcmp(errBoundMode, "ABS_AND_REL") == 0) {
                conf.errorBoundMode = QoZ::EB_ABS_AND_REL;
            } else if (strcmp(errBoundMode, "ABS_OR_REL") == 0) {
                conf.errorBoundMode = QoZ::EB_ABS_OR_REL;
            } else {
                printf("Error: wrong error bound mode setting by using the option '-M'\n");
                usage();
            }
        }
        if (tuningTarget != nullptr) {
            if (strcmp(tuningTarget, "PSNR") == 0) conf.tuningTarget = QoZ::TUNING_TARGET_RD;
            else if (strcmp(tuningTarget, "CR") == 0) conf.tuningTarget = QoZ::TUNING_TARGET_CR;
            else if (strcmp(tuningTarget, "SSIM") == 0) conf.tuningTarget = QoZ::TUNING_TARGET_SSIM;
            else if (strcmp(tuningTarget, "AC") == 0) conf.tuningTarget = QoZ::TUNING_TARGET_AC;
            else {
                printf("Error: wrong tuning target setting by using the option '-T'\n");
                usage();
            }
        }
        if (compression) {
            if (dataType == kFloat) compress<float>(inPath, cmpPath, conf);
            else compress<double>(inPath, cmpPath, conf);
        }
        if (decompression) {
            if (report && inPath == nullptr) {
                printf("Error: Since you add -a option (analysis), please specify the original data path by -i <path>.\n");
                return 1;
            }
            if (dataType == kFloat) decompress<float>(inPath, cmpPath, decPath, conf, binaryOutput, report);
            else decompress<double>(inPath, cmpPath, decPath, conf, binaryOutput, report);
        }
    } catch (const QoZ::Error &e) {
        if (delCmpPath) remove(cmpPath);
        fail(e.what());
    }
    if (delCmpPath) remove(cmpPath);
    return 0;
}
