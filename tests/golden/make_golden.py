"""Generate the golden fixtures in this folder from the reference build.

Each case: a seeded input field (<name>.in, raw little-endian) and the stream
the reference `faz` tool writes for it (<name>.faz).  The array the reference
decompresses from that stream is recorded by its SHA-256 (dec_sha256 in
manifest.json), which also lists the command line, INI settings, dtype and
dims of every case.  (A single-point field is not a case: the reference
aborts in free() on it.)

The reference tool is oracle/_ref/faz, built from the reference sources by
oracle/build_ref.sh (with its bundled zstd 1.4.5).  Run from the repository
root, with FAZ_REFERENCE_ROOT naming the reference checkout when the tool is
not built yet:  python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
from faz_gb300.fields import spectral_field  # noqa: E402

FAZ = os.path.join(ROOT, "oracle", "_ref", "faz")


def random_walk(shape, seed, dtype=np.float32):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(shape)
    for ax in range(len(shape)):
        a = np.cumsum(a, axis=ax)
    return a.astype(dtype)


def cases():
    """(name, array, cli flags, ini dict)"""
    interp_cubic = {"GlobalSettings": {"CmprAlgo": "ALGO_INTERP"},
                    "AlgoSettings": {"InterpolationAlgo": "INTERP_ALGO_CUBIC"}}
    interp_linear = {"GlobalSettings": {"CmprAlgo": "ALGO_INTERP"},
                     "AlgoSettings": {"InterpolationAlgo": "INTERP_ALGO_LINEAR"}}

    def ini(extra_algo=None, base=interp_cubic):
        d = {k: dict(v) for k, v in base.items()}
        if extra_algo:
            d["AlgoSettings"].update(extra_algo)
        return d

    out = []
    out.append(("c3d_cubic_walk", random_walk((20, 30, 40), 1), ["-M", "REL", "1e-3"], ini()))
    out.append(("c3d_linear", spectral_field((33, 17, 65), slope=-3.0, seed=2), ["-M", "REL", "1e-2"],
                ini(base=interp_linear)))
    out.append(("c3d_noisy_1e4", spectral_field((48, 48, 48), slope=-2.0, noise=0.05, seed=3),
                ["-M", "REL", "1e-4"], ini()))
    out.append(("c3d_spec_1e3", spectral_field((40, 56, 72), slope=-3.5, aniso=(1, 2, 4), seed=4),
                ["-M", "REL", "1e-3"], ini()))
    out.append(("c2d_cubic", spectral_field((100, 150), slope=-3.0, seed=5), ["-M", "REL", "1e-3"], ini()))
    out.append(("c1d_cubic", spectral_field((5000,), slope=-2.5, seed=6), ["-M", "REL", "1e-3"], ini()))
    out.append(("c3d_f64", spectral_field((20, 30, 40), slope=-3.0, seed=7, dtype=np.float64),
                ["-M", "REL", "1e-5"], ini()))
    out.append(("c3d_anchor_ab", spectral_field((40, 40, 40), slope=-3.0, seed=8), ["-M", "REL", "1e-3", "-C", "16"],
                ini({"alpha": "1.5", "beta": "2.0"})))
    out.append(("c3d_alpha_lt1", spectral_field((36, 28, 44), slope=-3.0, seed=9), ["-M", "REL", "1e-3"],
                ini({"alpha": "0.5", "beta": "0.25"})))
    out.append(("c3d_dir5_abs", spectral_field((24, 36, 20), slope=-3.0, seed=10), ["-M", "ABS", "0.05"],
                ini({"InterpDirection": "5"})))
    out.append(("c3d_dir3_linear", spectral_field((24, 20, 36), slope=-3.0, seed=11), ["-M", "REL", "1e-3"],
                ini({"InterpDirection": "3"}, base=interp_linear)))
    out.append(("c3d_fixbs8", spectral_field((30, 30, 30), slope=-3.0, seed=12), ["-M", "REL", "1e-3"],
                ini({"fixBlockSize": "8"})))
    out.append(("c3d_ibs16", spectral_field((34, 30, 50), slope=-3.0, seed=13), ["-M", "REL", "1e-3"],
                ini({"InterpBlockSize": "16"})))
    out.append(("c4d_cubic", spectral_field((6, 7, 8, 9), slope=-3.0, seed=14), ["-M", "REL", "1e-3"], ini()))
    out.append(("tiny_2x3x4", spectral_field((2, 3, 4), slope=-3.0, seed=15), ["-M", "REL", "1e-3"], ini()))
    out.append(("tiny_5x5x5", spectral_field((5, 5, 5), slope=-3.0, seed=16), ["-M", "REL", "1e-3"], ini()))
    out.append(("tiny_7x1x9", spectral_field((7, 1, 9), slope=-3.0, seed=17), ["-M", "REL", "1e-3"], ini()))
    out.append(("const_16", np.full((16, 16, 16), 7.5, dtype=np.float32), ["-M", "ABS", "0.01"], ini()))
    out.append(("trim1", spectral_field((32, 32, 32), slope=-3.0, seed=18, lo=-1, hi=1), ["-M", "ABS", "0.05"],
                ini({"trimToZero": "1"})))
    out.append(("trim2", spectral_field((32, 32, 32), slope=-3.0, seed=19, lo=-1, hi=1), ["-M", "ABS", "0.05"],
                ini({"trimToZero": "2"})))
    out.append(("c2d_abs_and_rel", spectral_field((64, 96), slope=-3.0, seed=20),
                ["-M", "ABS_AND_REL", "-A", "0.5", "-R", "1e-3"], ini()))
    out.append(("c3d_spikes", spectral_field((40, 40, 40), slope=-3.0, seed=21, spikes=0.05),
                ["-M", "REL", "1e-3"], ini()))
    out.append(("c3d_odd_65", spectral_field((65, 33, 17), slope=-3.0, seed=22), ["-M", "REL", "1e-3"], ini()))
    # tuner-driven streams: the stream header records the tuner's decisions
    out.append(("qoz_48", spectral_field((48, 48, 48), slope=-3.0, seed=23), ["-M", "REL", "1e-3", "-q"],
                None))
    out.append(("sz3_48", spectral_field((48, 48, 48), slope=-3.0, seed=24), ["-M", "REL", "1e-3"], None))
    # default configuration (ALGO_INTERP_LORENZO, SZ3 tuner) on fields large
    # enough to be sampled: interpolation chosen (direction trial kept / not)
    out.append(("sz3_interp_dir5", spectral_field((56, 60, 64), slope=-3.5, aniso=(4, 2, 1), seed=41),
                ["-M", "REL", "1e-3"], None))
    out.append(("sz3_interp_1e2", spectral_field((56, 60, 64), slope=-3.0, seed=33), ["-M", "REL", "1e-2"], None))
    # ... and Lorenzo chosen: sums of 2-D functions, which the 3-D Lorenzo
    # predictor reproduces, plus noise
    out.append(("sz3_lorenzo_1e3", sum2d((56, 60, 64), 0.0005, seed=51), ["-M", "REL", "1e-3"], None))
    out.append(("sz3_lorenzo_1e2", sum2d((56, 60, 64), 0.0005, seed=52), ["-M", "REL", "1e-2"], None))
    out.append(("sz3_lorenzo_abs", sum2d((56, 60, 64), 0.001, seed=53), ["-M", "ABS", "0.02"], None))
    out.append(("sz3_lorenzo_f64_16384", sum2d((56, 60, 64), 1e-8, seed=54, dtype=np.float64),
                ["-M", "REL", "5e-7"], None))
    # rough fields at a tight bound: Lorenzo with the interval estimate's
    # 131072 quantisation bins (codes wider than 16 bits)
    out.append(("sz3_lorenzo_f64_131072", spectral_field((56, 60, 64), slope=-1.5, noise=0.0, seed=55,
                                                         dtype=np.float64), ["-M", "REL", "1e-6"], None))
    # (the float32 version of this field aborts the reference tool in its
    # Huffman encoder's fixed-size buffer; the GPU tests compare it with the
    # oracle instead)
    # QoZ tuner (-q): per-level predictors and alpha/beta from trial compressions
    out.append(("qoz_2blk_1e3", spectral_field((50, 120, 170), slope=-3.0, aniso=(1, 2, 2), seed=61),
                ["-M", "REL", "1e-3", "-q"], None))
    out.append(("qoz_f64_1e5", spectral_field((48, 56, 64), slope=-3.5, seed=62, dtype=np.float64),
                ["-M", "REL", "1e-5", "-q"], None))
    out.append(("qoz_1e2", spectral_field((40, 72, 90), slope=-2.5, noise=0.02, seed=63),
                ["-M", "REL", "1e-2", "-q"], None))
    out.append(("qoz_2d", spectral_field((400, 500), slope=-3.0, seed=64), ["-M", "REL", "5e-3", "-q"], None))
    # explicit Lorenzo / regression fast frontend
    lor = {"GlobalSettings": {"CmprAlgo": "ALGO_LORENZO_REG"}, "AlgoSettings": {}}
    out.append(("lorreg_default", spectral_field((40, 44, 52), slope=-3.0, seed=55), ["-M", "REL", "1e-3"], lor))
    out.append(("lorreg_qb131072", spectral_field((40, 44, 52), slope=-1.5, seed=58), ["-M", "REL", "1e-6"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_LORENZO_REG"},
                 "AlgoSettings": {"QuantizationBinTotal": "131072"}}))
    out.append(("lorreg_l2_bs4", spectral_field((37, 41, 29), slope=-2.5, seed=56), ["-M", "REL", "1e-3"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_LORENZO_REG"},
                 "AlgoSettings": {"Lorenzo2ndOrder": "YES", "BlockSize": "4"}}))
    out.append(("lor_only_f64", spectral_field((30, 33, 35), slope=-3.0, seed=57, dtype=np.float64),
                ["-M", "REL", "1e-4"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_LORENZO_REG"}, "AlgoSettings": {"Regression": "NO"}}))
    # 1-D / 2-D default configuration: the SZ3 tuner's Lorenzo trial runs the
    # general frontend (Lorenzo + 2-layer Lorenzo), chosen or not
    out.append(("sz3_2d_interp", spectral_field((300, 400), slope=-4.5, aniso=(4, 1), seed=71), ["-M", "REL", "1e-3"],
                None))
    out.append(("sz3_2d_interp_1e2", spectral_field((300, 400), slope=-3.5, seed=71), ["-M", "REL", "1e-2"], None))
    out.append(("sz3_2d_lorenzo", sum1d((300, 400), 0.0005, seed=72), ["-M", "REL", "1e-3"], None))
    out.append(("sz3_2d_lorenzo_f64", sum1d((260, 330), 0.0002, seed=73, dtype=np.float64), ["-M", "REL", "1e-4"],
                None))
    out.append(("sz3_1d_lorenzo", random_walk((20000,), 74), ["-M", "REL", "1e-3"], None))
    out.append(("sz3_1d_interp", spectral_field((20000,), slope=-3.5, seed=75), ["-M", "REL", "1e-3"], None))
    # explicit ALGO_LORENZO_REG on 1-D / 2-D data (general frontend, Lorenzo only)
    out.append(("lor2d_l2", spectral_field((97, 131), slope=-2.5, noise=0.01, seed=76), ["-M", "REL", "1e-3"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_LORENZO_REG"},
                 "AlgoSettings": {"Lorenzo2ndOrder": "YES", "Regression": "NO"}}))
    out.append(("lor2d_only_f64", spectral_field((60, 77), slope=-3.0, seed=77, dtype=np.float64),
                ["-M", "REL", "1e-4"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_LORENZO_REG"}, "AlgoSettings": {"Regression": "NO"}}))
    out.append(("lor2d_l2only_bs8", spectral_field((70, 45), slope=-3.5, seed=78), ["-M", "ABS", "0.02"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_LORENZO_REG"},
                 "AlgoSettings": {"Lorenzo": "NO", "Lorenzo2ndOrder": "YES", "Regression": "NO", "BlockSize": "8"}}))
    out.append(("lor1d_l2", random_walk((3001,), 79), ["-M", "REL", "1e-3"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_LORENZO_REG"},
                 "AlgoSettings": {"Lorenzo2ndOrder": "YES", "Regression": "NO"}}))
    # ALGO_INTERP_BLOCKED (3-D): per-block interpolator and direction chosen
    # by trial, blocks of interpBlockSize at every level
    blk = {"GlobalSettings": {"CmprAlgo": "ALGO_INTERP_BLOCKED"}, "AlgoSettings": {}}
    out.append(("blk_default", spectral_field((40, 56, 72), slope=-3.0, seed=94), ["-M", "REL", "1e-3"], blk))
    out.append(("blk_f64_bs16", spectral_field((33, 47, 65), slope=-3.5, aniso=(1, 2, 4), seed=95,
                                               dtype=np.float64), ["-M", "REL", "1e-5"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_INTERP_BLOCKED"}, "AlgoSettings": {"InterpBlockSize": "16"}}))
    out.append(("blk_sbs8_abs", spectral_field((48, 48, 48), slope=-2.5, noise=0.02, seed=96), ["-M", "ABS", "0.05"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_INTERP_BLOCKED"},
                 "AlgoSettings": {"blockwiseSampleBlockSize": "8"}}))
    out.append(("blk_anchor_ab", spectral_field((64, 40, 50), slope=-3.0, seed=97), ["-M", "REL", "1e-4"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_INTERP_BLOCKED"},
                 "AlgoSettings": {"maxStep": "16", "alpha": "1.5", "beta": "3"}}))
    out.append(("blk_odd_bs8", spectral_field((17, 23, 130), slope=-3.0, seed=98), ["-M", "REL", "1e-3"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_INTERP_BLOCKED"},
                 "AlgoSettings": {"InterpBlockSize": "8", "trimToZero": "1"}}))
    # explicit ALGO_LORENZO_REG on 1-D / 2-D data with the linear-regression
    # predictor (the default Config: Lorenzo + regression, composed)
    lreg = {"GlobalSettings": {"CmprAlgo": "ALGO_LORENZO_REG"}, "AlgoSettings": {}}
    out.append(("reg2d_default", spectral_field((97, 131), slope=-3.5, noise=0.1, seed=86), ["-M", "REL", "1e-3"],
                lreg))
    out.append(("reg2d_l1l2reg_bs8", spectral_field((70, 45), slope=-3.0, seed=87), ["-M", "ABS", "0.02"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_LORENZO_REG"},
                 "AlgoSettings": {"Lorenzo2ndOrder": "YES", "BlockSize": "8"}}))
    out.append(("reg2d_l2reg", spectral_field((60, 77), slope=-4.0, aniso=(1, 3), noise=0.03, seed=88),
                ["-M", "REL", "1e-2"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_LORENZO_REG"},
                 "AlgoSettings": {"Lorenzo": "NO", "Lorenzo2ndOrder": "YES"}}))
    out.append(("reg2d_only_f64", spectral_field((49, 65), slope=-3.0, seed=89, dtype=np.float64),
                ["-M", "REL", "1e-4"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_LORENZO_REG"}, "AlgoSettings": {"Lorenzo": "NO"}}))
    out.append(("reg2d_f64_1e7", spectral_field((81, 66), slope=-2.0, noise=0.01, seed=90, dtype=np.float64),
                ["-M", "REL", "1e-7"], lreg))
    out.append(("reg1d_default", spectral_field((20000,), slope=-3.5, seed=91), ["-M", "REL", "1e-3"], lreg))
    out.append(("reg1d_thin", spectral_field((3841,), slope=-4.0, seed=92), ["-M", "REL", "1e-4"], lreg))
    out.append(("reg1d_only_f64_bs64", spectral_field((4033,), slope=-3.0, seed=93, dtype=np.float64),
                ["-M", "REL", "1e-5"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_LORENZO_REG"},
                 "AlgoSettings": {"Lorenzo": "NO", "BlockSize": "64"}}))
    # rate-driven tuning without -q (Tuning's QoZ branch from the INI's rates;
    # the first is the learned tuner's labelling INI, whose Lorenzo candidate
    # is dropped above a relative bound of 1e-3)
    label_ini = {"GlobalSettings": {}, "AlgoSettings": {"autoTuningRate": "0.005", "predictorTuningRate": "0.005",
                                                         "maxStep": "32", "levelwisePredictionSelection": "4",
                                                         "sampleBlockSize": "32", "testLorenzo": "1"}}
    out.append(("rate_label_ini_1e2", spectral_field((50, 120, 170), slope=-3.0, aniso=(1, 2, 2), seed=81),
                ["-M", "REL", "1e-2"], label_ini))
    # at relative bounds <= 1e-3 the Lorenzo candidate runs: a field the 3-D
    # Lorenzo predictor reproduces (sums of 2-D functions) selects it
    out.append(("rate_label_ini_1e3", spectral_field((64, 96, 80), slope=-3.0, seed=84), ["-M", "REL", "1e-3"],
                label_ini))
    out.append(("rate_label_ini_lorenzo", sum2d((64, 72, 80), 1e-4, 85), ["-M", "REL", "1e-3"], label_ini))
    out.append(("rate_2d_lorenzo", sum1d((300, 400), 1e-4, 89), ["-M", "REL", "1e-3"],
                {"GlobalSettings": {}, "AlgoSettings": {"autoTuningRate": "0.01", "predictorTuningRate": "0.01",
                                                        "testLorenzo": "1"}}))
    # OpenMP streams (OpenMP = YES): slabs along the slowest axis, one per
    # OpenMP thread (OMP_THREADS below)
    out.append(("omp_interp_3", spectral_field((40, 48, 56), slope=-3.0, seed=86), ["-M", "REL", "1e-3"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_INTERP", "OpenMP": "YES"},
                 "AlgoSettings": {"InterpolationAlgo": "INTERP_ALGO_CUBIC"}}))
    out.append(("omp_default_4", spectral_field((64, 80, 96), slope=-3.0, seed=87), ["-M", "REL", "1e-3"],
                {"GlobalSettings": {"OpenMP": "YES"}, "AlgoSettings": {}}))
    out.append(("omp_abs2d_5", spectral_field((300, 200), slope=-2.5, seed=88), ["-M", "ABS", "0.05"],
                {"GlobalSettings": {"CmprAlgo": "ALGO_INTERP", "OpenMP": "YES"}, "AlgoSettings": {}}))
    # predictor tuning alone (autoTuningRate 0): compression-ratio CompressTests
    pt = lambda **kw: {"GlobalSettings": {}, "AlgoSettings": dict({"predictorTuningRate": "0.01"}, **kw)}  # noqa: E731
    out.append(("pt_levelwise_3d", spectral_field((64, 80, 96), slope=-3.0, noise=0.01, seed=90), ["-M", "REL", "1e-3"],
                pt(levelwisePredictionSelection="4", maxStep="32", testLorenzo="1")))
    out.append(("pt_lorenzo_3d", sum2d((64, 72, 80), 1e-4, 91), ["-M", "REL", "1e-3"], pt(testLorenzo="1")))
    out.append(("pt_lorenzo_2d", spectral_field((300, 400), slope=-3.0, noise=0.01, seed=92), ["-M", "REL", "5e-4"],
                pt(testLorenzo="1", sampleBlockSize="32")))
    out.append(("pt_f64", spectral_field((48, 56, 64), slope=-3.0, noise=0.01, seed=93, dtype=np.float64),
                ["-M", "REL", "1e-5"], pt(predictorTuningRate="0.02")))
    # profiling-driven sampling (profiling = 1) and a B-M sample of its own
    # (autoTuningRate != predictorTuningRate); seeds whose decisions are the
    # same with the host's zstd as with the reference's 1.4.5
    out.append(("prof_3d", flat_outside((96, 128, 160), 0.6, 95), ["-M", "REL", "1e-3"],
                {"GlobalSettings": {}, "AlgoSettings": {"autoTuningRate": "0.01", "predictorTuningRate": "0.01",
                                                        "profiling": "1", "levelwisePredictionSelection": "4",
                                                        "maxStep": "32", "sampleBlockSize": "32"}}))
    out.append(("prof_rates_3d", flat_outside((96, 128, 160), 0.6, 94), ["-M", "REL", "1e-2"],
                {"GlobalSettings": {}, "AlgoSettings": {"autoTuningRate": "0.005", "predictorTuningRate": "0.02",
                                                        "profiling": "1", "testLorenzo": "1",
                                                        "sampleBlockSize": "16"}}))
    out.append(("prof_2d", flat_outside((400, 500), 0.7, 96), ["-M", "REL", "1e-3"],
                {"GlobalSettings": {}, "AlgoSettings": {"autoTuningRate": "0.01", "predictorTuningRate": "0.01",
                                                        "profiling": "1", "levelwisePredictionSelection": "6",
                                                        "maxStep": "64"}}))
    # sampling by block variance (var_first = 1), with and without profiling
    out.append(("varfirst_3d", spectral_field((80, 96, 112), slope=-2.5, noise=0.05, seed=97), ["-M", "REL", "5e-3"],
                {"GlobalSettings": {}, "AlgoSettings": {"autoTuningRate": "0.005", "predictorTuningRate": "0.02",
                                                        "var_first": "1", "sampleBlockSize": "16"}}))
    out.append(("varfirst_prof_2d", flat_outside((400, 500), 0.7, 100), ["-M", "REL", "1e-3"],
                {"GlobalSettings": {}, "AlgoSettings": {"autoTuningRate": "0.01", "predictorTuningRate": "0.01",
                                                        "var_first": "1", "profiling": "1",
                                                        "levelwisePredictionSelection": "6", "maxStep": "64"}}))
    # the compression-ratio tuning target (TUNING_TARGET_CR: alpha/beta lists
    # with -1, bit rates compared alone)
    out.append(("cr_target_3d", spectral_field((64, 80, 96), slope=-3.0, noise=0.01, seed=99), ["-M", "REL", "1e-3"],
                {"GlobalSettings": {"tuningTarget": "TUNING_TARGET_CR"},
                 "AlgoSettings": {"autoTuningRate": "0.01", "predictorTuningRate": "0.01",
                                  "levelwisePredictionSelection": "4", "maxStep": "32", "sampleBlockSize": "16"}}))
    out.append(("cr_target_lorenzo", sum2d((64, 72, 80), 1e-4, 101), ["-M", "REL", "1e-3"],
                {"GlobalSettings": {"tuningTarget": "TUNING_TARGET_CR"},
                 "AlgoSettings": {"autoTuningRate": "0.01", "predictorTuningRate": "0.01", "testLorenzo": "1",
                                  "sampleBlockSize": "16"}}))
    # the SSIM and autocorrelation tuning targets (the alpha/beta search scores
    # each CompressTest by the reconstruction's SSIM or 1 - autocorrelation)
    out.append(("ssim_target_3d", spectral_field((64, 80, 96), slope=-2.0, noise=0.0, seed=150), ["-M", "REL", "1e-4"],
                {"GlobalSettings": {"tuningTarget": "TUNING_TARGET_SSIM"},
                 "AlgoSettings": {"autoTuningRate": "0.01", "predictorTuningRate": "0.01",
                                  "levelwisePredictionSelection": "4", "maxStep": "32", "sampleBlockSize": "16"}}))
    out.append(("ssim_target_2d", spectral_field((400, 500), slope=-2.0, noise=0.05, seed=124), ["-M", "REL", "3e-3"],
                {"GlobalSettings": {"tuningTarget": "TUNING_TARGET_SSIM"},
                 "AlgoSettings": {"autoTuningRate": "0.01", "predictorTuningRate": "0.01",
                                  "levelwisePredictionSelection": "6", "maxStep": "64"}}))
    out.append(("ssim_target_q", spectral_field((48, 56, 64), slope=-2.5, noise=0.02, seed=113),
                ["-M", "REL", "1e-3", "-q"], {"GlobalSettings": {"tuningTarget": "TUNING_TARGET_SSIM"},
                                               "AlgoSettings": {}}))
    out.append(("ac_target_3d", spectral_field((64, 80, 96), slope=-2.0, noise=0.06, seed=200), ["-M", "REL", "1e-4"],
                {"GlobalSettings": {"tuningTarget": "TUNING_TARGET_AC"},
                 "AlgoSettings": {"autoTuningRate": "0.01", "predictorTuningRate": "0.01",
                                  "levelwisePredictionSelection": "4", "maxStep": "32", "sampleBlockSize": "16"}}))
    out.append(("ac_target_2d", spectral_field((400, 500), slope=-3.0, noise=0.02, seed=115), ["-M", "REL", "5e-3"],
                {"GlobalSettings": {"tuningTarget": "TUNING_TARGET_AC"},
                 "AlgoSettings": {"autoTuningRate": "0.01", "predictorTuningRate": "0.01",
                                  "levelwisePredictionSelection": "6", "maxStep": "64"}}))
    out.append(("ac_target_lorenzo", sum2d((64, 72, 80), 1e-3, 242), ["-M", "REL", "1e-3"],
                {"GlobalSettings": {"tuningTarget": "TUNING_TARGET_AC"},
                 "AlgoSettings": {"autoTuningRate": "0.01", "predictorTuningRate": "0.01", "testLorenzo": "1",
                                  "sampleBlockSize": "16"}}))
    out.append(("rate_ab_only", spectral_field((48, 56, 64), slope=-3.0, seed=82), ["-M", "REL", "1e-3"],
                {"GlobalSettings": {}, "AlgoSettings": {"autoTuningRate": "0.01", "predictorTuningRate": "0.01"}}))
    out.append(("rate_2d", spectral_field((400, 500), slope=-3.0, seed=83), ["-M", "REL", "5e-3"],
                {"GlobalSettings": {}, "AlgoSettings": {"autoTuningRate": "0.01", "predictorTuningRate": "0.01",
                                                        "levelwisePredictionSelection": "6", "maxStep": "64"}}))
    return out


def sum1d(shape, noise, seed, dtype=np.float32):
    """f(i) + g(j) plus white noise of `noise` x range (the 2-D Lorenzo
    predictor reproduces sums of 1-D functions)."""
    rng = np.random.default_rng(seed)
    f = rng.standard_normal((shape[0], 1))
    g = rng.standard_normal((1, shape[1]))
    base = np.cumsum(f, axis=0) + np.cumsum(g, axis=1)
    return (base + noise * rng.standard_normal(shape) * (base.max() - base.min())).astype(dtype)


def flat_outside(shape, frac, seed, dtype=np.float32):
    """A spectral field (k^-3, 2% noise) in the leading `frac` of every axis,
    constant elsewhere (blocks the QoZ tuner's profiling filters out)."""
    x = spectral_field(shape, slope=-3.0, noise=0.02, seed=seed, dtype=dtype)
    m = np.zeros(shape, bool)
    m[tuple(slice(0, int(n * frac)) for n in shape)] = True
    return np.where(m, x, dtype(1.0)).astype(dtype)


def sum2d(shape, noise, seed, dtype=np.float32):
    """f(i,j) + g(j,k) + h(i,k) plus white noise of `noise` x range."""
    rng = np.random.default_rng(seed)
    f = rng.standard_normal((shape[0], shape[1], 1))
    g = rng.standard_normal((1, shape[1], shape[2]))
    h = rng.standard_normal((shape[0], 1, shape[2]))
    base = f + g + h
    return (base + noise * rng.standard_normal(shape) * (base.max() - base.min())).astype(dtype)


# OpenMP thread count of the reference run (the stream's slab count)
OMP_THREADS = {"omp_interp_3": 3, "omp_default_4": 4, "omp_abs2d_5": 5}
# Cases whose stream the reference tool writes but cannot decode.  reg1d_thin:
# the 1-D field's last block holds one point, the composed predictor picks
# regression for it, regression refuses a one-point block and the frontend
# falls back to Lorenzo without recording a selection; the decoder still reads
# one selection per block, past the end of the decoded selections
# (ComposedPredictor.hpp:65-68, SZGeneralFrontend.hpp:96-100), and crashes.
REF_DECODE_FAILS = {"reg1d_thin"}


def write_ini(path, d):
    with open(path, "w") as f:
        for sec, kv in d.items():
            f.write(f"[{sec}]\n")
            for k, v in kv.items():
                f.write(f"{k} = {v}\n")


def sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def main(only=None):
    """Generate every case, or (names given on the command line) only those,
    replacing their manifest entries."""
    if not os.path.exists(FAZ):
        subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh"), os.environ["FAZ_REFERENCE_ROOT"]])
    manifest = []
    old = {}
    mpath = os.path.join(HERE, "manifest.json")
    if only and os.path.exists(mpath):
        old = {c["name"]: c for c in json.load(open(mpath))["cases"]}
    for name, arr, flags, ini in cases():
        if only and name not in only:
            if name in old:
                manifest.append(old[name])
            continue
        arr = np.ascontiguousarray(arr)
        dims = list(arr.shape)
        inp = os.path.join(HERE, name + ".in")
        arr.tofile(inp)
        dt = "-f" if arr.dtype == np.float32 else "-d"
        cli_dims = [f"-{len(dims)}"] + [str(d) for d in reversed(dims)]
        with tempfile.TemporaryDirectory() as td:
            # "-F 0" goes first: the reference parses it with sscanf("%d") into
            # a bool, which overwrites neighbouring option variables
            # (test/faz.cpp:327-332), so options given before it can be lost.
            cmd = [FAZ, dt, "-F", "0", "-i", inp, "-z", os.path.join(HERE, name + ".faz")] + cli_dims + flags
            if ini is not None:
                ip = os.path.join(td, "cfg.ini")
                write_ini(ip, ini)
                cmd += ["-c", ip]
            env = dict(os.environ)
            if name in OMP_THREADS:
                env["OMP_NUM_THREADS"] = str(OMP_THREADS[name])
            subprocess.check_call(cmd, cwd=td, stdout=subprocess.DEVNULL, env=env)
            dcmd = [FAZ, dt, "-z", os.path.join(HERE, name + ".faz"), "-o", os.path.join(HERE, name + ".dec")] + \
                cli_dims + ["-M", "ABS", "1"]
            rc = subprocess.call(dcmd, cwd=td, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            if rc != 0 and name not in REF_DECODE_FAILS:
                raise subprocess.CalledProcessError(rc, dcmd)
            if rc == 0 and name in REF_DECODE_FAILS:
                raise RuntimeError(name + ": the reference decoded a stream it is listed as failing on")
        decp = os.path.join(HERE, name + ".dec")
        entry = {"name": name, "dtype": str(arr.dtype), "dims": dims, "flags": flags, "ini": ini,
                 "sha256": {ext: sha(os.path.join(HERE, name + ext)) for ext in (".in", ".faz")},
                 "dec_sha256": None if name in REF_DECODE_FAILS else sha(decp)}
        if name in REF_DECODE_FAILS:
            entry["ref_decode"] = "the reference tool's decoder exits with signal %d on this stream" % -rc
        if name in OMP_THREADS:
            entry["omp_threads"] = OMP_THREADS[name]
        manifest.append(entry)
        if os.path.exists(decp):
            os.remove(decp)
        print(name, os.path.getsize(os.path.join(HERE, name + ".faz")))
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "reference_tool": "oracle/_ref/faz (zstd 1.4.5)",
                   "cases": manifest}, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:] or None)
