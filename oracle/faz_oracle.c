/*
 * faz_oracle.c - CPU oracle for FAZ's interpolation-predictor path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C restatement of the reference
 * algorithm used to check the CUDA path; tests/, __graft_entry__.smoke() and
 * the CPU-baseline leg of bench.py are its only users.  The product library
 * (faz_gb300/) never links or calls it.
 *
 * Parity of this restatement is pinned against streams written by the
 * reference's own build (tests/golden/, generated by
 * tests/golden/make_golden.py from oracle/_ref/faz).
 *
 * Covered (reference file:line, paths relative to the reference root):
 *   error bound      include/QoZ/utils/Statistic.hpp:12-66
 *   interpolation    include/QoZ/compressor/SZInterpolationCompressor.hpp:42-199, 324-529,
 *                    820-923, 1306-1417, 3076-3442; include/QoZ/utils/Interpolators.hpp:9-36
 *   quantiser        include/QoZ/quantizer/IntegerQuantizer.hpp:69-226
 *   Huffman          include/QoZ/encoder/HuffmanEncoder.hpp:93-296, 455-633
 *   map order        include/QoZ/utils/ska_hash/unordered_map.hpp:295-304, 412-450, 605-643
 *                    and flat_hash_map.hpp:1268-1300 (fibonacci_hash_policy)
 *   zstd framing     include/QoZ/lossless/Lossless_zstd.hpp:22-47
 *   trailer          include/QoZ/utils/Config.hpp:240-388, include/QoZ/api/sz.hpp:54-205
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/faz_gb300.h"

/* ------------------------------------------------------------------ utils */

typedef struct {
    uint8_t *p;
    size_t n, cap;
} bytes_t;

static void b_reserve(bytes_t *b, size_t more) {
    if (b->n + more > b->cap) {
        size_t c = b->cap ? b->cap : 4096;
        while (c < b->n + more) c *= 2;
        b->p = (uint8_t *)realloc(b->p, c);
        b->cap = c;
    }
}
static void b_put(bytes_t *b, const void *src, size_t len) {
    b_reserve(b, len);
    memcpy(b->p + b->n, src, len);
    b->n += len;
}
#define PUT(b, v)                      \
    do {                               \
        __typeof__(v) _t = (v);        \
        b_put((b), &_t, sizeof(_t));   \
    } while (0)
#define PUTGET(r, v) r_get((r), &(v), sizeof(v))

typedef struct {
    const uint8_t *p;
    size_t n, pos;
    int bad;
} rd_t;
static void r_get(rd_t *r, void *dst, size_t len) {
    if (r->pos + len > r->n) { r->bad = 1; memset(dst, 0, len); return; }
    memcpy(dst, r->p + r->pos, len);
    r->pos += len;
}

static void put_be32(bytes_t *b, int32_t v) {
    uint8_t t[4] = {(uint8_t)(v >> 24), (uint8_t)(v >> 16), (uint8_t)(v >> 8), (uint8_t)v};
    b_put(b, t, 4);
}
static int32_t get_be32(rd_t *r) {
    uint8_t t[4];
    r_get(r, t, 4);
    return (int32_t)(((uint32_t)t[0] << 24) | ((uint32_t)t[1] << 16) | ((uint32_t)t[2] << 8) | t[3]);
}

static char g_err[512];
static void set_err(const char *m) { snprintf(g_err, sizeof g_err, "%s", m); }
const char *orc_last_error(void) { return g_err; }

/* ------------------------------------------------------------------- zstd */

typedef size_t (*zcomp_t)(void *, size_t, const void *, size_t, int);
typedef size_t (*zdecomp_t)(void *, size_t, const void *, size_t);
typedef unsigned (*ziserr_t)(size_t);
typedef size_t (*zbound_t)(size_t);
typedef unsigned (*zver_t)(void);
static void *g_z;
static zcomp_t z_comp;
static zdecomp_t z_decomp;
static ziserr_t z_iserr;
static zbound_t z_bound;
static zver_t z_ver;
static char g_zpath[1024] = "libzstd.so.1";

int orc_set_zstd(const char *path) {
    if (g_z) { dlclose(g_z); g_z = NULL; }
    snprintf(g_zpath, sizeof g_zpath, "%s", path && *path ? path : "libzstd.so.1");
    return 0;
}
static int z_load(void) {
    if (g_z) return 0;
    g_z = dlopen(g_zpath, RTLD_NOW | RTLD_LOCAL);
    if (!g_z) { set_err("cannot load zstd library"); return -1; }
    z_comp = (zcomp_t)dlsym(g_z, "ZSTD_compress");
    z_decomp = (zdecomp_t)dlsym(g_z, "ZSTD_decompress");
    z_iserr = (ziserr_t)dlsym(g_z, "ZSTD_isError");
    z_bound = (zbound_t)dlsym(g_z, "ZSTD_compressBound");
    z_ver = (zver_t)dlsym(g_z, "ZSTD_versionNumber");
    if (!z_comp || !z_decomp || !z_iserr || !z_bound || !z_ver) { set_err("zstd symbols missing"); return -1; }
    return 0;
}
unsigned orc_zstd_version(void) { return z_load() ? 0 : z_ver(); }

/* ------------------------------------------------------------ core context */

typedef struct {
    int N;
    size_t dims[4], offs[4], num;
    int levels;       /* interpolation_level after init() */
    int anchor;
    size_t maxStep;
    int perms[24][4];
    int nperm;
    int *codes;
    size_t ncodes, capcodes, qidx;
    /* blockwise tuning (compress_block / decompress_block): one interpolator
     * and direction per block, levels coarse to fine, blocks in order */
    uint8_t *bops, *bdirs;
    size_t nbops, capbops, bidx;
    int bad_blocks;  /* decompress: the list ran out */
} orc_ctx;

typedef struct {
    int interp, dir, blocksize, fixBlockSize;
    double alpha, beta;
    int nlist;
    const uint8_t *interp_list, *dir_list;
    int blockwise;  /* compress_block / decompress_block */
    int bwsbs;      /* blockwiseSampleBlockSize */
} orc_params;

static void bops_push(orc_ctx *c, int op, int dir) {
    if (c->nbops == c->capbops) {
        c->capbops = c->capbops ? c->capbops * 2 : 256;
        c->bops = (uint8_t *)realloc(c->bops, c->capbops);
        c->bdirs = (uint8_t *)realloc(c->bdirs, c->capbops);
    }
    c->bops[c->nbops] = (uint8_t)op;
    c->bdirs[c->nbops] = (uint8_t)dir;
    c->nbops++;
}

static void codes_push(orc_ctx *c, int v) {
    if (c->ncodes == c->capcodes) {
        c->capcodes = c->capcodes ? c->capcodes * 2 : 4096;
        c->codes = (int *)realloc(c->codes, c->capcodes * sizeof(int));
    }
    c->codes[c->ncodes++] = v;
}

/* smallest L with 2^L >= d, i.e. ceil(log2(d)) for d >= 1 */
static int ceil_log2(size_t d) {
    int l = 0;
    while (((size_t)1 << l) < d) l++;
    return l;
}

/* SZInterpolationCompressor::init - SZInterpolationCompressor.hpp:820-852 */
static void ctx_init(orc_ctx *c, int N, const size_t *dims, size_t maxStep) {
    memset(c, 0, sizeof *c);
    c->N = N;
    c->num = 1;
    c->levels = 0;
    for (int i = 0; i < N; i++) {
        c->dims[i] = dims[i];
        c->num *= dims[i];
        int l = ceil_log2(dims[i]);
        if (l > c->levels) c->levels = l;
    }
    c->maxStep = maxStep;
    if (maxStep > 0) {
        c->anchor = 1;
        c->levels += 1;
        int lm = 0;
        while (((size_t)1 << (lm + 1)) <= maxStep) lm++; /* floor(log2(maxStep)) */
        lm += 1;
        if (lm <= c->levels) c->levels = lm;
    }
    c->offs[N - 1] = 1;
    for (int i = N - 2; i >= 0; i--) c->offs[i] = c->offs[i + 1] * dims[i + 1];
    /* all permutations of 0..N-1 in lexicographic order (std::next_permutation) */
    int seq[4];
    for (int i = 0; i < N; i++) seq[i] = i;
    c->nperm = 0;
    for (;;) {
        memcpy(c->perms[c->nperm++], seq, sizeof seq);
        int i = N - 2;
        while (i >= 0 && seq[i] >= seq[i + 1]) i--;
        if (i < 0) break;
        int j = N - 1;
        while (seq[j] <= seq[i]) j--;
        int t = seq[i]; seq[i] = seq[j]; seq[j] = t;
        for (int a = i + 1, b = N - 1; a < b; a++, b--) { t = seq[a]; seq[a] = seq[b]; seq[b] = t; }
    }
}

#define T float
#define SFX f32
#include "oracle_interp.inc"
#undef T
#undef SFX
#define T double
#define SFX f64
#include "oracle_interp.inc"
#undef T
#undef SFX

/* --------------------------------------------------------------- Huffman */

/*
 * Order in which ska::unordered_map<int,size_t> (filled by frequency[s[i]]++,
 * HuffmanEncoder.hpp:534-537) yields its keys.  The table chains entries in
 * power-of-two bucket arrays; a key's bucket is the top log2(B) bits of
 * key * 11400714819323198485 (fibonacci_hash_policy); new keys go to the head
 * of their chain; the table doubles (minimum 4 buckets) when an insert would
 * exceed one entry per bucket, moving entries bucket 0..B-1, each chain head
 * to tail, to the head of their new chain; iteration walks buckets from B-1
 * down to 0, each chain head to tail.
 */
static void ska_order(const int *keys, size_t nkeys, int *order_out) {
    size_t B = 0;       /* 0 = initial empty state (one sentinel bucket) */
    int shift = 63;
    int *head = NULL;
    int *next = (int *)malloc((nkeys ? nkeys : 1) * sizeof(int));
    for (size_t k = 0; k < nkeys; k++) {
        if (B == 0 || k + 1 > B) {
            size_t nbkt = B == 0 ? 4 : 2 * B;
            if (nbkt < 4) nbkt = 4;
            int lg = 0;
            while (((size_t)1 << lg) < nbkt) lg++;
            int *nh = (int *)malloc(nbkt * sizeof(int));
            for (size_t i = 0; i < nbkt; i++) nh[i] = -1;
            int nshift = 64 - lg;
            for (size_t b = 0; b < B; b++) {
                int e = head[b];
                while (e >= 0) {
                    int nx = next[e];
                    size_t idx = (size_t)((uint64_t)(int64_t)keys[e] * 11400714819323198485ull >> nshift);
                    next[e] = nh[idx];
                    nh[idx] = e;
                    e = nx;
                }
            }
            free(head);
            head = nh;
            B = nbkt;
            shift = nshift;
        }
        size_t idx = (size_t)((uint64_t)(int64_t)keys[k] * 11400714819323198485ull >> shift);
        next[k] = head[idx];
        head[idx] = (int)k;
    }
    size_t o = 0;
    for (size_t b = B; b-- > 0;) {
        for (int e = head[b]; e >= 0; e = next[e]) order_out[o++] = e;
    }
    free(head);
    free(next);
}

typedef struct hnode {
    struct hnode *left, *right;
    size_t freq;
    char t;
    int c;
} hnode;

typedef struct {
    hnode *pool;
    int npool;
    hnode **qq; /* heap, entries 1..qend-1 */
    int qend;
    uint64_t *code;
    uint8_t *len;
    int stateNum;
    int offset;
    int nodeCount;
    hnode *root;
} huff_t;

/* qinsert / qremove - HuffmanEncoder.hpp:455-485 */
static void h_insert(huff_t *h, hnode *n) {
    int j, i = h->qend++;
    while ((j = i >> 1)) {
        if (h->qq[j]->freq <= n->freq) break;
        h->qq[i] = h->qq[j];
        i = j;
    }
    h->qq[i] = n;
}
static hnode *h_remove(huff_t *h) {
    int i = 1, l;
    hnode *n = h->qq[1];
    if (h->qend < 2) return NULL;
    h->qend--;
    h->qq[1] = h->qq[h->qend];
    while ((l = i << 1) < h->qend) {
        if (l + 1 < h->qend && h->qq[l + 1]->freq < h->qq[l]->freq) l++;
        if (h->qq[i]->freq > h->qq[l]->freq) {
            hnode *p = h->qq[i];
            h->qq[i] = h->qq[l];
            h->qq[l] = p;
            i = l;
        } else break;
    }
    return n;
}

/* build_code - HuffmanEncoder.hpp:493-521, codes up to 64 bits */
static void h_build(huff_t *h, hnode *n, int len, uint64_t out) {
    if (n->t) {
        h->code[n->c] = len == 0 ? 0 : (len <= 64 ? out << (64 - len) : out);
        h->len[n->c] = (uint8_t)len;
        return;
    }
    h_build(h, n->left, len + 1, out << 1);
    h_build(h, n->right, len + 1, (out << 1) | 1);
}

/* init / preprocess_encode - HuffmanEncoder.hpp:93-116, 529-566 */
static int huff_build(huff_t *h, const int *s, size_t n) {
    memset(h, 0, sizeof *h);
    int mx = s[0], mn = s[0];
    for (size_t i = 0; i < n; i++) {
        if (s[i] > mx) mx = s[i];
        if (s[i] < mn) mn = s[i];
    }
    size_t range = (size_t)((int64_t)mx - mn + 1);
    size_t *cnt = (size_t *)calloc(range, sizeof(size_t));
    int *keys = (int *)malloc(range * sizeof(int));
    size_t nk = 0;
    for (size_t i = 0; i < n; i++) {
        size_t k = (size_t)((int64_t)s[i] - mn);
        if (cnt[k]++ == 0) keys[nk++] = s[i];
    }
    int *ord = (int *)malloc(nk * sizeof(int));
    ska_order(keys, nk, ord);
    h->offset = mn;
    h->stateNum = mx - mn + 2;
    h->pool = (hnode *)calloc((size_t)h->stateNum * 4, sizeof(hnode));
    h->qq = (hnode **)calloc((size_t)h->stateNum * 4 + 2, sizeof(hnode *));
    h->qend = 1;
    h->code = (uint64_t *)calloc(h->stateNum, sizeof(uint64_t));
    h->len = (uint8_t *)calloc(h->stateNum, 1);
    for (size_t i = 0; i < nk; i++) {
        int key = keys[ord[i]];
        hnode *nd = &h->pool[h->npool++];
        nd->c = key - mn;
        nd->freq = cnt[key - mn];
        nd->t = 1;
        h_insert(h, nd);
    }
    while (h->qend > 2) {
        /* new_node(0, 0, qremove(), qremove()): the reference's compiler
         * evaluates the right argument first, so the first node removed
         * becomes the right child. */
        hnode *b = h_remove(h);
        hnode *a = h_remove(h);
        hnode *nd = &h->pool[h->npool++];
        nd->left = a;
        nd->right = b;
        nd->freq = a->freq + b->freq;
        nd->t = 0;
        h_insert(h, nd);
    }
    h->root = h->qq[1];
    h_build(h, h->root, 0, 0);
    h->nodeCount = (int)(2 * nk - 1);
    free(cnt);
    free(keys);
    free(ord);
    return 0;
}
static void huff_free(huff_t *h) {
    free(h->pool);
    free(h->qq);
    free(h->code);
    free(h->len);
}

/* pad_tree preorder numbering - HuffmanEncoder.hpp:569-584 */
static void h_pad(hnode *n, uint32_t i, uint32_t *L, uint32_t *R, int *C, uint8_t *t, uint32_t *ninode) {
    C[i] = n->c;
    t[i] = (uint8_t)n->t;
    if (n->left) {
        (*ninode)++;
        L[i] = *ninode;
        h_pad(n->left, *ninode, L, R, C, t, ninode);
    }
    if (n->right) {
        (*ninode)++;
        R[i] = *ninode;
        h_pad(n->right, *ninode, L, R, C, t, ninode);
    }
}

/* save - HuffmanEncoder.hpp:119-137, 607-633 */
static void huff_save(huff_t *h, bytes_t *b) {
    PUT(b, (int32_t)h->offset);
    put_be32(b, h->nodeCount);
    put_be32(b, h->stateNum / 2);
    uint32_t nc = (uint32_t)h->nodeCount;
    uint32_t *L = (uint32_t *)calloc(nc, 4), *R = (uint32_t *)calloc(nc, 4);
    int *C = (int *)calloc(nc, 4);
    uint8_t *t = (uint8_t *)calloc(nc, 1);
    uint32_t ninode = 0;
    h_pad(h->root, 0, L, R, C, t, &ninode);
    uint8_t endian = 0;
    b_put(b, &endian, 1);
    int w = nc <= 256 ? 1 : (nc <= 65536 ? 2 : 4);
    for (int pass = 0; pass < 2; pass++) {
        uint32_t *A = pass ? R : L;
        for (uint32_t i = 0; i < nc; i++) {
            if (w == 1) { uint8_t v = (uint8_t)A[i]; b_put(b, &v, 1); }
            else if (w == 2) { uint16_t v = (uint16_t)A[i]; b_put(b, &v, 2); }
            else b_put(b, &A[i], 4);
        }
    }
    b_put(b, C, (size_t)nc * 4);
    b_put(b, t, nc);
    free(L); free(R); free(C); free(t);
}

/* encode - HuffmanEncoder.hpp:150-227: size_t byte count, then the codes
 * concatenated most-significant bit first. */
static void huff_encode(huff_t *h, const int *s, size_t n, bytes_t *b) {
    uint64_t bits = 0;
    for (size_t i = 0; i < n; i++) bits += h->len[s[i] - h->offset];
    uint64_t nbytes = (bits + 7) / 8;
    PUT(b, (uint64_t)nbytes);
    b_reserve(b, nbytes);
    uint8_t *o = b->p + b->n;
    memset(o, 0, nbytes);
    uint64_t pos = 0;
    for (size_t i = 0; i < n; i++) {
        int st = s[i] - h->offset;
        int l = h->len[st];
        uint64_t c = h->code[st];
        for (int k = 0; k < l; k++, pos++)
            if ((c >> (63 - k)) & 1) o[pos >> 3] |= (uint8_t)(0x80 >> (pos & 7));
    }
    b->n += nbytes;
}

/* load + decode - HuffmanEncoder.hpp:236-296 */
static int huff_decode(rd_t *r, size_t target, int *out) {
    int32_t offset;
    r_get(r, &offset, 4);
    int32_t nodeCount = get_be32(r);
    (void)get_be32(r);
    if (r->bad || nodeCount <= 0) return -1;
    uint32_t nc = (uint32_t)nodeCount;
    int w = nc <= 256 ? 1 : (nc <= 65536 ? 2 : 4);
    uint8_t endian;
    r_get(r, &endian, 1);
    uint32_t *L = (uint32_t *)calloc(nc, 4), *R = (uint32_t *)calloc(nc, 4);
    int *C = (int *)calloc(nc, 4);
    uint8_t *t = (uint8_t *)calloc(nc, 1);
    for (int pass = 0; pass < 2; pass++) {
        uint32_t *A = pass ? R : L;
        for (uint32_t i = 0; i < nc; i++) {
            if (w == 1) { uint8_t v; r_get(r, &v, 1); A[i] = v; }
            else if (w == 2) { uint16_t v; r_get(r, &v, 2); A[i] = v; }
            else r_get(r, &A[i], 4);
        }
    }
    r_get(r, C, (size_t)nc * 4);
    r_get(r, t, nc);
    uint64_t enc;
    r_get(r, &enc, 8);
    if (r->bad || r->pos + enc > r->n) { free(L); free(R); free(C); free(t); return -1; }
    const uint8_t *bits = r->p + r->pos;
    int rc = 0;
    /* a tree of more than 256 nodes is rebuilt with a non-leaf root */
    int root_leaf = nc <= 256 ? t[0] : 0;
    if (root_leaf) {
        for (size_t i = 0; i < target; i++) out[i] = C[0] + offset;
    } else {
        uint32_t nd = 0;
        size_t cnt = 0;
        uint64_t i = 0;
        while (cnt < target) {
            if ((i >> 3) >= enc) { rc = -1; break; }
            int bit = (bits[i >> 3] >> (7 - (i & 7))) & 1;
            i++;
            nd = bit ? R[nd] : L[nd];
            if (nd == 0 || nd >= nc) { rc = -1; break; }
            if (t[nd]) {
                out[cnt++] = C[nd] + offset;
                nd = 0;
            }
        }
    }
    r->pos += enc;
    free(L); free(R); free(C); free(t);
    return rc;
}

#define T float
#define SFX f32
#include "oracle_lorenzo.inc"
#undef T
#undef SFX
#define T double
#define SFX f64
#include "oracle_lorenzo.inc"
#undef T
#undef SFX

static int z_framed_size(const uint8_t *p, size_t n, size_t *out);

#define T float
#define SFX f32
#include "oracle_metrics.inc"
#undef T
#undef SFX
#define T double
#define SFX f64
#include "oracle_metrics.inc"
#undef T
#undef SFX

#define T float
#define SFX f32
#include "oracle_general.inc"
#undef T
#undef SFX
#define T double
#define SFX f64
#include "oracle_general.inc"
#undef T
#undef SFX

/* ----------------------------------------------------- config and trailer */

/* Config::Config(Dims...) - Config.hpp:64-74, member defaults 394-499 */
int orc_config_init(faz_config *c, int N, const uint64_t *dims) {
    memset(c, 0, sizeof *c);
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
    c->rng = -1;
    c->alpha = -1;
    c->beta = -1;
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
    return 0;
}

/* Config::save - Config.hpp:240-309 */
static void conf_save(const faz_config *c, bytes_t *b) {
    PUT(b, (char)c->N);
    for (int i = 0; i < c->N; i++) PUT(b, (uint64_t)c->dims[i]);
    PUT(b, (uint64_t)c->num);
    PUT(b, c->cmprAlgo);
    PUT(b, c->errorBoundMode);
    PUT(b, c->tuningTarget);
    PUT(b, c->absErrorBound);
    PUT(b, c->relErrorBound);
    PUT(b, c->alpha);
    PUT(b, c->beta);
    PUT(b, c->lorenzo);
    PUT(b, c->lorenzo2);
    PUT(b, c->regression);
    PUT(b, c->regression2);
    PUT(b, c->interpAlgo);
    PUT(b, c->interpDirection);
    PUT(b, c->interpBlockSize);
    PUT(b, c->lossless);
    PUT(b, c->encoder);
    PUT(b, c->quantbinCnt);
    PUT(b, c->blockSize);
    PUT(b, c->levelwisePredictionSelection);
    PUT(b, c->blockwiseTuning);
    PUT(b, c->stride);
    PUT(b, (uint64_t)c->maxStep);
    PUT(b, c->pred_dim);
    PUT(b, c->openmp);
    PUT(b, c->fixBlockSize);
    PUT(b, c->blockwiseSampleBlockSize);
    PUT(b, c->crossBlock);
    PUT(b, c->wavelet);
    PUT(b, (uint64_t)c->firstSize);
    PUT(b, c->offsetPredictor);
    PUT(b, (uint64_t)c->coeffs_num);
    if (c->coeffs_num > 0) {
        PUT(b, (uint64_t)c->coeffs_dims_len);
        for (int i = 0; i < c->coeffs_dims_len; i++) PUT(b, (uint64_t)c->coeffs_dims[i]);
    }
    PUT(b, c->pid);
    PUT(b, c->blockOrder);
    PUT(b, c->sperr);
    PUT(b, c->sperrWithoutWave);
    PUT(b, c->pyBind);
    if (c->pyBind) PUT(b, (uint64_t)0); /* empty metadata string */
    PUT(b, c->conditioning);
    if (c->conditioning > 0) b_put(b, c->meta, 17);
}

/* Config::load - Config.hpp:311-388 */
static int conf_load(faz_config *c, rd_t *r) {
    char n;
    r_get(r, &n, 1);
    if (n < 1 || n > 4) return -1;
    c->N = n;
    for (int i = 0; i < n; i++) r_get(r, &c->dims[i], 8);
    r_get(r, &c->num, 8);
    r_get(r, &c->cmprAlgo, 1);
    r_get(r, &c->errorBoundMode, 1);
    r_get(r, &c->tuningTarget, 1);
    r_get(r, &c->absErrorBound, 8);
    r_get(r, &c->relErrorBound, 8);
    r_get(r, &c->alpha, 8);
    r_get(r, &c->beta, 8);
    r_get(r, &c->lorenzo, 1);
    r_get(r, &c->lorenzo2, 1);
    r_get(r, &c->regression, 1);
    r_get(r, &c->regression2, 1);
    r_get(r, &c->interpAlgo, 1);
    r_get(r, &c->interpDirection, 1);
    r_get(r, &c->interpBlockSize, 4);
    r_get(r, &c->lossless, 1);
    r_get(r, &c->encoder, 1);
    r_get(r, &c->quantbinCnt, 4);
    r_get(r, &c->blockSize, 4);
    r_get(r, &c->levelwisePredictionSelection, 4);
    r_get(r, &c->blockwiseTuning, 1);
    r_get(r, &c->stride, 4);
    r_get(r, &c->maxStep, 8);
    r_get(r, &c->pred_dim, 4);
    r_get(r, &c->openmp, 1);
    r_get(r, &c->fixBlockSize, 4);
    r_get(r, &c->blockwiseSampleBlockSize, 4);
    r_get(r, &c->crossBlock, 4);
    r_get(r, &c->wavelet, 4);
    r_get(r, &c->firstSize, 8);
    r_get(r, &c->offsetPredictor, 4);
    r_get(r, &c->coeffs_num, 8);
    if (c->coeffs_num > 0) {
        uint64_t len;
        r_get(r, &len, 8);
        if (len > 4) return -1;
        c->coeffs_dims_len = (int)len;
        for (uint64_t i = 0; i < len; i++) r_get(r, &c->coeffs_dims[i], 8);
    }
    r_get(r, &c->pid, 4);
    r_get(r, &c->blockOrder, 4);
    r_get(r, &c->sperr, 4);
    r_get(r, &c->sperrWithoutWave, 1);
    r_get(r, &c->pyBind, 1);
    if (c->pyBind) {
        uint64_t ms;
        r_get(r, &ms, 8);
        r->pos += ms;
    }
    r_get(r, &c->conditioning, 4);
    if (c->conditioning > 0) r_get(r, c->meta, 17);
    return r->bad ? -1 : 0;
}

/* data_range + calAbsErrorBound - Statistic.hpp:12-66 */
static int eb_resolve(faz_config *c, int dtype, const void *data) {
    if (c->errorBoundMode == FAZ_EB_ABS) return 0;
    double rng;
    if (dtype == FAZ_FLOAT) {
        const float *d = (const float *)data;
        float mx = d[0], mn = d[0];
        for (size_t i = 1; i < c->num; i++) {
            if (mx < d[i]) mx = d[i];
            if (mn > d[i]) mn = d[i];
        }
        rng = (double)(float)(mx - mn);
    } else {
        const double *d = (const double *)data;
        double mx = d[0], mn = d[0];
        for (size_t i = 1; i < c->num; i++) {
            if (mx < d[i]) mx = d[i];
            if (mn > d[i]) mn = d[i];
        }
        rng = mx - mn;
    }
    switch (c->errorBoundMode) {
    case FAZ_EB_REL:
        c->absErrorBound = c->relErrorBound * rng;
        break;
    case FAZ_EB_PSNR: {
        double v1 = c->psnrErrorBound + 10 * log10(1 - 2.0 / 3.0 * 0.99);
        c->absErrorBound = rng * pow(10, v1 / (-20));
        c->relErrorBound = c->absErrorBound / rng;
        break;
    }
    case FAZ_EB_L2NORM:
        c->absErrorBound = sqrt(3.0 / c->num) * c->l2normErrorBound;
        break;
    case FAZ_EB_ABS_AND_REL: {
        double rr = c->relErrorBound * rng;
        c->absErrorBound = c->absErrorBound < rr ? c->absErrorBound : rr;
        break;
    }
    case FAZ_EB_ABS_OR_REL: {
        double rr = c->relErrorBound * rng;
        c->absErrorBound = c->absErrorBound > rr ? c->absErrorBound : rr;
        break;
    }
    default:
        set_err("error bound mode not supported");
        return -1;
    }
    if (c->errorBoundMode != FAZ_EB_L2NORM) c->rng = rng;
    c->errorBoundMode = FAZ_EB_ABS;
    return 0;
}

/* ----------------------------------------------------------- public calls */

/*
 * Interpolation-only compression (the ALGO_INTERP body of
 * SZInterpolationCompressor::compress, lines 324-529): returns the quantisation
 * codes and unpredictable values in stream order plus the pre-zstd payload.
 * `conf` must already hold an absolute error bound.
 */
int orc_interp_compress(const faz_config *conf, int dtype, const void *data, int **codes_out,
                        size_t *ncodes, void **unpred_out, size_t *nunpred, uint8_t **payload,
                        size_t *payload_size) {
    orc_ctx c;
    size_t dims[4];
    for (int i = 0; i < conf->N; i++) dims[i] = conf->dims[i];
    ctx_init(&c, conf->N, dims, conf->maxStep);
    orc_params p = {conf->interpAlgo, conf->interpDirection, conf->interpBlockSize, conf->fixBlockSize,
                    conf->alpha, conf->beta, conf->interp_list_len, conf->interpAlgo_list,
                    conf->interpDirection_list, conf->blockwiseTuning, conf->blockwiseSampleBlockSize};
    if (conf->blockwiseTuning && (conf->N != 3 || conf->crossBlock || conf->blockOrder || conf->interpBlockSize < 1)) {
        /* block_interpolation_block3d is written for 3-D data; crossBlock and
         * other block orders are not covered */
        set_err("oracle covers blockwise tuning for 3-D data, crossBlock 0, block order 0");
        return -2;
    }
    if (conf->interpDirection >= c.nperm) { set_err("bad direction"); return -1; }
    for (int i = 0; i < conf->interp_list_len; i++)
        if (conf->interpDirection_list[i] >= c.nperm) { set_err("bad direction"); return -1; }
    size_t es = dtype == FAZ_FLOAT ? 4 : 8;
    void *work = malloc(c.num * es);
    memcpy(work, data, c.num * es);
    void *unpred;
    size_t nun;
    double eb;
    int radius = conf->quantbinCnt / 2;
    if (dtype == FAZ_FLOAT) {
        run_f32 r; memset(&r, 0, sizeof r); r.c = &c; r.data = (float *)work;
        r.q.radius = radius;
        r.q.trim = conf->trimToZero;
        q_set_eb_f32(&r.q, conf->absErrorBound);
        levels_f32(&r, &p, 0, 0, NULL);
        unpred = r.q.unpred;
        nun = r.q.nunpred;
        eb = r.q.eb;
    } else {
        run_f64 r; memset(&r, 0, sizeof r); r.c = &c; r.data = (double *)work;
        r.q.radius = radius;
        r.q.trim = conf->trimToZero;
        q_set_eb_f64(&r.q, conf->absErrorBound);
        levels_f64(&r, &p, 0, 0, NULL);
        unpred = r.q.unpred;
        nun = r.q.nunpred;
        eb = r.q.eb;
    }
    free(work);
    /* stream header - SZInterpolationCompressor.hpp:485-512 */
    bytes_t b = {0};
    for (int i = 0; i < conf->N; i++) PUT(&b, (uint64_t)conf->dims[i]);
    PUT(&b, (uint32_t)conf->interpBlockSize);
    PUT(&b, (int32_t)conf->interpAlgo);
    PUT(&b, (int32_t)conf->interpDirection);
    PUT(&b, conf->alpha);
    PUT(&b, conf->beta);
    PUT(&b, (uint64_t)conf->maxStep);
    PUT(&b, (int32_t)conf->interp_list_len);
    PUT(&b, (uint8_t)conf->blockwiseTuning);
    PUT(&b, (int32_t)conf->fixBlockSize);
    PUT(&b, (uint64_t)conf->crossBlock);
    PUT(&b, (int32_t)conf->trimToZero);
    PUT(&b, (int32_t)conf->blockOrder);
    if (conf->blockwiseTuning) {
        /* compress_block (lines 753-757): the per-block choices */
        PUT(&b, (uint64_t)c.nbops);
        b_put(&b, c.bops, c.nbops);
        b_put(&b, c.bdirs, c.nbops);
    } else if (conf->interp_list_len > 0) {
        b_put(&b, conf->interpAlgo_list, conf->interp_list_len);
        b_put(&b, conf->interpDirection_list, conf->interp_list_len);
    }
    free(c.bops);
    free(c.bdirs);
    /* LinearQuantizer::save - IntegerQuantizer.hpp:185-201 */
    PUT(&b, (uint8_t)2);
    PUT(&b, eb);
    PUT(&b, (int32_t)radius);
    PUT(&b, (uint64_t)nun);
    b_put(&b, unpred, nun * es);
    huff_t h;
    huff_build(&h, c.codes, c.ncodes);
    huff_save(&h, &b);
    huff_encode(&h, c.codes, c.ncodes, &b);
    huff_free(&h);
    if (codes_out) *codes_out = c.codes; else free(c.codes);
    if (ncodes) *ncodes = c.ncodes;
    if (unpred_out) *unpred_out = unpred; else free(unpred);
    if (nunpred) *nunpred = nun;
    *payload = b.p;
    *payload_size = b.n;
    return 0;
}

/* Lossless_zstd::compress output size: size_t raw length + zstd frame
 * (include/QoZ/lossless/Lossless_zstd.hpp:22-32). */
static int z_framed_size(const uint8_t *p, size_t n, size_t *out) {
    if (z_load()) return -5;
    size_t bound = z_bound(n);
    uint8_t *tmp = (uint8_t *)malloc(bound ? bound : 1);
    size_t zs = z_comp(tmp, bound, p, n, 3);
    free(tmp);
    if (z_iserr(zs)) { set_err("zstd compress failed"); return -5; }
    *out = zs + 8;
    return 0;
}

/* data_range<T> (Statistic.hpp:12-21): max - min in the element type */
static double data_range(int dtype, const void *data, size_t n) {
    if (dtype == FAZ_FLOAT) {
        const float *d = (const float *)data;
        float mx = d[0], mn = d[0];
        for (size_t i = 1; i < n; i++) {
            if (mx < d[i]) mx = d[i];
            if (mn > d[i]) mn = d[i];
        }
        return (double)(float)(mx - mn);
    }
    const double *d = (const double *)data;
    double mx = d[0], mn = d[0];
    for (size_t i = 1; i < n; i++) {
        if (mx < d[i]) mx = d[i];
        if (mn > d[i]) mn = d[i];
    }
    return mx - mn;
}

#define T float
#define SFX f32
#include "oracle_qoz.inc"
#undef T
#undef SFX
#define T double
#define SFX f64
#include "oracle_qoz.inc"
#undef T
#undef SFX

/*
 * QoZ tuning (Tuning with conf.QoZ, include/QoZ/api/impl/SZInterp.hpp:1588-2557,
 * TUNING_TARGET_RD, no wavelets, no profiling): QoZ defaults, sampled blocks,
 * per-level interpolator and direction by summed prediction loss (tuning-2
 * compressions), then the alpha/beta search by bit rate and PSNR of trial
 * compressions (CompressTest).  On return conf holds the decisions.
 */
static int qoz_tune(faz_config *conf, int dtype, const void *data) {
    int N = conf->N;
    if (N != 2 && N != 3) { set_err("oracle QoZ tuner covers 2-D and 3-D data"); return -2; }
    if (conf->tuningTarget > 3 || conf->wavelet > 0 || conf->FZ) { set_err("oracle QoZ tuner covers the RD, CR, SSIM and AC targets"); return -2; }
    size_t es = dtype == FAZ_FLOAT ? 4 : 8;
    double rngT = dtype == FAZ_FLOAT ? (double)(float)conf->rng : conf->rng;   /* T rng = conf.rng */
    double rel_bound = conf->relErrorBound > 0 ? conf->relErrorBound : conf->absErrorBound / rngT;
    /* waveAutoFix (default 1) drops the Lorenzo trial above a relative bound
     * of 1e-3 (SZInterp.hpp:1592-1594) */
    if (rel_bound > 1e-3 || conf->tuningTarget == 2) conf->testLorenzo = 0;  /* and with the SSIM target */
    if (conf->QoZ) {
        if (conf->autoTuningRate <= 0) conf->autoTuningRate = N == 2 ? 0.01 : 0.005;
        if (conf->predictorTuningRate <= 0) conf->predictorTuningRate = N == 2 ? 0.01 : 0.005;
        if (conf->maxStep <= 0) conf->maxStep = N == 2 ? 64 : 32;
        if (conf->levelwisePredictionSelection <= 0) conf->levelwisePredictionSelection = N == 2 ? 6 : 4;
        if (conf->sampleBlockSize <= 0) conf->sampleBlockSize = N == 2 ? 64 : 32;
        /* FAZ features off (SZInterp.hpp:1611-1622); pyBind, sperr, conditioning and
         * sperrWithoutWave are trailer fields */
        conf->profiling = 0;
        conf->testLorenzo = 0;
        conf->sperr = -1;
        conf->conditioning = 0;
        conf->pyBind = 0;
        conf->sperrWithoutWave = 0;
    }
    if (conf->autoTuningRate < 0) {
        set_err("oracle QoZ-branch tuner covers autoTuningRate >= 0");
        return -2;
    }
    int max_interp_level = -1;
    for (int i = 0; i < N; i++) {
        int l = (int)ceil(log2((double)conf->dims[i]));
        if (max_interp_level < l) max_interp_level = l;
    }
    if (conf->maxStep > 0) {
        int t = (int)(unsigned)log2((double)conf->maxStep);
        if (t <= max_interp_level) max_interp_level = t;
        if (conf->levelwisePredictionSelection > max_interp_level) conf->levelwisePredictionSelection = max_interp_level;
    }
    size_t shortest = conf->dims[0];
    for (int i = 0; i < N; i++) if (conf->dims[i] < shortest) shortest = conf->dims[i];
    if (conf->sampleBlockSize <= 0) conf->sampleBlockSize = N == 2 ? 64 : 32;   /* SZInterp.hpp:1783-1786 */
    size_t minimum_sbs = 16;
    if ((size_t)conf->sampleBlockSize < minimum_sbs) conf->sampleBlockSize = (int)minimum_sbs;
    while ((size_t)conf->sampleBlockSize >= shortest) conf->sampleBlockSize /= 2;
    while (conf->autoTuningRate > 0 && (size_t)conf->sampleBlockSize >= 2 * minimum_sbs &&
           (pow(conf->sampleBlockSize, N) / (double)conf->num) > 1.5 * conf->autoTuningRate)
        conf->sampleBlockSize /= 2;
    size_t sbs = (size_t)conf->sampleBlockSize, bsz = sbs + 1;
    size_t per = N == 3 ? bsz * bsz * bsz : bsz * bsz;
    if (!(conf->predictorTuningRate > 0 && conf->predictorTuningRate < 1)) { set_err("predictorTuningRate outside (0,1)"); return -2; }
    size_t gdims[4];
    for (int i = 0; i < N; i++) gdims[i] = conf->dims[i];
    /* profiling: the blocks whose subsampled range exceeds the bound
     * (SZInterp.hpp:1820-1842); profiling_coeff scales the B-M CompressTests */
    size_t totalblock_num = 1;
    for (int i = 0; i < N; i++) totalblock_num *= (conf->dims[i] - 1) / sbs;
    double pcoeff = 1;
    size_t *pst = NULL, npst = 0;
    if (conf->profiling) {
        npst = dtype == FAZ_FLOAT
                   ? qoz_profile_f32((const float *)data, N, gdims, sbs, conf->absErrorBound, sbs / 4, &pst)
                   : qoz_profile_f64((const double *)data, N, gdims, sbs, conf->absErrorBound, sbs / 4, &pst);
        if (npst <= (size_t)(int)(0.3 * conf->predictorTuningRate)) conf->profiling = 0;
        if (conf->profiling) pcoeff = (double)npst / totalblock_num;
    }
    void *blocks;
    size_t nblk;
    if (conf->var_first) {
        /* sampleBlocks with var_first (SZInterp.hpp:1020-1037, 1086-1124): the
         * blocks of largest variance; without profiling only 3-D data samples
         * any block in the reference */
        if (!conf->profiling && N != 3) {
            free(pst);
            set_err("var_first sampling without profiling covers 3-D data");
            return -2;
        }
        size_t *cand = pst, ncand = npst;
        if (!conf->profiling) {
            ncand = totalblock_num;
            cand = (size_t *)malloc(ncand * 3 * sizeof(size_t));
            size_t t = 0;
            for (size_t x = 0; x < gdims[0] - sbs; x += sbs)
                for (size_t y = 0; y < gdims[1] - sbs; y += sbs)
                    for (size_t z = 0; z < gdims[2] - sbs; z += sbs) {
                        cand[3 * t] = x; cand[3 * t + 1] = y; cand[3 * t + 2] = z;
                        t++;
                    }
        }
        size_t k = (size_t)(totalblock_num * conf->predictorTuningRate);
        if (conf->profiling && k > npst) k = npst;
        if (k == 0) k = 1;
        nblk = dtype == FAZ_FLOAT ? qoz_sample_var_f32((const float *)data, N, gdims, sbs, cand, ncand, k, (float **)&blocks)
                                  : qoz_sample_var_f64((const double *)data, N, gdims, sbs, cand, ncand, k,
                                                       (double **)&blocks);
        if (cand != pst) free(cand);
    } else if (conf->profiling)
        nblk = dtype == FAZ_FLOAT ? qoz_sample_profiled_f32((const float *)data, N, gdims, sbs, conf->predictorTuningRate,
                                                            pst, npst, totalblock_num, (float **)&blocks)
                                  : qoz_sample_profiled_f64((const double *)data, N, gdims, sbs,
                                                            conf->predictorTuningRate, pst, npst, totalblock_num,
                                                            (double **)&blocks);
    else
        nblk = dtype == FAZ_FLOAT
                   ? qoz_sample_f32((const float *)data, N, gdims, sbs, conf->predictorTuningRate, (float **)&blocks)
                   : qoz_sample_f64((const double *)data, N, gdims, sbs, conf->predictorTuningRate, (double **)&blocks);
    free(pst);
    double o_alpha = conf->alpha, o_beta = conf->beta;
    /* without the alpha/beta search the decisions compare compression ratios
     * of CompressTests (TUNING_TARGET_CR) */
    const int cr_tests = conf->autoTuningRate == 0;
    double best_lorenzo_ratio = 0, best_interp_cr = 0;
    if (conf->testLorenzo && cr_tests) {
        /* SZInterp.hpp:1925-1932 */
        double br, m;
        int rc = dtype == FAZ_FLOAT
                     ? gen_test_f32((const float *)blocks, nblk, N, bsz, conf->absErrorBound, conf->rng, 1.0, &br, &m, NULL)
                     : gen_test_f64((const double *)blocks, nblk, N, bsz, conf->absErrorBound, conf->rng, 1.0, &br, &m, NULL);
        if (rc) { free(blocks); return rc; }
        best_lorenzo_ratio = (double)es * 8.0 / br;
    }
    if (conf->autoTuningRate > 0) {
        /* setABwithRelBound(rel_bound, 0) (SZInterp.hpp:1394-1420) */
        double a, b;
        if (rel_bound >= 0.01) { a = 2; b = 2; }
        else if (rel_bound >= 0.007) { a = 1.75; b = 2; }
        else if (rel_bound >= 0.004) { a = 1.5; b = 2; }
        else if (rel_bound > 0.001) { a = 1.25; b = 1.5; }
        else { a = 1; b = 1; }
        conf->alpha = a;
        conf->beta = b;
    }
    int L = conf->levelwisePredictionSelection;
    uint8_t il[FAZ_MAX_LEVELS], dl[FAZ_MAX_LEVELS];
    int dirs[2] = {0, N == 3 ? 5 : 1};
    size_t bd[4] = {bsz, bsz, bsz, bsz};
    if (L > 0) {
        /* one compressor (one quantiser) for every trial of this loop */
        quant_f32 q32; quant_f64 q64;
        memset(&q32, 0, sizeof q32); memset(&q64, 0, sizeof q64);
        q32.radius = q64.radius = 32768;
        q32.trim = q64.trim = conf->trimToZero;
        q_set_eb_f32(&q32, conf->absErrorBound);
        q_set_eb_f64(&q64, conf->absErrorBound);
        void *work = malloc(per * es);
        for (int level = L; level > 0; level--) {
            int start_level = level == L ? 9999 : level, end_level = level - 1;
            int best_op = 1, best_dir = 0;
            double best = DBL_MAX;
            for (int op = 0; op < 2; op++)
                for (int di = 0; di < 2; di++) {
                    orc_params p = {op, dirs[di], conf->interpBlockSize, conf->fixBlockSize, conf->alpha, conf->beta,
                                    0, NULL, NULL};
                    double cur = 0;
                    for (size_t k = 0; k < nblk; k++) {
                        orc_ctx c;
                        ctx_init(&c, N, bd, conf->maxStep);
                        memcpy(work, (const uint8_t *)blocks + k * per * es, per * es);
                        if (dtype == FAZ_FLOAT) cur += qoz_run_f32(&q32, &c, (float *)work, 2, &p, start_level, end_level, NULL);
                        else cur += qoz_run_f64(&q64, &c, (double *)work, 2, &p, start_level, end_level, NULL);
                        free(c.codes);
                    }
                    if (cur < best) { best = cur; best_op = op; best_dir = dirs[di]; }
                }
            il[level - 1] = (uint8_t)best_op;
            dl[level - 1] = (uint8_t)best_dir;
        }
        /* the candidate loop leaves its last candidate in the configuration */
        conf->interpAlgo = 1;
        conf->interpDirection = (uint8_t)dirs[1];
        free(work);
        free(q32.unpred);
        free(q64.unpred);
        if (cr_tests) {
            /* CompressTest of the Config as the loop leaves it: its last
             * candidate on every level, the lists not yet in the Config
             * (SZInterp.hpp:2020-2032) */
            orc_params p = {1, dirs[1], conf->interpBlockSize, conf->fixBlockSize, conf->alpha, conf->beta, 0, NULL,
                            NULL};
            double br, m;
            int rc = dtype == FAZ_FLOAT
                         ? qoz_compress_test_f32((const float *)blocks, nblk, N, bsz, &p, conf->absErrorBound,
                                                 conf->trimToZero, conf->maxStep, conf->rng, 1.0, &br, &m, NULL)
                         : qoz_compress_test_f64((const double *)blocks, nblk, N, bsz, &p, conf->absErrorBound,
                                                 conf->trimToZero, conf->maxStep, conf->rng, 1.0, &br, &m, NULL);
            if (rc) { free(blocks); return rc; }
            best_interp_cr = (double)es * 8.0 / br;
        }
    } else {
        /* one interpolator and direction for every level, by the compression
         * ratio of a CompressTest per candidate (SZInterp.hpp:2036-2076) */
        int best_op = 1, best_dir = 0;
        double best_cr = 0;
        for (int op = 0; op < 2; op++)
            for (int di = 0; di < 2; di++) {
                orc_params p = {op, dirs[di], conf->interpBlockSize, conf->fixBlockSize, conf->alpha, conf->beta,
                                0, NULL, NULL};
                double br, m;
                int rc = dtype == FAZ_FLOAT
                             ? qoz_compress_test_f32((const float *)blocks, nblk, N, bsz, &p, conf->absErrorBound,
                                                     conf->trimToZero, conf->maxStep, conf->rng, 1.0, &br, &m, NULL)
                             : qoz_compress_test_f64((const double *)blocks, nblk, N, bsz, &p, conf->absErrorBound,
                                                     conf->trimToZero, conf->maxStep, conf->rng, 1.0, &br, &m, NULL);
                if (rc) { free(blocks); return rc; }
                double cr = (double)es * 8.0 / br;
                if (cr > best_cr) { best_cr = cr; best_op = op; best_dir = dirs[di]; }
            }
        conf->interpAlgo = best_op;
        conf->interpDirection = (uint8_t)best_dir;
        if (cr_tests) best_interp_cr = best_cr;
    }
    conf->alpha = o_alpha;
    conf->beta = o_beta;
    /* SZInterp.hpp:2083 */
    int use_interp = best_interp_cr >= best_lorenzo_ratio || best_lorenzo_ratio >= 80 || best_interp_cr >= 80;
    /* B-M tuning (SZInterp.hpp:2187-2515) */
    if (conf->autoTuningRate > 0 && use_interp && conf->autoTuningRate != conf->predictorTuningRate) {
        /* its own sample at autoTuningRate, without profiling (SZInterp.hpp:2199-2202) */
        free(blocks);
        nblk = dtype == FAZ_FLOAT
                   ? qoz_sample_f32((const float *)data, N, gdims, sbs, conf->autoTuningRate, (float **)&blocks)
                   : qoz_sample_f64((const double *)data, N, gdims, sbs, conf->autoTuningRate, (double **)&blocks);
    }
    /* the SSIM and AC targets score the search's CompressTests by the
     * reconstructions of the sampled blocks (oracle_metrics.inc); the
     * original's SSIM cube statistics are computed once */
    const int tgt = conf->tuningTarget;
    tmetric_f32 tm32;
    tmetric_f64 tm64;
    memset(&tm32, 0, sizeof tm32);
    memset(&tm64, 0, sizeof tm64);
    double *om = NULL, *os = NULL, *orr = NULL;
    if (conf->autoTuningRate > 0 && (tgt == 2 || tgt == 3)) {
        const size_t ss = (size_t)conf->SSIMBlockSize;
        tm32.target = tm64.target = tgt;
        tm32.N = tm64.N = N;
        tm32.bsz = tm64.bsz = bsz;
        tm32.s = tm64.s = ss;
        if (tgt == 2) {
            size_t nc = dtype == FAZ_FLOAT ? ssim_stats_f32((const float *)blocks, nblk, N, bsz, ss, &om, &os, &orr)
                                           : ssim_stats_f64((const double *)blocks, nblk, N, bsz, ss, &om, &os, &orr);
            tm32.om = tm64.om = om;
            tm32.os = tm64.os = os;
            tm32.orr = tm64.orr = orr;
            tm32.ncube = tm64.ncube = nc;
        } else if (dtype == FAZ_FLOAT) {
            tm32.flat = (float *)malloc(nblk * per * sizeof(float));
        } else {
            tm64.flat = (double *)malloc(nblk * per * sizeof(double));
        }
    }
#define TM_RESET(t) ((t).metric = 0, (t).idx = 0, (t).nflat = 0, &(t))
#define TM32 (tgt >= 2 ? TM_RESET(tm32) : NULL)
#define TM64 (tgt >= 2 ? TM_RESET(tm64) : NULL)
    if (conf->autoTuningRate > 0) {
        double bestalpha = 1, bestbeta = 1, bestb = 9999, bestm = 0;
        /* init_alphalist / init_betalist (SZInterp.hpp:868-933); the CR
         * target compares bit rates alone (its CompressTest metric is 0) */
        const int cr = conf->tuningTarget == 1;
        static const double alist_rd[] = {1, 1.25, 1.5, 1.75, 2, 2.25, 2.5, 2.75, 3}, blist_rd[] = {1.5, 2, 3, 4};
        static const double alist_cr[] = {-1, 1, 1.25, 1.5, 1.75, 2}, blist_cr[] = {-1, 1.5, 2, 3};
        const double *alist = cr ? alist_cr : alist_rd, *blist = cr ? blist_cr : blist_rd;
        /* abList 0, 1, 2: alpha up to 2, 2.5, 3 */
        const int na = cr ? 6 : (conf->abList == 0 ? 5 : (conf->abList == 1 ? 7 : 9)), nbeta = 4;
        double oriabseb = conf->absErrorBound;
        for (int i = 0; i < na; i++) {
            for (int j = 0; j < nbeta; j++) {
                double alpha = alist[i], beta = blist[j];
                conf->absErrorBound = oriabseb;
                if ((alpha >= 1 && alpha > beta) || (alpha < 0 && beta != -1)) continue;
                orc_params p = {conf->interpAlgo, conf->interpDirection, conf->interpBlockSize, conf->fixBlockSize,
                                alpha, beta, L, il, dl};
                double br, m;
                int rc = dtype == FAZ_FLOAT
                             ? qoz_compress_test_f32((const float *)blocks, nblk, N, bsz, &p, conf->absErrorBound,
                                                     conf->trimToZero, conf->maxStep, conf->rng, pcoeff, &br, &m, TM32)
                             : qoz_compress_test_f64((const double *)blocks, nblk, N, bsz, &p, conf->absErrorBound,
                                                     conf->trimToZero, conf->maxStep, conf->rng, pcoeff, &br, &m, TM64);
                if (rc) { free(blocks); return rc; }
                if (getenv("ORC_TUNE_TRACE")) fprintf(stderr, "orc ab %g %g bitrate %.17g metric %.17g\n", alpha, beta, br, m);
                if (cr) m = 0;
                if ((!cr && m >= bestm && br <= bestb) || (cr && br <= bestb)) {
                    bestalpha = alpha; bestbeta = beta; bestb = br; bestm = m;
                } else if ((!cr && m <= bestm && br >= bestb) || (cr && br > bestb)) {
                    if ((alpha >= 1 && pow(alpha, max_interp_level - 1) <= beta) ||
                        (alpha < 1 && alpha * (max_interp_level - 1) <= beta))
                        break;
                    continue;
                } else {
                    double fix = br / bestb;
                    double br2, m2;
                    rc = dtype == FAZ_FLOAT
                             ? qoz_compress_test_f32((const float *)blocks, nblk, N, bsz, &p, conf->absErrorBound * fix,
                                                     conf->trimToZero, conf->maxStep, conf->rng, pcoeff, &br2, &m2, TM32)
                             : qoz_compress_test_f64((const double *)blocks, nblk, N, bsz, &p, conf->absErrorBound * fix,
                                                     conf->trimToZero, conf->maxStep, conf->rng, pcoeff, &br2, &m2, TM64);
                    if (rc) { free(blocks); return rc; }
                    if (cr) m2 = 0;
                    double a = (m - m2) / (br - br2);
                    double bb = m - a * br;
                    double reg = a * bestb + bb;
                    if (reg > bestm) { bestalpha = alpha; bestbeta = beta; bestb = br; bestm = m; }
                }
                if ((alpha >= 1 && pow(alpha, max_interp_level - 1) <= beta) ||
                    (alpha < 1 && alpha * (max_interp_level - 1) <= beta))
                    break;
            }
        }
        conf->absErrorBound = oriabseb;
        if (conf->testLorenzo) {
            /* the Lorenzo candidate: CompressTest with ALGO_LORENZO_REG against
             * the best alpha/beta point (SZInterp.hpp:2428-2486) */
            double br, m;
            int rc = dtype == FAZ_FLOAT ? gen_test_f32((const float *)blocks, nblk, N, bsz, oriabseb, conf->rng, pcoeff, &br, &m, TM32)
                                        : gen_test_f64((const double *)blocks, nblk, N, bsz, oriabseb, conf->rng, pcoeff, &br, &m, TM64);
            if (rc) { free(blocks); return rc; }
            if (cr) m = 0;
            if ((!cr && m >= bestm && br <= bestb) || (cr && br <= bestb)) {
                bestb = br; bestm = m; bestalpha = -1; bestbeta = -1; use_interp = 0;
            } else if ((!cr && m <= bestm && br >= bestb) || (cr && br > bestb)) {
                use_interp = 1;
            } else {
                double fix = br / bestb, br2, m2;
                rc = dtype == FAZ_FLOAT
                         ? gen_test_f32((const float *)blocks, nblk, N, bsz, oriabseb * fix, conf->rng, pcoeff, &br2, &m2, TM32)
                         : gen_test_f64((const double *)blocks, nblk, N, bsz, oriabseb * fix, conf->rng, pcoeff, &br2, &m2, TM64);
                if (rc) { free(blocks); return rc; }
                if (cr) m2 = 0;
                double a = (m - m2) / (br - br2);
                if (a > 0) {
                    double b = m - a * br;
                    double reg = a * bestb + b;
                    if (reg > bestm) { bestb = br; bestm = m; bestalpha = -1; bestbeta = -1; use_interp = 0; }
                }
            }
        }
        conf->alpha = bestalpha;
        conf->beta = bestbeta;
        conf->wavelet_rel_coeff = 1;
        conf->wavelet = 0;
    }
#undef TM32
#undef TM64
#undef TM_RESET
    free(om);
    free(os);
    free(orr);
    free(tm32.flat);
    free(tm64.flat);
    if (L > 0 && use_interp) {
        conf->interp_list_len = L;
        for (int i = 0; i < L; i++) { conf->interpAlgo_list[i] = il[i]; conf->interpDirection_list[i] = dl[i]; }
    }
    /* Lorenzo: the caller runs the Lorenzo follow-up */
    conf->cmprAlgo = use_interp ? FAZ_ALGO_INTERP : FAZ_ALGO_LORENZO_REG;
    free(blocks);
    return 0;
}

/* Fast-frontend payload of a 3-D field (SZ_compress_LorenzoReg with N == 3,
 * include/QoZ/api/impl/SZLorenzoReg.hpp:94-114). */
static int lorenzo3_payload(int dtype, const void *data, const size_t *dims, int bs, int pd, int lo, int lo2, int reg,
                            double eb, int radius, bytes_t *out) {
    if (dtype == FAZ_FLOAT) {
        fparams_f32 P;
        fparams_init_f32(&P, bs, pd, lo, lo2, reg, eb);
        return fast3_compress_f32((const float *)data, dims, &P, eb, radius, out);
    }
    fparams_f64 P;
    fparams_init_f64(&P, bs, pd, lo, lo2, reg, eb);
    return fast3_compress_f64((const double *)data, dims, &P, eb, radius, out);
}

/* compressed size (zstd framing included) of a Lorenzo trial on 3-D data */
static int lorenzo3_size(int dtype, const void *data, const size_t *dims, int bs, int pd, double eb, int radius,
                         size_t *size) {
    bytes_t b = {0};
    int rc = lorenzo3_payload(dtype, data, dims, bs, pd, 1, 1, 0, eb, radius, &b);
    if (!rc) rc = z_framed_size(b.p, b.n, size);
    free(b.p);
    return rc;
}

/* General-frontend payload of a 1-D or 2-D field (SZ_compress_LorenzoReg with
 * N < 3, include/QoZ/api/impl/SZLorenzoReg.hpp:94-114): Lorenzo, two-layer
 * Lorenzo and linear-regression predictors as the Config enables them. */
static int gen_payload(int dtype, const void *data, int N, const size_t *dims, int bs, int lo, int lo2, int reg,
                       double eb, int radius, bytes_t *out) {
    if (dtype == FAZ_FLOAT) return gen_compress_f32((const float *)data, N, dims, bs, lo, lo2, reg, eb, radius, out);
    return gen_compress_f64((const double *)data, N, dims, bs, lo, lo2, reg, eb, radius, out);
}

static int gen_size(int dtype, const void *data, int N, const size_t *dims, int bs, double eb, int radius,
                    size_t *size) {
    bytes_t b = {0};
    int rc = gen_payload(dtype, data, N, dims, bs, 1, 1, 0, eb, radius, &b);
    if (!rc) rc = z_framed_size(b.p, b.n, size);
    free(b.p);
    return rc;
}

/* do_not_use_this_interp_compress_block_test (SZInterp.hpp:558-577) */
static int blockinterp_ratio(int dtype, const void *data, int N, const size_t *dims, size_t num, double eb, int op,
                             int dir, int bs, double *ratio) {
    bytes_t b = {0};
    int rc = dtype == FAZ_FLOAT ? blockinterp_compress_f32((const float *)data, N, dims, eb, op, dir, bs, &b)
                                : blockinterp_compress_f64((const double *)data, N, dims, eb, op, dir, bs, &b);
    size_t sz = 0;
    if (!rc) rc = z_framed_size(b.p, b.n, &sz);
    free(b.p);
    if (!rc) *ratio = num * 1.0 * (dtype == FAZ_FLOAT ? 4 : 8) / sz;
    return rc;
}

static void *sample_of(int dtype, const void *data, int N, const size_t *dims, size_t *sn, size_t *sd, size_t *sb) {
    if (dtype == FAZ_FLOAT) return sampling_f32((const float *)data, N, dims, sn, sd, sb);
    return sampling_f64((const double *)data, N, dims, sn, sd, sb);
}

/* Config::setDims side effects (Config.hpp:77-89) */
static void conf_set_dims_defaults(faz_config *c) {
    c->blockSize = c->N == 1 ? 128 : (c->N == 2 ? 16 : 6);
    c->pred_dim = c->N;
    c->stride = c->blockSize;
}

/* Lorenzo follow-up of both tuners (SZInterp.hpp:2779-2837, 2797-2845): the
 * Lorenzo settings, the quantisation-interval estimate and the pred_dim and
 * 16384-bin trials on the sample smp (sn points, dims sd), from the Lorenzo
 * ratio best_l. */
static int lorenzo_followup(faz_config *conf, int dtype, const void *data, const void *smp, size_t sn,
                            const size_t *sd, double best_l) {
    const int N = conf->N;
    size_t dims[4];
    for (int i = 0; i < N; i++) dims[i] = conf->dims[i];
    const size_t es = dtype == FAZ_FLOAT ? 4 : 8;
    const double eb = conf->absErrorBound;
    size_t osz;
    double ratio;
    int rc;
    faz_config lc = *conf;
    lc.cmprAlgo = FAZ_ALGO_LORENZO_REG;
    lc.lorenzo = 1; lc.lorenzo2 = 1; lc.regression = 0; lc.regression2 = 0; lc.openmp = 0;
    lc.blockSize = 5;
    conf_set_dims_defaults(&lc);   /* setDims(sample dims) */
    if (N == 3) {
        if (dtype == FAZ_FLOAT)
            lc.quantbinCnt = opt_quant_intervals_f32((const float *)data, dims[0], dims[1], dims[2], eb);
        else
            lc.quantbinCnt = opt_quant_intervals_f64((const double *)data, dims[0], dims[1], dims[2], eb);
        lc.pred_dim = 2;
        rc = lorenzo3_size(dtype, smp, sd, lc.blockSize, lc.pred_dim, eb, lc.quantbinCnt / 2, &osz);
        if (rc) return rc;
        ratio = sn * 1.0 * es / osz;
        if (ratio > best_l * 1.02) best_l = ratio; else lc.pred_dim = 3;
    }
    if (conf->relErrorBound < 1.01e-6 && best_l > 5 && lc.quantbinCnt != 16384) {
        int q0 = lc.quantbinCnt;
        lc.quantbinCnt = 16384;
        rc = N == 3 ? lorenzo3_size(dtype, smp, sd, lc.blockSize, lc.pred_dim, eb, lc.quantbinCnt / 2, &osz)
                    : gen_size(dtype, smp, N, sd, lc.blockSize, eb, lc.quantbinCnt / 2, &osz);
        if (rc) return rc;
        ratio = sn * 1.0 * es / osz;
        if (ratio > best_l * 1.02) best_l = ratio; else lc.quantbinCnt = q0;
    }
    conf_set_dims_defaults(&lc);   /* setDims(full dims) */
    *conf = lc;
    return 0;
}

/*
 * ALGO_INTERP_LORENZO without QoZ tuning (SZ_compress_Interp_lorenzo,
 * SZInterp.hpp:2561-2880, with the SZ3 branch of Tuning, 2115-2187): range and
 * relative bound, sampling, Lorenzo trial, linear / cubic block-interpolation
 * trials, direction trial (kept above a 2% gain), interp-or-Lorenzo choice;
 * for Lorenzo the quantisation-interval estimate and the pred_dim and 16384-bin
 * trials.  On return conf holds the decisions (cmprAlgo, interpAlgo,
 * interpDirection, quantbinCnt, Lorenzo settings).  3-D data only when the
 * field is large enough to be sampled.
 */
static int sz3_tune(faz_config *conf, int dtype, const void *data) {
    int N = conf->N;
    size_t dims[4];
    for (int i = 0; i < N; i++) dims[i] = conf->dims[i];
    size_t es = dtype == FAZ_FLOAT ? 4 : 8;
    if (conf->rng < 0) conf->rng = data_range(dtype, data, conf->num);
    if (conf->relErrorBound <= 0) conf->relErrorBound = conf->absErrorBound / conf->rng;
    /* Tuning's QoZ branch: QoZ, or any predictorTuningRate in (0, 1) (SZInterp.hpp:1857) */
    if (conf->QoZ || (conf->predictorTuningRate > 0 && conf->predictorTuningRate < 1)) {
        int rc = qoz_tune(conf, dtype, data);
        if (rc || conf->cmprAlgo != FAZ_ALGO_LORENZO_REG) return rc;
        /* Lorenzo chosen (SZInterp.hpp:2797-2845): the Lorenzo ratio of the
         * sample under the Lorenzo settings, then the follow-up */
        size_t sn, sd[4], sb;
        void *smp = sample_of(dtype, data, N, dims, &sn, sd, &sb);
        conf->lorenzo = 1; conf->lorenzo2 = 1; conf->regression = 0; conf->regression2 = 0; conf->openmp = 0;
        conf->blockSize = 5;
        if (sn == conf->num) { free(smp); return 0; }
        faz_config lc = *conf;
        conf_set_dims_defaults(&lc);   /* setDims(sample dims) */
        size_t osz;
        rc = N == 3 ? lorenzo3_size(dtype, smp, sd, lc.blockSize, lc.pred_dim, conf->absErrorBound, lc.quantbinCnt / 2, &osz)
                    : gen_size(dtype, smp, N, sd, lc.blockSize, conf->absErrorBound, lc.quantbinCnt / 2, &osz);
        if (!rc) rc = lorenzo_followup(conf, dtype, data, smp, sn, sd, sn * 1.0 * es / osz);
        free(smp);
        return rc;
    }
    if (conf->autoTuningRate > 0 || conf->predictorTuningRate > 0 || conf->preTrim > 0 || conf->wavelet > 0) {
        set_err("oracle covers the SZ3 and QoZ tuners only");
        return -2;
    }
    size_t sn, sd[4], sb;
    void *smp = sample_of(dtype, data, N, dims, &sn, sd, &sb);
    if (sn == conf->num) {
        free(smp);
        conf->cmprAlgo = FAZ_ALGO_INTERP;
        return 0;
    }
    if (N == 4) { free(smp); set_err("oracle tunes sampled 1-D to 3-D fields"); return -2; }
    double eb = conf->absErrorBound;
    size_t osz;
    /* the Lorenzo trial: lorenzo + lorenzo2, blockSize 5 (SZInterp.hpp:2115-2140) */
    int rc = N == 3 ? lorenzo3_size(dtype, smp, sd, 5, 3, eb, conf->quantbinCnt / 2, &osz)
                    : gen_size(dtype, smp, N, sd, 5, eb, conf->quantbinCnt / 2, &osz);
    if (rc) { free(smp); return rc; }
    double best_l = sn * 1.0 * es / osz, best_i = 0, ratio;
    for (int op = 0; op <= 1; op++) {
        rc = blockinterp_ratio(dtype, smp, N, sd, sn, eb, op, conf->interpDirection, (int)sb, &ratio);
        if (rc) { free(smp); return rc; }
        if (ratio > best_i) { best_i = ratio; conf->interpAlgo = op; }
    }
    int dop = N == 3 ? 5 : (N == 2 ? 1 : 0);  /* factorial(N) - 1 */
    rc = blockinterp_ratio(dtype, smp, N, sd, sn, eb, conf->interpAlgo, dop, (int)sb, &ratio);
    if (rc) { free(smp); return rc; }
    if (ratio > best_i * 1.02) { best_i = ratio; conf->interpDirection = dop; }
    int use_interp = !(best_l > best_i && best_l < 80 && best_i < 80);
    if (use_interp) {
        free(smp);
        conf->cmprAlgo = FAZ_ALGO_INTERP;
        return 0;
    }
    rc = lorenzo_followup(conf, dtype, data, smp, sn, sd, best_l);
    free(smp);
    return rc;
}

/* Pre-zstd payload of a resolved configuration (SZ_compress_dispatcher,
 * include/QoZ/api/impl/SZDispatcher.hpp:12-36). */
static int payload_for(faz_config *conf, int dtype, const void *data, uint8_t **payload, size_t *psize) {
    if (conf->cmprAlgo == FAZ_ALGO_INTERP)
        return orc_interp_compress(conf, dtype, data, NULL, NULL, NULL, NULL, payload, psize);
    if (conf->cmprAlgo == FAZ_ALGO_LORENZO_REG && conf->N < 3) {
        if (conf->regression2) {
            set_err("oracle covers the 1-D / 2-D general frontend without regression2");
            return -2;
        }
        size_t dims[2] = {conf->dims[0], conf->N == 2 ? conf->dims[1] : 1};
        bytes_t b = {0};
        int rc = gen_payload(dtype, data, conf->N, dims, conf->blockSize, conf->lorenzo, conf->lorenzo2,
                             conf->regression, conf->absErrorBound, conf->quantbinCnt / 2, &b);
        if (rc) { free(b.p); return rc; }
        *payload = b.p;
        *psize = b.n;
        return 0;
    }
    if (conf->cmprAlgo == FAZ_ALGO_LORENZO_REG) {
        if (conf->N != 3 || conf->regression2) { set_err("oracle covers the 3-D fast frontend"); return -2; }
        if (conf->blockSize < 1) { set_err("bad block size"); return -1; }
        size_t dims[3] = {conf->dims[0], conf->dims[1], conf->dims[2]};
        bytes_t b = {0};
        int rc = lorenzo3_payload(dtype, data, dims, conf->blockSize, conf->pred_dim, conf->lorenzo, conf->lorenzo2,
                                  conf->regression, conf->absErrorBound, conf->quantbinCnt / 2, &b);
        if (rc) { free(b.p); return rc; }
        *payload = b.p;
        *psize = b.n;
        return 0;
    }
    set_err("unsupported cmprAlgo");
    return -2;
}

/* SZ_compress<T>: error bound, tuner (ALGO_INTERP_LORENZO), payload,
 * Lossless_zstd framing, Config trailer, int32 trailer size. */
static int blocked_prepare(faz_config *c);

int orc_compress(const faz_config *conf_in, int dtype, const void *data, uint8_t **out, size_t *out_size,
                 uint8_t **payload_out, size_t *payload_size_out) {
    faz_config conf = *conf_in;
    if (conf.N < 1 || conf.N > 4) { set_err("N must be 1..4"); return -1; }
    if (conf.cmprAlgo != FAZ_ALGO_INTERP && conf.cmprAlgo != FAZ_ALGO_LORENZO_REG &&
        conf.cmprAlgo != FAZ_ALGO_INTERP_LORENZO && conf.cmprAlgo != FAZ_ALGO_INTERP_BLOCKED) {
        set_err("unsupported cmprAlgo");
        return -2;
    }
    if (eb_resolve(&conf, dtype, data)) return -1;
    if (conf.cmprAlgo == FAZ_ALGO_INTERP_BLOCKED) {
        int rc = blocked_prepare(&conf);
        if (rc) return rc;
    }
    if (conf.cmprAlgo == FAZ_ALGO_INTERP_LORENZO) {
        int rc = sz3_tune(&conf, dtype, data);
        if (rc) return rc;
    }
    uint8_t *payload;
    size_t psize;
    int rc = payload_for(&conf, dtype, data, &payload, &psize);
    if (rc) return rc;
    if (z_load()) { free(payload); return -5; }
    bytes_t b = {0};
    PUT(&b, (uint64_t)psize);
    size_t bound = z_bound(psize);
    b_reserve(&b, bound);
    size_t zs = z_comp(b.p + b.n, bound, payload, psize, 3);
    if (z_iserr(zs)) { free(payload); free(b.p); set_err("zstd compress failed"); return -5; }
    b.n += zs;
    size_t before = b.n;
    conf_save(&conf, &b);
    PUT(&b, (int32_t)(b.n - before));
    if (payload_out) { *payload_out = payload; *payload_size_out = psize; }
    else free(payload);
    *out = b.p;
    *out_size = b.n;
    return 0;
}

/* SZ_compress_Interp_blocked (include/QoZ/api/impl/SZInterp.hpp:3021-3500)
 * up to its compress_block call: the stream becomes ALGO_INTERP with
 * blockwise tuning, blocks of interpBlockSize (default 32 in 3-D) at every
 * level, per-block trials on blockwiseSampleBlockSize (default the block,
 * at least 4).  The alpha/beta search it runs for autoTuningRate > 0 is not
 * covered. */
static int blocked_prepare(faz_config *c) {
    if (c->N != 3) { set_err("ALGO_INTERP_BLOCKED is defined for 3-D data"); return -2; }
    if (c->autoTuningRate > 0) { set_err("oracle covers ALGO_INTERP_BLOCKED without autotuning"); return -2; }
    if (c->crossBlock || c->blockOrder) { set_err("oracle covers crossBlock 0, block order 0"); return -2; }
    c->cmprAlgo = FAZ_ALGO_INTERP;
    if (c->interpBlockSize <= 0) c->interpBlockSize = 32;
    int max_level = (int)log2((double)c->interpBlockSize) + 1;
    if (c->maxStep > 0) {
        int t = (int)log2((double)c->maxStep);
        if (t < max_level) max_level = t;
    }
    if (c->levelwisePredictionSelection > max_level) c->levelwisePredictionSelection = max_level;
    if (c->blockwiseSampleBlockSize == 0) c->blockwiseSampleBlockSize = c->interpBlockSize;
    if (c->blockwiseSampleBlockSize < 4) c->blockwiseSampleBlockSize = 4;
    c->fixBlockSize = c->interpBlockSize;
    c->blockwiseTuning = 1;
    return 0;
}

/* The tuner's decisions for a field, without compressing (for tests). */
int orc_sz3_tune(faz_config *conf, int dtype, const void *data) {
    if (eb_resolve(conf, dtype, data)) return -1;
    return sz3_tune(conf, dtype, data);
}

/* Split a stream into payload (zstd-decompressed) and trailer config. */
int orc_read_stream(const uint8_t *cmp, size_t cmp_size, faz_config *conf, uint8_t **payload,
                    size_t *payload_size) {
    if (cmp_size < 4) { set_err("stream too short"); return -4; }
    int32_t cs;
    memcpy(&cs, cmp + cmp_size - 4, 4);
    if (cs <= 0 || (size_t)cs + 4 > cmp_size) { set_err("bad trailer size"); return -4; }
    rd_t r = {cmp + cmp_size - 4 - cs, (size_t)cs, 0, 0};
    memset(conf, 0, sizeof *conf);
    if (conf_load(conf, &r)) { set_err("bad trailer"); return -4; }
    size_t body = cmp_size - 4 - cs;
    if (body < 8) { set_err("stream too short"); return -4; }
    uint64_t raw;
    memcpy(&raw, cmp, 8);
    if (z_load()) return -5;
    uint8_t *p = (uint8_t *)malloc(raw ? raw : 1);
    size_t got = z_decomp(p, raw, cmp + 8, body - 8);
    if (z_iserr(got) || got != raw) { free(p); set_err("zstd decompress failed"); return -5; }
    *payload = p;
    *payload_size = raw;
    return 0;
}

/* Config::save / Config::load bytes (include/QoZ/utils/Config.hpp:240-388),
 * for the OpenMP stream container */
int orc_config_save(const faz_config *conf, uint8_t **out, size_t *out_size) {
    bytes_t b = {0};
    conf_save(conf, &b);
    *out = b.p;
    *out_size = b.n;
    return 0;
}

int orc_config_load(const uint8_t *p, size_t n, faz_config *conf, size_t *used) {
    rd_t r = {p, n, 0, 0};
    memset(conf, 0, sizeof *conf);
    if (conf_load(conf, &r)) { set_err("bad Config"); return -4; }
    *used = r.pos;
    return 0;
}

/* SZ_decompress<T> / SZInterpolationCompressor::decompress (lines 42-199) */
int orc_decompress(const uint8_t *cmp, size_t cmp_size, int dtype, void **out, faz_config *conf_out) {
    faz_config conf;
    uint8_t *payload;
    size_t psize;
    int rc = orc_read_stream(cmp, cmp_size, &conf, &payload, &psize);
    if (rc) return rc;
    if (conf.cmprAlgo == FAZ_ALGO_LORENZO_REG && conf.N < 3) {
        /* SZ_decompress_LorenzoReg with N < 3: the general frontend */
        if (conf.regression2) {
            free(payload);
            set_err("oracle decodes 1-D / 2-D general-frontend streams without regression2");
            return -2;
        }
        size_t dims[2] = {conf.dims[0], conf.N == 2 ? conf.dims[1] : 1};
        size_t es = dtype == FAZ_FLOAT ? 4 : 8;
        void *dec = malloc(conf.num * es + es);
        rd_t r = {payload, psize, 0, 0};
        int rc2 = dtype == FAZ_FLOAT
                      ? gen_decompress_f32(&r, conf.N, dims, conf.lorenzo, conf.lorenzo2, conf.regression, (float *)dec)
                      : gen_decompress_f64(&r, conf.N, dims, conf.lorenzo, conf.lorenzo2, conf.regression,
                                           (double *)dec);
        free(payload);
        if (rc2) { free(dec); return rc2; }
        *out = dec;
        if (conf_out) *conf_out = conf;
        return 0;
    }
    if (conf.cmprAlgo == FAZ_ALGO_LORENZO_REG) {
        /* SZ_decompress_LorenzoReg with N == 3 (SZLorenzoReg.hpp:117-135) */
        if (conf.N != 3 || conf.regression2) {
            free(payload);
            set_err("oracle decodes 3-D fast-frontend streams");
            return -2;
        }
        size_t dims[3] = {conf.dims[0], conf.dims[1], conf.dims[2]};
        size_t es = dtype == FAZ_FLOAT ? 4 : 8;
        void *dec = malloc(conf.num * es + es);
        rd_t r = {payload, psize, 0, 0};
        int rc2 = dtype == FAZ_FLOAT ? fast3_decompress_f32(&r, dims, (float *)dec)
                                     : fast3_decompress_f64(&r, dims, (double *)dec);
        free(payload);
        if (rc2) { free(dec); return rc2; }
        *out = dec;
        if (conf_out) *conf_out = conf;
        return 0;
    }
    if (conf.cmprAlgo != FAZ_ALGO_INTERP) {
        free(payload);
        set_err("oracle decodes ALGO_INTERP streams");
        return -2;
    }
    rd_t r = {payload, psize, 0, 0};
    int N = conf.N;
    size_t dims[4];
    for (int i = 0; i < N; i++) { uint64_t v; r_get(&r, &v, 8); dims[i] = v; }
    uint32_t bsz;
    int32_t interp, dir, nlist, fixbs, trim, border;
    double alpha, beta;
    uint64_t maxStep, cross;
    uint8_t bwt;
    r_get(&r, &bsz, 4);
    r_get(&r, &interp, 4);
    r_get(&r, &dir, 4);
    r_get(&r, &alpha, 8);
    r_get(&r, &beta, 8);
    r_get(&r, &maxStep, 8);
    r_get(&r, &nlist, 4);
    r_get(&r, &bwt, 1);
    r_get(&r, &fixbs, 4);
    r_get(&r, &cross, 8);
    r_get(&r, &trim, 4);
    r_get(&r, &border, 4);
    uint8_t il[FAZ_MAX_LEVELS], dl[FAZ_MAX_LEVELS];
    uint64_t nbops = 0;
    const uint8_t *bops = NULL, *bdirs = NULL;
    if (bwt) {
        /* decompress_block (lines 233-239): the per-block choices */
        if (N != 3 || cross || border) { free(payload); set_err("oracle decodes blockwise 3-D streams"); return -2; }
        r_get(&r, &nbops, 8);
        if (r.bad || nbops > (r.n - r.pos) / 2) { free(payload); set_err("bad block list"); return -4; }
        bops = r.p + r.pos;
        bdirs = r.p + r.pos + nbops;
        r.pos += 2 * nbops;
        nlist = 0;
    } else {
        if (nlist < 0 || nlist > FAZ_MAX_LEVELS) { free(payload); set_err("bad level list"); return -4; }
        if (nlist > 0) { r_get(&r, il, nlist); r_get(&r, dl, nlist); }
    }
    uint8_t qtag;
    double eb;
    int32_t radius;
    uint64_t nun;
    r_get(&r, &qtag, 1);
    r_get(&r, &eb, 8);
    r_get(&r, &radius, 4);
    r_get(&r, &nun, 8);
    size_t es = dtype == FAZ_FLOAT ? 4 : 8;
    if (r.bad || r.pos + nun * es > r.n) { free(payload); set_err("truncated payload"); return -4; }
    const uint8_t *unp = r.p + r.pos;
    r.pos += nun * es;
    orc_ctx c;
    ctx_init(&c, N, dims, maxStep);
    c.codes = (int *)malloc(c.num * sizeof(int));
    c.ncodes = c.num;
    if (huff_decode(&r, c.num, c.codes)) { free(payload); free(c.codes); set_err("bad Huffman data"); return -4; }
    orc_params p = {interp, dir, (int)bsz, fixbs, alpha, beta, nlist, il, dl, bwt ? 1 : 0, 0};
    if (bwt) {
        c.bops = (uint8_t *)bops;
        c.bdirs = (uint8_t *)bdirs;
        c.nbops = nbops;
    }
    void *dec = malloc(c.num * es);
    if (dtype == FAZ_FLOAT) {
        run_f32 rr; memset(&rr, 0, sizeof rr); rr.c = &c; rr.data = (float *)dec; rr.decompress = 1;
        rr.q.radius = radius;
        rr.q.trim = trim;
        rr.q.unpred = (float *)malloc(nun * 4 + 4);
        memcpy(rr.q.unpred, unp, nun * 4);
        rr.q.nunpred = nun;
        q_set_eb_f32(&rr.q, eb);
        levels_f32(&rr, &p, 0, 0, NULL);
        free(rr.q.unpred);
    } else {
        run_f64 rr; memset(&rr, 0, sizeof rr); rr.c = &c; rr.data = (double *)dec; rr.decompress = 1;
        rr.q.radius = radius;
        rr.q.trim = trim;
        rr.q.unpred = (double *)malloc(nun * 8 + 8);
        memcpy(rr.q.unpred, unp, nun * 8);
        rr.q.nunpred = nun;
        q_set_eb_f64(&rr.q, eb);
        levels_f64(&rr, &p, 0, 0, NULL);
        free(rr.q.unpred);
    }
    free(c.codes);
    free(payload);
    if (c.bad_blocks || (bwt && c.bidx != nbops)) {
        free(dec);
        set_err("block list does not match the blocks");
        return -4;
    }
    *out = dec;
    if (conf_out) *conf_out = conf;
    return 0;
}

void orc_free(void *p) { free(p); }

/* The order ska_order() gives, exposed for tests. */
void orc_ska_order(const int *keys, size_t n, int *order) { ska_order(keys, n, order); }
