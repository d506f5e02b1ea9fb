// huffman_host.cpp - Huffman codebook construction and tree (de)serialisation.
//
// The GPU histogram gives every symbol's count and first stream position; the
// tree is then built on the host exactly as HuffmanEncoder::init does
// (include/QoZ/encoder/HuffmanEncoder.hpp:529-566): leaves enter a binary heap
// in the iteration order of the ska::unordered_map the reference fills with
// frequency[s[i]]++, pairs are merged until one root remains, and codes are
// read off the tree (left 0, right 1, build_code 493-521).  The serialised
// tree follows save/pad_tree (119-137, 569-633).
#include <algorithm>
#include <cstring>
#include <numeric>

#include "internal.h"

namespace faz {

namespace {

// Iteration order of ska::unordered_map<int, size_t> after inserting `keys`
// in order (include/QoZ/utils/ska_hash/unordered_map.hpp): separate chaining
// over a power-of-two bucket array (at least 4 buckets), bucket index = the
// top log2(B) bits of key * 0x9E3779B97F4A7C15 (fibonacci_hash_policy), new
// entries at the head of their chain, the array doubling when an insert
// would exceed one entry per bucket (entries move bucket by bucket, each
// chain front to back, to the head of their new chain), iteration from the
// last bucket down to bucket 0, each chain front to back.
std::vector<int> map_iteration_order(const std::vector<int> &keys) {
    const size_t n = keys.size();
    std::vector<int> next(n, -1);
    std::vector<int> head;
    size_t nb = 0;
    int shift = 63;
    auto bucket = [](int key, int sh) -> size_t {
        return (size_t)(((uint64_t)(int64_t)key * 0x9E3779B97F4A7C15ull) >> sh);
    };
    for (size_t k = 0; k < n; k++) {
        if (nb == 0 || k + 1 > nb) {
            size_t nnb = nb == 0 ? 4 : nb * 2;
            int lg = 0;
            while (((size_t)1 << lg) < nnb) lg++;
            int nsh = 64 - lg;
            std::vector<int> nh(nnb, -1);
            for (size_t b = 0; b < nb; b++) {
                for (int e = head[b]; e >= 0;) {
                    int nx = next[e];
                    size_t j = bucket(keys[e], nsh);
                    next[e] = nh[j];
                    nh[j] = e;
                    e = nx;
                }
            }
            head.swap(nh);
            nb = nnb;
            shift = nsh;
        }
        size_t j = bucket(keys[k], shift);
        next[k] = head[j];
        head[j] = (int)k;
    }
    std::vector<int> order;
    order.reserve(n);
    for (size_t b = nb; b-- > 0;)
        for (int e = head[b]; e >= 0; e = next[e]) order.push_back(e);
    return order;
}

// Binary min-heap on freq with the reference's sift rules (qinsert stops on
// parent <= new, qremove descends to the smaller child while parent > child).
// Entries carry their node's frequency, so comparisons touch the heap array
// alone.
struct Heap {
    struct E {
        uint64_t freq;
        int node;
    };
    std::vector<E> q;  // 1-based
    explicit Heap(size_t cap) {
        q.reserve(cap + 1);
        q.push_back({0, -1});
    }
    void insert(int nd, uint64_t fn) {
        q.push_back({fn, nd});
        size_t i = q.size() - 1, j;
        while ((j = i >> 1)) {
            if (q[j].freq <= fn) break;
            q[i] = q[j];
            i = j;
        }
        q[i] = {fn, nd};
    }
    int remove() {
        const int top = q[1].node;
        const E last = q.back();
        q.pop_back();
        const size_t end = q.size();
        if (end > 1) {
            q[1] = last;
            // the element moved to the top sinks; the choice of the smaller
            // child is unpredictable, so it is computed without a branch
            size_t i = 1, l;
            const E x = q[1];
            while ((l = i << 1) < end) {
                const size_t r = l + 1 < end ? l + 1 : l;
                l += (size_t)(q[r].freq < q[l].freq);
                if (!(x.freq > q[l].freq)) break;
                q[i] = q[l];
                i = l;
            }
            q[i] = x;
        }
        return top;
    }
    size_t size() const { return q.size() - 1; }
};

template <typename W>
void put_le(std::vector<uint8_t> &o, W v) {
    uint8_t b[sizeof(W)];
    std::memcpy(b, &v, sizeof(W));
    o.insert(o.end(), b, b + sizeof(W));
}

}  // namespace

int build_codebook(const std::vector<int> &syms, const std::vector<uint64_t> &counts,
                   const std::vector<uint64_t> &first, Codebook &cb, std::string &err) {
    const size_t d = syms.size();
    if (d == 0) {
        err = "Huffman input is empty";
        return FAZ_ERR_ARG;
    }
    // distinct symbols in order of first occurrence = map insertion order
    // (first positions are distinct stream positions)
    std::vector<std::pair<uint64_t, int>> byfirst(d);
    for (size_t i = 0; i < d; i++) byfirst[i] = {first[i], (int)i};
    std::sort(byfirst.begin(), byfirst.end());
    std::vector<int> keys(d);
    for (size_t i = 0; i < d; i++) keys[i] = syms[byfirst[i].second];
    std::vector<int> ord = map_iteration_order(keys);
    int mn = *std::min_element(syms.begin(), syms.end());
    int mx = *std::max_element(syms.begin(), syms.end());
    cb.offset = mn;
    cb.stateNum = mx - mn + 2;
    // nodes: leaves 0 .. d-1 in heap insertion order, then the merged nodes;
    // a merged node's children always have smaller indices
    const size_t nn = 2 * d - 1;
    std::vector<int> left(nn, -1), right(nn, -1), state(d);
    std::vector<uint64_t> freq(nn);
    Heap h(nn);
    for (size_t k = 0; k < d; k++) {
        const int si = byfirst[ord[k]].second;
        freq[k] = counts[si];
        state[k] = syms[si] - mn;
        h.insert((int)k, freq[k]);
    }
    size_t next = d;
    while (h.size() > 1) {
        // the reference evaluates new_node(0, 0, qremove(), qremove()) right
        // to left: the first node removed is the right child
        const int b = h.remove();
        const int a = h.remove();
        left[next] = a;
        right[next] = b;
        freq[next] = freq[a] + freq[b];
        h.insert((int)next, freq[next]);
        next++;
    }
    const int root = h.q[1].node;
    // code lengths and bits (left 0, right 1), parents before children
    std::vector<uint8_t> len(nn, 0);
    std::vector<uint64_t> bits(nn, 0);
    for (size_t i = nn; i-- > d;) {
        if (len[i] >= 64) {
            err = "Huffman code longer than 64 bits";
            return FAZ_ERR_UNSUPPORTED;
        }
        len[left[i]] = len[right[i]] = (uint8_t)(len[i] + 1);
        bits[left[i]] = bits[i] << 1;
        bits[right[i]] = (bits[i] << 1) | 1;
    }
    cb.code.assign(cb.stateNum, 0);
    cb.len.assign(cb.stateNum, 0);
    cb.maxlen = 0;
    for (size_t k = 0; k < d; k++) {
        const int l = len[k];
        cb.code[state[k]] = l == 0 ? 0 : bits[k] << (64 - l);
        cb.len[state[k]] = (uint8_t)l;
        cb.maxlen = std::max(cb.maxlen, l);
    }
    // serialise (pad_tree): preorder numbering - a node, its left subtree,
    // its right subtree - from subtree sizes, then the L/R/C/t arrays
    const uint32_t nc = (uint32_t)nn;
    cb.nodeCount = (int)nc;
    std::vector<uint32_t> size(nn, 1), num(nn, 0);
    for (size_t i = d; i < nn; i++) size[i] = 1 + size[left[i]] + size[right[i]];
    num[root] = 0;
    std::vector<uint32_t> L(nc, 0), R(nc, 0);
    std::vector<int32_t> C(nc, 0);
    std::vector<uint8_t> t(nc, 0);
    for (size_t i = nn; i-- > 0;) {
        const uint32_t me = num[i];
        if (i < d) {
            C[me] = state[i];
            t[me] = 1;
            continue;
        }
        num[left[i]] = me + 1;
        num[right[i]] = me + 1 + size[left[i]];
        L[me] = num[left[i]];
        R[me] = num[right[i]];
    }
    const int w = nc <= 256 ? 1 : (nc <= 65536 ? 2 : 4);
    std::vector<uint8_t> &o = cb.tree;
    o.assign(1 + 2 * (size_t)nc * w + (size_t)nc * 4 + nc, 0);
    uint8_t *p = o.data();
    *p++ = 0;  // endian byte: little endian
    for (int pass = 0; pass < 2; pass++) {
        const std::vector<uint32_t> &A = pass ? R : L;
        for (uint32_t i = 0; i < nc; i++, p += w) {
            if (w == 1) {
                *p = (uint8_t)A[i];
            } else if (w == 2) {
                const uint16_t v = (uint16_t)A[i];
                std::memcpy(p, &v, 2);
            } else {
                std::memcpy(p, &A[i], 4);
            }
        }
    }
    std::memcpy(p, C.data(), (size_t)nc * 4);
    p += (size_t)nc * 4;
    std::memcpy(p, t.data(), nc);
    return FAZ_OK;
}

// HuffmanEncoder::load (include/QoZ/encoder/HuffmanEncoder.hpp:276-296) plus
// a 2^kLutBits-entry lookup table for the GPU decoder.
int parse_tree(const uint8_t *&p, const uint8_t *end, DecodeTablesHost &t, std::string &err) {
    auto need = [&](size_t k) { return (size_t)(end - p) >= k; };
    if (!need(12)) {
        err = "truncated Huffman header";
        return FAZ_ERR_FORMAT;
    }
    int32_t offset;
    std::memcpy(&offset, p, 4);
    uint32_t nc = ((uint32_t)p[4] << 24) | ((uint32_t)p[5] << 16) | ((uint32_t)p[6] << 8) | p[7];
    p += 12;  // offset, nodeCount, stateNum/2
    if (nc == 0 || nc > (1u << 24)) {
        err = "bad Huffman node count";
        return FAZ_ERR_FORMAT;
    }
    int w = nc <= 256 ? 1 : (nc <= 65536 ? 2 : 4);
    size_t bytes = 1 + 2 * (size_t)nc * w + (size_t)nc * 4 + nc;
    if (!need(bytes)) {
        err = "truncated Huffman tree";
        return FAZ_ERR_FORMAT;
    }
    const uint8_t *q = p + 1;
    t.offset = offset;
    t.nodeCount = (int)nc;
    t.left.assign(nc, 0);
    t.right.assign(nc, 0);
    t.sym.assign(nc, 0);
    t.leaf.assign(nc, 0);
    for (int pass = 0; pass < 2; pass++) {
        std::vector<uint32_t> &A = pass ? t.right : t.left;
        for (uint32_t i = 0; i < nc; i++) {
            uint32_t v;
            if (w == 1) v = q[0];
            else if (w == 2) { uint16_t x; std::memcpy(&x, q, 2); v = x; }
            else std::memcpy(&v, q, 4);
            q += w;
            A[i] = v;
        }
    }
    std::memcpy(t.sym.data(), q, (size_t)nc * 4);
    q += (size_t)nc * 4;
    std::memcpy(t.leaf.data(), q, nc);
    p += bytes;
    // a tree of more than 256 nodes is rebuilt with an internal root
    bool root_leaf = nc <= 256 && t.leaf[0];
    t.constant = root_leaf;
    t.constant_state = t.sym[0];
    if (root_leaf) return FAZ_OK;
    t.leaf[0] = 0;
    // children are numbered after their parent (preorder): reject anything
    // else so that every walk ends
    for (uint32_t i = 0; i < nc; i++) {
        if (t.leaf[i]) continue;
        if (t.left[i] <= i || t.right[i] <= i || t.left[i] >= nc || t.right[i] >= nc) {
            err = "malformed Huffman tree";
            return FAZ_ERR_FORMAT;
        }
    }
    const int K = kLutBits;
    t.lut.assign((size_t)1 << K, 0);
    for (uint32_t v = 0; v < (1u << K); v++) {
        uint32_t nd = 0;
        int b = 0;
        for (; b < K; b++) {
            int bit = (v >> (K - 1 - b)) & 1;
            nd = bit ? t.right[nd] : t.left[nd];
            if (t.leaf[nd]) break;
        }
        if (b < K) t.lut[v] = ((uint32_t)(b + 1) << 24) | ((uint32_t)t.sym[nd] & 0xffffff);
        else t.lut[v] = 0x80000000u | nd;
    }
    return FAZ_OK;
}

}  // namespace faz
