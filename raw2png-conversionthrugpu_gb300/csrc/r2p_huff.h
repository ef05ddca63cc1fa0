// r2p_huff.h -- dynamic Huffman DEFLATE blocks (RFC 1951 3.2.7): code
// lengths, canonical codes and the block header.
//
// Plain sequential integer code shared by the GPU kernel (one thread builds a
// block's codes) and the host unit test (tests/cpp/huff_check.cpp), which
// checks it against zlib's inflate and against a heap-built Huffman code.
#pragma once
#include "r2p_common.h"

namespace r2p {

constexpr int kLLSyms = 286;   // literal/length alphabet
constexpr int kDSyms = 30;     // distance alphabet
constexpr int kCLSyms = 19;    // code-length alphabet
constexpr int kMaxCodeLen = 15;
constexpr int kMaxCLLen = 7;
// Header bits after BFINAL/BTYPE: 14 + 19 * 3 + (286 + 30) * (7 + 7) <= 4495
// (+ the 3 block-type bits ahead of them).
constexpr int kHdrWords = 144;

// Minimum-redundancy code lengths computed in place, after Moffat and
// Katajainen, "In-place calculation of minimum-redundancy codes" (WADS 1995).
// A[0..n-1] holds n >= 2 weights in non-decreasing order.
//
// Phase 1 pairs the two smallest items repeatedly.  Internal node k (k = 0
// .. n-2, created in order of non-decreasing weight) keeps its weight in A[k]
// until it is paired, then the index of its parent; the root n-2 keeps the
// total weight.
//
// The two queue heads and the items behind them are kept in registers (wr,
// wr1 for the internal nodes root, root + 1; wl, wl1 for the leaves leaf,
// leaf + 1), so each comparison waits on no memory load: the GPU runs this
// loop on one thread, where a load per comparison was the whole cost.  Node
// root + 1 exists once root + 1 < next; the node made in this step becomes a
// cached head when the queue in front of it is that short.  The leaves
// ahead are never overwritten before they are taken (leaf >= next + 2).
R2P_HD void mk_phase1(uint32_t* A, int n)
{
    A[0] += A[1];
    int root = 0, leaf = 2;
    uint32_t wr = A[0], wr1 = 0;
    uint32_t wl = leaf < n ? A[leaf] : 0u, wl1 = leaf + 1 < n ? A[leaf + 1] : 0u;
    for (int next = 1; next < n - 1; next++) {
        uint32_t w;
        if (leaf >= n || wr < wl) {                 // the queue is never empty here
            w = wr;
            A[root++] = (uint32_t)next;
            wr = wr1;
            wr1 = root + 1 < next ? A[root + 1] : 0u;
        } else {
            w = wl;
            leaf++;
            wl = wl1;
            wl1 = leaf + 1 < n ? A[leaf + 1] : 0u;
        }
        if (leaf >= n || (root < next && wr < wl)) {
            w += wr;
            A[root++] = (uint32_t)next;
            wr = wr1;
            wr1 = root + 1 < next ? A[root + 1] : 0u;
        } else {
            w += wl;
            leaf++;
            wl = wl1;
            wl1 = leaf + 1 < n ? A[leaf + 1] : 0u;
        }
        A[next] = w;
        if (root == next) wr = w;
        else if (root + 1 == next) wr1 = w;
    }
}

// Phases 2 and 3 restated per depth level (the GPU runs them in parallel):
// with c[d] internal nodes at depth d, level d offers 2 * c[d-1] places (one
// at the root level), of which the leaves take lv[d] = places - c[d]; leaves
// fill levels from the top, largest weight (index n-1) first.  P holds
// phase 1's output; L receives the code length of each sorted weight, D is
// scratch for the n-1 internal depths.  Returns the largest length.
R2P_HD int mk_levels(const uint32_t* P, int n, uint32_t* D, uint32_t* L)
{
    D[n - 2] = 0;
    for (int k = n - 3; k >= 0; k--) D[k] = D[P[k]] + 1;     // a parent's index exceeds its child's
    uint32_t c[64];
    for (int d = 0; d < 64; d++) c[d] = 0;
    for (int k = 0; k < n - 1; k++) c[D[k]]++;
    int idx = n - 1, d = 0;
    uint32_t places = 1;
    for (; idx >= 0; d++) {
        const uint32_t lv = places - c[d];
        for (uint32_t k = 0; k < lv; k++) L[idx--] = (uint32_t)d;
        places = 2 * c[d];
    }
    return d - 1;
}

// The whole computation in place (phases 2-3 as the published sequential
// loops): on return A[i] is the code length of the i-th weight.
R2P_HD void mk_lengths_inplace(uint32_t* A, int n)
{
    mk_phase1(A, n);
    A[n - 2] = 0;
    for (int next = n - 3; next >= 0; next--) A[next] = A[A[next]] + 1;
    int avail = 1, used = 0, depth = 0, next = n - 1, root = n - 2;
    while (avail > 0) {
        while (root >= 0 && (int)A[root] == depth) {
            used++;
            root--;
        }
        while (avail > used) {
            A[next--] = (uint32_t)depth;
            avail--;
        }
        avail = 2 * used;
        depth++;
        used = 0;
    }
}

// Lengths <= maxlen for n >= 2 sorted weights W (all >= 1) into L (same
// order; W is kept).  When the optimal code is too deep the weights are
// divided by 2, 4, ... (rounding up, which keeps their order and keeps them
// >= 1) and the code rebuilt; equal weights give depth ceil(log2 n), so this
// ends for any n <= 2^maxlen.
R2P_HD void limited_lengths(const uint32_t* W, int n, int maxlen, uint32_t* L)
{
    for (uint32_t sh = 0;; sh++) {
        const uint32_t add = (1u << sh) - 1u;
        for (int i = 0; i < n; i++) L[i] = (uint32_t)(((uint64_t)W[i] + add) >> sh);
        mk_lengths_inplace(L, n);
        if ((int)L[0] <= maxlen) return;
    }
}

// Symbols with freq > 0 sorted by (freq, symbol), by insertion (small
// alphabets and host use); returns their count.
R2P_HD int sort_used(const uint32_t* freq, int nsym, uint16_t* sym)
{
    int n = 0;
    for (int s = 0; s < nsym; s++) {
        if (!freq[s]) continue;
        int j = n++;
        while (j > 0 && freq[sym[j - 1]] > freq[s]) {
            sym[j] = sym[j - 1];
            j--;
        }
        sym[j] = (uint16_t)s;
    }
    return n;
}

// Length per symbol from sorted used symbols (n of them): 0 for unused; a
// lone symbol gets length 1.
R2P_HD void lengths_from_sorted(const uint32_t* freq, const uint16_t* sym, int n, int maxlen, uint8_t* len,
                                uint32_t* w_tmp, uint32_t* l_tmp)
{
    if (n == 1) {
        len[sym[0]] = 1;
        return;
    }
    if (n < 2) return;
    for (int i = 0; i < n; i++) w_tmp[i] = freq[sym[i]];
    limited_lengths(w_tmp, n, maxlen, l_tmp);
    for (int i = 0; i < n; i++) len[sym[i]] = (uint8_t)l_tmp[i];
}

// Canonical codes (RFC 1951 3.2.2), bit-reversed for LSB-first output.
R2P_HD void canonical_codes(const uint8_t* len, int nsym, uint16_t* code)
{
    uint32_t cnt[kMaxCodeLen + 1], next[kMaxCodeLen + 1];
    for (int b = 0; b <= kMaxCodeLen; b++) cnt[b] = 0;
    for (int s = 0; s < nsym; s++) cnt[len[s]]++;
    cnt[0] = 0;
    uint32_t c = 0;
    next[0] = 0;
    for (int b = 1; b <= kMaxCodeLen; b++) {
        c = (c + cnt[b - 1]) << 1;
        next[b] = c;
    }
    for (int s = 0; s < nsym; s++) {
        const int l = len[s];
        code[s] = l ? (uint16_t)bitrev(next[l]++, l) : (uint16_t)0;
    }
}

// Append n <= 25 bits (LSB first) at bit position pos of zeroed words w.
R2P_HD void put_bits(uint32_t* w, uint32_t& pos, uint32_t v, int n)
{
    const uint32_t q = pos >> 5, sh = pos & 31u;
    w[q] |= v << sh;
    if (sh + (uint32_t)n > 32u) w[q + 1] |= v >> (32u - sh);
    pos += (uint32_t)n;
}

// Run-length symbols for one run of `run` equal code lengths l (RFC 1951
// 3.2.7): zeros as 18 (11-138) and 17 (3-10), other lengths once and then 16
// (repeat 3-6); what is left over is written out.  rle_run_count gives the
// number of symbols, rle_run_write writes them (symbol, extra value).
R2P_HD int rle_run_count(int l, int run)
{
    int r = run, k = 0;
    if (l == 0) {
        for (; r >= 11; k++) r -= r < 138 ? r : 138;
        if (r >= 3) {
            k++;
            r = 0;
        }
    } else {
        k = 1;
        for (r--; r >= 3; k++) r -= r < 6 ? r : 6;
    }
    return k + r;
}

R2P_HD void rle_run_write(int l, int run, uint8_t* rs, uint8_t* rx)
{
    int r = run, k = 0;
    if (l == 0) {
        while (r >= 11) {
            const int t = r < 138 ? r : 138;
            rs[k] = 18;
            rx[k++] = (uint8_t)(t - 11);
            r -= t;
        }
        if (r >= 3) {
            rs[k] = 17;
            rx[k++] = (uint8_t)(r - 3);
            r = 0;
        }
    } else {
        rs[k] = (uint8_t)l;
        rx[k++] = 0;
        r--;
        while (r >= 3) {
            const int t = r < 6 ? r : 6;
            rs[k] = 16;
            rx[k++] = (uint8_t)(t - 3);
            r -= t;
        }
    }
    while (r > 0) {
        rs[k] = (uint8_t)l;
        rx[k++] = 0;
        r--;
    }
}

// Extra bits after a code-length symbol.
R2P_HD int cl_extra_bits(int sym) { return sym == 16 ? 2 : sym == 17 ? 3 : sym == 18 ? 7 : 0; }

// The code-length code (lengths <= 7; a lone symbol is completed by an unused
// one, as inflate wants a complete code here) and HCLEN's count: the
// permuted positions up to the last used, at least 4.
R2P_HD int cl_code_build(const uint32_t* cf, uint8_t* cl_len, uint16_t* cl_code)
{
    uint16_t sym[kCLSyms];
    uint32_t wt[kCLSyms], lt[kCLSyms];
    for (int s = 0; s < kCLSyms; s++) cl_len[s] = 0;
    const int nu = sort_used(cf, kCLSyms, sym);
    lengths_from_sorted(cf, sym, nu, kMaxCLLen, cl_len, wt, lt);
    if (nu == 1) cl_len[sym[0] == 0 ? 1 : 0] = 1;
    canonical_codes(cl_len, kCLSyms, cl_code);
    const uint8_t ord[kCLSyms] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    int ncl = kCLSyms;
    while (ncl > 4 && cl_len[ord[ncl - 1]] == 0) ncl--;
    return ncl;
}

// HLIT, HDIST, HCLEN and the HCLEN code-length-code lengths, from bit pos.
R2P_HD void put_header_counts(uint32_t* hw, uint32_t& pos, int nll, int nd, int ncl, const uint8_t* cl_len)
{
    const uint8_t ord[kCLSyms] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    put_bits(hw, pos, (uint32_t)(nll - 257), 5);
    put_bits(hw, pos, (uint32_t)(nd - 1), 5);
    put_bits(hw, pos, (uint32_t)(ncl - 4), 4);
    for (int k = 0; k < ncl; k++) put_bits(hw, pos, cl_len[ord[k]], 3);
}

// Dynamic block header after the 3 block-type bits: HLIT, HDIST, HCLEN, the
// code-length code's lengths (in the RFC's permuted order), then both
// alphabets' code lengths as one run-length coded sequence (16: repeat the
// previous length 3-6 times, 17: 3-10 zeros, 18: 11-138 zeros).  ll_len has
// kLLSyms entries (ll_len[256] > 0), d_len kDSyms.  hw: kHdrWords zeroed
// words, written from bit pos0 (< 32) on; returns the end bit position.
R2P_HD uint32_t build_dyn_header(const uint8_t* ll_len, const uint8_t* d_len, uint32_t* hw, uint32_t pos0 = 0)
{
    int nll = kLLSyms;
    while (nll > 257 && ll_len[nll - 1] == 0) nll--;
    int nd = kDSyms;
    while (nd > 1 && d_len[nd - 1] == 0) nd--;
    const int n = nll + nd;
    uint8_t rs[kLLSyms + kDSyms], rx[kLLSyms + kDSyms];
    int nr = 0;
    for (int i = 0; i < n;) {
        const uint8_t l = i < nll ? ll_len[i] : d_len[i - nll];
        int run = 1;
        while (i + run < n && (i + run < nll ? ll_len[i + run] : d_len[i + run - nll]) == l) run++;
        rle_run_write(l, run, rs + nr, rx + nr);
        nr += rle_run_count(l, run);
        i += run;
    }
    uint32_t cf[kCLSyms];
    for (int s = 0; s < kCLSyms; s++) cf[s] = 0;
    for (int j = 0; j < nr; j++) cf[rs[j]]++;
    uint8_t cl_len[kCLSyms];
    uint16_t cl_code[kCLSyms];
    const int ncl = cl_code_build(cf, cl_len, cl_code);
    uint32_t pos = pos0;
    put_header_counts(hw, pos, nll, nd, ncl, cl_len);
    for (int j = 0; j < nr; j++) {
        const int s = rs[j];
        put_bits(hw, pos, cl_code[s], cl_len[s]);
        const int ne = cl_extra_bits(s);
        if (ne) put_bits(hw, pos, rx[j], ne);
    }
    return pos;
}

// Length symbol (257..285) and extra bits of a match length 3..258.
R2P_HD void length_symbol(int len, int& sym, int& nextra, int& extra)
{
    const int l = len - 3;
    if (len == 258) { sym = 285; nextra = 0; extra = 0; return; }
    if (l < 8) { sym = 257 + l; nextra = 0; extra = 0; return; }
    int lg = 0;
    while ((l >> (lg + 1)) != 0) lg++;
    nextra = lg - 2;
    sym = 257 + 4 * nextra + 4 + ((l >> nextra) & 3);
    extra = l & ((1 << nextra) - 1);
}

}  // namespace r2p
