// huff_check.cpp -- host check of the dynamic Huffman block builder
// (raw2png-conversionthrugpu_gb300/csrc/r2p_huff.h), driven by
// tests/test_huff.py.
//
//   huff_check lengths < freqs.txt     one line of frequencies per alphabet in,
//                                      the code lengths (max 15) out
//   huff_check rle in.bin out.bin blk  raw DEFLATE of in.bin: dynamic Huffman
//                                      blocks of blk bytes over a run-length
//                                      parse (distance-1 matches of 3..258),
//                                      each non-final block closed by an empty
//                                      stored block, BFINAL on the last
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "../../raw2png-conversionthrugpu_gb300/csrc/r2p_huff.h"

using namespace r2p;

namespace {

struct Token {
    int lit;    // >= 0: literal byte; -1: match
    int len;
};

std::vector<Token> rle_tokens(const uint8_t* p, int n)
{
    std::vector<Token> t;
    int prev = -1;
    for (int i = 0; i < n;) {
        int L = 0;
        if ((int)p[i] == prev) {
            while (L < 258 && i + L < n && p[i + L] == prev) L++;
        }
        if (L >= 3) {
            t.push_back({-1, L});
            i += L;
        } else {
            t.push_back({p[i], 1});
            prev = p[i];
            i++;
        }
    }
    return t;
}

struct Bits {
    std::vector<uint32_t> w;
    uint32_t pos = 0;
    void put(uint32_t v, int n)
    {
        while (w.size() < (pos + n) / 32 + 2) w.push_back(0);
        put_bits(w.data(), pos, v, n);
    }
    void align() { pos = (pos + 7) & ~7u; }
};

void lengths_for(const uint32_t* f, int nsym, int maxlen, uint8_t* len)
{
    std::vector<uint16_t> sym(nsym);
    std::vector<uint32_t> a(nsym), b(nsym);
    for (int s = 0; s < nsym; s++) len[s] = 0;
    const int n = sort_used(f, nsym, sym.data());
    lengths_from_sorted(f, sym.data(), n, maxlen, len, a.data(), b.data());
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc >= 2 && !std::strcmp(argv[1], "lengths")) {
        char buf[1 << 16];
        while (std::fgets(buf, sizeof(buf), stdin)) {
            std::vector<uint32_t> f;
            std::istringstream is(buf);
            unsigned long v;
            while (is >> v) f.push_back((uint32_t)v);
            std::vector<uint8_t> len(f.size());
            lengths_for(f.data(), (int)f.size(), kMaxCodeLen, len.data());
            // the per-level form of phases 2-3 gives the same lengths as the loops
            std::vector<uint16_t> sym(f.size());
            const int nu = sort_used(f.data(), (int)f.size(), sym.data());
            if (nu >= 2) {
                std::vector<uint32_t> a(nu), b(nu), P(nu), D(nu), L(nu);
                for (int i = 0; i < nu; i++) a[i] = P[i] = f[sym[i]];
                mk_lengths_inplace(a.data(), nu);
                mk_phase1(P.data(), nu);
                mk_levels(P.data(), nu, D.data(), L.data());
                for (int i = 0; i < nu; i++)
                    if (L[i] != a[i]) {
                        std::printf("LEVELS-MISMATCH\n");
                        return 1;
                    }
            }
            for (size_t i = 0; i < len.size(); i++) std::printf(i ? " %d" : "%d", len[i]);
            std::printf("\n");
        }
        return 0;
    }
    if (argc == 5 && !std::strcmp(argv[1], "rle")) {
        FILE* f = std::fopen(argv[2], "rb");
        if (!f) return 2;
        std::vector<uint8_t> in;
        uint8_t chunk[65536];
        size_t k;
        while ((k = std::fread(chunk, 1, sizeof(chunk), f)) > 0) in.insert(in.end(), chunk, chunk + k);
        std::fclose(f);
        const int blk = std::atoi(argv[4]);
        Bits out;
        for (size_t b0 = 0; b0 < in.size() || b0 == 0; b0 += blk) {
            const int n = (int)std::min<size_t>(blk, in.size() - b0);
            const bool last = b0 + blk >= in.size();
            std::vector<Token> t = rle_tokens(in.data() + b0, n);
            uint32_t ll[kLLSyms] = {0}, dd[kDSyms] = {0};
            for (const Token& x : t) {
                if (x.lit >= 0) ll[x.lit]++;
                else {
                    int s, ne, ex;
                    length_symbol(x.len, s, ne, ex);
                    ll[s]++;
                    dd[0]++;
                }
            }
            ll[256] = 1;
            uint8_t ll_len[kLLSyms], d_len[kDSyms];
            lengths_for(ll, kLLSyms, kMaxCodeLen, ll_len);
            lengths_for(dd, kDSyms, kMaxCodeLen, d_len);
            uint16_t ll_code[kLLSyms], d_code[kDSyms];
            canonical_codes(ll_len, kLLSyms, ll_code);
            canonical_codes(d_len, kDSyms, d_code);
            uint32_t hw[kHdrWords] = {0};
            const uint32_t hbits = build_dyn_header(ll_len, d_len, hw);
            out.put(last ? 1 : 0, 1);
            out.put(2, 2);                                  // BTYPE = 10
            for (uint32_t i = 0; i < hbits; i += 16) out.put((hw[i >> 5] >> (i & 31)) & 0xFFFF, (int)std::min(16u, hbits - i));
            for (const Token& x : t) {
                if (x.lit >= 0) {
                    out.put(ll_code[x.lit], ll_len[x.lit]);
                } else {
                    int s, ne, ex;
                    length_symbol(x.len, s, ne, ex);
                    out.put(ll_code[s], ll_len[s]);
                    if (ne) out.put((uint32_t)ex, ne);
                    out.put(d_code[0], d_len[0]);
                }
            }
            out.put(ll_code[256], ll_len[256]);
            if (!last) {                                    // empty stored block: byte-aligned boundary
                out.put(0, 3);
                out.align();
                out.put(0, 16);
                out.put(0xFFFF, 16);
            }
            if (in.empty()) break;
        }
        out.align();
        FILE* g = std::fopen(argv[3], "wb");
        if (!g) return 2;
        std::fwrite(out.w.data(), 1, out.pos / 8, g);
        std::fclose(g);
        return 0;
    }
    std::fprintf(stderr, "usage: huff_check lengths | huff_check rle in out block\n");
    return 2;
}
