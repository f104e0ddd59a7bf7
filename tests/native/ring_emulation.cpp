// Host emulation of the nine-prime ring pipeline exactly as the transform
// kernels run it: the same device functions (dm_ntt.cuh, dm_field.cuh compiled
// for the CPU), the register passes of 16 residues per thread (and of 32, the
// forward transform's radix-32 alternative, checked against them), the swizzled
// shared-memory exchanges, the last-pass twiddle order, the lazy value bounds,
// the MAC, the even/odd cross terms, the inverse and the Garner CRT.  Results
// are compared with schoolbook negacyclic products in Z_q for every ring size
// 2^0 .. 2^12, with all-(q-1) worst-case operands.  Also checks that every
// exchange is a bijection onto its row and free of shared-memory bank
// conflicts for the kernels' block shapes.  Exit status 0 = all checks pass.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "dm_ntt.cuh"
#include "dm_tables.h"

using namespace dm;

namespace {

std::mt19937_64 rng(20261203);
int fails = 0;

void fail(const char* what, int L) {
    std::printf("FAIL %s (L=%d)\n", what, L);
    ++fails;
}

fq random_word() {
    fq x;
    for (int i = 0; i < 4; ++i) x.w[i] = (uint32_t)rng();
    return x;
}
fq random_fq() {
    fq x = random_word();
    x.w[3] &= 0xFFFFu;
    return fq_canon(x);
}
fq q_minus_one() { return fq{{0xFFFFFFB4u, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFu}}; }

std::vector<fq> schoolbook(const std::vector<fq>& a, const std::vector<fq>& b) {
    const size_t n = a.size();
    std::vector<fq> c(n, fq_zero());
    for (size_t i = 0; i < n; ++i)
        for (size_t j = 0; j < n; ++j) {
            const fq t = fq_mul(a[i], b[j]);
            if (i + j < n)
                c[i + j] = fq_add(c[i + j], t);
            else
                c[i + j - n] = fq_sub(c[i + j - n], t);
        }
    return c;
}

const Tw* last_table(const std::vector<Tw>& t, int pi, int L) {
    return t.data() + (size_t)pi * kLastSpan + (1u << L) - 16u;
}

// Forward transform of one row (prime pi), slot order out, values in [0, p).
std::vector<uint32_t> forward_row(const std::vector<fq>& x, int L, int pi) {
    const HostTables& T = host_tables();
    const uint32_t p = T.pc.p[pi];
    const Tw* tw = T.fwd.data() + (size_t)pi * kMaxRing;
    const uint32_t s = 1u << L;
    std::vector<uint32_t> out(s);
    if (L < 4) {
        std::vector<uint32_t> a(s);
        for (uint32_t c = 0; c < s; ++c) a[c] = residue_fwd(x[c], T.pc, pi);
        switch (L) {
            case 0: ntt_fwd_small<0>(a.data(), tw, p); break;
            case 1: ntt_fwd_small<1>(a.data(), tw, p); break;
            case 2: ntt_fwd_small<2>(a.data(), tw, p); break;
            default: ntt_fwd_small<3>(a.data(), tw, p); break;
        }
        for (uint32_t c = 0; c < s; ++c) out[c] = ntt_fwd_final(a[c], T.pc.one_s[pi], p);
        return out;
    }
    const uint32_t nt = s / kNttE;
    const int np = ntt_pass_count(L);
    std::vector<std::vector<uint32_t>> R(nt, std::vector<uint32_t>(kNttE));
    std::vector<uint32_t> sm(2u * s, 0xFFFFFFFFu);
    const uint32_t base = 1u << L;  // the second row of a block
    for (uint32_t t = 0; t < nt; ++t)
        for (int r = 0; r < kNttE; ++r) R[t][r] = residue_fwd(x[ntt_place(L, 0, t, r)], T.pc, pi);
    for (int pass = 0; pass < np; ++pass) {
        for (uint32_t t = 0; t < nt; ++t) ntt_fwd_pass(R[t].data(), L, pass, t, tw, last_table(T.fwd_last, pi, L), p);
        for (uint32_t t = 0; t < nt; ++t)
            for (int r = 0; r < kNttE; ++r)
                if ((uint64_t)R[t][r] >= 16ull * p) fail("forward pass output bound 16p", L);
        if (pass + 1 < np) {
            for (uint32_t t = 0; t < nt; ++t)
                for (int r = 0; r < kNttE; ++r) {
                    const uint32_t w = ntt_swz_base(base, L, pass, t) ^ ntt_swz_reg(L, pass, r);
                    if (w != ntt_swz(base + ntt_place(L, pass, t, r)) || (w >> L) != 1) fail("exchange word", L);
                    sm[w] = R[t][r];
                }
            for (uint32_t t = 0; t < nt; ++t)
                for (int r = 0; r < kNttE; ++r) R[t][r] = sm[ntt_swz_base(base, L, pass + 1, t) ^ ntt_swz_reg(L, pass + 1, r)];
        }
    }
    for (uint32_t t = 0; t < nt; ++t)
        for (int r = 0; r < kNttE; ++r) out[t * kNttE + r] = ntt_fwd_final(R[t][r], T.pc.one_s[pi], p);
    return out;
}

// The same transform in the radix-2^LE pass shape of the forward kernel's
// alternative (LE = 5: 32 residues per thread, 2^(L-5) threads per row, the
// natural twiddle table in every pass), for L >= LE.
template <int LE>
std::vector<uint32_t> forward_row_e(const std::vector<fq>& x, int L, int pi) {
    constexpr int E = 1 << LE;
    const HostTables& T = host_tables();
    const uint32_t p = T.pc.p[pi];
    const Tw* tw = T.fwd.data() + (size_t)pi * kMaxRing;
    const uint32_t s = 1u << L;
    const uint32_t nt = s / E;
    const int np = ntt_pass_count_e<LE>(L);
    std::vector<std::vector<uint32_t>> R(nt, std::vector<uint32_t>(E));
    std::vector<uint32_t> sm(2u * s, 0xFFFFFFFFu);
    const uint32_t base = 1u << L;
    for (uint32_t t = 0; t < nt; ++t)
        for (int r = 0; r < E; ++r) R[t][r] = residue_fwd(x[ntt_place_e<LE>(L, 0, t, r)], T.pc, pi);
    for (int pass = 0; pass < np; ++pass) {
        for (uint32_t t = 0; t < nt; ++t) ntt_fwd_pass_e<LE>(R[t].data(), L, pass, t, tw, p);
        for (uint32_t t = 0; t < nt; ++t)
            for (int r = 0; r < E; ++r)
                if ((uint64_t)R[t][r] >= 16ull * p) fail("radix-32 pass output bound 16p", L);
        if (pass + 1 < np) {
            for (uint32_t t = 0; t < nt; ++t)
                for (int r = 0; r < E; ++r) {
                    const uint32_t w = ntt_swz_base_e<LE>(base, L, pass, t) ^ ntt_swz_reg_e<LE>(L, pass, r);
                    if (w != ntt_swz_e<LE>(base + ntt_place_e<LE>(L, pass, t, r)) || (w >> L) != 1)
                        fail("radix-32 exchange word", L);
                    sm[w] = R[t][r];
                }
            for (uint32_t t = 0; t < nt; ++t)
                for (int r = 0; r < E; ++r)
                    R[t][r] = sm[ntt_swz_base_e<LE>(base, L, pass + 1, t) ^ ntt_swz_reg_e<LE>(L, pass + 1, r)];
        }
    }
    std::vector<uint32_t> out(s);
    for (uint32_t t = 0; t < nt; ++t)
        for (int r = 0; r < E; ++r) out[t * E + r] = ntt_fwd_final(R[t][r], T.pc.one_s[pi], p);
    return out;
}

// Inverse of one row of reduced slots; mode 0 plain, 1 / 2 the even/odd cross
// terms (twist by w_i or w_i^-1 and the extra 1/4), as the finish kernels do.
std::vector<uint32_t> inverse_row(std::vector<uint32_t> in, int L, int pi, int mode) {
    const HostTables& T = host_tables();
    const uint32_t p = T.pc.p[pi];
    const Tw* tw = T.fwd.data() + (size_t)pi * kMaxRing;
    const Tw* ti = T.inv.data() + (size_t)pi * kMaxRing;
    const uint32_t s = 1u << L;
    for (uint32_t i = 0; i < s; ++i) {
        if (mode == 1) in[i] = shoup_mul(in[i], tw[s + i], p);
        if (mode == 2) in[i] = shoup_mul(in[i], ti[s + i], p);
    }
    const uint32_t f = mode == 0 ? T.ninv[pi][L] : T.ninv4[pi][L];
    const uint32_t fs = mode == 0 ? T.ninvs[pi][L] : T.ninv4s[pi][L];
    std::vector<uint32_t> out(s);
    if (L < 4) {
        switch (L) {
            case 0: ntt_inv_small<0>(in.data(), ti, p); break;
            case 1: ntt_inv_small<1>(in.data(), ti, p); break;
            case 2: ntt_inv_small<2>(in.data(), ti, p); break;
            default: ntt_inv_small<3>(in.data(), ti, p); break;
        }
        for (uint32_t c = 0; c < s; ++c) out[c] = red_below(shoup_mul(in[c], f, fs, p), p);
        return out;
    }
    const uint32_t nt = s / kNttE;
    std::vector<std::vector<uint32_t>> R(nt, std::vector<uint32_t>(kNttE));
    std::vector<uint32_t> sm(s);
    for (uint32_t t = 0; t < nt; ++t)
        for (int r = 0; r < kNttE; ++r) R[t][r] = in[t * kNttE + r];
    for (int pass = ntt_pass_count(L) - 1; pass >= 0; --pass) {
        for (uint32_t t = 0; t < nt; ++t) ntt_inv_pass(R[t].data(), L, pass, t, ti, last_table(T.inv_last, pi, L), p);
        if (pass > 0) {
            for (uint32_t t = 0; t < nt; ++t)
                for (int r = 0; r < kNttE; ++r) sm[ntt_swz_base(0, L, pass, t) ^ ntt_swz_reg(L, pass, r)] = R[t][r];
            for (uint32_t t = 0; t < nt; ++t)
                for (int r = 0; r < kNttE; ++r) R[t][r] = sm[ntt_swz_base(0, L, pass - 1, t) ^ ntt_swz_reg(L, pass - 1, r)];
        }
    }
    for (uint32_t t = 0; t < nt; ++t)
        for (int r = 0; r < kNttE; ++r) out[ntt_place(L, 0, t, r)] = red_below(shoup_mul(R[t][r], f, fs, p), p);
    return out;
}

std::vector<fq> crt(const std::vector<std::vector<uint32_t>>& rows, uint32_t s) {
    const HostTables& T = host_tables();
    std::vector<fq> o(s);
    for (uint32_t c = 0; c < s; ++c) {
        uint32_t r[kPrimes];
        for (int i = 0; i < kPrimes; ++i) r[i] = rows[i][c];
        o[c] = crt_to_fq(r, T.pc, T.cc);
    }
    return o;
}

// Bank check of every exchange for a block of `rows` rows of 2^(L-LE) threads:
// for each warp and register, the 32 words stored (and loaded) sit in 32
// different banks.
template <int LE = kNttLogE>
void check_banks(int L, int rows) {
    const uint32_t T = 1u << (L - LE), threads = T * rows;
    for (int pass = 0; pass + 1 < ntt_pass_count_e<LE>(L); ++pass)
        for (int dir = 0; dir < 2; ++dir)
            for (uint32_t w0 = 0; w0 < threads; w0 += 32)
                for (int r = 0; r < (1 << LE); ++r) {
                    uint32_t used = 0;
                    for (uint32_t lane = 0; lane < 32 && w0 + lane < threads; ++lane) {
                        const uint32_t th = w0 + lane, row = th / T, t = th % T;
                        const int ps = pass + dir;
                        const uint32_t word = ntt_swz_base_e<LE>(row << L, L, ps, t) ^ ntt_swz_reg_e<LE>(L, ps, r);
                        used |= 1u << (word % 32);
                    }
                    const uint32_t lanes = threads - w0 < 32 ? threads - w0 : 32;
                    if (__builtin_popcount(used) != (int)lanes) {
                        fail("shared-memory bank conflict", L);
                        return;
                    }
                }
}

}  // namespace

int main(int argc, char** argv) {
    const int max_L = argc > 1 ? std::atoi(argv[1]) : kLogMaxProverRing;
    const HostTables& T = host_tables();
    for (int pi = 0; pi < kPrimes; ++pi) {  // forward residues: congruent, below 8p, extremes included
        const uint32_t p = T.pc.p[pi];
        if (p >= (1u << 28)) fail("prime below 2^28", -1);
        for (int it = 0; it < 50000; ++it) {
            fq x = random_word();
            if (it < 16)
                for (int w = 0; w < 4; ++w) x.w[w] = (it >> w) & 1 ? 0xFFFFFFFFu : 0u;
            const uint32_t r = residue_fwd(x, T.pc, pi);
            const unsigned __int128 v = ((unsigned __int128)x.w[3] << 96) | ((unsigned __int128)x.w[2] << 64) |
                                        ((unsigned __int128)x.w[1] << 32) | x.w[0];
            if (r >= 8ull * p || r % p != (uint32_t)(v % p)) {
                fail("forward residue", -1);
                break;
            }
        }
    }
    for (int L = 5; L <= max_L; ++L)  // blocks of 64 and of 32 threads for small rings (the tuning knob)
        for (int group : {64, 32}) {
            const int rows = (1 << (L - 4)) >= group ? 1 : group >> (L - 4);
            check_banks(L, rows);
            const int rows5 = (1 << (L - 5)) >= group ? 1 : group >> (L - 5);
            check_banks<5>(L, rows5);
        }
    for (int L = 0; L <= max_L; ++L) {
        const uint32_t s = 1u << L;
        // a commitment coordinate: sum of `cols` products, the first of all-(q-1) operands
        const int cols = L <= 8 ? 4 : 2;
        std::vector<fq> want(s, fq_zero());
        std::vector<std::vector<uint32_t>> acc(kPrimes, std::vector<uint32_t>(s, 0));
        for (int col = 0; col < cols; ++col) {
            std::vector<fq> a(s), b(s);
            for (uint32_t i = 0; i < s; ++i) {
                a[i] = col == 0 ? q_minus_one() : random_fq();
                b[i] = col == 0 ? q_minus_one() : random_fq();
            }
            const std::vector<fq> c = schoolbook(a, b);
            for (uint32_t i = 0; i < s; ++i) want[i] = fq_add(want[i], c[i]);
            for (int pi = 0; pi < kPrimes; ++pi) {
                const std::vector<uint32_t> A = forward_row(a, L, pi), B = forward_row(b, L, pi);
                if (L >= 5 && (forward_row_e<5>(a, L, pi) != A || forward_row_e<5>(b, L, pi) != B))
                    fail("radix-32 passes differ from radix-16", L);
                for (uint32_t i = 0; i < s; ++i)
                    acc[pi][i] = red64((uint64_t)acc[pi][i] + (uint64_t)A[i] * B[i], T.pc, pi);
            }
        }
        std::vector<std::vector<uint32_t>> rows(kPrimes);
        for (int pi = 0; pi < kPrimes; ++pi) rows[pi] = inverse_row(acc[pi], L, pi, 0);
        const std::vector<fq> got = crt(rows, s);
        for (uint32_t i = 0; i < s; ++i)
            if (!fq_eq(got[i], want[i])) {
                fail("sum of products", L);
                break;
            }
        if (L == 0) continue;
        // even/odd cross terms from the size-2^L transforms: (X g_o) m_e and g_e m_o at 2^(L-1)
        const uint32_t h = s / 2;
        std::vector<fq> g(s), m(s), ge(h), xgo(h), me(h), mo(h);
        for (uint32_t i = 0; i < s; ++i) {
            g[i] = random_fq();
            m[i] = random_fq();
        }
        for (uint32_t j = 0; j < h; ++j) {
            ge[j] = g[2 * j];
            me[j] = m[2 * j];
            mo[j] = m[2 * j + 1];
            xgo[j] = j == 0 ? fq_neg(g[s - 1]) : g[2 * j - 1];
        }
        const std::vector<fq> wl = schoolbook(xgo, me), wr = schoolbook(ge, mo);
        std::vector<std::vector<uint32_t>> rl(kPrimes), rr(kPrimes);
        for (int pi = 0; pi < kPrimes; ++pi) {
            const uint32_t p = T.pc.p[pi];
            const std::vector<uint32_t> G = forward_row(g, L, pi), M = forward_row(m, L, pi);
            std::vector<uint32_t> al(h), ar(h);
            for (uint32_t i = 0; i < h; ++i) {
                const uint32_t gx = G[2 * i], gy = G[2 * i + 1], mx = M[2 * i], my = M[2 * i + 1];
                al[i] = red64((uint64_t)red_below(gx + p - gy, p) * red_below(mx + my, p), T.pc, pi);
                ar[i] = red64((uint64_t)red_below(gx + gy, p) * red_below(mx + p - my, p), T.pc, pi);
            }
            rl[pi] = inverse_row(al, L - 1, pi, 1);
            rr[pi] = inverse_row(ar, L - 1, pi, 2);
        }
        const std::vector<fq> gl = crt(rl, h), gr = crt(rr, h);
        for (uint32_t i = 0; i < h; ++i)
            if (!fq_eq(gl[i], wl[i]) || !fq_eq(gr[i], wr[i])) {
                fail("even/odd cross terms", L);
                break;
            }
    }
    std::printf("%s (ring sizes up to 2^%d)\n", fails ? "FAILED" : "ok", max_L);
    return fails ? 1 : 0;
}
