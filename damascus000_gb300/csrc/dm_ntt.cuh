// Register-resident negacyclic NTT building blocks (host and device).
//
// A "row" is one polynomial of 2^L coefficients under one CRT prime.  T = 2^(L-4)
// threads cooperate on a row and each holds 16 elements in registers.  The L
// Cooley-Tukey stages run in passes of up to four stages; within a pass every
// butterfly pairs two registers of the same thread, and rows are re-distributed
// through shared memory between passes.
//
// In pass p the thread's 16 elements are the index bits [lo, lo + 4) with
// lo = max(0, L - 4 - 4p); the remaining L - 4 bits come from the thread index t.
// The last pass therefore leaves each thread holding 16 consecutive slots, which
// the multiply-accumulate consumes directly (slot pairs 2i, 2i+1 are the
// evaluations at +w_i, -w_i).
#pragma once

#include "dm_field.cuh"

namespace dm {

constexpr int kNttE = 16;  // elements per thread
constexpr int kNttLogE = 4;

// Montgomery product with a constant whose product with p^-1 is precomputed:
// v * w * 2^-32 mod p for v < 2^32, w < p, wp = w * p^-1 mod 2^32 (three multiplies).
DM_HD uint32_t mont_tw(uint32_t v, uint32_t w, uint32_t wp, uint32_t p) {
#if defined(__CUDA_ARCH__)
    const uint32_t th = __umulhi(v, w);
    const uint32_t m = v * wp;
    const uint32_t mh = __umulhi(m, p);
#else
    const uint32_t th = (uint32_t)(((uint64_t)v * w) >> 32);
    const uint32_t m = v * wp;
    const uint32_t mh = (uint32_t)(((uint64_t)m * p) >> 32);
#endif
    const uint32_t r = th - mh;
    return th < mh ? r + p : r;
}

// ---- redundant representation for the forward transform ----
// Values live in [0, 2^32) and are congruent mod p (not reduced).  A sum u + t
// with t < p needs a correction only when the 32-bit add carries (subtract p),
// a difference only when it borrows (add p).  The carry / borrow is the high
// word of the 64-bit sum / difference (0 or 1, 0 or 2^32 - 1) and the
// correction is one multiply-add.

// u + t (mod p), u < 2^32, t < p  ->  [0, 2^32)
DM_HD uint32_t add_lazy(uint32_t u, uint32_t t, uint32_t p) {
    const uint64_t s = (uint64_t)u + t;
    return (uint32_t)s - (uint32_t)(s >> 32) * p;
}
// u - t (mod p), u < 2^32, t < p  ->  [0, 2^32)
DM_HD uint32_t sub_lazy(uint32_t u, uint32_t t, uint32_t p) {
    const uint64_t d = (uint64_t)u - t;
    return (uint32_t)d - (uint32_t)(d >> 32) * p;
}
// v * w * 2^-32 mod p in [0, p) for any v < 2^32 (w < p, wp = w * p^-1 mod 2^32).
// The correction stays a compare-and-select: a borrow-flag form of it measured
// wrong on sm_103a whenever v * wp = 0 (mod 2^32).
DM_HD uint32_t mont_tw_c(uint32_t v, uint32_t w, uint32_t wp, uint32_t p) { return mont_tw(v, w, wp, p); }

// Residue of a Z_q element modulo prime i with three-multiply Montgomery terms.
DM_HD uint32_t residue_fast(const fq& x, const PrimeConsts& c, int i) {
    const uint32_t p = c.p[i];
    uint32_t r = mont_tw(x.w[0], c.r1[i], c.r1p[i], p);
    r = add_mod(r, mont_tw(x.w[1], c.k32[i], c.k32p[i], p), p);
    r = add_mod(r, mont_tw(x.w[2], c.k64[i], c.k64p[i], p), p);
    r = add_mod(r, mont_tw(x.w[3], c.k96[i], c.k96p[i], p), p);
    return r;
}

DM_HD int ntt_pass_count(int L) { return L <= kNttLogE ? 1 : (L + kNttLogE - 1) / kNttLogE; }
DM_HD int ntt_pass_lo(int L, int pass) {
    const int lo = L - kNttLogE - kNttLogE * pass;
    return lo > 0 ? lo : 0;
}
// Element index of register r of thread t in pass `pass` (L >= 4).
DM_HD uint32_t ntt_place(int L, int pass, uint32_t t, uint32_t r) {
    const int lo = ntt_pass_lo(L, pass);
    return ((t >> lo) << (lo + kNttLogE)) | (r << lo) | (t & ((1u << lo) - 1u));
}
// Shared-memory word of element j: XOR bits 2..4 with bits 5..7 (keeps 4-word
// groups intact for 128-bit accesses, spreads 32-word strides over banks).
DM_HD uint32_t ntt_swz(uint32_t j) { return j ^ (((j >> 5) & 7u) << 2); }

// Residue in the redundant range [0, 2^32) (the forward transform's input).
DM_HD uint32_t residue_lazy(const fq& x, const PrimeConsts& c, int i) {
    const uint32_t p = c.p[i];
    uint32_t r = mont_tw_c(x.w[0], c.r1[i], c.r1p[i], p);
    r = add_lazy(r, mont_tw_c(x.w[1], c.k32[i], c.k32p[i], p), p);
    r = add_lazy(r, mont_tw_c(x.w[2], c.k64[i], c.k64p[i], p), p);
    r = add_lazy(r, mont_tw_c(x.w[3], c.k96[i], c.k96p[i], p), p);
    return r;
}
// [0, 2^32) -> [0, p): x * R * R^-1.
DM_HD uint32_t normalize_lazy(uint32_t x, const PrimeConsts& c, int i) {
    return mont_tw_c(x, c.r1[i], c.r1p[i], c.p[i]);
}

// Forward stages with the redundant representation (inputs and outputs in [0, 2^32)).
DM_HD void ntt_fwd_pass_lazy(uint32_t a[kNttE], int L, int pass, uint32_t t, const uint32_t* zeta,
                             const uint32_t* zetap, uint32_t p) {
    const int lo = ntt_pass_lo(L, pass);
    const int st_end = (4 * pass + 4 < L) ? 4 * pass + 4 : L;
    DM_UNROLL
    for (int st = 4 * pass; st < st_end; ++st) {
        const int bb = L - 1 - st;
        const int rb = bb - lo;
        DM_UNROLL
        for (int r = 0; r < kNttE; ++r) {
            if (r & (1 << rb)) continue;
            const uint32_t j = ntt_place(L, pass, t, (uint32_t)r);
            const uint32_t k = (1u << st) + (j >> (bb + 1));
            const uint32_t v = mont_tw_c(a[r | (1 << rb)], zeta[k], zetap[k], p);
            const uint32_t u = a[r];
            a[r] = add_lazy(u, v, p);
            a[r | (1 << rb)] = sub_lazy(u, v, p);
        }
    }
}

// Forward stages [4*pass, min(4*pass+4, L)) on the 16 registers of thread t.
// zeta / zetap: this prime's bit-reversed twiddles (Montgomery form) and their
// products with p^-1.
DM_HD void ntt_fwd_pass(uint32_t a[kNttE], int L, int pass, uint32_t t, const uint32_t* zeta, const uint32_t* zetap,
                        uint32_t p) {
    const int lo = ntt_pass_lo(L, pass);
    const int st_end = (4 * pass + 4 < L) ? 4 * pass + 4 : L;
    DM_UNROLL
    for (int st = 4 * pass; st < st_end; ++st) {
        const int bb = L - 1 - st;  // bit of the butterfly distance
        const int rb = bb - lo;     // same bit within r
        DM_UNROLL
        for (int r = 0; r < kNttE; ++r) {
            if (r & (1 << rb)) continue;
            const uint32_t j = ntt_place(L, pass, t, (uint32_t)r);
            const uint32_t k = (1u << st) + (j >> (bb + 1));
            const uint32_t v = mont_tw(a[r | (1 << rb)], zeta[k], zetap[k], p);
            const uint32_t u = a[r];
            a[r] = add_mod(u, v, p);
            a[r | (1 << rb)] = sub_mod(u, v, p);
        }
    }
}

// Inverse (Gentleman-Sande) stages of the same pass, run in the reverse order:
// passes go from last to first and stages within a pass from the deepest up.
DM_HD void ntt_inv_pass(uint32_t a[kNttE], int L, int pass, uint32_t t, const uint32_t* zinv, const uint32_t* zinvp,
                        uint32_t p) {
    const int lo = ntt_pass_lo(L, pass);
    const int st_end = (4 * pass + 4 < L) ? 4 * pass + 4 : L;
    DM_UNROLL
    for (int st = st_end - 1; st >= 4 * pass; --st) {
        const int bb = L - 1 - st;
        const int rb = bb - lo;
        DM_UNROLL
        for (int r = 0; r < kNttE; ++r) {
            if (r & (1 << rb)) continue;
            const uint32_t j = ntt_place(L, pass, t, (uint32_t)r);
            const uint32_t k = (1u << st) + (j >> (bb + 1));
            const uint32_t u = a[r], v = a[r | (1 << rb)];
            a[r] = add_mod(u, v, p);
            a[r | (1 << rb)] = mont_tw(sub_mod(u, v, p), zinv[k], zinvp[k], p);
        }
    }
}

}  // namespace dm
