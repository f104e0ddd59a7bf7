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

// The pass shape is a parameter LE (2^LE residues per thread, LE stages per
// pass): 4 everywhere, and 5 as the forward transform's alternative radix-32
// passes (one exchange fewer at 2^9 and 2^10).  The un-suffixed names are LE = 4.
template <int LE>
DM_HD int ntt_pass_count_e(int L) { return L <= LE ? 1 : (L + LE - 1) / LE; }
template <int LE>
DM_HD int ntt_pass_lo_e(int L, int pass) {
    const int lo = L - LE - LE * pass;
    return lo > 0 ? lo : 0;
}
// Element index of register r of thread t in pass `pass` (L >= LE).  Pass 0
// holds element r * 2^(L-LE) + t (coalesced loads); the last pass 2^LE
// contiguous slots.
template <int LE>
DM_HD uint32_t ntt_place_e(int L, int pass, uint32_t t, uint32_t r) {
    const int lo = ntt_pass_lo_e<LE>(L, pass);
    return ((t >> lo) << (lo + LE)) | (r << lo) | (t & ((1u << lo) - 1u));
}
DM_HD int ntt_pass_count(int L) { return ntt_pass_count_e<kNttLogE>(L); }
DM_HD int ntt_pass_lo(int L, int pass) { return ntt_pass_lo_e<kNttLogE>(L, pass); }
DM_HD uint32_t ntt_place(int L, int pass, uint32_t t, uint32_t r) { return ntt_place_e<kNttLogE>(L, pass, t, r); }
// Shared-memory word of block-wide element index i: bits 0..4 XOR bits 4..8.  A
// bijection that makes every pass's scalar stores and loads bank-conflict free
// for the block shapes of the transform kernels (rows of 2^L words, 2^(L-4)
// threads per row).
DM_HD uint32_t ntt_swz(uint32_t i) { return i ^ ((i >> 4) & 31u); }
// The same for radix-2^LE passes: bits 0..4 XOR bits LE..LE+4 (for LE = 4 the
// function above; LE = 5 moves the folded field above the register field of
// the last pass, where bits 0..4 are the register index).
template <int LE>
DM_HD uint32_t ntt_swz_e(uint32_t i) { return i ^ ((i >> LE) & 31u); }

// ---- lazy Harvey butterflies (p < 2^28) ----
//
// A forward butterfly with u < B and v = Shoup(x) < 2p gives u + v < B + 2p
// and u - v + 2p < B + 2p, so values grow by 2p per stage.  Every pass starts
// below 8p (the first from the lazy residues, later ones after one conditional
// subtraction of 8p per register), so four stages stay below 16p < 2^32 for
// p < 2^28: no reduction inside a pass, 5 instructions per butterfly (3 of them
// multiplies), and the reduction between passes is an add and a min on the
// integer ALU, leaving the multiplier pipe to the butterflies.
//
// Twiddle of the butterfly on register r in stage st of a pass:
// k = 2^st + (j >> (bb + 1)) with j = place(t, r) and bb = L - 1 - st.  The
// register field sits at bits [lo, lo + 4) of j and bb = lo + rb, so
// k = 2^st + ((t >> lo) << (3 - rb)) + (r >> (rb + 1)): a stage needs only
// 8 >> rb distinct twiddles per thread (15 per four-stage pass, not 32).

// The (2^(LE-1) >> rb) twiddles tw[kb ..] of a stage.  kb is a multiple of their
// count (2^st >= their count whenever L >= LE), so pairs are 16-byte aligned and
// load as one 16-byte word.
template <int LE>
DM_HD void ntt_load_twiddles_e(Tw w[1 << (LE - 1)], const Tw* tw, uint32_t kb, int rb) {
    const int ng = (1 << (LE - 1)) >> rb;
    if (ng == 1) {
        w[0] = tw[kb];
        return;
    }
#if defined(__CUDA_ARCH__)
    const uint4* q = reinterpret_cast<const uint4*>(tw + kb);
    DM_UNROLL
    for (int g = 0; g < ng / 2; ++g) {
        const uint4 v = q[g];
        w[2 * g] = Tw{v.x, v.y};
        w[2 * g + 1] = Tw{v.z, v.w};
    }
#else
    for (int g = 0; g < ng; ++g) w[g] = tw[kb + g];
#endif
}
DM_HD void ntt_load_twiddles(Tw w[8], const Tw* tw, uint32_t kb, int rb) { ntt_load_twiddles_e<kNttLogE>(w, tw, kb, rb); }

// The last pass (lo = 0) gives every thread its own 8 >> rb twiddles per stage,
// so in the natural order a warp's 16-byte loads stride 16 * (ng / 2) bytes and
// touch twice or four times the sectors they use.  The last-pass table of ring
// 2^L stores stage st's entries k = 2^st + th * ng + g at
// 2^st + 2 * ((g >> 1) * 2^st / ng + th) + (g & 1): the pair (g, g + 1) of
// consecutive threads th sits in consecutive 16-byte words.
DM_HD uint32_t ntt_last_pos(int L, int st, uint32_t th, int g) {
    const int ng = 8 >> (L - 1 - st);
    if (ng == 1) return (1u << st) + th;
    return (1u << st) + 2u * ((uint32_t)(g >> 1) * ((1u << st) / (uint32_t)ng) + th) + (uint32_t)(g & 1);
}
DM_HD void ntt_load_twiddles_last(Tw w[8], const Tw* twl, int L, int st, uint32_t th) {
    const int ng = 8 >> (L - 1 - st);
    if (ng == 1) {
        w[0] = twl[(1u << st) + th];
        return;
    }
#if defined(__CUDA_ARCH__)
    const uint4* q = reinterpret_cast<const uint4*>(twl + (1u << st));
    const uint32_t m = (1u << st) / (uint32_t)ng;
    DM_UNROLL
    for (int g = 0; g < ng / 2; ++g) {
        const uint4 v = q[g * m + th];
        w[2 * g] = Tw{v.x, v.y};
        w[2 * g + 1] = Tw{v.z, v.w};
    }
#else
    for (int g = 0; g < ng; ++g) w[g] = twl[ntt_last_pos(L, st, th, g)];
#endif
}

// x mod p in [0, 2p) for any x < 2^32: Shoup product by 1 (one_s = floor(2^32 / p)).
DM_HD uint32_t shoup_one(uint32_t x, uint32_t one_s, uint32_t p) { return x - mulhi32(x, one_s) * p; }

// Forward stages [LE*pass, min(LE*pass+LE, L)) on the 2^LE registers of thread t
// (radix-2^LE pass shape; see ntt_fwd_pass for LE = 4).  Values start every pass
// below 8p and grow by 2p per stage; a pass of five stages brings them below 8p
// again before its fifth (16p + 2p would not fit 32 bits for p near 2^28), so
// outputs stay below 16p.  twl, the last-pass twiddle order, exists for LE = 4
// only: other shapes read the natural table in every pass (twl unused).
template <int LE>
DM_HD void ntt_fwd_pass_e(uint32_t a[1 << LE], int L, int pass, uint32_t t, const Tw* tw, uint32_t p) {
    constexpr int E = 1 << LE;
    const int lo = ntt_pass_lo_e<LE>(L, pass);
    const int st0 = LE * pass;
    const int st_end = (st0 + LE < L) ? st0 + LE : L;
    const uint32_t p2 = 2 * p, p8 = 8 * p;
    const uint32_t th = t >> lo;
    if (pass > 0) {
        DM_UNROLL
        for (int r = 0; r < E; ++r) a[r] = red_below(a[r], p8);  // [0, 8p)
    }
    DM_UNROLL
    for (int st = st0; st < st_end; ++st) {
        if (st - st0 == 4) {
            DM_UNROLL
            for (int r = 0; r < E; ++r) a[r] = red_below(a[r], p8);  // from [0, 16p) to [0, 8p)
        }
        const int rb = L - 1 - st - lo;  // bit of the butterfly distance within r
        Tw w[E / 2];
        ntt_load_twiddles_e<LE>(w, tw, (1u << st) + (th << (LE - 1 - rb)), rb);
        DM_UNROLL
        for (int r = 0; r < E; ++r) {
            if (r & (1 << rb)) continue;
            const uint32_t u = a[r];
            const uint32_t v = shoup_mul(a[r | (1 << rb)], w[r >> (rb + 1)], p);  // [0, 2p)
            a[r] = u + v;
            a[r | (1 << rb)] = u - v + p2;
        }
    }
}

// Forward (Cooley-Tukey) stages [4*pass, min(4*pass+4, L)) on the 16 registers
// of thread t; inputs below 8p (first pass) or below 16p (later passes, which
// subtract 8p first), outputs below 16p.  tw: this prime's bit-reversed twiddles
// psi^brv(k) with Shoup constants; twl: the same in the last-pass order of ring
// 2^L (used by the pass with lo = 0).
DM_HD void ntt_fwd_pass(uint32_t a[kNttE], int L, int pass, uint32_t t, const Tw* tw, const Tw* twl, uint32_t p) {
    const int lo = ntt_pass_lo(L, pass);
    const int st_end = (4 * pass + 4 < L) ? 4 * pass + 4 : L;
    const uint32_t p2 = 2 * p;
    const uint32_t th = t >> lo;
    if (pass > 0) {
        const uint32_t p8 = 8 * p;
        DM_UNROLL
        for (int r = 0; r < kNttE; ++r) a[r] = red_below(a[r], p8);  // [0, 8p)
    }
    DM_UNROLL
    for (int st = 4 * pass; st < st_end; ++st) {
        const int rb = L - 1 - st - lo;  // bit of the butterfly distance within r
        Tw w[8];
        if (lo == 0)
            ntt_load_twiddles_last(w, twl, L, st, th);
        else
            ntt_load_twiddles(w, tw, (1u << st) + (th << (3 - rb)), rb);
        DM_UNROLL
        for (int r = 0; r < kNttE; ++r) {
            if (r & (1 << rb)) continue;
            const uint32_t u = a[r];
            const uint32_t v = shoup_mul(a[r | (1 << rb)], w[r >> (rb + 1)], p);  // [0, 2p)
            a[r] = u + v;
            a[r | (1 << rb)] = u - v + p2;
        }
    }
}
// Forward output (any 32-bit value, in practice below 16p) to [0, p).
DM_HD uint32_t ntt_fwd_final(uint32_t x, uint32_t one_s, uint32_t p) { return red_below(shoup_one(x, one_s, p), p); }

// Inverse (Gentleman-Sande) stages of the same pass in reverse order (passes
// from last to first, stages within a pass from the deepest up); inputs and
// outputs in [0, 2p) (a sum doubles the bound, so it is reduced every stage).
// tw / twl: the inverse twiddles in natural and last-pass order.
DM_HD void ntt_inv_pass(uint32_t a[kNttE], int L, int pass, uint32_t t, const Tw* tw, const Tw* twl, uint32_t p) {
    const int lo = ntt_pass_lo(L, pass);
    const int st_end = (4 * pass + 4 < L) ? 4 * pass + 4 : L;
    const uint32_t p2 = 2 * p;
    const uint32_t th = t >> lo;
    DM_UNROLL
    for (int st = st_end - 1; st >= 4 * pass; --st) {
        const int rb = L - 1 - st - lo;
        Tw w[8];
        if (lo == 0)
            ntt_load_twiddles_last(w, twl, L, st, th);
        else
            ntt_load_twiddles(w, tw, (1u << st) + (th << (3 - rb)), rb);
        DM_UNROLL
        for (int r = 0; r < kNttE; ++r) {
            if (r & (1 << rb)) continue;
            const uint32_t u = a[r], v = a[r | (1 << rb)];
            a[r] = red_below(u + v, p2);
            a[r | (1 << rb)] = shoup_mul(u - v + p2, w[r >> (rb + 1)], p);
        }
    }
}

// Shared-memory exchange between passes.  The swizzle is linear over GF(2) and
// a row-base | place(t, 0) word has no bits in the register field, so the word
// of register r is swz(base | place(t, 0)) ^ swz(r << lo): one XOR with a
// compile-time constant per access.
template <int LE>
DM_HD uint32_t ntt_swz_base_e(uint32_t base, int L, int pass, uint32_t t) {
    return ntt_swz_e<LE>(base | ntt_place_e<LE>(L, pass, t, 0));
}
template <int LE>
DM_HD uint32_t ntt_swz_reg_e(int L, int pass, int r) {
    return ntt_swz_e<LE>((uint32_t)r << ntt_pass_lo_e<LE>(L, pass));
}
DM_HD uint32_t ntt_swz_base(uint32_t base, int L, int pass, uint32_t t) {
    return ntt_swz_base_e<kNttLogE>(base, L, pass, t);
}
DM_HD uint32_t ntt_swz_reg(int L, int pass, int r) { return ntt_swz_reg_e<kNttLogE>(L, pass, r); }

// Whole transforms of one ring of size s = 2^L < 16 held in registers (one
// thread per ring and prime): forward from [0, 8p) (outputs below 14p), inverse
// on [0, 2p).
template <int L>
DM_HD void ntt_fwd_small(uint32_t* a, const Tw* tw, uint32_t p) {
    constexpr int s = 1 << L;
    const uint32_t p2 = 2 * p;
    DM_UNROLL
    for (int st = 0; st < L; ++st) {
        const int len = s >> (st + 1);
        DM_UNROLL
        for (int j = 0; j < s; ++j) {
            if (j & len) continue;
            const uint32_t k = (1u << st) + (uint32_t)(j >> (L - st));
            const uint32_t u = a[j];  // below 8p + 2p st < 14p
            const uint32_t v = shoup_mul(a[j + len], tw[k], p);
            a[j] = u + v;
            a[j + len] = u - v + p2;
        }
    }
}
template <int L>
DM_HD void ntt_inv_small(uint32_t* a, const Tw* tw, uint32_t p) {
    constexpr int s = 1 << L;
    const uint32_t p2 = 2 * p;
    DM_UNROLL
    for (int st = L - 1; st >= 0; --st) {
        const int len = s >> (st + 1);
        DM_UNROLL
        for (int j = 0; j < s; ++j) {
            if (j & len) continue;
            const uint32_t k = (1u << st) + (uint32_t)(j >> (L - st));
            const uint32_t u = a[j], v = a[j + len];
            a[j] = red_below(u + v, p2);
            a[j + len] = shoup_mul(u - v + p2, tw[k], p);
        }
    }
}

}  // namespace dm
