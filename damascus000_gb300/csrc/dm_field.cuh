// Exact integer arithmetic shared by host and device code.
//
//  * Z_q with q = 2^112 - 75 on four 32-bit limbs (little endian, the 16-byte
//    serde form of src/algebra/field.rs:112-129).  Multiplication is a 4x4 limb
//    schoolbook product reduced with 2^112 = 75 (mod q), the same pseudo-Mersenne
//    identity as field.rs:229-258; host code multiplies reduced values with
//    64-bit halves instead (same results).
//  * Arithmetic modulo the nine NTT primes p < 2^28 (p = 1 mod 2^14) that carry
//    every ring product: Shoup products by constants give [0, 2p), so the
//    transforms run four stages on values below 16p < 2^32 without reducing
//    (lazy Harvey butterflies), and products of two reduced residues fit 56 bits.
//  * Garner recombination of the nine residues into Z_q with a centred lift
//    (the integer result of src/algebra/ntt.rs:372-427; P = 2^251.98 leaves room
//    for any commitment sum, |X| < 2^250, up to depth 13).
#pragma once

#include "dm_common.cuh"

namespace dm {

struct fq {
    uint32_t w[4];
};

DM_HD fq fq_zero() { return fq{{0u, 0u, 0u, 0u}}; }
DM_HD fq fq_from_u32(uint32_t v) { return fq{{v, 0u, 0u, 0u}}; }
DM_HD bool fq_is_zero(const fq& a) { return (a.w[0] | a.w[1] | a.w[2] | a.w[3]) == 0u; }
DM_HD bool fq_eq(const fq& a, const fq& b) {
    return a.w[0] == b.w[0] && a.w[1] == b.w[1] && a.w[2] == b.w[2] && a.w[3] == b.w[3];
}

// q = 2^112 - 75 in limbs.
constexpr uint32_t kQ0 = 0xFFFFFFB5u, kQ1 = 0xFFFFFFFFu, kQ2 = 0xFFFFFFFFu, kQ3 = 0x0000FFFFu;

// x < 2^113 -> x mod q, using x >= q  <=>  x + 75 >= 2^112.
DM_HD fq fq_canon(const fq& x) {
    uint64_t c = (uint64_t)x.w[0] + 75u;
    uint32_t t0 = (uint32_t)c;
    c = (c >> 32) + x.w[1];
    uint32_t t1 = (uint32_t)c;
    c = (c >> 32) + x.w[2];
    uint32_t t2 = (uint32_t)c;
    c = (c >> 32) + x.w[3];
    uint32_t t3 = (uint32_t)c;
    if (t3 >> 16) return fq{{t0, t1, t2, t3 & 0xFFFFu}};
    return x;
}

DM_HD fq fq_add(const fq& a, const fq& b) {
    fq s;
    uint64_t c = (uint64_t)a.w[0] + b.w[0];
    s.w[0] = (uint32_t)c;
    c = (c >> 32) + a.w[1] + b.w[1];
    s.w[1] = (uint32_t)c;
    c = (c >> 32) + a.w[2] + b.w[2];
    s.w[2] = (uint32_t)c;
    c = (c >> 32) + a.w[3] + b.w[3];
    s.w[3] = (uint32_t)c;
    return fq_canon(s);
}

DM_HD fq fq_sub(const fq& a, const fq& b) {
    // d = a - b (mod 2^128); if it borrowed, add q.
    uint64_t br;
    fq d;
    uint64_t t = (uint64_t)a.w[0] - b.w[0];
    d.w[0] = (uint32_t)t;
    br = (t >> 63) & 1u;
    t = (uint64_t)a.w[1] - b.w[1] - br;
    d.w[1] = (uint32_t)t;
    br = (t >> 63) & 1u;
    t = (uint64_t)a.w[2] - b.w[2] - br;
    d.w[2] = (uint32_t)t;
    br = (t >> 63) & 1u;
    t = (uint64_t)a.w[3] - b.w[3] - br;
    d.w[3] = (uint32_t)t;
    br = (t >> 63) & 1u;
    if (br) {
        uint64_t c = (uint64_t)d.w[0] + kQ0;
        d.w[0] = (uint32_t)c;
        c = (c >> 32) + d.w[1] + kQ1;
        d.w[1] = (uint32_t)c;
        c = (c >> 32) + d.w[2] + kQ2;
        d.w[2] = (uint32_t)c;
        c = (c >> 32) + d.w[3] + kQ3;
        d.w[3] = (uint32_t)c;
    }
    return d;
}

DM_HD fq fq_neg(const fq& a) { return fq_sub(fq_zero(), a); }

// r[0..7] < 2^256 -> r mod q.
DM_HD fq fq_reduce8(const uint32_t r[8]) {
    // hi = r >> 112 (144 bits), t = (r mod 2^112) + 75 * hi < 2^152.
    uint32_t h0 = (r[3] >> 16) | (r[4] << 16);
    uint32_t h1 = (r[4] >> 16) | (r[5] << 16);
    uint32_t h2 = (r[5] >> 16) | (r[6] << 16);
    uint32_t h3 = (r[6] >> 16) | (r[7] << 16);
    uint32_t h4 = r[7] >> 16;
    uint64_t c = (uint64_t)r[0] + (uint64_t)h0 * 75u;
    uint32_t t0 = (uint32_t)c;
    c = (c >> 32) + r[1] + (uint64_t)h1 * 75u;
    uint32_t t1 = (uint32_t)c;
    c = (c >> 32) + r[2] + (uint64_t)h2 * 75u;
    uint32_t t2 = (uint32_t)c;
    c = (c >> 32) + (r[3] & 0xFFFFu) + (uint64_t)h3 * 75u;
    uint32_t t3 = (uint32_t)c;
    c = (c >> 32) + (uint64_t)h4 * 75u;
    uint32_t t4 = (uint32_t)c;
    // second fold: hi2 = t >> 112 < 2^40.
    uint64_t m = ((uint64_t)(t3 >> 16) | ((uint64_t)t4 << 16)) * 75u;  // < 2^47
    fq o;
    c = (uint64_t)t0 + (uint32_t)m;
    o.w[0] = (uint32_t)c;
    c = (c >> 32) + t1 + (m >> 32);
    o.w[1] = (uint32_t)c;
    c = (c >> 32) + t2;
    o.w[2] = (uint32_t)c;
    c = (c >> 32) + (t3 & 0xFFFFu);
    o.w[3] = (uint32_t)c;  // o < 2^112 + 2^47 < 2q
    return fq_canon(o);
}

DM_HD fq fq_mul_limbs(const fq& a, const fq& b) {
    uint32_t r[8] = {0, 0, 0, 0, 0, 0, 0, 0};
DM_UNROLL
    for (int i = 0; i < 4; ++i) {
        uint64_t c = 0;
DM_UNROLL
        for (int j = 0; j < 4; ++j) {
            c += (uint64_t)a.w[i] * b.w[j] + r[i + j];
            r[i + j] = (uint32_t)c;
            c >>= 32;
        }
        r[i + 4] = (uint32_t)c;
    }
    return fq_reduce8(r);
}

#if !defined(__CUDA_ARCH__) && defined(__SIZEOF_INT128__)
// Host form for inputs below 2^112 (every reduced value): four 64 x 64-bit
// products instead of sixteen 32 x 32, the same reduction 2^112 = 75 (mod q) to
// the canonical value, so the result equals fq_mul_limbs bit for bit.  False
// for wider inputs (words of an unchecked proof), which take the limb form.
inline bool fq_mul_wide(const fq& a, const fq& b, fq* out) {
    if ((a.w[3] | b.w[3]) >> 16) return false;
    typedef unsigned __int128 u128;
    const uint64_t a0 = a.w[0] | (uint64_t)a.w[1] << 32, a1 = a.w[2] | (uint64_t)a.w[3] << 32;
    const uint64_t b0 = b.w[0] | (uint64_t)b.w[1] << 32, b1 = b.w[2] | (uint64_t)b.w[3] << 32;
    const u128 p00 = (u128)a0 * b0;
    const u128 mid = (u128)a0 * b1 + (u128)a1 * b0;  // a1, b1 < 2^48: < 2^113
    const u128 p11 = (u128)a1 * b1;                  // < 2^96
    const uint64_t r0 = (uint64_t)p00;
    u128 t = (p00 >> 64) + (uint64_t)mid;
    const uint64_t r1 = (uint64_t)t;
    t = (t >> 64) + (mid >> 64) + p11;  // the product's bits from 128 on (< 2^96)
    const u128 m112 = ((u128)1 << 112) - 1;
    const u128 lo = ((u128)(r1 & ((1ull << 48) - 1)) << 64) | r0;  // product mod 2^112
    const u128 hi = (t << 16) | (r1 >> 48);                         // product >> 112, < 2^112
    u128 r = lo + hi * 75u;                                         // < 2^119
    r = (r & m112) + (r >> 112) * 75u;                              // < 2^112 + 2^14 < 2q
    const u128 q = ((u128)1 << 112) - 75u;
    if (r >= q) r -= q;
    out->w[0] = (uint32_t)r;
    out->w[1] = (uint32_t)(r >> 32);
    out->w[2] = (uint32_t)(r >> 64);
    out->w[3] = (uint32_t)(r >> 96);
    return true;
}
#endif

DM_HD fq fq_mul(const fq& a, const fq& b) {
#if !defined(__CUDA_ARCH__) && defined(__SIZEOF_INT128__)
    fq w;
    if (fq_mul_wide(a, b, &w)) return w;
#endif
    return fq_mul_limbs(a, b);
}

// a + c * b (mod q): the fold map of src/protocol/prover.rs:332-457.
DM_HD fq fq_fma(const fq& a, const fq& c, const fq& b) { return fq_add(a, fq_mul(c, b)); }

// ---- conversions between 16-byte little-endian words and limbs (host side) ----
inline fq fq_from_bytes(const uint8_t* p) {
    fq r;
    for (int i = 0; i < 4; ++i)
        r.w[i] = (uint32_t)p[4 * i] | ((uint32_t)p[4 * i + 1] << 8) | ((uint32_t)p[4 * i + 2] << 16) |
                 ((uint32_t)p[4 * i + 3] << 24);
    return r;
}
inline void fq_to_bytes(const fq& a, uint8_t* p) {
    for (int i = 0; i < 4; ++i) {
        p[4 * i] = (uint8_t)a.w[i];
        p[4 * i + 1] = (uint8_t)(a.w[i] >> 8);
        p[4 * i + 2] = (uint8_t)(a.w[i] >> 16);
        p[4 * i + 3] = (uint8_t)(a.w[i] >> 24);
    }
}
// Arbitrary 128-bit value reduced mod q (deserialisation, field.rs:121-129).
inline fq fq_from_u128_words(const fq& x) {
    uint32_t r[8] = {x.w[0], x.w[1], x.w[2], x.w[3], 0, 0, 0, 0};
    return fq_reduce8(r);
}
// Exponentiation and inversion by Fermat (field.rs:89-109).
inline fq fq_pow(fq base, const fq& e) {
    fq r = fq_from_u32(1);
    for (int limb = 0; limb < 4; ++limb)
        for (int bit = 0; bit < 32; ++bit) {
            if ((e.w[limb] >> bit) & 1u) r = fq_mul(r, base);
            base = fq_mul(base, base);
        }
    return r;
}
inline fq fq_inv(const fq& a) {
    const fq qm2{{kQ0 - 2u, kQ1, kQ2, kQ3}};
    return fq_pow(a, qm2);
}

// ====================== arithmetic modulo an NTT prime ======================

DM_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}
DM_HD uint32_t umin32(uint32_t a, uint32_t b) { return a < b ? a : b; }

// x mod p in [0, m) for x in [0, 2m): min(x, x - m) (x - m wraps when x < m).
DM_HD uint32_t red_below(uint32_t x, uint32_t m) { return umin32(x, x - m); }

// Shoup product x * w mod p in [0, 2p) for any x < 2^32, with w < p < 2^31 and
// ws = floor(w * 2^32 / p): q = floor(x * ws / 2^32) is floor(x w / p) or one less.
DM_HD uint32_t shoup_mul(uint32_t x, uint32_t w, uint32_t ws, uint32_t p) {
    const uint32_t q = mulhi32(x, ws);
    return x * w - q * p;
}

// A twiddle (or any constant factor) with its Shoup constant, loaded as one 8-byte word.
struct alignas(8) Tw {
    uint32_t w, s;
};
DM_HD uint32_t shoup_mul(uint32_t x, Tw t, uint32_t p) { return shoup_mul(x, t.w, t.s, p); }

// Generic reductions (any p < 2^32) used by the reference-prime FFI path too.
DM_HD uint32_t add_mod(uint32_t a, uint32_t b, uint32_t p) {
    uint32_t s = a + b;
    return (s < a || s >= p) ? s - p : s;
}
DM_HD uint32_t sub_mod(uint32_t a, uint32_t b, uint32_t p) {
    uint32_t d = a - b;
    return a < b ? d + p : d;
}

// Constants of the nine NTT primes handed to kernels by value.
struct PrimeConsts {
    uint32_t p[kPrimes];
    uint32_t one_s[kPrimes];  // floor(2^32 / p): Shoup constant of 1
    uint32_t c1[kPrimes];     // 2^32 mod p
    uint32_t c1s[kPrimes];    // floor(c1 * 2^32 / p)
    uint32_t c2[kPrimes];     // 2^64 mod p
    uint32_t c2s[kPrimes];
    uint32_t c3[kPrimes];     // 2^96 mod p
};

// A 64-bit value mod p in [0, 4p): hi * (2^32 mod p) + lo * 1, two Shoup products.
DM_HD uint32_t red64_lazy(uint64_t t, const PrimeConsts& c, int i) {
    const uint32_t p = c.p[i];
    return shoup_mul((uint32_t)(t >> 32), c.c1[i], c.c1s[i], p) + shoup_mul((uint32_t)t, 1u, c.one_s[i], p);
}
DM_HD uint32_t red64(uint64_t t, const PrimeConsts& c, int i) {
    const uint32_t p = c.p[i];
    return red_below(red_below(red64_lazy(t, c, i), 2 * p), p);
}
// hi * 2^64 + lo (hi < 2^32) mod p in [0, p).
DM_HD uint32_t red96(uint32_t hi, uint64_t lo, const PrimeConsts& c, int i) {
    const uint32_t p = c.p[i];
    const uint32_t a = red_below(red64_lazy(lo, c, i), 2 * p);            // [0, 2p)
    const uint32_t b = shoup_mul(hi, c.c2[i], c.c2s[i], p);                 // [0, 2p)
    return red_below(red_below(a + b, 2 * p), p);
}

// Residue of a 128-bit word x = sum_j x_j 2^(32 j) modulo prime i, in [0, 4p):
// x_0 + x_1 c1 + x_2 c2 + x_3 c3 < 2^32 + 3 * 2^62 fits one 64-bit accumulation.
DM_HD uint32_t residue_lazy(const fq& x, const PrimeConsts& c, int i) {
    const uint64_t t = (uint64_t)x.w[0] + (uint64_t)x.w[1] * c.c1[i] + (uint64_t)x.w[2] * c.c2[i] +
                       (uint64_t)x.w[3] * c.c3[i];
    return red64_lazy(t, c, i);
}
// The same residue below 8p with one multiply fewer, as a forward transform
// input: the low word (< 2^32 < 16.01p) is brought below 4.01p by two
// conditional subtractions instead of a Shoup product by 1.
DM_HD uint32_t residue_fwd(const fq& x, const PrimeConsts& c, int i) {
    const uint32_t p = c.p[i];
    const uint64_t t = (uint64_t)x.w[0] + (uint64_t)x.w[1] * c.c1[i] + (uint64_t)x.w[2] * c.c2[i] +
                       (uint64_t)x.w[3] * c.c3[i];
    return shoup_mul((uint32_t)(t >> 32), c.c1[i], c.c1s[i], p) + red_below(red_below((uint32_t)t, 8 * p), 4 * p);
}
DM_HD uint32_t residue(const fq& x, const PrimeConsts& c, int i) {
    const uint32_t p = c.p[i];
    return red_below(red_below(residue_lazy(x, c, i), 2 * p), p);
}

// Garner constants for recombining residues into Z_q (a centred lift, as
// src/algebra/ntt.rs:400-427 does with BigUint).
struct CrtConsts {
    uint32_t inv[kPrimes][kPrimes];   // inv[j][i] = p_j^-1 mod p_i   (j < i)
    uint32_t invs[kPrimes][kPrimes];  // Shoup constants of inv
    uint32_t half_digits[kPrimes];    // mixed-radix digits of (P - 1) / 2
    fq radix_mod_q[kPrimes];          // prod_{j<i} p_j mod q
    fq p_mod_q;                       // P mod q
};

// r[i] < p_i -> the integer X with |X| < P/2 congruent to r, reduced mod q.
// Mixed-radix digits by Garner (each step one Shoup product), then one
// multi-limb accumulation of sum v_i * (prod_{j<i} p_j mod q) (< 2^147) and a
// single reduction mod q; X > (P-1)/2 (a negative value) subtracts P mod q.
DM_HD fq crt_to_fq(const uint32_t r[kPrimes], const PrimeConsts& pc, const CrtConsts& cc) {
    uint32_t v[kPrimes];
    DM_UNROLL
    for (int i = 0; i < kPrimes; ++i) {
        const uint32_t p = pc.p[i];
        uint32_t t = r[i];  // [0, p), then [0, 2p) after each step
        DM_UNROLL
        for (int j = 0; j < i; ++j) {
            // v_j < p_j < 2^28 < 2 p_i: one conditional subtraction gives v_j mod p_i
            const uint32_t vj = red_below(v[j], p);
            const uint32_t tr = red_below(t, p);
            t = shoup_mul(tr + p - vj, cc.inv[j][i], cc.invs[j][i], p);
        }
        v[i] = red_below(t, p);
    }
    int gt = 0, decided = 0;
    DM_UNROLL
    for (int i = kPrimes - 1; i >= 0; --i) {
        if (!decided && v[i] != cc.half_digits[i]) {
            gt = v[i] > cc.half_digits[i];
            decided = 1;
        }
    }
    uint64_t acc[6] = {0, 0, 0, 0, 0, 0};
    DM_UNROLL
    for (int i = 0; i < kPrimes; ++i)
        DM_UNROLL
        for (int w = 0; w < 4; ++w) {
            const uint64_t prod = (uint64_t)v[i] * cc.radix_mod_q[i].w[w];
            acc[w] += (uint32_t)prod;
            acc[w + 1] += prod >> 32;
        }
    uint32_t x8[8];
    uint64_t carry = 0;
    DM_UNROLL
    for (int w = 0; w < 6; ++w) {
        carry += acc[w];
        x8[w] = (uint32_t)carry;
        carry >>= 32;
    }
    x8[6] = (uint32_t)carry;
    x8[7] = 0;
    fq x = fq_reduce8(x8);
    if (gt) x = fq_sub(x, cc.p_mod_q);
    return x;
}

}  // namespace dm
