// Exact integer arithmetic shared by host and device code.
//
//  * Z_q with q = 2^112 - 75 on four 32-bit limbs (little endian, the 16-byte
//    serde form of src/algebra/field.rs:112-129).  Multiplication is a 4x4 limb
//    schoolbook product reduced with 2^112 = 75 (mod q), the same pseudo-Mersenne
//    identity as field.rs:229-258.
//  * Montgomery arithmetic modulo the eight 29..32-bit CRT primes of
//    src/utils/config.rs:9-18, with R = 2^32.  Five primes exceed 2^31, so lazy
//    [0, 2p) butterflies do not fit a 32-bit word; every value stays in [0, p).
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

DM_HD fq fq_mul(const fq& a, const fq& b) {
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

// ====================== arithmetic modulo a CRT prime ======================

// Montgomery product a * b * 2^-32 mod p, for a < 2^32 and b < p.  Signed
// variant: t - m*p has zero low word, so the result is hi(t) - hi(m*p) in (-p, p).
DM_HD uint32_t mont_mul(uint32_t a, uint32_t b, uint32_t p, uint32_t pinv) {
#if defined(__CUDA_ARCH__)
    uint32_t tl = a * b;
    uint32_t th = __umulhi(a, b);
    uint32_t m = tl * pinv;
    uint32_t mh = __umulhi(m, p);
#else
    uint64_t t = (uint64_t)a * b;
    uint32_t tl = (uint32_t)t;
    uint32_t th = (uint32_t)(t >> 32);
    uint32_t m = tl * pinv;
    uint32_t mh = (uint32_t)(((uint64_t)m * p) >> 32);
    (void)tl;
#endif
    uint32_t r = th - mh;
    return th < mh ? r + p : r;
}

DM_HD uint32_t add_mod(uint32_t a, uint32_t b, uint32_t p) {
    uint32_t s = a + b;
    return (s < a || s >= p) ? s - p : s;
}
DM_HD uint32_t sub_mod(uint32_t a, uint32_t b, uint32_t p) {
    uint32_t d = a - b;
    return a < b ? d + p : d;
}
// A 64-bit accumulator hi * 2^32 + lo reduced mod p: mont_mul(hi, R^2) = hi * R,
// mont_mul(lo, R) = lo (mod p).
DM_HD uint32_t reduce_u64(uint64_t x, uint32_t p, uint32_t pinv, uint32_t r1, uint32_t r2) {
    uint32_t h = mont_mul((uint32_t)(x >> 32), r2, p, pinv);
    uint32_t l = mont_mul((uint32_t)x, r1, p, pinv);
    return add_mod(h, l, p);
}

// Constants of the eight primes handed to kernels by value (kernel-parameter space).
struct PrimeConsts {
    uint32_t p[kPrimes];
    uint32_t pinv[kPrimes];   // p^-1 mod 2^32
    uint32_t r1[kPrimes];     // R mod p (Montgomery form of 1)
    uint32_t r2[kPrimes];     // R^2 mod p
    uint32_t k32[kPrimes];    // 2^32 * R mod p
    uint32_t k64[kPrimes];    // 2^64 * R mod p
    uint32_t k96[kPrimes];    // 2^96 * R mod p
    uint32_t qres[kPrimes];   // q mod p
    uint32_t r1p[kPrimes], k32p[kPrimes], k64p[kPrimes], k96p[kPrimes];  // the above times p^-1 mod 2^32
};

// Residue of a Z_q element (four limbs) modulo prime i: sum_j x_j * 2^(32 j).
DM_HD uint32_t residue(const fq& x, const PrimeConsts& c, int i) {
    uint32_t p = c.p[i], pi = c.pinv[i];
    uint32_t r = mont_mul(x.w[0], c.r1[i], p, pi);
    r = add_mod(r, mont_mul(x.w[1], c.k32[i], p, pi), p);
    r = add_mod(r, mont_mul(x.w[2], c.k64[i], p, pi), p);
    r = add_mod(r, mont_mul(x.w[3], c.k96[i], p, pi), p);
    return r;
}

// Garner constants for recombining residues into Z_q (a centered lift, as
// src/algebra/ntt.rs:400-427 does with BigUint).
struct CrtConsts {
    uint32_t inv[kPrimes][kPrimes];  // inv[j][i] = p_j^-1 * R mod p_i   (j < i)
    uint32_t invp[kPrimes][kPrimes]; // inv[j][i] * p_i^-1 mod 2^32
    uint32_t half_digits[kPrimes];   // mixed-radix digits of (P - 1) / 2
    fq radix_mod_q[kPrimes];         // prod_{j<i} p_j mod q
    fq p_mod_q;                      // P mod q
};

// Same result as crt_to_fq with three-multiply Montgomery steps and one
// multi-limb accumulation of sum v_i * (prod_{j<i} p_j mod q) (< 2^147) before a
// single reduction mod q.
DM_HD fq crt_to_fq_fast(const uint32_t r[kPrimes], const PrimeConsts& pc, const CrtConsts& cc) {
    uint32_t v[kPrimes];
    DM_UNROLL
    for (int i = 0; i < kPrimes; ++i) {
        const uint32_t p = pc.p[i];
        uint32_t t = r[i];
        DM_UNROLL
        for (int j = 0; j < i; ++j) {
            // v_j mod p_i as v_j * R * R^-1
            uint32_t th, mh;
#if defined(__CUDA_ARCH__)
            th = __umulhi(v[j], pc.r1[i]);
            mh = __umulhi(v[j] * pc.r1p[i], p);
#else
            th = (uint32_t)(((uint64_t)v[j] * pc.r1[i]) >> 32);
            mh = (uint32_t)(((uint64_t)(uint32_t)(v[j] * pc.r1p[i]) * p) >> 32);
#endif
            const uint32_t vj = th < mh ? th - mh + p : th - mh;
            const uint32_t d = sub_mod(t, vj, p);
#if defined(__CUDA_ARCH__)
            th = __umulhi(d, cc.inv[j][i]);
            mh = __umulhi(d * cc.invp[j][i], p);
#else
            th = (uint32_t)(((uint64_t)d * cc.inv[j][i]) >> 32);
            mh = (uint32_t)(((uint64_t)(uint32_t)(d * cc.invp[j][i]) * p) >> 32);
#endif
            t = th < mh ? th - mh + p : th - mh;
        }
        v[i] = t;
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

// r[i] < p_i -> the integer X with |X| < P/2 congruent to r, reduced mod q.
DM_HD fq crt_to_fq(const uint32_t r[kPrimes], const PrimeConsts& pc, const CrtConsts& cc) {
    uint32_t v[kPrimes];
DM_UNROLL
    for (int i = 0; i < kPrimes; ++i) {
        uint32_t p = pc.p[i], pi = pc.pinv[i];
        uint32_t t = r[i];
DM_UNROLL
        for (int j = 0; j < i; ++j) {
            uint32_t vj = mont_mul(v[j], pc.r1[i], p, pi);  // v_j mod p_i
            t = mont_mul(sub_mod(t, vj, p), cc.inv[j][i], p, pi);
        }
        v[i] = t;
    }
    // X > (P-1)/2  <=>  digits compare greater from the top.
    int gt = 0, decided = 0;
DM_UNROLL
    for (int i = kPrimes - 1; i >= 0; --i) {
        if (!decided && v[i] != cc.half_digits[i]) {
            gt = v[i] > cc.half_digits[i];
            decided = 1;
        }
    }
    fq acc = fq_zero();
DM_UNROLL
    for (int i = 0; i < kPrimes; ++i) acc = fq_add(acc, fq_mul(fq_from_u32(v[i]), cc.radix_mod_q[i]));
    if (gt) acc = fq_sub(acc, cc.p_mod_q);
    return acc;
}

}  // namespace dm
