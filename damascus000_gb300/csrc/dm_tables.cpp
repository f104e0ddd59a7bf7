#include "dm_tables.h"

#include <mutex>

namespace dm {

const uint32_t kCrtPrimes[kPrimes] = {3892314113u, 2281701377u, 2013265921u, 2885681153u,
                                      2483027969u, 1811939329u, 469762049u,  4194304001u};

uint32_t pow_mod(uint32_t b, uint64_t e, uint32_t p) {
    uint64_t r = 1, x = b % p;
    while (e) {
        if (e & 1) r = r * x % p;
        x = x * x % p;
        e >>= 1;
    }
    return (uint32_t)r;
}

uint32_t bitrev(uint32_t x, int bits) {
    uint32_t r = 0;
    for (int b = 0; b < bits; ++b)
        if (x & (1u << b)) r |= 1u << (bits - 1 - b);
    return r;
}

namespace {

// Smallest generator of Z_p^* (checks x^((p-1)/f) != 1 for each prime f | p-1).
uint32_t generator_of(uint32_t p) {
    uint32_t f[32];
    int nf = 0;
    uint64_t v = p - 1;
    for (uint64_t d = 2; d * d <= v; d += (d == 2 ? 1 : 2))
        if (v % d == 0) {
            f[nf++] = (uint32_t)d;
            while (v % d == 0) v /= d;
        }
    if (v > 1) f[nf++] = (uint32_t)v;
    for (uint32_t g = 2;; ++g) {
        bool ok = true;
        for (int i = 0; i < nf && ok; ++i)
            if (pow_mod(g, (p - 1) / f[i], p) == 1) ok = false;
        if (ok) return g;
    }
}

uint32_t inv_mod(uint32_t a, uint32_t p) { return pow_mod(a, p - 2, p); }
uint32_t to_mont(uint32_t a, uint32_t p) { return (uint32_t)((((uint64_t)a) << 32) % p); }

// Minimal little-endian 256-bit integer for the CRT constants.
struct U256 {
    uint64_t w[4] = {0, 0, 0, 0};
};
void mul_small(U256& a, uint64_t m) {
    unsigned __int128 c = 0;
    for (int i = 0; i < 4; ++i) {
        c += (unsigned __int128)a.w[i] * m;
        a.w[i] = (uint64_t)c;
        c >>= 64;
    }
}
uint64_t divmod_small(U256& a, uint64_t m) {  // a /= m, returns remainder
    unsigned __int128 r = 0;
    for (int i = 3; i >= 0; --i) {
        unsigned __int128 cur = (r << 64) | a.w[i];
        a.w[i] = (uint64_t)(cur / m);
        r = cur % m;
    }
    return (uint64_t)r;
}
fq mod_q(const U256& a) {
    uint32_t r[8];
    for (int i = 0; i < 4; ++i) {
        r[2 * i] = (uint32_t)a.w[i];
        r[2 * i + 1] = (uint32_t)(a.w[i] >> 32);
    }
    return fq_reduce8(r);
}

HostTables build() {
    HostTables t;
    t.zeta.resize((size_t)kPrimes * kMaxRing);
    t.zinv.resize((size_t)kPrimes * kMaxRing);
    t.zetap.resize((size_t)kPrimes * kMaxRing);
    t.zinvp.resize((size_t)kPrimes * kMaxRing);
    for (int i = 0; i < kPrimes; ++i) {
        const uint32_t p = kCrtPrimes[i];
        t.pc.p[i] = p;
        uint32_t inv = 1;  // Newton iteration for p^-1 mod 2^32
        for (int k = 0; k < 5; ++k) inv *= 2u - p * inv;
        t.pc.pinv[i] = inv;
        const uint64_t R = ((uint64_t)1 << 32) % p;
        t.pc.r1[i] = (uint32_t)R;
        t.pc.r2[i] = (uint32_t)(R * R % p);
        t.pc.k32[i] = (uint32_t)((uint64_t)t.pc.r2[i]);                // 2^32 * R = R^2
        t.pc.k64[i] = (uint32_t)((uint64_t)t.pc.r2[i] * R % p);        // 2^64 * R = R^3
        t.pc.k96[i] = (uint32_t)((uint64_t)t.pc.k64[i] * R % p);       // 2^96 * R = R^4
        t.pc.r1p[i] = t.pc.r1[i] * inv;
        t.pc.k32p[i] = t.pc.k32[i] * inv;
        t.pc.k64p[i] = t.pc.k64[i] * inv;
        t.pc.k96p[i] = t.pc.k96[i] * inv;
        // q mod p
        unsigned __int128 q = (((unsigned __int128)1) << 112) - 75;
        t.pc.qres[i] = (uint32_t)(q % p);

        const uint32_t g = generator_of(p);
        const uint32_t psi = pow_mod(g, (p - 1) / (2ull * kMaxRing), p);
        t.psi[i] = psi;
        const uint32_t psi_inv = inv_mod(psi, p);
        for (uint32_t k = 0; k < kMaxRing; ++k) {
            uint32_t e = bitrev(k, kLogMaxRing);
            t.zeta[(size_t)i * kMaxRing + k] = to_mont(pow_mod(psi, e, p), p);
            t.zinv[(size_t)i * kMaxRing + k] = to_mont(pow_mod(psi_inv, e, p), p);
            t.zetap[(size_t)i * kMaxRing + k] = t.zeta[(size_t)i * kMaxRing + k] * t.pc.pinv[i];
            t.zinvp[(size_t)i * kMaxRing + k] = t.zinv[(size_t)i * kMaxRing + k] * t.pc.pinv[i];
        }
        const uint32_t inv4 = inv_mod(4, p);
        for (int L = 0; L <= kLogMaxRing; ++L) {
            uint32_t ninv = inv_mod(pow_mod(2, L, p), p);
            t.ninv_r2[i][L] = (uint32_t)((uint64_t)ninv * t.pc.r2[i] % p);
            t.ninv4_r2[i][L] = (uint32_t)((uint64_t)ninv * inv4 % p * t.pc.r2[i] % p);
        }
    }
    // Garner constants.
    for (int j = 0; j < kPrimes; ++j)
        for (int i = 0; i < kPrimes; ++i)
            t.cc.inv[j][i] = (j < i) ? to_mont(inv_mod(kCrtPrimes[j] % kCrtPrimes[i], kCrtPrimes[i]), kCrtPrimes[i]) : 0;
    for (int j = 0; j < kPrimes; ++j)
        for (int i = 0; i < kPrimes; ++i) t.cc.invp[j][i] = t.cc.inv[j][i] * t.pc.pinv[i];
    U256 prod;
    prod.w[0] = 1;
    for (int i = 0; i < kPrimes; ++i) {
        t.cc.radix_mod_q[i] = mod_q(prod);
        mul_small(prod, kCrtPrimes[i]);
    }
    t.cc.p_mod_q = mod_q(prod);
    // (P - 1) / 2 in mixed radix; P is odd so P - 1 only clears bit 0.
    U256 half = prod;
    half.w[0] -= 1;
    for (int i = 0; i < 4; ++i) half.w[i] = (half.w[i] >> 1) | (i < 3 ? half.w[i + 1] << 63 : 0);
    for (int i = 0; i < kPrimes; ++i) t.cc.half_digits[i] = (uint32_t)divmod_small(half, kCrtPrimes[i]);
    return t;
}

}  // namespace

const HostTables& host_tables() {
    static HostTables* tables = nullptr;
    static std::once_flag once;
    std::call_once(once, [] { tables = new HostTables(build()); });
    return *tables;
}

}  // namespace dm
