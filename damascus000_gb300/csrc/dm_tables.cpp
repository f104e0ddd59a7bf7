#include "dm_tables.h"

#include "dm_ntt.cuh"

#include <mutex>

namespace dm {

const uint32_t kRefCrtPrimes[kRefPrimes] = {3892314113u, 2281701377u, 2013265921u, 2885681153u,
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

uint32_t shoup_const(uint32_t w, uint32_t p) { return (uint32_t)(((uint64_t)w << 32) / p); }

namespace {

// Deterministic Miller-Rabin for n < 2^32 (bases 2, 7, 61).
bool is_prime_u32(uint32_t n) {
    if (n < 2) return false;
    for (uint32_t sp : {2u, 3u, 5u, 7u, 11u, 13u, 61u})
        if (n % sp == 0) return n == sp;
    uint32_t d = n - 1;
    int s = 0;
    while ((d & 1) == 0) {
        d >>= 1;
        ++s;
    }
    for (uint32_t a : {2u, 7u, 61u}) {
        uint64_t x = pow_mod(a, d, n);
        if (x == 1 || x == n - 1) continue;
        bool comp = true;
        for (int r = 1; r < s && comp; ++r) {
            x = x * x % n;
            if (x == n - 1) comp = false;
        }
        if (comp) return false;
    }
    return true;
}

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

// Minimal little-endian 384-bit integer for the CRT constants (P < 2^252).
struct U384 {
    uint64_t w[6] = {0, 0, 0, 0, 0, 0};
};
void mul_small(U384& a, uint64_t m) {
    unsigned __int128 c = 0;
    for (int i = 0; i < 6; ++i) {
        c += (unsigned __int128)a.w[i] * m;
        a.w[i] = (uint64_t)c;
        c >>= 64;
    }
}
uint64_t divmod_small(U384& a, uint64_t m) {  // a /= m, returns remainder
    unsigned __int128 r = 0;
    for (int i = 5; i >= 0; --i) {
        unsigned __int128 cur = (r << 64) | a.w[i];
        a.w[i] = (uint64_t)(cur / m);
        r = cur % m;
    }
    return (uint64_t)r;
}
// a mod q via 2^256 mod q folding: split into 256-bit low part and the rest.
fq mod_q(const U384& a) {
    // a < 2^384: a = lo + hi * 2^256, 2^256 mod q computed by fq arithmetic.
    uint32_t lo[8], hi[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 4; ++i) {
        lo[2 * i] = (uint32_t)a.w[i];
        lo[2 * i + 1] = (uint32_t)(a.w[i] >> 32);
    }
    for (int i = 0; i < 2; ++i) {
        hi[2 * i] = (uint32_t)a.w[4 + i];
        hi[2 * i + 1] = (uint32_t)(a.w[4 + i] >> 32);
    }
    const fq l = fq_reduce8(lo), h = fq_reduce8(hi);
    uint32_t two256[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    // 2^255 reduced, then doubled
    two256[7] = 0x80000000u;
    fq t = fq_reduce8(two256);
    t = fq_add(t, t);
    return fq_add(l, fq_mul(h, t));
}

HostTables build() {
    HostTables t;
    // the nine largest primes below 2^28 of the form k * 2^14 + 1
    int found = 0;
    for (uint32_t k = ((1u << 28) - 1) >> 14; found < kPrimes && k > 0; --k) {
        const uint32_t p = (k << 14) + 1;
        if (p < (1u << 28) && is_prime_u32(p)) t.primes[found++] = p;
    }
    const size_t tab = (size_t)kPrimes * kMaxRing;
    t.fwd.resize(tab);
    t.inv.resize(tab);
    t.fwd_last.resize((size_t)kPrimes * kLastSpan);
    t.inv_last.resize((size_t)kPrimes * kLastSpan);
    for (int i = 0; i < kPrimes; ++i) {
        const uint32_t p = t.primes[i];
        PrimeConsts& c = t.pc;
        c.p[i] = p;
        c.one_s[i] = shoup_const(1, p);
        c.c1[i] = (uint32_t)((1ull << 32) % p);
        c.c1s[i] = shoup_const(c.c1[i], p);
        c.c2[i] = (uint32_t)((uint64_t)c.c1[i] * c.c1[i] % p);
        c.c2s[i] = shoup_const(c.c2[i], p);
        c.c3[i] = (uint32_t)((uint64_t)c.c2[i] * c.c1[i] % p);

        const uint32_t g = generator_of(p);
        const uint32_t psi = pow_mod(g, (p - 1) / (2ull * kMaxRing), p);
        const uint32_t psi_inv = inv_mod(psi, p);
        for (uint32_t k = 0; k < kMaxRing; ++k) {
            const uint32_t e = bitrev(k, kLogMaxRing);
            const size_t at = (size_t)i * kMaxRing + k;
            const uint32_t z = pow_mod(psi, e, p), zi = pow_mod(psi_inv, e, p);
            t.fwd[at] = Tw{z, shoup_const(z, p)};
            t.inv[at] = Tw{zi, shoup_const(zi, p)};
        }
        for (int L = 4; L <= kLogMaxProverRing; ++L) {
            const size_t off = (size_t)i * kLastSpan + (1u << L) - 16u;
            for (int st = 4 * (ntt_pass_count(L) - 1); st < L; ++st) {
                const uint32_t ng = 8u >> (L - 1 - st);
                for (uint32_t j = 0; j < (1u << st); ++j) {
                    const uint32_t pos = ntt_last_pos(L, st, j / ng, (int)(j % ng));
                    t.fwd_last[off + pos] = t.fwd[(size_t)i * kMaxRing + (1u << st) + j];
                    t.inv_last[off + pos] = t.inv[(size_t)i * kMaxRing + (1u << st) + j];
                }
            }
        }
        const uint32_t inv4 = inv_mod(4, p);
        for (int L = 0; L <= kLogMaxRing; ++L) {
            const uint32_t ninv = inv_mod(pow_mod(2, L, p), p);
            t.ninv[i][L] = ninv;
            t.ninvs[i][L] = shoup_const(ninv, p);
            t.ninv4[i][L] = (uint32_t)((uint64_t)ninv * inv4 % p);
            t.ninv4s[i][L] = shoup_const(t.ninv4[i][L], p);
        }
    }
    // Garner constants.
    for (int j = 0; j < kPrimes; ++j)
        for (int i = 0; i < kPrimes; ++i) {
            t.cc.inv[j][i] = (j < i) ? inv_mod(t.primes[j] % t.primes[i], t.primes[i]) : 0;
            t.cc.invs[j][i] = shoup_const(t.cc.inv[j][i], t.primes[i]);
        }
    U384 prod;
    prod.w[0] = 1;
    for (int i = 0; i < kPrimes; ++i) {
        t.cc.radix_mod_q[i] = mod_q(prod);
        mul_small(prod, t.primes[i]);
    }
    t.cc.p_mod_q = mod_q(prod);
    // (P - 1) / 2 in mixed radix; P is odd so P - 1 only clears bit 0.
    U384 half = prod;
    half.w[0] -= 1;
    for (int i = 0; i < 6; ++i) half.w[i] = (half.w[i] >> 1) | (i < 5 ? half.w[i + 1] << 63 : 0);
    for (int i = 0; i < kPrimes; ++i) t.cc.half_digits[i] = (uint32_t)divmod_small(half, t.primes[i]);
    return t;
}

RefHostTables build_ref() {
    RefHostTables t;
    t.zeta.resize((size_t)kRefPrimes * kMaxRing);
    t.zinv.resize((size_t)kRefPrimes * kMaxRing);
    for (int i = 0; i < kRefPrimes; ++i) {
        const uint32_t p = kRefCrtPrimes[i];
        t.pc.p[i] = p;
        uint32_t inv = 1;  // Newton iteration for p^-1 mod 2^32
        for (int k = 0; k < 5; ++k) inv *= 2u - p * inv;
        t.pc.pinv[i] = inv;
        const uint64_t R = ((uint64_t)1 << 32) % p;
        const uint32_t r2 = (uint32_t)(R * R % p);
        const uint32_t g = generator_of(p);
        const uint32_t psi = pow_mod(g, (p - 1) / (2ull * kMaxRing), p);
        const uint32_t psi_inv = inv_mod(psi, p);
        for (uint32_t k = 0; k < kMaxRing; ++k) {
            const uint32_t e = bitrev(k, kLogMaxRing);
            t.zeta[(size_t)i * kMaxRing + k] = to_mont(pow_mod(psi, e, p), p);
            t.zinv[(size_t)i * kMaxRing + k] = to_mont(pow_mod(psi_inv, e, p), p);
        }
        for (int L = 0; L <= kLogMaxRing; ++L) {
            const uint32_t ninv = inv_mod(pow_mod(2, L, p), p);
            t.pc.ninv_r2[i][L] = (uint32_t)((uint64_t)ninv * r2 % p);
        }
    }
    return t;
}

}  // namespace

const HostTables& host_tables() {
    static HostTables* tables = nullptr;
    static std::once_flag once;
    std::call_once(once, [] { tables = new HostTables(build()); });
    return *tables;
}

const RefHostTables& ref_host_tables() {
    static RefHostTables* tables = nullptr;
    static std::once_flag once;
    std::call_once(once, [] { tables = new RefHostTables(build_ref()); });
    return *tables;
}

}  // namespace dm
