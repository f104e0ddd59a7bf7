// Host protocol pieces of the library compiled for the CPU and checked against
// the reference's own unit tests for them:
//   challenge_sampler_rejects_zero_candidates (src/protocol/transcript.rs:130-142)
//   serde_uses_fixed_width_encoding           (src/algebra/field.rs:305-311)
//   hard_spec_constants_are_wired             (src/utils/config.rs:106-114)
// plus the verifier's one-pass commitment update (module_fold) against two
// module_add_scaled calls, the form of src/protocol/verifier.rs:64-103, and the
// host multiply against the device limb form.
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "host_blake3.h"
#include "protocol.h"

using namespace dm;

static int failures = 0;
#define CHECK(cond)                                                  \
    do {                                                             \
        if (!(cond)) {                                               \
            std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #cond); \
            ++failures;                                              \
        }                                                            \
    } while (0)

static fq fq_from_u64(uint64_t v) { return fq{{(uint32_t)v, (uint32_t)(v >> 32), 0u, 0u}}; }

static fq random_fq(std::mt19937_64& rng) {
    uint32_t r[8];
    for (int i = 0; i < 8; ++i) r[i] = (uint32_t)rng();
    return fq_reduce8(r);
}

static Module random_module(std::mt19937_64& rng, uint32_t n) {
    Module m = Module::zero(n);
    for (auto& v : m.c) v = random_fq(rng);
    return m;
}

int main() {
    // the sampler returns the first nonzero candidate, trying counters in order
    {
        std::vector<uint32_t> seen;
        const fq v = sample_nonzero_challenge([&](uint32_t counter) {
            seen.push_back(counter);
            return counter < 2 ? fq_zero() : fq_from_u64(9);
        });
        CHECK(fq_eq(v, fq_from_u64(9)));
        CHECK((seen == std::vector<uint32_t>{0, 1, 2}));
    }
    // an element serialises to 16 little-endian bytes and back
    {
        const fq v = fq_from_u64(42);
        uint8_t b[16];
        fq_to_bytes(v, b);
        CHECK(b[0] == 42);
        for (int i = 1; i < 16; ++i) CHECK(b[i] == 0);
        CHECK(fq_eq(fq_from_bytes(b), v));
        std::vector<uint8_t> enc;
        Module m = Module::zero(4);
        m.c[3] = v;
        encode_module(enc, m);
        CHECK(enc.size() == 8 + kRank * (8 + 4 * 16));  // u64 8, then per coordinate u64 n + n words
    }
    // the protocol's fixed constants
    {
        CHECK(kMinDepth == 6);
        CHECK(kRank == 8);
        CHECK(kBytesPerCoeff == 13);
        CHECK(kRefPrimes == 8);
        uint32_t d = 0;
        uint64_t dim = 0;
        CHECK(square_layout_for_byte_len(1, &d, &dim) && d == 6 && dim == 64);  // MIN_RING_DEGREE = 2^6
        CHECK(coeff_count_for_byte_len(13) == 1 && coeff_count_for_byte_len(14) == 2);
    }
    // the host multiply (64-bit halves) equals the device limb form on every input:
    // reduced values, edge values, and words of 2^112 and above (limb fallback)
    {
        std::mt19937_64 rng(11);
        const fq qm1{{kQ0 - 1, kQ1, kQ2, kQ3}}, top{{0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFu}};
        const fq wide{{0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}}, just{{0u, 0u, 0u, 0x10000u}};
        const fq edge[] = {fq_zero(), fq_from_u32(1), fq_from_u32(75), qm1, top, wide, just};
        for (const fq& a : edge)
            for (const fq& b : edge) CHECK(fq_eq(fq_mul(a, b), fq_mul_limbs(a, b)));
        for (int i = 0; i < 1000000; ++i) {
            fq a = random_fq(rng), b = random_fq(rng);
            if (i % 7 == 0) a.w[3] = (uint32_t)rng();  // unreduced words
            CHECK(fq_eq(fq_mul(a, b), fq_mul_limbs(a, b)));
            if (failures > 10) return 1;
        }
    }
    // module_fold == two module_add_scaled calls, plain and on the even coefficients
    {
        std::mt19937_64 rng(7);
        for (uint32_t n : {1u, 2u, 8u, 64u, 2048u, 4096u}) {
            const Module base = random_module(rng, n), l = random_module(rng, n), r = random_module(rng, n);
            const fq x = random_fq(rng), xi = fq_inv(x);
            Module t, two, one;
            CHECK(module_add_scaled(base, l, xi, t) && module_add_scaled(t, r, x, two));
            CHECK(module_fold(base, false, l, xi, r, x, one));
            CHECK(one == two);
            if (n >= 2) {
                const Module le = random_module(rng, n / 2), re = random_module(rng, n / 2);
                const fq y = random_fq(rng), yi = fq_inv(y);
                Module t2, two2, one2;
                CHECK(module_add_scaled(module_even(base), le, yi, t2) && module_add_scaled(t2, re, y, two2));
                CHECK(module_fold(base, true, le, yi, re, y, one2));
                CHECK(one2 == two2);
                CHECK(!module_fold(base, true, l, yi, r, y, one2));  // ring lengths differ
            }
            if (n == 4096) {  // the same with the work split over the host pool
                Module serial;
                {
                    HostSerialScope scope;
                    CHECK(module_fold(base, false, l, xi, r, x, serial));
                }
                CHECK(serial == one);
            }
        }
    }
    if (failures) return 1;
    std::printf("ok\n");
    return 0;
}
