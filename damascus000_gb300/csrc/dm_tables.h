// Host-side construction of the per-prime Montgomery constants, the negacyclic
// NTT twiddle tables and the Garner CRT constants.
#pragma once

#include <vector>

#include "dm_field.cuh"

namespace dm {

// CRT primes in the reference's order (src/utils/config.rs:9-18).
extern const uint32_t kCrtPrimes[kPrimes];

struct HostTables {
    PrimeConsts pc;
    CrtConsts cc;
    // zeta[i * kMaxRing + k] = psi_i^brv12(k) * R mod p_i, psi_i a primitive
    // 2*kMaxRing-th root of unity; zinv holds the inverses (also Montgomery form).
    std::vector<uint32_t> zeta, zinv;
    // zetap[i] = zeta[i] * p^-1 mod 2^32 (likewise zinvp): three-multiply Montgomery twiddles
    std::vector<uint32_t> zetap, zinvp;
    // ninv_r2[i][L] = (2^L)^-1 * R^2 mod p_i : final scale of an inverse NTT of size
    // 2^L applied to Montgomery products (one R^-1 factor pending).
    uint32_t ninv_r2[kPrimes][kLogMaxRing + 1];
    // same with an extra 1/4 (the even/odd split of a forward transform).
    uint32_t ninv4_r2[kPrimes][kLogMaxRing + 1];
    // ordinary (non-Montgomery) cyclic roots for the reference-compatible cyclic NTT
    uint32_t psi[kPrimes];
};

// Builds all tables (deterministic; a few milliseconds).
const HostTables& host_tables();

uint32_t pow_mod(uint32_t b, uint64_t e, uint32_t p);
uint32_t bitrev(uint32_t x, int bits);

}  // namespace dm
