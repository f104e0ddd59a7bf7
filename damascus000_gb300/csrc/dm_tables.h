// Host-side construction of the NTT prime constants, the negacyclic twiddle
// tables and the Garner CRT constants (deterministic, a few milliseconds).
#pragma once

#include <vector>

#include "dm_field.cuh"
#include "dm_ref.cuh"

namespace dm {

struct HostTables {
    uint32_t primes[kPrimes];  // the nine largest primes p < 2^28 with p = 1 mod 2^14
    PrimeConsts pc;
    CrtConsts cc;
    // fwd[i * kMaxRing + k] = psi_i^brv13(k) mod p_i (psi_i a primitive
    // 2*kMaxRing-th root of unity) with its Shoup constant floor(z * 2^32 / p);
    // inv holds the inverses.
    std::vector<Tw> fwd, inv;
    // [prime][kLastSpan]: the same twiddles in the last-pass order of each ring
    // size 2^L (L = 4..12, block at 2^L - 16; see ntt_last_pos).
    std::vector<Tw> fwd_last, inv_last;
    // Final scale of an inverse transform of size 2^L: n^-1, and n^-1 / 4 for
    // the even/odd cross terms (with Shoup constants).
    uint32_t ninv[kPrimes][kLogMaxRing + 1], ninvs[kPrimes][kLogMaxRing + 1];
    uint32_t ninv4[kPrimes][kLogMaxRing + 1], ninv4s[kPrimes][kLogMaxRing + 1];
};
const HostTables& host_tables();

// The reference primes' Montgomery tables for the FFI convolution hook.
struct RefHostTables {
    RefPrimeConsts pc;
    std::vector<uint32_t> zeta, zinv;  // [prime][kMaxRing], Montgomery form
};
const RefHostTables& ref_host_tables();

uint32_t pow_mod(uint32_t b, uint64_t e, uint32_t p);
uint32_t bitrev(uint32_t x, int bits);
uint32_t shoup_const(uint32_t w, uint32_t p);

}  // namespace dm
