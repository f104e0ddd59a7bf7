// Arithmetic modulo the reference's eight CRT primes (src/utils/config.rs:9-18).
// Only the reference-compatible FFI hook damascus_cuda_ntt_batch uses them: its
// caller passes these primes and expects per-prime residues back.  Montgomery
// products with R = 2^32 (five of the primes exceed 2^31, so values stay in [0, p)).
#pragma once

#include <cuda_runtime.h>

#include "dm_field.cuh"

namespace dm {

// Montgomery product a * b * 2^-32 mod p, for a < 2^32 and b < p.  Signed
// variant: t - m*p has zero low word, so the result is hi(t) - hi(m*p) in (-p, p).
DM_HD uint32_t mont_mul(uint32_t a, uint32_t b, uint32_t p, uint32_t pinv) {
    const uint32_t tl = a * b;
    const uint32_t th = mulhi32(a, b);
    const uint32_t m = tl * pinv;
    const uint32_t mh = mulhi32(m, p);
    const uint32_t r = th - mh;
    return th < mh ? r + p : r;
}

struct RefPrimeConsts {
    uint32_t p[kRefPrimes];
    uint32_t pinv[kRefPrimes];                        // p^-1 mod 2^32
    uint32_t ninv_r2[kRefPrimes][kLogMaxRing + 1];     // (2^L)^-1 * R^2 mod p
};

// Device copies for the FFI convolution: Montgomery-form negacyclic twiddles
// psi^brv(k) * R and their inverses, [prime][kMaxRing].
struct RefDeviceTables {
    RefPrimeConsts pc;
    const uint32_t* zeta = nullptr;
    const uint32_t* zinv = nullptr;
};

extern const uint32_t kRefCrtPrimes[kRefPrimes];

cudaError_t upload_ref_tables(RefDeviceTables* out);
void free_ref_tables(RefDeviceTables* t);
// Per-prime length-2^Ln cyclic convolution of residue vectors [8][2^Ln] (Ln <= 12).
cudaError_t launch_cyclic_conv(const RefDeviceTables& T, const uint32_t* d_a, const uint32_t* d_b, uint32_t* d_out,
                               uint32_t Ln, cudaStream_t st);

}  // namespace dm
