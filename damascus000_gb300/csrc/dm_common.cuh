// Shared definitions for the Damascus Fold GB300 library.
#pragma once

#include <cstddef>
#include <cstdint>

#if defined(__CUDACC__)
#define DM_HD __host__ __device__ __forceinline__
#define DM_D __device__ __forceinline__
#else
#define DM_HD inline
#define DM_D inline
#endif

#if defined(__CUDACC__)
#define DM_UNROLL _Pragma("unroll")
#else
#define DM_UNROLL
#endif

namespace dm {

// Module rank K of R_q^K (src/utils/config.rs:7).
constexpr int kRank = 8;
// NTT primes carrying the ring products: nine primes p < 2^28 with p = 1 mod 2^14
// (their product P > 2^251 bounds every commitment sum, |X| < 2^248, up to depth 12).
constexpr int kPrimes = 9;
// Primes per thread block of the transforms (kPrimes / kPrimesPerBlock blocks
// per polynomial): 1 or 3.  One prime per block measured faster (smaller blocks,
// more of them resident, their load phases overlap better).
#ifndef DM_PRIMES_PER_BLOCK
#define DM_PRIMES_PER_BLOCK 1
#endif
constexpr int kPrimesPerBlock = DM_PRIMES_PER_BLOCK;
static_assert(kPrimesPerBlock == 1 || kPrimesPerBlock == 3, "transform block shapes");
// The reference's eight CRT primes (src/utils/config.rs:9-18), used only by the
// reference-compatible FFI convolution hook, whose caller passes them in.
constexpr int kRefPrimes = 8;
// Largest negacyclic NTT the twiddle tables cover: 2^13 points (the prover uses
// ring degrees up to 2^12; the reference-compatible cyclic convolution of
// length n <= 2^12 zero-pads to 2n).
constexpr int kLogMaxRing = 13;
// Largest ring degree of the commitment / fold kernels.
constexpr int kLogMaxProverRing = 12;
constexpr uint32_t kMaxRing = 1u << kLogMaxRing;
// Deepest fold the prover accepts: the ring of degree 2^d must fit the transform
// kernels (2^12) and N * n * q^2 < P / 2 must hold (2^248 < 2^250.9 at d = 12).
constexpr int kMaxDepth = 12;
// Minimum fold depth (src/utils/config.rs:5).
constexpr int kMinDepth = 6;
constexpr int kBytesPerCoeff = 13;

}  // namespace dm
