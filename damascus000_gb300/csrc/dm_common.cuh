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
// (their product P = 2^251.98 bounds every commitment sum, |X| < 2^250, up to depth 13).
constexpr int kPrimes = 9;
// Primes per thread of the forward transforms (kPrimes / kPrimesPerThread blocks
// per polynomial): 1 or 3.  Three read each 16-byte coefficient once for three
// residue rows (a third of the load traffic through L1) but triple the unrolled
// code; one measured faster (the larger kernel stalls on instruction fetch).
#ifndef DM_PRIMES_PER_THREAD
#define DM_PRIMES_PER_THREAD 1
#endif
constexpr int kPrimesPerThread = DM_PRIMES_PER_THREAD;
static_assert(kPrimesPerThread == 1 || kPrimesPerThread == 3, "transform block shapes");
// The reference's eight CRT primes (src/utils/config.rs:9-18), used only by the
// reference-compatible FFI convolution hook, whose caller passes them in.
constexpr int kRefPrimes = 8;
// Largest negacyclic NTT the twiddle tables cover: 2^13 points (the prover uses
// ring degrees up to 2^13; the reference-compatible cyclic convolution of
// length n <= 2^12 zero-pads to 2n).
constexpr int kLogMaxRing = 13;
// Largest ring degree of the commitment / fold kernels.
constexpr int kLogMaxProverRing = 13;
constexpr uint32_t kMaxRing = 1u << kLogMaxRing;
// Last-pass twiddle tables: one block of 2^L entries per ring size 2^L, L = 4..13,
// at offset 2^L - 16 within a prime's span.
constexpr uint32_t kLastSpan = (2u << kLogMaxProverRing) - 16u;
// Deepest fold the prover accepts: the ring of degree 2^d must fit the transform
// kernels (2^13) and N * n * q^2 < P / 2 must hold (2^250 < 2^250.98 at d = 13;
// d = 14 would need a tenth prime).
constexpr int kMaxDepth = 13;
// Minimum fold depth (src/utils/config.rs:5).
constexpr int kMinDepth = 6;
constexpr int kBytesPerCoeff = 13;

}  // namespace dm
