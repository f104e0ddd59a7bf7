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
// Number of CRT primes (src/utils/config.rs:9-18).
constexpr int kPrimes = 8;
// Largest negacyclic NTT the twiddle tables cover: 2^13 points (the prover uses
// ring degrees up to 2^12; the reference-compatible cyclic convolution of
// length n <= 2^12 zero-pads to 2n).
constexpr int kLogMaxRing = 13;
// Largest ring degree of the commitment / fold kernels.
constexpr int kLogMaxProverRing = 12;
constexpr uint32_t kMaxRing = 1u << kLogMaxRing;
// Depth limit for which summing all N columns in the NTT domain stays inside the
// CRT range: N * n * q^2 < P / 2 holds up to d = 11 (2^246 < 2^247.016).
constexpr int kMaxDepth = 11;
// Minimum fold depth (src/utils/config.rs:5).
constexpr int kMinDepth = 6;
constexpr int kBytesPerCoeff = 13;

}  // namespace dm
