// Kernel launch interfaces outside the multi-job ring arithmetic.  Device buffer
// layouts used throughout:
//   coefficient domain : uint4 per Z_q element (16-byte LE), arrays [poly][coeff]
//   generators         : [vec][coord][coeff]  (src/commitment/sis.rs:212-229 order)
//   NTT domain         : uint32 residues [poly][prime][slot] (9 primes), slot = the
//                        bit-reversed evaluation index of the negacyclic transform
//   MAC partial sums   : uint32 [part][row][slot], row = coord * 9 + prime
#pragma once

#include <cuda_runtime.h>

#include "dm_field.cuh"

namespace dm {

// Per-device copies of the NTT prime tables.
struct DeviceTables {
    PrimeConsts pc;
    CrtConsts cc;
    const Tw* fwd = nullptr;  // [prime][kMaxRing]: psi^brv(k) with Shoup constants
    const Tw* inv = nullptr;  // inverses
    const Tw* fwd_last = nullptr;  // [prime][kLastSpan]: last-pass order per ring size
    const Tw* inv_last = nullptr;
};

// Uploads the tables to the current device and sets the kernels' shared-memory
// limits (once per device and context).
cudaError_t upload_tables(DeviceTables* out);
void free_tables(DeviceTables* t);

// ---- hashing / expansion (k_hash.cu) ----
// BLAKE3 digest of a device buffer; cv_scratch holds 2 * 8 * nchunks words.
cudaError_t launch_file_hash(const uint8_t* d_file, uint64_t len, uint32_t* d_cv_scratch, uint32_t* d_out8,
                             cudaStream_t st);
size_t file_hash_scratch_words(uint64_t len);
// generators [N][8][n] from the 32-byte g_0 seed (sis.rs:212-245)
cudaError_t launch_gen_generators(const uint8_t g_seed[32], uint64_t N, uint32_t log_n, uint4* d_g, cudaStream_t st);
// witness [n*n] from 13-byte chunks (io.rs:51-59)
cudaError_t launch_unpack_witness(const uint8_t* d_file, uint64_t len, uint64_t total_coeffs, uint4* d_m,
                                  cudaStream_t st);

// ---- folds (k_fold.cu) ----
// out = (l + r * c) mod q over split 64-bit halves (reference FFI fold).
cudaError_t launch_fold_split(const uint64_t* l_lo, const uint64_t* l_hi, const uint64_t* r_lo, const uint64_t* r_hi,
                              uint64_t* o_lo, uint64_t* o_hi, uint64_t len, fq c, cudaStream_t st);
// verifier: both generator folds of one round in one pass (verifier.rs:57-120, 141-178)
cudaError_t launch_fold_gen_round(const uint4* d_src, uint4* d_dst, uint64_t N, uint32_t L, fq x_inv, fq y_inv,
                                  bool vec_stage, bool poly_stage, cudaStream_t st);
// a[i] = a[i] mod q for arbitrary 128-bit words
cudaError_t launch_canon(uint4* d_a, uint64_t n, cudaStream_t st);

// ---- measurement (k_probe.cu) ----
// Issue-rate probe of one integer multiply form (0: 32-bit multiply-add, 1: high
// half of a 32 x 32 product, 2: 32 x 32 -> 64 multiply-add): `blocks` blocks of
// independent chains, int_mul_probe_ops(blocks, iters) operations per launch.
cudaError_t launch_int_mul_probe(int kind, uint32_t* d_sink, int blocks, uint32_t seed, int iters, cudaStream_t st);
uint64_t int_mul_probe_ops(int blocks, int iters);

}  // namespace dm
