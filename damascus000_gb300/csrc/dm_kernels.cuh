// Kernel launch interfaces.  All device buffers use these layouts:
//   coefficient domain : uint4 per Z_q element (16-byte LE), arrays [poly][coeff]
//   generators         : [vec][coord][coeff]  (src/commitment/sis.rs:212-229 order)
//   NTT domain         : uint32 residues [poly][prime][slot], slot = bit-reversed
//                        evaluation index of the negacyclic transform
//   MAC partial sums   : uint32 [part][coord*8 + prime][slot]
#pragma once

#include <cuda_runtime.h>

#include "dm_field.cuh"

namespace dm {

struct DeviceTables {
    PrimeConsts pc;
    CrtConsts cc;
    uint32_t ninv_r2[kPrimes][kLogMaxRing + 1];
    uint32_t ninv4_r2[kPrimes][kLogMaxRing + 1];
    const uint32_t* zeta;  // device [prime][kMaxRing]
    const uint32_t* zinv;
    const uint32_t* zetap = nullptr;  // zeta * p^-1 mod 2^32
    const uint32_t* zinvp = nullptr;
};

// Uploads the tables to the current device (called once per device).
cudaError_t upload_tables(DeviceTables* out);

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

// ---- NTT / MAC / CRT (k_ntt.cu) ----
// coef [npolys][2^L] -> residues [npolys][8][2^L]
cudaError_t launch_ntt_fwd(const DeviceTables& T, const uint4* d_coef, uint32_t* d_res, uint64_t npolys,
                           uint32_t L, cudaStream_t st);

struct MacJob {
    uint32_t g_base;  // first generator vector index
    uint32_t m_base;  // first witness vector index
    uint32_t count;   // number of columns summed
};
// Plain MAC: for each job, partials[job][part][k*8+p][slot] = sum_i G[g_base+i][k][p][slot] * M[m_base+i][p][slot]
cudaError_t launch_mac(const DeviceTables& T, const uint32_t* d_G, const uint32_t* d_M, uint32_t L,
                       const MacJob* jobs, int njobs, uint32_t parts, uint32_t* d_partials, cudaStream_t st);
// Split MAC over ring size 2^L (L >= 1): check (2^L slots) and the even/odd cross terms
// Lp = sum (X g_o) m_e and Rp = sum g_e m_o at 2^(L-1).  Partials: chk [parts][64][2^L],
// then lp [parts][64][2^(L-1)], then rp [parts][64][2^(L-1)].
cudaError_t launch_mac_split(const DeviceTables& T, const uint32_t* d_G, const uint32_t* d_M, uint32_t L,
                             uint32_t count, uint32_t parts, uint32_t* d_chk, uint32_t* d_lp, uint32_t* d_rp,
                             cudaStream_t st);

enum FinishMode : uint32_t { kFinishPlain = 0, kFinishSplitL = 1, kFinishSplitR = 2 };
struct FinishJob {
    const uint32_t* partials;
    uint32_t parts;
    uint32_t L;     // output ring size 2^L
    uint32_t mode;  // FinishMode
    uint4* out;     // [8][2^L]
};
// Sums the partials, inverse-transforms and recombines by CRT into Z_q.
cudaError_t launch_finish(const DeviceTables& T, const FinishJob* jobs, int njobs, cudaStream_t st);

// Per-prime length-2^Ln cyclic convolution of residue vectors [8][2^Ln] (Ln <= 12).
cudaError_t launch_cyclic_conv(const DeviceTables& T, const uint32_t* d_a, const uint32_t* d_b, uint32_t* d_out,
                               uint32_t Ln, cudaStream_t st);
// out = (l + r * c) mod q over split 64-bit halves (reference FFI fold).
cudaError_t launch_fold_split(const uint64_t* l_lo, const uint64_t* l_hi, const uint64_t* r_lo, const uint64_t* r_hi,
                              uint64_t* o_lo, uint64_t* o_hi, uint64_t len, fq c, cudaStream_t st);
// out[i] = a[i] * b[i] in R_q for count pairs of degree 2^L (coefficient domain).
cudaError_t launch_ring_mul(const DeviceTables& T, const uint32_t* d_A_res, const uint32_t* d_B_res, uint4* d_out,
                            uint64_t count, uint32_t L, cudaStream_t st);

// ---- folds and commitment algebra (k_fold.cu) ----
// dst[e] = src[e] + c * src[e + half]     (vector fold, prover.rs:332-395)
cudaError_t launch_fold_vec(const uint4* d_src, uint4* d_dst, uint64_t half, fq c, cudaStream_t st);
// dst[poly][j] = src[poly][2j] + c * odd_j, odd_j = src[2j+1], or with shift (X * g_odd):
// odd_0 = -src[s-1], odd_j = src[2j-1]    (prover.rs:397-457)
cudaError_t launch_fold_poly(const uint4* d_src, uint4* d_dst, uint64_t npolys, uint32_t L_out, fq c, bool shift,
                             cudaStream_t st);
// verifier: both generator folds of one round in one pass (verifier.rs:57-120, 141-178)
cudaError_t launch_fold_gen_round(const uint4* d_src, uint4* d_dst, uint64_t N, uint32_t L, fq x_inv, fq y_inv,
                                  bool vec_stage, bool poly_stage, cudaStream_t st);
// out = c + a*l + b*r (elementwise over n)
cudaError_t launch_combine(const uint4* d_c, const uint4* d_l, const uint4* d_r, fq a, fq b, uint4* d_out, uint64_t n,
                           cudaStream_t st);
// out[k][j] = ct[k][2j] + a*lp[k][j] + b*rp[k][j], j < 2^Lh
cudaError_t launch_combine_even(const uint4* d_ct, const uint4* d_lp, const uint4* d_rp, fq a, fq b, uint4* d_out,
                                uint32_t Lh, cudaStream_t st);
// a[i] = a[i] mod q for arbitrary 128-bit words
cudaError_t launch_canon(uint4* d_a, uint64_t n, cudaStream_t st);
// *flag |= (a != b) over n elements
cudaError_t launch_compare(const uint4* d_a, const uint4* d_b, uint64_t n, uint32_t* d_flag, cudaStream_t st);

}  // namespace dm
