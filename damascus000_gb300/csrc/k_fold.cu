// Coefficient-domain kernels outside the prover's job lists: the verifier's
// generator folds (src/protocol/verifier.rs:57-120, 141-178), canonicalisation of
// caller-provided 128-bit words, and the reference FFI's split-word fold
// (src/protocol/prover.rs:343-362 through src/utils/gpu.rs:69-93).
#include <cuda_runtime.h>

#include "dm_kernels.cuh"

namespace dm {

namespace {

DM_D fq ld(const uint4* p, uint64_t i) {
    const uint4 v = p[i];
    return fq{{v.x, v.y, v.z, v.w}};
}
DM_D void st(uint4* p, uint64_t i, const fq& a) { p[i] = make_uint4(a.w[0], a.w[1], a.w[2], a.w[3]); }

unsigned grid_for(uint64_t n, unsigned bx = 256) {
    const uint64_t b = (n + bx - 1) / bx;
    return (unsigned)(b < 152ull * 64 ? (b ? b : 1) : 152ull * 64);
}

#define GRID_STRIDE(i, n) \
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (uint64_t)gridDim.x * blockDim.x)

// acc += a * b over eight limbs (a, b below 2^112; the caller keeps the sum below 2^256).
__device__ __forceinline__ void acc_mul(uint32_t acc[8], const fq& a, const fq& b) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        uint64_t c = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            c += (uint64_t)a.w[i] * b.w[j] + acc[i + j];
            acc[i + j] = (uint32_t)c;
            c >>= 32;
        }
#pragma unroll
        for (int k = i + 4; k < 8; ++k) {
            c += acc[k];
            acc[k] = (uint32_t)c;
            c >>= 32;
        }
    }
}

// Generator folds of one verifier round: vector stage g' = g_L + x^-1 g_R, then the
// poly stage g'' = g'_e + y^-1 X g'_o.  dst is [N'][8][n'] with N' = N/2 (or N) and
// n' = n/2 (or n).  With both stages an output is s0 + x^-1 s1 + y' s2 + x^-1 y' s3
// (s0, s1 the even coefficient of both halves, s2, s3 the odd one before it, and
// y' = -y^-1 for the coefficient that wraps around X^n = -1): the three products
// of canonical values are summed unreduced (below 2^226) and reduced once, the
// same canonical value as folding the stages one after the other.
__global__ void fold_gen_round_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst, uint64_t N,
                                      uint32_t L, fq x_inv, fq y_inv, fq xy_inv, fq neg_y_inv, fq neg_xy_inv,
                                      int vec_stage, int poly_stage) {
    const uint64_t Nout = vec_stage ? N / 2 : N;
    const uint32_t Lout = poly_stage ? L - 1 : L;
    const uint64_t total = Nout * kRank << Lout;
    const uint64_t half_elems = (N / 2) * kRank << L;
    GRID_STRIDE(e, total) {
        const uint64_t row = e >> Lout;  // (i, k)
        const uint32_t j = (uint32_t)(e & ((1u << Lout) - 1));
        const uint64_t base = row << L;
        auto gval = [&](uint32_t t) -> fq {
            fq a = ld(src, base + t);
            if (vec_stage) a = fq_fma(a, x_inv, ld(src, base + t + half_elems));
            return a;
        };
        fq out;
        if (poly_stage && vec_stage) {
            const uint32_t n = 1u << L;
            const uint32_t o = j == 0 ? n - 1 : 2 * j - 1;
            const fq s0 = ld(src, base + 2 * j), s1 = ld(src, base + 2 * j + half_elems);
            const fq s2 = ld(src, base + o), s3 = ld(src, base + o + half_elems);
            uint32_t acc[8] = {s0.w[0], s0.w[1], s0.w[2], s0.w[3], 0u, 0u, 0u, 0u};
            acc_mul(acc, x_inv, s1);
            acc_mul(acc, j == 0 ? neg_y_inv : y_inv, s2);
            acc_mul(acc, j == 0 ? neg_xy_inv : xy_inv, s3);
            out = fq_reduce8(acc);
        } else if (poly_stage) {
            const uint32_t n = 1u << L;
            const fq odd = j == 0 ? fq_neg(gval(n - 1)) : gval(2 * j - 1);
            out = fq_fma(gval(2 * j), y_inv, odd);
        } else {
            out = gval(j);
        }
        st(dst, e, out);
    }
}

// Reference FFI fold on split halves (cuda/fold_kernel.cu:189-206); inputs are
// reduced mod q first so any 128-bit words are accepted.
__global__ void fold_split_kernel(const uint64_t* __restrict__ l_lo, const uint64_t* __restrict__ l_hi,
                                  const uint64_t* __restrict__ r_lo, const uint64_t* __restrict__ r_hi,
                                  uint64_t* __restrict__ o_lo, uint64_t* __restrict__ o_hi, uint64_t len, fq c) {
    GRID_STRIDE(e, len) {
        uint32_t a8[8] = {(uint32_t)l_lo[e], (uint32_t)(l_lo[e] >> 32), (uint32_t)l_hi[e], (uint32_t)(l_hi[e] >> 32),
                          0, 0, 0, 0};
        uint32_t b8[8] = {(uint32_t)r_lo[e], (uint32_t)(r_lo[e] >> 32), (uint32_t)r_hi[e], (uint32_t)(r_hi[e] >> 32),
                          0, 0, 0, 0};
        const fq v = fq_fma(fq_reduce8(a8), c, fq_reduce8(b8));
        o_lo[e] = (uint64_t)v.w[0] | ((uint64_t)v.w[1] << 32);
        o_hi[e] = (uint64_t)v.w[2] | ((uint64_t)v.w[3] << 32);
    }
}

__global__ void canon_kernel(uint4* __restrict__ a, uint64_t n) {
    GRID_STRIDE(e, n) {
        const uint4 v = a[e];
        uint32_t r[8] = {v.x, v.y, v.z, v.w, 0, 0, 0, 0};
        st(a, e, fq_reduce8(r));
    }
}

}  // namespace

cudaError_t launch_canon(uint4* d_a, uint64_t n, cudaStream_t s) {
    if (!n) return cudaSuccess;
    canon_kernel<<<grid_for(n), 256, 0, s>>>(d_a, n);
    return cudaGetLastError();
}

cudaError_t launch_fold_split(const uint64_t* l_lo, const uint64_t* l_hi, const uint64_t* r_lo, const uint64_t* r_hi,
                              uint64_t* o_lo, uint64_t* o_hi, uint64_t len, fq c, cudaStream_t s) {
    if (!len) return cudaSuccess;
    fold_split_kernel<<<grid_for(len), 256, 0, s>>>(l_lo, l_hi, r_lo, r_hi, o_lo, o_hi, len, c);
    return cudaGetLastError();
}

cudaError_t launch_fold_gen_round(const uint4* d_src, uint4* d_dst, uint64_t N, uint32_t L, fq x_inv, fq y_inv,
                                  bool vec_stage, bool poly_stage, cudaStream_t s) {
    const uint64_t total = (vec_stage ? N / 2 : N) * kRank << (poly_stage ? L - 1 : L);
    if (!total) return cudaSuccess;
    const fq xy_inv = fq_mul(x_inv, y_inv);
    fold_gen_round_kernel<<<grid_for(total), 256, 0, s>>>(d_src, d_dst, N, L, x_inv, y_inv, xy_inv, fq_neg(y_inv),
                                                           fq_neg(xy_inv), vec_stage ? 1 : 0, poly_stage ? 1 : 0);
    return cudaGetLastError();
}

}  // namespace dm
