// The reference-compatible FFI convolution (damascus_cuda_ntt_batch): per-prime
// length-n cyclic convolutions of residue vectors modulo the reference's eight
// CRT primes, which the caller passes (src/utils/gpu.rs:69-93, contract of
// cuda/ntt_kernel.cu:106-293).  Shared-memory transforms with Montgomery
// products; this path is off the prover's hot path.
#include <cuda_runtime.h>

#include "dm_tables.h"

namespace dm {

namespace {

constexpr int kNttThreads = 512;

// In-place forward transforms of nsub sub-arrays of size 2^L in shared memory;
// sub-array t uses prime t mod 8, or fixed_prime when it is >= 0.
DM_D void smem_ntt_fwd(uint32_t* a, uint32_t nsub, uint32_t L, const RefPrimeConsts& pc,
                       const uint32_t* __restrict__ zeta, int fixed_prime = -1) {
    if (L == 0) return;
    const uint32_t half = 1u << (L - 1);
    const uint32_t total = nsub * half;
    for (uint32_t st = 0; st < L; ++st) {
        const uint32_t lg_len = L - 1 - st;
        const uint32_t len = 1u << lg_len;
        for (uint32_t B = threadIdx.x; B < total; B += blockDim.x) {
            const uint32_t t = B >> (L - 1), b = B & (half - 1);
            const uint32_t pi = fixed_prime >= 0 ? (uint32_t)fixed_prime : (t % kRefPrimes);
            const uint32_t g = b >> lg_len;
            const uint32_t j = (g << (lg_len + 1)) | (b & (len - 1));
            const uint32_t z = __ldg(zeta + pi * kMaxRing + (1u << st) + g);
            const uint32_t p = pc.p[pi];
            uint32_t* x = a + (t << L);
            const uint32_t v = mont_mul(x[j + len], z, p, pc.pinv[pi]);
            const uint32_t u = x[j];
            x[j] = add_mod(u, v, p);
            x[j + len] = sub_mod(u, v, p);
        }
        __syncthreads();
    }
}

// In-place inverse transforms (bit-reversed in, natural out), without the final scale.
DM_D void smem_ntt_inv(uint32_t* a, uint32_t nsub, uint32_t L, const RefPrimeConsts& pc,
                       const uint32_t* __restrict__ zinv, int fixed_prime = -1) {
    if (L == 0) return;
    const uint32_t half = 1u << (L - 1);
    const uint32_t total = nsub * half;
    for (uint32_t st = 0; st < L; ++st) {
        const uint32_t len = 1u << st;
        const uint32_t m = 1u << (L - 1 - st);
        for (uint32_t B = threadIdx.x; B < total; B += blockDim.x) {
            const uint32_t t = B >> (L - 1), b = B & (half - 1);
            const uint32_t pi = fixed_prime >= 0 ? (uint32_t)fixed_prime : (t % kRefPrimes);
            const uint32_t g = b >> st;
            const uint32_t j = (g << (st + 1)) | (b & (len - 1));
            const uint32_t z = __ldg(zinv + pi * kMaxRing + m + g);
            const uint32_t p = pc.p[pi];
            uint32_t* x = a + (t << L);
            const uint32_t u = x[j], v = x[j + len];
            x[j] = add_mod(u, v, p);
            x[j + len] = mont_mul(sub_mod(u, v, p), z, p, pc.pinv[pi]);
        }
        __syncthreads();
    }
}

// Length-n cyclic convolution per prime (the reference FFI's contract,
// cuda/ntt_kernel.cu:106-293): the linear product by a negacyclic transform of
// size 2n (no wrap-around), folded as c[j] = lin[j] + lin[j + n].  CTA per prime.
__global__ void __launch_bounds__(kNttThreads) cyclic_conv_kernel(const uint32_t* __restrict__ A,
                                                                  const uint32_t* __restrict__ B,
                                                                  uint32_t* __restrict__ out, uint32_t Ln,
                                                                  RefPrimeConsts pc,
                                                                  const uint32_t* __restrict__ zeta,
                                                                  const uint32_t* __restrict__ zinv) {
    extern __shared__ uint32_t sm[];
    const int pi = blockIdx.x;
    const uint32_t n = 1u << Ln, L = Ln + 1, s = 2u * n;
    const uint32_t p = pc.p[pi], pv = pc.pinv[pi];
    uint32_t* a = sm;
    uint32_t* b = sm + s;
    for (uint32_t e = threadIdx.x; e < s; e += blockDim.x) {
        a[e] = e < n ? A[(size_t)pi * n + e] : 0u;
        b[e] = e < n ? B[(size_t)pi * n + e] : 0u;
    }
    __syncthreads();
    smem_ntt_fwd(sm, 2, L, pc, zeta, pi);
    for (uint32_t e = threadIdx.x; e < s; e += blockDim.x) a[e] = mont_mul(a[e], b[e], p, pv);
    __syncthreads();
    smem_ntt_inv(a, 1, L, pc, zinv, pi);
    for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
        const uint32_t lo = mont_mul(a[e], pc.ninv_r2[pi][L], p, pv);
        const uint32_t hi = mont_mul(a[e + n], pc.ninv_r2[pi][L], p, pv);
        out[(size_t)pi * n + e] = add_mod(lo, hi, p);
    }
}

cudaError_t smem_opt_in(const void* fn, size_t bytes) {
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

cudaError_t upload_ref_tables(RefDeviceTables* out) {
    const RefHostTables& H = ref_host_tables();
    out->pc = H.pc;
    uint32_t *z = nullptr, *zi = nullptr;
    const size_t bytes = sizeof(uint32_t) * H.zeta.size();
    cudaError_t e = cudaMalloc(&z, bytes);
    if (e != cudaSuccess) return e;
    e = cudaMalloc(&zi, bytes);
    if (e != cudaSuccess) {
        cudaFree(z);
        return e;
    }
    e = cudaMemcpy(z, H.zeta.data(), bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(zi, H.zinv.data(), bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(z);
        cudaFree(zi);
        return e;
    }
    out->zeta = z;
    out->zinv = zi;
    return cudaSuccess;
}

void free_ref_tables(RefDeviceTables* t) {
    if (t->zeta) cudaFree(const_cast<uint32_t*>(t->zeta));
    if (t->zinv) cudaFree(const_cast<uint32_t*>(t->zinv));
    t->zeta = t->zinv = nullptr;
}

cudaError_t launch_cyclic_conv(const RefDeviceTables& T, const uint32_t* d_a, const uint32_t* d_b, uint32_t* d_out,
                               uint32_t Ln, cudaStream_t st) {
    if (Ln + 1 > (uint32_t)kLogMaxRing) return cudaErrorInvalidValue;
    const size_t smem = (size_t)2 * (2u << Ln) * sizeof(uint32_t);
    cudaError_t e = smem_opt_in((const void*)cyclic_conv_kernel, smem < 48 * 1024 ? 48 * 1024 : smem);
    if (e != cudaSuccess) return e;
    cyclic_conv_kernel<<<kRefPrimes, kNttThreads, smem, st>>>(d_a, d_b, d_out, Ln, T.pc, T.zeta, T.zinv);
    return cudaGetLastError();
}

}  // namespace dm
