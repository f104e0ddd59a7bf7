// Negacyclic NTT over the eight CRT primes, the NTT-domain multiply-accumulate
// of the commitment (src/commitment/sis.rs:146-167) and the CRT recombination
// into Z_q (src/algebra/ntt.rs:372-427).
//
// Forward transform: Cooley-Tukey with the negacyclic twist merged into the
// twiddles (zeta[k] = psi^brv(k), psi a primitive 2n-th root), natural order in,
// bit-reversed evaluation order out: slot j holds a(psi^(2 brv(j) + 1)).  Slots
// 2i and 2i+1 are the evaluations at +w_i and -w_i with w_i = zeta[n/2 + i], so
// the even/odd halves of a polynomial are one butterfly layer away; the prover's
// odd/even stage uses that instead of re-transforming.
// Inverse: Gentleman-Sande with zeta^-1, scaled by n^-1 (and R to cancel the
// Montgomery factor of the pointwise products).
#include <cuda_runtime.h>

#include <vector>

#include "dm_kernels.cuh"
#include "dm_tables.h"

namespace dm {

namespace {

constexpr int kNttThreads = 512;

// In-place forward transforms of nsub sub-arrays of size 2^L in shared memory;
// sub-array t uses prime t & 7, or fixed_prime when it is >= 0.
DM_D void smem_ntt_fwd(uint32_t* a, uint32_t nsub, uint32_t L, const PrimeConsts& pc,
                       const uint32_t* __restrict__ zeta, int fixed_prime = -1) {
    if (L == 0) return;
    const uint32_t half = 1u << (L - 1);
    const uint32_t total = nsub * half;
    for (uint32_t st = 0; st < L; ++st) {
        const uint32_t lg_len = L - 1 - st;
        const uint32_t len = 1u << lg_len;
        for (uint32_t B = threadIdx.x; B < total; B += blockDim.x) {
            const uint32_t t = B >> (L - 1), b = B & (half - 1);
            const uint32_t pi = fixed_prime >= 0 ? (uint32_t)fixed_prime : (t & 7u);
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
DM_D void smem_ntt_inv(uint32_t* a, uint32_t nsub, uint32_t L, const PrimeConsts& pc,
                       const uint32_t* __restrict__ zinv, int fixed_prime = -1) {
    if (L == 0) return;
    const uint32_t half = 1u << (L - 1);
    const uint32_t total = nsub * half;
    for (uint32_t st = 0; st < L; ++st) {
        const uint32_t len = 1u << st;
        const uint32_t m = 1u << (L - 1 - st);
        for (uint32_t B = threadIdx.x; B < total; B += blockDim.x) {
            const uint32_t t = B >> (L - 1), b = B & (half - 1);
            const uint32_t pi = fixed_prime >= 0 ? (uint32_t)fixed_prime : (t & 7u);
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

// coef [npolys][s] -> res [npolys][8][s]; each CTA transforms ppc polynomials.
__global__ void __launch_bounds__(kNttThreads) ntt_fwd_kernel(const uint4* __restrict__ coef,
                                                              uint32_t* __restrict__ res, uint64_t npolys,
                                                              uint32_t L, uint32_t ppc, PrimeConsts pc,
                                                              const uint32_t* __restrict__ zeta) {
    extern __shared__ uint32_t sm[];
    const uint32_t s = 1u << L;
    const uint64_t poly0 = (uint64_t)blockIdx.x * ppc;
    if (poly0 >= npolys) return;
    const uint32_t npc = (uint32_t)(npolys - poly0 < (uint64_t)ppc ? npolys - poly0 : (uint64_t)ppc);
    for (uint32_t e = threadIdx.x; e < (npc << L); e += blockDim.x) {
        const uint32_t lp = e >> L, c = e & (s - 1);
        const uint4 v = coef[(poly0 << L) + e];
        const fq x{{v.x, v.y, v.z, v.w}};
#pragma unroll
        for (int pi = 0; pi < kPrimes; ++pi) sm[((lp * kPrimes + pi) << L) + c] = residue(x, pc, pi);
    }
    __syncthreads();
    smem_ntt_fwd(sm, npc * kPrimes, L, pc, zeta);
    uint32_t* out = res + ((poly0 * kPrimes) << L);
    for (uint32_t e = threadIdx.x; e < ((npc * kPrimes) << L); e += blockDim.x) out[e] = sm[e];
}

// Plain MAC.  grid (ceil(s/bx), 64, njobs*parts).
struct MacJobs {
    MacJob j[4];
};
__global__ void mac_kernel(const uint32_t* __restrict__ G, const uint32_t* __restrict__ M, uint32_t L, MacJobs jobs,
                           uint32_t parts, PrimeConsts pc, uint32_t* __restrict__ partials) {
    const uint32_t s = 1u << L;
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= s) return;
    const uint32_t kp = blockIdx.y, k = kp >> 3, pi = kp & 7u;
    const uint32_t job = blockIdx.z / parts, part = blockIdx.z % parts;
    const MacJob J = jobs.j[job];
    const uint32_t i0 = (uint32_t)((uint64_t)J.count * part / parts);
    const uint32_t i1 = (uint32_t)((uint64_t)J.count * (part + 1) / parts);
    const uint32_t p = pc.p[pi], pv = pc.pinv[pi];
    uint64_t acc = 0;
    for (uint32_t i = i0; i < i1; ++i) {
        const uint64_t gi = (uint64_t)(J.g_base + i) * kRank + k;
        const uint32_t gv = G[((gi * kPrimes + pi) << L) + slot];
        const uint32_t mv = M[(((uint64_t)(J.m_base + i) * kPrimes + pi) << L) + slot];
        acc += mont_mul(gv, mv, p, pv);
    }
    partials[(((uint64_t)blockIdx.z * 64 + kp) << L) + slot] = reduce_u64(acc, p, pv, pc.r1[pi], pc.r2[pi]);
}

// Split MAC: thread per slot pair (2i, 2i+1) of ring size 2^L.
__global__ void mac_split_kernel(const uint32_t* __restrict__ G, const uint32_t* __restrict__ M, uint32_t L,
                                 uint32_t count, uint32_t parts, PrimeConsts pc, uint32_t* __restrict__ chk,
                                 uint32_t* __restrict__ lp, uint32_t* __restrict__ rp) {
    const uint32_t h = 1u << (L - 1);
    const uint32_t i2 = blockIdx.x * blockDim.x + threadIdx.x;
    if (i2 >= h) return;
    const uint32_t kp = blockIdx.y, k = kp >> 3, pi = kp & 7u;
    const uint32_t part = blockIdx.z;
    const uint32_t c0 = (uint32_t)((uint64_t)count * part / parts);
    const uint32_t c1 = (uint32_t)((uint64_t)count * (part + 1) / parts);
    const uint32_t p = pc.p[pi], pv = pc.pinv[pi];
    uint64_t a0 = 0, a1 = 0, al = 0, ar = 0;
    for (uint32_t i = c0; i < c1; ++i) {
        const uint64_t gi = (uint64_t)i * kRank + k;
        const uint2 gv = *reinterpret_cast<const uint2*>(G + ((gi * kPrimes + pi) << L) + 2 * i2);
        const uint2 mv = *reinterpret_cast<const uint2*>(M + (((uint64_t)i * kPrimes + pi) << L) + 2 * i2);
        a0 += mont_mul(gv.x, mv.x, p, pv);
        a1 += mont_mul(gv.y, mv.y, p, pv);
        al += mont_mul(sub_mod(gv.x, gv.y, p), add_mod(mv.x, mv.y, p), p, pv);
        ar += mont_mul(add_mod(gv.x, gv.y, p), sub_mod(mv.x, mv.y, p), p, pv);
    }
    const uint32_t r1 = pc.r1[pi], r2 = pc.r2[pi];
    uint2 c;
    c.x = reduce_u64(a0, p, pv, r1, r2);
    c.y = reduce_u64(a1, p, pv, r1, r2);
    *reinterpret_cast<uint2*>(chk + (((uint64_t)part * 64 + kp) << L) + 2 * i2) = c;
    lp[(((uint64_t)part * 64 + kp) << (L - 1)) + i2] = reduce_u64(al, p, pv, r1, r2);
    rp[(((uint64_t)part * 64 + kp) << (L - 1)) + i2] = reduce_u64(ar, p, pv, r1, r2);
}

struct FinishJobs {
    FinishJob j[4];
};
struct InttScale {
    uint32_t ninv_r2[kPrimes][kLogMaxRing + 1];
    uint32_t ninv4_r2[kPrimes][kLogMaxRing + 1];
};
// grid (8 coords, njobs); smem 8 * 2^L words.
__global__ void __launch_bounds__(kNttThreads) finish_kernel(FinishJobs jobs, PrimeConsts pc, CrtConsts cc,
                                                             InttScale sc, const uint32_t* __restrict__ zeta,
                                                             const uint32_t* __restrict__ zinv) {
    extern __shared__ uint32_t sm[];
    const FinishJob J = jobs.j[blockIdx.y];
    const uint32_t k = blockIdx.x;
    const uint32_t L = J.L, s = 1u << L;
    for (uint32_t e = threadIdx.x; e < (kPrimes << L); e += blockDim.x) {
        const uint32_t pi = e >> L, c = e & (s - 1);
        const uint32_t p = pc.p[pi], pv = pc.pinv[pi];
        uint32_t acc = 0;
        for (uint32_t part = 0; part < J.parts; ++part)
            acc = add_mod(acc, J.partials[(((uint64_t)part * 64 + k * 8 + pi) << L) + c], p);
        if (J.mode == kFinishSplitL) acc = mont_mul(acc, __ldg(zeta + pi * kMaxRing + s + c), p, pv);
        if (J.mode == kFinishSplitR) acc = mont_mul(acc, __ldg(zinv + pi * kMaxRing + s + c), p, pv);
        sm[e] = acc;
    }
    __syncthreads();
    smem_ntt_inv(sm, kPrimes, L, pc, zinv);
    for (uint32_t c = threadIdx.x; c < s; c += blockDim.x) {
        uint32_t r[kPrimes];
#pragma unroll
        for (int pi = 0; pi < kPrimes; ++pi) {
            const uint32_t f = (J.mode == kFinishPlain) ? sc.ninv_r2[pi][L] : sc.ninv4_r2[pi][L];
            r[pi] = mont_mul(sm[(pi << L) + c], f, pc.p[pi], pc.pinv[pi]);
        }
        const fq v = crt_to_fq_fast(r, pc, cc);
        J.out[((uint64_t)k << L) + c] = make_uint4(v.w[0], v.w[1], v.w[2], v.w[3]);
    }
}

// Pointwise products of transformed pairs, inverse transform and CRT: one CTA per pair.
__global__ void __launch_bounds__(kNttThreads) ring_mul_kernel(const uint32_t* __restrict__ A,
                                                               const uint32_t* __restrict__ B,
                                                               uint4* __restrict__ out, uint32_t L, PrimeConsts pc,
                                                               CrtConsts cc, InttScale sc,
                                                               const uint32_t* __restrict__ zinv) {
    extern __shared__ uint32_t sm[];
    const uint32_t s = 1u << L;
    const uint64_t pair = blockIdx.x;
    const uint32_t* a = A + ((pair * kPrimes) << L);
    const uint32_t* b = B + ((pair * kPrimes) << L);
    for (uint32_t e = threadIdx.x; e < (kPrimes << L); e += blockDim.x) {
        const uint32_t pi = e >> L;
        sm[e] = mont_mul(a[e], b[e], pc.p[pi], pc.pinv[pi]);
    }
    __syncthreads();
    smem_ntt_inv(sm, kPrimes, L, pc, zinv);
    for (uint32_t c = threadIdx.x; c < s; c += blockDim.x) {
        uint32_t r[kPrimes];
#pragma unroll
        for (int pi = 0; pi < kPrimes; ++pi) r[pi] = mont_mul(sm[(pi << L) + c], sc.ninv_r2[pi][L], pc.p[pi], pc.pinv[pi]);
        const fq v = crt_to_fq_fast(r, pc, cc);
        out[(pair << L) + c] = make_uint4(v.w[0], v.w[1], v.w[2], v.w[3]);
    }
}

// Length-n cyclic convolution per prime (the reference FFI's contract,
// cuda/ntt_kernel.cu:106-293): the linear product by a negacyclic transform of
// size 2n (no wrap-around), folded as c[j] = lin[j] + lin[j + n].  CTA per prime.
__global__ void __launch_bounds__(kNttThreads) cyclic_conv_kernel(const uint32_t* __restrict__ A,
                                                                  const uint32_t* __restrict__ B,
                                                                  uint32_t* __restrict__ out, uint32_t Ln,
                                                                  PrimeConsts pc, InttScale sc,
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
        const uint32_t lo = mont_mul(a[e], sc.ninv_r2[pi][L], p, pv);
        const uint32_t hi = mont_mul(a[e + n], sc.ninv_r2[pi][L], p, pv);
        out[(size_t)pi * n + e] = add_mod(lo, hi, p);
    }
}

InttScale scale_of(const DeviceTables& T) {
    InttScale s;
    for (int i = 0; i < kPrimes; ++i)
        for (int L = 0; L <= kLogMaxRing; ++L) {
            s.ninv_r2[i][L] = T.ninv_r2[i][L];
            s.ninv4_r2[i][L] = T.ninv4_r2[i][L];
        }
    return s;
}

cudaError_t smem_opt_in(const void* fn, size_t bytes) {
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

cudaError_t upload_tables(DeviceTables* out) {
    const HostTables& H = host_tables();
    out->pc = H.pc;
    out->cc = H.cc;
    for (int i = 0; i < kPrimes; ++i)
        for (int L = 0; L <= kLogMaxRing; ++L) {
            out->ninv_r2[i][L] = H.ninv_r2[i][L];
            out->ninv4_r2[i][L] = H.ninv4_r2[i][L];
        }
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
    const size_t max_smem = (size_t)kPrimes * (1u << kLogMaxProverRing) * sizeof(uint32_t);
    if ((e = smem_opt_in((const void*)ntt_fwd_kernel, max_smem)) != cudaSuccess) return e;
    if ((e = smem_opt_in((const void*)finish_kernel, max_smem)) != cudaSuccess) return e;
    if ((e = smem_opt_in((const void*)ring_mul_kernel, max_smem)) != cudaSuccess) return e;
    return cudaSuccess;
}

cudaError_t launch_ntt_fwd(const DeviceTables& T, const uint4* d_coef, uint32_t* d_res, uint64_t npolys, uint32_t L,
                           cudaStream_t st) {
    if (npolys == 0) return cudaSuccess;
    if (L > (uint32_t)kLogMaxProverRing) return cudaErrorInvalidValue;
    const uint32_t s = 1u << L;
    const uint32_t ppc = s >= 512 ? 1u : 512u / s;
    const uint64_t grid = (npolys + ppc - 1) / ppc;
    const size_t smem = (size_t)ppc * kPrimes * s * sizeof(uint32_t);
    ntt_fwd_kernel<<<(unsigned)grid, kNttThreads, smem, st>>>(d_coef, d_res, npolys, L, ppc, T.pc, T.zeta);
    return cudaGetLastError();
}

cudaError_t launch_mac(const DeviceTables& T, const uint32_t* d_G, const uint32_t* d_M, uint32_t L,
                       const MacJob* jobs, int njobs, uint32_t parts, uint32_t* d_partials, cudaStream_t st) {
    if (njobs <= 0 || njobs > 4 || parts == 0) return cudaErrorInvalidValue;
    MacJobs J{};
    for (int i = 0; i < njobs; ++i) J.j[i] = jobs[i];
    const uint32_t s = 1u << L;
    const uint32_t bx = s < 128 ? s : 128;
    dim3 grid((s + bx - 1) / bx, 64, (unsigned)(njobs * parts));
    mac_kernel<<<grid, bx, 0, st>>>(d_G, d_M, L, J, parts, T.pc, d_partials);
    return cudaGetLastError();
}

cudaError_t launch_mac_split(const DeviceTables& T, const uint32_t* d_G, const uint32_t* d_M, uint32_t L,
                             uint32_t count, uint32_t parts, uint32_t* d_chk, uint32_t* d_lp, uint32_t* d_rp,
                             cudaStream_t st) {
    if (L == 0 || parts == 0) return cudaErrorInvalidValue;
    const uint32_t h = 1u << (L - 1);
    const uint32_t bx = h < 128 ? h : 128;
    dim3 grid((h + bx - 1) / bx, 64, parts);
    mac_split_kernel<<<grid, bx, 0, st>>>(d_G, d_M, L, count, parts, T.pc, d_chk, d_lp, d_rp);
    return cudaGetLastError();
}

cudaError_t launch_finish(const DeviceTables& T, const FinishJob* jobs, int njobs, cudaStream_t st) {
    if (njobs <= 0 || njobs > 4) return cudaErrorInvalidValue;
    FinishJobs J{};
    uint32_t maxL = 0;
    for (int i = 0; i < njobs; ++i) {
        J.j[i] = jobs[i];
        maxL = jobs[i].L > maxL ? jobs[i].L : maxL;
    }
    const size_t smem = (size_t)kPrimes * (1u << maxL) * sizeof(uint32_t);
    finish_kernel<<<dim3(kRank, njobs), kNttThreads, smem, st>>>(J, T.pc, T.cc, scale_of(T), T.zeta, T.zinv);
    return cudaGetLastError();
}

cudaError_t launch_cyclic_conv(const DeviceTables& T, const uint32_t* d_a, const uint32_t* d_b, uint32_t* d_out,
                               uint32_t Ln, cudaStream_t st) {
    if (Ln + 1 > (uint32_t)kLogMaxRing) return cudaErrorInvalidValue;
    const size_t smem = 2ull * 2 * (1u << Ln) * sizeof(uint32_t);
    cudaError_t e = smem_opt_in((const void*)cyclic_conv_kernel, smem < 48 * 1024 ? 48 * 1024 : smem);
    if (e != cudaSuccess) return e;
    cyclic_conv_kernel<<<kPrimes, kNttThreads, smem, st>>>(d_a, d_b, d_out, Ln, T.pc, scale_of(T), T.zeta, T.zinv);
    return cudaGetLastError();
}

cudaError_t launch_ring_mul(const DeviceTables& T, const uint32_t* d_A_res, const uint32_t* d_B_res, uint4* d_out,
                            uint64_t count, uint32_t L, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    const size_t smem = (size_t)kPrimes * (1u << L) * sizeof(uint32_t);
    ring_mul_kernel<<<(unsigned)count, kNttThreads, smem, st>>>(d_A_res, d_B_res, d_out, L, T.pc, T.cc, scale_of(T),
                                                                T.zinv);
    return cudaGetLastError();
}

}  // namespace dm
