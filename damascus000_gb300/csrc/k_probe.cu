// Integer-multiply issue rates of the device, measured: the peaks against which
// the transform's counted multiplies are reported.  The transform spends its
// multiplier on three forms -- 32-bit multiply-add (mul.lo), the high half of a
// 32 x 32 product (mul.hi, the Shoup quotient) and the 32 x 32 -> 64 multiply-add
// of the residue step (mad.wide) -- whose rates differ, so each is timed alone:
// every thread runs eight independent chains of the one form.
#include <cuda_runtime.h>

#include "dm_kernels.cuh"

namespace {

constexpr int kProbeThreads = 512;
constexpr int kProbeChains = 8;

template <int KIND>
__global__ void __launch_bounds__(kProbeThreads) int_mul_probe_kernel(uint32_t* sink, uint32_t seed, int iters) {
    uint32_t a[kProbeChains];
    uint64_t w[kProbeChains];
#pragma unroll
    for (int i = 0; i < kProbeChains; ++i) {
        a[i] = seed * (threadIdx.x + 7u * i + 1u);
        w[i] = a[i];
    }
    const uint32_t m = 0x9E3779B1u ^ seed;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < kProbeChains; ++i) {
            if (KIND == 0) a[i] = a[i] * m + (uint32_t)i;
            if (KIND == 1) a[i] = __umulhi(a[i], m) + a[i];
            if (KIND == 2) w[i] = (uint64_t)(uint32_t)w[i] * m + w[i];
        }
    }
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kProbeChains; ++i) s ^= a[i] ^ (uint32_t)w[i] ^ (uint32_t)(w[i] >> 32);
    if (s == 0x2545F491u) atomicOr(sink, s);  // keeps the chains live; practically never taken
}

}  // namespace

namespace dm {

cudaError_t launch_int_mul_probe(int kind, uint32_t* d_sink, int blocks, uint32_t seed, int iters, cudaStream_t st) {
    if (kind == 0) int_mul_probe_kernel<0><<<blocks, kProbeThreads, 0, st>>>(d_sink, seed, iters);
    else if (kind == 1) int_mul_probe_kernel<1><<<blocks, kProbeThreads, 0, st>>>(d_sink, seed, iters);
    else int_mul_probe_kernel<2><<<blocks, kProbeThreads, 0, st>>>(d_sink, seed, iters);
    return cudaGetLastError();
}

uint64_t int_mul_probe_ops(int blocks, int iters) { return (uint64_t)blocks * kProbeThreads * iters * kProbeChains; }

}  // namespace dm
