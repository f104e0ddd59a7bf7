// BLAKE3 on the device: the file id (src/utils/io.rs:33), the generator
// expansion (src/commitment/sis.rs:212-245), and the 13-byte witness packing
// (src/utils/io.rs:51-59, field.rs:65-71).
#include <cuda_runtime.h>

#include "dm_blake3.cuh"
#include "dm_jobs.cuh"
#include "dm_kernels.cuh"

namespace dm {

namespace {

__global__ void unpack_kernel(const uint8_t* __restrict__ file, uint64_t len, uint64_t total,
                              uint4* __restrict__ m) {
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < total;
         j += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t w[4] = {0, 0, 0, 0};
        const uint64_t off = j * kBytesPerCoeff;
        if (off < len) {
            const uint64_t n = len - off < (uint64_t)kBytesPerCoeff ? len - off : (uint64_t)kBytesPerCoeff;
            for (uint32_t b = 0; b < n; ++b) w[b >> 2] |= (uint32_t)file[off + b] << (8 * (b & 3));
        }
        m[j] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// Loads up to 64 bytes of a block as 16 little-endian words (zero padded).
DM_D void load_block(const uint8_t* p, uint32_t n, uint32_t m[16]) {
    if (n == 64 && ((reinterpret_cast<uintptr_t>(p) & 15u) == 0)) {
        const uint4* q = reinterpret_cast<const uint4*>(p);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uint4 v = q[i];
            m[4 * i] = v.x;
            m[4 * i + 1] = v.y;
            m[4 * i + 2] = v.z;
            m[4 * i + 3] = v.w;
        }
        return;
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) m[i] = 0;
    for (uint32_t b = 0; b < n; ++b) m[b >> 2] |= (uint32_t)p[b] << (8 * (b & 3));
}

// Chaining value of every chunk (one thread per 1 KiB chunk).  With a single
// chunk the last block is finalised as the root and written to out8.
__global__ void chunk_kernel(const uint8_t* __restrict__ file, uint64_t len, uint64_t nchunks,
                             uint32_t* __restrict__ cvs, uint32_t* __restrict__ out8) {
    const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const uint64_t off = c * kB3ChunkLen;
    const uint32_t clen = (uint32_t)(len - off < kB3ChunkLen ? len - off : kB3ChunkLen);
    const uint32_t nblocks = clen == 0 ? 1u : (clen + 63u) / 64u;
    uint32_t cv[8] = {DM_B3_IV0, DM_B3_IV1, DM_B3_IV2, DM_B3_IV3, DM_B3_IV4, DM_B3_IV5, DM_B3_IV6, DM_B3_IV7};
    uint32_t m[16], out[16];
    for (uint32_t b = 0; b < nblocks; ++b) {
        const uint32_t bl = clen - b * 64u < 64u ? clen - b * 64u : 64u;
        load_block(file + off + b * 64u, clen == 0 ? 0u : bl, m);
        uint32_t flags = (b == 0 ? kB3ChunkStart : 0u);
        if (b + 1 == nblocks) flags |= kB3ChunkEnd | (nchunks == 1 ? kB3Root : 0u);
        b3_compress(cv, m, nchunks == 1 ? 0ull : c, clen == 0 ? 0u : bl, flags, out);
#pragma unroll
        for (int i = 0; i < 8; ++i) cv[i] = out[i];
    }
    uint32_t* dst = nchunks == 1 ? out8 : cvs + c * 8;
#pragma unroll
    for (int i = 0; i < 8; ++i) dst[i] = cv[i];
}

// Pairwise merge of chaining values level by level (a lone last node is carried
// up unchanged), which reproduces BLAKE3's left-complete tree; the last merge is
// the root.  Single CTA, ping-pong buffers a/b of 8 * n words.
__global__ void __launch_bounds__(1024) tree_kernel(uint32_t* a, uint32_t* b, uint64_t n, uint32_t* __restrict__ out8) {
    const uint32_t iv[8] = {DM_B3_IV0, DM_B3_IV1, DM_B3_IV2, DM_B3_IV3, DM_B3_IV4, DM_B3_IV5, DM_B3_IV6, DM_B3_IV7};
    uint32_t* src = a;
    uint32_t* dst = b;
    while (n > 1) {
        const uint64_t pairs = n / 2;
        const bool root = (n == 2);
        for (uint64_t j = threadIdx.x; j < pairs; j += blockDim.x) {
            uint32_t m[16], out[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) m[i] = src[2 * j * 8 + i];
            b3_compress(iv, m, 0, 64, kB3Parent | (root ? kB3Root : 0u), out);
            uint32_t* d = root ? out8 : dst + j * 8;
#pragma unroll
            for (int i = 0; i < 8; ++i) d[i] = out[i];
        }
        if ((n & 1) && threadIdx.x == 0)
            for (int i = 0; i < 8; ++i) dst[pairs * 8 + i] = src[(n - 1) * 8 + i];
        __syncthreads();
        n = pairs + (n & 1);
        uint32_t* t = src;
        src = dst;
        dst = t;
    }
}

}  // namespace

size_t file_hash_scratch_words(uint64_t len) {
    const uint64_t nchunks = len == 0 ? 1 : (len + kB3ChunkLen - 1) / kB3ChunkLen;
    return (size_t)(2 * 8 * nchunks);
}

cudaError_t launch_file_hash(const uint8_t* d_file, uint64_t len, uint32_t* d_cv_scratch, uint32_t* d_out8,
                             cudaStream_t st) {
    const uint64_t nchunks = len == 0 ? 1 : (len + kB3ChunkLen - 1) / kB3ChunkLen;
    chunk_kernel<<<(unsigned)((nchunks + 127) / 128), 128, 0, st>>>(d_file, len, nchunks, d_cv_scratch, d_out8);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || nchunks == 1) return e;
    tree_kernel<<<1, 1024, 0, st>>>(d_cv_scratch, d_cv_scratch + 8 * nchunks, nchunks, d_out8);
    return cudaGetLastError();
}

// The generator expansion of one statement through the multi-job kernel the
// prover uses (gen_jobs_kernel, k_jobs.cu), as a single job.
cudaError_t launch_gen_generators(const uint8_t g_seed[32], uint64_t N, uint32_t log_n, uint4* d_g,
                                  cudaStream_t st) {
    GenJob job{};
    for (int i = 0; i < 8; ++i) job.key[i] = b3_load_le32(g_seed + 4 * i);
    job.dst = d_g;
    job.total = N * kRank << log_n;
    job.log_n = log_n;
    if (job.total == 0) return cudaSuccess;
    return launch_gen_jobs(&job, 1, st);
}

cudaError_t launch_unpack_witness(const uint8_t* d_file, uint64_t len, uint64_t total_coeffs, uint4* d_m,
                                  cudaStream_t st) {
    if (total_coeffs == 0) return cudaSuccess;
    const uint64_t blocks = (total_coeffs + 255) / 256;
    unpack_kernel<<<(unsigned)(blocks < 152ull * 32 ? blocks : 152ull * 32), 256, 0, st>>>(d_file, len, total_coeffs,
                                                                                            d_m);
    return cudaGetLastError();
}

}  // namespace dm
