// Multi-job stage kernels outside the ring arithmetic: coefficient-domain folds
// and commitment algebra, generator expansion, witness unpacking and the file
// hash.  Each takes a list of jobs, so one launch covers the same stage of many
// requests.
#include <cuda_runtime.h>

#include "dm_blake3.cuh"
#include "dm_jobkit.cuh"

namespace dm {

namespace {

using namespace jobkit;

// ================================================================ folds
constexpr int kFoldThreads = 256;
constexpr int kFoldItems = 4;  // elements per thread

__global__ void __launch_bounds__(kFoldThreads) fold_jobs_kernel(JobList<FoldJob> J) {
    const FoldJob jb = J.j[find_job(J)];
    const uint64_t base = (uint64_t)(blockIdx.x - jb.cta0) * kFoldThreads * kFoldItems + threadIdx.x;
    if (jb.mode == kFoldVec || jb.mode == kFoldPoly || jb.mode == kFoldPolyX) {
        // The folds the bytes go through (witness and generators): every item's two
        // inputs loaded before the first multiply, so a thread has all its loads
        // in flight at once.
        uint4 va[kFoldItems], vb[kFoldItems];
        bool neg[kFoldItems];
#pragma unroll
        for (int it = 0; it < kFoldItems; ++it) {
            const uint64_t e = base + (uint64_t)it * kFoldThreads;
            neg[it] = false;
            if (e >= jb.n) continue;
            if (jb.mode == kFoldVec) {
                va[it] = jb.a[e];
                vb[it] = jb.b[e];
            } else {
                const uint32_t h = 1u << jb.Lout;
                const uint64_t b2 = (e >> jb.Lout) << (jb.Lout + 1);
                const uint32_t j = (uint32_t)(e & (h - 1));
                va[it] = jb.a[b2 + 2 * j];
                if (jb.mode == kFoldPolyX) {
                    neg[it] = j == 0;  // X * odd wraps its top coefficient around with a sign
                    vb[it] = jb.a[j == 0 ? b2 + 2 * h - 1 : b2 + 2 * j - 1];
                } else {
                    vb[it] = jb.a[b2 + 2 * j + 1];
                }
            }
        }
#pragma unroll
        for (int it = 0; it < kFoldItems; ++it) {
            const uint64_t e = base + (uint64_t)it * kFoldThreads;
            if (e >= jb.n) return;
            fq b{{vb[it].x, vb[it].y, vb[it].z, vb[it].w}};
            if (neg[it]) b = fq_neg(b);
            stq(jb.dst, e, fq_fma(fq{{va[it].x, va[it].y, va[it].z, va[it].w}}, jb.x, b));
        }
        return;
    }
#pragma unroll
    for (int it = 0; it < kFoldItems; ++it) {
        const uint64_t e = base + (uint64_t)it * kFoldThreads;
        if (e >= jb.n) return;
        fq out;
        switch (jb.mode) {
            case kFoldVec:
                out = fq_fma(ldq(jb.a, e), jb.x, ldq(jb.b, e));
                break;
            case kFoldPoly:
            case kFoldPolyX: {
                const uint32_t h = 1u << jb.Lout;
                const uint64_t poly = e >> jb.Lout;
                const uint32_t j = (uint32_t)(e & (h - 1));
                const uint64_t b2 = poly << (jb.Lout + 1);
                fq odd;
                if (jb.mode == kFoldPolyX)
                    odd = j == 0 ? fq_neg(ldq(jb.a, b2 + 2 * h - 1)) : ldq(jb.a, b2 + 2 * j - 1);
                else
                    odd = ldq(jb.a, b2 + 2 * j + 1);
                out = fq_fma(ldq(jb.a, b2 + 2 * j), jb.x, odd);
                break;
            }
            case kCombine:
                out = fq_add(fq_fma(ldq(jb.a, e), jb.x, ldq(jb.b, e)), fq_mul(jb.y, ldq(jb.c, e)));
                break;
            case kCombineEven: {
                const uint64_t k = e >> jb.Lout;
                const uint32_t j = (uint32_t)(e & ((1u << jb.Lout) - 1));
                const fq even = ldq(jb.a, (k << (jb.Lout + 1)) + 2 * j);
                out = fq_add(fq_fma(even, jb.x, ldq(jb.b, e)), fq_mul(jb.y, ldq(jb.c, e)));
                break;
            }
            default: {
                const uint4 v = jb.a[e];
                uint32_t r[8] = {v.x, v.y, v.z, v.w, 0, 0, 0, 0};
                out = fq_reduce8(r);
                break;
            }
        }
        stq(jb.dst, e, out);
    }
}

// ================================================================ hashing / expansion
constexpr int kGenThreads = 256;
constexpr int kGenItems = 4;

// 32-bit add issued on the FMA pipe (a * one + b with `one` a kernel argument
// equal to 1, opaque to the compiler).  BLAKE3 is all adds, XORs and rotates;
// moving the adds off the integer ALU pipe leaves that pipe only the XORs and
// rotates.
DM_D uint32_t fadd(uint32_t a, uint32_t b, uint32_t one) {
    uint32_t r;
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(one), "r"(b));
    return r;
}
// Rotation right by 7 on the FMA pipe: x * 2^25 + floor(x * 2^25 / 2^32), with
// r7 = 2^25 a kernel argument so the compiler keeps the multiplies (the two
// parts have disjoint bits, so their sum is the rotation).  Used for part of
// the rotations to balance the two pipes: the ALU pipe bounds the expansion.
DM_D uint32_t frotr7(uint32_t x, uint32_t r7) {
    uint32_t r;
    asm("{\n\t.reg .u32 h;\n\tmul.hi.u32 h, %1, %2;\n\tmad.lo.u32 %0, %1, %2, h;\n\t}" : "=r"(r) : "r"(x), "r"(r7));
    return r;
}

// The generator message (src/commitment/sis.rs:231-245): the 25-byte block
// "g" || i || k || c (u64 LE each) as words m0 = 0x67 | i << 8, m1 = i >> 24,
// m2 = k << 8, m4 = c << 8; words 3, 5 .. 15 are zero for k < 8 and c < 2^24
// (the launcher checks the ring size), so their adds are left out.
#define DM_GEN_NZ(X) ((X) == 0 || (X) == 1 || (X) == 2 || (X) == 4)
#define DM_GEN_G(a, b, c, d, X, Y, ROT7)                     \
    do {                                                      \
        a = fadd(b, a, one);                                  \
        if (DM_GEN_NZ(X)) a = fadd(m[DM_GEN_NZ(X) ? (X) : 0], a, one); \
        d = b3_rotr(d ^ a, 16);                               \
        c = fadd(d, c, one);                                  \
        b = b3_rotr(b ^ c, 12);                               \
        a = fadd(b, a, one);                                  \
        if (DM_GEN_NZ(Y)) a = fadd(m[DM_GEN_NZ(Y) ? (Y) : 0], a, one); \
        d = b3_rotr(d ^ a, 8);                                \
        c = fadd(d, c, one);                                  \
        b = ROT7(b ^ c);                                      \
    } while (0)
#define DM_ROT7_ALU(x) b3_rotr((x), 7)
#define DM_ROT7_FMA(x) frotr7((x), r7)
// Column steps on the ALU rotation, diagonal steps on the FMA-pipe rotation.
#define DM_GEN_COLUMNS(S0, S1, S2, S3, S4, S5, S6, S7)      \
    do {                                                    \
        DM_GEN_G(v0, v4, v8, v12, S0, S1, DM_ROT7_ALU);     \
        DM_GEN_G(v1, v5, v9, v13, S2, S3, DM_ROT7_ALU);     \
        DM_GEN_G(v2, v6, v10, v14, S4, S5, DM_ROT7_ALU);    \
        DM_GEN_G(v3, v7, v11, v15, S6, S7, DM_ROT7_ALU);    \
    } while (0)
#define DM_GEN_DIAGONALS(S8, S9, S10, S11, S12, S13, S14, S15) \
    do {                                                       \
        DM_GEN_G(v0, v5, v10, v15, S8, S9, DM_ROT7_FMA);       \
        DM_GEN_G(v1, v6, v11, v12, S10, S11, DM_ROT7_FMA);     \
        DM_GEN_G(v2, v7, v8, v13, S12, S13, DM_ROT7_FMA);      \
        DM_GEN_G(v3, v4, v9, v14, S14, S15, DM_ROT7_FMA);      \
    } while (0)
#define DM_GEN_ROUND(S0, S1, S2, S3, S4, S5, S6, S7, S8, S9, S10, S11, S12, S13, S14, S15) \
    do {                                                                                   \
        DM_GEN_COLUMNS(S0, S1, S2, S3, S4, S5, S6, S7);                                    \
        DM_GEN_DIAGONALS(S8, S9, S10, S11, S12, S13, S14, S15);                            \
    } while (0)

__global__ void __launch_bounds__(kGenThreads) gen_jobs_kernel(JobList<GenJob> J, uint32_t one, uint32_t r7) {
    const GenJob jb = J.j[find_job(J)];
    const uint64_t base = (uint64_t)(blockIdx.x - jb.cta0) * kGenThreads * kGenItems + threadIdx.x;
    const uint32_t* key = jb.key;
    // The first compression round's column steps on words (0, 1), (2, 3), (4, 5), (6, 7) depend on
    // i, k, c and nothing respectively: the last once per thread, the first two
    // again only when the item's (i, k) changes (never within a thread once a
    // ring has 1024 coefficients).
    uint32_t m[5] = {0, 0, 0, 0, 0};
    uint32_t c3a = key[3], c3b = key[7], c3c = DM_B3_IV3, c3d = kB3ChunkStart | kB3ChunkEnd | kB3Root | kB3Keyed;
    DM_GEN_G(c3a, c3b, c3c, c3d, 6, 7, DM_ROT7_ALU);
    uint32_t c0a = 0, c0b = 0, c0c = 0, c0d = 0, c1a = 0, c1b = 0, c1c = 0, c1d = 0;
    uint64_t last_ik = ~0ull;
    for (int it = 0; it < kGenItems; ++it) {
        const uint64_t e = base + (uint64_t)it * kGenThreads;
        if (e >= jb.total) return;
        const uint32_t c = (uint32_t)(e & ((1ull << jb.log_n) - 1));
        const uint64_t ik = e >> jb.log_n;  // i * 8 + k
        if (ik != last_ik) {
            last_ik = ik;
            const uint64_t i = ik >> 3;
            m[0] = 0x67u | ((uint32_t)i << 8);
            m[1] = (uint32_t)(i >> 24);
            m[2] = ((uint32_t)ik & 7u) << 8;
            c0a = key[0], c0b = key[4], c0c = DM_B3_IV0, c0d = 0;
            DM_GEN_G(c0a, c0b, c0c, c0d, 0, 1, DM_ROT7_ALU);
            c1a = key[1], c1b = key[5], c1c = DM_B3_IV1, c1d = 0;
            DM_GEN_G(c1a, c1b, c1c, c1d, 2, 3, DM_ROT7_ALU);
        }
        m[4] = c << 8;
        uint32_t v0 = c0a, v4 = c0b, v8 = c0c, v12 = c0d;
        uint32_t v1 = c1a, v5 = c1b, v9 = c1c, v13 = c1d;
        uint32_t v2 = key[2], v6 = key[6], v10 = DM_B3_IV2, v14 = 25;
        uint32_t v3 = c3a, v7 = c3b, v11 = c3c, v15 = c3d;
        DM_GEN_G(v2, v6, v10, v14, 4, 5, DM_ROT7_ALU);
        DM_GEN_DIAGONALS(8, 9, 10, 11, 12, 13, 14, 15);
        DM_GEN_ROUND(2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8);
        DM_GEN_ROUND(3, 4, 10, 12, 13, 2, 7, 14, 6, 5, 9, 0, 11, 15, 8, 1);
        DM_GEN_ROUND(10, 7, 12, 9, 14, 3, 13, 15, 4, 0, 11, 2, 5, 8, 1, 6);
        DM_GEN_ROUND(12, 13, 9, 11, 15, 10, 14, 8, 7, 2, 5, 3, 0, 1, 6, 4);
        DM_GEN_ROUND(9, 14, 11, 5, 8, 12, 15, 1, 13, 3, 0, 10, 2, 6, 4, 7);
        DM_GEN_ROUND(11, 15, 5, 0, 1, 9, 8, 6, 14, 10, 2, 12, 3, 4, 7, 13);
        uint32_t r8[8] = {v0 ^ v8, v1 ^ v9, v2 ^ v10, v3 ^ v11, v4 ^ v12, v5 ^ v13, v6 ^ v14, v7 ^ v15};
        stq(jb.dst, e, fq_reduce8(r8));
    }
}

// A block unpacks kUnpackItems x 256 coefficients, i.e. 1024 x 13 = 13,312 bytes
// of the file (a multiple of 16): when the file is 16-byte aligned and the
// block's bytes lie inside it, they come in through shared memory in 16-byte
// loads, and each coefficient's 13 bytes are assembled from four words.  Blocks
// past the file's end (the square layout's zero padding) only write zeros.
constexpr int kUnpackThreads = 256;
constexpr int kUnpackItems = 4;
constexpr uint32_t kUnpackBlockCoeffs = kUnpackThreads * kUnpackItems;
constexpr uint32_t kUnpackBlockBytes = kUnpackBlockCoeffs * kBytesPerCoeff;
static_assert(kUnpackBlockBytes % 16 == 0, "16-byte loads cover a block's bytes");

__global__ void __launch_bounds__(kUnpackThreads) unpack_jobs_kernel(JobList<UnpackJob> J) {
    __shared__ __align__(16) uint8_t bytes[kUnpackBlockBytes];
    const UnpackJob jb = J.j[find_job(J)];
    const uint64_t j0 = (uint64_t)(blockIdx.x - jb.cta0) * kUnpackBlockCoeffs;
    const uint64_t base = j0 * kBytesPerCoeff;
    const bool staged = base + kUnpackBlockBytes <= jb.len && (reinterpret_cast<uintptr_t>(jb.file) & 15u) == 0;
    if (staged) {  // uniform per block
        const uint4* src = reinterpret_cast<const uint4*>(jb.file + base);
        uint4* dst = reinterpret_cast<uint4*>(bytes);
        for (uint32_t i = threadIdx.x; i < kUnpackBlockBytes / 16; i += kUnpackThreads) dst[i] = src[i];
        __syncthreads();
    }
#pragma unroll
    for (int it = 0; it < kUnpackItems; ++it) {
        const uint32_t t = it * kUnpackThreads + threadIdx.x;  // coefficient within the block
        const uint64_t j = j0 + t;
        if (j >= jb.total) return;
        uint32_t w[4] = {0, 0, 0, 0};
        if (staged) {
            // the coefficient's 13 bytes lie in the four words from its byte offset
            // rounded down (the offset is at most 3 bytes into the first word)
            const uint32_t bo = t * kBytesPerCoeff, sh = (bo & 3u) * 8u;
            const uint32_t* words = reinterpret_cast<const uint32_t*>(bytes) + (bo >> 2);
            const uint32_t v0 = words[0], v1 = words[1], v2 = words[2], v3 = words[3];
            w[0] = __funnelshift_r(v0, v1, sh);
            w[1] = __funnelshift_r(v1, v2, sh);
            w[2] = __funnelshift_r(v2, v3, sh);
            w[3] = (v3 >> sh) & 0xFFu;
        } else {
            const uint64_t off = j * kBytesPerCoeff;
            if (off < jb.len) {
                const uint64_t n = jb.len - off < (uint64_t)kBytesPerCoeff ? jb.len - off : (uint64_t)kBytesPerCoeff;
                for (uint32_t b = 0; b < n; ++b) w[b >> 2] |= (uint32_t)jb.file[off + b] << (8 * (b & 3));
            }
        }
        jb.dst[j] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

DM_D void load_block16(const uint8_t* p, uint32_t n, uint32_t m[16]) {
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

// Chunk chaining values, one thread per 1 KiB chunk (a single chunk is the root).
__global__ void __launch_bounds__(128) hash_chunk_jobs_kernel(JobList<HashJob> J) {
    const HashJob jb = J.j[find_job(J)];
    const uint64_t nchunks = jb.len == 0 ? 1 : (jb.len + kB3ChunkLen - 1) / kB3ChunkLen;
    const uint64_t c = (uint64_t)(blockIdx.x - jb.cta0) * 128 + threadIdx.x;
    if (c >= nchunks) return;
    const uint64_t off = c * kB3ChunkLen;
    const uint32_t clen = (uint32_t)(jb.len - off < kB3ChunkLen ? jb.len - off : kB3ChunkLen);
    const uint32_t nblocks = clen == 0 ? 1u : (clen + 63u) / 64u;
    uint32_t cv[8] = {DM_B3_IV0, DM_B3_IV1, DM_B3_IV2, DM_B3_IV3, DM_B3_IV4, DM_B3_IV5, DM_B3_IV6, DM_B3_IV7};
    uint32_t m[16], out[16];
    for (uint32_t b = 0; b < nblocks; ++b) {
        const uint32_t bl = clen - b * 64u < 64u ? clen - b * 64u : 64u;
        load_block16(jb.file + off + b * 64u, clen == 0 ? 0u : bl, m);
        uint32_t flags = (b == 0 ? kB3ChunkStart : 0u);
        if (b + 1 == nblocks) flags |= kB3ChunkEnd | (nchunks == 1 ? kB3Root : 0u);
        b3_compress(cv, m, nchunks == 1 ? 0ull : c, clen == 0 ? 0u : bl, flags, out);
#pragma unroll
        for (int i = 0; i < 8; ++i) cv[i] = out[i];
    }
    uint32_t* dst = nchunks == 1 ? jb.out8 : jb.scratch + c * 8;
#pragma unroll
    for (int i = 0; i < 8; ++i) dst[i] = cv[i];
}

// Pairwise tree merge, one CTA per job (a lone last node is carried up).
__global__ void __launch_bounds__(1024) hash_tree_jobs_kernel(JobList<HashJob> J) {
    const HashJob jb = J.j[blockIdx.x];
    uint64_t n = jb.len == 0 ? 1 : (jb.len + kB3ChunkLen - 1) / kB3ChunkLen;
    if (n == 1) return;
    const uint32_t iv[8] = {DM_B3_IV0, DM_B3_IV1, DM_B3_IV2, DM_B3_IV3, DM_B3_IV4, DM_B3_IV5, DM_B3_IV6, DM_B3_IV7};
    uint32_t* src = jb.scratch;
    uint32_t* dst = jb.scratch + 8 * n;
    while (n > 1) {
        const uint64_t pairs = n / 2;
        const bool root = (n == 2);
        for (uint64_t j = threadIdx.x; j < pairs; j += blockDim.x) {
            uint32_t m[16], out[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) m[i] = src[2 * j * 8 + i];
            b3_compress(iv, m, 0, 64, kB3Parent | (root ? kB3Root : 0u), out);
            uint32_t* d = root ? jb.out8 : dst + j * 8;
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

cudaError_t launch_fold_jobs(FoldJob* jobs, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs) return cudaErrorInvalidValue;
    JobList<FoldJob> JL;
    const uint32_t ctas = assign_ctas<FoldJob>(jobs, n, JL, [](const FoldJob& j) -> uint64_t {
        return (j.n + kFoldThreads * kFoldItems - 1) / (kFoldThreads * kFoldItems);
    });
    if (!ctas) return cudaSuccess;
    fold_jobs_kernel<<<ctas, kFoldThreads, 0, st>>>(JL);
    return cudaGetLastError();
}

cudaError_t launch_gen_jobs(GenJob* jobs, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs) return cudaErrorInvalidValue;
    for (int i = 0; i < n; ++i)  // message words 5 and 6 are zero for c < 2^24
        if (jobs[i].log_n > 24) return cudaErrorInvalidValue;
    JobList<GenJob> JL;
    const uint32_t ctas = assign_ctas<GenJob>(jobs, n, JL, [](const GenJob& j) -> uint64_t {
        return (j.total + kGenThreads * kGenItems - 1) / (kGenThreads * kGenItems);
    });
    if (!ctas) return cudaSuccess;
    gen_jobs_kernel<<<ctas, kGenThreads, 0, st>>>(JL, 1u, 1u << 25);
    return cudaGetLastError();
}

cudaError_t launch_unpack_jobs(UnpackJob* jobs, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs) return cudaErrorInvalidValue;
    JobList<UnpackJob> JL;
    const uint32_t ctas = assign_ctas<UnpackJob>(jobs, n, JL, [](const UnpackJob& j) -> uint64_t {
        return (j.total + kUnpackBlockCoeffs - 1) / kUnpackBlockCoeffs;
    });
    if (!ctas) return cudaSuccess;
    unpack_jobs_kernel<<<ctas, kUnpackThreads, 0, st>>>(JL);
    return cudaGetLastError();
}

cudaError_t launch_hash_jobs(HashJob* jobs, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs) return cudaErrorInvalidValue;
    JobList<HashJob> JL;
    const uint32_t ctas = assign_ctas<HashJob>(jobs, n, JL, [](const HashJob& j) -> uint64_t {
        const uint64_t c = j.len == 0 ? 1 : (j.len + kB3ChunkLen - 1) / kB3ChunkLen;
        return (c + 127) / 128;
    });
    hash_chunk_jobs_kernel<<<ctas, 128, 0, st>>>(JL);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    hash_tree_jobs_kernel<<<n, 1024, 0, st>>>(JL);
    return cudaGetLastError();
}

}  // namespace dm
