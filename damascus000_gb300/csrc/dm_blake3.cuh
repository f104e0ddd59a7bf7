// BLAKE3 compression function (host and device), written from the BLAKE3
// specification.  The reference uses the blake3 crate 1.8.3 for the file id
// (src/utils/io.rs:33), the generator seed and coefficients
// (src/commitment/sis.rs:208-245) and the transcript (src/protocol/transcript.rs:50-61).
#pragma once

#include "dm_common.cuh"

namespace dm {

constexpr uint32_t kB3ChunkStart = 1u, kB3ChunkEnd = 2u, kB3Parent = 4u, kB3Root = 8u, kB3Keyed = 16u;
constexpr uint32_t kB3BlockLen = 64u, kB3ChunkLen = 1024u;

#if defined(__CUDA_ARCH__)
DM_HD uint32_t b3_rotr(uint32_t x, uint32_t n) { return __funnelshift_r(x, x, n); }
#else
DM_HD uint32_t b3_rotr(uint32_t x, uint32_t n) { return (x >> n) | (x << (32u - n)); }
#endif

#define DM_B3_IV0 0x6A09E667u
#define DM_B3_IV1 0xBB67AE85u
#define DM_B3_IV2 0x3C6EF372u
#define DM_B3_IV3 0xA54FF53Au
#define DM_B3_IV4 0x510E527Fu
#define DM_B3_IV5 0x9B05688Cu
#define DM_B3_IV6 0x1F83D9ABu
#define DM_B3_IV7 0x5BE0CD19u

#define DM_B3_G(a, b, c, d, mx, my)      \
    do {                                 \
        a = a + b + (mx);                \
        d = b3_rotr(d ^ a, 16);          \
        c = c + d;                       \
        b = b3_rotr(b ^ c, 12);          \
        a = a + b + (my);                \
        d = b3_rotr(d ^ a, 8);           \
        c = c + d;                       \
        b = b3_rotr(b ^ c, 7);           \
    } while (0)

// One round with message word order S0..S15 (the permuted schedule).
#define DM_B3_ROUND(m, S0, S1, S2, S3, S4, S5, S6, S7, S8, S9, S10, S11, S12, S13, S14, S15) \
    do {                                                                                    \
        DM_B3_G(v0, v4, v8, v12, m[S0], m[S1]);                                             \
        DM_B3_G(v1, v5, v9, v13, m[S2], m[S3]);                                             \
        DM_B3_G(v2, v6, v10, v14, m[S4], m[S5]);                                            \
        DM_B3_G(v3, v7, v11, v15, m[S6], m[S7]);                                            \
        DM_B3_G(v0, v5, v10, v15, m[S8], m[S9]);                                            \
        DM_B3_G(v1, v6, v11, v12, m[S10], m[S11]);                                          \
        DM_B3_G(v2, v7, v8, v13, m[S12], m[S13]);                                           \
        DM_B3_G(v3, v4, v9, v14, m[S14], m[S15]);                                           \
    } while (0)

// out[0..7] = chaining value; if full_out, out[8..15] = second half of the output block.
DM_HD void b3_compress(const uint32_t cv[8], const uint32_t m[16], uint64_t counter, uint32_t block_len,
                       uint32_t flags, uint32_t out[16], bool full_out = false) {
    uint32_t v0 = cv[0], v1 = cv[1], v2 = cv[2], v3 = cv[3], v4 = cv[4], v5 = cv[5], v6 = cv[6], v7 = cv[7];
    uint32_t v8 = DM_B3_IV0, v9 = DM_B3_IV1, v10 = DM_B3_IV2, v11 = DM_B3_IV3;
    uint32_t v12 = (uint32_t)counter, v13 = (uint32_t)(counter >> 32), v14 = block_len, v15 = flags;
    DM_B3_ROUND(m, 0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15);
    DM_B3_ROUND(m, 2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8);
    DM_B3_ROUND(m, 3, 4, 10, 12, 13, 2, 7, 14, 6, 5, 9, 0, 11, 15, 8, 1);
    DM_B3_ROUND(m, 10, 7, 12, 9, 14, 3, 13, 15, 4, 0, 11, 2, 5, 8, 1, 6);
    DM_B3_ROUND(m, 12, 13, 9, 11, 15, 10, 14, 8, 7, 2, 5, 3, 0, 1, 6, 4);
    DM_B3_ROUND(m, 9, 14, 11, 5, 8, 12, 15, 1, 13, 3, 0, 10, 2, 6, 4, 7);
    DM_B3_ROUND(m, 11, 15, 5, 0, 1, 9, 8, 6, 14, 10, 2, 12, 3, 4, 7, 13);
    out[0] = v0 ^ v8;
    out[1] = v1 ^ v9;
    out[2] = v2 ^ v10;
    out[3] = v3 ^ v11;
    out[4] = v4 ^ v12;
    out[5] = v5 ^ v13;
    out[6] = v6 ^ v14;
    out[7] = v7 ^ v15;
    if (full_out) {
        out[8] = v8 ^ cv[0];
        out[9] = v9 ^ cv[1];
        out[10] = v10 ^ cv[2];
        out[11] = v11 ^ cv[3];
        out[12] = v12 ^ cv[4];
        out[13] = v13 ^ cv[5];
        out[14] = v14 ^ cv[6];
        out[15] = v15 ^ cv[7];
    }
}

DM_HD uint32_t b3_load_le32(const uint8_t* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

// Message block of the generator coefficient derivation (src/commitment/sis.rs:231-245):
// "g" || u64 vec_idx || u64 coord || u64 coeff_idx, 25 bytes, zero padded.
DM_HD void b3_generator_block(uint64_t vec_idx, uint64_t coord, uint64_t coeff, uint32_t m[16]) {
    const uint32_t vl = (uint32_t)vec_idx, vh = (uint32_t)(vec_idx >> 32);
    const uint32_t kl = (uint32_t)coord, kh = (uint32_t)(coord >> 32);
    const uint32_t cl = (uint32_t)coeff, ch = (uint32_t)(coeff >> 32);
    m[0] = 0x67u | (vl << 8);
    m[1] = (vl >> 24) | (vh << 8);
    m[2] = (vh >> 24) | (kl << 8);
    m[3] = (kl >> 24) | (kh << 8);
    m[4] = (kh >> 24) | (cl << 8);
    m[5] = (cl >> 24) | (ch << 8);
    m[6] = ch >> 24;
DM_UNROLL
    for (int i = 7; i < 16; ++i) m[i] = 0u;
}

}  // namespace dm
