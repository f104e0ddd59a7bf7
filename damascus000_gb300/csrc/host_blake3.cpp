#include "host_blake3.h"

#include <atomic>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "dm_blake3.cuh"

namespace dm {

namespace {
const uint32_t kIV[8] = {DM_B3_IV0, DM_B3_IV1, DM_B3_IV2, DM_B3_IV3, DM_B3_IV4, DM_B3_IV5, DM_B3_IV6, DM_B3_IV7};

void words16(const uint8_t* p, uint32_t m[16]) {
    for (int i = 0; i < 16; ++i) m[i] = b3_load_le32(p + 4 * i);
}

// ---- lane-parallel compressions ----
//
// kLanes independent compressions at once in generic vector types (one lane per
// chunk, or per parent node): the compiler maps them to the host's SIMD unit
// (NEON on aarch64, SSE on x86-64) without architecture intrinsics, so the same
// code builds and gives the same digests on both.
constexpr int kLanes = 4;
typedef uint32_t LaneVec __attribute__((vector_size(4 * kLanes)));

#if defined(__aarch64__)
// Rotations by 16 and 8 are byte permutations: one table lookup on a host with a
// native byte permute (NEON), where two shifts and an OR cost three.
typedef uint8_t ByteVec __attribute__((vector_size(4 * kLanes)));
inline LaneVec b3_rotr(LaneVec x, uint32_t n) {
    if (n == 16) {
        const ByteVec perm = {2, 3, 0, 1, 6, 7, 4, 5, 10, 11, 8, 9, 14, 15, 12, 13};
        return (LaneVec)__builtin_shuffle((ByteVec)x, perm);
    }
    if (n == 8) {
        const ByteVec perm = {1, 2, 3, 0, 5, 6, 7, 4, 9, 10, 11, 8, 13, 14, 15, 12};
        return (LaneVec)__builtin_shuffle((ByteVec)x, perm);
    }
    return (x >> n) | (x << (32u - n));
}
#else
inline LaneVec b3_rotr(LaneVec x, uint32_t n) { return (x >> n) | (x << (32u - n)); }
#endif
inline LaneVec splat(uint32_t s) {
    LaneVec v = {};
    return v + s;
}

// The chaining value half of kLanes compressions: cv (per lane) is replaced by
// the output words 0..7.
inline void compress_lanes(LaneVec cv[8], const LaneVec m[16], const LaneVec& ctr_lo, const LaneVec& ctr_hi,
                           uint32_t block_len, uint32_t flags) {
    LaneVec v0 = cv[0], v1 = cv[1], v2 = cv[2], v3 = cv[3], v4 = cv[4], v5 = cv[5], v6 = cv[6], v7 = cv[7];
    LaneVec v8 = splat(DM_B3_IV0), v9 = splat(DM_B3_IV1), v10 = splat(DM_B3_IV2), v11 = splat(DM_B3_IV3);
    LaneVec v12 = ctr_lo, v13 = ctr_hi, v14 = splat(block_len), v15 = splat(flags);
    DM_B3_ROUND(m, 0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15);
    DM_B3_ROUND(m, 2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8);
    DM_B3_ROUND(m, 3, 4, 10, 12, 13, 2, 7, 14, 6, 5, 9, 0, 11, 15, 8, 1);
    DM_B3_ROUND(m, 10, 7, 12, 9, 14, 3, 13, 15, 4, 0, 11, 2, 5, 8, 1, 6);
    DM_B3_ROUND(m, 12, 13, 9, 11, 15, 10, 14, 8, 7, 2, 5, 3, 0, 1, 6, 4);
    DM_B3_ROUND(m, 9, 14, 11, 5, 8, 12, 15, 1, 13, 3, 0, 10, 2, 6, 4, 7);
    DM_B3_ROUND(m, 11, 15, 5, 0, 1, 9, 8, 6, 14, 10, 2, 12, 3, 4, 7, 13);
    cv[0] = v0 ^ v8;
    cv[1] = v1 ^ v9;
    cv[2] = v2 ^ v10;
    cv[3] = v3 ^ v11;
    cv[4] = v4 ^ v12;
    cv[5] = v5 ^ v13;
    cv[6] = v6 ^ v14;
    cv[7] = v7 ^ v15;
}

// Two groups of kLanes compressions with the same block length and flags,
// interleaved round by round: two independent dependency chains per step keep
// more of the host's vector pipes busy than one.
#define DM_B3_G2(i0, i1, i2, i3, s0, s1)                    \
    do {                                                    \
        DM_B3_G(v##i0, v##i1, v##i2, v##i3, m[s0], m[s1]);  \
        DM_B3_G(w##i0, w##i1, w##i2, w##i3, n[s0], n[s1]);  \
    } while (0)
#define DM_B3_ROUND2(S0, S1, S2, S3, S4, S5, S6, S7, S8, S9, S10, S11, S12, S13, S14, S15) \
    do {                                                                                  \
        DM_B3_G2(0, 4, 8, 12, S0, S1);                                                    \
        DM_B3_G2(1, 5, 9, 13, S2, S3);                                                    \
        DM_B3_G2(2, 6, 10, 14, S4, S5);                                                   \
        DM_B3_G2(3, 7, 11, 15, S6, S7);                                                   \
        DM_B3_G2(0, 5, 10, 15, S8, S9);                                                   \
        DM_B3_G2(1, 6, 11, 12, S10, S11);                                                 \
        DM_B3_G2(2, 7, 8, 13, S12, S13);                                                  \
        DM_B3_G2(3, 4, 9, 14, S14, S15);                                                  \
    } while (0)
inline void compress_lanes2(LaneVec cv[8], const LaneVec m[16], const LaneVec& lo_a, const LaneVec& hi_a,
                            LaneVec cw[8], const LaneVec n[16], const LaneVec& lo_b, const LaneVec& hi_b,
                            uint32_t block_len, uint32_t flags) {
    LaneVec v0 = cv[0], v1 = cv[1], v2 = cv[2], v3 = cv[3], v4 = cv[4], v5 = cv[5], v6 = cv[6], v7 = cv[7];
    LaneVec v8 = splat(DM_B3_IV0), v9 = splat(DM_B3_IV1), v10 = splat(DM_B3_IV2), v11 = splat(DM_B3_IV3);
    LaneVec v12 = lo_a, v13 = hi_a, v14 = splat(block_len), v15 = splat(flags);
    LaneVec w0 = cw[0], w1 = cw[1], w2 = cw[2], w3 = cw[3], w4 = cw[4], w5 = cw[5], w6 = cw[6], w7 = cw[7];
    LaneVec w8 = v8, w9 = v9, w10 = v10, w11 = v11, w12 = lo_b, w13 = hi_b, w14 = v14, w15 = v15;
    DM_B3_ROUND2(0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15);
    DM_B3_ROUND2(2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8);
    DM_B3_ROUND2(3, 4, 10, 12, 13, 2, 7, 14, 6, 5, 9, 0, 11, 15, 8, 1);
    DM_B3_ROUND2(10, 7, 12, 9, 14, 3, 13, 15, 4, 0, 11, 2, 5, 8, 1, 6);
    DM_B3_ROUND2(12, 13, 9, 11, 15, 10, 14, 8, 7, 2, 5, 3, 0, 1, 6, 4);
    DM_B3_ROUND2(9, 14, 11, 5, 8, 12, 15, 1, 13, 3, 0, 10, 2, 6, 4, 7);
    DM_B3_ROUND2(11, 15, 5, 0, 1, 9, 8, 6, 14, 10, 2, 12, 3, 4, 7, 13);
    cv[0] = v0 ^ v8;
    cv[1] = v1 ^ v9;
    cv[2] = v2 ^ v10;
    cv[3] = v3 ^ v11;
    cv[4] = v4 ^ v12;
    cv[5] = v5 ^ v13;
    cv[6] = v6 ^ v14;
    cv[7] = v7 ^ v15;
    cw[0] = w0 ^ w8;
    cw[1] = w1 ^ w9;
    cw[2] = w2 ^ w10;
    cw[3] = w3 ^ w11;
    cw[4] = w4 ^ w12;
    cw[5] = w5 ^ w13;
    cw[6] = w6 ^ w14;
    cw[7] = w7 ^ w15;
}
#undef DM_B3_ROUND2
#undef DM_B3_G2

// Message words i of kLanes 64-byte blocks that start `stride` bytes apart.
// Four lanes: each lane's 16 words are four vectors (little-endian hosts: the
// byte order of the words is the memory order), transposed in 4 x 4 tiles.
static_assert(kLanes == 4, "the transpose below is for four lanes");
static_assert(__BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__, "message words are loaded in memory order");
inline void load_lanes(const uint8_t* p, size_t stride, LaneVec m[16]) {
    typedef uint32_t Idx __attribute__((vector_size(4 * kLanes)));
    const Idx lo = {0, 4, 1, 5}, hi = {2, 6, 3, 7}, first = {0, 1, 4, 5}, second = {2, 3, 6, 7};
    for (int j = 0; j < 4; ++j) {
        LaneVec q[4];
        for (int l = 0; l < 4; ++l) std::memcpy(&q[l], p + l * stride + 16 * j, 16);
        const LaneVec t0 = __builtin_shuffle(q[0], q[1], lo), t1 = __builtin_shuffle(q[0], q[1], hi);
        const LaneVec t2 = __builtin_shuffle(q[2], q[3], lo), t3 = __builtin_shuffle(q[2], q[3], hi);
        m[4 * j + 0] = __builtin_shuffle(t0, t2, first);
        m[4 * j + 1] = __builtin_shuffle(t0, t2, second);
        m[4 * j + 2] = __builtin_shuffle(t1, t3, first);
        m[4 * j + 3] = __builtin_shuffle(t1, t3, second);
    }
}

inline void store_lanes(const LaneVec cv[8], uint32_t* out) {  // out: kLanes x 8 words
    alignas(64) uint32_t t[8][kLanes];
    for (int i = 0; i < 8; ++i) std::memcpy(t[i], &cv[i], sizeof(LaneVec));
    for (int l = 0; l < kLanes; ++l)
        for (int i = 0; i < 8; ++i) out[8 * l + i] = t[i][l];
}

// Chaining values of kLanes full (1024-byte, non-root) chunks first .. first + kLanes - 1.
void full_chunk_cvs_lanes(const uint8_t* data, uint64_t first, const uint32_t key[8], uint32_t flags,
                          uint32_t* out) {
    LaneVec cv[8], m[16];
    for (int i = 0; i < 8; ++i) cv[i] = splat(key[i]);
    alignas(64) uint32_t lo[kLanes], hi[kLanes];
    for (int l = 0; l < kLanes; ++l) {
        lo[l] = (uint32_t)(first + l);
        hi[l] = (uint32_t)((first + l) >> 32);
    }
    LaneVec ctr_lo, ctr_hi;
    std::memcpy(&ctr_lo, lo, sizeof(LaneVec));
    std::memcpy(&ctr_hi, hi, sizeof(LaneVec));
    const uint8_t* base = data + first * kB3ChunkLen;
    for (uint32_t b = 0; b < kB3ChunkLen / kB3BlockLen; ++b) {
        load_lanes(base + b * kB3BlockLen, kB3ChunkLen, m);
        const uint32_t f = flags | (b == 0 ? kB3ChunkStart : 0u) | (b + 1 == kB3ChunkLen / kB3BlockLen ? kB3ChunkEnd : 0u);
        compress_lanes(cv, m, ctr_lo, ctr_hi, kB3BlockLen, f);
    }
    store_lanes(cv, out);
}

// Chaining values of 2 x kLanes full chunks first .. first + 2 kLanes - 1, as two
// interleaved groups (used on aarch64; compiled everywhere).
[[maybe_unused]] void full_chunk_cvs_lanes2(const uint8_t* data, uint64_t first, const uint32_t key[8], uint32_t flags,
                           uint32_t* out) {
    LaneVec cv[8], cw[8], m[16], n[16];
    for (int i = 0; i < 8; ++i) cv[i] = cw[i] = splat(key[i]);
    alignas(64) uint32_t lo[2 * kLanes], hi[2 * kLanes];
    for (int l = 0; l < 2 * kLanes; ++l) {
        lo[l] = (uint32_t)(first + l);
        hi[l] = (uint32_t)((first + l) >> 32);
    }
    LaneVec lo_a, hi_a, lo_b, hi_b;
    std::memcpy(&lo_a, lo, sizeof(LaneVec));
    std::memcpy(&hi_a, hi, sizeof(LaneVec));
    std::memcpy(&lo_b, lo + kLanes, sizeof(LaneVec));
    std::memcpy(&hi_b, hi + kLanes, sizeof(LaneVec));
    const uint8_t* base = data + first * kB3ChunkLen;
    for (uint32_t b = 0; b < kB3ChunkLen / kB3BlockLen; ++b) {
        load_lanes(base + b * kB3BlockLen, kB3ChunkLen, m);
        load_lanes(base + kLanes * kB3ChunkLen + b * kB3BlockLen, kB3ChunkLen, n);
        const uint32_t f = flags | (b == 0 ? kB3ChunkStart : 0u) | (b + 1 == kB3ChunkLen / kB3BlockLen ? kB3ChunkEnd : 0u);
        compress_lanes2(cv, m, lo_a, hi_a, cw, n, lo_b, hi_b, kB3BlockLen, f);
    }
    store_lanes(cv, out);
    store_lanes(cw, out + 8 * kLanes);
}

// Chaining value of chunk c (any length, never the root).
void one_chunk_cv(const uint8_t* data, size_t len, uint64_t c, const uint32_t key[8], uint32_t flags, uint32_t out[8]) {
    const size_t off = c * kB3ChunkLen;
    const size_t clen = len - off < kB3ChunkLen ? len - off : kB3ChunkLen;
    const size_t nblocks = clen ? (clen + 63) / 64 : 1;
    uint32_t cv[8];
    std::memcpy(cv, key, 32);
    for (size_t b = 0; b < nblocks; ++b) {
        uint8_t block[64];
        const size_t bl = clen - b * 64 < 64 ? clen - b * 64 : 64;
        std::memset(block, 0, 64);
        std::memcpy(block, data + off + b * 64, bl);
        uint32_t m[16], o[16];
        words16(block, m);
        const uint32_t f = flags | (b == 0 ? kB3ChunkStart : 0u) | (b + 1 == nblocks ? kB3ChunkEnd : 0u);
        b3_compress(cv, m, c, (uint32_t)bl, f, o);
        std::memcpy(cv, o, 32);
    }
    std::memcpy(out, cv, 32);
}

// Chaining values of chunks [begin, end) of a message of len bytes into cvs
// (8 words per chunk): groups of kLanes full chunks in the lanes, the rest one by one.
void chunk_cvs_range(const uint8_t* data, size_t len, size_t begin, size_t end, const uint32_t key[8],
                     uint32_t flags, uint32_t* cvs) {
    const size_t full = len / kB3ChunkLen;  // chunks with all 1024 bytes
    size_t c = begin;
#if defined(__aarch64__)
    // two interleaved groups need 32 vector registers of state: NEON has them
    // (2.14 GB/s per Neoverse-V2 core against 1.34 for one group); the x86-64
    // baseline has 16 and runs one group faster
    for (; c + 2 * kLanes <= end && c + 2 * kLanes <= full; c += 2 * kLanes)
        full_chunk_cvs_lanes2(data, c, key, flags, cvs + 8 * c);
#endif
    for (; c + kLanes <= end && c + kLanes <= full; c += kLanes) full_chunk_cvs_lanes(data, c, key, flags, cvs + 8 * c);
    for (; c < end; ++c) one_chunk_cv(data, len, c, key, flags, cvs + 8 * c);
}

// Parents of one tree level: n nodes (8 words each) in src -> (n + 1) / 2 in dst,
// an odd last node carried up unchanged; with n == 2 the one parent is the root.
void merge_level(const uint32_t* src, size_t n, const uint32_t key[8], uint32_t flags, uint32_t* dst) {
    const size_t pairs = n / 2;
    const uint32_t pf = flags | kB3Parent | (n == 2 ? kB3Root : 0u);
    size_t j = 0;
    if (n > 2) {
        const LaneVec zero = {};
        for (; j + kLanes <= pairs; j += kLanes) {
            LaneVec cv[8], m[16];
            for (int i = 0; i < 8; ++i) cv[i] = splat(key[i]);
            load_lanes(reinterpret_cast<const uint8_t*>(src + 16 * j), 64, m);
            compress_lanes(cv, m, zero, zero, kB3BlockLen, pf);
            store_lanes(cv, dst + 8 * j);
        }
    }
    for (; j < pairs; ++j) {
        uint32_t o[16];
        b3_compress(key, src + 16 * j, 0, kB3BlockLen, pf, o);
        std::memcpy(dst + 8 * j, o, 32);
    }
    if (n & 1) std::memcpy(dst + 8 * pairs, src + 8 * (n - 1), 32);
}

void words_to_bytes(const uint32_t w[8], uint8_t out[32]) {
    for (int i = 0; i < 8; ++i) {
        out[4 * i] = (uint8_t)w[i];
        out[4 * i + 1] = (uint8_t)(w[i] >> 8);
        out[4 * i + 2] = (uint8_t)(w[i] >> 16);
        out[4 * i + 3] = (uint8_t)(w[i] >> 24);
    }
}

// Root of the tree over nchunks >= 2 chunk chaining values (the tree is left
// complete, which pairing level by level with the odd node carried up reproduces).
void tree_root(std::vector<uint32_t>& a, size_t nchunks, const uint32_t key[8], uint32_t flags, uint8_t out[32]) {
    std::vector<uint32_t> b(8 * ((nchunks + 1) / 2));
    uint32_t* src = a.data();
    uint32_t* dst = b.data();
    size_t n = nchunks;
    while (n > 1) {
        merge_level(src, n, key, flags, dst);
        n = (n + 1) / 2;
        std::swap(src, dst);
    }
    words_to_bytes(src, out);
}
}  // namespace

Blake3Hasher::Blake3Hasher() : flags_(0) {
    std::memcpy(key_, kIV, sizeof(key_));
    std::memcpy(cv_, key_, sizeof(cv_));
}

Blake3Hasher::Blake3Hasher(const uint8_t key[32]) : flags_(kB3Keyed) {
    for (int i = 0; i < 8; ++i) key_[i] = b3_load_le32(key + 4 * i);
    std::memcpy(cv_, key_, sizeof(cv_));
}

void Blake3Hasher::compress_buffered_block() {
    uint32_t m[16], out[16];
    words16(buf_, m);
    const uint32_t f = flags_ | (blocks_done_ == 0 ? kB3ChunkStart : 0u);
    b3_compress(cv_, m, chunk_counter_, kB3BlockLen, f, out);
    std::memcpy(cv_, out, 32);
    ++blocks_done_;
    buf_len_ = 0;
}

// Merges completed subtrees: one parent per trailing zero bit of total_chunks.
void Blake3Hasher::push_chunk_cv(const uint32_t cv_in[8], uint64_t total_chunks) {
    uint32_t cv[8];
    std::memcpy(cv, cv_in, 32);
    while ((total_chunks & 1) == 0) {
        uint32_t m[16], out[16];
        std::memcpy(m, stack_[depth_ - 1], 32);
        std::memcpy(m + 8, cv, 32);
        b3_compress(key_, m, 0, kB3BlockLen, flags_ | kB3Parent, out);
        std::memcpy(cv, out, 32);
        --depth_;
        total_chunks >>= 1;
    }
    std::memcpy(stack_[depth_++], cv, 32);
}

void Blake3Hasher::update(const void* data, size_t len) {
    const uint8_t* p = static_cast<const uint8_t*>(data);
    while (len > 0) {
        // A full chunk is closed only once more input arrives (its last block needs CHUNK_END).
        if (blocks_done_ * kB3BlockLen + buf_len_ == kB3ChunkLen) {
            uint32_t m[16], out[16];
            words16(buf_, m);
            b3_compress(cv_, m, chunk_counter_, kB3BlockLen, flags_ | kB3ChunkEnd | (blocks_done_ == 0 ? kB3ChunkStart : 0u),
                        out);
            push_chunk_cv(out, chunk_counter_ + 1);
            ++chunk_counter_;
            std::memcpy(cv_, key_, 32);
            blocks_done_ = 0;
            buf_len_ = 0;
        }
        if (buf_len_ == kB3BlockLen) compress_buffered_block();
        // Fast path: whole blocks straight from the input while more follows.
        size_t take = kB3BlockLen - buf_len_;
        const size_t chunk_room = kB3ChunkLen - (blocks_done_ * kB3BlockLen + buf_len_);
        if (take > chunk_room) take = chunk_room;
        if (take > len) take = len;
        std::memcpy(buf_ + buf_len_, p, take);
        buf_len_ += (uint32_t)take;
        p += take;
        len -= take;
    }
}

void Blake3Hasher::update_u64(uint64_t v) {
    uint8_t t[8];
    for (int i = 0; i < 8; ++i) t[i] = (uint8_t)(v >> (8 * i));
    update(t, 8);
}

void Blake3Hasher::finalize(uint8_t out[32]) const {
    // Pending output: the current chunk's last block.
    uint32_t cv[8], m[16], outw[16];
    std::memcpy(cv, cv_, 32);
    uint8_t block[64];
    std::memset(block, 0, sizeof(block));
    std::memcpy(block, buf_, buf_len_);
    words16(block, m);
    uint64_t counter = chunk_counter_;
    uint32_t blen = buf_len_;
    uint32_t flags = flags_ | kB3ChunkEnd | (blocks_done_ == 0 ? kB3ChunkStart : 0u);
    for (int d = depth_; d > 0; --d) {
        b3_compress(cv, m, counter, blen, flags, outw);  // chaining value of the pending node
        std::memcpy(m, stack_[d - 1], 32);
        std::memcpy(m + 8, outw, 32);
        std::memcpy(cv, key_, 32);
        counter = 0;
        blen = kB3BlockLen;
        flags = flags_ | kB3Parent;
    }
    b3_compress(cv, m, 0, blen, flags | kB3Root, outw);
    for (int i = 0; i < 8; ++i) {
        out[4 * i] = (uint8_t)outw[i];
        out[4 * i + 1] = (uint8_t)(outw[i] >> 8);
        out[4 * i + 2] = (uint8_t)(outw[i] >> 16);
        out[4 * i + 3] = (uint8_t)(outw[i] >> 24);
    }
}

namespace {
// One-shot hash: a single chunk through the incremental hasher (its last block is
// the root), longer inputs as chunk chaining values in the lanes plus the tree.
void hash_oneshot(const uint8_t* key_bytes, const void* data, size_t len, uint8_t out[32]) {
    if (len <= kB3ChunkLen) {
        Blake3Hasher h = key_bytes ? Blake3Hasher(key_bytes) : Blake3Hasher();
        h.update(data, len);
        h.finalize(out);
        return;
    }
    uint32_t key[8];
    if (key_bytes)
        for (int i = 0; i < 8; ++i) key[i] = b3_load_le32(key_bytes + 4 * i);
    else
        std::memcpy(key, kIV, 32);
    const uint32_t flags = key_bytes ? kB3Keyed : 0u;
    const size_t nchunks = (len + kB3ChunkLen - 1) / kB3ChunkLen;
    std::vector<uint32_t> cvs(8 * nchunks);
    chunk_cvs_range(static_cast<const uint8_t*>(data), len, 0, nchunks, key, flags, cvs.data());
    tree_root(cvs, nchunks, key, flags, out);
}
}  // namespace

void blake3_hash(const void* data, size_t len, uint8_t out[32]) { hash_oneshot(nullptr, data, len, out); }

void blake3_keyed_hash(const uint8_t key[32], const void* data, size_t len, uint8_t out[32]) {
    hash_oneshot(key, data, len, out);
}

// ============================================================== host pool

namespace {

class Pool {
   public:
    static Pool& get() {
        static Pool* p = new Pool();  // lives until exit; threads are detached
        return *p;
    }
    size_t size() const { return workers_; }
    // Runs tasks[1..] on the workers and tasks[0] on the caller.  The counter is
    // decremented and signalled under done_mu, so the caller cannot see zero and
    // return (destroying done_mu / done_cv on its stack) before the last task has
    // released the mutex.
    void run(const std::vector<std::function<void()>>& tasks) {
        if (tasks.empty()) return;
        size_t left = tasks.size() - 1;
        std::mutex done_mu;
        std::condition_variable done_cv;
        {
            std::lock_guard<std::mutex> g(mu_);
            for (size_t i = 1; i < tasks.size(); ++i)
                queue_.push_back([&, i] {
                    tasks[i]();
                    std::lock_guard<std::mutex> g2(done_mu);
                    if (--left == 0) done_cv.notify_all();
                });
        }
        cv_.notify_all();
        tasks[0]();
        std::unique_lock<std::mutex> lk(done_mu);
        done_cv.wait(lk, [&] { return left == 0; });
    }

   private:
    Pool() {
        unsigned n = std::thread::hardware_concurrency();
        workers_ = n > 1 ? n : 1;
        for (size_t i = 0; i + 1 < workers_; ++i) std::thread([this] { loop(); }).detach();
    }
    void loop() {
        for (;;) {
            std::function<void()> f;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return !queue_.empty(); });
                f = std::move(queue_.front());
                queue_.pop_front();
            }
            f();
        }
    }
    size_t workers_ = 1;
    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<std::function<void()>> queue_;
};

struct ChunkArgs {
    const uint8_t* data;
    size_t len;
    uint32_t* cvs;
};

// Task bounds are rounded to whole pairs of lane groups, so every pair but the last runs interleaved.
void chunk_cvs(void* a, size_t begin, size_t end) {
    const ChunkArgs* A = static_cast<const ChunkArgs*>(a);
    const size_t nchunks = (A->len + kB3ChunkLen - 1) / kB3ChunkLen;
    begin *= 2 * kLanes;
    end = end * 2 * kLanes < nchunks ? end * 2 * kLanes : nchunks;
    chunk_cvs_range(A->data, A->len, begin, end, kIV, 0u, A->cvs);
}

}  // namespace

namespace {
thread_local bool t_serial = false;
}  // namespace

HostSerialScope::HostSerialScope() : prev_(t_serial) { t_serial = true; }
HostSerialScope::~HostSerialScope() { t_serial = prev_; }

void host_parallel_for(size_t n, size_t min_per_task, void (*fn)(void*, size_t, size_t), void* arg) {
    if (t_serial) {
        fn(arg, 0, n);
        return;
    }
    Pool& P = Pool::get();
    size_t tasks = (n + min_per_task - 1) / (min_per_task ? min_per_task : 1);
    if (tasks > P.size()) tasks = P.size();
    if (tasks <= 1) {
        fn(arg, 0, n);
        return;
    }
    std::vector<std::function<void()>> v;
    for (size_t t = 0; t < tasks; ++t) {
        const size_t b = n * t / tasks, e = n * (t + 1) / tasks;
        v.push_back([=] { fn(arg, b, e); });
    }
    P.run(v);
}

void blake3_hash_parallel(const void* data, size_t len, uint8_t out[32]) {
    const size_t nchunks = (len + kB3ChunkLen - 1) / kB3ChunkLen;
    if (len < (64u << 10) || nchunks < 2 || t_serial) {
        blake3_hash(data, len, out);
        return;
    }
    std::vector<uint32_t> a(8 * nchunks);
    ChunkArgs args{static_cast<const uint8_t*>(data), len, a.data()};
    host_parallel_for((nchunks + 2 * kLanes - 1) / (2 * kLanes), 2, chunk_cvs, &args);
    tree_root(a, nchunks, kIV, 0u, out);
}

}  // namespace dm
