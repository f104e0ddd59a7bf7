/*
 * CPU oracle for the Damascus Fold commit/prove/verify path.
 *
 * TEST INFRASTRUCTURE ONLY: a plain-C restatement of the reference crate
 * damascus-core, used by tests/ as the parity checker and by bench.py as the
 * timed CPU baseline ("port").  It is never linked into the shipped library.
 *
 * Each function names the reference file:line it restates.  Paths are relative
 * to the reference project root.  Off-tree algorithms restated from their
 * published definitions: BLAKE3 (blake3 crate 1.8.3, Cargo.lock:66-67),
 * BigUint modular reduction and Garner CRT (num-bigint 0.4.6, Cargo.lock:392),
 * bincode 1.3.3 fixint little-endian encoding (Cargo.lock:51-52).
 *
 * Parity: pinned on the reference's known-answer/property tests and the
 * published BLAKE3 digest of the empty input; transcripts, commitments and
 * records are "parity unpinned" beyond self-consistency (see the header).
 */
#include "damascus_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

/* src/utils/config.rs:4-21 */
static const u128 MSIS_Q = (((u128)0xFFFFFFFFFFFFULL) << 64) | (u128)0xFFFFFFFFFFFFFFB5ULL;
#define MIN_FOLD_DEPTH 6
#define MODULE_RANK 8
#define BYTES_PER_COEFF 13
static const uint64_t CRT_PRIMES[8] = {3892314113ULL, 2281701377ULL, 2013265921ULL, 2885681153ULL,
                                       2483027969ULL, 1811939329ULL, 469762049ULL,  4194304001ULL};

static u128 load_u128(const uint8_t* p) {
    u128 v = 0;
    for (int i = 15; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}
static void store_u128(uint8_t* p, u128 v) {
    for (int i = 0; i < 16; ++i) {
        p[i] = (uint8_t)(v & 0xFF);
        v >>= 8;
    }
}
static void store_u64(uint8_t* p, uint64_t v) {
    for (int i = 0; i < 8; ++i) p[i] = (uint8_t)(v >> (8 * i));
}
static uint64_t load_u64(const uint8_t* p) {
    uint64_t v = 0;
    for (int i = 7; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}

/* ======================================================================
 * Field Z_q, q = 2^112 - 75 (src/algebra/field.rs)
 * ==================================================================== */

/* field.rs:137-147 */
static u128 fp_add(u128 a, u128 b) {
    u128 s = a + b;
    return s >= MSIS_Q ? s - MSIS_Q : s;
}
/* field.rs:156-166 */
static u128 fp_sub(u128 a, u128 b) { return a >= b ? a - b : MSIS_Q - (b - a); }
/* field.rs:188-198 */
static u128 fp_neg(u128 a) { return a == 0 ? 0 : MSIS_Q - a; }

/* field.rs:250-258 */
static u128 reduce_pseudo_mersenne(u128 low, u128 high) {
    const u128 mask112 = (((u128)1) << 112) - 1;
    u128 acc = low + high * 75;
    u128 hi = acc >> 112;
    acc = (acc & mask112) + hi * 75;
    while (acc >= MSIS_Q) acc -= MSIS_Q;
    return acc;
}
/* field.rs:229-248: 56-bit limbs */
static u128 fp_mul(u128 lhs, u128 rhs) {
    const u128 limb_mask = (((u128)1) << 56) - 1;
    const u128 mask112 = (((u128)1) << 112) - 1;
    u128 a0 = lhs & limb_mask, a1 = lhs >> 56;
    u128 b0 = rhs & limb_mask, b1 = rhs >> 56;
    u128 c0 = a0 * b0;
    u128 c1 = a0 * b1 + a1 * b0;
    u128 c2 = a1 * b1;
    u128 c1_lo = c1 & limb_mask, c1_hi = c1 >> 56;
    u128 low_sum = c0 + (c1_lo << 56);
    u128 low = low_sum & mask112;
    u128 carry = low_sum >> 112;
    u128 high = c2 + c1_hi + carry;
    return reduce_pseudo_mersenne(low, high);
}
/* field.rs:93-109: inv = pow(q - 2) */
static u128 fp_pow(u128 base, u128 exp) {
    u128 result = 1;
    while (exp > 0) {
        if (exp & 1) result = fp_mul(result, base);
        base = fp_mul(base, base);
        exp >>= 1;
    }
    return result;
}
static u128 fp_inv(u128 a) { return fp_pow(a, MSIS_Q - 2); }

/* field.rs:45-63: little-endian bytes as a big integer, reduced mod q.
 * Restated as Horner's rule from the most significant byte. */
static u128 fp_from_le_bytes_mod_order(const uint8_t* bytes, size_t len) {
    u128 acc = 0;
    for (size_t i = len; i-- > 0;) acc = ((acc << 8) | bytes[i]) % MSIS_Q;
    return acc;
}
/* field.rs:65-71 */
static u128 fp_from_le_chunk(const uint8_t* bytes, size_t len) {
    u128 acc = 0;
    for (size_t i = 0; i < len; ++i) acc |= ((u128)bytes[i]) << (8 * i);
    return acc % MSIS_Q;
}

void orc_fp_add(const uint8_t a[16], const uint8_t b[16], uint8_t out[16]) {
    store_u128(out, fp_add(load_u128(a) % MSIS_Q, load_u128(b) % MSIS_Q));
}
void orc_fp_sub(const uint8_t a[16], const uint8_t b[16], uint8_t out[16]) {
    store_u128(out, fp_sub(load_u128(a) % MSIS_Q, load_u128(b) % MSIS_Q));
}
void orc_fp_mul(const uint8_t a[16], const uint8_t b[16], uint8_t out[16]) {
    store_u128(out, fp_mul(load_u128(a) % MSIS_Q, load_u128(b) % MSIS_Q));
}
void orc_fp_inv(const uint8_t a[16], uint8_t out[16]) { store_u128(out, fp_inv(load_u128(a) % MSIS_Q)); }
void orc_fp_from_le_bytes_mod_order(const uint8_t* bytes, size_t len, uint8_t out[16]) {
    store_u128(out, fp_from_le_bytes_mod_order(bytes, len));
}
void orc_fp_from_u128_bytes(const uint8_t in[16], uint8_t out[16]) {
    store_u128(out, load_u128(in) % MSIS_Q);
}

/* ======================================================================
 * BLAKE3, restated from the BLAKE3 specification (blake3 crate 1.8.3).
 * ==================================================================== */
#define B3_CHUNK_START 1u
#define B3_CHUNK_END 2u
#define B3_PARENT 4u
#define B3_ROOT 8u
#define B3_KEYED_HASH 16u
#define B3_BLOCK_LEN 64
#define B3_CHUNK_LEN 1024

static const uint32_t B3_IV[8] = {0x6A09E667u, 0xBB67AE85u, 0x3C6EF372u, 0xA54FF53Au,
                                  0x510E527Fu, 0x9B05688Cu, 0x1F83D9ABu, 0x5BE0CD19u};
static const unsigned B3_PERM[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};

static uint32_t rotr32(uint32_t x, unsigned n) { return (x >> n) | (x << (32 - n)); }

static void b3_g(uint32_t* s, int a, int b, int c, int d, uint32_t mx, uint32_t my) {
    s[a] = s[a] + s[b] + mx;
    s[d] = rotr32(s[d] ^ s[a], 16);
    s[c] = s[c] + s[d];
    s[b] = rotr32(s[b] ^ s[c], 12);
    s[a] = s[a] + s[b] + my;
    s[d] = rotr32(s[d] ^ s[a], 8);
    s[c] = s[c] + s[d];
    s[b] = rotr32(s[b] ^ s[c], 7);
}

static void b3_compress(const uint32_t cv[8], const uint32_t block[16], uint64_t counter,
                        uint32_t block_len, uint32_t flags, uint32_t out[16]) {
    uint32_t s[16], m[16], t[16];
    for (int i = 0; i < 8; ++i) s[i] = cv[i];
    s[8] = B3_IV[0];
    s[9] = B3_IV[1];
    s[10] = B3_IV[2];
    s[11] = B3_IV[3];
    s[12] = (uint32_t)counter;
    s[13] = (uint32_t)(counter >> 32);
    s[14] = block_len;
    s[15] = flags;
    memcpy(m, block, sizeof(m));
    for (int r = 0; r < 7; ++r) {
        b3_g(s, 0, 4, 8, 12, m[0], m[1]);
        b3_g(s, 1, 5, 9, 13, m[2], m[3]);
        b3_g(s, 2, 6, 10, 14, m[4], m[5]);
        b3_g(s, 3, 7, 11, 15, m[6], m[7]);
        b3_g(s, 0, 5, 10, 15, m[8], m[9]);
        b3_g(s, 1, 6, 11, 12, m[10], m[11]);
        b3_g(s, 2, 7, 8, 13, m[12], m[13]);
        b3_g(s, 3, 4, 9, 14, m[14], m[15]);
        if (r < 6) {
            for (int i = 0; i < 16; ++i) t[i] = m[B3_PERM[i]];
            memcpy(m, t, sizeof(m));
        }
    }
    for (int i = 0; i < 8; ++i) {
        out[i] = s[i] ^ s[i + 8];
        out[i + 8] = s[i + 8] ^ cv[i];
    }
}

static void b3_words_from_bytes(const uint8_t* bytes, size_t len, uint32_t words[16]) {
    uint8_t buf[64];
    memset(buf, 0, sizeof(buf));
    memcpy(buf, bytes, len);
    for (int i = 0; i < 16; ++i)
        words[i] = (uint32_t)buf[4 * i] | ((uint32_t)buf[4 * i + 1] << 8) |
                   ((uint32_t)buf[4 * i + 2] << 16) | ((uint32_t)buf[4 * i + 3] << 24);
}

/* A pending compression (the spec's "Output"): finalised as a chaining value or as root. */
typedef struct {
    uint32_t cv[8];
    uint32_t block[16];
    uint64_t counter;
    uint32_t block_len;
    uint32_t flags;
} b3_output;

static void b3_output_cv(const b3_output* o, uint32_t cv_out[8]) {
    uint32_t full[16];
    b3_compress(o->cv, o->block, o->counter, o->block_len, o->flags, full);
    memcpy(cv_out, full, 32);
}
static void b3_output_root32(const b3_output* o, uint8_t out[32]) {
    uint32_t full[16];
    b3_compress(o->cv, o->block, 0, o->block_len, o->flags | B3_ROOT, full);
    for (int i = 0; i < 8; ++i) {
        out[4 * i] = (uint8_t)full[i];
        out[4 * i + 1] = (uint8_t)(full[i] >> 8);
        out[4 * i + 2] = (uint8_t)(full[i] >> 16);
        out[4 * i + 3] = (uint8_t)(full[i] >> 24);
    }
}

/* The chunk's output: all blocks but the last are compressed; the last is pending. */
static b3_output b3_chunk_output(const uint32_t key[8], const uint8_t* chunk, size_t len,
                                 uint64_t chunk_counter, uint32_t flags) {
    uint32_t cv[8];
    memcpy(cv, key, 32);
    size_t nblocks = len == 0 ? 1 : (len + B3_BLOCK_LEN - 1) / B3_BLOCK_LEN;
    b3_output o;
    for (size_t b = 0; b < nblocks; ++b) {
        size_t off = b * B3_BLOCK_LEN;
        size_t blen = len - off < B3_BLOCK_LEN ? len - off : B3_BLOCK_LEN;
        if (len == 0) blen = 0;
        uint32_t words[16];
        b3_words_from_bytes(chunk + off, blen, words);
        uint32_t f = flags | (b == 0 ? B3_CHUNK_START : 0);
        if (b + 1 == nblocks) {
            memcpy(o.cv, cv, 32);
            memcpy(o.block, words, 64);
            o.counter = chunk_counter;
            o.block_len = (uint32_t)blen;
            o.flags = f | B3_CHUNK_END;
        } else {
            uint32_t full[16];
            b3_compress(cv, words, chunk_counter, B3_BLOCK_LEN, f, full);
            memcpy(cv, full, 32);
        }
    }
    return o;
}

static b3_output b3_parent_output(const uint32_t key[8], const uint32_t left[8], const uint32_t right[8],
                                  uint32_t flags) {
    b3_output o;
    memcpy(o.cv, key, 32);
    memcpy(o.block, left, 32);
    memcpy(o.block + 8, right, 32);
    o.counter = 0;
    o.block_len = B3_BLOCK_LEN;
    o.flags = flags | B3_PARENT;
    return o;
}

/* Incremental-hasher formulation: chaining-value stack merged by chunk count. */
static void b3_hash_stack(const uint32_t key[8], uint32_t flags, const uint8_t* data, size_t len,
                          uint8_t out[32]) {
    uint32_t stack[64][8];
    int depth = 0;
    size_t nchunks = len == 0 ? 1 : (len + B3_CHUNK_LEN - 1) / B3_CHUNK_LEN;
    b3_output last;
    memset(&last, 0, sizeof last); /* set by the last chunk; nchunks >= 1 */
    for (size_t c = 0; c < nchunks; ++c) {
        size_t off = c * B3_CHUNK_LEN;
        size_t clen = len - off < B3_CHUNK_LEN ? len - off : B3_CHUNK_LEN;
        if (len == 0) clen = 0;
        b3_output o = b3_chunk_output(key, data + off, clen, c, flags);
        if (c + 1 == nchunks) {
            last = o;
            break;
        }
        uint32_t cv[8];
        b3_output_cv(&o, cv);
        uint64_t total = c + 1;
        while ((total & 1) == 0) {
            b3_output p = b3_parent_output(key, stack[depth - 1], cv, flags);
            b3_output_cv(&p, cv);
            --depth;
            total >>= 1;
        }
        memcpy(stack[depth++], cv, 32);
    }
    b3_output o = last;
    while (depth > 0) {
        uint32_t cv[8];
        b3_output_cv(&o, cv);
        o = b3_parent_output(key, stack[depth - 1], cv, flags);
        --depth;
    }
    b3_output_root32(&o, out);
}

/* Recursive formulation: the left subtree holds the largest power-of-two number
 * of chunks that leaves at least one chunk on the right. */
static b3_output b3_subtree(const uint32_t key[8], uint32_t flags, const uint8_t* data, size_t len,
                            uint64_t first_chunk) {
    size_t nchunks = len == 0 ? 1 : (len + B3_CHUNK_LEN - 1) / B3_CHUNK_LEN;
    if (nchunks == 1) return b3_chunk_output(key, data, len, first_chunk, flags);
    size_t left_chunks = 1;
    while (left_chunks * 2 < nchunks) left_chunks *= 2;
    size_t left_len = left_chunks * B3_CHUNK_LEN;
    b3_output l = b3_subtree(key, flags, data, left_len, first_chunk);
    b3_output r = b3_subtree(key, flags, data + left_len, len - left_len, first_chunk + left_chunks);
    uint32_t lcv[8], rcv[8];
    b3_output_cv(&l, lcv);
    b3_output_cv(&r, rcv);
    return b3_parent_output(key, lcv, rcv, flags);
}

void orc_blake3_hash(const uint8_t* data, size_t len, uint8_t out[32]) {
    b3_hash_stack(B3_IV, 0, data, len, out);
}
void orc_blake3_hash_recursive(const uint8_t* data, size_t len, uint8_t out[32]) {
    b3_output o = b3_subtree(B3_IV, 0, data, len, 0);
    b3_output_root32(&o, out);
}
void orc_blake3_keyed_hash(const uint8_t key[32], const uint8_t* data, size_t len, uint8_t out[32]) {
    uint32_t kw[16];
    b3_words_from_bytes(key, 32, kw); /* key words 0..7; the upper words are zero */
    b3_hash_stack(kw, B3_KEYED_HASH, data, len, out);
}

/* Incremental hasher used by the transcript: buffers input, hashes at finalize. */
typedef struct {
    uint8_t* buf;
    size_t len, cap;
} b3_buf;
static void bbuf_put(b3_buf* b, const void* data, size_t len) {
    if (b->len + len > b->cap) {
        size_t nc = b->cap ? b->cap : 256;
        while (nc < b->len + len) nc *= 2;
        b->buf = (uint8_t*)realloc(b->buf, nc);
        b->cap = nc;
    }
    memcpy(b->buf + b->len, data, len);
    b->len += len;
}
static void bbuf_u64(b3_buf* b, uint64_t v) {
    uint8_t t[8];
    store_u64(t, v);
    bbuf_put(b, t, 8);
}

/* ======================================================================
 * NTT over the CRT primes (src/algebra/ntt.rs)
 * ==================================================================== */

/* ntt.rs:318-340 */
static uint64_t mod_add(uint64_t a, uint64_t b, uint64_t m) {
    uint64_t s = a + b;
    return s >= m ? s - m : s;
}
static uint64_t mod_sub(uint64_t a, uint64_t b, uint64_t m) { return a >= b ? a - b : m - (b - a); }
static uint64_t mod_mul(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)(((u128)a * b) % m); }
/* ntt.rs:342-352 */
static uint64_t mod_pow(uint64_t base, u128 exp, uint64_t m) {
    uint64_t r = 1;
    while (exp > 0) {
        if (exp & 1) r = mod_mul(r, base, m);
        base = mod_mul(base, base, m);
        exp >>= 1;
    }
    return r;
}

/* ntt.rs:287-316 */
static uint64_t multiplicative_generator(uint64_t modulus) {
    uint64_t factors[64];
    int nf = 0;
    uint64_t value = modulus - 1, divisor = 2;
    while (divisor * divisor <= value) {
        if (value % divisor == 0) {
            factors[nf++] = divisor;
            while (value % divisor == 0) value /= divisor;
        }
        divisor += divisor == 2 ? 1 : 2;
    }
    if (value > 1) factors[nf++] = value;
    for (uint64_t cand = 2; cand < modulus; ++cand) {
        int ok = 1;
        for (int i = 0; i < nf; ++i)
            if (mod_pow(cand, (modulus - 1) / factors[i], modulus) == 1) {
                ok = 0;
                break;
            }
        if (ok) return cand;
    }
    return 0;
}

/* ntt.rs:10-47: per (size, prime) plan with per-stage roots and bit-reversal */
typedef struct {
    size_t size;
    uint64_t modulus, inv_size;
    uint64_t stage_roots[40], inv_stage_roots[40];
    int nstages;
    size_t* bitrev;
} ntt_plan;

#define PLAN_CACHE_MAX 256
static ntt_plan* g_plans[PLAN_CACHE_MAX];
static int g_nplans = 0;
static pthread_mutex_t g_plan_lock = PTHREAD_MUTEX_INITIALIZER;

static ntt_plan* plan_new(size_t size, uint64_t modulus) {
    if (size == 0 || (size & (size - 1)) || (modulus - 1) % size) return NULL;
    ntt_plan* p = (ntt_plan*)calloc(1, sizeof(ntt_plan));
    p->size = size;
    p->modulus = modulus;
    uint64_t gen = multiplicative_generator(modulus);
    uint64_t root = mod_pow(gen, (modulus - 1) / size, modulus); /* ntt.rs:275-285 */
    uint64_t inv_root = mod_pow(root, modulus - 2, modulus);
    int s = 0;
    for (size_t len = 2; len <= size; len <<= 1, ++s) {
        p->stage_roots[s] = mod_pow(root, size / len, modulus);
        p->inv_stage_roots[s] = mod_pow(inv_root, size / len, modulus);
    }
    p->nstages = s;
    p->inv_size = mod_pow(size % modulus, modulus - 2, modulus);
    p->bitrev = (size_t*)malloc(sizeof(size_t) * size);
    int bits = 0;
    while (((size_t)1 << bits) < size) ++bits;
    for (size_t i = 0; i < size; ++i) { /* ntt.rs:354-362 */
        size_t r = 0;
        for (int b = 0; b < bits; ++b)
            if (i & ((size_t)1 << b)) r |= (size_t)1 << (bits - 1 - b);
        p->bitrev[i] = r;
    }
    return p;
}

/* ntt.rs:256-273: cached behind a lock */
static ntt_plan* cached_plan(size_t size, uint64_t modulus) {
    pthread_mutex_lock(&g_plan_lock);
    for (int i = 0; i < g_nplans; ++i)
        if (g_plans[i]->size == size && g_plans[i]->modulus == modulus) {
            ntt_plan* p = g_plans[i];
            pthread_mutex_unlock(&g_plan_lock);
            return p;
        }
    ntt_plan* p = plan_new(size, modulus);
    if (p && g_nplans < PLAN_CACHE_MAX) g_plans[g_nplans++] = p;
    pthread_mutex_unlock(&g_plan_lock);
    return p;
}

/* ntt.rs:242-254 */
static void butterfly_chunk(uint64_t* chunk, size_t len, uint64_t wlen, uint64_t m) {
    size_t half = len / 2;
    uint64_t w = 1;
    for (size_t i = 0; i < half; ++i) {
        uint64_t t = mod_mul(chunk[half + i], w, m);
        uint64_t u = chunk[i];
        chunk[i] = mod_add(u, t, m);
        chunk[half + i] = mod_sub(u, t, m);
        w = mod_mul(w, wlen, m);
    }
}
/* ntt.rs:364-370 */
static void bit_reverse_permute(uint64_t* v, const ntt_plan* p) {
    for (size_t i = 0; i < p->size; ++i) {
        size_t o = p->bitrev[i];
        if (i < o) {
            uint64_t t = v[i];
            v[i] = v[o];
            v[o] = t;
        }
    }
}
/* ntt.rs:58-74 */
static void forward_ntt(uint64_t* v, const ntt_plan* p) {
    bit_reverse_permute(v, p);
    size_t len = 2;
    for (int s = 0; s < p->nstages; ++s, len <<= 1)
        for (size_t c = 0; c < p->size; c += len) butterfly_chunk(v + c, len, p->stage_roots[s], p->modulus);
}
/* ntt.rs:76-96 */
static void inverse_ntt(uint64_t* v, const ntt_plan* p) {
    bit_reverse_permute(v, p);
    size_t len = 2;
    for (int s = 0; s < p->nstages; ++s, len <<= 1)
        for (size_t c = 0; c < p->size; c += len)
            butterfly_chunk(v + c, len, p->inv_stage_roots[s], p->modulus);
    for (size_t i = 0; i < p->size; ++i) v[i] = mod_mul(v[i], p->inv_size, p->modulus);
}

int orc_forward_ntt(uint64_t* values, size_t len, uint64_t modulus) {
    ntt_plan* p = cached_plan(len, modulus);
    if (!p) return -1;
    forward_ntt(values, p);
    return 0;
}
int orc_inverse_ntt(uint64_t* values, size_t len, uint64_t modulus) {
    ntt_plan* p = cached_plan(len, modulus);
    if (!p) return -1;
    inverse_ntt(values, p);
    return 0;
}
int orc_ntt_roundtrip(uint64_t* values, size_t len, uint64_t modulus) {
    if (orc_forward_ntt(values, len, modulus)) return -1;
    return orc_inverse_ntt(values, len, modulus);
}

/* ---- 256-bit unsigned helpers for Garner CRT (num-bigint BigUint semantics) ---- */
typedef struct {
    uint64_t w[4];
} u256;
static u256 u256_zero(void) {
    u256 r = {{0, 0, 0, 0}};
    return r;
}
static uint64_t u256_mod_small(const u256* a, uint64_t m) {
    u128 r = 0;
    for (int i = 3; i >= 0; --i) {
        r = ((r << 32) | (a->w[i] >> 32)) % m;
        r = ((r << 32) | (a->w[i] & 0xFFFFFFFFu)) % m;
    }
    return (uint64_t)r;
}
static u256 u256_mul_small(const u256* a, uint64_t b) {
    u256 r;
    u128 carry = 0;
    for (int i = 0; i < 4; ++i) {
        u128 t = (u128)a->w[i] * b + carry;
        r.w[i] = (uint64_t)t;
        carry = t >> 64;
    }
    return r;
}
static u256 u256_add(const u256* a, const u256* b) {
    u256 r;
    u128 carry = 0;
    for (int i = 0; i < 4; ++i) {
        u128 t = (u128)a->w[i] + b->w[i] + carry;
        r.w[i] = (uint64_t)t;
        carry = t >> 64;
    }
    return r;
}
static u256 u256_sub(const u256* a, const u256* b) {
    u256 r;
    uint64_t borrow = 0;
    for (int i = 0; i < 4; ++i) {
        u128 t = (u128)a->w[i] - b->w[i] - borrow;
        r.w[i] = (uint64_t)t;
        borrow = (uint64_t)(t >> 127) & 1;
    }
    return r;
}
static int u256_cmp(const u256* a, const u256* b) {
    for (int i = 3; i >= 0; --i) {
        if (a->w[i] != b->w[i]) return a->w[i] > b->w[i] ? 1 : -1;
    }
    return 0;
}
static u256 u256_shr1(const u256* a) {
    u256 r;
    for (int i = 0; i < 4; ++i) r.w[i] = (a->w[i] >> 1) | (i < 3 ? a->w[i + 1] << 63 : 0);
    return r;
}
static u128 u256_mod_q(const u256* a) {
    u128 r = 0;
    for (int i = 3; i >= 0; --i)
        for (int sh = 48; sh >= 0; sh -= 16) r = ((r << 16) | ((a->w[i] >> sh) & 0xFFFF)) % MSIS_Q;
    return r;
}

/* ntt.rs:372-398 */
typedef struct {
    u256 prefix[8];
    uint64_t inverses[8];
    u256 total, half;
} crt_data;
static crt_data g_crt;
static pthread_once_t g_crt_once = PTHREAD_ONCE_INIT;
static void crt_init(void) {
    u256 product = u256_zero();
    product.w[0] = 1;
    for (int i = 0; i < 8; ++i) {
        g_crt.prefix[i] = product;
        uint64_t pm = u256_mod_small(&product, CRT_PRIMES[i]);
        g_crt.inverses[i] = mod_pow(pm, CRT_PRIMES[i] - 2, CRT_PRIMES[i]);
        product = u256_mul_small(&product, CRT_PRIMES[i]);
    }
    g_crt.total = product;
    g_crt.half = u256_shr1(&product);
}
/* ntt.rs:400-427: Garner with a centered lift, then mod q */
static u128 reconstruct_mod_q(const uint64_t residues[8]) {
    u256 acc = u256_zero();
    for (int i = 0; i < 8; ++i) {
        uint64_t p = CRT_PRIMES[i];
        uint64_t current = u256_mod_small(&acc, p);
        uint64_t delta = mod_sub(residues[i], current, p);
        uint64_t correction = mod_mul(delta, g_crt.inverses[i], p);
        u256 term = u256_mul_small(&g_crt.prefix[i], correction);
        acc = u256_add(&acc, &term);
    }
    if (u256_cmp(&acc, &g_crt.half) > 0) {
        u256 dist = u256_sub(&g_crt.total, &acc);
        u128 d = u256_mod_q(&dist);
        return d == 0 ? 0 : MSIS_Q - d;
    }
    return u256_mod_q(&acc);
}

/* ntt.rs:226-240 */
static void naive_negacyclic(const u128* a, const u128* b, size_t n, u128* out) {
    for (size_t i = 0; i < n; ++i) out[i] = 0;
    for (size_t i = 0; i < n; ++i)
        for (size_t j = 0; j < n; ++j) {
            size_t idx = i + j;
            u128 term = fp_mul(a[i], b[j]);
            if (idx >= n) {
                idx -= n;
                term = fp_neg(term);
            }
            out[idx] = fp_add(out[idx], term);
        }
}

/* ntt.rs:112-224: zero-padded cyclic NTT of size 2n per prime, fold, Garner CRT */
static int negacyclic_multiply(const u128* lhs, const u128* rhs, size_t n, u128* out) {
    if (n == 0 || (n & (n - 1))) return -1;
    size_t ntt_size = 2 * n;
    for (int i = 0; i < 8; ++i)
        if ((CRT_PRIMES[i] - 1) % ntt_size) {
            naive_negacyclic(lhs, rhs, n, out);
            return 0;
        }
    pthread_once(&g_crt_once, crt_init);
    uint64_t* a = (uint64_t*)malloc(sizeof(uint64_t) * ntt_size);
    uint64_t* b = (uint64_t*)malloc(sizeof(uint64_t) * ntt_size);
    uint64_t* res = (uint64_t*)malloc(sizeof(uint64_t) * 8 * n);
    for (int pi = 0; pi < 8; ++pi) {
        uint64_t m = CRT_PRIMES[pi];
        ntt_plan* plan = cached_plan(ntt_size, m);
        memset(a, 0, sizeof(uint64_t) * ntt_size);
        memset(b, 0, sizeof(uint64_t) * ntt_size);
        for (size_t i = 0; i < n; ++i) {
            a[i] = (uint64_t)(lhs[i] % m);
            b[i] = (uint64_t)(rhs[i] % m);
        }
        forward_ntt(a, plan);
        forward_ntt(b, plan);
        for (size_t i = 0; i < ntt_size; ++i) a[i] = mod_mul(a[i], b[i], m);
        inverse_ntt(a, plan);
        for (size_t i = 0; i < n; ++i) res[pi * n + i] = mod_sub(a[i], a[i + n], m);
    }
    for (size_t i = 0; i < n; ++i) {
        uint64_t r[8];
        for (int pi = 0; pi < 8; ++pi) r[pi] = res[pi * n + i];
        out[i] = reconstruct_mod_q(r);
    }
    free(a);
    free(b);
    free(res);
    return 0;
}

static u128* load_vec(const uint8_t* b, size_t n) {
    u128* v = (u128*)malloc(sizeof(u128) * (n ? n : 1));
    for (size_t i = 0; i < n; ++i) v[i] = load_u128(b + 16 * i);
    return v;
}
static void store_vec(uint8_t* b, const u128* v, size_t n) {
    for (size_t i = 0; i < n; ++i) store_u128(b + 16 * i, v[i]);
}

int orc_negacyclic_multiply(const uint8_t* a, const uint8_t* b, size_t n, uint8_t* out) {
    u128 *x = load_vec(a, n), *y = load_vec(b, n), *z = (u128*)malloc(sizeof(u128) * (n ? n : 1));
    for (size_t i = 0; i < n; ++i) {
        x[i] %= MSIS_Q;
        y[i] %= MSIS_Q;
    }
    int rc = negacyclic_multiply(x, y, n, z);
    if (!rc) store_vec(out, z, n);
    free(x);
    free(y);
    free(z);
    return rc;
}
void orc_naive_negacyclic(const uint8_t* a, const uint8_t* b, size_t n, uint8_t* out) {
    u128 *x = load_vec(a, n), *y = load_vec(b, n), *z = (u128*)malloc(sizeof(u128) * (n ? n : 1));
    for (size_t i = 0; i < n; ++i) {
        x[i] %= MSIS_Q;
        y[i] %= MSIS_Q;
    }
    naive_negacyclic(x, y, n, z);
    store_vec(out, z, n);
    free(x);
    free(y);
    free(z);
}
/* ntt.rs:98-110 */
int orc_convolution(const uint8_t* a, size_t na, const uint8_t* b, size_t nb, uint8_t* out) {
    if (!na || !nb) return -1;
    u128 *x = load_vec(a, na), *y = load_vec(b, nb);
    u128* z = (u128*)calloc(na + nb - 1, sizeof(u128));
    for (size_t i = 0; i < na; ++i)
        for (size_t j = 0; j < nb; ++j) z[i + j] = fp_add(z[i + j], fp_mul(x[i] % MSIS_Q, y[j] % MSIS_Q));
    store_vec(out, z, na + nb - 1);
    free(x);
    free(y);
    free(z);
    return 0;
}
/* poly.rs:144-154 */
int orc_mul_by_x(const uint8_t* a, size_t n, uint8_t* out) {
    if (!n) return -1;
    u128* x = load_vec(a, n);
    u128* z = (u128*)malloc(sizeof(u128) * n);
    z[0] = fp_neg(x[n - 1] % MSIS_Q);
    for (size_t i = 1; i < n; ++i) z[i] = x[i - 1] % MSIS_Q;
    store_vec(out, z, n);
    free(x);
    free(z);
    return 0;
}

/* ======================================================================
 * io / layout (src/utils/io.rs)
 * ==================================================================== */

/* io.rs:72-76 */
uint64_t orc_coeff_count_for_byte_len(uint64_t byte_len) {
    uint64_t c = byte_len / BYTES_PER_COEFF + (byte_len % BYTES_PER_COEFF ? 1 : 0);
    return c ? c : 1;
}
/* io.rs:100-120 */
int orc_layout_for_byte_len(uint64_t byte_len, uint32_t* depth, uint64_t* dimension) {
    uint64_t coeffs = orc_coeff_count_for_byte_len(byte_len);
    for (uint32_t d = MIN_FOLD_DEPTH; d < 32; ++d) {
        uint64_t dim = (uint64_t)1 << d;
        if (dim * dim >= coeffs) {
            *depth = d;
            *dimension = dim;
            return 0;
        }
    }
    return -1;
}
/* io.rs:29-70 */
int orc_expand_file(const uint8_t* file, size_t len, uint64_t max_preprocess_bytes, uint8_t file_id[32],
                    uint32_t* depth, uint8_t* witness_out, size_t witness_cap) {
    orc_blake3_hash(file, len, file_id);
    uint64_t dim;
    if (orc_layout_for_byte_len(len, depth, &dim)) return -1;
    uint64_t cap = dim * dim;
    if (cap * 16 * 2 > max_preprocess_bytes) return -2; /* io.rs:42-49 */
    if (!witness_out) return 0;
    if (witness_cap < cap * 16) return -3;
    memset(witness_out, 0, cap * 16);
    for (size_t idx = 0, off = 0; off < len; ++idx, off += BYTES_PER_COEFF) {
        size_t clen = len - off < BYTES_PER_COEFF ? len - off : BYTES_PER_COEFF;
        store_u128(witness_out + 16 * idx, fp_from_le_chunk(file + off, clen));
    }
    return 0;
}

/* ======================================================================
 * Module elements R_q^8 (src/algebra/module.rs) and the commitment
 * ==================================================================== */
typedef struct {
    size_t n;
    u128* c; /* [8][n] */
} module_el;

static module_el mod_zero(size_t n) {
    module_el m;
    m.n = n;
    m.c = (u128*)calloc(8 * (n ? n : 1), sizeof(u128));
    return m;
}
static module_el mod_clone(const module_el* a) {
    module_el m = mod_zero(a->n);
    memcpy(m.c, a->c, sizeof(u128) * 8 * a->n);
    return m;
}
static void mod_free(module_el* m) {
    free(m->c);
    m->c = NULL;
}
static int mod_eq(const module_el* a, const module_el* b) {
    return a->n == b->n && memcmp(a->c, b->c, sizeof(u128) * 8 * a->n) == 0;
}
/* module.rs:34-59: a + s*b (returns -1 on ring length mismatch) */
static int mod_add_scaled(const module_el* a, const module_el* b, u128 s, module_el* out) {
    if (a->n != b->n) return -1;
    *out = mod_zero(a->n);
    for (size_t i = 0; i < 8 * a->n; ++i) out->c[i] = fp_add(a->c[i], fp_mul(b->c[i], s));
    return 0;
}
/* module.rs:83-93, poly.rs:87-96: even / odd halves */
static void mod_odd_even(const module_el* a, module_el* even, module_el* odd) {
    size_t h = a->n / 2;
    *even = mod_zero(h);
    *odd = mod_zero(h);
    for (int k = 0; k < 8; ++k)
        for (size_t i = 0; i < h; ++i) {
            even->c[k * h + i] = a->c[k * a->n + 2 * i];
            odd->c[k * h + i] = a->c[k * a->n + 2 * i + 1];
        }
}
/* sis.rs:208-210 */
void orc_derive_subseed(const uint8_t seed[32], const uint8_t* label, size_t label_len, uint8_t out[32]) {
    orc_blake3_keyed_hash(seed, label, label_len, out);
}
/* sis.rs:231-245 */
static u128 derive_field(const uint8_t seed[32], size_t vec_idx, size_t coord, size_t coeff_idx) {
    uint8_t input[25];
    uint8_t h[32];
    input[0] = 'g';
    store_u64(input + 1, vec_idx);
    store_u64(input + 9, coord);
    store_u64(input + 17, coeff_idx);
    orc_blake3_keyed_hash(seed, input, sizeof(input), h);
    return fp_from_le_bytes_mod_order(h, 32);
}
/* sis.rs:212-229, layout [vec][coord][coeff] */
static u128* derive_generators(const uint8_t g_seed[32], size_t N, size_t n) {
    u128* g = (u128*)malloc(sizeof(u128) * N * 8 * n);
    for (size_t i = 0; i < N; ++i)
        for (size_t k = 0; k < 8; ++k)
            for (size_t c = 0; c < n; ++c) g[(i * 8 + k) * n + c] = derive_field(g_seed, i, k, c);
    return g;
}
int orc_derive_generators(const uint8_t g_seed[32], size_t vector_len, size_t ring_len, uint8_t* out) {
    u128* g = derive_generators(g_seed, vector_len, ring_len);
    store_vec(out, g, vector_len * 8 * ring_len);
    free(g);
    return 0;
}

/* sis.rs:146-167: acc = sum_i g_i * m_i, with ring products by NTT or naive.
 * Columns may be split across threads; the sum mod q is order-independent. */
typedef struct {
    const u128 *m, *g;
    size_t n, lo, hi;
    int use_ntt;
    u128* acc;
    int rc;
} commit_job;
static void* commit_worker(void* arg) {
    commit_job* j = (commit_job*)arg;
    size_t n = j->n;
    u128* prod = (u128*)malloc(sizeof(u128) * n);
    for (size_t i = j->lo; i < j->hi; ++i)
        for (int k = 0; k < 8; ++k) {
            const u128* gk = j->g + (i * 8 + k) * n;
            const u128* mi = j->m + i * n;
            if (j->use_ntt) {
                if (negacyclic_multiply(gk, mi, n, prod)) j->rc = -1;
            } else {
                naive_negacyclic(gk, mi, n, prod);
            }
            for (size_t c = 0; c < n; ++c) j->acc[k * n + c] = fp_add(j->acc[k * n + c], prod[c]);
        }
    free(prod);
    return NULL;
}
static int commit_with_generators(const u128* m, const u128* g, size_t N, size_t n, int use_ntt,
                                  int threads, module_el* out) {
    if (N == 0) {
        *out = mod_zero(1);
        return 0;
    }
    *out = mod_zero(n);
    if (threads < 1) threads = 1;
    if ((size_t)threads > N) threads = (int)N;
    commit_job* jobs = (commit_job*)calloc(threads, sizeof(commit_job));
    pthread_t* tids = (pthread_t*)calloc(threads, sizeof(pthread_t));
    for (int t = 0; t < threads; ++t) {
        jobs[t].m = m;
        jobs[t].g = g;
        jobs[t].n = n;
        jobs[t].lo = N * t / threads;
        jobs[t].hi = N * (t + 1) / threads;
        jobs[t].use_ntt = use_ntt;
        jobs[t].acc = (u128*)calloc(8 * n, sizeof(u128));
        if (threads > 1)
            pthread_create(&tids[t], NULL, commit_worker, &jobs[t]);
        else
            commit_worker(&jobs[t]);
    }
    int rc = 0;
    for (int t = 0; t < threads; ++t) {
        if (threads > 1) pthread_join(tids[t], NULL);
        if (jobs[t].rc) rc = jobs[t].rc;
        for (size_t i = 0; i < 8 * n; ++i) out->c[i] = fp_add(out->c[i], jobs[t].acc[i]);
        free(jobs[t].acc);
    }
    free(jobs);
    free(tids);
    return rc;
}
int orc_commit_with_generators(const uint8_t* witness, const uint8_t* g, size_t N, size_t n, int use_ntt,
                               int threads, uint8_t* out) {
    u128* m = load_vec(witness, N * n);
    u128* gg = load_vec(g, N * 8 * n);
    for (size_t i = 0; i < N * n; ++i) m[i] %= MSIS_Q;
    for (size_t i = 0; i < N * 8 * n; ++i) gg[i] %= MSIS_Q;
    module_el c;
    int rc = commit_with_generators(m, gg, N, n, use_ntt, threads, &c);
    store_vec(out, c.c, 8 * c.n);
    mod_free(&c);
    free(m);
    free(gg);
    return rc;
}

/* ======================================================================
 * Transcript (src/protocol/transcript.rs)
 * ==================================================================== */

/* transcript.rs:82-90 */
static void absorb_commitment(b3_buf* b, const module_el* m) {
    bbuf_u64(b, 8);
    uint8_t t[16];
    for (int k = 0; k < 8; ++k) {
        bbuf_u64(b, m->n);
        for (size_t i = 0; i < m->n; ++i) {
            store_u128(t, m->c[k * m->n + i]);
            bbuf_put(b, t, 16);
        }
    }
}
/* transcript.rs:42-80 */
static u128 transcript_challenge(const uint8_t epoch_seed[32], const uint8_t file_id[32], const char* label,
                                 uint64_t round, const module_el* c, const module_el* l, const module_el* r) {
    b3_buf b = {NULL, 0, 0};
    bbuf_put(&b, epoch_seed, 32);
    size_t ll = strlen(label);
    bbuf_u64(&b, ll);
    bbuf_put(&b, label, ll);
    bbuf_u64(&b, 32);
    bbuf_put(&b, file_id, 32);
    bbuf_u64(&b, 0); /* epoch_index */
    bbuf_u64(&b, round);
    absorb_commitment(&b, c);
    absorb_commitment(&b, l);
    absorb_commitment(&b, r);
    size_t prefix = b.len;
    u128 out = 0;
    for (uint32_t counter = 0;; ++counter) { /* transcript.rs:66-75 */
        b.len = prefix;
        uint8_t t[4] = {(uint8_t)counter, (uint8_t)(counter >> 8), (uint8_t)(counter >> 16),
                        (uint8_t)(counter >> 24)};
        bbuf_put(&b, t, 4);
        uint8_t h[32];
        orc_blake3_hash(b.buf, b.len, h);
        out = fp_from_le_bytes_mod_order(h, 32);
        if (out != 0) break;
    }
    free(b.buf);
    return out;
}
void orc_challenge(const uint8_t epoch_seed[32], const uint8_t file_id[32], const char* label, uint64_t round,
                   const uint8_t* c, size_t n_c, const uint8_t* l, size_t n_l, const uint8_t* r, size_t n_r,
                   uint8_t out[16]) {
    module_el mc = {n_c, load_vec(c, 8 * n_c)}, ml = {n_l, load_vec(l, 8 * n_l)},
              mr = {n_r, load_vec(r, 8 * n_r)};
    store_u128(out, transcript_challenge(epoch_seed, file_id, label, round, &mc, &ml, &mr));
    mod_free(&mc);
    mod_free(&ml);
    mod_free(&mr);
}

/* ======================================================================
 * bincode 1.x (fixint, little endian) for Statement / RoundRecord
 * ==================================================================== */
static size_t module_size(size_t n) { return 8 + 8 * (8 + 16 * n); }
size_t orc_record_size(uint64_t nv, uint64_t np) { return 8 + 2 * module_size(nv) + 2 * module_size(np); }
static size_t statement_size(size_t n) { return 32 + 8 + 8 + module_size(n) + 32; }
size_t orc_proof_size_for_depth(uint32_t d) {
    size_t total = statement_size((size_t)1 << d) + 8 + 16;
    for (uint32_t j = 0; j < d; ++j) total += orc_record_size((uint64_t)1 << (d - j), (uint64_t)1 << (d - j - 1));
    return total;
}
/* module.rs:95-103: a slice of Polys, each a Vec<Fp> */
static uint8_t* put_module(uint8_t* p, const module_el* m) {
    store_u64(p, 8);
    p += 8;
    for (int k = 0; k < 8; ++k) {
        store_u64(p, m->n);
        p += 8;
        for (size_t i = 0; i < m->n; ++i, p += 16) store_u128(p, m->c[k * m->n + i]);
    }
    return p;
}
/* module.rs:106-115 + field.rs:121-129: reads 8 Polys of uniform length; Fp reduced mod q */
static int get_module(const uint8_t** pp, const uint8_t* end, module_el* out) {
    const uint8_t* p = *pp;
    if (end - p < 8) return -1;
    uint64_t count = load_u64(p);
    p += 8;
    size_t n0 = 0;
    u128* tmp = NULL;
    for (uint64_t k = 0; k < count; ++k) {
        if (end - p < 8) {
            free(tmp);
            return -1;
        }
        uint64_t n = load_u64(p);
        p += 8;
        if ((uint64_t)(end - p) / 16 < n) {
            free(tmp);
            return -1;
        }
        if (k >= 8) { /* more than K polys: rank mismatch once fully read */
            p += 16 * n;
            continue;
        }
        if (k == 0) {
            n0 = n;
            tmp = (u128*)calloc(8 * (n ? n : 1), sizeof(u128));
        }
        if (n != n0) { /* from_coords: coordinate length mismatch */
            p += 16 * n;
            n0 = (size_t)-1;
            continue;
        }
        for (uint64_t i = 0; i < n; ++i, p += 16) tmp[k * n + i] = load_u128(p) % MSIS_Q;
    }
    if (count != 8 || n0 == (size_t)-1) {
        free(tmp);
        return -1;
    }
    out->n = n0;
    out->c = tmp;
    *pp = p;
    return 0;
}

typedef struct {
    uint64_t round;
    module_el l_vec, r_vec, l_poly, r_poly;
} round_record;
static void record_free(round_record* r) {
    mod_free(&r->l_vec);
    mod_free(&r->r_vec);
    mod_free(&r->l_poly);
    mod_free(&r->r_poly);
}
static size_t record_encode(const round_record* r, uint8_t* buf) {
    uint8_t* p = buf;
    store_u64(p, r->round);
    p += 8;
    p = put_module(p, &r->l_vec);
    p = put_module(p, &r->r_vec);
    p = put_module(p, &r->l_poly);
    p = put_module(p, &r->r_poly);
    return (size_t)(p - buf);
}
static int record_decode(const uint8_t** pp, const uint8_t* end, round_record* r) {
    memset(r, 0, sizeof(*r));
    if (end - *pp < 8) return -1;
    r->round = load_u64(*pp);
    *pp += 8;
    if (get_module(pp, end, &r->l_vec)) return -1;
    if (get_module(pp, end, &r->r_vec)) {
        record_free(r);
        return -1;
    }
    if (get_module(pp, end, &r->l_poly)) {
        record_free(r);
        return -1;
    }
    if (get_module(pp, end, &r->r_poly)) {
        record_free(r);
        return -1;
    }
    return 0;
}

typedef struct {
    uint8_t file_id[32];
    uint64_t original_len_bytes, d;
    module_el com_0;
    uint8_t g_0_seed[32];
} statement;
static size_t statement_encode(const statement* s, uint8_t* buf) {
    uint8_t* p = buf;
    memcpy(p, s->file_id, 32);
    p += 32;
    store_u64(p, s->original_len_bytes);
    p += 8;
    store_u64(p, s->d);
    p += 8;
    p = put_module(p, &s->com_0);
    memcpy(p, s->g_0_seed, 32);
    p += 32;
    return (size_t)(p - buf);
}
static int statement_decode(const uint8_t** pp, const uint8_t* end, statement* s) {
    memset(s, 0, sizeof(*s));
    if (end - *pp < 48) return -1;
    memcpy(s->file_id, *pp, 32);
    s->original_len_bytes = load_u64(*pp + 32);
    s->d = load_u64(*pp + 40);
    *pp += 48;
    if (get_module(pp, end, &s->com_0)) return -1;
    if (end - *pp < 32) {
        mod_free(&s->com_0);
        return -1;
    }
    memcpy(s->g_0_seed, *pp, 32);
    *pp += 32;
    return 0;
}

/* ======================================================================
 * Prover (src/protocol/prover.rs)
 * ==================================================================== */
struct orc_prover {
    uint8_t epoch_seed[32];
    statement st;
    u128* message; /* [N][n] */
    u128* g;       /* [N][8][n] */
    size_t N, n;
    module_el current;
    uint64_t round, rounds;
    int use_ntt, threads;
};

/* prover.rs:61-111 */
orc_prover* orc_prover_new(const uint8_t* file, size_t len, const uint8_t seed_generators[32],
                           const uint8_t epoch_seed[32], uint64_t max_preprocess_bytes, int use_ntt, int threads,
                           int* err) {
    uint32_t d;
    uint64_t dim;
    uint8_t file_id[32];
    *err = 0;
    int rc = orc_expand_file(file, len, max_preprocess_bytes, file_id, &d, NULL, 0);
    if (rc) {
        *err = rc;
        return NULL;
    }
    orc_layout_for_byte_len(len, &d, &dim);
    orc_prover* p = (orc_prover*)calloc(1, sizeof(orc_prover));
    memcpy(p->epoch_seed, epoch_seed, 32);
    p->N = p->n = dim;
    p->rounds = d;
    p->use_ntt = use_ntt;
    p->threads = threads;
    uint8_t* w = (uint8_t*)malloc(dim * dim * 16);
    orc_expand_file(file, len, max_preprocess_bytes, file_id, &d, w, dim * dim * 16);
    p->message = load_vec(w, dim * dim);
    free(w);
    orc_derive_subseed(seed_generators, (const uint8_t*)"g0", 2, p->st.g_0_seed); /* sis.rs:70 */
    p->g = derive_generators(p->st.g_0_seed, dim, dim);
    memcpy(p->st.file_id, file_id, 32);
    p->st.original_len_bytes = len;
    p->st.d = d;
    if (commit_with_generators(p->message, p->g, dim, dim, use_ntt, threads, &p->st.com_0)) {
        *err = -4;
        orc_prover_free(p);
        return NULL;
    }
    p->current = mod_clone(&p->st.com_0);
    return p;
}
void orc_prover_free(orc_prover* p) {
    if (!p) return;
    free(p->message);
    free(p->g);
    mod_free(&p->st.com_0);
    mod_free(&p->current);
    free(p);
}
uint32_t orc_prover_rounds_total(const orc_prover* p) { return (uint32_t)p->rounds; }
size_t orc_prover_statement(const orc_prover* p, uint8_t* buf, size_t cap) {
    size_t need = statement_size(p->st.com_0.n);
    if (buf && cap >= need) statement_encode(&p->st, buf);
    return need;
}
void orc_prover_dims(const orc_prover* p, uint64_t* N, uint64_t* n) {
    *N = p->N;
    *n = p->n;
}
void orc_prover_current_commitment(const orc_prover* p, uint8_t* out) { store_vec(out, p->current.c, 8 * p->current.n); }
void orc_prover_state(const orc_prover* p, uint8_t* w, uint8_t* g) {
    if (w) store_vec(w, p->message, p->N * p->n);
    if (g) store_vec(g, p->g, p->N * 8 * p->n);
}

/* prover.rs:140-313 */
int orc_prover_fold_round(orc_prover* p, uint64_t round_idx, uint8_t* buf, size_t cap, size_t* out_len) {
    if (round_idx != p->round || p->round >= p->rounds) return -1;
    size_t N = p->N, n = p->n;
    round_record rec;
    memset(&rec, 0, sizeof(rec));
    rec.round = round_idx;
    module_el vfc;         /* vector_fold_commitment */
    u128 *fm, *fg;         /* folded message / generators */
    size_t fN;
    if (N > 1) { /* prover.rs:148-214 */
        size_t mid = N / 2;
        if (commit_with_generators(p->message, p->g + mid * 8 * n, mid, n, p->use_ntt, p->threads, &rec.l_vec) ||
            commit_with_generators(p->message + mid * n, p->g, mid, n, p->use_ntt, p->threads, &rec.r_vec))
            return -2;
        u128 x = transcript_challenge(p->epoch_seed, p->st.file_id, "vec", round_idx, &p->current, &rec.l_vec,
                                      &rec.r_vec);
        u128 x_inv = fp_inv(x);
        module_el t;
        mod_add_scaled(&p->current, &rec.l_vec, x_inv, &t);
        mod_add_scaled(&t, &rec.r_vec, x, &vfc);
        mod_free(&t);
        fN = mid;
        fm = (u128*)malloc(sizeof(u128) * mid * n);
        fg = (u128*)malloc(sizeof(u128) * mid * 8 * n);
        for (size_t i = 0; i < mid * n; ++i) fm[i] = fp_add(p->message[i], fp_mul(p->message[mid * n + i], x));
        for (size_t i = 0; i < mid * 8 * n; ++i) fg[i] = fp_add(p->g[i], fp_mul(p->g[mid * 8 * n + i], x_inv));
        module_el check;
        if (commit_with_generators(fm, fg, mid, n, p->use_ntt, p->threads, &check)) return -2;
        int ok = mod_eq(&check, &vfc);
        mod_free(&check);
        if (!ok) return -3; /* "vector folding invariant failed" */
    } else {              /* prover.rs:215-227 */
        module_el zero = mod_zero(n);
        transcript_challenge(p->epoch_seed, p->st.file_id, "vec", round_idx, &p->current, &zero, &zero);
        rec.l_vec = zero;
        rec.r_vec = mod_clone(&zero);
        vfc = mod_clone(&p->current);
        fN = N;
        fm = (u128*)malloc(sizeof(u128) * N * n);
        fg = (u128*)malloc(sizeof(u128) * N * 8 * n);
        memcpy(fm, p->message, sizeof(u128) * N * n);
        memcpy(fg, p->g, sizeof(u128) * N * 8 * n);
    }

    module_el next_c;
    u128 *nm, *ng;
    size_t nn;
    if (n > 1) { /* prover.rs:231-264 */
        size_t h = n / 2;
        u128* me = (u128*)malloc(sizeof(u128) * fN * h);
        u128* mo = (u128*)malloc(sizeof(u128) * fN * h);
        u128* ge = (u128*)malloc(sizeof(u128) * fN * 8 * h);
        u128* go = (u128*)malloc(sizeof(u128) * fN * 8 * h);
        for (size_t i = 0; i < fN; ++i)
            for (size_t c = 0; c < h; ++c) {
                me[i * h + c] = fm[i * n + 2 * c];
                mo[i * h + c] = fm[i * n + 2 * c + 1];
            }
        for (size_t e = 0; e < fN * 8; ++e) { /* prover.rs:408-419: odd half multiplied by X */
            for (size_t c = 0; c < h; ++c) {
                ge[e * h + c] = fg[e * n + 2 * c];
                go[e * h + c] = fg[e * n + 2 * c + 1];
            }
            u128 last = go[e * h + h - 1];
            for (size_t c = h - 1; c > 0; --c) go[e * h + c] = go[e * h + c - 1];
            go[e * h] = fp_neg(last);
        }
        if (commit_with_generators(me, go, fN, h, p->use_ntt, p->threads, &rec.l_poly) ||
            commit_with_generators(mo, ge, fN, h, p->use_ntt, p->threads, &rec.r_poly))
            return -2;
        u128 y = transcript_challenge(p->epoch_seed, p->st.file_id, "poly", round_idx, &vfc, &rec.l_poly,
                                      &rec.r_poly);
        u128 y_inv = fp_inv(y);
        module_el ce, co, t;
        mod_odd_even(&vfc, &ce, &co);
        mod_add_scaled(&ce, &rec.l_poly, y_inv, &t);
        mod_add_scaled(&t, &rec.r_poly, y, &next_c);
        mod_free(&ce);
        mod_free(&co);
        mod_free(&t);
        nm = (u128*)malloc(sizeof(u128) * fN * h);
        ng = (u128*)malloc(sizeof(u128) * fN * 8 * h);
        for (size_t i = 0; i < fN * h; ++i) nm[i] = fp_add(me[i], fp_mul(mo[i], y));
        for (size_t i = 0; i < fN * 8 * h; ++i) ng[i] = fp_add(ge[i], fp_mul(go[i], y_inv));
        nn = h;
        free(me);
        free(mo);
        free(ge);
        free(go);
        free(fm);
        free(fg);
    } else { /* prover.rs:265-277 */
        module_el zero = mod_zero(1);
        transcript_challenge(p->epoch_seed, p->st.file_id, "poly", round_idx, &vfc, &zero, &zero);
        rec.l_poly = zero;
        rec.r_poly = mod_clone(&zero);
        next_c = mod_clone(&vfc);
        nm = fm;
        ng = fg;
        nn = n;
    }
    /* prover.rs:279-291 */
    module_el recomputed;
    if (commit_with_generators(nm, ng, fN, nn, p->use_ntt, p->threads, &recomputed)) return -2;
    int ok = mod_eq(&recomputed, &next_c);
    mod_free(&recomputed);
    mod_free(&vfc);
    if (!ok) {
        mod_free(&next_c);
        record_free(&rec);
        return -3; /* "round folding invariant failed" */
    }
    free(p->message);
    free(p->g);
    p->message = nm;
    p->g = ng;
    p->N = fN;
    p->n = nn;
    mod_free(&p->current);
    p->current = next_c;
    p->round += 1;
    size_t need = orc_record_size(rec.l_vec.n, rec.l_poly.n);
    if (out_len) *out_len = need;
    if (buf && cap >= need) record_encode(&rec, buf);
    record_free(&rec);
    return (buf && cap < need) ? -5 : 0;
}

/* prover.rs:133-138 */
int orc_prover_final_opening(const orc_prover* p, uint8_t out[16]) {
    if (!(p->round == p->rounds && p->N == 1 && p->n == 1)) return -1;
    store_u128(out, p->message[0]);
    return 0;
}

int orc_prove(const uint8_t* file, size_t len, const uint8_t seed_generators[32], const uint8_t epoch_seed[32],
              int use_ntt, int threads, uint8_t* out, size_t cap, size_t* out_len) {
    int err;
    orc_prover* p = orc_prover_new(file, len, seed_generators, epoch_seed, UINT64_MAX, use_ntt, threads, &err);
    if (!p) return err ? err : -1;
    size_t need = orc_proof_size_for_depth((uint32_t)p->rounds);
    *out_len = need;
    if (cap < need) {
        orc_prover_free(p);
        return -5;
    }
    uint8_t* q = out + statement_encode(&p->st, out);
    store_u64(q, p->rounds);
    q += 8;
    for (uint64_t r = 0; r < p->rounds; ++r) {
        size_t l;
        int rc = orc_prover_fold_round(p, r, q, (size_t)(out + cap - q), &l);
        if (rc) {
            orc_prover_free(p);
            return rc;
        }
        q += l;
    }
    if (orc_prover_final_opening(p, q)) {
        orc_prover_free(p);
        return -6;
    }
    orc_prover_free(p);
    return 0;
}

/* ======================================================================
 * Verifier (src/protocol/verifier.rs)
 * ==================================================================== */
struct orc_verifier {
    uint8_t epoch_seed[32];
    statement st;
    module_el current;
    u128* g; /* [N][8][n] */
    size_t N, n;
    uint64_t round, rounds;
};

/* verifier.rs:22-43 */
orc_verifier* orc_verifier_new(const uint8_t* sbytes, size_t len, const uint8_t epoch_seed[32], int* err) {
    const uint8_t* p = sbytes;
    orc_verifier* v = (orc_verifier*)calloc(1, sizeof(orc_verifier));
    *err = 0;
    if (statement_decode(&p, sbytes + len, &v->st)) {
        free(v);
        *err = -1;
        return NULL;
    }
    uint32_t d;
    uint64_t dim;
    if (orc_layout_for_byte_len(v->st.original_len_bytes, &d, &dim)) {
        mod_free(&v->st.com_0);
        free(v);
        *err = -2;
        return NULL;
    }
    memcpy(v->epoch_seed, epoch_seed, 32);
    v->N = dim;
    v->n = v->st.com_0.n;
    v->rounds = v->st.d;
    v->g = derive_generators(v->st.g_0_seed, v->N, v->n);
    v->current = mod_clone(&v->st.com_0);
    return v;
}
orc_verifier* orc_verifier_clone(const orc_verifier* s) {
    orc_verifier* v = (orc_verifier*)calloc(1, sizeof(orc_verifier));
    *v = *s;
    v->st.com_0 = mod_clone(&s->st.com_0);
    v->current = mod_clone(&s->current);
    v->g = (u128*)malloc(sizeof(u128) * s->N * 8 * s->n);
    memcpy(v->g, s->g, sizeof(u128) * s->N * 8 * s->n);
    return v;
}
void orc_verifier_free(orc_verifier* v) {
    if (!v) return;
    mod_free(&v->st.com_0);
    mod_free(&v->current);
    free(v->g);
    free(v);
}
void orc_verifier_dims(const orc_verifier* v, uint64_t* N, uint64_t* n) {
    *N = v->N;
    *n = v->current.n;
}

/* verifier.rs:57-120 */
static int verifier_update(orc_verifier* v, const round_record* rec) {
    if (rec->round != v->round) return -1;
    size_t N = v->N, n = v->n;
    module_el vfc;
    u128* fg;
    size_t fN;
    if (N > 1) {
        size_t mid = N / 2;
        u128 x = transcript_challenge(v->epoch_seed, v->st.file_id, "vec", v->round, &v->current, &rec->l_vec,
                                      &rec->r_vec);
        u128 x_inv = fp_inv(x);
        module_el t;
        if (mod_add_scaled(&v->current, &rec->l_vec, x_inv, &t)) return -2;
        if (mod_add_scaled(&t, &rec->r_vec, x, &vfc)) {
            mod_free(&t);
            return -2;
        }
        mod_free(&t);
        fN = mid;
        fg = (u128*)malloc(sizeof(u128) * mid * 8 * n);
        for (size_t i = 0; i < mid * 8 * n; ++i) fg[i] = fp_add(v->g[i], fp_mul(v->g[mid * 8 * n + i], x_inv));
    } else {
        module_el zero = mod_zero(v->current.n);
        transcript_challenge(v->epoch_seed, v->st.file_id, "vec", v->round, &v->current, &zero, &zero);
        int ok = mod_eq(&rec->l_vec, &zero) && mod_eq(&rec->r_vec, &zero);
        mod_free(&zero);
        if (!ok) return -3;
        vfc = mod_clone(&v->current);
        fN = N;
        fg = (u128*)malloc(sizeof(u128) * N * 8 * n);
        memcpy(fg, v->g, sizeof(u128) * N * 8 * n);
    }
    module_el next_c;
    u128* ng;
    size_t nn;
    if (n > 1) {
        size_t h = n / 2;
        ng = (u128*)malloc(sizeof(u128) * fN * 8 * h);
        u128 y = transcript_challenge(v->epoch_seed, v->st.file_id, "poly", v->round, &vfc, &rec->l_poly,
                                      &rec->r_poly);
        u128 y_inv = fp_inv(y);
        if (vfc.n < 2) { /* odd_even_decomposition of a scalar commitment panics in the reference */
            mod_free(&vfc);
            free(fg);
            free(ng);
            return -4;
        }
        module_el ce, co, t;
        mod_odd_even(&vfc, &ce, &co);
        int bad = mod_add_scaled(&ce, &rec->l_poly, y_inv, &t);
        if (!bad) {
            bad = mod_add_scaled(&t, &rec->r_poly, y, &next_c);
            mod_free(&t);
        }
        mod_free(&ce);
        mod_free(&co);
        mod_free(&vfc);
        if (bad) {
            free(fg);
            free(ng);
            return -2;
        }
        for (size_t e = 0; e < fN * 8; ++e) {
            u128* o = ng + e * h;
            const u128* s = fg + e * n;
            for (size_t c = 0; c < h; ++c) {
                u128 odd_shifted = c == 0 ? fp_neg(s[n - 1]) : s[2 * c - 1];
                o[c] = fp_add(s[2 * c], fp_mul(odd_shifted, y_inv));
            }
        }
        free(fg);
        nn = h;
    } else {
        module_el zero = mod_zero(1);
        transcript_challenge(v->epoch_seed, v->st.file_id, "poly", v->round, &vfc, &zero, &zero);
        int ok = mod_eq(&rec->l_poly, &zero) && mod_eq(&rec->r_poly, &zero);
        mod_free(&zero);
        if (!ok) {
            mod_free(&vfc);
            free(fg);
            return -3;
        }
        next_c = vfc;
        ng = fg;
        nn = n;
    }
    free(v->g);
    v->g = ng;
    v->N = fN;
    v->n = nn;
    mod_free(&v->current);
    v->current = next_c;
    v->round += 1;
    return 0;
}
int orc_verifier_update(orc_verifier* v, const uint8_t* bytes, size_t len) {
    const uint8_t* p = bytes;
    round_record rec;
    if (record_decode(&p, bytes + len, &rec)) return -10;
    int rc = verifier_update(v, &rec);
    record_free(&rec);
    return rc;
}
/* verifier.rs:122-134 */
int orc_verifier_final(const orc_verifier* v, const uint8_t opening[16]) {
    if (v->round != v->rounds) return -1;
    if (v->N != 1) return -2;
    u128 o = load_u128(opening) % MSIS_Q;
    module_el rhs = mod_zero(v->n);
    for (size_t i = 0; i < 8 * v->n; ++i) rhs.c[i] = fp_mul(v->g[i], o);
    int ok = mod_eq(&rhs, &v->current);
    mod_free(&rhs);
    return ok ? 0 : -3;
}

int orc_verify(const uint8_t* proof, size_t len, const uint8_t epoch_seed[32]) {
    const uint8_t *p = proof, *end = proof + len;
    statement st;
    if (statement_decode(&p, end, &st)) return -10;
    size_t slen = (size_t)(p - proof);
    mod_free(&st.com_0);
    int err;
    orc_verifier* v = orc_verifier_new(proof, slen, epoch_seed, &err);
    if (!v) return -11;
    if (end - p < 8) {
        orc_verifier_free(v);
        return -10;
    }
    uint64_t count = load_u64(p);
    p += 8;
    for (uint64_t r = 0; r < count; ++r) {
        round_record rec;
        if (record_decode(&p, end, &rec)) {
            orc_verifier_free(v);
            return -10;
        }
        int rc = verifier_update(v, &rec);
        record_free(&rec);
        if (rc) {
            orc_verifier_free(v);
            return rc;
        }
    }
    if (end - p < 16) {
        orc_verifier_free(v);
        return -10;
    }
    int rc = orc_verifier_final(v, p);
    orc_verifier_free(v);
    return rc;
}
