#include "protocol.h"

#include <cstring>

#include "host_blake3.h"

namespace dm {

size_t module_encoded_size(uint32_t n) { return 8 + (size_t)kRank * (8 + 16 * (size_t)n); }
size_t record_encoded_size(uint32_t nv, uint32_t np) { return 8 + 2 * module_encoded_size(nv) + 2 * module_encoded_size(np); }
size_t statement_encoded_size(uint32_t n) { return 32 + 8 + 8 + module_encoded_size(n) + 32; }
size_t proof_encoded_size(uint32_t d) {
    size_t t = statement_encoded_size(1u << d) + 8 + 16;
    for (uint32_t j = 0; j < d; ++j) t += record_encoded_size(1u << (d - j), 1u << (d - j - 1));
    return t;
}

void put_u64(std::vector<uint8_t>& out, uint64_t v) {
    for (int i = 0; i < 8; ++i) out.push_back((uint8_t)(v >> (8 * i)));
}
static uint64_t get_u64(const uint8_t* p) {
    uint64_t v = 0;
    for (int i = 7; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}

// module.rs:95-103: a slice of 8 Polys; Poly = Vec<Fp>; Fp = [u8; 16].
void encode_module(std::vector<uint8_t>& out, const Module& m) {
    put_u64(out, kRank);
    const size_t base = out.size();
    out.resize(base + (size_t)kRank * (8 + 16 * (size_t)m.n));
    uint8_t* p = out.data() + base;
    for (int k = 0; k < kRank; ++k) {
        for (int i = 0; i < 8; ++i) p[i] = (uint8_t)((uint64_t)m.n >> (8 * i));
        p += 8;
        for (uint32_t j = 0; j < m.n; ++j, p += 16) fq_to_bytes(m.c[(size_t)k * m.n + j], p);
    }
}

void encode_record(std::vector<uint8_t>& out, const RoundRecord& r) {
    put_u64(out, r.round);
    encode_module(out, r.l_vec);
    encode_module(out, r.r_vec);
    encode_module(out, r.l_poly);
    encode_module(out, r.r_poly);
}

void encode_statement(std::vector<uint8_t>& out, const Statement& s) {
    out.insert(out.end(), s.file_id, s.file_id + 32);
    put_u64(out, s.original_len_bytes);
    put_u64(out, s.d);
    encode_module(out, s.com_0);
    out.insert(out.end(), s.g_0_seed, s.g_0_seed + 32);
}

// Vec<Poly> of any length is read in full before the rank (== 8) and the
// coordinate lengths (module.rs:106-115) are checked.
bool decode_module(const uint8_t*& pp, const uint8_t* end, Module& m) {
    const uint8_t* p = pp;
    if (end - p < 8) return false;
    const uint64_t count = get_u64(p);
    p += 8;
    uint64_t n0 = 0;
    bool uniform = true;
    std::vector<fq> c;
    for (uint64_t k = 0; k < count; ++k) {
        if (end - p < 8) return false;
        const uint64_t n = get_u64(p);
        p += 8;
        if ((uint64_t)(end - p) / 16 < n) return false;
        if (k == 0) {
            n0 = n;
            if (count == (uint64_t)kRank) c.resize((size_t)kRank * n);
        }
        if (n != n0) uniform = false;
        if (count == (uint64_t)kRank && uniform)
            for (uint64_t j = 0; j < n; ++j) c[k * n + j] = fq_from_u128_words(fq_from_bytes(p + 16 * j));
        p += 16 * n;
    }
    if (count != (uint64_t)kRank || !uniform || n0 > 0xFFFFFFFFull) return false;
    m.n = (uint32_t)n0;
    m.c = std::move(c);
    pp = p;
    return true;
}

bool decode_record(const uint8_t*& p, const uint8_t* end, RoundRecord& r) {
    if (end - p < 8) return false;
    r.round = get_u64(p);
    p += 8;
    return decode_module(p, end, r.l_vec) && decode_module(p, end, r.r_vec) && decode_module(p, end, r.l_poly) &&
           decode_module(p, end, r.r_poly);
}

bool decode_statement(const uint8_t*& p, const uint8_t* end, Statement& s) {
    if (end - p < 48) return false;
    std::memcpy(s.file_id, p, 32);
    s.original_len_bytes = get_u64(p + 32);
    s.d = get_u64(p + 40);
    p += 48;
    if (!decode_module(p, end, s.com_0)) return false;
    if (end - p < 32) return false;
    std::memcpy(s.g_0_seed, p, 32);
    p += 32;
    return true;
}

namespace {
struct ScaledArgs {
    const fq* a;
    const fq* b;
    fq s;
    fq* r;
};
void scaled_range(void* p, size_t begin, size_t end) {
    const ScaledArgs* A = static_cast<const ScaledArgs*>(p);
    for (size_t i = begin; i < end; ++i) A->r[i] = fq_fma(A->a[i], A->s, A->b[i]);
}
}  // namespace

bool module_add_scaled(const Module& a, const Module& b, const fq& s, Module& out) {
    if (a.n != b.n) return false;
    Module r;
    r.n = a.n;
    r.c.resize(a.c.size());
    ScaledArgs args{a.c.data(), b.c.data(), s, r.c.data()};
    host_parallel_for(a.c.size(), 2048, scaled_range, &args);  // 112-bit products: split large modules
    out = std::move(r);
    return true;
}

namespace {
struct FoldArgs {
    const fq* base;
    const fq* l;
    const fq* r;
    fq sl, sr;
    fq* out;
    uint32_t step;  // 2 for the even coefficients of base, else 1
};
void fold_range(void* p, size_t begin, size_t end) {
    const FoldArgs* A = static_cast<const FoldArgs*>(p);
    // coordinate k, coefficient j of the output is coefficient step*j of the
    // base's coordinate k: index (k*n + j) * step = i * step
    for (size_t i = begin; i < end; ++i)
        A->out[i] = fq_fma(fq_fma(A->base[i * A->step], A->sl, A->l[i]), A->sr, A->r[i]);
}
}  // namespace

bool module_fold(const Module& base, bool even, const Module& l, const fq& sl, const Module& r, const fq& sr,
                 Module& out) {
    const uint32_t n = even ? base.n / 2 : base.n;
    if (l.n != n || r.n != n || (even && base.n < 2)) return false;
    Module m;
    m.n = n;
    m.c.resize((size_t)kRank * n);
    FoldArgs args{base.c.data(), l.c.data(), r.c.data(), sl, sr, m.c.data(), even ? 2u : 1u};
    host_parallel_for(m.c.size(), 2048, fold_range, &args);
    out = std::move(m);
    return true;
}

Module module_even(const Module& a) {
    Module r = Module::zero(a.n / 2);
    for (int k = 0; k < kRank; ++k)
        for (uint32_t j = 0; j < a.n / 2; ++j) r.c[(size_t)k * r.n + j] = a.c[(size_t)k * a.n + 2 * j];
    return r;
}

uint64_t coeff_count_for_byte_len(uint64_t len) {
    const uint64_t c = len / kBytesPerCoeff + (len % kBytesPerCoeff ? 1 : 0);
    return c ? c : 1;
}

bool square_layout_for_byte_len(uint64_t len, uint32_t* depth, uint64_t* dimension) {
    const uint64_t coeffs = coeff_count_for_byte_len(len);
    for (uint32_t d = kMinDepth; d < 32; ++d) {
        const uint64_t dim = 1ull << d;
        if (dim * dim >= coeffs) {
            *depth = d;
            *dimension = dim;
            return true;
        }
    }
    return false;
}

fq fq_from_hash(const uint8_t h[32]) {
    uint32_t r[8];
    for (int i = 0; i < 8; ++i)
        r[i] = (uint32_t)h[4 * i] | ((uint32_t)h[4 * i + 1] << 8) | ((uint32_t)h[4 * i + 2] << 16) |
               ((uint32_t)h[4 * i + 3] << 24);
    return fq_reduce8(r);
}

Transcript::Transcript(const uint8_t epoch_seed[32], const uint8_t file_id[32]) {
    std::memcpy(epoch_seed_, epoch_seed, 32);
    std::memcpy(file_id_, file_id, 32);
}

fq Transcript::challenge_vec(uint64_t round, const Module& c, const Module& l, const Module& r) const {
    return challenge("vec", round, c, l, r);
}
fq Transcript::challenge_poly(uint64_t round, const Module& c, const Module& l, const Module& r) const {
    return challenge("poly", round, c, l, r);
}

// transcript.rs:82-90: u64 K || per coordinate u64 n || n x 16-byte LE words
static void append_commitment(std::vector<uint8_t>& msg, const Module& m) {
    put_u64(msg, kRank);
    for (int k = 0; k < kRank; ++k) {
        put_u64(msg, m.n);
        const size_t base = msg.size();
        msg.resize(base + (size_t)m.n * 16);
        uint8_t* p = msg.data() + base;
        const fq* c = m.c.data() + (size_t)k * m.n;
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__
        std::memcpy(p, c, (size_t)m.n * 16);  // limbs are little-endian words
#else
        for (uint32_t j = 0; j < m.n; ++j) fq_to_bytes(c[j], p + 16 * j);
#endif
    }
}

// transcript.rs:42-75: the absorbed bytes are assembled once and hashed in
// parallel; only the trailing u32 counter changes between attempts.
fq Transcript::challenge(const char* label, uint64_t round, const Module& c, const Module& l, const Module& r) const {
    // one buffer per thread, reused: a fresh multi-megabyte vector per challenge
    // costs a page fault per 4 KiB
    thread_local std::vector<uint8_t> msg;
    msg.clear();
    msg.reserve(128 + 3 * (8 + (size_t)kRank * 8) + 16 * (c.c.size() + l.c.size() + r.c.size()));
    msg.insert(msg.end(), epoch_seed_, epoch_seed_ + 32);
    const size_t ll = std::strlen(label);
    put_u64(msg, ll);
    msg.insert(msg.end(), label, label + ll);
    put_u64(msg, 32);
    msg.insert(msg.end(), file_id_, file_id_ + 32);
    put_u64(msg, 0);  // epoch_index
    put_u64(msg, round);
    append_commitment(msg, c);
    append_commitment(msg, l);
    append_commitment(msg, r);
    const size_t prefix = msg.size();
    msg.resize(prefix + 4);
    return sample_nonzero_challenge([&](uint32_t counter) {
        for (int i = 0; i < 4; ++i) msg[prefix + i] = (uint8_t)(counter >> (8 * i));
        uint8_t out[32];
        blake3_hash_parallel(msg.data(), msg.size(), out);
        return fq_from_hash(out);
    });
}

}  // namespace dm
