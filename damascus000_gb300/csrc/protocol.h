// Host-side protocol objects mirroring the reference's Rust types, their
// bincode 1.x encoding (fixint, little endian), and the Fiat-Shamir transcript.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "dm_field.cuh"

namespace dm {

// sample_nonzero_challenge (src/protocol/transcript.rs:66-75): candidates for
// counters 0, 1, 2, ... (wrapping) until one is nonzero.
template <class Candidate>
fq sample_nonzero_challenge(Candidate&& candidate) {
    for (uint32_t counter = 0;; ++counter) {
        const fq v = candidate(counter);
        if (!fq_is_zero(v)) return v;
    }
}

// ModuleElement<8> (src/algebra/module.rs:9): 8 coordinates of one ring length.
struct Module {
    uint32_t n = 0;
    std::vector<fq> c;  // [8][n]
    static Module zero(uint32_t n) {
        Module m;
        m.n = n;
        m.c.assign((size_t)kRank * n, fq_zero());
        return m;
    }
    bool operator==(const Module& o) const {
        if (n != o.n) return false;
        for (size_t i = 0; i < c.size(); ++i)
            if (!fq_eq(c[i], o.c[i])) return false;
        return true;
    }
};

// Statement<8> (src/commitment/sis.rs:24-30).
struct Statement {
    uint8_t file_id[32];
    uint64_t original_len_bytes = 0;
    uint64_t d = 0;
    Module com_0;
    uint8_t g_0_seed[32];
};

// RoundRecord (src/protocol/prover.rs:14-21).
struct RoundRecord {
    uint64_t round = 0;
    Module l_vec, r_vec, l_poly, r_poly;
};

// ---- bincode ----
size_t module_encoded_size(uint32_t n);
size_t record_encoded_size(uint32_t n_vec, uint32_t n_poly);
size_t statement_encoded_size(uint32_t n);
size_t proof_encoded_size(uint32_t d);  // (Statement, Vec<RoundRecord>, Fp)
void put_u64(std::vector<uint8_t>& out, uint64_t v);
void encode_module(std::vector<uint8_t>& out, const Module& m);
void encode_record(std::vector<uint8_t>& out, const RoundRecord& r);
void encode_statement(std::vector<uint8_t>& out, const Statement& s);
// Decoders advance p; they fail (false) exactly where bincode + the reference's
// Deserialize impls fail: short input, a rank other than 8, or unequal coordinate
// lengths.  Field elements are reduced mod q (field.rs:121-129).
bool decode_module(const uint8_t*& p, const uint8_t* end, Module& m);
bool decode_record(const uint8_t*& p, const uint8_t* end, RoundRecord& r);
bool decode_statement(const uint8_t*& p, const uint8_t* end, Statement& s);

// ---- module algebra on the host ----
// a + s * b; false on ring length mismatch (module.rs:34-59).
bool module_add_scaled(const Module& a, const Module& b, const fq& s, Module& out);
Module module_even(const Module& a);
// One verifier commitment update in a single pass: out = b + sl*l + sr*r with b =
// base, or its even coefficients when `even` (src/protocol/verifier.rs:64-103),
// each coefficient through the same two fused multiply-adds as two calls of
// module_add_scaled.  False when the ring lengths differ.
bool module_fold(const Module& base, bool even, const Module& l, const fq& sl, const Module& r, const fq& sr,
                 Module& out);

// ---- layout (src/utils/io.rs:72-120) ----
uint64_t coeff_count_for_byte_len(uint64_t len);
bool square_layout_for_byte_len(uint64_t len, uint32_t* depth, uint64_t* dimension);

// ---- transcript (src/protocol/transcript.rs) ----
class Transcript {
   public:
    Transcript() = default;
    Transcript(const uint8_t epoch_seed[32], const uint8_t file_id[32]);
    fq challenge_vec(uint64_t round, const Module& c, const Module& l, const Module& r) const;
    fq challenge_poly(uint64_t round, const Module& c, const Module& l, const Module& r) const;

   private:
    fq challenge(const char* label, uint64_t round, const Module& c, const Module& l, const Module& r) const;
    uint8_t epoch_seed_[32];
    uint8_t file_id_[32];
};

// 32-byte LE hash -> Z_q (field.rs:45-63).
fq fq_from_hash(const uint8_t h[32]);

}  // namespace dm
