/*
 * CPU oracle for the Damascus Fold commit/prove/verify path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference
 * Rust crate (damascus-core) used as the parity checker for the CUDA path and
 * as the timed CPU baseline. Nothing in the shipped library links or calls it.
 *
 * Parity status: pinned against the reference's own known-answer and property
 * tests (field, NTT, ring, commitment linearity, protocol invariants), plus the
 * published BLAKE3 digest of the empty input.  The reference has no golden byte
 * vectors for BLAKE3 trees, transcripts, commitments or records, and it cannot
 * be built here (no Rust toolchain), so those outputs are "parity unpinned"
 * beyond self-consistency (two BLAKE3 formulations, NTT vs naive products).
 *
 * Buffers crossing this interface hold field elements as 16-byte little-endian
 * words, exactly the reference's serde form (src/algebra/field.rs:112-129).
 */
#ifndef DAMASCUS_ORACLE_H
#define DAMASCUS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- field Z_q (src/algebra/field.rs) ---- */
void orc_fp_add(const uint8_t a[16], const uint8_t b[16], uint8_t out[16]);
void orc_fp_sub(const uint8_t a[16], const uint8_t b[16], uint8_t out[16]);
void orc_fp_mul(const uint8_t a[16], const uint8_t b[16], uint8_t out[16]);
void orc_fp_inv(const uint8_t a[16], uint8_t out[16]);
void orc_fp_from_le_bytes_mod_order(const uint8_t* bytes, size_t len, uint8_t out[16]);
void orc_fp_from_u128_bytes(const uint8_t in[16], uint8_t out[16]);

/* ---- BLAKE3 (blake3 crate 1.8.3, restated from the BLAKE3 specification) ---- */
void orc_blake3_hash(const uint8_t* data, size_t len, uint8_t out[32]);
void orc_blake3_keyed_hash(const uint8_t key[32], const uint8_t* data, size_t len, uint8_t out[32]);
/* Same digest computed by the spec's recursive tree definition (cross-check). */
void orc_blake3_hash_recursive(const uint8_t* data, size_t len, uint8_t out[32]);

/* ---- NTT / ring (src/algebra/ntt.rs, src/algebra/poly.rs) ---- */
int orc_ntt_roundtrip(uint64_t* values, size_t len, uint64_t modulus);
int orc_forward_ntt(uint64_t* values, size_t len, uint64_t modulus);
int orc_inverse_ntt(uint64_t* values, size_t len, uint64_t modulus);
int orc_convolution(const uint8_t* a, size_t na, const uint8_t* b, size_t nb, uint8_t* out);
int orc_negacyclic_multiply(const uint8_t* a, const uint8_t* b, size_t n, uint8_t* out);
void orc_naive_negacyclic(const uint8_t* a, const uint8_t* b, size_t n, uint8_t* out);
int orc_mul_by_x(const uint8_t* a, size_t n, uint8_t* out);

/* ---- io / layout (src/utils/io.rs) ---- */
uint64_t orc_coeff_count_for_byte_len(uint64_t byte_len);
/* depth d and dimension 2^d of the square layout */
int orc_layout_for_byte_len(uint64_t byte_len, uint32_t* depth, uint64_t* dimension);
/* expands a file into the square witness (dimension^2 coefficients x 16 B). */
int orc_expand_file(const uint8_t* file, size_t len, uint64_t max_preprocess_bytes,
                    uint8_t file_id[32], uint32_t* depth, uint8_t* witness_out, size_t witness_cap);

/* ---- commitment (src/commitment/sis.rs) ---- */
void orc_derive_subseed(const uint8_t seed[32], const uint8_t* label, size_t label_len, uint8_t out[32]);
/* generators: vector_len x 8 x ring_len coefficients, layout [vec][coord][coeff] */
int orc_derive_generators(const uint8_t g_seed[32], size_t vector_len, size_t ring_len, uint8_t* out);
/* com = sum_i g_i * m_i; witness [N][n], g [N][8][n], out [8][n].  use_ntt picks
 * negacyclic_multiply (1) or naive_negacyclic (0); threads splits the columns. */
int orc_commit_with_generators(const uint8_t* witness, const uint8_t* g, size_t vector_len,
                               size_t ring_len, int use_ntt, int threads, uint8_t* out);

/* ---- transcript (src/protocol/transcript.rs) ---- */
/* commitments: each is 8 coords of its own ring length (n_c, n_l, n_r). */
void orc_challenge(const uint8_t epoch_seed[32], const uint8_t file_id[32], const char* label,
                   uint64_t round, const uint8_t* c, size_t n_c, const uint8_t* l, size_t n_l,
                   const uint8_t* r, size_t n_r, uint8_t out[16]);

/* ---- prover (src/protocol/prover.rs) ---- */
typedef struct orc_prover orc_prover;
orc_prover* orc_prover_new(const uint8_t* file, size_t len, const uint8_t seed_generators[32],
                           const uint8_t epoch_seed[32], uint64_t max_preprocess_bytes,
                           int use_ntt, int threads, int* err);
void orc_prover_free(orc_prover* p);
uint32_t orc_prover_rounds_total(const orc_prover* p);
/* bincode(Statement) */
size_t orc_prover_statement(const orc_prover* p, uint8_t* buf, size_t cap);
/* runs fold_round(round); writes bincode(RoundRecord) */
int orc_prover_fold_round(orc_prover* p, uint64_t round, uint8_t* buf, size_t cap, size_t* out_len);
int orc_prover_final_opening(const orc_prover* p, uint8_t out[16]);
/* current commitment [8][n] and the current (N, n) */
void orc_prover_dims(const orc_prover* p, uint64_t* vector_len, uint64_t* ring_len);
void orc_prover_current_commitment(const orc_prover* p, uint8_t* out);
/* generators / witness of the current state, for kernel-level parity */
void orc_prover_state(const orc_prover* p, uint8_t* witness_out, uint8_t* g_out);
/* one-shot: bincode((Statement, Vec<RoundRecord>, Fp)) */
int orc_prove(const uint8_t* file, size_t len, const uint8_t seed_generators[32],
              const uint8_t epoch_seed[32], int use_ntt, int threads, uint8_t* out, size_t cap,
              size_t* out_len);
size_t orc_proof_size_for_depth(uint32_t d);
size_t orc_record_size(uint64_t ring_len_vec, uint64_t ring_len_poly);

/* ---- verifier (src/protocol/verifier.rs) ---- */
typedef struct orc_verifier orc_verifier;
orc_verifier* orc_verifier_new(const uint8_t* statement, size_t len, const uint8_t epoch_seed[32], int* err);
orc_verifier* orc_verifier_clone(const orc_verifier* v);
void orc_verifier_free(orc_verifier* v);
/* 0 = accepted this round; nonzero = rejected (deserialize or replay error) */
int orc_verifier_update(orc_verifier* v, const uint8_t* record, size_t len);
int orc_verifier_final(const orc_verifier* v, const uint8_t opening[16]);
void orc_verifier_dims(const orc_verifier* v, uint64_t* vector_len, uint64_t* ring_len);
/* one-shot verify of a bincode((Statement, Vec<RoundRecord>, Fp)) proof; 0 = accept */
int orc_verify(const uint8_t* proof, size_t len, const uint8_t epoch_seed[32]);

#ifdef __cplusplus
}
#endif
#endif
