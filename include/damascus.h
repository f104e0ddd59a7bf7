/*
 * damascus.h -- C ABI of the GB300 (sm_103a) Damascus Fold prover/verifier.
 *
 * A drop-in for the reference crate damascus-core behind DAMASCUS_GPU=1: the
 * Rust host code links libdamascus_gb300.so from build.rs and calls these
 * functions through `extern "C"`.  Every entry point names the reference
 * interface it replaces (paths relative to the reference project root).
 *
 * Conventions
 *  - Field elements (Fp, q = 2^112 - 75) are 16-byte little-endian words, the
 *    reference's serde form (src/algebra/field.rs:112-129).
 *  - Serialized objects are bincode 1.x (fixint, little endian) byte-identical to
 *    bincode::serialize of the reference types: Statement<8>
 *    (src/commitment/sis.rs:24-30), RoundRecord (src/protocol/prover.rs:14-21).
 *    A proof is bincode((Statement<8>, Vec<RoundRecord>, Fp)).
 *  - Buffers are caller-owned host memory unless the name says _device.
 *  - Return value: 0 on success, a negative DAMASCUS_E* code otherwise; the text
 *    of the last error of a context is available from damascus_last_error().
 *  - There is no CPU fallback: without a GB300 the context cannot be created.
 *  - A context serialises its synchronous calls; provers and verifiers created
 *    from one context may be driven from different threads (one thread each).
 */
#ifndef DAMASCUS_GB300_H
#define DAMASCUS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DAMASCUS_OK 0
#define DAMASCUS_EINVAL (-1)
#define DAMASCUS_ENOMEM_BUDGET (-2)
#define DAMASCUS_ECUDA (-3)
#define DAMASCUS_ETIMEOUT (-4)
#define DAMASCUS_EVERIFY (-5)
#define DAMASCUS_EINVARIANT (-6)
#define DAMASCUS_ESTATE (-7)
#define DAMASCUS_ESIZE (-8)
#define DAMASCUS_EDESERIALIZE (-9)
#define DAMASCUS_EUNSUPPORTED (-10)
#define DAMASCUS_ECANCELED (-11)

typedef struct damascus_ctx damascus_ctx;
typedef struct damascus_prover damascus_prover;
typedef struct damascus_verifier damascus_verifier;

/* ------------------------------------------------------------------ context */
/* Replaces the device probe of src/utils/gpu.rs:19-67 (cuda_backend_ready).
 * hbm_budget_bytes = 0 picks 90% of the free device memory. */
int damascus_ctx_create(int device, uint64_t hbm_budget_bytes, damascus_ctx** out);
void damascus_ctx_destroy(damascus_ctx* ctx);
const char* damascus_last_error(damascus_ctx* ctx);
/* Text of the last failure of damascus_ctx_create on this thread. */
const char* damascus_create_error(void);
uint64_t damascus_ctx_budget(damascus_ctx* ctx);
uint64_t damascus_ctx_reserved(damascus_ctx* ctx);
/* RuntimeConfig.max_preprocess_bytes (src/utils/config.rs:21, 69-87) of the
 * context's file entry points that take no limit of their own: damascus_prove,
 * damascus_prove_device(_timed), damascus_commit and engine submissions.  A file
 * whose witness expansion (2 x 16 bytes per coefficient of the square layout)
 * exceeds it fails with DAMASCUS_EINVAL and the reference's message
 * (src/utils/io.rs:42-49), as DamascusProver::initialize_with_config does.
 * 0 restores the reference default of 512 MiB (depth <= 12); a new context
 * starts there.  damascus_prover_new keeps its own argument. */
int damascus_ctx_set_max_preprocess_bytes(damascus_ctx* ctx, uint64_t max_preprocess_bytes);
uint64_t damascus_ctx_max_preprocess_bytes(damascus_ctx* ctx);

/* ------------------------------------------------------------------ field */
/* src/algebra/field.rs:137-198, 45-63, 106-109 */
void damascus_fp_add(const uint8_t a[16], const uint8_t b[16], uint8_t out[16]);
void damascus_fp_sub(const uint8_t a[16], const uint8_t b[16], uint8_t out[16]);
void damascus_fp_mul(const uint8_t a[16], const uint8_t b[16], uint8_t out[16]);
void damascus_fp_inv(const uint8_t a[16], uint8_t out[16]);
void damascus_fp_from_le_bytes_mod_order(const uint8_t* bytes, size_t len, uint8_t out[16]);

/* ------------------------------------------------------------------ host hashing */
/* blake3::hash / blake3::keyed_hash as used at src/utils/io.rs:33 and
 * src/commitment/sis.rs:208-210 (host implementation). */
void damascus_blake3(const uint8_t* data, size_t len, uint8_t out[32]);
void damascus_blake3_keyed(const uint8_t key[32], const uint8_t* data, size_t len, uint8_t out[32]);
/* Transcript::challenge_vec / challenge_poly (src/protocol/transcript.rs:22-80).
 * label is "vec" or "poly"; c, l, r are 8 x n_* field elements each. */
int damascus_transcript_challenge(const uint8_t epoch_seed[32], const uint8_t file_id[32], const char* label,
                                  uint64_t round, const uint8_t* c, uint64_t n_c, const uint8_t* l, uint64_t n_l,
                                  const uint8_t* r, uint64_t n_r, uint8_t out[16]);

/* ------------------------------------------------------------------ layout */
/* src/utils/io.rs:72-120: coefficient count, depth d and dimension 2^d. */
uint64_t damascus_coeff_count_for_byte_len(uint64_t byte_len);
int damascus_layout_for_byte_len(uint64_t byte_len, uint32_t* depth, uint64_t* dimension);
/* Bytes of one serialized proof / record / statement (bincode sizes). */
size_t damascus_proof_size(uint64_t file_len);
size_t damascus_record_size(uint64_t ring_len_vec, uint64_t ring_len_poly);
size_t damascus_statement_size(uint64_t ring_len);
/* Device memory one prover holds for a file of file_len bytes. */
uint64_t damascus_prover_footprint(uint64_t file_len);

/* ------------------------------------------------------------------ commitment */
/* blake3 file id on the GPU (src/utils/io.rs:33). */
int damascus_file_id(damascus_ctx* ctx, const uint8_t* file, size_t len, uint8_t out[32]);
/* derive_generator_families_from_seed (src/commitment/sis.rs:198-245): out is
 * vector_len x 8 x ring_len field elements, [vec][coord][coeff]. */
int damascus_derive_generators(damascus_ctx* ctx, const uint8_t g_seed[32], uint64_t vector_len, uint64_t ring_len,
                               uint8_t* out);
/* commit_with_generators_ntt (src/commitment/sis.rs:146-167): sum_i g_i * m_i in
 * R_q^8.  witness [N][n], generators [N][8][n], out [8][n]. */
int damascus_commit_with_generators(damascus_ctx* ctx, const uint8_t* witness, const uint8_t* generators,
                                    uint64_t vector_len, uint64_t ring_len, uint8_t* com_out);
/* ModuleSisCommitter::new(seed) + commit_with_ntt (src/commitment/sis.rs:68-70,
 * 115-131): the generators of an N x n witness are derived on the device from
 * keyed_hash(seed_generators, "g0"), with no host round trip.  witness [N][n],
 * out [8][n]; N = 0 writes the zero module of ring length one (8 x 16 bytes). */
int damascus_commit_witness(damascus_ctx* ctx, const uint8_t* witness, uint64_t vector_len, uint64_t ring_len,
                            const uint8_t seed_generators[32], uint8_t* com_out);
/* ModuleSisCommitter::new + register_with_ntt (src/commitment/sis.rs:68-70, 179-195)
 * via expand_file_to_square_polys (src/utils/io.rs:29-70): writes bincode(Statement).
 * The context's max_preprocess_bytes applies, as the expansion's limit. */
int damascus_commit(damascus_ctx* ctx, const uint8_t* file, size_t len, const uint8_t seed_generators[32],
                    uint8_t* statement_out, size_t cap, size_t* statement_len);
/* negacyclic_multiply (src/algebra/ntt.rs:112-195), batched: out_i = a_i * b_i in
 * R_q with ring degree n (a power of two <= 4096); arrays are count x n elements. */
int damascus_ring_mul_batch(damascus_ctx* ctx, const uint8_t* a, const uint8_t* b, uint8_t* out, uint64_t n,
                            uint64_t count);
/* Same on device-resident arrays (16-byte elements); asynchronous on the context
 * stream unless sync != 0. */
int damascus_ring_mul_batch_device(damascus_ctx* ctx, const void* d_a, const void* d_b, void* d_out, uint64_t n,
                                   uint64_t count, int sync);

/* ------------------------------------------------------------------ prover */
/* DamascusProver::initialize_with_config (src/protocol/prover.rs:61-111) with
 * SystemParams.seed_generators / epoch_seed and RuntimeConfig.max_preprocess_bytes
 * (0 = the reference default of 512 MiB). */
int damascus_prover_new(damascus_ctx* ctx, const uint8_t* file, size_t len, const uint8_t seed_generators[32],
                        const uint8_t epoch_seed[32], uint64_t max_preprocess_bytes, damascus_prover** out);
void damascus_prover_free(damascus_prover* p);
uint32_t damascus_prover_rounds_total(const damascus_prover* p);
uint64_t damascus_prover_current_round(const damascus_prover* p);
/* current_dimensions (prover.rs:125-127) */
void damascus_prover_dimensions(const damascus_prover* p, uint64_t* vector_len, uint64_t* ring_len);
/* statement() serialized (prover.rs:129-131) */
int damascus_prover_statement(const damascus_prover* p, uint8_t* buf, size_t cap, size_t* len);
/* current_commitment() as 8 x n field elements (prover.rs:121-123) */
int damascus_prover_current_commitment(const damascus_prover* p, uint8_t* buf, size_t cap, size_t* len);
/* fold_round(round) (prover.rs:140-313): writes bincode(RoundRecord).  A buffer
 * smaller than damascus_record_size(ring_len, ring_len / 2) fails with
 * DAMASCUS_ESIZE (and *record_len = the size needed) before the round runs. */
int damascus_prover_fold_round(damascus_prover* p, uint64_t round, uint8_t* record_out, size_t cap,
                               size_t* record_len);
/* The same, also returning RoundOutput's timings (prover.rs:26-31): the wall
 * time of the vector-fold stage, of the polynomial-fold stage and of the whole
 * round, in milliseconds (any may be null). */
int damascus_prover_fold_round_timed(damascus_prover* p, uint64_t round, uint8_t* record_out, size_t cap,
                                     size_t* record_len, double* vector_ms, double* poly_ms, double* total_ms);
/* final_opening (prover.rs:133-138); DAMASCUS_ESTATE before the last round. */
int damascus_prover_final_opening(const damascus_prover* p, uint8_t out[16]);

/* One-shot commit + d fold rounds + opening: writes
 * bincode((Statement, Vec<RoundRecord>, Fp)); capacity from damascus_proof_size().
 * The context's max_preprocess_bytes applies (damascus_ctx_set_max_preprocess_bytes). */
int damascus_prove(damascus_ctx* ctx, const uint8_t* file, size_t len, const uint8_t seed_generators[32],
                   const uint8_t epoch_seed[32], uint8_t* proof_out, size_t cap, size_t* proof_len);
/* Same with the file already in device memory. */
int damascus_prove_device(damascus_ctx* ctx, const void* d_file, size_t len, const uint8_t seed_generators[32],
                          const uint8_t epoch_seed[32], uint8_t* proof_out, size_t cap, size_t* proof_len);

/* damascus_prove_device, also returning the device time (CUDA events on the
 * prover's stream) from its first operation to its last. */
int damascus_prove_device_timed(damascus_ctx* ctx, const void* d_file, size_t len, const uint8_t seed_generators[32],
                                const uint8_t epoch_seed[32], uint8_t* proof_out, size_t cap, size_t* proof_len,
                                double* device_ms);

/* ------------------------------------------------------------------ verifier */
/* DamascusVerifier::new (src/protocol/verifier.rs:22-43) from bincode(Statement). */
int damascus_verifier_new(damascus_ctx* ctx, const uint8_t* statement, size_t len, const uint8_t epoch_seed[32],
                          damascus_verifier** out);
void damascus_verifier_free(damascus_verifier* v);
/* update_commitment (verifier.rs:57-120) from bincode(RoundRecord); a record that
 * does not deserialize returns DAMASCUS_EDESERIALIZE, a rejected one DAMASCUS_EVERIFY. */
int damascus_verifier_update_commitment(damascus_verifier* v, const uint8_t* record, size_t len);
/* verify_final_opening (verifier.rs:122-134): 0 accepts, DAMASCUS_EVERIFY rejects. */
int damascus_verifier_verify_final_opening(damascus_verifier* v, const uint8_t opening[16]);
uint64_t damascus_verifier_round(const damascus_verifier* v);
void damascus_verifier_dimensions(const damascus_verifier* v, uint64_t* vector_len, uint64_t* ring_len);
/* One-shot verification of a damascus_prove() proof: 0 accepts. */
int damascus_verify(damascus_ctx* ctx, const uint8_t* proof, size_t len, const uint8_t epoch_seed[32]);

/* ------------------------------------------------------------------ batching / serving */
/* Continuous-batching engine (no counterpart in the reference, which proves one
 * file at a time): submitted commit+prove requests are admitted against the
 * context's HBM budget, keep their state on the device across rounds, and the
 * same stage of every ready request runs in shared launches while host threads
 * compute the Fiat-Shamir challenges of others.  host_threads / max_waves <= 0
 * pick defaults (cores - 1 / 16 stage waves in flight, each on its own stream).
 * Proofs are the same bytes damascus_prove returns. */
typedef struct damascus_engine damascus_engine;
int damascus_engine_create(damascus_ctx* ctx, int host_threads, int max_waves, damascus_engine** out);
/* The engine's settings.  A negative value keeps the default, which the
 * DM_ENGINE_* environment variable named beside it overrides; host_threads and
 * max_waves keep theirs at 0. */
typedef struct damascus_engine_options {
    int host_threads;    /* Fiat-Shamir workers; 0: one fewer than the host's cores */
    int max_waves;       /* stage waves in flight, each on its own stream; 0: 16 */
    int priority_depth;  /* requests this deep or deeper run their stages on high-priority
                            streams; 0: no split; default 11 (DM_ENGINE_PRIORITY_DEPTH) */
    int polling;         /* 1: a poller thread queries each wave's completion event (default);
                            0: a host callback per wave (DM_ENGINE_POLL) */
    int spin_us;         /* awake wait of the scheduler and two workers before they block;
                            0: block at once; default 200 (DM_ENGINE_SPIN_US) */
    int admission_batch; /* admissions per scheduling pass while a request is ready; 0: every
                            queued request that fits first; default 1 (DM_ENGINE_ADMIT_BATCH) */
} damascus_engine_options;
/* damascus_engine_create with every setting; opts NULL: the defaults. */
int damascus_engine_create_with_options(damascus_ctx* ctx, const damascus_engine_options* opts,
                                        damascus_engine** out);
void damascus_engine_destroy(damascus_engine* e);
/* Copies the file and returns at once with a ticket.  The context's
 * max_preprocess_bytes applies at admission: a larger file's request fails with
 * DAMASCUS_EINVAL (from poll / wait) and leaves the others undisturbed. */
int damascus_engine_submit(damascus_engine* e, const uint8_t* file, size_t len, const uint8_t seed_generators[32],
                           const uint8_t epoch_seed[32], uint64_t* ticket);
/* Same with the file already in device memory; d_file must stay valid until the
 * request finishes. */
int damascus_engine_submit_device(damascus_engine* e, const void* d_file, size_t len,
                                  const uint8_t seed_generators[32], const uint8_t epoch_seed[32], uint64_t* ticket);
/* Same with the file in host memory that the caller keeps valid and unchanged
 * until the request finishes: the engine's host-to-device copy reads it
 * directly, with no copy into the engine's staging buffer.  Page-locked memory
 * (cudaHostAlloc, cudaHostRegister) keeps that copy asynchronous. */
int damascus_engine_submit_borrowed(damascus_engine* e, const uint8_t* file, size_t len,
                                    const uint8_t seed_generators[32], const uint8_t epoch_seed[32], uint64_t* ticket);
/* 1 = finished (proof kept for damascus_engine_take), 0 = running, < 0 = failed. */
int damascus_engine_poll(damascus_engine* e, uint64_t ticket, size_t* proof_len, double* latency_ms);
/* Blocks until the ticket finishes; same results as poll. */
int damascus_engine_wait(damascus_engine* e, uint64_t ticket, size_t* proof_len, double* latency_ms);
/* Blocks until one of the n tickets has finished (its proof is ready or it
 * failed) and sets *which to that ticket's index in tickets; poll or wait then
 * returns its result at once.  A client collecting many requests takes each
 * proof as soon as it is ready this way, not in submission order.  Tickets the
 * engine does not know are skipped; DAMASCUS_EINVAL when it knows none. */
int damascus_engine_wait_any(damascus_engine* e, const uint64_t* tickets, size_t n, size_t* which);
/* wait with a limit: DAMASCUS_ETIMEOUT when the request has not finished within
 * timeout_ms; it keeps running and the ticket stays valid. */
int damascus_engine_wait_timeout(damascus_engine* e, uint64_t ticket, double timeout_ms, size_t* proof_len,
                                 double* latency_ms);
/* Ends a request early.  A queued request ends at once; an admitted one at its
 * next stage boundary: a stage already on the GPU completes first, so no kernel
 * is interrupted.  The request then finishes with DAMASCUS_ECANCELED (from poll
 * or wait) and releases its memory; the others are undisturbed.
 * DAMASCUS_ESTATE when it had already finished, DAMASCUS_EINVAL for an unknown
 * ticket. */
int damascus_engine_cancel(damascus_engine* e, uint64_t ticket);
/* Requests submitted from now on fail with DAMASCUS_ETIMEOUT when still
 * unfinished timeout_ms after their submission (checked at admission and at
 * stage boundaries, as cancel is).  0 removes the limit. */
int damascus_engine_set_request_timeout(damascus_engine* e, double timeout_ms);
/* Admissions per scheduling pass while an admitted request is ready to launch
 * (default 1: the engine launches after each admission, so the GPU starts on the
 * first requests while later ones are set up and requests submitted together do
 * not run their stages in lockstep).  0 admits every queued request that fits
 * the budget before launching, which coalesces their first stages into one
 * wave. */
int damascus_engine_set_admission_batch(damascus_engine* e, int requests_per_pass);
/* Watchdog reading: unfinished requests and the milliseconds since any stage
 * (or request) finished, 0 while nothing is unfinished.  No kernel of the engine
 * waits on a flag, so an age that keeps growing with requests unfinished points
 * at the host side or a stalled device; the caller decides what to do. */
int damascus_engine_health(damascus_engine* e, uint64_t* unfinished, double* ms_since_progress);
/* Copies a finished proof out and forgets it (DAMASCUS_ESIZE keeps it). */
int damascus_engine_take(damascus_engine* e, uint64_t ticket, uint8_t* proof_out, size_t cap);
/* Points *data at a finished proof of *len bytes that the engine still holds
 * (no copy): valid until damascus_engine_take or damascus_engine_release of the
 * ticket, or the engine's destruction.  A binding that builds its own byte
 * object from it copies the proof once.  DAMASCUS_ESTATE when the ticket has no
 * finished proof waiting. */
int damascus_engine_result(damascus_engine* e, uint64_t ticket, const uint8_t** data, size_t* len);
/* Forgets a finished proof without copying it out. */
int damascus_engine_release(damascus_engine* e, uint64_t ticket);
int damascus_engine_drain(damascus_engine* e);
int damascus_engine_stats(damascus_engine* e, uint64_t* completed, uint64_t* failed, uint64_t* waves,
                          uint64_t* launches, uint64_t* peak_reserved_bytes);
/* Where the engine's time went: summed host time of the Fiat-Shamir stage parts
 * (all workers), and wall time with no stage wave on the GPU while admitted
 * requests were unfinished. */
int damascus_engine_profile(damascus_engine* e, double* host_stage_ms, double* gpu_idle_ms);
/* The scheduler thread's busy time: admitting requests (setup and their Init
 * stage launches) and planning and launching stage waves, in milliseconds. */
int damascus_engine_scheduler_profile(damascus_engine* e, double* admit_ms, double* launch_ms);

/* Streaming verifier service (no counterpart in the reference, which verifies
 * one proof at a time through DamascusVerifier, src/protocol/verifier.rs:22-134).
 * Proofs in the damascus_prove() container are verified by `workers` threads
 * (<= 0: one per host core, at most 16), each on its own stream, admitted in
 * arrival order against the context's HBM budget.  Initial generator families
 * g_0(seed, N, n) are kept in HBM, up to cache_bytes (0 disables), and shared by
 * proofs of the same shape and system seed.  Each verdict equals
 * damascus_verify()'s on the same bytes. */
typedef struct damascus_verify_service damascus_verify_service;
int damascus_verify_service_create(damascus_ctx* ctx, int workers, uint64_t cache_bytes,
                                   damascus_verify_service** out);
/* Finishes the submitted proofs, then frees the service. */
void damascus_verify_service_destroy(damascus_verify_service* s);
/* Copies the proof and returns at once with a ticket. */
int damascus_verify_service_submit(damascus_verify_service* s, const uint8_t* proof, size_t len,
                                   const uint8_t epoch_seed[32], uint64_t* ticket);
/* 1 = finished: *verdict = DAMASCUS_OK for an accepted proof, else the code
 * damascus_verify() returns (its text via damascus_last_error); the ticket is
 * then forgotten.  0 = still running; DAMASCUS_EINVAL = unknown ticket. */
int damascus_verify_service_poll(damascus_verify_service* s, uint64_t ticket, int* verdict, double* latency_ms);
/* Blocks until the ticket finishes; same results as poll. */
int damascus_verify_service_wait(damascus_verify_service* s, uint64_t ticket, int* verdict, double* latency_ms);
int damascus_verify_service_drain(damascus_verify_service* s);
int damascus_verify_service_stats(damascus_verify_service* s, uint64_t* completed, uint64_t* accepted,
                                  uint64_t* rejected, uint64_t* cache_hits, uint64_t* cache_misses,
                                  uint64_t* peak_reserved_bytes);

/* ------------------------------------------------------------------ reference FFI */
/* Drop-in for the reference's own CUDA hooks, same signatures and argument
 * meaning (src/utils/gpu.rs:69-93; cuda/fold_kernel.cu:209, cuda/ntt_kernel.cu:106).
 * damascus_cuda_fold_batch: out = left + right * challenge (mod q) over len
 * elements given as split lo/hi 64-bit halves.
 * damascus_cuda_ntt_batch: for each of the 8 CRT primes, the length-n cyclic
 * convolution of host_a and host_b (8 x n residues each) into host_out; the root
 * tables are accepted for ABI compatibility and checked for shape only.
 * Both return 0 on success and a positive step code on failure, as the
 * reference's callers expect (gpu.rs:122-131, 191-193). */
int damascus_cuda_fold_batch(const uint64_t* left_lo, const uint64_t* left_hi, const uint64_t* right_lo,
                             const uint64_t* right_hi, uint64_t* out_lo, uint64_t* out_hi, size_t len,
                             uint64_t challenge_lo, uint64_t challenge_hi);
int damascus_cuda_ntt_batch(const uint64_t* host_a, const uint64_t* host_b, uint64_t* host_out, size_t n,
                            const uint64_t* primes, const uint64_t* stage_roots, const uint64_t* inv_roots,
                            const uint64_t* inv_sizes);

/* BLAKE3 hash of len bytes already in device memory -- the same 32 bytes
 * damascus_file_id returns for them -- for callers that cannot allocate device
 * memory: serving loops confined to a pre-reserved budget, and hosts whose
 * device allocator belongs to another framework.  It has no counterpart in the
 * reference.
 * d_file: len bytes of device memory; d_out32: 32 bytes of device memory; the
 * kernels run asynchronously on `stream` (a cudaStream_t, 0 for the default
 * stream) on the current device.  The call makes no device allocation: its
 * scratch is a 4 MiB static device array that every device loading this library
 * holds until exit, so len is limited to 64 MiB (larger returns DAMASCUS_ESIZE):
 * files of depth <= 11 fit, those of depth 12 and 13 do not.
 * The first call on a device resolves that array's address (cudaGetSymbolAddress)
 * and should come before any stream capture; a failed resolution is retried by
 * the next call.  All calls share the array and nothing in it needs clearing
 * between calls; calls that overlap on the GPU (other streams, or other threads)
 * race on it and must be serialised. */
int damascus_file_id_noalloc(const void* d_file, size_t len, void* d_out32, void* stream);

/* ------------------------------------------------------------------ generator cache */
/* Provers' initial generator families g_0(seed, S) and their forward transforms
 * kept in HBM (no reference counterpart: the reference expands them for every
 * proof, src/commitment/sis.rs:198-245).  A (seed, ring size) pair is cached the
 * second time a prover of this context sees it, up to cap_bytes (charged to the
 * context budget; requests come first and evict unreferenced entries).  The
 * reference's SystemParams::default uses one seed for every file
 * (src/utils/config.rs:19, 33-44), so a deployment expands and transforms each
 * shape once; per-file seeds only pay a lookup.  Verifiers of the context
 * (damascus_verify, the verifier service) read a cached family's coefficients as
 * their initial generators instead of expanding them.  Off by default; 0 turns
 * it off (DAMASCUS_ESTATE while a running prover or verifier holds an entry).
 * Proof bytes and verdicts never depend on it. */
int damascus_ctx_set_generator_cache(damascus_ctx* ctx, uint64_t cap_bytes);
int damascus_ctx_generator_cache_stats(damascus_ctx* ctx, uint64_t* hits, uint64_t* fills, uint64_t* misses,
                                       uint64_t* bytes);

/* ------------------------------------------------------------------ measurement */
/* Per-kernel CUDA-event timing on the launching stream (off by default). */
int damascus_ctx_set_profiling(damascus_ctx* ctx, int on);
void damascus_ctx_reset_stats(damascus_ctx* ctx);
/* Launch trace (turns profiling on): from here every timed launch group (one
 * kernel kind of one stage, on its stream) is kept with its stream number and
 * its start and end in milliseconds after this call. */
int damascus_ctx_trace_start(damascus_ctx* ctx);
/* Waits for the traced work and writes CSV lines "kind,stream,start_ms,end_ms,
 * algo_bytes,kernels" (a start is when the stream reached the group).  Engines
 * add host rows on the same time base: "sched_wave" / "sched_wave_deep" (a
 * wave's planning and launching: its stream, request count and launches),
 * "wave_done" (the wave's completion callback) and "fiat_shamir" (one request's
 * host step; the second field is its depth), and per request stage, with the
 * request's ticket in the fifth field, "req_wait" (ready until its wave
 * launched), "req_gpu" (launched until the completion callback) and "req_host"
 * (callback until its host step finished).  A small buffer gives
 * DAMASCUS_ESIZE and *len = the bytes needed; the lines are kept for the next
 * call.  stop != 0 ends the trace. */
int damascus_ctx_trace_read(damascus_ctx* ctx, char* buf, size_t cap, size_t* len, int stop);
/* 0 and fills the totals if the kernel ran since the last reset. */
int damascus_ctx_kernel_stat(damascus_ctx* ctx, const char* name, uint64_t* launches, double* total_ms,
                             double* algo_bytes, double* algo_ops);
/* Waits for all work queued on the device. */
int damascus_ctx_synchronize(damascus_ctx* ctx);
/* Writes 256 MiB (more than the 129 MB L2) on the context stream and waits. */
int damascus_ctx_flush_l2(damascus_ctx* ctx);
/* Measured issue rates (operations per second, best of three launches after a
 * warm-up) of the three integer multiply forms the forward transform spends its
 * multiplier on: [0] 32-bit multiply-add, [1] high half of a 32 x 32 product,
 * [2] 32 x 32 -> 64 multiply-add.  The peaks against which bench.py states the
 * transform's counted multiplies (no reference counterpart). */
int damascus_measure_int_multiply(damascus_ctx* ctx, double ops_per_s[3]);

/* ------------------------------------------------------------------ launch-shape tuning */
/* Knobs of the kernels' launch shapes per ring size 2^log_ring (no reference
 * counterpart: the reference has no device launch shapes).  Defaults are the
 * built-in choices; damascus000_gb300/autotune.py measures the candidates with
 * damascus_tuning_measure and sets the fastest.  Results never depend on them. */
enum {
    DAMASCUS_TUNE_NTT_GROUP = 0,  /* threads per block of the forward transform, rings below 2^10: 32 or 64 */
    DAMASCUS_TUNE_MAC_TRIPLE = 1, /* resident blocks per SM the column split of a triple MAC fills: 1..32 */
    DAMASCUS_TUNE_MAC_SPLIT = 2,  /* the same for the split (vector-stage) MAC */
    DAMASCUS_TUNE_MAC_PLAIN = 3,  /* the same for the single-sum MAC */
    DAMASCUS_TUNE_SPLIT_COORDS = 4, /* commitment coordinates per thread of the split MAC: 1, 2, 4 or 8 */
    DAMASCUS_TUNE_TRIPLE_COORDS = 5, /* the same for the triple MAC: 1, 2 or 4 */
    DAMASCUS_TUNE_NTT_RADIX = 6      /* residues per thread of the forward transform, rings of 2^5 and up: 16 or 32
                                        (radix-16 or radix-32 register passes) */
};
int damascus_tuning_set(damascus_ctx* ctx, int knob, uint32_t log_ring, int value);
int damascus_tuning_get(damascus_ctx* ctx, int knob, uint32_t log_ring, int* value);
/* Mean device time of one launch over `reps` launches (CUDA events, context
 * stream, after one warm-up launch) of the knob's kernel with `value`, on
 * synthetic device data: `count` polynomials (transform), column pairs (triple
 * MAC: one launch over full pairs plus one in the form whose second witness
 * half is known zero, both timed) or columns (split, single-sum MAC). */
int damascus_tuning_measure(damascus_ctx* ctx, int knob, uint32_t log_ring, int value, uint32_t count, int reps,
                            double* ms_per_launch);

#ifdef __cplusplus
}
#endif
#endif
