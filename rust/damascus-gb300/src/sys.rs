//! Raw declarations of every entry point of `include/damascus.h` (the C ABI of
//! libdamascus_gb300.so), one `pub fn` per C function with the same name,
//! argument order and meaning.  Fixed-size C arrays (`uint8_t out[16]`) are
//! pointers to that many bytes.  Return codes: 0 on success, a negative
//! `DAMASCUS_E*` value otherwise (the reference FFI hooks return positive step
//! codes, as `damascus-core`'s callers expect).
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub const DAMASCUS_OK: c_int = 0;
pub const DAMASCUS_EINVAL: c_int = -1;
pub const DAMASCUS_ENOMEM_BUDGET: c_int = -2;
pub const DAMASCUS_ECUDA: c_int = -3;
pub const DAMASCUS_ETIMEOUT: c_int = -4;
pub const DAMASCUS_EVERIFY: c_int = -5;
pub const DAMASCUS_EINVARIANT: c_int = -6;
pub const DAMASCUS_ESTATE: c_int = -7;
pub const DAMASCUS_ESIZE: c_int = -8;
pub const DAMASCUS_EDESERIALIZE: c_int = -9;
pub const DAMASCUS_EUNSUPPORTED: c_int = -10;
pub const DAMASCUS_ECANCELED: c_int = -11;

pub const DAMASCUS_TUNE_NTT_GROUP: c_int = 0;
pub const DAMASCUS_TUNE_MAC_TRIPLE: c_int = 1;
pub const DAMASCUS_TUNE_MAC_SPLIT: c_int = 2;
pub const DAMASCUS_TUNE_MAC_PLAIN: c_int = 3;
pub const DAMASCUS_TUNE_SPLIT_COORDS: c_int = 4;
pub const DAMASCUS_TUNE_TRIPLE_COORDS: c_int = 5;
pub const DAMASCUS_TUNE_NTT_RADIX: c_int = 6;

/// Opaque handles (never constructed on the Rust side).
#[repr(C)]
pub struct Ctx {
    _p: [u8; 0],
}
#[repr(C)]
pub struct Prover {
    _p: [u8; 0],
}
#[repr(C)]
pub struct Verifier {
    _p: [u8; 0],
}
/// `damascus_engine_options`: a negative value keeps the default (which the
/// DM_ENGINE_* environment variable overrides); host_threads and max_waves keep
/// theirs at 0.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct EngineOptions {
    pub host_threads: c_int,
    pub max_waves: c_int,
    pub priority_depth: c_int,
    pub polling: c_int,
    pub spin_us: c_int,
    pub admission_batch: c_int,
}

impl Default for EngineOptions {
    fn default() -> Self {
        EngineOptions { host_threads: 0, max_waves: 0, priority_depth: -1, polling: -1, spin_us: -1, admission_batch: -1 }
    }
}

#[repr(C)]
pub struct Engine {
    _p: [u8; 0],
}
#[repr(C)]
pub struct VerifyService {
    _p: [u8; 0],
}

extern "C" {
    pub fn damascus_ctx_create(device: c_int, hbm_budget_bytes: u64, out: *mut *mut Ctx) -> c_int;
    pub fn damascus_ctx_destroy(ctx: *mut Ctx);
    pub fn damascus_last_error(ctx: *mut Ctx) -> *const c_char;
    pub fn damascus_create_error() -> *const c_char;
    pub fn damascus_ctx_budget(ctx: *mut Ctx) -> u64;
    pub fn damascus_ctx_reserved(ctx: *mut Ctx) -> u64;
    pub fn damascus_ctx_set_max_preprocess_bytes(ctx: *mut Ctx, max_preprocess_bytes: u64) -> c_int;
    pub fn damascus_ctx_max_preprocess_bytes(ctx: *mut Ctx) -> u64;
    pub fn damascus_fp_add(a: *const u8, b: *const u8, out: *mut u8);
    pub fn damascus_fp_sub(a: *const u8, b: *const u8, out: *mut u8);
    pub fn damascus_fp_mul(a: *const u8, b: *const u8, out: *mut u8);
    pub fn damascus_fp_inv(a: *const u8, out: *mut u8);
    pub fn damascus_fp_from_le_bytes_mod_order(bytes: *const u8, len: usize, out: *mut u8);
    pub fn damascus_blake3(data: *const u8, len: usize, out: *mut u8);
    pub fn damascus_blake3_keyed(key: *const u8, data: *const u8, len: usize, out: *mut u8);
    pub fn damascus_transcript_challenge(epoch_seed: *const u8, file_id: *const u8, label: *const c_char, round: u64, c: *const u8, n_c: u64, l: *const u8, n_l: u64, r: *const u8, n_r: u64, out: *mut u8) -> c_int;
    pub fn damascus_coeff_count_for_byte_len(byte_len: u64) -> u64;
    pub fn damascus_layout_for_byte_len(byte_len: u64, depth: *mut u32, dimension: *mut u64) -> c_int;
    pub fn damascus_proof_size(file_len: u64) -> usize;
    pub fn damascus_record_size(ring_len_vec: u64, ring_len_poly: u64) -> usize;
    pub fn damascus_statement_size(ring_len: u64) -> usize;
    pub fn damascus_prover_footprint(file_len: u64) -> u64;
    pub fn damascus_file_id(ctx: *mut Ctx, file: *const u8, len: usize, out: *mut u8) -> c_int;
    pub fn damascus_derive_generators(ctx: *mut Ctx, g_seed: *const u8, vector_len: u64, ring_len: u64, out: *mut u8) -> c_int;
    pub fn damascus_commit_with_generators(ctx: *mut Ctx, witness: *const u8, generators: *const u8, vector_len: u64, ring_len: u64, com_out: *mut u8) -> c_int;
    pub fn damascus_commit_witness(ctx: *mut Ctx, witness: *const u8, vector_len: u64, ring_len: u64, seed_generators: *const u8, com_out: *mut u8) -> c_int;
    pub fn damascus_commit(ctx: *mut Ctx, file: *const u8, len: usize, seed_generators: *const u8, statement_out: *mut u8, cap: usize, statement_len: *mut usize) -> c_int;
    pub fn damascus_ring_mul_batch(ctx: *mut Ctx, a: *const u8, b: *const u8, out: *mut u8, n: u64, count: u64) -> c_int;
    pub fn damascus_ring_mul_batch_device(ctx: *mut Ctx, d_a: *const c_void, d_b: *const c_void, d_out: *mut c_void, n: u64, count: u64, sync: c_int) -> c_int;
    pub fn damascus_prover_new(ctx: *mut Ctx, file: *const u8, len: usize, seed_generators: *const u8, epoch_seed: *const u8, max_preprocess_bytes: u64, out: *mut *mut Prover) -> c_int;
    pub fn damascus_prover_free(p: *mut Prover);
    pub fn damascus_prover_rounds_total(p: *const Prover) -> u32;
    pub fn damascus_prover_current_round(p: *const Prover) -> u64;
    pub fn damascus_prover_dimensions(p: *const Prover, vector_len: *mut u64, ring_len: *mut u64);
    pub fn damascus_prover_statement(p: *const Prover, buf: *mut u8, cap: usize, len: *mut usize) -> c_int;
    pub fn damascus_prover_current_commitment(p: *const Prover, buf: *mut u8, cap: usize, len: *mut usize) -> c_int;
    pub fn damascus_prover_fold_round(p: *mut Prover, round: u64, record_out: *mut u8, cap: usize, record_len: *mut usize) -> c_int;
    pub fn damascus_prover_fold_round_timed(p: *mut Prover, round: u64, record_out: *mut u8, cap: usize, record_len: *mut usize, vector_ms: *mut f64, poly_ms: *mut f64, total_ms: *mut f64) -> c_int;
    pub fn damascus_prover_final_opening(p: *const Prover, out: *mut u8) -> c_int;
    pub fn damascus_prove(ctx: *mut Ctx, file: *const u8, len: usize, seed_generators: *const u8, epoch_seed: *const u8, proof_out: *mut u8, cap: usize, proof_len: *mut usize) -> c_int;
    pub fn damascus_prove_device(ctx: *mut Ctx, d_file: *const c_void, len: usize, seed_generators: *const u8, epoch_seed: *const u8, proof_out: *mut u8, cap: usize, proof_len: *mut usize) -> c_int;
    pub fn damascus_prove_device_timed(ctx: *mut Ctx, d_file: *const c_void, len: usize, seed_generators: *const u8, epoch_seed: *const u8, proof_out: *mut u8, cap: usize, proof_len: *mut usize, device_ms: *mut f64) -> c_int;
    pub fn damascus_verifier_new(ctx: *mut Ctx, statement: *const u8, len: usize, epoch_seed: *const u8, out: *mut *mut Verifier) -> c_int;
    pub fn damascus_verifier_free(v: *mut Verifier);
    pub fn damascus_verifier_update_commitment(v: *mut Verifier, record: *const u8, len: usize) -> c_int;
    pub fn damascus_verifier_verify_final_opening(v: *mut Verifier, opening: *const u8) -> c_int;
    pub fn damascus_verifier_round(v: *const Verifier) -> u64;
    pub fn damascus_verifier_dimensions(v: *const Verifier, vector_len: *mut u64, ring_len: *mut u64);
    pub fn damascus_verify(ctx: *mut Ctx, proof: *const u8, len: usize, epoch_seed: *const u8) -> c_int;
    pub fn damascus_engine_create(ctx: *mut Ctx, host_threads: c_int, max_waves: c_int, out: *mut *mut Engine) -> c_int;
    pub fn damascus_engine_create_with_options(ctx: *mut Ctx, opts: *const EngineOptions, out: *mut *mut Engine) -> c_int;
    pub fn damascus_engine_destroy(e: *mut Engine);
    pub fn damascus_engine_submit(e: *mut Engine, file: *const u8, len: usize, seed_generators: *const u8, epoch_seed: *const u8, ticket: *mut u64) -> c_int;
    pub fn damascus_engine_submit_device(e: *mut Engine, d_file: *const c_void, len: usize, seed_generators: *const u8, epoch_seed: *const u8, ticket: *mut u64) -> c_int;
    pub fn damascus_engine_submit_borrowed(e: *mut Engine, file: *const u8, len: usize, seed_generators: *const u8, epoch_seed: *const u8, ticket: *mut u64) -> c_int;
    pub fn damascus_engine_poll(e: *mut Engine, ticket: u64, proof_len: *mut usize, latency_ms: *mut f64) -> c_int;
    pub fn damascus_engine_wait(e: *mut Engine, ticket: u64, proof_len: *mut usize, latency_ms: *mut f64) -> c_int;
    pub fn damascus_engine_wait_any(e: *mut Engine, tickets: *const u64, n: usize, which: *mut usize) -> c_int;
    pub fn damascus_engine_wait_timeout(e: *mut Engine, ticket: u64, timeout_ms: f64, proof_len: *mut usize, latency_ms: *mut f64) -> c_int;
    pub fn damascus_engine_cancel(e: *mut Engine, ticket: u64) -> c_int;
    pub fn damascus_engine_set_request_timeout(e: *mut Engine, timeout_ms: f64) -> c_int;
    pub fn damascus_engine_set_admission_batch(e: *mut Engine, requests_per_pass: c_int) -> c_int;
    pub fn damascus_engine_health(e: *mut Engine, unfinished: *mut u64, ms_since_progress: *mut f64) -> c_int;
    pub fn damascus_engine_take(e: *mut Engine, ticket: u64, proof_out: *mut u8, cap: usize) -> c_int;
    pub fn damascus_engine_result(e: *mut Engine, ticket: u64, data: *mut *const u8, len: *mut usize) -> c_int;
    pub fn damascus_engine_release(e: *mut Engine, ticket: u64) -> c_int;
    pub fn damascus_engine_drain(e: *mut Engine) -> c_int;
    pub fn damascus_engine_stats(e: *mut Engine, completed: *mut u64, failed: *mut u64, waves: *mut u64, launches: *mut u64, peak_reserved_bytes: *mut u64) -> c_int;
    pub fn damascus_ctx_trace_start(ctx: *mut Ctx) -> c_int;
    pub fn damascus_ctx_trace_read(ctx: *mut Ctx, buf: *mut c_char, cap: usize, len: *mut usize, stop: c_int) -> c_int;
    pub fn damascus_engine_profile(e: *mut Engine, host_stage_ms: *mut f64, gpu_idle_ms: *mut f64) -> c_int;
    pub fn damascus_engine_scheduler_profile(e: *mut Engine, admit_ms: *mut f64, launch_ms: *mut f64) -> c_int;
    pub fn damascus_verify_service_create(ctx: *mut Ctx, workers: c_int, cache_bytes: u64, out: *mut *mut VerifyService) -> c_int;
    pub fn damascus_verify_service_destroy(s: *mut VerifyService);
    pub fn damascus_verify_service_submit(s: *mut VerifyService, proof: *const u8, len: usize, epoch_seed: *const u8, ticket: *mut u64) -> c_int;
    pub fn damascus_verify_service_poll(s: *mut VerifyService, ticket: u64, verdict: *mut c_int, latency_ms: *mut f64) -> c_int;
    pub fn damascus_verify_service_wait(s: *mut VerifyService, ticket: u64, verdict: *mut c_int, latency_ms: *mut f64) -> c_int;
    pub fn damascus_verify_service_drain(s: *mut VerifyService) -> c_int;
    pub fn damascus_verify_service_stats(s: *mut VerifyService, completed: *mut u64, accepted: *mut u64, rejected: *mut u64, cache_hits: *mut u64, cache_misses: *mut u64, peak_reserved_bytes: *mut u64) -> c_int;
    pub fn damascus_cuda_fold_batch(left_lo: *const u64, left_hi: *const u64, right_lo: *const u64, right_hi: *const u64, out_lo: *mut u64, out_hi: *mut u64, len: usize, challenge_lo: u64, challenge_hi: u64) -> c_int;
    pub fn damascus_cuda_ntt_batch(host_a: *const u64, host_b: *const u64, host_out: *mut u64, n: usize, primes: *const u64, stage_roots: *const u64, inv_roots: *const u64, inv_sizes: *const u64) -> c_int;
    pub fn damascus_file_id_noalloc(d_file: *const c_void, len: usize, d_out32: *mut c_void, stream: *mut c_void) -> c_int;
    pub fn damascus_ctx_set_generator_cache(ctx: *mut Ctx, cap_bytes: u64) -> c_int;
    pub fn damascus_ctx_generator_cache_stats(ctx: *mut Ctx, hits: *mut u64, fills: *mut u64, misses: *mut u64, bytes: *mut u64) -> c_int;
    pub fn damascus_ctx_set_profiling(ctx: *mut Ctx, on: c_int) -> c_int;
    pub fn damascus_ctx_reset_stats(ctx: *mut Ctx);
    pub fn damascus_ctx_kernel_stat(ctx: *mut Ctx, name: *const c_char, launches: *mut u64, total_ms: *mut f64, algo_bytes: *mut f64, algo_ops: *mut f64) -> c_int;
    pub fn damascus_ctx_synchronize(ctx: *mut Ctx) -> c_int;
    pub fn damascus_ctx_flush_l2(ctx: *mut Ctx) -> c_int;
    pub fn damascus_measure_int_multiply(ctx: *mut Ctx, ops_per_s: *mut f64) -> c_int;
    pub fn damascus_tuning_set(ctx: *mut Ctx, knob: c_int, log_ring: u32, value: c_int) -> c_int;
    pub fn damascus_tuning_get(ctx: *mut Ctx, knob: c_int, log_ring: u32, value: *mut c_int) -> c_int;
    pub fn damascus_tuning_measure(ctx: *mut Ctx, knob: c_int, log_ring: u32, value: c_int, count: u32, reps: c_int, ms_per_launch: *mut f64) -> c_int;
}
