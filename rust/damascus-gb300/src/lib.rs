//! Safe Rust API over libdamascus_gb300, the GB300 (sm_103a) Damascus Fold
//! prover/verifier, for `damascus-core` behind DAMASCUS_GPU=1.
//!
//! Mirrors the reference crate's entry points (paths relative to its root):
//! `DamascusProver::initialize_with_config` / `fold_round` / `final_opening`
//! (src/protocol/prover.rs:61-138, 140-313) as [`Prover`];
//! `DamascusVerifier::new` / `update_commitment` / `verify_final_opening`
//! (src/protocol/verifier.rs:22-134) as [`Verifier`];
//! `ModuleSisCommitter::commit_with_ntt` (src/commitment/sis.rs:115-131) as
//! [`Context::commit_witness`]; `negacyclic_multiply` (src/algebra/ntt.rs:112)
//! as [`Context::ring_mul_batch`]; and the reference's own CUDA hooks
//! (src/utils/gpu.rs:69-207) in [`gpu`].  Statements, records and proofs cross
//! as their bincode 1.x bytes, byte-identical to the reference types, so the
//! caller deserializes them with its own `bincode::deserialize`.  Field
//! elements are 16-byte little-endian words.  There is no CPU fallback: without
//! a GB300 (or with DAMASCUS_GPU=0 at build time) every constructor fails.
//!
//! Not compiled here: neither the build machine nor the GPU machine of this
//! repository has cargo or rustc; the Python binding (damascus000_gb300) and
//! the tests exercise the same C entry points.

pub mod gpu;
pub mod sys;

use std::fmt;
#[cfg(damascus_cuda_available)]
use std::os::raw::c_int;

/// A negative `DAMASCUS_E*` code with the library's message.
#[derive(Clone, Debug, PartialEq, Eq)]
pub struct Error {
    pub code: i32,
    pub message: String,
}

impl fmt::Display for Error {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        write!(f, "damascus_gb300 error {}: {}", self.code, self.message)
    }
}

impl std::error::Error for Error {}

pub type Result<T> = std::result::Result<T, Error>;

#[cfg(damascus_cuda_available)]
fn cstr(p: *const std::os::raw::c_char) -> String {
    if p.is_null() {
        return String::new();
    }
    unsafe { std::ffi::CStr::from_ptr(p) }.to_string_lossy().into_owned()
}

#[cfg(not(damascus_cuda_available))]
fn unavailable<T>() -> Result<T> {
    Err(Error { code: sys::DAMASCUS_ECUDA, message: "built without libdamascus_gb300 (DAMASCUS_GPU=0)".into() })
}

/// A device, its stream, tables and HBM budget (`damascus_ctx`).
pub struct Context {
    #[allow(dead_code)]
    raw: *mut sys::Ctx,
}

// The library serialises a context's synchronous calls; provers and verifiers
// made from it may run on other threads (one thread each).
unsafe impl Send for Context {}
unsafe impl Sync for Context {}

#[cfg(damascus_cuda_available)]
impl Context {
    /// `hbm_budget_bytes = 0` takes 90 % of the device's free memory.
    pub fn new(device: i32, hbm_budget_bytes: u64) -> Result<Self> {
        let mut raw = std::ptr::null_mut();
        let rc = unsafe { sys::damascus_ctx_create(device as c_int, hbm_budget_bytes, &mut raw) };
        if rc != 0 {
            return Err(Error { code: rc, message: cstr(unsafe { sys::damascus_create_error() }) });
        }
        Ok(Context { raw })
    }

    fn check(&self, rc: c_int) -> Result<()> {
        if rc == 0 {
            Ok(())
        } else {
            Err(Error { code: rc, message: cstr(unsafe { sys::damascus_last_error(self.raw) }) })
        }
    }

    /// RuntimeConfig::max_preprocess_bytes of prove, commit and engine
    /// submissions (0: the reference default of 512 MiB).
    pub fn set_max_preprocess_bytes(&self, bytes: u64) -> Result<()> {
        self.check(unsafe { sys::damascus_ctx_set_max_preprocess_bytes(self.raw, bytes) })
    }

    /// bincode((Statement, Vec<RoundRecord>, Fp)) of commit + d fold rounds + opening.
    pub fn prove(&self, file: &[u8], seed_generators: &[u8; 32], epoch_seed: &[u8; 32]) -> Result<Vec<u8>> {
        let cap = unsafe { sys::damascus_proof_size(file.len() as u64) };
        let mut out = vec![0u8; cap];
        let mut len = 0usize;
        self.check(unsafe {
            sys::damascus_prove(self.raw, file.as_ptr(), file.len(), seed_generators.as_ptr(), epoch_seed.as_ptr(),
                                out.as_mut_ptr(), cap, &mut len)
        })?;
        out.truncate(len);
        Ok(out)
    }

    /// Ok(true) accepts, Ok(false) rejects (DAMASCUS_EVERIFY or a record that does
    /// not deserialize); other failures are errors.
    pub fn verify(&self, proof: &[u8], epoch_seed: &[u8; 32]) -> Result<bool> {
        match unsafe { sys::damascus_verify(self.raw, proof.as_ptr(), proof.len(), epoch_seed.as_ptr()) } {
            0 => Ok(true),
            sys::DAMASCUS_EVERIFY | sys::DAMASCUS_EDESERIALIZE => Ok(false),
            rc => self.check(rc).map(|_| false),
        }
    }

    /// bincode(Statement) of `ModuleSisCommitter::new(seed)` + `register_with_ntt`
    /// over the file's square witness.
    pub fn commit(&self, file: &[u8], seed_generators: &[u8; 32]) -> Result<Vec<u8>> {
        let (mut depth, mut dim) = (0u32, 0u64);
        self.check(unsafe { sys::damascus_layout_for_byte_len(file.len() as u64, &mut depth, &mut dim) })?;
        let cap = unsafe { sys::damascus_statement_size(dim) };
        let mut out = vec![0u8; cap];
        let mut len = 0usize;
        self.check(unsafe {
            sys::damascus_commit(self.raw, file.as_ptr(), file.len(), seed_generators.as_ptr(), out.as_mut_ptr(), cap,
                                 &mut len)
        })?;
        out.truncate(len);
        Ok(out)
    }

    /// `commit_with_ntt`: witness is `vector_len` polynomials of `ring_len`
    /// 16-byte coefficients; returns 8 coordinates of `ring_len` words.
    pub fn commit_witness(&self, witness: &[u8], vector_len: usize, ring_len: usize, seed_generators: &[u8; 32])
                          -> Result<Vec<u8>> {
        if witness.len() != vector_len * ring_len * 16 {
            return Err(Error { code: sys::DAMASCUS_EINVAL, message: "witness length is not N x n x 16".into() });
        }
        let mut out = vec![0u8; 8 * ring_len.max(1) * 16];
        self.check(unsafe {
            sys::damascus_commit_witness(self.raw, witness.as_ptr(), vector_len as u64, ring_len as u64,
                                         seed_generators.as_ptr(), out.as_mut_ptr())
        })?;
        Ok(out)
    }

    /// `negacyclic_multiply` of `count` pairs of degree-`n` polynomials.
    pub fn ring_mul_batch(&self, a: &[u8], b: &[u8], n: usize, count: usize) -> Result<Vec<u8>> {
        if a.len() != n * count * 16 || b.len() != a.len() {
            return Err(Error { code: sys::DAMASCUS_EINVAL, message: "operands are not count x n x 16 bytes".into() });
        }
        let mut out = vec![0u8; a.len()];
        self.check(unsafe {
            sys::damascus_ring_mul_batch(self.raw, a.as_ptr(), b.as_ptr(), out.as_mut_ptr(), n as u64, count as u64)
        })?;
        Ok(out)
    }

    /// Keeps provers' initial generator families in HBM up to `cap_bytes` (0: off).
    pub fn set_generator_cache(&self, cap_bytes: u64) -> Result<()> {
        self.check(unsafe { sys::damascus_ctx_set_generator_cache(self.raw, cap_bytes) })
    }
}

#[cfg(not(damascus_cuda_available))]
impl Context {
    pub fn new(_device: i32, _hbm_budget_bytes: u64) -> Result<Self> {
        unavailable()
    }
}

impl Drop for Context {
    fn drop(&mut self) {
        #[cfg(damascus_cuda_available)]
        unsafe {
            sys::damascus_ctx_destroy(self.raw)
        }
    }
}

/// `DamascusProver` on the GPU: witness, generators and fold state stay in HBM
/// across rounds.
#[cfg(damascus_cuda_available)]
pub struct Prover<'c> {
    ctx: &'c Context,
    raw: *mut sys::Prover,
}

#[cfg(damascus_cuda_available)]
impl<'c> Prover<'c> {
    /// `initialize_with_config` with SystemParams.seed_generators / epoch_seed and
    /// RuntimeConfig.max_preprocess_bytes (0: 512 MiB).
    pub fn new(ctx: &'c Context, file: &[u8], seed_generators: &[u8; 32], epoch_seed: &[u8; 32],
               max_preprocess_bytes: u64) -> Result<Self> {
        let mut raw = std::ptr::null_mut();
        ctx.check(unsafe {
            sys::damascus_prover_new(ctx.raw, file.as_ptr(), file.len(), seed_generators.as_ptr(), epoch_seed.as_ptr(),
                                     max_preprocess_bytes, &mut raw)
        })?;
        Ok(Prover { ctx, raw })
    }

    pub fn rounds_total(&self) -> u32 {
        unsafe { sys::damascus_prover_rounds_total(self.raw) }
    }

    /// (vector_len, ring_len) of the current round.
    pub fn current_dimensions(&self) -> (u64, u64) {
        let (mut a, mut b) = (0u64, 0u64);
        unsafe { sys::damascus_prover_dimensions(self.raw, &mut a, &mut b) };
        (a, b)
    }

    /// bincode(Statement).
    pub fn statement(&self) -> Result<Vec<u8>> {
        let (_, n) = self.current_dimensions();
        let cap = unsafe { sys::damascus_statement_size(n) };
        let mut out = vec![0u8; cap];
        let mut len = 0usize;
        self.ctx.check(unsafe { sys::damascus_prover_statement(self.raw, out.as_mut_ptr(), cap, &mut len) })?;
        out.truncate(len);
        Ok(out)
    }

    /// bincode(RoundRecord) of `fold_round(round)`.
    pub fn fold_round(&mut self, round: u64) -> Result<Vec<u8>> {
        let (nv, np) = self.current_dimensions();
        let cap = unsafe { sys::damascus_record_size(nv, (np / 2).max(1)) };
        let mut out = vec![0u8; cap];
        let mut len = 0usize;
        self.ctx.check(unsafe { sys::damascus_prover_fold_round(self.raw, round, out.as_mut_ptr(), cap, &mut len) })?;
        out.truncate(len);
        Ok(out)
    }

    /// `fold_round` with `RoundOutput`'s timings (src/protocol/prover.rs:26-31):
    /// the record and the vector-fold, poly-fold and whole-round wall times.
    pub fn fold_round_timed(&mut self, round: u64) -> Result<(Vec<u8>, [std::time::Duration; 3])> {
        let (nv, np) = self.current_dimensions();
        let cap = unsafe { sys::damascus_record_size(nv, (np / 2).max(1)) };
        let mut out = vec![0u8; cap];
        let mut len = 0usize;
        let mut ms = [0f64; 3];
        let [v, p, t] = &mut ms;
        self.ctx.check(unsafe {
            sys::damascus_prover_fold_round_timed(self.raw, round, out.as_mut_ptr(), cap, &mut len, v, p, t)
        })?;
        out.truncate(len);
        Ok((out, ms.map(|x| std::time::Duration::from_secs_f64(x / 1000.0))))
    }

    /// The terminal opening m* (16-byte LE) once every round has run.
    pub fn final_opening(&self) -> Result<[u8; 16]> {
        let mut out = [0u8; 16];
        self.ctx.check(unsafe { sys::damascus_prover_final_opening(self.raw, out.as_mut_ptr()) })?;
        Ok(out)
    }
}

#[cfg(damascus_cuda_available)]
impl Drop for Prover<'_> {
    fn drop(&mut self) {
        unsafe { sys::damascus_prover_free(self.raw) }
    }
}

/// `DamascusVerifier`: host transcript replay, device generator folds.
#[cfg(damascus_cuda_available)]
pub struct Verifier<'c> {
    ctx: &'c Context,
    raw: *mut sys::Verifier,
}

#[cfg(damascus_cuda_available)]
impl<'c> Verifier<'c> {
    pub fn new(ctx: &'c Context, statement: &[u8], epoch_seed: &[u8; 32]) -> Result<Self> {
        let mut raw = std::ptr::null_mut();
        ctx.check(unsafe {
            sys::damascus_verifier_new(ctx.raw, statement.as_ptr(), statement.len(), epoch_seed.as_ptr(), &mut raw)
        })?;
        Ok(Verifier { ctx, raw })
    }

    /// Ok(false): the record was rejected (or does not deserialize).
    pub fn update_commitment(&mut self, record: &[u8]) -> Result<bool> {
        match unsafe { sys::damascus_verifier_update_commitment(self.raw, record.as_ptr(), record.len()) } {
            0 => Ok(true),
            sys::DAMASCUS_EVERIFY | sys::DAMASCUS_EDESERIALIZE => Ok(false),
            rc => self.ctx.check(rc).map(|_| false),
        }
    }

    pub fn verify_final_opening(&mut self, opening: &[u8; 16]) -> Result<bool> {
        match unsafe { sys::damascus_verifier_verify_final_opening(self.raw, opening.as_ptr()) } {
            0 => Ok(true),
            sys::DAMASCUS_EVERIFY => Ok(false),
            rc => self.ctx.check(rc).map(|_| false),
        }
    }
}

#[cfg(damascus_cuda_available)]
impl Drop for Verifier<'_> {
    fn drop(&mut self) {
        unsafe { sys::damascus_verifier_free(self.raw) }
    }
}

/// The continuous-batching engine: files submitted from any thread are proven
/// concurrently under the context's HBM budget; each proof equals
/// [`Context::prove`]'s bytes.
#[cfg(damascus_cuda_available)]
pub struct Engine<'c> {
    ctx: &'c Context,
    raw: *mut sys::Engine,
}

#[cfg(damascus_cuda_available)]
unsafe impl Send for Engine<'_> {}
#[cfg(damascus_cuda_available)]
unsafe impl Sync for Engine<'_> {}

#[cfg(damascus_cuda_available)]
impl<'c> Engine<'c> {
    /// `host_threads` / `max_waves` <= 0 take the library's defaults.
    pub fn new(ctx: &'c Context, host_threads: i32, max_waves: i32) -> Result<Self> {
        let mut raw = std::ptr::null_mut();
        ctx.check(unsafe { sys::damascus_engine_create(ctx.raw, host_threads, max_waves, &mut raw) })?;
        Ok(Engine { ctx, raw })
    }

    /// With every setting (`sys::EngineOptions::default()` keeps the library's).
    pub fn with_options(ctx: &'c Context, opts: &sys::EngineOptions) -> Result<Self> {
        let mut raw = std::ptr::null_mut();
        ctx.check(unsafe { sys::damascus_engine_create_with_options(ctx.raw, opts, &mut raw) })?;
        Ok(Engine { ctx, raw })
    }

    /// Copies the file and returns a ticket at once.
    pub fn submit(&self, file: &[u8], seed_generators: &[u8; 32], epoch_seed: &[u8; 32]) -> Result<u64> {
        let mut ticket = 0u64;
        self.ctx.check(unsafe {
            sys::damascus_engine_submit(self.raw, file.as_ptr(), file.len(), seed_generators.as_ptr(),
                                        epoch_seed.as_ptr(), &mut ticket)
        })?;
        Ok(ticket)
    }

    /// Submits a file the engine reads in place (no staging copy).
    ///
    /// # Safety
    /// `file` must stay valid and unchanged until the request finishes (its
    /// `wait` returned); page-locked memory keeps the device copy asynchronous.
    pub unsafe fn submit_borrowed(&self, file: &[u8], seed_generators: &[u8; 32], epoch_seed: &[u8; 32]) -> Result<u64> {
        let mut ticket = 0u64;
        self.ctx.check(sys::damascus_engine_submit_borrowed(self.raw, file.as_ptr(), file.len(), seed_generators.as_ptr(),
                                                            epoch_seed.as_ptr(), &mut ticket))?;
        Ok(ticket)
    }

    /// Blocks until one of `tickets` has finished; returns its index (its `wait`
    /// then returns at once), so proofs are taken in the order they finish.
    pub fn wait_any(&self, tickets: &[u64]) -> Result<usize> {
        let mut which = 0usize;
        self.ctx.check(unsafe { sys::damascus_engine_wait_any(self.raw, tickets.as_ptr(), tickets.len(), &mut which) })?;
        Ok(which)
    }

    /// Blocks until the ticket finishes: (proof, latency in ms).
    pub fn wait(&self, ticket: u64) -> Result<(Vec<u8>, f64)> {
        let (mut len, mut ms) = (0usize, 0f64);
        let rc = unsafe { sys::damascus_engine_wait(self.raw, ticket, &mut len, &mut ms) };
        if rc < 0 {
            return self.ctx.check(rc).map(|_| (Vec::new(), 0.0));
        }
        // one copy, from the engine's buffer into the returned vector
        let mut data: *const u8 = std::ptr::null();
        self.ctx.check(unsafe { sys::damascus_engine_result(self.raw, ticket, &mut data, &mut len) })?;
        let out = if len == 0 { Vec::new() } else { unsafe { std::slice::from_raw_parts(data, len) }.to_vec() };
        self.ctx.check(unsafe { sys::damascus_engine_release(self.raw, ticket) })?;
        Ok((out, ms))
    }
}

#[cfg(damascus_cuda_available)]
impl Drop for Engine<'_> {
    fn drop(&mut self) {
        unsafe { sys::damascus_engine_destroy(self.raw) }
    }
}
