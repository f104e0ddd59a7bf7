// extern "C" entry points declared in include/damascus.h.
#include <cuda_runtime.h>
#include <execinfo.h>
#include <signal.h>
#include <unistd.h>

#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/damascus.h"
#include "dm_jobs.cuh"
#include "dm_tables.h"
#include "engine.h"
#include "proof.h"
#include "serve.h"
#include "host_blake3.h"
#include "verify_service.h"

using namespace dm;

struct damascus_ctx {
    Context* ctx;
    std::string err_copy;
    std::string trace;  // trace lines read from the context, not yet copied out
};
struct damascus_prover {
    damascus_ctx* owner;
    GpuProver* p;
};
struct damascus_verifier {
    damascus_ctx* owner;
    GpuVerifier* v;
};
struct damascus_verify_service {
    damascus_ctx* owner;
    VerifyService* s;
};
struct damascus_engine {
    damascus_ctx* owner;
    Engine* e;
    std::mutex mu;
    std::map<uint64_t, std::vector<uint8_t>> results;
    std::map<uint64_t, std::pair<int, double>> status;
};

namespace {

thread_local std::string g_create_error;

// With DAMASCUS_CRASH_TRACE=1 in the environment, a fatal signal in any thread
// of the process prints the native backtrace of that thread, then hands the
// signal to the handler that was installed before (e.g. Python's faulthandler).
using SigHandler = void (*)(int);
SigHandler g_prev_handler[32];
void crash_trace(int sig) {
    void* frames[64];
    const int n = backtrace(frames, 64);
    const char msg[] = "damascus: fatal signal, native backtrace:\n";
    (void)!write(2, msg, sizeof(msg) - 1);
    backtrace_symbols_fd(frames, n, 2);
    SigHandler prev = sig < 32 ? g_prev_handler[sig] : SIG_DFL;
    signal(sig, prev == SIG_ERR || prev == nullptr ? SIG_DFL : prev);
    raise(sig);
}
struct CrashTraceInstaller {
    CrashTraceInstaller() {
        const char* v = getenv("DAMASCUS_CRASH_TRACE");
        if (v && v[0] == '1')
            for (int sig : {SIGSEGV, SIGBUS, SIGABRT}) g_prev_handler[sig] = signal(sig, crash_trace);
    }
} g_crash_trace_installer;

// Reference default of RuntimeConfig.max_preprocess_bytes (src/utils/config.rs:21, 69-87).
constexpr uint64_t kDefaultMaxPreprocess = Context::kDefaultMaxPreprocess;

int set_err(damascus_ctx* c, int code, const std::string& msg) {
    if (c) c->ctx->set_error(msg);
    return code;
}

// Scoped device buffer for the synchronous helpers (charged to the budget).
struct Scratch {
    DevMem m;
    int alloc(Context* c, size_t b) { return m.alloc(c, b); }
};

fq fq_arg(const uint8_t* p) { return fq_from_u128_words(fq_from_bytes(p)); }

bool pow2(uint64_t v) { return v && !(v & (v - 1)); }
uint32_t log2u(uint64_t v) {
    uint32_t l = 0;
    while ((1ull << l) < v) ++l;
    return l;
}

}  // namespace

extern "C" {

// ------------------------------------------------------------------ context
int damascus_ctx_create(int device, uint64_t hbm_budget_bytes, damascus_ctx** out) {
    if (!out) return DAMASCUS_EINVAL;
    Context* c = nullptr;
    std::string err;
    int rc = Context::create(device, hbm_budget_bytes, &c, &err);
    if (rc != kOk) {
        g_create_error = err;
        *out = nullptr;
        return rc;
    }
    *out = new damascus_ctx{c, {}};
    return DAMASCUS_OK;
}

void damascus_ctx_destroy(damascus_ctx* ctx) {
    if (!ctx) return;
    delete ctx->ctx;
    delete ctx;
}

const char* damascus_last_error(damascus_ctx* ctx) {
    if (!ctx) return "null context";
    ctx->err_copy = ctx->ctx->last_error();
    return ctx->err_copy.c_str();
}

const char* damascus_create_error(void) { return g_create_error.c_str(); }
uint64_t damascus_ctx_budget(damascus_ctx* ctx) { return ctx ? ctx->ctx->budget() : 0; }
uint64_t damascus_ctx_reserved(damascus_ctx* ctx) { return ctx ? ctx->ctx->reserved() : 0; }

// ------------------------------------------------------------------ field
void damascus_fp_add(const uint8_t a[16], const uint8_t b[16], uint8_t out[16]) {
    fq_to_bytes(fq_add(fq_arg(a), fq_arg(b)), out);
}
void damascus_fp_sub(const uint8_t a[16], const uint8_t b[16], uint8_t out[16]) {
    fq_to_bytes(fq_sub(fq_arg(a), fq_arg(b)), out);
}
void damascus_fp_mul(const uint8_t a[16], const uint8_t b[16], uint8_t out[16]) {
    fq_to_bytes(fq_mul(fq_arg(a), fq_arg(b)), out);
}
void damascus_fp_inv(const uint8_t a[16], uint8_t out[16]) { fq_to_bytes(fq_inv(fq_arg(a)), out); }
void damascus_fp_from_le_bytes_mod_order(const uint8_t* bytes, size_t len, uint8_t out[16]) {
    // Horner over 16-byte words from the most significant end: acc = acc * 2^128 + w.
    fq acc = fq_zero();
    fq two128;  // 2^128 mod q = 2^16 * 75
    {
        uint32_t r[8] = {0, 0, 0, 0, 1, 0, 0, 0};
        two128 = fq_reduce8(r);
    }
    size_t nwords = (len + 15) / 16;
    for (size_t w = nwords; w-- > 0;) {
        uint8_t buf[16] = {0};
        const size_t off = w * 16, n = len - off < 16 ? len - off : 16;
        std::memcpy(buf, bytes + off, n);
        acc = fq_add(fq_mul(acc, two128), fq_from_u128_words(fq_from_bytes(buf)));
    }
    fq_to_bytes(acc, out);
}

// ------------------------------------------------------------------ hashing
void damascus_blake3(const uint8_t* data, size_t len, uint8_t out[32]) { blake3_hash_parallel(data, len, out); }
void damascus_blake3_keyed(const uint8_t key[32], const uint8_t* data, size_t len, uint8_t out[32]) {
    blake3_keyed_hash(key, data, len, out);
}

int damascus_transcript_challenge(const uint8_t epoch_seed[32], const uint8_t file_id[32], const char* label,
                                  uint64_t round, const uint8_t* c, uint64_t n_c, const uint8_t* l, uint64_t n_l,
                                  const uint8_t* r, uint64_t n_r, uint8_t out[16]) {
    auto load = [](const uint8_t* p, uint64_t n) {
        Module m = Module::zero((uint32_t)n);
        for (size_t i = 0; i < m.c.size(); ++i) m.c[i] = fq_arg(p + 16 * i);
        return m;
    };
    Transcript t(epoch_seed, file_id);
    const Module mc = load(c, n_c), ml = load(l, n_l), mr = load(r, n_r);
    fq v;
    if (std::strcmp(label, "vec") == 0)
        v = t.challenge_vec(round, mc, ml, mr);
    else if (std::strcmp(label, "poly") == 0)
        v = t.challenge_poly(round, mc, ml, mr);
    else
        return DAMASCUS_EINVAL;
    fq_to_bytes(v, out);
    return DAMASCUS_OK;
}

// ------------------------------------------------------------------ layout
uint64_t damascus_coeff_count_for_byte_len(uint64_t byte_len) { return coeff_count_for_byte_len(byte_len); }
int damascus_layout_for_byte_len(uint64_t byte_len, uint32_t* depth, uint64_t* dimension) {
    return square_layout_for_byte_len(byte_len, depth, dimension) ? DAMASCUS_OK : DAMASCUS_EINVAL;
}
size_t damascus_proof_size(uint64_t file_len) {
    uint32_t d;
    uint64_t dim;
    if (!square_layout_for_byte_len(file_len, &d, &dim)) return 0;
    return proof_encoded_size(d);
}
size_t damascus_record_size(uint64_t nv, uint64_t np) { return record_encoded_size((uint32_t)nv, (uint32_t)np); }
size_t damascus_statement_size(uint64_t n) { return statement_encoded_size((uint32_t)n); }
uint64_t damascus_prover_footprint(uint64_t file_len) { return GpuProver::footprint(file_len); }

// ------------------------------------------------------------------ commitment
int damascus_file_id(damascus_ctx* ctx, const uint8_t* file, size_t len, uint8_t out[32]) {
    if (!ctx || (!file && len)) return DAMASCUS_EINVAL;
    Context* C = ctx->ctx;
    std::lock_guard<std::mutex> g(C->mutex());
    cudaSetDevice(C->device());
    Scratch f, sc, o;
    if (f.alloc(C, len + 16) || sc.alloc(C, file_hash_scratch_words(len) * 4) || o.alloc(C, 32))
        return set_err(ctx, DAMASCUS_ENOMEM_BUDGET, "HBM budget exhausted");
    cudaStream_t s = C->stream();
    cudaError_t e = len ? cudaMemcpyAsync(f.m.as<uint8_t>(), file, len, cudaMemcpyHostToDevice, s) : cudaSuccess;
    if (e == cudaSuccess) e = launch_file_hash(f.m.as<uint8_t>(), len, sc.m.as<uint32_t>(), o.m.as<uint32_t>(), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, o.m.as<uint8_t>(), 32, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_err(ctx, DAMASCUS_ECUDA, std::string("file_id: ") + cudaGetErrorString(e));
    return DAMASCUS_OK;
}

int damascus_derive_generators(damascus_ctx* ctx, const uint8_t g_seed[32], uint64_t N, uint64_t n, uint8_t* out) {
    if (!ctx || !out || !pow2(n) || n > (1u << kLogMaxProverRing) || N == 0) return set_err(ctx, DAMASCUS_EINVAL, "bad generator shape");
    Context* C = ctx->ctx;
    std::lock_guard<std::mutex> g(C->mutex());
    cudaSetDevice(C->device());
    const size_t bytes = N * kRank * n * 16;
    Scratch gb;
    if (gb.alloc(C, bytes)) return set_err(ctx, DAMASCUS_ENOMEM_BUDGET, "HBM budget exhausted");
    cudaStream_t s = C->stream();
    cudaError_t e = launch_gen_generators(g_seed, N, log2u(n), gb.m.as<uint4>(), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, gb.m.as<uint8_t>(), bytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_err(ctx, DAMASCUS_ECUDA, std::string("derive_generators: ") + cudaGetErrorString(e));
    return DAMASCUS_OK;
}

// The commitment sum_i g_i * m_i (sis.rs:146-167) of a host witness with the
// generators either copied from the host (and reduced mod q, as any 128-bit words
// are accepted) or expanded on the device from g_seed.
static int commit_common(damascus_ctx* ctx, const uint8_t* witness, const uint8_t* generators,
                         const uint8_t g_seed[32], uint64_t N, uint64_t n, uint8_t* com_out, const char* what) {
    if (!ctx || !witness || !(generators || g_seed) || !com_out || N == 0 || !pow2(n) ||
        n > (1u << kLogMaxProverRing))
        return set_err(ctx, DAMASCUS_EINVAL, "bad commitment shape");
    // CRT headroom of the single NTT-domain sum: N * n * q^2 < P / 2 (P > 2^251).
    if (N * n > (1ull << 26)) return set_err(ctx, DAMASCUS_EUNSUPPORTED, "N * n above 2^26 exceeds the CRT range");
    if (N > 0xFFFFFFFFull / kRank) return set_err(ctx, DAMASCUS_EINVAL, "too many columns");
    Context* C = ctx->ctx;
    std::lock_guard<std::mutex> g(C->mutex());
    cudaSetDevice(C->device());
    const DeviceTables& T = C->tables();
    const uint32_t L = log2u(n);
    const uint32_t rows = kRank * kPrimes;
    const uint32_t parts = C->mac_parts(kTuneMacPlain, L, (uint32_t)n, (uint32_t)N);
    Scratch m, gg, mh, gh, part, out;
    if (m.alloc(C, N * n * 16) || gg.alloc(C, N * kRank * n * 16) || mh.alloc(C, N * kPrimes * n * 4) ||
        gh.alloc(C, N * kRank * kPrimes * n * 4) || part.alloc(C, (size_t)parts * rows * n * 4) ||
        out.alloc(C, kRank * n * 16))
        return set_err(ctx, DAMASCUS_ENOMEM_BUDGET, "HBM budget exhausted");
    cudaStream_t s = C->stream();
    NttJob nj[2] = {{m.m.as<uint4>(), mh.m.as<uint32_t>(), (uint32_t)N, 0},
                    {gg.m.as<uint4>(), gh.m.as<uint32_t>(), (uint32_t)(N * kRank), 0}};
    MacJobX mj{gh.m.as<uint32_t>(), mh.m.as<uint32_t>(), part.m.as<uint32_t>(), nullptr, nullptr, 0, 0, (uint32_t)N,
               parts, 0, 0, L};
    FinishJobX fj{part.m.as<uint32_t>(), out.m.as<uint4>(), nullptr, nullptr, parts, kFinishPlain, rows, 0};
    cudaError_t e = cudaMemcpyAsync(m.m.as<uint8_t>(), witness, N * n * 16, cudaMemcpyHostToDevice, s);
    // inputs may be any 128-bit words: reduce them mod q first
    if (e == cudaSuccess) e = launch_canon(m.m.as<uint4>(), N * n, s);
    if (generators) {
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(gg.m.as<uint8_t>(), generators, N * kRank * n * 16, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = launch_canon(gg.m.as<uint4>(), N * kRank * n, s);
    } else if (e == cudaSuccess) {
        e = launch_gen_generators(g_seed, N, L, gg.m.as<uint4>(), s);  // already below q
    }
    if (e == cudaSuccess) e = launch_ntt_jobs(T, nj, 2, L, s, C->tuning(kTuneNttGroup, L), C->tuning(kTuneNttRadix, L));
    if (e == cudaSuccess) e = launch_mac_jobs(T, &mj, 1, false, s);
    if (e == cudaSuccess) e = launch_finish_jobs(T, &fj, 1, L, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(com_out, out.m.as<uint8_t>(), kRank * n * 16, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_err(ctx, DAMASCUS_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return DAMASCUS_OK;
}

int damascus_commit_with_generators(damascus_ctx* ctx, const uint8_t* witness, const uint8_t* generators, uint64_t N,
                                    uint64_t n, uint8_t* com_out) {
    if (!generators) return set_err(ctx, DAMASCUS_EINVAL, "null generators");
    return commit_common(ctx, witness, generators, nullptr, N, n, com_out, "commit_with_generators");
}

int damascus_commit_witness(damascus_ctx* ctx, const uint8_t* witness, uint64_t N, uint64_t n,
                            const uint8_t seed_generators[32], uint8_t* com_out) {
    if (!ctx || !seed_generators || !com_out) return set_err(ctx, DAMASCUS_EINVAL, "null argument");
    if (N == 0) {  // an empty witness commits to the zero module of ring length one (sis.rs:120-122)
        std::memset(com_out, 0, kRank * 16);
        return DAMASCUS_OK;
    }
    uint8_t g_seed[32];
    blake3_keyed_hash(seed_generators, "g0", 2, g_seed);  // ModuleSisCommitter::new, sis.rs:68-70
    return commit_common(ctx, witness, nullptr, g_seed, N, n, com_out, "commit_witness");
}

int damascus_commit(damascus_ctx* ctx, const uint8_t* file, size_t len, const uint8_t seed_generators[32],
                    uint8_t* statement_out, size_t cap, size_t* statement_len) {
    if (!ctx || (!file && len) || !seed_generators) return DAMASCUS_EINVAL;
    static const uint8_t kZeroEpoch[32] = {0};
    GpuProver p(ctx->ctx);
    int rc = p.init(file, len, false, seed_generators, kZeroEpoch, ctx->ctx->max_preprocess());
    if (rc != kOk) return rc;
    std::vector<uint8_t> buf;
    encode_statement(buf, p.statement());
    if (statement_len) *statement_len = buf.size();
    if (!statement_out || cap < buf.size()) return set_err(ctx, DAMASCUS_ESIZE, "statement buffer too small");
    std::memcpy(statement_out, buf.data(), buf.size());
    return DAMASCUS_OK;
}

int damascus_ring_mul_batch_device(damascus_ctx* ctx, const void* d_a, const void* d_b, void* d_out, uint64_t n,
                                   uint64_t count, int sync);

int damascus_ring_mul_batch(damascus_ctx* ctx, const uint8_t* a, const uint8_t* b, uint8_t* out, uint64_t n,
                            uint64_t count) {
    if (!ctx || !a || !b || !out || !pow2(n) || n > (1u << kLogMaxProverRing)) return set_err(ctx, DAMASCUS_EINVAL, "bad ring shape");
    if (count == 0) return DAMASCUS_OK;
    Context* C = ctx->ctx;
    Scratch da, db, dout;
    const size_t bytes = count * n * 16;
    {
        std::lock_guard<std::mutex> g(C->mutex());
        cudaSetDevice(C->device());
        if (da.alloc(C, bytes) || db.alloc(C, bytes) || dout.alloc(C, bytes))
            return set_err(ctx, DAMASCUS_ENOMEM_BUDGET, "HBM budget exhausted");
        cudaError_t e = cudaMemcpyAsync(da.m.as<uint8_t>(), a, bytes, cudaMemcpyHostToDevice, C->stream());
        if (e == cudaSuccess) e = cudaMemcpyAsync(db.m.as<uint8_t>(), b, bytes, cudaMemcpyHostToDevice, C->stream());
        if (e == cudaSuccess) e = launch_canon(da.m.as<uint4>(), count * n, C->stream());
        if (e == cudaSuccess) e = launch_canon(db.m.as<uint4>(), count * n, C->stream());
        if (e != cudaSuccess) return set_err(ctx, DAMASCUS_ECUDA, std::string("H2D: ") + cudaGetErrorString(e));
    }
    int rc = damascus_ring_mul_batch_device(ctx, da.m.as<void>(), db.m.as<void>(), dout.m.as<void>(), n, count, 0);
    if (rc != DAMASCUS_OK) return rc;
    std::lock_guard<std::mutex> g(C->mutex());
    cudaError_t e = cudaMemcpyAsync(out, dout.m.as<uint8_t>(), bytes, cudaMemcpyDeviceToHost, C->stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(C->stream());
    if (e != cudaSuccess) return set_err(ctx, DAMASCUS_ECUDA, std::string("D2H: ") + cudaGetErrorString(e));
    return DAMASCUS_OK;
}

int damascus_ring_mul_batch_device(damascus_ctx* ctx, const void* d_a, const void* d_b, void* d_out, uint64_t n,
                                   uint64_t count, int sync) {
    if (!ctx || !pow2(n) || n > (1u << kLogMaxProverRing)) return set_err(ctx, DAMASCUS_EINVAL, "bad ring shape");
    if (count == 0) return DAMASCUS_OK;
    if (count * kPrimes > 0xFFFFFFFFull || ((count * kPrimes * n) >> 8) > 0xFFFFFFFFull)
        return set_err(ctx, DAMASCUS_EINVAL, "too many products in one call");
    Context* C = ctx->ctx;
    std::lock_guard<std::mutex> g(C->mutex());
    cudaSetDevice(C->device());
    const DeviceTables& T = C->tables();
    const uint32_t L = log2u(n);
    Scratch ra, rb;
    if (ra.alloc(C, count * kPrimes * n * 4) || rb.alloc(C, count * kPrimes * n * 4))
        return set_err(ctx, DAMASCUS_ENOMEM_BUDGET, "HBM budget exhausted");
    cudaStream_t s = C->stream();
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (C->profiling()) {
        e0 = C->take_event();
        cudaEventRecord(e0, s);
    }
    NttJob nj[2] = {{static_cast<const uint4*>(d_a), ra.m.as<uint32_t>(), (uint32_t)count, 0},
                    {static_cast<const uint4*>(d_b), rb.m.as<uint32_t>(), (uint32_t)count, 0}};
    cudaError_t e = launch_ntt_jobs(T, nj, 2, L, s, C->tuning(kTuneNttGroup, L), C->tuning(kTuneNttRadix, L));
    if (e0) {
        e1 = C->take_event();
        cudaEventRecord(e1, s);
        C->record("ntt_fwd", e0, e1, (double)count * n * (32 + 2 * kPrimes * 4), (double)2 * count * kPrimes * (n / 2) * L);
        e0 = C->take_event();
        cudaEventRecord(e0, s);
    }
    // slotwise products feed the inverse transform directly (no product buffer)
    FinishJobX fj{ra.m.as<uint32_t>(), static_cast<uint4*>(d_out), nullptr, nullptr, 1, kFinishPlain,
                  (uint32_t)(count * kPrimes), 0, rb.m.as<uint32_t>()};
    if (e == cudaSuccess) e = launch_finish_jobs(T, &fj, 1, L, s);
    if (e0) {
        e1 = C->take_event();
        cudaEventRecord(e1, s);
        C->record("ring_mul", e0, e1, (double)count * n * (2 * kPrimes * 4 + 16), (double)count * kPrimes * (n / 2) * L, 2);
    }
    // Scratch is released when this returns: wait for the kernels that read it.
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    (void)sync;
    if (e != cudaSuccess) return set_err(ctx, DAMASCUS_ECUDA, std::string("ring_mul: ") + cudaGetErrorString(e));
    return DAMASCUS_OK;
}

// ------------------------------------------------------------------ prover
int damascus_prover_new(damascus_ctx* ctx, const uint8_t* file, size_t len, const uint8_t seed_generators[32],
                        const uint8_t epoch_seed[32], uint64_t max_preprocess_bytes, damascus_prover** out) {
    if (!ctx || !out || (!file && len) || !seed_generators || !epoch_seed) return DAMASCUS_EINVAL;
    GpuProver* p = new GpuProver(ctx->ctx);
    int rc = p->init(file, len, false, seed_generators, epoch_seed,
                     max_preprocess_bytes ? max_preprocess_bytes : kDefaultMaxPreprocess);
    if (rc != kOk) {
        delete p;
        *out = nullptr;
        return rc;
    }
    *out = new damascus_prover{ctx, p};
    return DAMASCUS_OK;
}

void damascus_prover_free(damascus_prover* p) {
    if (!p) return;
    delete p->p;
    delete p;
}
uint32_t damascus_prover_rounds_total(const damascus_prover* p) { return p ? p->p->rounds_total() : 0; }
uint64_t damascus_prover_current_round(const damascus_prover* p) { return p ? p->p->current_round() : 0; }
void damascus_prover_dimensions(const damascus_prover* p, uint64_t* N, uint64_t* n) {
    if (N) *N = p ? p->p->vector_len() : 0;
    if (n) *n = p ? p->p->ring_len() : 0;
}

int damascus_prover_statement(const damascus_prover* p, uint8_t* buf, size_t cap, size_t* len) {
    if (!p) return DAMASCUS_EINVAL;
    std::vector<uint8_t> v;
    encode_statement(v, p->p->statement());
    if (len) *len = v.size();
    if (!buf || cap < v.size()) return DAMASCUS_ESIZE;
    std::memcpy(buf, v.data(), v.size());
    return DAMASCUS_OK;
}

int damascus_prover_current_commitment(const damascus_prover* p, uint8_t* buf, size_t cap, size_t* len) {
    if (!p) return DAMASCUS_EINVAL;
    const Module& m = p->p->current_commitment();
    const size_t need = m.c.size() * 16;
    if (len) *len = need;
    if (!buf || cap < need) return DAMASCUS_ESIZE;
    for (size_t i = 0; i < m.c.size(); ++i) fq_to_bytes(m.c[i], buf + 16 * i);
    return DAMASCUS_OK;
}

int damascus_prover_fold_round_timed(damascus_prover* p, uint64_t round, uint8_t* record_out, size_t cap,
                                     size_t* record_len, double* vector_ms, double* poly_ms, double* total_ms) {
    if (!p) return DAMASCUS_EINVAL;
    // the record's size is known before the round runs: a small buffer fails
    // without advancing the prover, so the caller can retry
    const uint32_t n = p->p->ring_len();
    const size_t need = record_encoded_size(n, n > 1 ? n / 2 : 1);
    if (record_len) *record_len = need;
    if (!record_out || cap < need) return set_err(p->owner, DAMASCUS_ESIZE, "record buffer too small");
    RoundRecord rec;
    double t[3] = {0, 0, 0};
    int rc = p->p->fold_round(round, &rec, t);
    if (rc != kOk) return rc;
    std::vector<uint8_t> v;
    encode_record(v, rec);
    if (record_len) *record_len = v.size();
    if (v.size() > cap) return set_err(p->owner, DAMASCUS_ESIZE, "record larger than its computed size");
    std::memcpy(record_out, v.data(), v.size());
    if (vector_ms) *vector_ms = t[0];
    if (poly_ms) *poly_ms = t[1];
    if (total_ms) *total_ms = t[2];
    return DAMASCUS_OK;
}

int damascus_prover_fold_round(damascus_prover* p, uint64_t round, uint8_t* record_out, size_t cap,
                               size_t* record_len) {
    return damascus_prover_fold_round_timed(p, round, record_out, cap, record_len, nullptr, nullptr, nullptr);
}

int damascus_prover_final_opening(const damascus_prover* p, uint8_t out[16]) {
    if (!p || !out) return DAMASCUS_EINVAL;
    fq o;
    if (!p->p->final_opening(&o)) return DAMASCUS_ESTATE;
    fq_to_bytes(o, out);
    return DAMASCUS_OK;
}

static int prove_common(damascus_ctx* ctx, const uint8_t* file, size_t len, bool on_device, const uint8_t* seed,
                        const uint8_t* epoch, uint8_t* proof_out, size_t cap, size_t* proof_len,
                        double* device_ms = nullptr) {
    if (!ctx || (!file && len) || !seed || !epoch) return DAMASCUS_EINVAL;
    std::vector<uint8_t> proof;
    int rc = prove_all(ctx->ctx, file, len, on_device, seed, epoch, &proof, device_ms);
    if (rc != kOk) return rc;
    if (proof_len) *proof_len = proof.size();
    if (!proof_out || cap < proof.size()) return set_err(ctx, DAMASCUS_ESIZE, "proof buffer too small");
    std::memcpy(proof_out, proof.data(), proof.size());
    return DAMASCUS_OK;
}

int damascus_prove(damascus_ctx* ctx, const uint8_t* file, size_t len, const uint8_t seed_generators[32],
                   const uint8_t epoch_seed[32], uint8_t* proof_out, size_t cap, size_t* proof_len) {
    return prove_common(ctx, file, len, false, seed_generators, epoch_seed, proof_out, cap, proof_len);
}

int damascus_prove_device(damascus_ctx* ctx, const void* d_file, size_t len, const uint8_t seed_generators[32],
                          const uint8_t epoch_seed[32], uint8_t* proof_out, size_t cap, size_t* proof_len) {
    return prove_common(ctx, static_cast<const uint8_t*>(d_file), len, true, seed_generators, epoch_seed, proof_out,
                        cap, proof_len);
}

int damascus_prove_device_timed(damascus_ctx* ctx, const void* d_file, size_t len, const uint8_t seed_generators[32],
                                const uint8_t epoch_seed[32], uint8_t* proof_out, size_t cap, size_t* proof_len,
                                double* device_ms) {
    return prove_common(ctx, static_cast<const uint8_t*>(d_file), len, true, seed_generators, epoch_seed, proof_out,
                        cap, proof_len, device_ms);
}

int damascus_ctx_flush_l2(damascus_ctx* ctx) {
    if (!ctx) return DAMASCUS_EINVAL;
    return ctx->ctx->flush_l2();
}

// ------------------------------------------------------------------ generator cache
int damascus_ctx_set_max_preprocess_bytes(damascus_ctx* ctx, uint64_t max_preprocess_bytes) {
    if (!ctx) return DAMASCUS_EINVAL;
    ctx->ctx->set_max_preprocess(max_preprocess_bytes);
    return DAMASCUS_OK;
}

uint64_t damascus_ctx_max_preprocess_bytes(damascus_ctx* ctx) { return ctx ? ctx->ctx->max_preprocess() : 0; }

int damascus_ctx_set_generator_cache(damascus_ctx* ctx, uint64_t cap_bytes) {
    if (!ctx) return DAMASCUS_EINVAL;
    if (ctx->ctx->set_prover_cache(cap_bytes) != kOk)
        return set_err(ctx, DAMASCUS_ESTATE, "a running prover or verifier holds a cached generator family");
    return DAMASCUS_OK;
}

int damascus_ctx_generator_cache_stats(damascus_ctx* ctx, uint64_t* hits, uint64_t* fills, uint64_t* misses,
                                       uint64_t* bytes) {
    if (!ctx) return DAMASCUS_EINVAL;
    ProverGenCache::Stats st{};
    if (ctx->ctx->prover_cache()) st = ctx->ctx->prover_cache()->stats();
    if (hits) *hits = st.hits;
    if (fills) *fills = st.fills;
    if (misses) *misses = st.misses;
    if (bytes) *bytes = st.bytes;
    return DAMASCUS_OK;
}

// ------------------------------------------------------------------ tuning
int damascus_tuning_set(damascus_ctx* ctx, int knob, uint32_t log_ring, int value) {
    if (!ctx) return DAMASCUS_EINVAL;
    if (ctx->ctx->set_tuning(knob, log_ring, value) != kOk)
        return set_err(ctx, DAMASCUS_EINVAL, "tuning knob, ring size or value out of range");
    return DAMASCUS_OK;
}

int damascus_tuning_get(damascus_ctx* ctx, int knob, uint32_t log_ring, int* value) {
    if (!ctx || !value || knob < 0 || knob >= kTuneKnobs || log_ring > (uint32_t)kLogMaxProverRing)
        return DAMASCUS_EINVAL;
    *value = ctx->ctx->tuning(knob, log_ring);
    return DAMASCUS_OK;
}

int damascus_measure_int_multiply(damascus_ctx* ctx, double ops_per_s[3]) {
    if (!ctx || !ops_per_s) return DAMASCUS_EINVAL;
    Context* C = ctx->ctx;
    std::lock_guard<std::mutex> g(C->mutex());
    cudaSetDevice(C->device());
    cudaStream_t st = C->stream();
    Scratch sink;
    if (sink.alloc(C, 256)) return set_err(ctx, DAMASCUS_ENOMEM_BUDGET, "HBM budget exhausted");
    const int blocks = 4 * C->sm_count(), iters = 4096;
    const double ops = (double)int_mul_probe_ops(blocks, iters);
    cudaEvent_t a = nullptr, b = nullptr;
    cudaError_t e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    for (int kind = 0; kind < 3 && e == cudaSuccess; ++kind) {
        double best = 0;
        for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {  // the first launch warms up
            e = cudaEventRecord(a, st);
            if (e == cudaSuccess) e = launch_int_mul_probe(kind, sink.m.as<uint32_t>(), blocks, 3u + rep, iters, st);
            if (e == cudaSuccess) e = cudaEventRecord(b, st);
            if (e == cudaSuccess) e = cudaEventSynchronize(b);
            float ms = 0;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
            if (e == cudaSuccess && rep > 0 && ms > 0 && ops / (ms * 1e-3) > best) best = ops / (ms * 1e-3);
        }
        ops_per_s[kind] = best;
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (e != cudaSuccess) return set_err(ctx, DAMASCUS_ECUDA, std::string("integer multiply probe: ") + cudaGetErrorString(e));
    return DAMASCUS_OK;
}

int damascus_tuning_measure(damascus_ctx* ctx, int knob, uint32_t log_ring, int value, uint32_t count, int reps,
                            double* ms_per_launch) {
    if (!ctx || !ms_per_launch || count == 0 || reps <= 0 || log_ring > (uint32_t)kLogMaxProverRing)
        return DAMASCUS_EINVAL;
    const uint32_t L = log_ring;
    const uint64_t s = 1ull << L;
    const bool bad = knob == kTuneNttGroup       ? (L < 4 || (value != 32 && value != 64))
                     : knob == kTuneNttRadix     ? (L < 5 || (value != 16 && value != 32))
                     : knob == kTuneSplitCoords  ? (L < 1 || (value != 1 && value != 2 && value != 4 && value != 8))
                     : knob == kTuneTripleCoords ? (L < 1 || (value != 1 && value != 2 && value != 4))
                                                 : (knob <= 0 || knob >= kTuneKnobs || L < 1 || value < 1 || value > 32);
    if (bad) return set_err(ctx, DAMASCUS_EINVAL, "tuning knob, ring size or value out of range");
    Context* C = ctx->ctx;
    std::lock_guard<std::mutex> g(C->mutex());
    cudaSetDevice(C->device());
    const DeviceTables& T = C->tables();
    cudaStream_t st = C->stream();
    const uint32_t rows = kRank * kPrimes;
    Scratch a, b, part;
    std::function<cudaError_t()> launch;
    NttJob nj{};
    MacJobX mj{}, mj_pair{};
    if (knob == kTuneNttGroup || knob == kTuneNttRadix) {
        // count polynomials of arbitrary 128-bit words -> nine residue rows each
        if (a.alloc(C, count * s * 16) || b.alloc(C, count * kPrimes * s * 4))
            return set_err(ctx, DAMASCUS_ENOMEM_BUDGET, "HBM budget exhausted");
        cudaMemsetAsync(a.m.as<uint8_t>(), 0x5A, count * s * 16, st);
        nj = NttJob{a.m.as<uint4>(), b.m.as<uint32_t>(), count, 0};
        const int group = knob == kTuneNttGroup ? value : C->tuning(kTuneNttGroup, L);
        const int elems = knob == kTuneNttRadix ? value : C->tuning(kTuneNttRadix, L);
        launch = [&, group, elems] { return launch_ntt_jobs(T, &nj, 1, L, st, group, elems); };
    } else {
        // generator / witness residues (all 0x01010101 < p) over `count` columns (pairs for the triple MAC);
        // a coordinates knob measures its MAC with that MAC's blocks-per-SM knob as set
        const bool triple = knob == kTuneMacTriple || knob == kTuneTripleCoords;
        const bool split = knob == kTuneMacSplit || knob == kTuneSplitCoords;
        const bool coords = knob == kTuneSplitCoords || knob == kTuneTripleCoords;
        const int coords_knob = triple ? kTuneTripleCoords : kTuneSplitCoords;
        const int bps_knob = triple ? kTuneMacTriple : kTuneMacSplit;
        const uint64_t cols = triple ? 2ull * count : count;
        const uint32_t tpr = knob == kTuneMacPlain ? (uint32_t)s : (uint32_t)(s / 2);
        const uint32_t kc = coords ? (uint32_t)value : (uint32_t)C->tuning(coords_knob, L);
        const uint32_t parts = C->mac_parts_for(coords ? C->tuning(bps_knob, L) : value, tpr, count,
                                                (split || triple) ? rows / kc : rows);
        if (a.alloc(C, cols * rows * s * 4) || b.alloc(C, cols * kPrimes * s * 4) ||
            part.alloc(C, 3ull * parts * rows * s * 4))
            return set_err(ctx, DAMASCUS_ENOMEM_BUDGET, "HBM budget exhausted");
        cudaMemsetAsync(a.m.as<uint8_t>(), 0x01, cols * rows * s * 4, st);
        cudaMemsetAsync(b.m.as<uint8_t>(), 0x01, cols * kPrimes * s * 4, st);
        uint32_t* P = part.m.as<uint32_t>();
        const uint64_t ps = (uint64_t)parts * rows * s;
        mj = MacJobX{a.m.as<uint32_t>(), b.m.as<uint32_t>(), P, P + ps, P + 2 * ps, 0, 0, count, parts, 0, 0, L,
                     (split || triple) ? kc : 0u};
        mj_pair = mj;
        mj_pair.pair = count;  // the witness's columns from `count` on are zero: read at i only
        if (triple)  // both forms a proof runs: full pairs, then the known-zero-half form
            launch = [&] {
                cudaError_t r = launch_mac_triple_jobs(T, &mj, 1, st);
                return r == cudaSuccess ? launch_mac_triple_jobs(T, &mj_pair, 1, st) : r;
            };
        else
            launch = [&, split] { return launch_mac_jobs(T, &mj, 1, split, st); };
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = launch();  // warm-up
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaEventRecord(e0, st);
    for (int i = 0; i < reps && e == cudaSuccess; ++i) e = launch();
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e != cudaSuccess) return set_err(ctx, DAMASCUS_ECUDA, std::string("tuning_measure: ") + cudaGetErrorString(e));
    *ms_per_launch = (double)ms / reps;
    return DAMASCUS_OK;
}

// ------------------------------------------------------------------ verifier
int damascus_verifier_new(damascus_ctx* ctx, const uint8_t* statement, size_t len, const uint8_t epoch_seed[32],
                          damascus_verifier** out) {
    if (!ctx || !statement || !epoch_seed || !out) return DAMASCUS_EINVAL;
    GpuVerifier* v = new GpuVerifier(ctx->ctx);
    int rc = v->init(statement, len, epoch_seed);
    if (rc != kOk) {
        delete v;
        *out = nullptr;
        return rc;
    }
    *out = new damascus_verifier{ctx, v};
    return DAMASCUS_OK;
}

void damascus_verifier_free(damascus_verifier* v) {
    if (!v) return;
    delete v->v;
    delete v;
}

int damascus_verifier_update_commitment(damascus_verifier* v, const uint8_t* record, size_t len) {
    if (!v || !record) return DAMASCUS_EINVAL;
    const uint8_t* p = record;
    RoundRecord rec;
    if (!decode_record(p, record + len, rec)) return set_err(v->owner, DAMASCUS_EDESERIALIZE, "round record deserialization failed");
    return v->v->update_commitment(rec);
}

int damascus_verifier_verify_final_opening(damascus_verifier* v, const uint8_t opening[16]) {
    if (!v || !opening) return DAMASCUS_EINVAL;
    return v->v->verify_final_opening(fq_from_bytes(opening));
}

uint64_t damascus_verifier_round(const damascus_verifier* v) { return v ? v->v->round() : 0; }
void damascus_verifier_dimensions(const damascus_verifier* v, uint64_t* N, uint64_t* n) {
    if (N) *N = v ? v->v->vector_len() : 0;
    if (n) *n = v ? v->v->ring_len() : 0;
}

int damascus_verify(damascus_ctx* ctx, const uint8_t* proof, size_t len, const uint8_t epoch_seed[32]) {
    if (!ctx || !proof || !epoch_seed) return DAMASCUS_EINVAL;
    return verify_proof(ctx->ctx, proof, len, epoch_seed);
}

// ------------------------------------------------------------------ engine
int damascus_engine_create(damascus_ctx* ctx, int host_threads, int max_waves, damascus_engine** out) {
    if (!ctx || !out) return DAMASCUS_EINVAL;
    *out = nullptr;
    std::unique_ptr<Engine> eng(new Engine(ctx->ctx, host_threads, max_waves));
    if (!eng->init_error().empty()) return set_err(ctx, DAMASCUS_ECUDA, eng->init_error());
    *out = new damascus_engine{ctx, eng.release(), {}, {}, {}};
    return DAMASCUS_OK;
}

int damascus_engine_create_with_options(damascus_ctx* ctx, const damascus_engine_options* opts,
                                        damascus_engine** out) {
    if (!ctx || !out) return DAMASCUS_EINVAL;
    *out = nullptr;
    EngineOptions o;
    if (opts) {
        o.host_threads = opts->host_threads;
        o.max_waves = opts->max_waves;
        o.priority_depth = opts->priority_depth;
        o.polling = opts->polling;
        o.spin_us = opts->spin_us;
        o.admission_batch = opts->admission_batch;
    }
    std::unique_ptr<Engine> eng(new Engine(ctx->ctx, o));
    if (!eng->init_error().empty()) return set_err(ctx, DAMASCUS_ECUDA, eng->init_error());
    *out = new damascus_engine{ctx, eng.release(), {}, {}, {}};
    return DAMASCUS_OK;
}

void damascus_engine_destroy(damascus_engine* e) {
    if (!e) return;
    delete e->e;
    delete e;
}

int damascus_engine_submit(damascus_engine* e, const uint8_t* file, size_t len, const uint8_t seed_generators[32],
                           const uint8_t epoch_seed[32], uint64_t* ticket) {
    if (!e) return DAMASCUS_EINVAL;
    return e->e->submit(file, len, seed_generators, epoch_seed, ticket);
}

int damascus_engine_submit_device(damascus_engine* e, const void* d_file, size_t len,
                                  const uint8_t seed_generators[32], const uint8_t epoch_seed[32], uint64_t* ticket) {
    if (!e) return DAMASCUS_EINVAL;
    return e->e->submit(static_cast<const uint8_t*>(d_file), len, seed_generators, epoch_seed, ticket,
                        Engine::FileSource::kDevice);
}

int damascus_engine_submit_borrowed(damascus_engine* e, const uint8_t* file, size_t len,
                                    const uint8_t seed_generators[32], const uint8_t epoch_seed[32], uint64_t* ticket) {
    if (!e) return DAMASCUS_EINVAL;
    return e->e->submit(file, len, seed_generators, epoch_seed, ticket, Engine::FileSource::kHostBorrowed);
}

static int engine_result(damascus_engine* e, uint64_t ticket, bool block, size_t* proof_len, double* latency_ms) {
    {
        std::lock_guard<std::mutex> g(e->mu);
        auto st = e->status.find(ticket);
        if (st != e->status.end()) {
            if (proof_len) *proof_len = e->results[ticket].size();
            if (latency_ms) *latency_ms = st->second.second;
            return st->second.first;
        }
    }
    std::vector<uint8_t> proof;
    double lat = 0;
    std::string err;
    const int rc = block ? e->e->wait(ticket, &proof, &lat, &err) : e->e->poll(ticket, &proof, &lat, &err);
    if (rc == 0) return 0;
    if (rc < 0 && rc == DAMASCUS_EINVAL && err.empty()) return rc;  // unknown ticket
    std::lock_guard<std::mutex> g(e->mu);
    if (rc < 0) e->owner->ctx->set_error(err);
    e->status[ticket] = {rc, lat};
    if (proof_len) *proof_len = proof.size();
    if (latency_ms) *latency_ms = lat;
    e->results[ticket] = std::move(proof);
    return rc;
}

int damascus_engine_poll(damascus_engine* e, uint64_t ticket, size_t* proof_len, double* latency_ms) {
    if (!e) return DAMASCUS_EINVAL;
    return engine_result(e, ticket, false, proof_len, latency_ms);
}

int damascus_engine_wait(damascus_engine* e, uint64_t ticket, size_t* proof_len, double* latency_ms) {
    if (!e) return DAMASCUS_EINVAL;
    return engine_result(e, ticket, true, proof_len, latency_ms);
}

int damascus_engine_wait_any(damascus_engine* e, const uint64_t* tickets, size_t n, size_t* which) {
    if (!e || !tickets || !which || n == 0) return DAMASCUS_EINVAL;
    {
        std::lock_guard<std::mutex> g(e->mu);  // one collected earlier (by poll or wait) counts as finished
        for (size_t i = 0; i < n; ++i)
            if (e->status.count(tickets[i])) {
                *which = i;
                return DAMASCUS_OK;
            }
    }
    return e->e->wait_any(tickets, n, which);
}

int damascus_engine_wait_timeout(damascus_engine* e, uint64_t ticket, double timeout_ms, size_t* proof_len,
                                 double* latency_ms) {
    if (!e) return DAMASCUS_EINVAL;
    bool known;
    {
        std::lock_guard<std::mutex> g(e->mu);
        known = e->status.count(ticket) != 0;
    }
    if (known) return engine_result(e, ticket, false, proof_len, latency_ms);  // finished earlier
    std::vector<uint8_t> proof;
    double lat = 0;
    std::string err;
    const int rc = e->e->wait_for(ticket, timeout_ms, &proof, &lat, &err);
    if (rc == kETimeout || rc == 0) return rc == 0 ? 0 : DAMASCUS_ETIMEOUT;
    if (rc < 0 && rc == DAMASCUS_EINVAL && err.empty()) return rc;
    std::lock_guard<std::mutex> g(e->mu);
    if (rc < 0) e->owner->ctx->set_error(err);
    e->status[ticket] = {rc, lat};
    if (proof_len) *proof_len = proof.size();
    if (latency_ms) *latency_ms = lat;
    e->results[ticket] = std::move(proof);
    return rc;
}

int damascus_engine_cancel(damascus_engine* e, uint64_t ticket) {
    if (!e) return DAMASCUS_EINVAL;
    {
        std::lock_guard<std::mutex> g(e->mu);
        if (e->status.count(ticket))  // finished, result not taken yet
            return set_err(e->owner, DAMASCUS_ESTATE, "cancel: the request has already finished");
    }
    const int rc = e->e->cancel(ticket);
    if (rc == kEInval) return set_err(e->owner, DAMASCUS_EINVAL, "cancel: unknown ticket (or its proof was taken)");
    if (rc == kEState) return set_err(e->owner, DAMASCUS_ESTATE, "cancel: the request has already finished");
    return rc;
}

int damascus_engine_set_request_timeout(damascus_engine* e, double timeout_ms) {
    if (!e || timeout_ms < 0) return DAMASCUS_EINVAL;
    e->e->set_request_timeout(timeout_ms);
    return DAMASCUS_OK;
}

int damascus_engine_set_admission_batch(damascus_engine* e, int requests_per_pass) {
    if (!e || requests_per_pass < 0) return DAMASCUS_EINVAL;
    e->e->set_admission_batch(requests_per_pass);
    return DAMASCUS_OK;
}

int damascus_engine_health(damascus_engine* e, uint64_t* unfinished, double* ms_since_progress) {
    if (!e) return DAMASCUS_EINVAL;
    e->e->health(unfinished, ms_since_progress);
    return DAMASCUS_OK;
}

int damascus_engine_take(damascus_engine* e, uint64_t ticket, uint8_t* proof_out, size_t cap) {
    if (!e) return DAMASCUS_EINVAL;
    std::lock_guard<std::mutex> g(e->mu);
    auto it = e->results.find(ticket);
    if (it == e->results.end()) return DAMASCUS_ESTATE;
    if (!proof_out || cap < it->second.size()) return DAMASCUS_ESIZE;
    std::memcpy(proof_out, it->second.data(), it->second.size());
    e->results.erase(it);
    e->status.erase(ticket);
    return DAMASCUS_OK;
}

int damascus_engine_result(damascus_engine* e, uint64_t ticket, const uint8_t** data, size_t* len) {
    if (!e || !data || !len) return DAMASCUS_EINVAL;
    std::lock_guard<std::mutex> g(e->mu);
    auto it = e->results.find(ticket);
    if (it == e->results.end()) return DAMASCUS_ESTATE;
    *data = it->second.data();
    *len = it->second.size();
    return DAMASCUS_OK;
}

int damascus_engine_release(damascus_engine* e, uint64_t ticket) {
    if (!e) return DAMASCUS_EINVAL;
    std::lock_guard<std::mutex> g(e->mu);
    auto it = e->results.find(ticket);
    if (it == e->results.end()) return DAMASCUS_ESTATE;
    e->results.erase(it);
    e->status.erase(ticket);
    return DAMASCUS_OK;
}

int damascus_engine_drain(damascus_engine* e) {
    if (!e) return DAMASCUS_EINVAL;
    e->e->drain();
    return DAMASCUS_OK;
}

int damascus_engine_stats(damascus_engine* e, uint64_t* completed, uint64_t* failed, uint64_t* waves,
                          uint64_t* launches, uint64_t* peak_reserved_bytes) {
    if (!e) return DAMASCUS_EINVAL;
    const EngineStats s = e->e->stats();
    if (completed) *completed = s.completed;
    if (failed) *failed = s.failed;
    if (waves) *waves = s.waves;
    if (launches) *launches = s.launches;
    if (peak_reserved_bytes) *peak_reserved_bytes = s.peak_reserved;
    return DAMASCUS_OK;
}

int damascus_engine_profile(damascus_engine* e, double* host_stage_ms, double* gpu_idle_ms) {
    if (!e) return DAMASCUS_EINVAL;
    const EngineStats s = e->e->stats();
    if (host_stage_ms) *host_stage_ms = s.host_stage_ms;
    if (gpu_idle_ms) *gpu_idle_ms = s.gpu_idle_ms;
    return DAMASCUS_OK;
}

int damascus_engine_scheduler_profile(damascus_engine* e, double* admit_ms, double* launch_ms) {
    if (!e) return DAMASCUS_EINVAL;
    const EngineStats s = e->e->stats();
    if (admit_ms) *admit_ms = s.admit_ms;
    if (launch_ms) *launch_ms = s.launch_ms;
    return DAMASCUS_OK;
}

// ------------------------------------------------------------------ verifier service
int damascus_verify_service_create(damascus_ctx* ctx, int workers, uint64_t cache_bytes,
                                   damascus_verify_service** out) {
    if (!ctx || !out) return DAMASCUS_EINVAL;
    *out = nullptr;
    std::unique_ptr<VerifyService> svc(new VerifyService(ctx->ctx, workers, cache_bytes));
    if (!svc->init_error().empty()) return set_err(ctx, DAMASCUS_ECUDA, svc->init_error());
    *out = new damascus_verify_service{ctx, svc.release()};
    return DAMASCUS_OK;
}

void damascus_verify_service_destroy(damascus_verify_service* s) {
    if (!s) return;
    delete s->s;
    delete s;
}

int damascus_verify_service_submit(damascus_verify_service* s, const uint8_t* proof, size_t len,
                                   const uint8_t epoch_seed[32], uint64_t* ticket) {
    if (!s) return DAMASCUS_EINVAL;
    return s->s->submit(proof, len, epoch_seed, ticket);
}

static int verify_service_result(damascus_verify_service* s, uint64_t ticket, bool block, int* verdict,
                                 double* latency_ms) {
    if (!s) return DAMASCUS_EINVAL;
    int v = 0;
    std::string err;
    const int rc = block ? s->s->wait(ticket, &v, latency_ms, &err) : s->s->poll(ticket, &v, latency_ms, &err);
    if (rc == 1) {
        if (verdict) *verdict = v;
        if (v != DAMASCUS_OK) s->owner->ctx->set_error(err);
    }
    return rc;
}

int damascus_verify_service_poll(damascus_verify_service* s, uint64_t ticket, int* verdict, double* latency_ms) {
    return verify_service_result(s, ticket, false, verdict, latency_ms);
}

int damascus_verify_service_wait(damascus_verify_service* s, uint64_t ticket, int* verdict, double* latency_ms) {
    return verify_service_result(s, ticket, true, verdict, latency_ms);
}

int damascus_verify_service_drain(damascus_verify_service* s) {
    if (!s) return DAMASCUS_EINVAL;
    s->s->drain();
    return DAMASCUS_OK;
}

int damascus_verify_service_stats(damascus_verify_service* s, uint64_t* completed, uint64_t* accepted,
                                  uint64_t* rejected, uint64_t* cache_hits, uint64_t* cache_misses,
                                  uint64_t* peak_reserved_bytes) {
    if (!s) return DAMASCUS_EINVAL;
    const VerifyStats v = s->s->stats();
    if (completed) *completed = v.completed;
    if (accepted) *accepted = v.accepted;
    if (rejected) *rejected = v.rejected;
    if (cache_hits) *cache_hits = v.cache_hits;
    if (cache_misses) *cache_misses = v.cache_misses;
    if (peak_reserved_bytes) *peak_reserved_bytes = v.peak_reserved;
    return DAMASCUS_OK;
}

// ------------------------------------------------------------------ reference FFI
namespace {
damascus_ctx* default_ctx() {
    static damascus_ctx* c = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        if (damascus_ctx_create(0, 0, &c) != DAMASCUS_OK) c = nullptr;
    });
    return c;
}
}  // namespace

int damascus_cuda_fold_batch(const uint64_t* left_lo, const uint64_t* left_hi, const uint64_t* right_lo,
                             const uint64_t* right_hi, uint64_t* out_lo, uint64_t* out_hi, size_t len,
                             uint64_t challenge_lo, uint64_t challenge_hi) {
    if (!left_lo || !left_hi || !right_lo || !right_hi || !out_lo || !out_hi || len == 0) return 1;
    damascus_ctx* ctx = default_ctx();
    if (!ctx) return 2;
    Context* C = ctx->ctx;
    std::lock_guard<std::mutex> g(C->mutex());
    cudaSetDevice(C->device());
    Scratch b;
    const size_t w = len * 8;
    if (b.alloc(C, 6 * w)) return 3;
    uint64_t* base = b.m.as<uint64_t>();
    uint64_t *ll = base, *lh = base + len, *rl = base + 2 * len, *rh = base + 3 * len, *ol = base + 4 * len,
             *oh = base + 5 * len;
    cudaStream_t s = C->stream();
    const uint64_t cw[2] = {challenge_lo, challenge_hi};
    uint32_t c8[8] = {(uint32_t)cw[0], (uint32_t)(cw[0] >> 32), (uint32_t)cw[1], (uint32_t)(cw[1] >> 32), 0, 0, 0, 0};
    const fq c = fq_reduce8(c8);
    if (cudaMemcpyAsync(ll, left_lo, w, cudaMemcpyHostToDevice, s) != cudaSuccess) return 4;
    if (cudaMemcpyAsync(lh, left_hi, w, cudaMemcpyHostToDevice, s) != cudaSuccess) return 5;
    if (cudaMemcpyAsync(rl, right_lo, w, cudaMemcpyHostToDevice, s) != cudaSuccess) return 6;
    if (cudaMemcpyAsync(rh, right_hi, w, cudaMemcpyHostToDevice, s) != cudaSuccess) return 7;
    if (launch_fold_split(ll, lh, rl, rh, ol, oh, len, c, s) != cudaSuccess) return 8;
    if (cudaMemcpyAsync(out_lo, ol, w, cudaMemcpyDeviceToHost, s) != cudaSuccess) return 9;
    if (cudaMemcpyAsync(out_hi, oh, w, cudaMemcpyDeviceToHost, s) != cudaSuccess) return 10;
    if (cudaStreamSynchronize(s) != cudaSuccess) return 11;
    return 0;
}

int damascus_cuda_ntt_batch(const uint64_t* host_a, const uint64_t* host_b, uint64_t* host_out, size_t n,
                            const uint64_t* primes, const uint64_t* stage_roots, const uint64_t* inv_roots,
                            const uint64_t* inv_sizes) {
    if (!host_a || !host_b || !host_out || !primes || !stage_roots || !inv_roots || !inv_sizes || !pow2(n)) return 1;
    if (n > (1u << (kLogMaxRing - 1))) return 12;  // the cyclic convolution zero-pads to 2n <= 2^13
    for (int i = 0; i < kRefPrimes; ++i)
        if (primes[i] != kRefCrtPrimes[i]) return 13;  // the kernels are specialised to the reference's primes
    damascus_ctx* ctx = default_ctx();
    if (!ctx) return 2;
    Context* C = ctx->ctx;
    std::lock_guard<std::mutex> g(C->mutex());
    cudaSetDevice(C->device());
    Scratch b;
    const size_t words = (size_t)kRefPrimes * n;
    if (b.alloc(C, 3 * words * 4)) return 3;
    std::vector<uint32_t> ha(words), hb(words), ho(words);
    for (size_t i = 0; i < words; ++i) {
        const uint64_t p = primes[i / n];
        ha[i] = (uint32_t)(host_a[i] % p);
        hb[i] = (uint32_t)(host_b[i] % p);
    }
    uint32_t* da = b.m.as<uint32_t>();
    uint32_t *db = da + words, *dout = da + 2 * words;
    cudaStream_t s = C->stream();
    if (cudaMemcpyAsync(da, ha.data(), words * 4, cudaMemcpyHostToDevice, s) != cudaSuccess) return 6;
    if (cudaMemcpyAsync(db, hb.data(), words * 4, cudaMemcpyHostToDevice, s) != cudaSuccess) return 7;
    if (launch_cyclic_conv(C->ref_tables(), da, db, dout, log2u(n), s) != cudaSuccess) return 8;
    if (cudaMemcpyAsync(ho.data(), dout, words * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) return 15;
    if (cudaStreamSynchronize(s) != cudaSuccess) return 16;
    for (size_t i = 0; i < words; ++i) host_out[i] = ho[i];
    return 0;
}

// ------------------------------------------------------------------ measurement
int damascus_ctx_set_profiling(damascus_ctx* ctx, int on) {
    if (!ctx) return DAMASCUS_EINVAL;
    ctx->ctx->set_profiling(on != 0);
    return DAMASCUS_OK;
}
void damascus_ctx_reset_stats(damascus_ctx* ctx) {
    if (ctx) ctx->ctx->reset_stats();
}
int damascus_ctx_trace_start(damascus_ctx* ctx) {
    if (!ctx) return DAMASCUS_EINVAL;
    ctx->trace.clear();
    return ctx->ctx->start_trace();
}
int damascus_ctx_trace_read(damascus_ctx* ctx, char* buf, size_t cap, size_t* len, int stop) {
    if (!ctx) return DAMASCUS_EINVAL;
    std::string more;
    const int rc = ctx->ctx->read_trace(&more, stop != 0);
    if (rc != DAMASCUS_OK) return rc;
    ctx->trace += more;
    if (len) *len = ctx->trace.size();
    if (!buf || cap < ctx->trace.size()) return set_err(ctx, DAMASCUS_ESIZE, "trace buffer too small");
    std::memcpy(buf, ctx->trace.data(), ctx->trace.size());
    ctx->trace.clear();
    return DAMASCUS_OK;
}
int damascus_ctx_kernel_stat(damascus_ctx* ctx, const char* name, uint64_t* launches, double* total_ms,
                             double* algo_bytes, double* algo_ops) {
    if (!ctx || !name) return DAMASCUS_EINVAL;
    KernelStat s;
    if (!ctx->ctx->stat(name, &s)) return DAMASCUS_EINVAL;
    if (launches) *launches = s.launches;
    if (total_ms) *total_ms = s.total_ms;
    if (algo_bytes) *algo_bytes = s.bytes;
    if (algo_ops) *algo_ops = s.ops;
    return DAMASCUS_OK;
}
int damascus_ctx_synchronize(damascus_ctx* ctx) {
    if (!ctx) return DAMASCUS_EINVAL;
    cudaSetDevice(ctx->ctx->device());
    return cudaDeviceSynchronize() == cudaSuccess ? DAMASCUS_OK : DAMASCUS_ECUDA;
}

}  // extern "C"
