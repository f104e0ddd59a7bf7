#include "engine.h"

#include <cstring>
#include <limits>

#include "host_blake3.h"

namespace dm {

// ============================== Context ==============================

int Context::create(int device, uint64_t hbm_budget, Context** out, std::string* err) {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        *err = std::string("no CUDA device available: ") + cudaGetErrorString(e);
        return kECuda;
    }
    if (device < 0 || device >= count) {
        *err = "device index out of range";
        return kEInval;
    }
    if ((e = cudaSetDevice(device)) != cudaSuccess) {
        *err = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
        return kECuda;
    }
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, device)) != cudaSuccess) {
        *err = std::string("cudaGetDeviceProperties: ") + cudaGetErrorString(e);
        return kECuda;
    }
    if (prop.major < 10) {
        *err = "this library is built for sm_103a (GB300); device reports compute capability " +
               std::to_string(prop.major) + "." + std::to_string(prop.minor);
        return kEUnsupported;
    }
    std::unique_ptr<Context> c(new Context());
    c->device_ = device;
    if ((e = cudaStreamCreateWithFlags(&c->stream_, cudaStreamNonBlocking)) != cudaSuccess) {
        *err = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
        return kECuda;
    }
    if ((e = upload_tables(&c->tables_)) != cudaSuccess) {
        *err = std::string("table upload: ") + cudaGetErrorString(e);
        return kECuda;
    }
    // Keep freed blocks in the stream-ordered pool instead of returning them to the driver.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = std::numeric_limits<uint64_t>::max();
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    c->budget_ = hbm_budget ? hbm_budget : (uint64_t)(free_b * 0.9);
    *out = c.release();
    return kOk;
}

int Context::flush_l2() {
    constexpr size_t kFlushBytes = 256ull << 20;
    cudaSetDevice(device_);
    if (!flush_buf_ && cudaMalloc(&flush_buf_, kFlushBytes) != cudaSuccess) {
        flush_buf_ = nullptr;
        return kENoMem;
    }
    if (cudaMemsetAsync(flush_buf_, 0x5A, kFlushBytes, stream_) != cudaSuccess) return kECuda;
    return cudaStreamSynchronize(stream_) == cudaSuccess ? kOk : kECuda;
}

void* Context::get_pinned(size_t bytes) {
    {
        std::lock_guard<std::mutex> g(pin_mu_);
        for (size_t i = 0; i < pinned_free_.size(); ++i)
            if (pinned_free_[i].first >= bytes) {
                void* p = pinned_free_[i].second;
                pinned_free_.erase(pinned_free_.begin() + (long)i);
                return p;
            }
    }
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
    return p;
}

void Context::put_pinned(void* p, size_t bytes) {
    if (!p) return;
    std::lock_guard<std::mutex> g(pin_mu_);
    pinned_free_.emplace_back(bytes, p);
}

Context::~Context() {
    cudaSetDevice(device_);
    if (stream_) cudaStreamSynchronize(stream_);
    if (flush_buf_) cudaFree(flush_buf_);
    for (auto& pp : pinned_free_) cudaFreeHost(pp.second);
    flush_timings();
    for (cudaEvent_t e : event_pool_) cudaEventDestroy(e);
    if (tables_.zeta) cudaFree(const_cast<uint32_t*>(tables_.zeta));
    if (tables_.zinv) cudaFree(const_cast<uint32_t*>(tables_.zinv));
    if (stream_) cudaStreamDestroy(stream_);
}

bool Context::reserve(uint64_t bytes) {
    uint64_t cur = reserved_.load();
    do {
        if (cur + bytes > budget_) return false;
    } while (!reserved_.compare_exchange_weak(cur, cur + bytes));
    return true;
}
void Context::release(uint64_t bytes) { reserved_.fetch_sub(bytes); }

void Context::set_error(const std::string& e) {
    std::lock_guard<std::mutex> g(err_mu_);
    last_error_ = e;
}
std::string Context::last_error() {
    std::lock_guard<std::mutex> g(err_mu_);
    return last_error_;
}

cudaEvent_t Context::take_event() {
    std::lock_guard<std::mutex> g(prof_mu_);
    if (!event_pool_.empty()) {
        cudaEvent_t e = event_pool_.back();
        event_pool_.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void Context::record(const char* name, cudaEvent_t a, cudaEvent_t b, double bytes, double ops, int kernels) {
    std::lock_guard<std::mutex> g(prof_mu_);
    pending_.push_back(Pending{name, a, b, bytes, ops, kernels});
}

void Context::flush_timings() {
    std::vector<Pending> work;
    {
        std::lock_guard<std::mutex> g(prof_mu_);
        work.swap(pending_);
    }
    for (auto& p : work) {
        cudaEventSynchronize(p.b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.a, p.b);
        std::lock_guard<std::mutex> g(prof_mu_);
        KernelStat& s = stats_[p.name];
        s.launches += (uint64_t)p.kernels;
        s.total_ms += ms;
        s.bytes += p.bytes;
        s.ops += p.ops;
        event_pool_.push_back(p.a);
        event_pool_.push_back(p.b);
    }
}

bool Context::stat(const char* name, KernelStat* out) {
    flush_timings();
    std::lock_guard<std::mutex> g(prof_mu_);
    auto it = stats_.find(name);
    if (it == stats_.end()) return false;
    *out = it->second;
    return true;
}

void Context::reset_stats() {
    flush_timings();
    std::lock_guard<std::mutex> g(prof_mu_);
    stats_.clear();
}

// ============================== DevMem ==============================

int DevMem::alloc(Context* ctx, size_t bytes, cudaStream_t stream) {
    reset();
    if (bytes == 0) bytes = 16;
    bytes = (bytes + 255) & ~(size_t)255;
    if (!ctx->reserve(bytes)) return kENoMem;
    if (!stream) stream = ctx->stream();
    void* p = nullptr;
    if (cudaMallocAsync(&p, bytes, stream) != cudaSuccess) {
        cudaGetLastError();
        ctx->release(bytes);
        return kENoMem;
    }
    ctx_ = ctx;
    ptr_ = p;
    bytes_ = bytes;
    stream_ = stream;
    return kOk;
}

void DevMem::reset() {
    if (ptr_) {
        cudaFreeAsync(ptr_, stream_);
        ctx_->release(bytes_);
    }
    ptr_ = nullptr;
    bytes_ = 0;
    ctx_ = nullptr;
    stream_ = nullptr;
}

// ============================== helpers ==============================

namespace {

inline fq to_fq(const uint4& v) { return fq{{v.x, v.y, v.z, v.w}}; }

void unpack_module(const uint8_t* src, uint32_t n, Module& m) {
    m.n = n;
    m.c.resize((size_t)kRank * n);
    const uint4* p = reinterpret_cast<const uint4*>(src);
    for (size_t i = 0; i < m.c.size(); ++i) m.c[i] = to_fq(p[i]);
}

uint32_t mac_parts(uint32_t s, int njobs, uint32_t count) {
    const uint32_t ctas = ((s + 127) / 128) * 64u * (uint32_t)njobs;
    uint32_t parts = (1216u + ctas - 1) / ctas;
    if (parts > 16) parts = 16;
    if (parts > count) parts = count ? count : 1;
    return parts ? parts : 1;
}

}  // namespace

#define DM_CU(call, what)                                                                     \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return fail(kECuda, std::string(what) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Launch with optional event timing on the prover stream.
#define DM_LAUNCH(name, bytes, ops, call) DM_LAUNCH_N(name, bytes, ops, 1, call)
#define DM_LAUNCH_N(name, bytes, ops, nk, call)                                            \
    do {                                                                                   \
        cudaEvent_t ea_ = nullptr;                                                         \
        if (ctx_->profiling()) {                                                           \
            ea_ = ctx_->take_event();                                                      \
            cudaEventRecord(ea_, s_);                                                      \
        }                                                                                  \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) return fail(kECuda, std::string(name) + ": " + cudaGetErrorString(e_)); \
        if (ea_) {                                                                         \
            cudaEvent_t eb_ = ctx_->take_event();                                          \
            cudaEventRecord(eb_, s_);                                                      \
            ctx_->record(name, ea_, eb_, (double)(bytes), (double)(ops), (nk));            \
        }                                                                                  \
    } while (0)

// ============================== GpuProver ==============================

uint64_t GpuProver::footprint(uint64_t len) {
    uint32_t d;
    uint64_t S;
    if (!square_layout_for_byte_len(len, &d, &S)) return std::numeric_limits<uint64_t>::max();
    const uint64_t S2 = S * S;
    uint64_t b = 0;
    b += len + 16;                                   // file
    b += file_hash_scratch_words(len) * 4 + 64;       // hash scratch + id
    b += S2 * 16 + S2 / 2 * 16;                       // m_a, m_b
    b += 8 * S2 * 16 + 4 * S2 * 16;                   // g_a, g_b
    b += S2 * 32 + 8 * S2 * 32;                       // mhat, ghat
    b += 3ull * 16 * 64 * S * 4;                      // partials
    b += 8ull * 8 * S * 16 + 64;                      // commitments + flags
    return b;
}

void GpuProver::release_all() {
    DevMem* all[] = {&file_, &hash_scratch_, &file_id_, &m_a_, &m_b_, &g_a_, &g_b_, &mhat_, &ghat_, &partials_,
                     &comm_, &flags_};
    for (DevMem* m : all) m->reset();
}

GpuProver::~GpuProver() {
    if (s_) {
        cudaStreamSynchronize(s_);
        release_all();
        cudaStreamSynchronize(s_);
        cudaStreamDestroy(s_);
    }
    if (ev_start_) cudaEventDestroy(ev_start_);
    if (ev_end_) cudaEventDestroy(ev_end_);
    if (pinned_) ctx_->put_pinned(pinned_, pinned_bytes_);
}

double GpuProver::device_ms() const {
    float ms = 0.f;
    if (!ev_start_ || !ev_end_ || cudaEventElapsedTime(&ms, ev_start_, ev_end_) != cudaSuccess) return -1.0;
    return ms;
}

int GpuProver::fail(int code, const std::string& msg) {
    failed_ = true;
    ctx_->set_error(msg);
    return code;
}

int GpuProver::init(const uint8_t* file, uint64_t len, bool on_device, const uint8_t seed[32], const uint8_t epoch[32],
                    uint64_t max_preprocess_bytes) {
    uint32_t d;
    uint64_t S;
    if (!square_layout_for_byte_len(len, &d, &S)) return fail(kEInval, "square witness dimension overflow");
    const uint64_t est = S * S * 16 * 2;  // io.rs:42-49
    if (est > max_preprocess_bytes)
        return fail(kEInval, "full witness expansion requires " + std::to_string(est) +
                                 " bytes, above max_preprocess_bytes=" + std::to_string(max_preprocess_bytes) +
                                 "; split the file into smaller statements");
    if (d > (uint32_t)kMaxDepth)
        return fail(kEUnsupported, "fold depth " + std::to_string(d) + " exceeds the supported maximum " +
                                       std::to_string(kMaxDepth));
    if (len > 0 && file == nullptr) return fail(kEInval, "null file buffer");
    d_ = d;
    S_ = N_ = n_ = (uint32_t)S;
    DM_CU(cudaSetDevice(ctx_->device()), "cudaSetDevice");
    DM_CU(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking), "cudaStreamCreate");

    const uint64_t S2 = S * S;
    int rc = kOk;
    auto need = [&](DevMem& m, size_t bytes) {
        if (rc == kOk) rc = m.alloc(ctx_, bytes, s_);
    };
    if (!on_device) need(file_, len + 16);
    need(hash_scratch_, file_hash_scratch_words(len) * 4);
    need(file_id_, 64);
    need(m_a_, S2 * 16);
    need(m_b_, S2 / 2 * 16);
    need(g_a_, 8 * S2 * 16);
    need(g_b_, 4 * S2 * 16);
    need(mhat_, S2 * 32);
    need(ghat_, 8 * S2 * 32);
    need(partials_, 3ull * 16 * 64 * S * 4);
    need(comm_, 8ull * kRank * S * 16);
    need(flags_, 64);
    if (rc != kOk) return fail(rc, "HBM budget exhausted allocating prover state (" + std::to_string(footprint(len)) + " bytes)");
    pinned_bytes_ = 3ull * kRank * S * 16 + 64;
    pinned_ = static_cast<uint8_t*>(ctx_->get_pinned(pinned_bytes_));
    if (!pinned_) return fail(kECuda, "cudaMallocHost failed");

    DM_CU(cudaEventCreate(&ev_start_), "cudaEventCreate");
    DM_CU(cudaEventCreate(&ev_end_), "cudaEventCreate");
    DM_CU(cudaEventRecord(ev_start_, s_), "cudaEventRecord");
    const uint8_t* d_file = on_device ? file : file_.as<uint8_t>();
    if (!on_device && len) DM_CU(cudaMemcpyAsync(file_.as<uint8_t>(), file, len, cudaMemcpyHostToDevice, s_), "H2D file");
    DM_CU(cudaMemsetAsync(flags_.as<uint32_t>(), 0, 64, s_), "memset flags");

    const uint64_t nchunks = len == 0 ? 1 : (len + 1023) / 1024;
    DM_LAUNCH_N("file_hash", len + nchunks * 32, nchunks * 16, nchunks > 1 ? 2 : 1,
              launch_file_hash(d_file, len, hash_scratch_.as<uint32_t>(), file_id_.as<uint32_t>(), s_));
    DM_LAUNCH("unpack_witness", len + S2 * 16, S2,
              launch_unpack_witness(d_file, len, S2, m_a_.as<uint4>(), s_));
    blake3_keyed_hash(seed, "g0", 2, st_.g_0_seed);  // sis.rs:70, 208-210
    DM_LAUNCH("gen_generators", 8 * S2 * 16, 8 * S2,
              launch_gen_generators(st_.g_0_seed, S, d, g_a_.as<uint4>(), s_));
    st_.original_len_bytes = len;
    st_.d = d;
    rc = run_init_commit();
    if (rc != kOk) return rc;
    tr_ = Transcript(epoch, st_.file_id);
    return kOk;
}

// Initial commitment com_0 plus round 0's vector cross terms from one transform of m and g.
int GpuProver::run_init_commit() {
    const DeviceTables& T = ctx_->tables();
    const uint32_t L = d_, S = S_;
    const uint64_t S2 = (uint64_t)S * S;
    DM_LAUNCH("ntt_fwd", S2 * 48, (double)S * 8 * (S / 2) * L,
              launch_ntt_fwd(T, m_a_.as<uint4>(), mhat_.as<uint32_t>(), S, L, s_));
    DM_LAUNCH("ntt_fwd", 8 * S2 * 48, (double)8 * S * 8 * (S / 2) * L,
              launch_ntt_fwd(T, g_a_.as<uint4>(), ghat_.as<uint32_t>(), 8ull * S, L, s_));
    MacJob jobs[3] = {{0, 0, S}, {S / 2, 0, S / 2}, {0, S / 2, S / 2}};
    const int nj = S >= 2 ? 3 : 1;
    const uint32_t parts = mac_parts(S, nj, S / 2 ? S / 2 : 1);
    DM_LAUNCH("mac", 2 * S2 * 8 * 32 + 2 * S2 * 32, 2.0 * S2 * 64,
              launch_mac(T, ghat_.as<uint32_t>(), mhat_.as<uint32_t>(), L, jobs, nj, parts, partials_.as<uint32_t>(), s_));
    uint4* C = comm_.as<uint4>();
    const size_t slot = (size_t)kRank * S;
    FinishJob fj[3];
    for (int j = 0; j < nj; ++j)
        fj[j] = FinishJob{partials_.as<uint32_t>() + (size_t)j * parts * 64 * S, parts, L, kFinishPlain, C + j * slot};
    DM_LAUNCH("finish", 0, 0, launch_finish(T, fj, nj, s_));
    DM_CU(cudaMemcpyAsync(pinned_, C, nj * slot * 16, cudaMemcpyDeviceToHost, s_), "D2H commitments");
    DM_CU(cudaMemcpyAsync(pinned_ + 3 * slot * 16, file_id_.as<uint8_t>(), 32, cudaMemcpyDeviceToHost, s_), "D2H file id");
    DM_CU(cudaStreamSynchronize(s_), "init commit");
    std::memcpy(st_.file_id, pinned_ + 3 * slot * 16, 32);
    unpack_module(pinned_, S, st_.com_0);
    current_ = st_.com_0;
    if (nj == 3) {
        unpack_module(pinned_ + slot * 16, S, pend_l_);
        unpack_module(pinned_ + 2 * slot * 16, S, pend_r_);
    }
    return kOk;
}

int GpuProver::fold_round(uint64_t j, RoundRecord* out) {
    if (failed_) return fail(kEState, "prover is in a failed state");
    if (j != round_) return fail(kEState, "round index mismatch");
    if (round_ >= d_) return fail(kEState, "all rounds have finished");
    const DeviceTables& T = ctx_->tables();
    const uint32_t L = d_ - (uint32_t)j, s = 1u << L, h = s / 2;
    const uint64_t s2 = (uint64_t)s * s;
    const size_t slot = (size_t)kRank * S_;
    uint4* C = comm_.as<uint4>();
    uint4 *cC = C, *cL = C + slot, *cR = C + 2 * slot, *cCt = C + 3 * slot, *cV = C + 4 * slot, *cLp = C + 5 * slot,
          *cRp = C + 6 * slot, *cChk = C + 7 * slot;
    uint32_t* flags = flags_.as<uint32_t>();

    // ---- vector stage (prover.rs:148-214) ----
    const fq x = tr_.challenge_vec(j, current_, pend_l_, pend_r_);
    const fq xi = fq_inv(x);
    DM_LAUNCH("combine", (double)kRank * s * 64, kRank * s, launch_combine(cC, cL, cR, xi, x, cCt, (uint64_t)kRank * s, s_));
    DM_LAUNCH("fold_vec", (double)s2 / 2 * 48, s2 / 2, launch_fold_vec(m_a_.as<uint4>(), m_b_.as<uint4>(), s2 / 2, x, s_));
    DM_LAUNCH("fold_vec", (double)4 * s2 * 48, 4 * s2,
              launch_fold_vec(g_a_.as<uint4>(), g_b_.as<uint4>(), 4 * s2, xi, s_));
    DM_LAUNCH("ntt_fwd", (double)s2 / 2 * 48, (double)h * 8 * h * L,
              launch_ntt_fwd(T, m_b_.as<uint4>(), mhat_.as<uint32_t>(), h, L, s_));
    DM_LAUNCH("ntt_fwd", (double)4 * s2 * 48, (double)4 * s * 8 * h * L,
              launch_ntt_fwd(T, g_b_.as<uint4>(), ghat_.as<uint32_t>(), 4ull * s, L, s_));
    const uint32_t parts_a = mac_parts(h, 1, h);
    uint32_t* P = partials_.as<uint32_t>();
    uint32_t* pchk = P;
    uint32_t* plp = P + (size_t)parts_a * 64 * s;
    uint32_t* prp = plp + (size_t)parts_a * 64 * h;
    DM_LAUNCH("mac_split", (double)4 * s2 * 32 + (double)s2 / 2 * 32, (double)4 * s2 * 8 * 2,
              launch_mac_split(T, ghat_.as<uint32_t>(), mhat_.as<uint32_t>(), L, h, parts_a, pchk, plp, prp, s_));
    FinishJob fa[3] = {{pchk, parts_a, L, kFinishPlain, cV},
                       {plp, parts_a, L - 1, kFinishSplitL, cLp},
                       {prp, parts_a, L - 1, kFinishSplitR, cRp}};
    DM_LAUNCH("finish", 0, 0, launch_finish(T, fa, 3, s_));
    DM_LAUNCH("compare", (double)kRank * s * 32, kRank * s, launch_compare(cV, cCt, (uint64_t)kRank * s, flags, s_));
    uint8_t* hp = pinned_;
    DM_CU(cudaMemcpyAsync(hp, cCt, (size_t)kRank * s * 16, cudaMemcpyDeviceToHost, s_), "D2H Ct");
    DM_CU(cudaMemcpyAsync(hp + slot * 16, cLp, (size_t)kRank * h * 16, cudaMemcpyDeviceToHost, s_), "D2H Lp");
    DM_CU(cudaMemcpyAsync(hp + 2 * slot * 16, cRp, (size_t)kRank * h * 16, cudaMemcpyDeviceToHost, s_), "D2H Rp");
    DM_CU(cudaMemcpyAsync(hp + 3 * slot * 16, flags, 8, cudaMemcpyDeviceToHost, s_), "D2H flags");
    DM_CU(cudaStreamSynchronize(s_), "vector stage");
    uint32_t fl[2];
    std::memcpy(fl, hp + 3 * slot * 16, 8);
    if (fl[0]) return fail(kEInvariant, "vector folding invariant failed");
    Module ct, lp, rp;
    unpack_module(hp, s, ct);
    unpack_module(hp + slot * 16, h, lp);
    unpack_module(hp + 2 * slot * 16, h, rp);

    // ---- poly stage (prover.rs:231-291) ----
    const fq y = tr_.challenge_poly(j, ct, lp, rp);
    const fq yi = fq_inv(y);
    DM_LAUNCH("combine", (double)kRank * h * 64, kRank * h, launch_combine_even(cCt, cLp, cRp, yi, y, cC, L - 1, s_));
    DM_LAUNCH("fold_poly", (double)s2 / 2 * 24, s2 / 4,
              launch_fold_poly(m_b_.as<uint4>(), m_a_.as<uint4>(), h, L - 1, y, false, s_));
    DM_LAUNCH("fold_poly", (double)4 * s2 * 24, 2 * s2,
              launch_fold_poly(g_b_.as<uint4>(), g_a_.as<uint4>(), 4ull * s, L - 1, yi, true, s_));
    const uint32_t L2 = L - 1, s2n = h;  // next square size
    const uint64_t q2 = (uint64_t)s2n * s2n;
    DM_LAUNCH("ntt_fwd", (double)q2 * 48, (double)s2n * 8 * (s2n / 2) * L2,
              launch_ntt_fwd(T, m_a_.as<uint4>(), mhat_.as<uint32_t>(), s2n, L2, s_));
    DM_LAUNCH("ntt_fwd", (double)8 * q2 * 48, (double)8 * s2n * 8 * (s2n / 2) * L2,
              launch_ntt_fwd(T, g_a_.as<uint4>(), ghat_.as<uint32_t>(), 8ull * s2n, L2, s_));
    MacJob jobs[3] = {{0, 0, s2n}, {s2n / 2, 0, s2n / 2}, {0, s2n / 2, s2n / 2}};
    const int nj = s2n >= 2 ? 3 : 1;
    const uint32_t parts_b = mac_parts(s2n, nj, s2n / 2 ? s2n / 2 : 1);
    DM_LAUNCH("mac", (double)2 * q2 * 8 * 32 + 2 * q2 * 32, 2.0 * q2 * 64,
              launch_mac(T, ghat_.as<uint32_t>(), mhat_.as<uint32_t>(), L2, jobs, nj, parts_b, P, s_));
    FinishJob fb[3];
    uint4* outs[3] = {cChk, cL, cR};
    for (int t = 0; t < nj; ++t) fb[t] = FinishJob{P + (size_t)t * parts_b * 64 * s2n, parts_b, L2, kFinishPlain, outs[t]};
    DM_LAUNCH("finish", 0, 0, launch_finish(T, fb, nj, s_));
    DM_LAUNCH("compare", (double)kRank * s2n * 32, kRank * s2n,
              launch_compare(cChk, cC, (uint64_t)kRank * s2n, flags + 1, s_));
    DM_CU(cudaMemcpyAsync(hp, cC, (size_t)kRank * s2n * 16, cudaMemcpyDeviceToHost, s_), "D2H C");
    if (nj == 3) {
        DM_CU(cudaMemcpyAsync(hp + slot * 16, cL, (size_t)kRank * s2n * 16, cudaMemcpyDeviceToHost, s_), "D2H L");
        DM_CU(cudaMemcpyAsync(hp + 2 * slot * 16, cR, (size_t)kRank * s2n * 16, cudaMemcpyDeviceToHost, s_), "D2H R");
    }
    const bool last = (j + 1 == d_);
    if (last) DM_CU(cudaMemcpyAsync(hp + 3 * slot * 16 + 16, m_a_.as<uint4>(), 16, cudaMemcpyDeviceToHost, s_), "D2H m*");
    DM_CU(cudaMemcpyAsync(hp + 3 * slot * 16, flags, 8, cudaMemcpyDeviceToHost, s_), "D2H flags");
    if (last) DM_CU(cudaEventRecord(ev_end_, s_), "cudaEventRecord");
    DM_CU(cudaStreamSynchronize(s_), "poly stage");
    std::memcpy(fl, hp + 3 * slot * 16, 8);
    if (fl[1]) return fail(kEInvariant, "round folding invariant failed");

    RoundRecord rec;
    rec.round = j;
    rec.l_vec = std::move(pend_l_);
    rec.r_vec = std::move(pend_r_);
    rec.l_poly = std::move(lp);
    rec.r_poly = std::move(rp);
    unpack_module(hp, s2n, current_);
    if (nj == 3) {
        unpack_module(hp + slot * 16, s2n, pend_l_);
        unpack_module(hp + 2 * slot * 16, s2n, pend_r_);
    } else {
        pend_l_ = Module::zero(s2n);
        pend_r_ = Module::zero(s2n);
    }
    if (last) {
        opening_ = to_fq(*reinterpret_cast<const uint4*>(hp + 3 * slot * 16 + 16));
        have_opening_ = true;
    }
    N_ = n_ = s2n;
    round_ += 1;
    if (out) *out = std::move(rec);
    return kOk;
}

bool GpuProver::final_opening(fq* out) const {
    if (!(round_ == d_ && N_ == 1 && n_ == 1 && have_opening_)) return false;
    *out = opening_;
    return true;
}

// ============================== GpuVerifier ==============================

uint64_t GpuVerifier::footprint(uint64_t N, uint64_t n) { return 2 * N * kRank * n * 16 + 64; }

GpuVerifier::~GpuVerifier() {
    if (s_) {
        cudaStreamSynchronize(s_);
        g_[0].reset();
        g_[1].reset();
        cudaStreamSynchronize(s_);
        cudaStreamDestroy(s_);
    }
}

int GpuVerifier::fail(int code, const std::string& msg) {
    ctx_->set_error(msg);
    return code;
}

int GpuVerifier::init(const uint8_t* statement, size_t len, const uint8_t epoch[32]) {
    const uint8_t* p = statement;
    if (!decode_statement(p, statement + len, st_)) return fail(kEDeserialize, "statement deserialization failed");
    uint32_t d;
    uint64_t N;
    if (!square_layout_for_byte_len(st_.original_len_bytes, &d, &N))
        return fail(kEInval, "derive initial witness layout from statement");
    const uint32_t n = st_.com_0.n;
    if (n == 0 || (n & (n - 1)) || n > (1u << kLogMaxProverRing)) return fail(kEInval, "statement commitment ring length unsupported");
    if (N > (1u << kLogMaxProverRing)) return fail(kEUnsupported, "statement vector length unsupported");
    N_ = (uint32_t)N;
    n_ = n;
    rounds_ = st_.d;
    current_ = st_.com_0;
    tr_ = Transcript(epoch, st_.file_id);
    DM_CU(cudaSetDevice(ctx_->device()), "cudaSetDevice");
    DM_CU(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking), "cudaStreamCreate");
    const uint64_t bytes = (uint64_t)N * kRank * n * 16;
    if (g_[0].alloc(ctx_, bytes, s_) != kOk || g_[1].alloc(ctx_, bytes / 2 + 16, s_) != kOk)
        return fail(kENoMem, "HBM budget exhausted allocating verifier generators");
    uint32_t Ln = 0;
    while ((1u << Ln) < n) ++Ln;
    cudaError_t e = launch_gen_generators(st_.g_0_seed, N, Ln, g_[0].as<uint4>(), s_);
    if (e != cudaSuccess) return fail(kECuda, std::string("gen_generators: ") + cudaGetErrorString(e));
    cur_ = 0;
    return kOk;
}

int GpuVerifier::update_commitment(const RoundRecord& rec) {
    if (rec.round != round_) return fail(kEVerify, "round mismatch in round record");
    Module vfc;
    fq x_inv = fq_zero(), y_inv = fq_zero();
    const bool vec = N_ > 1;
    if (vec) {
        const fq x = tr_.challenge_vec(round_, current_, rec.l_vec, rec.r_vec);
        x_inv = fq_inv(x);
        Module t;
        if (!module_add_scaled(current_, rec.l_vec, x_inv, t) || !module_add_scaled(t, rec.r_vec, x, vfc))
            return fail(kEVerify, "module ring length mismatch");
    } else {
        const Module zero = Module::zero(current_.n);
        (void)tr_.challenge_vec(round_, current_, zero, zero);
        if (!(rec.l_vec == zero && rec.r_vec == zero))
            return fail(kEVerify, "scalar vector stage must emit zero vec cross-terms");
        vfc = current_;
    }
    const bool poly = n_ > 1;
    Module next;
    if (poly) {
        const fq y = tr_.challenge_poly(round_, vfc, rec.l_poly, rec.r_poly);
        y_inv = fq_inv(y);
        if (vfc.n < 2) return fail(kEVerify, "cannot split scalar commitment");
        Module t;
        if (!module_add_scaled(module_even(vfc), rec.l_poly, y_inv, t) || !module_add_scaled(t, rec.r_poly, y, next))
            return fail(kEVerify, "module ring length mismatch");
    } else {
        const Module zero = Module::zero(1);
        (void)tr_.challenge_poly(round_, vfc, zero, zero);
        if (!(rec.l_poly == zero && rec.r_poly == zero))
            return fail(kEVerify, "scalar stage must emit zero poly cross-terms");
        next = std::move(vfc);
    }
    uint32_t L = 0;
    while ((1u << L) < n_) ++L;
    cudaError_t e = launch_fold_gen_round(g_[cur_].as<uint4>(), g_[cur_ ^ 1].as<uint4>(), N_, L, x_inv, y_inv, vec,
                                          poly, s_);
    if (e != cudaSuccess) return fail(kECuda, std::string("fold_gen_round: ") + cudaGetErrorString(e));
    cur_ ^= 1;
    if (vec) N_ /= 2;
    if (poly) n_ /= 2;
    current_ = std::move(next);
    round_ += 1;
    return kOk;
}

int GpuVerifier::verify_final_opening(const fq& opening) {
    if (round_ != rounds_) return fail(kEVerify, "cannot verify final opening before all rounds replay");
    if (N_ != 1) return fail(kEVerify, "terminal generator family must have length one");
    std::vector<uint4> g((size_t)kRank * n_);
    cudaError_t e = cudaMemcpyAsync(g.data(), g_[cur_].as<uint4>(), g.size() * 16, cudaMemcpyDeviceToHost, s_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s_);
    if (e != cudaSuccess) return fail(kECuda, std::string("D2H generators: ") + cudaGetErrorString(e));
    Module rhs;
    rhs.n = n_;
    rhs.c.resize(g.size());
    const fq o = fq_from_u128_words(opening);
    for (size_t i = 0; i < g.size(); ++i) rhs.c[i] = fq_mul(to_fq(g[i]), o);
    if (!(rhs == current_)) return fail(kEVerify, "final opening mismatch");
    return kOk;
}

// ============================== one-shot ==============================

int prove_all(Context* ctx, const uint8_t* file, uint64_t len, bool on_device, const uint8_t seed[32],
              const uint8_t epoch[32], std::vector<uint8_t>* proof, double* device_ms) {
    GpuProver p(ctx);
    int rc = p.init(file, len, on_device, seed, epoch, std::numeric_limits<uint64_t>::max());
    if (rc != kOk) return rc;
    proof->clear();
    proof->reserve(proof_encoded_size(p.rounds_total()));
    encode_statement(*proof, p.statement());
    put_u64(*proof, p.rounds_total());
    for (uint32_t r = 0; r < p.rounds_total(); ++r) {
        RoundRecord rec;
        rc = p.fold_round(r, &rec);
        if (rc != kOk) return rc;
        encode_record(*proof, rec);
    }
    fq o;
    if (!p.final_opening(&o)) {
        ctx->set_error("final opening unavailable");
        return kEState;
    }
    const size_t base = proof->size();
    proof->resize(base + 16);
    fq_to_bytes(o, proof->data() + base);
    if (device_ms) *device_ms = p.device_ms();
    return kOk;
}

int verify_proof(Context* ctx, const uint8_t* proof, size_t len, const uint8_t epoch[32]) {
    const uint8_t *p = proof, *end = proof + len;
    Statement st;
    if (!decode_statement(p, end, st)) {
        ctx->set_error("statement deserialization failed");
        return kEDeserialize;
    }
    GpuVerifier v(ctx);
    int rc = v.init(proof, (size_t)(p - proof), epoch);
    if (rc != kOk) return rc;
    if (end - p < 8) {
        ctx->set_error("proof truncated");
        return kEDeserialize;
    }
    uint64_t count = 0;
    for (int i = 7; i >= 0; --i) count = (count << 8) | p[i];
    p += 8;
    for (uint64_t r = 0; r < count; ++r) {
        RoundRecord rec;
        if (!decode_record(p, end, rec)) {
            ctx->set_error("round record deserialization failed");
            return kEDeserialize;
        }
        rc = v.update_commitment(rec);
        if (rc != kOk) return rc;
    }
    if (end - p < 16) {
        ctx->set_error("proof truncated");
        return kEDeserialize;
    }
    return v.verify_final_opening(fq_from_bytes(p));
}

}  // namespace dm
