#include "engine.h"

#include <cstdio>
#include <cstring>
#include <limits>

#include "dm_jobs.cuh"
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
    c->sm_count_ = prop.multiProcessorCount > 0 ? prop.multiProcessorCount : 152;
    for (int k = 0; k < kTuneKnobs; ++k)
        for (int L = 0; L <= kLogMaxProverRing; ++L) c->tune_[k][L].store(tune_default(k, L));
    if ((e = cudaStreamCreateWithFlags(&c->stream_, cudaStreamNonBlocking)) != cudaSuccess) {
        *err = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
        return kECuda;
    }
    if ((e = upload_tables(&c->tables_)) != cudaSuccess || (e = upload_ref_tables(&c->ref_tables_)) != cudaSuccess) {
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

int Context::set_tuning(int knob, uint32_t L, int value) {
    if (knob < 0 || knob >= kTuneKnobs || L > (uint32_t)kLogMaxProverRing) return kEInval;
    if (knob == kTuneNttGroup ? (value != 32 && value != 64)
        : knob == kTuneSplitCoords  ? (value != 1 && value != 2 && value != 4 && value != 8)
        : knob == kTuneTripleCoords ? (value != 1 && value != 2 && value != 4)
        : knob == kTuneNttRadix     ? (value != 16 && value != 32)
                                   : (value < 1 || value > 32))
        return kEInval;
    tune_[knob][L].store(value, std::memory_order_relaxed);
    return kOk;
}

uint32_t Context::mac_parts(int knob, uint32_t L, uint32_t threads_per_row, uint32_t count) const {
    return mac_parts_for(tuning(knob, L), threads_per_row, count);
}

uint32_t Context::mac_parts_for(int blocks_per_sm, uint32_t threads_per_row, uint32_t count, uint32_t rows) const {
    const uint32_t per_part = ((threads_per_row + 127) / 128) * rows;
    uint32_t parts = (uint32_t)sm_count_ * (uint32_t)blocks_per_sm / per_part;
    if (parts > kMaxMacParts) parts = kMaxMacParts;
#ifndef DM_MIN_PART_COLS
#define DM_MIN_PART_COLS 8
#endif
    const uint32_t most = (count + DM_MIN_PART_COLS - 1) / DM_MIN_PART_COLS;  // columns per part at least this
    if (parts > most) parts = most;
    return parts ? parts : 1;
}

int Context::set_prover_cache(uint64_t cap_bytes) {
    cudaSetDevice(device_);
    if (prover_cache_) {
        // the old cache goes once nothing holds it: every entry must be unreferenced
        if (!prover_cache_->trim(~0ull >> 1) && prover_cache_->bytes() > 0) return kEState;
        prover_cache_.reset();
    }
    if (cap_bytes) prover_cache_.reset(new ProverGenCache(this, cap_bytes));
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
        // best fit: the smallest idle buffer that holds `bytes`, so a small request
        // does not take a large file's buffer
        size_t best = pinned_free_.size();
        for (size_t i = 0; i < pinned_free_.size(); ++i)
            if (pinned_free_[i].first >= bytes &&
                (best == pinned_free_.size() || pinned_free_[i].first < pinned_free_[best].first))
                best = i;
        if (best < pinned_free_.size()) {
            void* p = pinned_free_[best].second;
            pinned_free_.erase(pinned_free_.begin() + (long)best);
            return p;
        }
    }
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> g(pin_mu_);
    pinned_cap_[p] = bytes;
    return p;
}

void Context::put_pinned(void* p, size_t bytes) {
    if (!p) return;
    std::lock_guard<std::mutex> g(pin_mu_);
    // back into the pool at the size it was allocated with (a reused buffer may be
    // larger than the request that returns it)
    const auto it = pinned_cap_.find(p);
    pinned_free_.emplace_back(it != pinned_cap_.end() ? it->second : bytes, p);
}

Context::~Context() {
    cudaSetDevice(device_);
    prover_cache_.reset();  // returns its budget while the accounting is alive
    if (stream_) cudaStreamSynchronize(stream_);
    if (flush_buf_) cudaFree(flush_buf_);
    for (auto& pp : pinned_free_) cudaFreeHost(pp.second);

    flush_timings();
    for (cudaEvent_t e : event_pool_) cudaEventDestroy(e);
    free_tables(&tables_);
    free_ref_tables(&ref_tables_);
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

void Context::record(const char* name, cudaEvent_t a, cudaEvent_t b, double bytes, double ops, int kernels,
                     cudaStream_t st) {
    std::lock_guard<std::mutex> g(prof_mu_);
    pending_.push_back(Pending{name, a, b, bytes, ops, kernels, st});
}

int Context::start_trace() {
    cudaSetDevice(device_);
    flush_timings();
    cudaEvent_t ref = take_event();
    if (!ref) return kECuda;
    // every stream's earlier work ends before the reference point
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaEventRecord(ref, stream_);
    if (e == cudaSuccess) e = cudaEventSynchronize(ref);
    if (e != cudaSuccess) {
        set_error(std::string("start_trace: ") + cudaGetErrorString(e));
        return kECuda;
    }
    std::lock_guard<std::mutex> g(prof_mu_);
    if (trace_ref_) event_pool_.push_back(trace_ref_);
    trace_ref_ = ref;
    trace_host_ref_ = std::chrono::steady_clock::now();
    trace_csv_.clear();
    trace_streams_.clear();
    tracing_ = true;
    profiling_ = true;
    return kOk;
}

void Context::trace_host(const char* kind, int lane, std::chrono::steady_clock::time_point t0,
                         std::chrono::steady_clock::time_point t1, double count, int launches) {
    std::lock_guard<std::mutex> g(prof_mu_);
    if (!tracing_) return;
    using ms = std::chrono::duration<double, std::milli>;
    char line[160];
    std::snprintf(line, sizeof line, "%s,%d,%.4f,%.4f,%.0f,%d\n", kind, lane, ms(t0 - trace_host_ref_).count(),
                  ms(t1 - trace_host_ref_).count(), count, launches);
    trace_csv_ += line;
}

int Context::read_trace(std::string* csv, bool stop) {
    flush_timings();
    std::lock_guard<std::mutex> g(prof_mu_);
    if (csv) csv->swap(trace_csv_);
    trace_csv_.clear();
    if (stop) {
        tracing_ = false;
        if (trace_ref_) event_pool_.push_back(trace_ref_);
        trace_ref_ = nullptr;
        trace_streams_.clear();
    }
    return kOk;
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
        if (tracing_ && trace_ref_) {
            float t0 = 0.f, t1 = 0.f;
            cudaEventElapsedTime(&t0, trace_ref_, p.a);
            cudaEventElapsedTime(&t1, trace_ref_, p.b);
            size_t sid = 0;
            while (sid < trace_streams_.size() && trace_streams_[sid] != p.st) ++sid;
            if (sid == trace_streams_.size()) trace_streams_.push_back(p.st);
            char line[160];
            std::snprintf(line, sizeof line, "%s,%zu,%.4f,%.4f,%.0f,%d\n", p.name.c_str(), sid, t0, t1, p.bytes,
                          p.kernels);
            trace_csv_ += line;
        }
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

// ============================== GenCache ==============================

struct GenCache::Entry {
    void* ptr = nullptr;
    uint64_t bytes = 0;
    cudaEvent_t ready = nullptr;
    int refs = 0;
    uint64_t last_use = 0;
};

GenCache::~GenCache() {
    std::lock_guard<std::mutex> g(mu_);
    for (auto& kv : map_) {
        Entry* e = kv.second;
        if (e->ready) cudaEventSynchronize(e->ready);
        cudaFree(e->ptr);
        ctx_->release(e->bytes);
        if (e->ready) cudaEventDestroy(e->ready);
        delete e;
    }
    map_.clear();
}

bool GenCache::evict_one() {
    auto victim = map_.end();
    for (auto it = map_.begin(); it != map_.end(); ++it)
        if (it->second->refs == 0 && (victim == map_.end() || it->second->last_use < victim->second->last_use))
            victim = it;
    if (victim == map_.end()) return false;
    Entry* e = victim->second;
    // every holder synchronised its stream before releasing, so nothing reads it
    cudaFree(e->ptr);
    ctx_->release(e->bytes);
    cudaEventDestroy(e->ready);
    st_.bytes -= e->bytes;
    st_.entries -= 1;
    st_.evictions += 1;
    delete e;
    map_.erase(victim);
    return true;
}

bool GenCache::evict_for(uint64_t bytes) {
    for (;;) {
        if (st_.bytes + bytes <= cap_ && ctx_->reserve(bytes)) return true;
        if (!evict_one()) return false;
    }
}

bool GenCache::trim(uint64_t bytes) {
    std::lock_guard<std::mutex> g(mu_);
    for (;;) {
        if (ctx_->reserved() + bytes <= ctx_->budget()) return true;
        if (!evict_one()) return false;
    }
}

int GenCache::acquire(const uint8_t seed[32], uint64_t N, uint32_t log_n, cudaStream_t s, Ref* out) {
    std::vector<uint8_t> key(seed, seed + 32);
    for (int i = 0; i < 8; ++i) key.push_back((uint8_t)(N >> (8 * i)));
    key.push_back((uint8_t)log_n);
    const uint64_t bytes = (N * kRank << log_n) * 16;
    std::lock_guard<std::mutex> g(mu_);
    auto it = map_.find(key);
    if (it != map_.end()) {
        Entry* e = it->second;
        e->refs += 1;
        e->last_use = ++clock_;
        st_.hits += 1;
        *out = Ref{static_cast<const uint4*>(e->ptr), e->ready, e};
        return kOk;
    }
    st_.misses += 1;
    // a key is cached on its second sighting: proofs under per-file (or hostile)
    // seeds take the stream-ordered private path instead of a synchronous
    // allocation and an eviction each
    int& seen = seen_[key];
    if (seen++ == 0) {
        if (seen_.size() > 4096) seen_.clear();
        return kENoMem;
    }
    if (bytes > cap_ || !evict_for(bytes)) return kENoMem;
    Entry* e = new Entry;
    e->bytes = bytes;
    if (cudaMalloc(&e->ptr, bytes) != cudaSuccess) {
        cudaGetLastError();
        ctx_->release(bytes);
        delete e;
        return kENoMem;
    }
    // launched and recorded under the lock: a reader that finds the entry always
    // waits on a recorded event
    cudaEvent_t ta = nullptr;
    if (ctx_->profiling()) {
        ta = ctx_->take_event();
        cudaEventRecord(ta, s);
    }
    cudaError_t err = launch_gen_generators(seed, N, log_n, static_cast<uint4*>(e->ptr), s);
    if (ta) {
        cudaEvent_t tb = ctx_->take_event();
        cudaEventRecord(tb, s);
        ctx_->record("gen_generators", ta, tb, (double)bytes, (double)(bytes / 16));
    }
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&e->ready, cudaEventDisableTiming);
    if (err == cudaSuccess) err = cudaEventRecord(e->ready, s);
    if (err != cudaSuccess) {
        if (e->ready) cudaEventDestroy(e->ready);
        cudaStreamSynchronize(s);
        cudaFree(e->ptr);
        ctx_->release(bytes);
        delete e;
        return kECuda;
    }
    e->refs = 1;
    e->last_use = ++clock_;
    map_[key] = e;
    st_.bytes += bytes;
    st_.entries += 1;
    *out = Ref{static_cast<const uint4*>(e->ptr), e->ready, e};
    return kOk;
}

void GenCache::release(const Ref& r) {
    if (!r.entry) return;
    std::lock_guard<std::mutex> g(mu_);
    static_cast<Entry*>(r.entry)->refs -= 1;
}

GenCache::Stats GenCache::stats() {
    std::lock_guard<std::mutex> g(mu_);
    return st_;
}

// ============================== ProverGenCache ==============================

struct ProverGenCache::Entry {
    void* g = nullptr;
    void* ghat = nullptr;
    uint64_t bytes = 0;
    cudaEvent_t ready = nullptr;
    int refs = 0;
    uint64_t last_use = 0;
    bool published = false;  // the fill is enqueued and `ready` recorded
    bool poisoned = false;
    const void* filler = nullptr;  // the plan that fills it, until published
};

uint64_t ProverGenCache::entry_bytes(uint32_t L) {
    const uint64_t S2 = 1ull << (2 * L);
    return 8 * S2 * 16 + 8 * S2 * kPrimes * 4;
}

ProverGenCache::~ProverGenCache() {
    std::lock_guard<std::mutex> g(mu_);
    for (auto& kv : map_) {
        Entry* e = kv.second;
        if (e->ready) cudaEventSynchronize(e->ready);
        cudaFree(e->g);
        cudaFree(e->ghat);
        ctx_->release(e->bytes);
        if (e->ready) cudaEventDestroy(e->ready);
        delete e;
    }
    map_.clear();
}

bool ProverGenCache::evict_one() {
    auto victim = map_.end();
    for (auto it = map_.begin(); it != map_.end(); ++it)
        if (it->second->refs == 0 && (victim == map_.end() || it->second->last_use < victim->second->last_use))
            victim = it;
    if (victim == map_.end()) return false;
    Entry* e = victim->second;
    // holders release after their last reading stage completed on the device
    cudaFree(e->g);
    cudaFree(e->ghat);
    ctx_->release(e->bytes);
    cudaEventDestroy(e->ready);
    st_.bytes -= e->bytes;
    st_.entries -= 1;
    st_.evictions += 1;
    delete e;
    map_.erase(victim);
    return true;
}

int ProverGenCache::acquire(const uint8_t g0_seed[32], uint32_t L, const void* plan, Ref* out) {
    std::vector<uint8_t> key(g0_seed, g0_seed + 32);
    key.push_back((uint8_t)L);
    std::lock_guard<std::mutex> g(mu_);
    auto it = map_.find(key);
    if (it != map_.end()) {
        Entry* e = it->second;
        const bool same_plan = !e->published && plan && e->filler == plan;
        if (e->poisoned || (!e->published && !same_plan)) {
            // still being filled by a stage not yet enqueued (an event not yet
            // recorded cannot be waited on), or dropped by its last holder
            st_.misses += 1;
            return kENoMem;
        }
        e->refs += 1;
        e->last_use = ++clock_;
        st_.hits += 1;
        // in the filling plan itself the stream order covers the fill: no wait
        *out = Ref{static_cast<uint4*>(e->g), static_cast<uint32_t*>(e->ghat), same_plan ? nullptr : e->ready, e,
                   false};
        return kOk;
    }
    // first sighting: remember the key only (bounded; forgotten wholesale when full)
    int& seen = seen_[key];
    if (seen++ == 0) {
        if (seen_.size() > 4096) seen_.clear();
        st_.misses += 1;
        return kENoMem;
    }
    const uint64_t bytes = entry_bytes(L);
    if (bytes > cap_) {
        st_.misses += 1;
        return kENoMem;
    }
    for (;;) {
        if (st_.bytes + bytes <= cap_ && ctx_->reserve(bytes)) break;
        if (!evict_one()) {
            st_.misses += 1;
            return kENoMem;
        }
    }
    Entry* e = new Entry;
    e->bytes = bytes;
    const uint64_t S2 = 1ull << (2 * L);
    if (cudaMalloc(&e->g, 8 * S2 * 16) != cudaSuccess || cudaMalloc(&e->ghat, 8 * S2 * kPrimes * 4) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->ready, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        if (e->g) cudaFree(e->g);
        if (e->ghat) cudaFree(e->ghat);
        if (e->ready) cudaEventDestroy(e->ready);
        ctx_->release(bytes);
        delete e;
        st_.misses += 1;
        return kENoMem;
    }
    e->refs = 1;
    e->last_use = ++clock_;
    e->filler = plan;
    map_[key] = e;
    st_.bytes += bytes;
    st_.entries += 1;
    st_.fills += 1;
    *out = Ref{static_cast<uint4*>(e->g), static_cast<uint32_t*>(e->ghat), e->ready, e, true};
    return kOk;
}

void ProverGenCache::release(const Ref& r) {
    if (!r.entry) return;
    std::lock_guard<std::mutex> g(mu_);
    Entry* e = static_cast<Entry*>(r.entry);
    e->refs -= 1;
    if (e->poisoned && e->refs == 0) {
        for (auto it = map_.begin(); it != map_.end(); ++it)
            if (it->second == e) {
                cudaFree(e->g);
                cudaFree(e->ghat);
                ctx_->release(e->bytes);
                cudaEventDestroy(e->ready);
                st_.bytes -= e->bytes;
                st_.entries -= 1;
                delete e;
                map_.erase(it);
                break;
            }
    }
}

bool ProverGenCache::lookup(const uint8_t g0_seed[32], uint32_t L, Ref* out) {
    std::vector<uint8_t> key(g0_seed, g0_seed + 32);
    key.push_back((uint8_t)L);
    std::lock_guard<std::mutex> g(mu_);
    auto it = map_.find(key);
    if (it == map_.end() || !it->second->published || it->second->poisoned) return false;
    Entry* e = it->second;
    e->refs += 1;
    e->last_use = ++clock_;
    st_.hits += 1;
    *out = Ref{static_cast<uint4*>(e->g), static_cast<uint32_t*>(e->ghat), e->ready, e, false};
    return true;
}

void ProverGenCache::publish(const Ref& r) {
    if (!r.entry) return;
    std::lock_guard<std::mutex> g(mu_);
    static_cast<Entry*>(r.entry)->published = true;
    static_cast<Entry*>(r.entry)->filler = nullptr;
}

void ProverGenCache::poison(const Ref& r) {
    if (!r.entry) return;
    std::lock_guard<std::mutex> g(mu_);
    static_cast<Entry*>(r.entry)->poisoned = true;
    static_cast<Entry*>(r.entry)->filler = nullptr;
}

bool ProverGenCache::trim(uint64_t bytes) {
    std::lock_guard<std::mutex> g(mu_);
    for (;;) {
        if (ctx_->reserved() + bytes <= ctx_->budget()) return true;
        if (!evict_one()) return false;
    }
}

uint64_t ProverGenCache::bytes() {
    std::lock_guard<std::mutex> g(mu_);
    return st_.bytes;
}

ProverGenCache::Stats ProverGenCache::stats() {
    std::lock_guard<std::mutex> g(mu_);
    return st_;
}

// ============================== GpuVerifier ==============================

// What init allocates without a cache hit: g_0 and the first fold's half, each
// rounded to the allocator's 256 bytes.
uint64_t GpuVerifier::footprint(uint64_t N, uint64_t n) {
    const uint64_t full = N * kRank * n * 16;
    return ((full + 255) & ~(uint64_t)255) + ((full / 2 + 16 + 255) & ~(uint64_t)255);
}

GpuVerifier::~GpuVerifier() {
    if (done_) cudaEventDestroy(done_);
    if (s_) {
        cudaStreamSynchronize(s_);  // the folds may still read g_0 and the buffers
        g_[0].reset();
        g_[1].reset();
        if (cache_ && cache_ref_.entry) cache_->release(cache_ref_);
        if (prover_ref_.entry) ctx_->prover_cache()->release(prover_ref_);
        if (own_stream_) {
            cudaStreamSynchronize(s_);
            cudaStreamDestroy(s_);
        }
    }
}

int GpuVerifier::fail(int code, const std::string& msg) {
    err_ = msg;
    ctx_->set_error(msg);
    return code;
}

const uint4* GpuVerifier::source() const {
    if (round_ == 0 && prover_ref_.g) return prover_ref_.g;
    return (round_ == 0 && cache_ref_.g) ? cache_ref_.g : g_[cur_].as<uint4>();
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
    if (own_stream_) DM_CU(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking), "cudaStreamCreate");
    const uint64_t bytes = (uint64_t)N * kRank * n * 16;
    uint32_t Ln = 0;
    while ((1u << Ln) < n) ++Ln;
    cur_ = 0;
    // the provers' entry for this seed and ring holds g_0 in the verifier's layout
    // ([N][8][n]) when the family is square, as every proof's is
    if (N == n && ctx_->prover_cache() && ctx_->prover_cache()->lookup(st_.g_0_seed, Ln, &prover_ref_)) {
        DM_CU(cudaStreamWaitEvent(s_, prover_ref_.ready, 0), "cudaStreamWaitEvent");
        if (g_[1].alloc(ctx_, bytes / 2 + 16, s_) == kOk && g_[0].alloc(ctx_, bytes / 4 + 16, s_) == kOk) return kOk;
        g_[0].reset();
        g_[1].reset();
        cudaStreamSynchronize(s_);
        ctx_->prover_cache()->release(prover_ref_);
        prover_ref_ = ProverGenCache::Ref{};
    }
    if (cache_ && cache_->acquire(st_.g_0_seed, N, Ln, s_, &cache_ref_) == kOk) {
        // the first fold writes at most half of g_0, every later one at most a quarter
        // (both dimensions of a non-trivial family halve while above one)
        DM_CU(cudaStreamWaitEvent(s_, cache_ref_.ready, 0), "cudaStreamWaitEvent");
        if (g_[1].alloc(ctx_, bytes / 2 + 16, s_) == kOk && g_[0].alloc(ctx_, bytes / 4 + 16, s_) == kOk) return kOk;
        // no room beside the cached family: drop it (once its expansion, which may
        // be this stream's, has finished) and hold a private copy, as without a cache
        g_[0].reset();
        g_[1].reset();
        cudaStreamSynchronize(s_);
        cache_->release(cache_ref_);
        cache_->trim(footprint(N, n));
    }
    cache_ref_ = GenCache::Ref{};
    if (g_[0].alloc(ctx_, bytes, s_) != kOk || g_[1].alloc(ctx_, bytes / 2 + 16, s_) != kOk)
        return fail(kENoMem, "HBM budget exhausted allocating verifier generators");
    // one keyed BLAKE3 compression and 16 written bytes per coefficient
    DM_LAUNCH("gen_generators", bytes, bytes / 16, launch_gen_generators(st_.g_0_seed, N, Ln, g_[0].as<uint4>(), s_));
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
        if (!module_fold(current_, false, rec.l_vec, x_inv, rec.r_vec, x, vfc))
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
        if (!module_fold(vfc, true, rec.l_poly, y_inv, rec.r_poly, y, next))
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
    // reads the whole family, writes the folded one: two (or one) coefficients in per coefficient out
    const uint64_t in_elems = (uint64_t)N_ * kRank * n_;
    const uint64_t out_elems = in_elems >> ((vec ? 1 : 0) + (poly ? 1 : 0));
    DM_LAUNCH("fold_gen", (in_elems + out_elems) * 16, out_elems,
              launch_fold_gen_round(source(), g_[cur_ ^ 1].as<uint4>(), N_, L, x_inv, y_inv, vec, poly, s_));
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
    cudaError_t e = cudaSuccess;
    if (!own_stream_) {
        // on a borrowed (service worker's) stream, sleep rather than spin until the
        // folds are done: the service runs a verifier per core, and a spinning wait
        // takes a core from another proof's replay
        e = cudaEventCreateWithFlags(&done_, cudaEventBlockingSync | cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(done_, s_);
        if (e == cudaSuccess) e = cudaEventSynchronize(done_);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(g.data(), source(), g.size() * 16, cudaMemcpyDeviceToHost, s_);
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

int verify_proof(Context* ctx, const uint8_t* proof, size_t len, const uint8_t epoch[32], cudaStream_t stream,
                 GenCache* cache, std::string* err, bool* cache_hit) {
    if (cache_hit) *cache_hit = false;
    auto bad = [&](int code, const char* msg) {
        ctx->set_error(msg);
        if (err) *err = msg;
        return code;
    };
    const uint8_t *p = proof, *end = proof + len;
    Statement st;
    if (!decode_statement(p, end, st)) return bad(kEDeserialize, "statement deserialization failed");
    GpuVerifier v(ctx, stream, cache);
    auto done = [&](int rc) {
        if (rc != kOk && err && !v.error().empty()) *err = v.error();
        if (cache_hit) *cache_hit = v.cache_hit();
        return rc;
    };
    int rc = v.init(proof, (size_t)(p - proof), epoch);
    if (rc != kOk) return done(rc);
    if (end - p < 8) return done(bad(kEDeserialize, "proof truncated"));
    uint64_t count = 0;
    for (int i = 7; i >= 0; --i) count = (count << 8) | p[i];
    p += 8;
    for (uint64_t r = 0; r < count; ++r) {
        RoundRecord rec;
        if (!decode_record(p, end, rec)) return done(bad(kEDeserialize, "round record deserialization failed"));
        rc = v.update_commitment(rec);
        if (rc != kOk) return done(rc);
    }
    if (end - p < 16) return done(bad(kEDeserialize, "proof truncated"));
    return done(v.verify_final_opening(fq_from_bytes(p)));
}

bool proof_shape(const uint8_t* proof, size_t len, uint64_t* N, uint32_t* n, uint64_t* footprint) {
    const uint8_t* p = proof;
    Statement st;
    if (!decode_statement(p, proof + len, st)) return false;
    uint32_t d;
    uint64_t dim;
    if (!square_layout_for_byte_len(st.original_len_bytes, &d, &dim)) return false;
    const uint32_t ring = st.com_0.n;
    if (ring == 0 || (ring & (ring - 1)) || ring > (1u << kLogMaxProverRing) || dim > (1u << kLogMaxProverRing))
        return false;
    *N = dim;
    *n = ring;
    *footprint = GpuVerifier::footprint(dim, ring);
    return true;
}

}  // namespace dm
