// Device runtime: context (device, stream, tables, HBM budget, kernel timing),
// and the GPU prover / verifier that keep a proof's witness, generators and
// fold state resident in HBM across rounds.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "dm_jobs.cuh"
#include "dm_kernels.cuh"
#include "dm_ref.cuh"
#include "protocol.h"

namespace dm {

enum Status : int {
    kOk = 0,
    kEInval = -1,
    kENoMem = -2,       // HBM budget exhausted or allocation failed
    kECuda = -3,
    kETimeout = -4,
    kEVerify = -5,      // verification rejected
    kEInvariant = -6,   // prover recompute check failed
    kEState = -7,       // call out of order (round mismatch, rounds finished)
    kESize = -8,        // output buffer too small
    kEDeserialize = -9,
    kEUnsupported = -10,
    kECanceled = -11,   // the caller cancelled the request
};

struct KernelStat {
    uint64_t launches = 0;  // kernel launches (a recorded call may launch more than one)
    double total_ms = 0.0;
    double bytes = 0.0;  // algorithmic bytes moved
    double ops = 0.0;    // algorithmic integer operations
};

class ProverGenCache;

class Context {
   public:
    static int create(int device, uint64_t hbm_budget, Context** out, std::string* err);
    ~Context();

    int device() const { return device_; }
    cudaStream_t stream() const { return stream_; }
    const DeviceTables& tables() const { return tables_; }
    const RefDeviceTables& ref_tables() const { return ref_tables_; }

    // HBM budget accounting (bytes reserved by live provers/verifiers/requests).
    bool reserve(uint64_t bytes);
    void release(uint64_t bytes);
    uint64_t budget() const { return budget_; }
    uint64_t reserved() const { return reserved_.load(); }

    void set_error(const std::string& e);
    std::string last_error();

    // Optional per-kernel event timing on the launching stream.
    void set_profiling(bool on) { profiling_ = on; }
    bool profiling() const { return profiling_; }
    void record(const char* name, cudaEvent_t a, cudaEvent_t b, double bytes, double ops, int kernels = 1,
                cudaStream_t st = nullptr);
    void flush_timings();  // resolves recorded event pairs (synchronises the stream)
    // Launch trace: from start_trace() on, every timed launch group is also kept
    // with its stream and its start and end relative to a reference event, and
    // read_trace() returns them as CSV lines "kind,stream,start_ms,end_ms,bytes,
    // kernels" (the start is when the stream reached the group, which includes
    // any wait for the stream's previous work).  Turns profiling on.
    int start_trace();
    int read_trace(std::string* csv, bool stop);
    // Host rows of the same trace (host clock from the same reference point,
    // taken right after the reference event completed): `kind,lane,start_ms,
    // end_ms,count,launches` with lane and count chosen by the caller (the engine
    // logs each wave's planning and launching with its stream and request count,
    // and each Fiat-Shamir step).
    bool tracing() const { return tracing_.load(std::memory_order_relaxed); }
    void trace_host(const char* kind, int lane, std::chrono::steady_clock::time_point t0,
                    std::chrono::steady_clock::time_point t1, double count, int launches);
    bool stat(const char* name, KernelStat* out);
    void reset_stats();
    cudaEvent_t take_event();

    std::mutex& mutex() { return mu_; }

    // Launch-shape knobs (TuneKnob) per ring size 2^L; thread-safe.
    int tuning(int knob, uint32_t L) const { return tune_[knob][L].load(std::memory_order_relaxed); }
    int set_tuning(int knob, uint32_t L, int value);
    int sm_count() const { return sm_count_; }
    // Column splits of a MAC over `count` columns whose rows take threads_per_row
    // threads (128 per block): enough parts to fill sm_count x the knob's blocks
    // per SM, at most kMaxMacParts, at least eight columns per part (small rings:
    // fewer partial rows for the finish; measured +2 % on the serving stream),
    // at least one part.
    uint32_t mac_parts(int knob, uint32_t L, uint32_t threads_per_row, uint32_t count) const;
    // rows: the thread rows one part launches (kRows; kRows / kc for the split MAC)
    uint32_t mac_parts_for(int blocks_per_sm, uint32_t threads_per_row, uint32_t count,
                           uint32_t rows = kRank * kPrimes) const;

    // Provers' generator cache (off until a capacity is set; 0 turns it off and
    // frees it once no prover holds an entry).  Set it before proving starts.
    int set_prover_cache(uint64_t cap_bytes);
    ProverGenCache* prover_cache() const { return prover_cache_.get(); }

    // RuntimeConfig.max_preprocess_bytes of the one-shot and engine entry points
    // (src/utils/config.rs:21, 69-87; checked as src/utils/io.rs:42-49 does).
    // Default: the reference's 512 MiB.
    static constexpr uint64_t kDefaultMaxPreprocess = 512ull * 1024 * 1024;
    uint64_t max_preprocess() const { return max_preprocess_.load(std::memory_order_relaxed); }
    void set_max_preprocess(uint64_t bytes) {
        max_preprocess_.store(bytes ? bytes : kDefaultMaxPreprocess, std::memory_order_relaxed);
    }

   private:
    std::unique_ptr<ProverGenCache> prover_cache_;
    std::atomic<uint64_t> max_preprocess_{kDefaultMaxPreprocess};
    int device_ = 0;
    int sm_count_ = 152;
    std::atomic<int> tune_[kTuneKnobs][kLogMaxProverRing + 1];
    cudaStream_t stream_ = nullptr;
    DeviceTables tables_{};
    RefDeviceTables ref_tables_{};
    uint64_t budget_ = 0;
    std::atomic<uint64_t> reserved_{0};
    std::mutex mu_, err_mu_, prof_mu_;
    std::string last_error_;
    bool profiling_ = false;
    struct Pending {
        std::string name;
        cudaEvent_t a, b;
        double bytes, ops;
        int kernels;
        cudaStream_t st;
    };
    std::vector<Pending> pending_;
    std::atomic<bool> tracing_{false};
    std::chrono::steady_clock::time_point trace_host_ref_{};
    cudaEvent_t trace_ref_ = nullptr;
    std::string trace_csv_;
    std::vector<cudaStream_t> trace_streams_;
    std::vector<cudaEvent_t> event_pool_;
    std::map<std::string, KernelStat> stats_;
    void* flush_buf_ = nullptr;

   public:
    // Writes a buffer larger than L2 (256 MiB) on the context stream and waits.
    int flush_l2();
    // Pinned host staging buffers, recycled across provers.
    void* get_pinned(size_t bytes);
    void put_pinned(void* p, size_t bytes);

   private:
    std::mutex pin_mu_;
    std::vector<std::pair<size_t, void*>> pinned_free_;  // idle buffers: (allocated size, address)
    std::map<void*, size_t> pinned_cap_;                   // every buffer allocated: its size

};

// Scoped device allocation charged against the context budget.
class DevMem {
   public:
    DevMem() = default;
    ~DevMem() { reset(); }
    DevMem(const DevMem&) = delete;
    DevMem& operator=(const DevMem&) = delete;
    // Stream-ordered allocation from the device pool on `stream` (the context
    // stream when null); freed on the same stream.
    int alloc(Context* ctx, size_t bytes, cudaStream_t stream = nullptr);
    void reset();
    template <class T>
    T* as() const {
        return static_cast<T*>(ptr_);
    }
    size_t bytes() const { return bytes_; }

   private:
    Context* ctx_ = nullptr;
    void* ptr_ = nullptr;
    size_t bytes_ = 0;
    cudaStream_t stream_ = nullptr;
};

// Initial generator families g_0(seed, N, n) kept in HBM and shared read-only by
// verifiers.  g_0 depends on nothing but the system seed and the witness shape
// (src/commitment/sis.rs:198-245), and deployments use one seed for every file
// (SystemParams::default, src/utils/config.rs:19, 33-44), so a verifier of a stream
// of proofs expands each shape once.  A key is cached the second time it is seen.
// Entries are charged to the context budget, evicted least recently used when
// unreferenced, and capped at `cap_bytes`.
class GenCache {
   public:
    struct Ref {
        const uint4* g = nullptr;
        cudaEvent_t ready = nullptr;  // recorded after the expansion; readers wait on it
        void* entry = nullptr;
    };
    GenCache(Context* ctx, uint64_t cap_bytes) : ctx_(ctx), cap_(cap_bytes) {}
    ~GenCache();
    // The family for (seed, N, 2^log_n); on a miss of a key seen before it is
    // expanded on `s`.  kENoMem on a first sighting, or when it does not fit under
    // the cap or the budget: the caller expands its own.
    int acquire(const uint8_t seed[32], uint64_t N, uint32_t log_n, cudaStream_t s, Ref* out);
    // After every reader of `r` has finished on the device.
    void release(const Ref& r);
    // Evicts unreferenced entries, least recently used first, until `bytes` more
    // fit under the context budget; false when they still do not.
    bool trim(uint64_t bytes);
    struct Stats {
        uint64_t hits = 0, misses = 0, evictions = 0, bytes = 0, entries = 0;
    };
    Stats stats();

   private:
    struct Entry;
    bool evict_for(uint64_t bytes);  // called with mu_ held
    bool evict_one();                // called with mu_ held
    Context* ctx_;
    uint64_t cap_;
    std::mutex mu_;
    std::map<std::vector<uint8_t>, Entry*> map_;
    std::map<std::vector<uint8_t>, int> seen_;
    uint64_t clock_ = 0;
    Stats st_;
};

// Initial generator families of provers with their forward transforms, kept in
// HBM: g_0(seed, S) as coefficients ([S][8][S], 16 B each) and as nine-prime
// residues ([S][8][9][S] words), the two forms the commitment stage reads.  A
// key is cached the second time it is seen, so a stream of per-file seeds never
// pays for a fill while a deployment proving every file under one seed expands
// and transforms each shape once.  The prover that fills an entry writes it in
// its own Init stage (expansion and a transform of every column), records
// `ready` after that stage and publishes the entry; readers that acquire it
// afterwards wait on `ready`.  Entries are charged to the
// context budget and evicted least recently used when unreferenced.
class ProverGenCache {
   public:
    struct Ref {
        uint4* g = nullptr;
        uint32_t* ghat = nullptr;
        cudaEvent_t ready = nullptr;
        void* entry = nullptr;
        bool fill = false;  // the caller writes the entry and records `ready` after
    };
    ProverGenCache(Context* ctx, uint64_t cap_bytes) : ctx_(ctx), cap_(cap_bytes) {}
    ~ProverGenCache();
    static uint64_t entry_bytes(uint32_t L);
    // kOk with a hit or a fill; kENoMem when the key is not cached (first
    // sighting, no room under the cap or the budget, or a fill not yet enqueued by
    // another plan): the caller uses its own buffers.  `plan` identifies the
    // caller's stage plan: requests in the plan that fills an entry share it (their
    // stream runs the fill first) with no event to wait on (ready is null).
    int acquire(const uint8_t g0_seed[32], uint32_t L, const void* plan, Ref* out);
    // After the holder's last reading stage has finished on the device.
    void release(const Ref& r);
    // A published entry for (seed, 2^L), or false; nothing is filled or counted
    // as a sighting.  Verifiers of the context read g_0 from it (its coefficient
    // half is their initial family) after waiting on `ready`.
    bool lookup(const uint8_t g0_seed[32], uint32_t L, Ref* out);
    // A fill whose stage is enqueued with `ready` recorded after it: from now on
    // the entry is handed out.  Until then other provers use their own buffers.
    void publish(const Ref& r);
    // A fill whose stage failed to launch: the entry is dropped when unreferenced
    // and never handed out again.
    void poison(const Ref& r);
    bool trim(uint64_t bytes);  // evicts unreferenced entries until `bytes` more fit the budget
    uint64_t bytes();
    struct Stats {
        uint64_t hits = 0, fills = 0, misses = 0, evictions = 0, bytes = 0, entries = 0;
    };
    Stats stats();

   private:
    struct Entry;
    bool evict_one();  // called with mu_ held
    Context* ctx_;
    uint64_t cap_;
    std::mutex mu_;
    std::map<std::vector<uint8_t>, Entry*> map_;
    std::map<std::vector<uint8_t>, int> seen_;
    uint64_t clock_ = 0;
    Stats st_;
};

// Round-by-round verifier (src/protocol/verifier.rs:11-134): commitments and
// challenges on the host, generator folds enqueued on the device without syncs.
// With a stream the verifier borrows it (else it owns one).  When the context's
// provers' cache holds g_0 (same seed, square shape), or the verifier's own cache
// does, the first fold reads that shared copy and the verifier holds half and a
// quarter of it instead of one and a half.
class GpuVerifier {
   public:
    explicit GpuVerifier(Context* ctx, cudaStream_t stream = nullptr, GenCache* cache = nullptr)
        : ctx_(ctx), s_(stream), own_stream_(stream == nullptr), cache_(cache) {}
    ~GpuVerifier();
    int init(const uint8_t* statement, size_t len, const uint8_t epoch_seed[32]);
    int update_commitment(const RoundRecord& rec);
    int verify_final_opening(const fq& opening);
    uint64_t round() const { return round_; }
    uint32_t vector_len() const { return N_; }
    uint32_t ring_len() const { return current_.n; }
    bool cache_hit() const { return cache_ref_.g != nullptr || prover_ref_.g != nullptr; }
    const std::string& error() const { return err_; }
    static uint64_t footprint(uint64_t N, uint64_t n);

   private:
    int fail(int code, const std::string& msg);
    const uint4* source() const;  // the family the next fold reads
    Context* ctx_;
    cudaStream_t s_ = nullptr;
    bool own_stream_ = true;
    GenCache* cache_ = nullptr;
    GenCache::Ref cache_ref_{};
    ProverGenCache::Ref prover_ref_{};  // g_0 from the context's provers' cache
    std::string err_;
    Statement st_{};
    Transcript tr_;
    Module current_;
    uint32_t N_ = 0, n_ = 0;  // generator family dimensions
    uint64_t round_ = 0, rounds_ = 0;
    DevMem g_[2];
    int cur_ = 0;
    cudaEvent_t done_ = nullptr;
};

// One-shot helpers used by the C ABI.
int prove_all(Context* ctx, const uint8_t* file, uint64_t len, bool on_device, const uint8_t seed[32],
              const uint8_t epoch[32], std::vector<uint8_t>* proof, double* device_ms = nullptr);
// Decodes and replays a bincode((Statement, Vec<RoundRecord>, Fp)) proof.  With a
// stream and a cache the verification runs on that stream and shares g_0; with
// `err` the failure text is returned there as well as set on the context.
int verify_proof(Context* ctx, const uint8_t* proof, size_t len, const uint8_t epoch[32],
                 cudaStream_t stream = nullptr, GenCache* cache = nullptr, std::string* err = nullptr,
                 bool* cache_hit = nullptr);
// The statement's generator-family shape and the verifier's device footprint
// (false when the statement does not decode or its shape is unsupported).
bool proof_shape(const uint8_t* proof, size_t len, uint64_t* N, uint32_t* n, uint64_t* footprint);

}  // namespace dm
