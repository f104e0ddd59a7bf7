// One proof as a sequence of GPU stages separated by host Fiat-Shamir steps.
//
//   Init : file id, witness unpack, generator expansion, transforms of m and g,
//          commitment com_0 and round 0's vector cross terms
//   Vec  : fold m, g with x; transforms; recompute check + even/odd cross terms
//   Poly : fold m, g with y; transforms; recompute check + next vector cross terms
//
// Each stage emits jobs into a Plan; a Plan launches every job kind once (per
// ring size), so a single request and a batch of same-stage requests run through
// the same kernels.  After a stage's device->host copies land, complete_stage()
// runs the host part (checks, transcript, records) and arms the next stage.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "dm_jobs.cuh"
#include "engine.h"

namespace dm {

struct Copy {
    void* dst;
    const void* src;
    size_t bytes;
};

class Plan {
   public:
    std::vector<HashJob> hash;
    std::vector<UnpackJob> unpack;
    std::vector<GenJob> gen;
    std::vector<FoldJob> fold;
    std::vector<NttJob> ntt[kLogMaxProverRing + 1];
    // multiply-accumulates of every ring size (each job carries its own)
    std::vector<MacJobX> mac, split, triple;
    std::vector<FinishJobX> finish[kLogMaxProverRing + 1];
    std::vector<Copy> d2h;
    // Cached generator families: events the stream waits on before the first
    // launch (entries other stages filled) and events recorded after the last
    // (entries this plan fills), with the fills' references for poisoning when
    // the plan fails to launch.
    std::vector<cudaEvent_t> wait_events, record_events;
    std::vector<ProverGenCache::Ref> fills;
    // Launches every non-empty job kind in dependency order on `st`, then the copies.
    // Returns the number of kernel launches, or a negative status.
    int launch(Context* ctx, cudaStream_t st, std::string* err);
    void clear();

   private:
    int launch_all(Context* ctx, cudaStream_t st, std::string* err);

   public:
    bool empty() const;
};

enum class Stage { Init, Vec, Poly, Done, Failed };

class ProofState {
   public:
    explicit ProofState(Context* ctx) : ctx_(ctx) {}
    ~ProofState();
    ProofState(const ProofState&) = delete;
    ProofState& operator=(const ProofState&) = delete;

    // Validates the input, allocates device state on `stream` and stages the file.
    int setup(const uint8_t* file, uint64_t len, bool on_device, const uint8_t seed[32], const uint8_t epoch[32],
              uint64_t max_preprocess_bytes, cudaStream_t stream);
    void plan_stage(Plan& plan);  // jobs + copies of the current stage
    int complete_stage();         // host part once the stage's copies landed

    Stage stage() const { return stage_; }
    uint32_t stage_L() const;  // ring size exponent of the stage's transforms (batching key)
    uint32_t depth() const { return d_; }
    uint64_t round() const { return round_; }
    uint32_t vector_len() const { return N_; }
    uint32_t ring_len() const { return n_; }
    uint64_t file_len() const { return len_; }
    const Statement& statement() const { return st_; }
    const Module& current_commitment() const { return current_; }
    std::vector<RoundRecord>& records() { return records_; }
    bool opening(fq* out) const;
    const std::string& error() const { return err_; }
    int error_code() const { return err_code_; }
    static uint64_t footprint(uint64_t len);
    void encode_proof(std::vector<uint8_t>* out) const;  // bincode((Statement, Vec<RoundRecord>, Fp))
    // Frees the device state (stream-ordered on the setup stream) and the pinned buffer.
    void release();

   private:
    int fail(int code, const std::string& msg);
    bool plan_commit(Plan& P, uint32_t L, uint32_t cols, uint32_t c, const uint4* m_src, const uint4* g_src,
                     uint32_t* part, uint32_t* ghat = nullptr, bool g_transformed = false);
    const uint4* g_round0() const;  // the family round 0's vector fold reads
    Context* ctx_;
    cudaStream_t alloc_stream_ = nullptr;
    Stage stage_ = Stage::Init;
    uint32_t d_ = 0, S_ = 0, N_ = 0, n_ = 0;
    uint64_t round_ = 0, len_ = 0;
    Statement st_{};
    Transcript tr_;
    Module current_, pend_l_, pend_r_, ct_, lp_, rp_;
    fq x_{}, xi_{}, y_{}, yi_{};
    fq opening_{};
    bool have_opening_ = false;
    std::vector<RoundRecord> records_;
    std::string err_;
    int err_code_ = 0;
    const uint8_t* d_file_ = nullptr;
    DevMem file_, hash_scratch_, m_a_, m_b_, g_a_, g_b_, mhat_, ghat_, partials_, comm_, misc_;
    uint8_t* pinned_ = nullptr;
    size_t pinned_bytes_ = 0;
    uint32_t parts_ = 1;
    // Witness columns that can be nonzero: the file fills the coefficients in
    // order and the square layout pads with zeros, and folds keep zero columns
    // zero, so a stage's columns from min(mcols_, columns) on are zero.  Their
    // transforms and the generator columns that only meet them are skipped.
    uint32_t mcols_ = 0;
    uint8_t seed_[32];
    uint8_t epoch_copy_[32];
    // g_0 and its transform from the context's cache, held from the Init stage
    // until round 0's vector stage (the last reader) has completed
    ProverGenCache::Ref cached_{};
};

// Round-by-round prover (src/protocol/prover.rs:56-313): one ProofState driven
// stage by stage on its own stream.
class GpuProver {
   public:
    explicit GpuProver(Context* ctx) : ctx_(ctx), ps_(ctx) {}
    ~GpuProver();
    // file is a host pointer, or a device pointer when on_device.
    int init(const uint8_t* file, uint64_t len, bool on_device, const uint8_t seed_generators[32],
             const uint8_t epoch_seed[32], uint64_t max_preprocess_bytes);
    // times_ms (optional): wall time of the vector stage, the polynomial stage
    // and the whole round, as RoundOutput's vector_fold_time / poly_fold_time /
    // total_round_time (src/protocol/prover.rs:26-31)
    int fold_round(uint64_t round_idx, RoundRecord* out, double times_ms[3] = nullptr);
    bool final_opening(fq* out) const { return ps_.opening(out); }
    const Statement& statement() const { return ps_.statement(); }
    uint32_t rounds_total() const { return ps_.depth(); }
    uint64_t current_round() const { return ps_.round(); }
    const Module& current_commitment() const { return ps_.current_commitment(); }
    uint32_t vector_len() const { return ps_.vector_len(); }
    uint32_t ring_len() const { return ps_.ring_len(); }
    static uint64_t footprint(uint64_t len) { return ProofState::footprint(len); }
    double device_ms() const;  // first to last operation of the proof (CUDA events)
    void encode_proof(std::vector<uint8_t>* out) const { ps_.encode_proof(out); }

   private:
    int run_stage();
    int fail(int code, const std::string& msg);
    Context* ctx_;
    ProofState ps_;
    cudaStream_t s_ = nullptr;
    cudaEvent_t ev_start_ = nullptr, ev_end_ = nullptr;
    bool failed_ = false;
};

}  // namespace dm
