// Streaming verifier service.
//
// Proofs (bincode((Statement, Vec<RoundRecord>, Fp)), the container the one-shot
// verifier reads) are submitted from any thread and verified by a pool of
// workers, each with its own CUDA stream, so one proof's host replay (transcript
// hashing, challenge inversions, commitment updates) overlaps other proofs'
// generator expansion and folds on the device.  Jobs start in arrival order
// while the context's HBM budget holds their footprint.  Initial generator
// families are shared through a GenCache: proofs of the same shape under the
// same system seed expand g_0 once.  Each verdict is exactly what the one-shot
// verifier returns for the same bytes.
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"

namespace dm {

struct VerifyStats {
    uint64_t submitted = 0, completed = 0, accepted = 0, rejected = 0, retried = 0;
    uint64_t peak_reserved = 0;
    uint64_t cache_hits = 0, cache_misses = 0, cache_bytes = 0;
};

class VerifyService {
   public:
    // workers <= 0: one per host core, at most 16.  cache_bytes = 0 disables
    // the generator cache.
    VerifyService(Context* ctx, int workers, uint64_t cache_bytes);
    ~VerifyService();
    // Empty when the streams were created; otherwise the failed call (the
    // service then runs nothing and must be destroyed).
    const std::string& init_error() const { return init_error_; }

    // Copies the proof; returns a ticket.  Never blocks on the GPU.
    int submit(const uint8_t* proof, size_t len, const uint8_t epoch[32], uint64_t* ticket);
    // 1 = finished (*verdict = kOk for an accepted proof, else the one-shot
    // verifier's error code), 0 = still running, kEInval = unknown ticket.  A
    // finished ticket is forgotten once reported.
    int poll(uint64_t ticket, int* verdict, double* latency_ms, std::string* err);
    int wait(uint64_t ticket, int* verdict, double* latency_ms, std::string* err);
    void drain();
    VerifyStats stats();

   private:
    struct Job {
        std::vector<uint8_t> proof;
        uint8_t epoch[32];
        uint64_t footprint = 0;
        int verdict = 0;
        bool done = false;
        bool alone = false;  // retried after kENoMem: runs with no other job of the service
        double latency_ms = 0;
        std::string err;
        std::chrono::steady_clock::time_point t0;
    };
    void worker(int w);
    int take(uint64_t ticket, bool block, int* verdict, double* latency_ms, std::string* err);

    Context* ctx_;
    std::unique_ptr<GenCache> cache_;
    std::vector<cudaStream_t> streams_;
    std::vector<std::thread> threads_;
    std::mutex mu_;
    std::condition_variable work_cv_, done_cv_;
    std::deque<uint64_t> queue_;
    std::map<uint64_t, std::shared_ptr<Job>> jobs_;
    uint64_t next_ticket_ = 1;
    uint64_t admitted_bytes_ = 0;  // footprints of running jobs
    int running_ = 0;
    bool stop_ = false;
    VerifyStats st_;
    std::string init_error_;
};

}  // namespace dm
