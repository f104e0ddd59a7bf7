// Continuous-batching proof engine.
//
// Requests (commit + prove of one file) are admitted against the context's HBM
// budget and keep their witness, generators and fold state resident on the
// device until their last round.  A scheduler thread gathers the next GPU stage
// of every ready request into one Plan ("wave"): same-degree rounds of different
// requests land in the same kernel launches.  When a wave's kernels have finished
// (a poller thread queries each wave's event; the finishes write the results
// straight into mapped pinned host memory) its requests go to a pool of host
// workers, which run
// the Fiat-Shamir part of the stage (transcript hashing, recompute verdicts,
// records) and return the requests to the ready set.  Several waves are in
// flight at once, so the GPU works on some requests while the host hashes for
// others.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "proof.h"

namespace dm {

struct EngineStats {
    uint64_t submitted = 0, completed = 0, failed = 0, waves = 0, launches = 0;
    uint64_t bytes_done = 0;
    uint64_t peak_reserved = 0;
    double host_stage_ms = 0;  // summed time of the host part of stages (all workers)
    double gpu_idle_ms = 0;    // wall time with no wave in flight while requests were admitted
    double admit_ms = 0;       // scheduler thread: admitting requests (setup, Init stage launches)
    double launch_ms = 0;      // scheduler thread: planning and launching stage waves
    uint64_t cancelled = 0, timed_out = 0;
};

// Engine settings; a negative value (or 0 for the first two) keeps the default,
// which the DM_ENGINE_* environment variable of the same setting overrides.
struct EngineOptions {
    int host_threads = 0;     // Fiat-Shamir workers; 0: one fewer than the host's cores
    int max_waves = 0;        // stage waves in flight, each on its own stream; 0: 16
    int priority_depth = -1;  // requests this deep run on high-priority streams; 0: no split; default 11
    int polling = -1;         // 1: a poller thread queries each wave's event (default); 0: a host callback per wave
    int spin_us = -1;         // awake wait before blocking, microseconds; 0: block at once; default 200
    int admission_batch = -1; // admissions per scheduling pass while a request is ready; 0: all; default 1
};

class Engine {
   public:
    Engine(Context* ctx, int host_threads, int max_waves);
    Engine(Context* ctx, const EngineOptions& opt);
    ~Engine();
    // Empty when the streams and events were created; otherwise the failed call
    // (the engine then runs nothing and must be destroyed).
    const std::string& init_error() const { return init_error_; }

    // Where a submitted file lives.  kHostCopy: host memory the engine copies
    // into its own pinned staging before submit returns, so the caller may reuse
    // it at once.  kDevice: device memory.  kHostBorrowed: host memory that the
    // request's host-to-device copy reads directly, with no staging copy (page-
    // locked memory makes that copy asynchronous).  The last two must stay valid
    // and unchanged until the request finishes.
    enum class FileSource { kHostCopy, kDevice, kHostBorrowed };
    // Returns a ticket.  Never blocks on the GPU.
    int submit(const uint8_t* file, uint64_t len, const uint8_t seed[32], const uint8_t epoch[32], uint64_t* ticket,
               FileSource source = FileSource::kHostCopy);
    // 1 = finished (proof moved out), 0 = still running, < 0 = the request failed.
    int poll(uint64_t ticket, std::vector<uint8_t>* proof, double* latency_ms, std::string* err);
    // Blocks until the ticket finishes; same results as poll.
    int wait(uint64_t ticket, std::vector<uint8_t>* proof, double* latency_ms, std::string* err);
    // Blocks until one of the n tickets has finished (proof ready or failed) and
    // sets *which to its index; poll then returns its result at once.  Tickets
    // the engine does not know are skipped (kEInval when it knows none of them).
    int wait_any(const uint64_t* tickets, size_t n, size_t* which);
    // wait with a limit: kETimeout when the request has not finished within
    // timeout_ms (it keeps running; the ticket stays valid).
    int wait_for(uint64_t ticket, double timeout_ms, std::vector<uint8_t>* proof, double* latency_ms,
                 std::string* err);
    // Ends a request early: a queued one at once, an admitted one at its next
    // stage boundary (a stage already on the GPU completes first, so no kernel is
    // interrupted and no buffer freed under it).  It then finishes with
    // kECanceled and releases its memory.  kEState if it had already finished.
    int cancel(uint64_t ticket);
    // Requests submitted from now on fail with kETimeout when they are still
    // unfinished timeout_ms after submission (checked at admission and at stage
    // boundaries, as cancel is).  0: no limit.
    void set_request_timeout(double timeout_ms);
    // Admissions per scheduling pass while an admitted request is ready (0: all
    // that fit); see admit_batch_.
    void set_admission_batch(int n);
    // Watchdog reading: unfinished requests and the milliseconds since any
    // stage finished (0 when nothing is unfinished).  The GPU kernels wait on
    // nothing, so a growing age with requests unfinished means the host side
    // (or the device) stopped making progress.
    void health(uint64_t* unfinished, double* ms_since_progress);
    void drain();  // blocks until every submitted request has finished
    EngineStats stats();

   private:
    struct Request;
    struct Wave;
    // index of an idle wave stream, a high-priority one first when `high`
    // (called with mu_ held)
    int take_wave_stream(bool high = false);
    // Launches the next stage of `reqs` as one wave (called with mu_ held; drops
    // it while planning and launching).
    void launch_wave(std::vector<Request*> reqs, bool high, std::unique_lock<std::mutex>& lk);
    static void CUDART_CB on_wave_done(void* arg);
    // A wave's stage has finished on the device (or failed with `status`): its
    // requests go to the host workers.
    void complete_wave(Wave* w, cudaError_t status);
    void poller();
    // One sweep over the waves in flight (mu_ held on entry and exit, dropped
    // while querying); true when any completed.
    bool poll_once(std::unique_lock<std::mutex>& lk);
    void scheduler();
    void worker();
    void finish_request(Request* r);
    // The ticket's request has finished, or another thread has already collected
    // it (mu_ held): waits look the ticket up again on every wake-up instead of
    // holding a pointer to a request that a collector may free.
    bool finished_or_gone(uint64_t ticket) const;
    // kECanceled / kETimeout when r must end at this boundary, else 0 (mu_ held).
    int abort_code(const Request* r, std::chrono::steady_clock::time_point now) const;

    Context* ctx_;
    int max_waves_;
    cudaStream_t stream_ = nullptr;            // admission: allocations, file copies, frees
    std::vector<cudaStream_t> wave_streams_;  // one per in-flight wave, so waves overlap on the GPU
    std::vector<bool> wave_stream_busy_;
    // The first high_streams_ wave streams run at the device's greatest stream
    // priority; stages of requests of depth >= priority_depth_ (the longest
    // chains of stages, 2d + 1 each) launch there in their own wave, so the end of
    // a stream of requests is not left to the deepest ones alone.  Default 11,
    // DM_ENGINE_PRIORITY_DEPTH overrides it; 0: one wave of everything.
    int high_streams_ = 0;
    uint32_t priority_depth_ = 0;
    cudaEvent_t admit_ev_ = nullptr;  // the whole admission stream, for a request without an event of its own
    // Admission events of finished requests, for reuse (mu_ held).
    std::vector<cudaEvent_t> free_admit_events_;
    cudaEvent_t take_admit_event();
    std::mutex mu_;
    std::condition_variable sched_cv_, done_cv_, work_cv_;
    std::deque<Request*> queued_;  // submitted, not admitted
    std::vector<Request*> ready_;  // next stage can be launched
    std::deque<Request*> host_q_;  // stage results landed, host part pending
    std::map<uint64_t, std::unique_ptr<Request>> all_;
    uint64_t next_ticket_ = 1;
    int inflight_waves_ = 0;
    int active_ = 0;  // admitted, not finished
    std::chrono::steady_clock::time_point idle_since_{}, active_since_{};
    bool admit_blocked_ = false;  // the queue head waits for memory; cleared when a request finishes
    bool stop_ = false;
    double request_timeout_ms_ = 0;
    std::chrono::steady_clock::time_point last_progress_{};
    std::string init_error_;
    EngineStats stats_;
    std::thread sched_thread_;
    std::vector<std::thread> workers_;
    // Completion by polling (default): each wave records its stream's event, and
    // a poller thread queries the events of the waves in flight, yielding between
    // sweeps (it keeps one host core busy while waves run).  DM_ENGINE_POLL=0: a
    // host callback per wave instead.
    bool poll_ = true;
    // Short awake waits before blocking: the scheduler (while waves are in
    // flight) for a ready request, and up to kSpinningWorkers workers for a
    // landed stage, each for at most spin_us_ microseconds, watching a counter
    // that every hand-over bumps.  200 us: a lone d = 6 request 0.725 ms against
    // 0.84 blocking at once (the plain path: 0.67 ms); the saturated serving
    // stream and batched set within noise.  DM_ENGINE_SPIN_US; 0: block at once.
    int spin_us_ = 200;
    // Admissions per scheduling pass while some admitted request is ready: after
    // that many the pass launches, so the GPU starts on the first requests while
    // the rest are set up, and requests that arrive together do not all run their
    // stages in lockstep (their last, latency-bound rounds then overlap other
    // requests' work).  One measured best: serving stream 56.4 against 59.2 ms,
    // batched set 12.6 against 13.9 ms (2 and 4 in between).
    // DM_ENGINE_ADMIT_BATCH; 0: admit every queued request that fits first.
    int admit_batch_ = 1;
    static constexpr int kSpinningWorkers = 2;
    int spinning_workers_ = 0;
    std::atomic<uint64_t> sched_signal_{0}, work_signal_{0};
    void spin_for_signal(const std::atomic<uint64_t>& sig, uint64_t seen) const;
    std::vector<cudaEvent_t> wave_events_;
    std::vector<Wave*> polled_;
    std::condition_variable poll_cv_;
    std::thread poll_thread_;
};

}  // namespace dm
