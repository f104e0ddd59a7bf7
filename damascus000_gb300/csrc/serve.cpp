#include "serve.h"

#include "dm_nvtx.h"

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <limits>

namespace dm {

using Clock = std::chrono::steady_clock;

struct Engine::Request {
    uint64_t ticket = 0;
    uint8_t* pinned_file = nullptr;  // staged copy of the file (pinned host memory)
    size_t pinned_bytes = 0;
    const uint8_t* caller_file = nullptr;  // the caller's device or host buffer instead (no staging)
    bool on_device = false;
    uint64_t len = 0;
    uint8_t seed[32], epoch[32];
    std::unique_ptr<ProofState> ps;
    enum State { Queued, Active, Done, Failed } state = Queued;
    std::vector<uint8_t> proof;
    std::string err;
    int err_code = 0;
    uint64_t footprint = 0;
    Clock::time_point t_submit, t_done;
    bool cancel = false;          // the caller cancelled it
    bool has_deadline = false;    // the engine's request timeout applies
    Clock::time_point deadline{};
    // current stage, for the launch trace: ready, its wave launched, landed
    Clock::time_point t_ready{}, t_launch{}, t_landed{};
    // Recorded on the admission stream after the request's setup (allocations,
    // file upload): its first wave waits on it, and no other wave does.
    cudaEvent_t admitted = nullptr;
    bool first_wave = true;
};

struct Engine::Wave {
    Engine* eng;
    std::vector<Request*> reqs;
    int stream_idx;
};

namespace {
EngineOptions options_of(int host_threads, int max_waves) {
    EngineOptions o;
    o.host_threads = host_threads;
    o.max_waves = max_waves;
    return o;
}
// An explicit setting, else the environment variable, else the default.
int setting(int given, const char* env, int dflt) {
    if (given >= 0) return given;
    if (const char* v = std::getenv(env)) return std::atoi(v);
    return dflt;
}
}  // namespace

Engine::Engine(Context* ctx, int host_threads, int max_waves) : Engine(ctx, options_of(host_threads, max_waves)) {}

Engine::Engine(Context* ctx, const EngineOptions& opt)
    : ctx_(ctx), max_waves_(opt.max_waves > 0 ? opt.max_waves : 16) {
    const int host_threads = opt.host_threads;
    auto check = [this](cudaError_t e, const char* what) {
        if (e != cudaSuccess && init_error_.empty())
            init_error_ = std::string("engine setup, ") + what + ": " + cudaGetErrorString(e);
        return e == cudaSuccess;
    };
    wave_streams_.assign(max_waves_, nullptr);
    wave_stream_busy_.assign(max_waves_, false);
    // d = 11 (16 MiB files and up): on the serving stream +1.9 % against no split
    // (five interleaved A/B pairs on GB300s; d >= 10 measured alike and noisier)
    priority_depth_ = (uint32_t)setting(opt.priority_depth, "DM_ENGINE_PRIORITY_DEPTH", 11);
    int least = 0, greatest = 0;
    bool ok = check(cudaSetDevice(ctx_->device()), "cudaSetDevice") &&
              check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreateWithFlags") &&
              check(cudaEventCreateWithFlags(&admit_ev_, cudaEventDisableTiming), "cudaEventCreateWithFlags") &&
              check(cudaDeviceGetStreamPriorityRange(&least, &greatest), "cudaDeviceGetStreamPriorityRange");
    high_streams_ = priority_depth_ && max_waves_ >= 4 ? max_waves_ / 4 : 0;
    for (int i = 0; ok && i < max_waves_; ++i)
        ok = check(cudaStreamCreateWithPriority(&wave_streams_[i], cudaStreamNonBlocking,
                                                i < high_streams_ ? greatest : least),
                   "cudaStreamCreateWithPriority");
    // Wave completion by polling the waves' events: measured 34 % faster for a
    // lone small request than a host callback per wave (0.84 against 1.27 ms for a
    // d = 6 proof; 60 against 96 us from launch to the host seeing a stage done),
    // 3 % on the serving stream and 10 % on the batched set.  (Polling from the
    // scheduler thread between its launches instead of a thread of its own
    // measured 1-4 % slower.)  DM_ENGINE_POLL=0 restores the callbacks.
    poll_ = setting(opt.polling, "DM_ENGINE_POLL", 1) != 0;
    spin_us_ = setting(opt.spin_us, "DM_ENGINE_SPIN_US", spin_us_);
    admit_batch_ = setting(opt.admission_batch, "DM_ENGINE_ADMIT_BATCH", admit_batch_);
    wave_events_.assign(max_waves_, nullptr);
    for (int i = 0; ok && poll_ && i < max_waves_; ++i)
        ok = check(cudaEventCreateWithFlags(&wave_events_[i], cudaEventDisableTiming), "cudaEventCreateWithFlags");
    if (!ok) {
        cudaGetLastError();  // the failure is reported by init_error(), not by a later launch
        return;            // no threads: the destructor frees what was created
    }
    if (poll_) poll_thread_ = std::thread([this] { poller(); });
    int n = host_threads > 0 ? host_threads : (int)std::thread::hardware_concurrency() - 1;
    if (n < 1) n = 1;
    sched_thread_ = std::thread([this] { scheduler(); });
    for (int i = 0; i < n; ++i) workers_.emplace_back([this] { worker(); });
}

Engine::~Engine() {
    drain();
    {
        std::lock_guard<std::mutex> g(mu_);
        stop_ = true;
    }
    sched_cv_.notify_all();
    work_cv_.notify_all();
    poll_cv_.notify_all();
    if (sched_thread_.joinable()) sched_thread_.join();
    for (auto& t : workers_) t.join();
    if (poll_thread_.joinable()) poll_thread_.join();
    cudaSetDevice(ctx_->device());
    if (stream_) cudaStreamSynchronize(stream_);
    for (auto& kv : all_) {
        Request* r = kv.second.get();
        if (r->ps) r->ps->release();
        if (r->pinned_file) ctx_->put_pinned(r->pinned_file, r->pinned_bytes);
    }
    all_.clear();
    for (auto& s : wave_streams_) {
        if (!s) continue;
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    if (admit_ev_) cudaEventDestroy(admit_ev_);
    for (cudaEvent_t ev : free_admit_events_) cudaEventDestroy(ev);
    for (cudaEvent_t ev : wave_events_)
        if (ev) cudaEventDestroy(ev);
    if (stream_) {
        cudaStreamSynchronize(stream_);
        cudaStreamDestroy(stream_);
    }
}

int Engine::take_wave_stream(bool high) {
    const int n = (int)wave_stream_busy_.size();
    // high-priority waves try the first high_streams_ streams first; others the rest first
    for (int k = 0; k < n; ++k) {
        const int i = high ? k : (k + high_streams_) % n;
        if (!wave_stream_busy_[i]) {
            wave_stream_busy_[i] = true;
            return i;
        }
    }
    return -1;
}

int Engine::submit(const uint8_t* file, uint64_t len, const uint8_t seed[32], const uint8_t epoch[32],
                   uint64_t* ticket, FileSource source) {
    if ((!file && len) || !seed || !epoch || !ticket) return kEInval;
    std::unique_ptr<Request> r(new Request());
    r->len = len;
    std::memcpy(r->seed, seed, 32);
    std::memcpy(r->epoch, epoch, 32);
    r->footprint = ProofState::footprint(len);
    if (source != FileSource::kHostCopy) {
        r->caller_file = file;
        r->on_device = source == FileSource::kDevice;
    } else {
        r->pinned_bytes = len ? len : 1;
        r->pinned_file = static_cast<uint8_t*>(ctx_->get_pinned(r->pinned_bytes));
        if (!r->pinned_file) return kENoMem;
        if (len) std::memcpy(r->pinned_file, file, len);
    }
    r->ps.reset(new ProofState(ctx_));
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> g(mu_);
        if (request_timeout_ms_ > 0) {
            r->has_deadline = true;
            r->deadline = r->t_submit + std::chrono::microseconds((int64_t)(request_timeout_ms_ * 1000.0));
        }
        r->ticket = next_ticket_++;
        *ticket = r->ticket;
        queued_.push_back(r.get());
        all_[r->ticket] = std::move(r);
        stats_.submitted++;
    }
    sched_signal_.fetch_add(1, std::memory_order_release);
    sched_cv_.notify_one();
    return kOk;
}

void CUDART_CB Engine::on_wave_done(void* arg) {
    Wave* w = static_cast<Wave*>(arg);
    w->eng->complete_wave(w, cudaSuccess);
}

void Engine::complete_wave(Wave* w, cudaError_t status) {
    Engine* e = this;
    if (status != cudaSuccess)
        for (Request* r : w->reqs) {
            r->err_code = kECuda;
            r->err = std::string("stage on the GPU: ") + cudaGetErrorString(status);
        }
    if (e->ctx_->tracing()) {
        const Clock::time_point now = Clock::now();
        e->ctx_->trace_host("wave_done", w->stream_idx, now, now, (double)w->reqs.size(), 0);
        for (Request* r : w->reqs) r->t_landed = now;
    }
    {
        std::lock_guard<std::mutex> g(e->mu_);
        for (Request* r : w->reqs) e->host_q_.push_back(r);
        e->last_progress_ = Clock::now();
        if (--e->inflight_waves_ == 0) e->idle_since_ = Clock::now();
        e->wave_stream_busy_[w->stream_idx] = false;
    }
    e->work_signal_.fetch_add(1, std::memory_order_release);
    e->sched_signal_.fetch_add(1, std::memory_order_release);
    for (size_t i = 0; i < w->reqs.size(); ++i) e->work_cv_.notify_one();
    e->sched_cv_.notify_one();
    delete w;
}

void Engine::spin_for_signal(const std::atomic<uint64_t>& sig, uint64_t seen) const {
    const Clock::time_point until = Clock::now() + std::chrono::microseconds(spin_us_);
    while (sig.load(std::memory_order_acquire) == seen && Clock::now() < until) std::this_thread::yield();
}

bool Engine::poll_once(std::unique_lock<std::mutex>& lk) {
    std::vector<Wave*> snap = polled_, done;
    std::vector<cudaError_t> status;
    lk.unlock();
    for (Wave* w : snap) {
        const cudaError_t q = cudaEventQuery(wave_events_[w->stream_idx]);
        if (q == cudaErrorNotReady) continue;
        done.push_back(w);
        status.push_back(q);
    }
    if (done.empty()) {
        lk.lock();
        return false;
    }
    lk.lock();
    for (Wave* w : done) polled_.erase(std::find(polled_.begin(), polled_.end(), w));
    lk.unlock();
    for (size_t i = 0; i < done.size(); ++i) complete_wave(done[i], status[i]);
    lk.lock();
    return true;
}

void Engine::poller() {
    cudaSetDevice(ctx_->device());
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
        poll_cv_.wait(lk, [&] { return stop_ || !polled_.empty(); });
        if (polled_.empty()) return;  // stop_ with nothing in flight
        if (!poll_once(lk)) {
            lk.unlock();
            std::this_thread::yield();
            lk.lock();
        }
    }
}

void Engine::scheduler() {
    cudaSetDevice(ctx_->device());
    std::unique_lock<std::mutex> lk(mu_);
    auto runnable = [&] {
        return stop_ || (inflight_waves_ < max_waves_ && (!ready_.empty() || (!queued_.empty() && !admit_blocked_)));
    };
    for (;;) {
        if (!runnable() && spin_us_ > 0 && inflight_waves_ > 0) {
            // waves in flight: wait briefly awake for the next ready request
            const uint64_t seen = sched_signal_.load(std::memory_order_acquire);
            lk.unlock();
            spin_for_signal(sched_signal_, seen);
            lk.lock();
        }
        sched_cv_.wait(lk, runnable);
        if (stop_) return;
        // Admission in arrival order while the HBM budget holds the request's footprint.
        int admitted_now = 0;
        while (!queued_.empty()) {
            if (admit_batch_ > 0 && admitted_now >= admit_batch_ && !ready_.empty()) break;  // launch these first
            ++admitted_now;
            Request* r = queued_.front();
            if (const int code = abort_code(r, Clock::now())) {  // cancelled or expired while queued
                queued_.pop_front();
                r->err_code = code;
                r->err = code == kECanceled ? "request cancelled" : "request timed out while queued";
                lk.unlock();
                finish_request(r);
                lk.lock();
                continue;
            }
            // requests come before cached generator families: drop unreferenced
            // ones when a request does not fit
            if (ctx_->reserved() + r->footprint > ctx_->budget() && ctx_->prover_cache()) {
                // The trim's cudaFree waits for the device, and every wave in flight
                // ends in a completion that takes mu_: trim without holding it.
                // Only this thread admits, but a cancel may take r off the queue
                // meanwhile: look at the queue again.
                lk.unlock();
                ctx_->prover_cache()->trim(r->footprint);
                lk.lock();
                if (stop_) return;
                if (queued_.empty() || queued_.front() != r) continue;
            }
            const uint64_t reserved = ctx_->reserved();
            if (reserved + r->footprint > ctx_->budget()) {
                const bool idle = ready_.empty() && host_q_.empty() && inflight_waves_ == 0 && reserved == 0;
                if (!idle) {
                    admit_blocked_ = true;  // wait for running requests to release memory
                    break;
                }
            }
            queued_.pop_front();
            lk.unlock();
            const bool dev = r->on_device;
            const Clock::time_point t_admit = Clock::now();
            const int rc = r->ps->setup(r->caller_file ? r->caller_file : r->pinned_file, r->len, dev, r->seed, r->epoch,
                                        ctx_->max_preprocess(), stream_);
            const double admit_ms = std::chrono::duration<double, std::milli>(Clock::now() - t_admit).count();
            lk.lock();
            stats_.admit_ms += admit_ms;
            if (rc != kOk) {
                r->err = r->ps->error();
                r->err_code = rc;
                lk.unlock();
                finish_request(r);
                lk.lock();
                continue;
            }
            r->admitted = take_admit_event();
            if (r->admitted && cudaEventRecord(r->admitted, stream_) != cudaSuccess) {
                cudaGetLastError();
                free_admit_events_.push_back(r->admitted);
                r->admitted = nullptr;  // its first wave waits for the whole admission stream instead
            }
            r->state = Request::Active;
            if (active_++ == 0) active_since_ = Clock::now();
            r->t_ready = Clock::now();
            ready_.push_back(r);
            if (ctx_->reserved() > stats_.peak_reserved) stats_.peak_reserved = ctx_->reserved();
        }
        if (ready_.empty() || inflight_waves_ >= max_waves_) continue;
        std::vector<Request*> rest;
        rest.swap(ready_);
        {
            // requests cancelled or expired between stages end here: their last
            // stage has completed on the device
            std::vector<Request*> ended;
            const Clock::time_point now = Clock::now();
            size_t k = 0;
            for (Request* r : rest) {
                if (const int code = abort_code(r, now)) {
                    r->err_code = code;
                    r->err = code == kECanceled ? "request cancelled" : "request timed out";
                    ended.push_back(r);
                } else {
                    rest[k++] = r;
                }
            }
            rest.resize(k);
            if (!ended.empty()) {
                lk.unlock();
                for (Request* r : ended) finish_request(r);
                lk.lock();
            }
            if (rest.empty()) continue;
        }
        std::vector<Request*> deep;
        if (priority_depth_ && inflight_waves_ + 1 < max_waves_) {
            // the deepest requests' stages in a wave of their own on a high-priority stream
            size_t k = 0;
            for (Request* r : rest) {
                if (r->ps->depth() >= priority_depth_) deep.push_back(r);
                else rest[k++] = r;
            }
            rest.resize(k);
        }
        if (!deep.empty()) launch_wave(std::move(deep), true, lk);
        if (!rest.empty()) launch_wave(std::move(rest), false, lk);
    }
}

void Engine::launch_wave(std::vector<Request*> reqs, bool high, std::unique_lock<std::mutex>& lk) {
    const int si = take_wave_stream(high);
    if (si < 0) {  // no stream free: the requests wait for the next wave
        ready_.insert(ready_.end(), reqs.begin(), reqs.end());
        return;
    }
    Wave* w = new Wave{this, std::move(reqs), si};
    if (inflight_waves_++ == 0) {
        const Clock::time_point now = Clock::now();
        const Clock::time_point from = idle_since_ > active_since_ ? idle_since_ : active_since_;
        if (now > from) stats_.gpu_idle_ms += std::chrono::duration<double, std::milli>(now - from).count();
    }
    lk.unlock();
    const Clock::time_point t_launch = Clock::now();
    for (Request* r : w->reqs) r->t_launch = t_launch;
    NvtxRange range(high ? "wave (deep)" : "wave");
    cudaStream_t ws = wave_streams_[si];
    // a request's admission (allocations, file upload on stream_) precedes its first
    // wave's kernels; later waves have nothing to wait for there, in particular not
    // the uploads of requests admitted since
    bool wait_all = false;
    for (Request* r : w->reqs) {
        if (!r->first_wave) continue;
        r->first_wave = false;
        if (r->admitted) cudaStreamWaitEvent(ws, r->admitted, 0);
        else wait_all = true;
    }
    if (wait_all) {
        cudaEventRecord(admit_ev_, stream_);
        cudaStreamWaitEvent(ws, admit_ev_, 0);
    }
    Plan plan;
    for (Request* r : w->reqs) r->ps->plan_stage(plan);
    std::string err;
    const int n = plan.launch(ctx_, ws, &err);
    cudaError_t e = cudaSuccess;
    const size_t nreq = w->reqs.size();  // w belongs to the completion path once it is enqueued
    if (n >= 0) {
        if (poll_) {
            e = cudaEventRecord(wave_events_[si], ws);
            if (e == cudaSuccess) {
                std::lock_guard<std::mutex> g(mu_);
                polled_.push_back(w);
            }
            poll_cv_.notify_one();
        } else {
            e = cudaLaunchHostFunc(ws, on_wave_done, w);
        }
    }
    const Clock::time_point t_end = Clock::now();
    const double launch_ms = std::chrono::duration<double, std::milli>(t_end - t_launch).count();
    if (ctx_->tracing()) ctx_->trace_host(high ? "sched_wave_deep" : "sched_wave", si, t_launch, t_end, (double)nreq, n);
    lk.lock();
    stats_.launch_ms += launch_ms;
    if (n < 0 || e != cudaSuccess) {
        if (--inflight_waves_ == 0) idle_since_ = Clock::now();
        wave_stream_busy_[si] = false;
        std::vector<Request*> failed = w->reqs;
        delete w;
        lk.unlock();
        for (Request* r : failed) {
            r->err = n < 0 ? err : std::string("cudaLaunchHostFunc: ") + cudaGetErrorString(e);
            r->err_code = kECuda;
            finish_request(r);
        }
        lk.lock();
        return;
    }
    stats_.waves++;
    stats_.launches += (uint64_t)n;
}

void Engine::worker() {
    cudaSetDevice(ctx_->device());
    for (;;) {
        Request* r = nullptr;
        {
            std::unique_lock<std::mutex> lk(mu_);
            if (!stop_ && host_q_.empty() && spin_us_ > 0 && spinning_workers_ < kSpinningWorkers) {
                // a few workers wait briefly awake: a stage's requests reach the
                // host without a thread wake-up
                ++spinning_workers_;
                const uint64_t seen = work_signal_.load(std::memory_order_acquire);
                lk.unlock();
                spin_for_signal(work_signal_, seen);
                lk.lock();
                --spinning_workers_;
            }
            work_cv_.wait(lk, [&] { return stop_ || !host_q_.empty(); });
            if (host_q_.empty()) return;
            r = host_q_.front();
            host_q_.pop_front();
            if (const int code = abort_code(r, Clock::now())) {  // its stage landed: end it here
                r->err_code = code;
                r->err = code == kECanceled ? "request cancelled" : "request timed out";
            }
        }
        if (r->err_code) {
            finish_request(r);
            continue;
        }
        const Clock::time_point t0 = Clock::now();
        int rc;
        {
            NvtxRange fs("fiat-shamir");
            rc = r->ps->complete_stage();
        }
        if (rc == kOk && r->ps->stage() == Stage::Done) r->ps->encode_proof(&r->proof);
        const Clock::time_point t1 = Clock::now();
        const double host_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        if (ctx_->tracing()) {
            const int d = (int)r->ps->depth();
            const double id = (double)r->ticket;
            ctx_->trace_host("fiat_shamir", d, t0, t1, 1.0, 0);
            // the stage's path: waiting for a wave, wave launch until the host saw
            // it complete, then until the end of the host step (worker pickup included)
            ctx_->trace_host("req_wait", d, r->t_ready, r->t_launch, id, 0);
            ctx_->trace_host("req_gpu", d, r->t_launch, r->t_landed, id, 0);
            ctx_->trace_host("req_host", d, r->t_landed, t1, id, 0);
        }
        if (rc != kOk || r->ps->stage() == Stage::Done) {
            if (rc != kOk) {
                r->err = r->ps->error();
                r->err_code = rc;
            }
            {
                std::lock_guard<std::mutex> g(mu_);
                stats_.host_stage_ms += host_ms;
            }
            finish_request(r);
            continue;
        }
        {
            std::lock_guard<std::mutex> g(mu_);
            stats_.host_stage_ms += host_ms;
            r->t_ready = t1;
            ready_.push_back(r);
        }
        sched_signal_.fetch_add(1, std::memory_order_release);
        sched_cv_.notify_one();
    }
}

void Engine::finish_request(Request* r) {
    const bool ok = r->err_code == 0;
    r->ps->release();  // stream-ordered frees; returns the budget
    r->t_done = Clock::now();
    {
        std::lock_guard<std::mutex> g(mu_);
        if (r->pinned_file) ctx_->put_pinned(r->pinned_file, r->pinned_bytes);
        r->pinned_file = nullptr;
        if (r->admitted) free_admit_events_.push_back(r->admitted);
        r->admitted = nullptr;
        if (r->state == Request::Active) --active_;
        r->state = ok ? Request::Done : Request::Failed;
        admit_blocked_ = false;
        last_progress_ = Clock::now();
        if (ok) {
            stats_.completed++;
            stats_.bytes_done += r->len;
        } else {
            stats_.failed++;
            if (r->err_code == kECanceled) stats_.cancelled++;
            if (r->err_code == kETimeout) stats_.timed_out++;
        }
    }
    done_cv_.notify_all();
    sched_signal_.fetch_add(1, std::memory_order_release);
    sched_cv_.notify_one();
}

int Engine::poll(uint64_t ticket, std::vector<uint8_t>* proof, double* latency_ms, std::string* err) {
    std::lock_guard<std::mutex> g(mu_);
    auto it = all_.find(ticket);
    if (it == all_.end()) return kEInval;
    Request* r = it->second.get();
    if (r->state != Request::Done && r->state != Request::Failed) return 0;
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    const int rc = r->state == Request::Done ? 1 : (r->err_code ? r->err_code : kECuda);
    if (proof) *proof = std::move(r->proof);
    if (err) *err = r->err;
    all_.erase(it);
    return rc;
}

cudaEvent_t Engine::take_admit_event() {
    if (!free_admit_events_.empty()) {
        cudaEvent_t ev = free_admit_events_.back();
        free_admit_events_.pop_back();
        return ev;
    }
    cudaEvent_t ev = nullptr;
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return ev;
}

bool Engine::finished_or_gone(uint64_t ticket) const {
    // a ticket another thread has collected meanwhile is gone (its request freed)
    auto it = all_.find(ticket);
    if (it == all_.end()) return true;
    const Request* r = it->second.get();
    return r->state == Request::Done || r->state == Request::Failed;
}

int Engine::wait(uint64_t ticket, std::vector<uint8_t>* proof, double* latency_ms, std::string* err) {
    {
        std::unique_lock<std::mutex> lk(mu_);
        if (!all_.count(ticket)) return kEInval;
        done_cv_.wait(lk, [&] { return finished_or_gone(ticket); });
    }
    return poll(ticket, proof, latency_ms, err);
}

int Engine::wait_any(const uint64_t* tickets, size_t n, size_t* which) {
    if (!tickets || !which) return kEInval;
    std::unique_lock<std::mutex> lk(mu_);
    std::vector<size_t> known;
    known.reserve(n);
    for (size_t i = 0; i < n; ++i)
        if (all_.count(tickets[i])) known.push_back(i);
    if (known.empty()) return kEInval;
    done_cv_.wait(lk, [&] {
        for (size_t i : known)
            if (finished_or_gone(tickets[i])) {
                *which = i;
                return true;
            }
        return false;
    });
    return kOk;
}

int Engine::wait_for(uint64_t ticket, double timeout_ms, std::vector<uint8_t>* proof, double* latency_ms,
                     std::string* err) {
    {
        std::unique_lock<std::mutex> lk(mu_);
        if (!all_.count(ticket)) return kEInval;
        const bool done = done_cv_.wait_for(
            lk, std::chrono::microseconds((int64_t)(timeout_ms > 0 ? timeout_ms * 1000.0 : 0)),
            [&] { return finished_or_gone(ticket); });
        if (!done) return kETimeout;
    }
    return poll(ticket, proof, latency_ms, err);
}

int Engine::abort_code(const Request* r, Clock::time_point now) const {
    if (r->cancel) return kECanceled;
    if (r->has_deadline && now >= r->deadline) return kETimeout;
    return 0;
}

int Engine::cancel(uint64_t ticket) {
    Request* now = nullptr;  // a queued request ends here; an admitted one at its next stage boundary
    {
        std::lock_guard<std::mutex> g(mu_);
        auto it = all_.find(ticket);
        if (it == all_.end()) return kEInval;
        Request* r = it->second.get();
        if (r->state == Request::Done || r->state == Request::Failed) return kEState;
        r->cancel = true;
        if (r->state == Request::Queued) {
            auto q = std::find(queued_.begin(), queued_.end(), r);
            if (q != queued_.end()) {  // not being admitted right now: nothing of it is on the device
                queued_.erase(q);
                r->err_code = kECanceled;
                r->err = "request cancelled";
                now = r;
            }
        }
    }
    if (now) finish_request(now);
    sched_cv_.notify_one();
    return kOk;
}

void Engine::set_admission_batch(int n) {
    {
        std::lock_guard<std::mutex> g(mu_);
        admit_batch_ = n > 0 ? n : 0;
    }
    sched_cv_.notify_one();
}

void Engine::set_request_timeout(double timeout_ms) {
    std::lock_guard<std::mutex> g(mu_);
    request_timeout_ms_ = timeout_ms > 0 ? timeout_ms : 0;
}

void Engine::health(uint64_t* unfinished, double* ms_since_progress) {
    std::lock_guard<std::mutex> g(mu_);
    const uint64_t open = stats_.submitted - stats_.completed - stats_.failed;
    if (unfinished) *unfinished = open;
    if (ms_since_progress) {
        const Clock::time_point from = last_progress_ > Clock::time_point{} ? last_progress_ : Clock::now();
        *ms_since_progress = open ? std::chrono::duration<double, std::milli>(Clock::now() - from).count() : 0.0;
    }
}

void Engine::drain() {
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return stats_.completed + stats_.failed == stats_.submitted; });
}

EngineStats Engine::stats() {
    std::lock_guard<std::mutex> g(mu_);
    return stats_;
}

}  // namespace dm
