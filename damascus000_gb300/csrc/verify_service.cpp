#include "verify_service.h"

#include <cstring>

#include "host_blake3.h"

namespace dm {

VerifyService::VerifyService(Context* ctx, int workers, uint64_t cache_bytes) : ctx_(ctx) {
    if (workers <= 0) {
        const unsigned hc = std::thread::hardware_concurrency();
        workers = hc ? (int)(hc < 16 ? hc : 16) : 4;
    }
    if (cache_bytes) cache_.reset(new GenCache(ctx, cache_bytes));
    cudaError_t e = cudaSetDevice(ctx->device());
    streams_.resize(workers, nullptr);
    for (int w = 0; w < workers && e == cudaSuccess; ++w) e = cudaStreamCreateWithFlags(&streams_[w], cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        // reported by init_error(); no workers: the destructor frees what was created
        init_error_ = std::string("verifier service setup: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return;
    }
    for (int w = 0; w < workers; ++w) threads_.emplace_back([this, w] { worker(w); });
}

VerifyService::~VerifyService() {
    {
        std::lock_guard<std::mutex> g(mu_);
        stop_ = true;  // queued jobs still run; nothing new is accepted
    }
    work_cv_.notify_all();
    for (auto& t : threads_) t.join();
    cache_.reset();  // every holder has synchronised its stream
    for (cudaStream_t s : streams_)
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
}

int VerifyService::submit(const uint8_t* proof, size_t len, const uint8_t epoch[32], uint64_t* ticket) {
    if ((!proof && len) || !epoch || !ticket) return kEInval;
    auto job = std::make_shared<Job>();
    job->proof.assign(proof, proof + len);
    std::memcpy(job->epoch, epoch, 32);
    uint64_t N = 0, fp = 0;
    uint32_t n = 0;
    if (!proof_shape(job->proof.data(), len, &N, &n, &fp)) fp = 0;  // fails in the verifier with its own code
    job->footprint = fp;
    job->t0 = std::chrono::steady_clock::now();
    {
        std::lock_guard<std::mutex> g(mu_);
        if (stop_) return kEState;
        *ticket = next_ticket_++;
        jobs_[*ticket] = job;
        queue_.push_back(*ticket);
        st_.submitted += 1;
    }
    work_cv_.notify_one();
    return kOk;
}

void VerifyService::worker(int w) {
    cudaSetDevice(ctx_->device());
    HostSerialScope serial;  // one proof per worker already fills the cores
    std::unique_lock<std::mutex> lk(mu_);
    uint64_t trimmed_for = 0;  // the queue head this worker trimmed the cache for since it last waited
    auto wait = [&] {
        trimmed_for = 0;
        work_cv_.wait(lk);
    };
    for (;;) {
        if (queue_.empty()) {
            if (stop_) return;
            wait();
            continue;
        }
        const uint64_t ticket = queue_.front();
        std::shared_ptr<Job> job = jobs_[ticket];
        // Admission in arrival order.  Running jobs are counted both in the
        // context's reservations and here (their allocations may not have been
        // made yet): conservative by at most their footprint.  A job that cannot
        // fit even alone runs alone and fails or succeeds as the one-shot
        // verifier would.
        const uint64_t want = ctx_->reserved() + admitted_bytes_ + job->footprint;
        if (want > ctx_->budget() && cache_ && trimmed_for != ticket) {
            // jobs come before cached families: drop the ones nobody holds.  The
            // trim's cudaFree waits for the device: not under the service's lock,
            // which the other workers need to finish their jobs.
            trimmed_for = ticket;
            const uint64_t need = admitted_bytes_ + job->footprint;
            lk.unlock();
            cache_->trim(need);
            lk.lock();
            continue;  // the queue may have changed meanwhile
        }
        if ((want > ctx_->budget() || job->alone) && running_ > 0) {
            wait();
            continue;
        }
        if (want > ctx_->budget() && job->footprint <= ctx_->budget()) {
            // nothing of ours runs and memory held by other users of the context
            // is in the way: their releases do not signal this service, so look
            // again shortly
            trimmed_for = 0;
            work_cv_.wait_for(lk, std::chrono::milliseconds(2));
            continue;
        }
        queue_.pop_front();
        running_ += 1;
        admitted_bytes_ += job->footprint;
        lk.unlock();

        std::string err;
        bool hit = false;
        const int rc = verify_proof(ctx_, job->proof.data(), job->proof.size(), job->epoch, streams_[w],
                                    cache_.get(), &err, &hit);
        const double ms =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - job->t0).count();

        lk.lock();
        const uint64_t reserved = ctx_->reserved();
        if (reserved > st_.peak_reserved) st_.peak_reserved = reserved;
        running_ -= 1;
        admitted_bytes_ -= job->footprint;
        if (rc == kENoMem && !job->alone) {
            // the device memory of concurrent jobs (and of a cached family this job
            // added) was in the way: run it again with nothing else of ours running,
            // where the verdict is the one-shot verifier's
            job->alone = true;
            queue_.push_front(ticket);
            st_.retried += 1;
            work_cv_.notify_all();
            continue;
        }
        std::vector<uint8_t>().swap(job->proof);
        job->verdict = rc;
        job->err = std::move(err);
        job->latency_ms = ms;
        job->done = true;
        st_.completed += 1;
        if (rc == kOk) st_.accepted += 1;
        else st_.rejected += 1;
        done_cv_.notify_all();
        work_cv_.notify_all();
    }
}

int VerifyService::take(uint64_t ticket, bool block, int* verdict, double* latency_ms, std::string* err) {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = jobs_.find(ticket);
    if (it == jobs_.end()) return kEInval;
    std::shared_ptr<Job> job = it->second;
    if (block) done_cv_.wait(lk, [&] { return job->done; });
    if (!job->done) return 0;
    if (verdict) *verdict = job->verdict;
    if (latency_ms) *latency_ms = job->latency_ms;
    if (err) *err = job->err;
    jobs_.erase(it);
    return 1;
}

int VerifyService::poll(uint64_t ticket, int* verdict, double* latency_ms, std::string* err) {
    return take(ticket, false, verdict, latency_ms, err);
}

int VerifyService::wait(uint64_t ticket, int* verdict, double* latency_ms, std::string* err) {
    return take(ticket, true, verdict, latency_ms, err);
}

void VerifyService::drain() {
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return queue_.empty() && running_ == 0; });
}

VerifyStats VerifyService::stats() {
    VerifyStats s;
    {
        std::lock_guard<std::mutex> g(mu_);
        s = st_;
    }
    if (cache_) {
        const GenCache::Stats c = cache_->stats();
        s.cache_hits = c.hits;
        s.cache_misses = c.misses;
        s.cache_bytes = c.bytes;
    }
    return s;
}

}  // namespace dm
