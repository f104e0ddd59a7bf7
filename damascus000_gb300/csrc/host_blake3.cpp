#include "host_blake3.h"

#include <atomic>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "dm_blake3.cuh"

namespace dm {

namespace {
const uint32_t kIV[8] = {DM_B3_IV0, DM_B3_IV1, DM_B3_IV2, DM_B3_IV3, DM_B3_IV4, DM_B3_IV5, DM_B3_IV6, DM_B3_IV7};

void words16(const uint8_t* p, uint32_t m[16]) {
    for (int i = 0; i < 16; ++i) m[i] = b3_load_le32(p + 4 * i);
}
}  // namespace

Blake3Hasher::Blake3Hasher() : flags_(0) {
    std::memcpy(key_, kIV, sizeof(key_));
    std::memcpy(cv_, key_, sizeof(cv_));
}

Blake3Hasher::Blake3Hasher(const uint8_t key[32]) : flags_(kB3Keyed) {
    for (int i = 0; i < 8; ++i) key_[i] = b3_load_le32(key + 4 * i);
    std::memcpy(cv_, key_, sizeof(cv_));
}

void Blake3Hasher::compress_buffered_block() {
    uint32_t m[16], out[16];
    words16(buf_, m);
    const uint32_t f = flags_ | (blocks_done_ == 0 ? kB3ChunkStart : 0u);
    b3_compress(cv_, m, chunk_counter_, kB3BlockLen, f, out);
    std::memcpy(cv_, out, 32);
    ++blocks_done_;
    buf_len_ = 0;
}

// Merges completed subtrees: one parent per trailing zero bit of total_chunks.
void Blake3Hasher::push_chunk_cv(const uint32_t cv_in[8], uint64_t total_chunks) {
    uint32_t cv[8];
    std::memcpy(cv, cv_in, 32);
    while ((total_chunks & 1) == 0) {
        uint32_t m[16], out[16];
        std::memcpy(m, stack_[depth_ - 1], 32);
        std::memcpy(m + 8, cv, 32);
        b3_compress(key_, m, 0, kB3BlockLen, flags_ | kB3Parent, out);
        std::memcpy(cv, out, 32);
        --depth_;
        total_chunks >>= 1;
    }
    std::memcpy(stack_[depth_++], cv, 32);
}

void Blake3Hasher::update(const void* data, size_t len) {
    const uint8_t* p = static_cast<const uint8_t*>(data);
    while (len > 0) {
        // A full chunk is closed only once more input arrives (its last block needs CHUNK_END).
        if (blocks_done_ * kB3BlockLen + buf_len_ == kB3ChunkLen) {
            uint32_t m[16], out[16];
            words16(buf_, m);
            b3_compress(cv_, m, chunk_counter_, kB3BlockLen, flags_ | kB3ChunkEnd | (blocks_done_ == 0 ? kB3ChunkStart : 0u),
                        out);
            push_chunk_cv(out, chunk_counter_ + 1);
            ++chunk_counter_;
            std::memcpy(cv_, key_, 32);
            blocks_done_ = 0;
            buf_len_ = 0;
        }
        if (buf_len_ == kB3BlockLen) compress_buffered_block();
        // Fast path: whole blocks straight from the input while more follows.
        size_t take = kB3BlockLen - buf_len_;
        const size_t chunk_room = kB3ChunkLen - (blocks_done_ * kB3BlockLen + buf_len_);
        if (take > chunk_room) take = chunk_room;
        if (take > len) take = len;
        std::memcpy(buf_ + buf_len_, p, take);
        buf_len_ += (uint32_t)take;
        p += take;
        len -= take;
    }
}

void Blake3Hasher::update_u64(uint64_t v) {
    uint8_t t[8];
    for (int i = 0; i < 8; ++i) t[i] = (uint8_t)(v >> (8 * i));
    update(t, 8);
}

void Blake3Hasher::finalize(uint8_t out[32]) const {
    // Pending output: the current chunk's last block.
    uint32_t cv[8], m[16], outw[16];
    std::memcpy(cv, cv_, 32);
    uint8_t block[64];
    std::memset(block, 0, sizeof(block));
    std::memcpy(block, buf_, buf_len_);
    words16(block, m);
    uint64_t counter = chunk_counter_;
    uint32_t blen = buf_len_;
    uint32_t flags = flags_ | kB3ChunkEnd | (blocks_done_ == 0 ? kB3ChunkStart : 0u);
    for (int d = depth_; d > 0; --d) {
        b3_compress(cv, m, counter, blen, flags, outw);  // chaining value of the pending node
        std::memcpy(m, stack_[d - 1], 32);
        std::memcpy(m + 8, outw, 32);
        std::memcpy(cv, key_, 32);
        counter = 0;
        blen = kB3BlockLen;
        flags = flags_ | kB3Parent;
    }
    b3_compress(cv, m, 0, blen, flags | kB3Root, outw);
    for (int i = 0; i < 8; ++i) {
        out[4 * i] = (uint8_t)outw[i];
        out[4 * i + 1] = (uint8_t)(outw[i] >> 8);
        out[4 * i + 2] = (uint8_t)(outw[i] >> 16);
        out[4 * i + 3] = (uint8_t)(outw[i] >> 24);
    }
}

void blake3_hash(const void* data, size_t len, uint8_t out[32]) {
    Blake3Hasher h;
    h.update(data, len);
    h.finalize(out);
}

void blake3_keyed_hash(const uint8_t key[32], const void* data, size_t len, uint8_t out[32]) {
    Blake3Hasher h(key);
    h.update(data, len);
    h.finalize(out);
}

// ============================================================== host pool

namespace {

class Pool {
   public:
    static Pool& get() {
        static Pool* p = new Pool();  // lives until exit; threads are detached
        return *p;
    }
    size_t size() const { return workers_; }
    // Runs tasks[1..] on the workers and tasks[0] on the caller.  The counter is
    // decremented and signalled under done_mu, so the caller cannot see zero and
    // return (destroying done_mu / done_cv on its stack) before the last task has
    // released the mutex.
    void run(const std::vector<std::function<void()>>& tasks) {
        if (tasks.empty()) return;
        size_t left = tasks.size() - 1;
        std::mutex done_mu;
        std::condition_variable done_cv;
        {
            std::lock_guard<std::mutex> g(mu_);
            for (size_t i = 1; i < tasks.size(); ++i)
                queue_.push_back([&, i] {
                    tasks[i]();
                    std::lock_guard<std::mutex> g2(done_mu);
                    if (--left == 0) done_cv.notify_all();
                });
        }
        cv_.notify_all();
        tasks[0]();
        std::unique_lock<std::mutex> lk(done_mu);
        done_cv.wait(lk, [&] { return left == 0; });
    }

   private:
    Pool() {
        unsigned n = std::thread::hardware_concurrency();
        workers_ = n > 1 ? n : 1;
        for (size_t i = 0; i + 1 < workers_; ++i) std::thread([this] { loop(); }).detach();
    }
    void loop() {
        for (;;) {
            std::function<void()> f;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return !queue_.empty(); });
                f = std::move(queue_.front());
                queue_.pop_front();
            }
            f();
        }
    }
    size_t workers_ = 1;
    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<std::function<void()>> queue_;
};

struct ChunkArgs {
    const uint8_t* data;
    size_t len;
    uint32_t* cvs;
};

void chunk_cvs(void* a, size_t begin, size_t end) {
    const ChunkArgs* A = static_cast<const ChunkArgs*>(a);
    for (size_t c = begin; c < end; ++c) {
        const size_t off = c * kB3ChunkLen;
        const size_t clen = A->len - off < kB3ChunkLen ? A->len - off : kB3ChunkLen;
        const size_t nblocks = (clen + 63) / 64;
        uint32_t cv[8];
        std::memcpy(cv, kIV, 32);
        for (size_t b = 0; b < nblocks; ++b) {
            uint8_t block[64];
            const size_t bl = clen - b * 64 < 64 ? clen - b * 64 : 64;
            std::memset(block, 0, 64);
            std::memcpy(block, A->data + off + b * 64, bl);
            uint32_t m[16], out[16];
            words16(block, m);
            uint32_t f = (b == 0 ? kB3ChunkStart : 0u) | (b + 1 == nblocks ? kB3ChunkEnd : 0u);
            b3_compress(cv, m, c, (uint32_t)bl, f, out);
            std::memcpy(cv, out, 32);
        }
        std::memcpy(A->cvs + 8 * c, cv, 32);
    }
}

}  // namespace

namespace {
thread_local bool t_serial = false;
}  // namespace

HostSerialScope::HostSerialScope() : prev_(t_serial) { t_serial = true; }
HostSerialScope::~HostSerialScope() { t_serial = prev_; }

void host_parallel_for(size_t n, size_t min_per_task, void (*fn)(void*, size_t, size_t), void* arg) {
    if (t_serial) {
        fn(arg, 0, n);
        return;
    }
    Pool& P = Pool::get();
    size_t tasks = (n + min_per_task - 1) / (min_per_task ? min_per_task : 1);
    if (tasks > P.size()) tasks = P.size();
    if (tasks <= 1) {
        fn(arg, 0, n);
        return;
    }
    std::vector<std::function<void()>> v;
    for (size_t t = 0; t < tasks; ++t) {
        const size_t b = n * t / tasks, e = n * (t + 1) / tasks;
        v.push_back([=] { fn(arg, b, e); });
    }
    P.run(v);
}

void blake3_hash_parallel(const void* data, size_t len, uint8_t out[32]) {
    const size_t nchunks = (len + kB3ChunkLen - 1) / kB3ChunkLen;
    if (len < (64u << 10) || nchunks < 2 || t_serial) {
        blake3_hash(data, len, out);
        return;
    }
    std::vector<uint32_t> a(8 * nchunks), b(8 * nchunks);
    ChunkArgs args{static_cast<const uint8_t*>(data), len, a.data()};
    host_parallel_for(nchunks, 16, chunk_cvs, &args);
    // pairwise merge with carry; the final merge is the root
    size_t n = nchunks;
    uint32_t* src = a.data();
    uint32_t* dst = b.data();
    uint32_t outw[16];
    while (n > 1) {
        const size_t pairs = n / 2;
        for (size_t j = 0; j < pairs; ++j) {
            uint32_t m[16];
            std::memcpy(m, src + 16 * j, 64);
            const bool root = (n == 2);
            b3_compress(kIV, m, 0, kB3BlockLen, kB3Parent | (root ? kB3Root : 0u), outw);
            std::memcpy(dst + 8 * j, outw, 32);
        }
        if (n & 1) std::memcpy(dst + 8 * pairs, src + 8 * (n - 1), 32);
        n = pairs + (n & 1);
        std::swap(src, dst);
    }
    for (int i = 0; i < 8; ++i) {
        out[4 * i] = (uint8_t)src[i];
        out[4 * i + 1] = (uint8_t)(src[i] >> 8);
        out[4 * i + 2] = (uint8_t)(src[i] >> 16);
        out[4 * i + 3] = (uint8_t)(src[i] >> 24);
    }
}

}  // namespace dm
