// Incremental BLAKE3 hasher on the host (the Fiat-Shamir transcript stays on
// the host, src/protocol/transcript.rs:42-64).  Written from the BLAKE3
// specification; shares the compression function with the device code.
#pragma once

#include <cstddef>
#include <cstdint>

namespace dm {

class Blake3Hasher {
   public:
    Blake3Hasher();
    explicit Blake3Hasher(const uint8_t key[32]);
    void update(const void* data, size_t len);
    void update_u64(uint64_t v);
    void finalize(uint8_t out[32]) const;

   private:
    void push_chunk_cv(const uint32_t cv[8], uint64_t total_chunks);
    void compress_buffered_block();
    uint32_t key_[8];
    uint32_t flags_;
    uint32_t stack_[56][8];
    int depth_ = 0;
    // current chunk
    uint32_t cv_[8];
    uint64_t chunk_counter_ = 0;
    uint8_t buf_[64];
    uint32_t buf_len_ = 0;
    uint32_t blocks_done_ = 0;
};

void blake3_hash(const void* data, size_t len, uint8_t out[32]);
// Same digest; chunk chaining values are computed on the host worker pool for
// inputs of 64 KiB and more, then merged pairwise (left-complete tree).
void blake3_hash_parallel(const void* data, size_t len, uint8_t out[32]);

// Fixed pool of host threads: fn(begin, end) over a split of [0, n).
void host_parallel_for(size_t n, size_t min_per_task, void (*fn)(void*, size_t, size_t), void* arg);

// While alive, host_parallel_for and blake3_hash_parallel run on the calling
// thread alone: for callers that already keep every core busy with independent
// work (a verifier worker per core), where splitting each hash over the pool
// only adds hand-offs.  Results are unchanged.
class HostSerialScope {
   public:
    HostSerialScope();
    ~HostSerialScope();
    HostSerialScope(const HostSerialScope&) = delete;
    HostSerialScope& operator=(const HostSerialScope&) = delete;

   private:
    bool prev_;
};
void blake3_keyed_hash(const uint8_t key[32], const void* data, size_t len, uint8_t out[32]);

}  // namespace dm
