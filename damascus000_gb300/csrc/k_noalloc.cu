// BLAKE3 file id of a device buffer for callers that cannot allocate device
// memory: serving loops that run under a fixed, pre-reserved memory budget
// (an allocation there could fail or push another tenant out), and hosts whose
// device allocator is owned by another framework (a cudaMalloc beside it is
// invisible to its accounting, and cudaFree synchronises the device under it).
// The only scratch the file hash needs -- the chunk chaining values of the
// BLAKE3 tree -- lives in a file-scope device array of a fixed size, so the
// call makes no cudaMalloc / cudaFree / pool allocation of its own.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/damascus.h"
#include "dm_kernels.cuh"

namespace {

// Largest input: 64 MiB (65,536 BLAKE3 chunks).  That covers every file of
// depth <= 11 (at most 2048^2 * 13 bytes = 54.5 MB); files of depth 12 and 13,
// which the prover also accepts, are larger and get DAMASCUS_ESIZE here.
constexpr uint64_t kNoAllocMaxFileBytes = 64ull << 20;
constexpr uint64_t kNoAllocMaxChunks = kNoAllocMaxFileBytes / 1024;

// Two ping-pong levels of 8 words per chunk: 4 MiB, held by every device that
// loads this library until the process exits.
__device__ __align__(256) uint32_t g_noalloc_cv_scratch[2 * 8 * kNoAllocMaxChunks];

// Device address of the array per device, resolved on the first call that
// succeeds in resolving it: a failed attempt (say, inside a stream capture or
// before the device has a context) is not stored, so a later call retries.
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};

void* scratch_address(int dev) {
    std::lock_guard<std::mutex> g(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_cv_scratch) == cudaSuccess) g_scratch_ptr[dev] = p;
        else cudaGetLastError();  // reset the runtime's last error: the caller's next call is unaffected
    }
    return g_scratch_ptr[dev];
}

}  // namespace

extern "C" int damascus_file_id_noalloc(const void* d_file, size_t len, void* d_out32, void* stream) {
    if ((d_file == nullptr && len != 0) || d_out32 == nullptr) return DAMASCUS_EINVAL;
    if (len > kNoAllocMaxFileBytes) return DAMASCUS_ESIZE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return DAMASCUS_ECUDA;
    // The host-side name of the array is not a device address: resolve it per
    // device, with that device current.
    void* scratch = scratch_address(dev);
    if (scratch == nullptr) return DAMASCUS_ECUDA;
    const cudaError_t e = dm::launch_file_hash(static_cast<const uint8_t*>(d_file), len,
                                               static_cast<uint32_t*>(scratch), static_cast<uint32_t*>(d_out32),
                                               static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? DAMASCUS_OK : DAMASCUS_ECUDA;
}
