// BLAKE3 file id of a device buffer for callers that cannot allocate device
// memory: code running while a CUDA graph is being captured, serving loops that
// run under a fixed, pre-reserved memory budget, or hosts whose allocator is
// owned by another framework.  The only scratch the file hash needs -- the
// chunk chaining values of the BLAKE3 tree -- lives in a file-scope device array
// sized for the largest file this library proves, so the call makes no
// cudaMalloc / cudaFree / pool allocation of its own.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/damascus.h"
#include "dm_kernels.cuh"

namespace {

// Largest input: 64 MiB (65,536 BLAKE3 chunks).  Every file the prover accepts
// (depth <= 11, at most 2048^2 * 13 bytes = 54.5 MB) fits.
constexpr uint64_t kNoAllocMaxFileBytes = 64ull << 20;
constexpr uint64_t kNoAllocMaxChunks = kNoAllocMaxFileBytes / 1024;

// Two ping-pong levels of 8 words per chunk: 4 MiB, held by every device that
// loads this library until the process exits.
__device__ __align__(256) uint32_t g_noalloc_cv_scratch[2 * 8 * kNoAllocMaxChunks];

struct DeviceScratch {
    std::once_flag once;
    void* ptr = nullptr;
    cudaError_t err = cudaSuccess;
};
constexpr int kMaxDevices = 64;
DeviceScratch g_scratch[kMaxDevices];

}  // namespace

extern "C" int damascus_file_id_noalloc(const void* d_file, size_t len, void* d_out32, void* stream) {
    if ((d_file == nullptr && len != 0) || d_out32 == nullptr) return DAMASCUS_EINVAL;
    if (len > kNoAllocMaxFileBytes) return DAMASCUS_ESIZE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return DAMASCUS_ECUDA;
    // The host-side name of the array is not a device address: resolve it once
    // per device, with that device current.
    DeviceScratch& s = g_scratch[dev];
    std::call_once(s.once, [&s] { s.err = cudaGetSymbolAddress(&s.ptr, g_noalloc_cv_scratch); });
    if (s.err != cudaSuccess || s.ptr == nullptr) return DAMASCUS_ECUDA;
    const cudaError_t e = dm::launch_file_hash(static_cast<const uint8_t*>(d_file), len,
                                               static_cast<uint32_t*>(s.ptr), static_cast<uint32_t*>(d_out32),
                                               static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? DAMASCUS_OK : DAMASCUS_ECUDA;
}
