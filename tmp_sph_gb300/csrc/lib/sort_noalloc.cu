// sort_noalloc.cu — sph_sort_particles_noalloc: the stable (hash, index) sort with its scratch
// in a fixed device array of this library, so the call allocates nothing.
//
// Why it exists.  The reference's sortParticles(hash, index, n) (src/header/mesh.cuh:23) has
// no scratch argument.  A caller that binds that three-argument form and reserved all of its
// device memory up front (a step loop that must not grow its footprint, or must not meet an
// allocation failure half way through a run) can neither pass a buffer nor let the sort
// allocate one on every call.  This entry point serves it: the same radix sort as
// sph_sort_particles, same results, with the scratch taken from g_sort_scratch below.
//
// Limits and rules.
//  * n <= SPH_SORT_NOALLOC_MAX_N; larger n is refused with SPH_ERR_SCRATCH before anything is
//    launched (use sph_sort_particles with a caller buffer for those).
//  * The first call on a device does the setup: it looks up the device address of
//    g_sort_scratch for the current device (cudaGetSymbolAddress, which may load this module
//    on that device).  Make that first call, per device, before any stream capture begins.
//    Every later call made while its stream is not capturing looks the address up again, so
//    a device whose context was destroyed and recreated since (cudaDeviceReset) gets the
//    address of its new array; a call inside a capture uses the address of the last lookup.
//  * Nothing in the scratch has to start at zero: the sort clears its digit totals itself at
//    the start of every call and writes the key/value buffers and the per-tile histograms
//    before reading them.
//  * There is one scratch array per device.  Calls on the same device whose executions
//    overlap (different streams without ordering between them, or host threads racing)
//    race on it and give wrong results; order them on one stream or with events.
#include <cuda_runtime.h>

#include <mutex>

#include "sph_gb300.h"
#include "sph_internal.h"

namespace {

// Two ping-pong buffers of n 4-byte keys and values, one 256-digit histogram per tile of at
// least 1024 keys (n/4 bytes), the digit totals, and 256-byte alignment of each part: at most
// 9 n bytes plus 64 KiB.  setup() checks the sort's own requirement against this size.
constexpr size_t kScratchBytes = 9 * (size_t)SPH_SORT_NOALLOC_MAX_N + 65536;

__device__ __align__(256) unsigned char g_sort_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_sort_scratch on the current device: looked up on the first call and on
// every call whose stream is not being captured (the array moves when the context is
// recreated); inside a capture the last lookup's address is used.
int scratch_for_current_device(cudaStream_t stream, void** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return SPH_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) return SPH_ERR_ARG;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess) {
        cudaGetLastError();
        return SPH_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev] || cap == cudaStreamCaptureStatusNone) {
        if (sph::sort_scratch_bytes(SPH_SORT_NOALLOC_MAX_N) > kScratchBytes) return SPH_ERR_SCRATCH;
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_sort_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return SPH_ERR_CUDA;
        }
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return SPH_OK;
}

}  // namespace

extern "C" int sph_sort_particles_noalloc(int* hash, int* index, int n, int key_bits,
                                          void* stream) {
    if (n < 0 || key_bits < 1 || key_bits > 32 || (n > 0 && (!hash || !index)))
        return SPH_ERR_ARG;
    if (n > SPH_SORT_NOALLOC_MAX_N) return SPH_ERR_SCRATCH;
    if (n <= 1) return SPH_OK;
    void* scratch = nullptr;
    const int st = scratch_for_current_device((cudaStream_t)stream, &scratch);
    if (st != SPH_OK) return st;
    cudaError_t e = sph::radix_sort_pairs(reinterpret_cast<unsigned*>(hash), index,
                                          reinterpret_cast<unsigned*>(hash), index, n, key_bits,
                                          scratch, kScratchBytes, nullptr, (cudaStream_t)stream);
    return e == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}
