// Scratch memory of hyk_propagate_noalloc(), the propagation entry point for
// callers that cannot allocate device memory.
//
// hyk_propagate() keeps two counters in a caller-provided workspace: the
// persistent kernel's lane-queue counter and the one-launch-per-step form's
// finished-lane counter.  Some callers cannot provide one: code running where
// cudaMalloc is not allowed, such as inside another library's memory pool, a
// real-time loop that must not allocate, or a host integration that owns no
// CUDA allocator.  For them the counters live here, in a file-scope device
// array that every GPU which loads libhyk holds until the process exits.
//
// The array's host-side name is a stand-in, not a device address: its device
// address is looked up once per device with cudaGetSymbolAddress, with that
// device's context current, and only that pointer is passed to kernels.

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>

#include "hyk.h"  // HYK_NOALLOC_SCRATCH_BYTES: the size of the array below

static __device__ __align__(256) unsigned char g_hyk_noalloc_scratch[HYK_NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_mtx;
void *g_addr[64];
bool g_done[64];
}  // namespace

// Device address of the scratch array on `device` (whose context must be
// current on the calling thread).  The first call per device performs the
// lookup; later calls return the cached address.
extern "C" __attribute__((visibility("hidden"))) int hyk_noalloc_scratch(int device, void **ptr, size_t *bytes,
                                                                         char *err, size_t errlen) {
    if (device < 0 || device >= 64) {
        std::snprintf(err, errlen, "device ordinal %d out of range", device);
        return -1;
    }
    std::lock_guard<std::mutex> lk(g_mtx);
    if (!g_done[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_hyk_noalloc_scratch);
        if (e != cudaSuccess) {
            std::snprintf(err, errlen, "cudaGetSymbolAddress of the scratch array failed: %s", cudaGetErrorString(e));
            // Clear the runtime's sticky last error, so that a later runtime
            // call of this library does not report this failure as its own.
            (void)cudaGetLastError();
            return -2;
        }
        g_addr[device] = p;
        g_done[device] = true;
    }
    *ptr = g_addr[device];
    *bytes = HYK_NOALLOC_SCRATCH_BYTES;
    return 0;
}
