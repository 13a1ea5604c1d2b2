// noalloc.cu -- oneka_track for callers that cannot allocate device memory.
//
// oneka_track chronicles each realization into caller-owned scratch.  Some
// callers cannot provide it: they run inside a host whose device memory is
// carved up at start-up by that host's own allocator (a plugin in a serving
// process, a pooled runtime that forbids cudaMalloc after initialization), or
// they reach the GPU through a binding that only passes buffers the host
// already owns.  oneka_track_noalloc serves them from a fixed array that lives
// inside this library instead: g_noalloc_slots below, ONEKA_NOALLOC_SCRATCH_BYTES
// (32 MiB).  The CUDA runtime loads this library's device code lazily, on its
// first use on a device, so the array is reserved on a device at the first
// call there (the first oneka_track_noalloc, or any other first launch of the
// library on that device), not when the library is loaded.  A host that hands
// the rest of the GPU to its own allocator should make one call during its own
// set-up, before that allocator takes the memory.  The array is then held until
// the process exits.
//
// The array is shared by every call on a device and keeps what the last call
// left in it; each call clears the slots it is about to use before tracking.
// Two calls whose work overlaps on the GPU (different streams, or another
// host thread) race on the array and corrupt each other's counts: order them
// on one stream or serialize them.
//
// Host code may not use g_noalloc_slots as a pointer: in host code the name
// is a host-side stand-in, not the device address.  The first call on each
// device, with that device current, asks the runtime for the array's device
// address (cudaGetSymbolAddress) and caches it for the process; that first call
// should come before any stream capture.  A cudaDeviceReset (or any teardown
// of the device's primary context) unloads the array and leaves the cached
// address stale: it is not supported while this library is in use.
#include <mutex>

#include "oneka_internal.cuh"

namespace {

__device__ __align__(256) uint32_t g_noalloc_slots[ONEKA_NOALLOC_SCRATCH_BYTES / 4];

constexpr int kMaxDevices = 128;
std::mutex g_mu;
void* g_addr[kMaxDevices];   // device address of g_noalloc_slots on each device, once set up

int noalloc_scratch(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        oneka::set_error("oneka_track_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
        return ONEKA_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        oneka::set_error("oneka_track_noalloc: device ordinal %d is beyond %d", dev, kMaxDevices);
        return ONEKA_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_slots);
        if (e != cudaSuccess || !p) {
            oneka::set_error("oneka_track_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return ONEKA_ERR_CUDA;
        }
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return ONEKA_OK;
}

}  // namespace

extern "C" int oneka_track_noalloc(const OnekaSite* site, const OnekaRealizations* real, int32_t nreal,
                                   const double* release, int32_t npaths, const OnekaTrackOpts* opts,
                                   const OnekaGrid* grid, const OnekaFrame* frames, int32_t* counts,
                                   int64_t* registered, const OnekaTrackOut* out, void* stream) {
    if (!counts || nreal <= 0)   // tracking only (no chronicle, no scratch), or nothing to do
        return oneka_track(site, real, nreal, release, npaths, opts, grid, frames, counts, registered, out,
                           nullptr, 0, stream);
    const size_t slot = oneka_track_scratch_bytes(grid, 1);
    if (slot == 0) {
        oneka::set_error("invalid argument: grid (nrows, ncols, dx, dy must be > 0)");
        return ONEKA_ERR_INVALID;
    }
    if (slot > (size_t)ONEKA_NOALLOC_SCRATCH_BYTES) {
        oneka::set_error("oneka_track_noalloc: a %d x %d grid needs %zu bytes per realization slot; "
                         "the library's fixed scratch holds %zu bytes (use oneka_track with caller scratch)",
                         grid->nrows, grid->ncols, slot, (size_t)ONEKA_NOALLOC_SCRATCH_BYTES);
        return ONEKA_ERR_SCRATCH;
    }
    void* scratch = nullptr;
    const int rc = noalloc_scratch(&scratch);
    if (rc != ONEKA_OK) return rc;
    size_t nslots = (size_t)ONEKA_NOALLOC_SCRATCH_BYTES / slot;
    if (nreal > 0 && (size_t)nreal < nslots) nslots = (size_t)nreal;
    const size_t used = nslots * slot;
    // the array keeps the previous call's contents: clear the slots this call uses
    const cudaError_t e = cudaMemsetAsync(scratch, 0, used, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        oneka::set_error("oneka_track_noalloc: cudaMemsetAsync: %s", cudaGetErrorString(e));
        return ONEKA_ERR_CUDA;
    }
    return oneka_track(site, real, nreal, release, npaths, opts, grid, frames, counts, registered, out,
                       scratch, used, stream);
}
