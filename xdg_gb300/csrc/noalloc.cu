// noalloc.cu -- the packed tet walk without any device-memory allocation.
//
// xdgcu_walk_elements_packed (api.cu) allocates the scratch of its offset
// scan with cudaMallocAsync on every call.  Some callers cannot let a library
// allocate: a transport code or framework whose own allocator owns the
// device memory (a caching pool that reserves the free memory at start-up,
// so a foreign cudaMalloc fails or fragments it), or a particle loop that
// must not call into the allocator at all once set up.  For them this entry
// point takes its scratch from a file-scope static device array instead.
//
// The array holds the per-block sums of the scan for at most
// XDGCU_NOALLOC_MAX_TRACKS tracks (4097 int64 = 32 KiB).  Every GPU that
// loads this library keeps it until the process exits.  Host code cannot use
// the array's name as a device address, so the first call on each device
// looks the address up with cudaGetSymbolAddress (with that device current)
// and caches it; that first call should come before any stream capture.  The
// cached address belongs to the device's primary context: after a
// cudaDeviceReset (or a reset of the primary context) the library cannot be
// used on that device again in the same process.
// All calls share the array and it keeps the last call's contents.  Nothing
// in it needs to start at zero: the scan writes every block sum before it
// reads it.  Calls whose work overlaps on the GPU (different streams, or
// different host threads) race on the array and must be serialised by the
// caller.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/xdgcu.h"
#include "internal.cuh"
#include "walk.h"

namespace xdgcu {

namespace {

constexpr int64_t kNoAllocScratch = (XDGCU_NOALLOC_MAX_TRACKS + 1023) / 1024 + 1;
static_assert(kNoAllocScratch >= 1, "scratch size");

static __device__ __align__(256) int64_t g_walk_scan_scratch[kNoAllocScratch];

std::mutex g_mu;
int64_t* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_walk_scan_scratch on the current device (looked up on
// the first call per device).
cudaError_t scratch_address(int dev, int64_t** out) {
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_walk_scan_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<int64_t*>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

}  // namespace

// Shared with api.cu: fills the geometry part of WalkArgs for a context and
// reports its face order, or returns an error message.
const char* walk_args_for(const xdgcu_ctx* ctx, WalkArgs* a, int* face_order, int* device);
int set_last_error(int code, const char* msg);

}  // namespace xdgcu

using namespace xdgcu;

extern "C" int xdgcu_walk_elements_packed_noalloc(
    xdgcu_ctx* ctx, int64_t n, const int32_t* start_index, const double* start, const double* u,
    const double* distance, int32_t max_segs, int64_t capacity, int32_t* seg_elem, double* seg_len,
    int64_t* offsets, int32_t* status, int32_t precision, void* stream) {
  if (!ctx) return set_last_error(XDGCU_ERR_INVALID_ARG, "null context");
  if (n < 0 || capacity < 0) return set_last_error(XDGCU_ERR_INVALID_ARG, "negative size");
  if (n > XDGCU_NOALLOC_MAX_TRACKS)
    return set_last_error(XDGCU_ERR_INVALID_ARG,
                          "walk_elements_packed_noalloc: more than XDGCU_NOALLOC_MAX_TRACKS "
                          "(4194304) tracks in one call; split the batch");
  if (precision != XDGCU_FP64 && precision != XDGCU_MIXED)
    return set_last_error(XDGCU_ERR_INVALID_ARG, "precision must be XDGCU_FP64 or XDGCU_MIXED");
  if (!offsets) return set_last_error(XDGCU_ERR_INVALID_ARG, "offsets required");
  if (n > 0 && (!start_index || !start || !u || !distance || max_segs <= 0))
    return set_last_error(XDGCU_ERR_INVALID_ARG, "bad inputs");
  if (capacity > 0 && (!seg_elem || !seg_len))
    return set_last_error(XDGCU_ERR_INVALID_ARG, "null segment arrays");
  WalkArgs a{};
  int face_order = 0, dev = 0;
  if (const char* msg = walk_args_for(ctx, &a, &face_order, &dev))
    return set_last_error(XDGCU_ERR_STATE, msg);
  if (dev < 0 || dev >= kMaxDevices) return set_last_error(XDGCU_ERR_INVALID_ARG, "device id");
  DeviceGuard guard(dev);
  if (!guard.ok()) return set_last_error(XDGCU_ERR_CUDA, "cudaSetDevice failed");
  // device memory of the context's device only: host pointers would need
  // staging buffers, and another GPU's memory is not this device's to walk into
  for (const void* p : {(const void*)start_index, (const void*)start, (const void*)u,
                        (const void*)distance, (const void*)seg_elem, (const void*)seg_len,
                        (const void*)offsets, (const void*)status}) {
    if (!p) continue;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess ||
        (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)) {
      cudaGetLastError();
      return set_last_error(XDGCU_ERR_INVALID_ARG,
                            "walk_elements_packed_noalloc takes device pointers only");
    }
    if (at.type == cudaMemoryTypeDevice && at.device != dev)
      return set_last_error(XDGCU_ERR_INVALID_ARG,
                            "walk_elements_packed_noalloc: an array is on another device than "
                            "the context's");
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (n == 0) {
    const cudaError_t e = cudaMemsetAsync(offsets, 0, sizeof(int64_t), st);
    return e == cudaSuccess ? XDGCU_OK : set_last_error(XDGCU_ERR_CUDA, cudaGetErrorString(e));
  }
  int64_t* scratch = nullptr;
  cudaError_t e = scratch_address(dev, &scratch);
  if (e != cudaSuccess) return set_last_error(XDGCU_ERR_CUDA, cudaGetErrorString(e));
  a.n = n;
  a.max_segs = max_segs;
  a.capacity = capacity;
  a.start = start_index;
  a.org = start;
  a.dir = u;
  a.dist = distance;
  a.seg_elem = seg_elem;
  a.seg_len = seg_len;
  a.offsets = offsets;
  a.status = status;
  a.counters = nullptr;
  const bool mixed = precision == XDGCU_MIXED;
  a.out_mode = WALK_COUNT;
  e = launch_walk(mixed, face_order, a, st);
  if (e == cudaSuccess) e = scan_offsets(offsets, n, scratch, st);
  if (e == cudaSuccess) {
    a.out_mode = WALK_PACKED;
    e = launch_walk(mixed, face_order, a, st);
  }
  return e == cudaSuccess ? XDGCU_OK : set_last_error(XDGCU_ERR_CUDA, cudaGetErrorString(e));
}
