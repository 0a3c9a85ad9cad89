// mg_insert_noalloc: the full insertion on a scratch area that lives in the
// library itself, for callers that cannot allocate GPU memory.
//
// Some callers of this library cannot call cudaMalloc: code running inside a
// memory pool that forbids outside allocations, plugins hosted by a
// framework that owns every device allocation, or real-time paths where an
// allocation (and the device-wide synchronisation it can imply) is not
// allowed.  For them this entry point needs nothing but the inputs and the
// output cube: its scratch (the binning lists, sort buffers, per-tile plan and
// split-K partials that mg_insert keeps in the caller's workspace) is one
// file-scope device array of MG_NOALLOC_SCRATCH_BYTES, reserved on every GPU
// that loads the library for as long as the process lives.
//
// Set-up: the first call on a device (with that device current) looks the
// array up with cudaGetSymbolAddress and caches the address; make that first
// call before any stream capture.  Every call reuses the same array and the
// pipeline re-initialises, on the device, everything that must start from
// zero; two calls that overlap on the GPU (for example on two streams) race
// on the array and corrupt each other.  The call synchronises the stream
// (it reads back the status word) and allocates nothing: no cudaMalloc, no
// cudaFree, no allocating library routine.
#include <string>

#include "mg_internal.cuh"

namespace mg {
void set_last_error(const std::string& msg);  // mg_api.cu
}

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[MG_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array for the current device (looked up once
// per device; the host-side symbol is not a device address).
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return MG_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return MG_ERR_UNSUPPORTED;
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) return MG_ERR_CUDA;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return MG_OK;
}

}  // namespace

extern "C" int mg_insert_noalloc(const mg_problem* p, void* stream) {
  if (!p) return MG_ERR_INVALID_ARGUMENT;
  void* ws = nullptr;
  int rc = scratch_address(&ws);
  if (rc) {
    mg::set_last_error("mg_insert_noalloc: cannot locate the device scratch array");
    return rc;
  }
  const size_t cap = MG_NOALLOC_SCRATCH_BYTES;
  // capacities that fit the array: a quarter of what is left after the fixed
  // part goes to split-K partial tiles, the rest to the (tile, particle) list
  size_t fixed = 0;
  rc = mg_workspace_size(p, 0, 0, &fixed);
  if (rc) return rc;
  if (fixed > cap) {
    mg::set_last_error("mg_insert_noalloc: problem too large for the built-in scratch (" +
                       std::to_string(fixed) + " bytes needed before any particle pairs, " +
                       std::to_string(cap) + " available); use mg_insert with a workspace");
    return MG_ERR_WORKSPACE;
  }
  size_t one_partial = 0, one_partial0 = 0;
  rc = mg_workspace_size(p, 0, 1, &one_partial);
  if (rc) return rc;
  rc = mg_workspace_size(p, 0, 0, &one_partial0);
  if (rc) return rc;
  const size_t partial_bytes = one_partial > one_partial0 ? one_partial - one_partial0 : 1;
  long long cap_partial = (long long)((cap - fixed) / 4 / partial_bytes);
  // largest pair capacity whose workspace still fits (binary search)
  long long lo = 0, hi = (long long)((cap - fixed) / 16) + 1;
  while (hi - lo > 1) {
    const long long mid = lo + (hi - lo) / 2;
    size_t b = 0;
    rc = mg_workspace_size(p, mid, cap_partial, &b);
    if (rc) return rc;
    if (b <= cap) lo = mid; else hi = mid;
  }
  rc = mg_insert(p, ws, cap, lo, cap_partial, stream);
  if (rc) return rc;
  return mg_check(ws, stream);
}
