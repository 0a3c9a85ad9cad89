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
// Set-up: every call (with the target device current) looks the array up
// with cudaGetSymbolAddress, which allocates nothing and is cheap; nothing is
// cached, so a device reset or a re-created primary context (which reloads
// the module and may move the array) never leaves a stale address.  Every
// call reuses the same array and the pipeline re-initialises, on the device,
// everything that must start from zero; two calls that overlap on the GPU
// (for example on two streams) race on the array and corrupt each other.
// The call synchronises the stream (it reads back the status word), so it
// cannot be captured in a CUDA graph, and it allocates nothing: no
// cudaMalloc, no cudaFree, no allocating library routine.
//
// The array is shared out as: the fixed part of the workspace layout, then
// (tensor-core forms with Gaussian lines) an eighth of the array held back
// for the per-particle spectrum store, then a quarter of the rest for
// split-K partial tiles and the largest (tile, particle) pair capacity that
// fits.  A spectrum store that does not fit its share is skipped and the
// lines are evaluated inside the contraction (same results).
#include <string>

#include "mg_internal.cuh"

namespace mg {
void set_last_error(const std::string& msg);  // mg_api.cu
}

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[MG_NOALLOC_SCRATCH_BYTES];

// Device address of the scratch array on the current device (the host-side
// symbol is not a device address), looked up on every call.
int scratch_address(void** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || p == nullptr) return MG_ERR_CUDA;
  *out = p;
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
  // room held back for the spectrum store (tensor-core forms, Gaussian lines)
  const bool tc = p->form == MG_FORM_BF16X3 || p->form == MG_FORM_F16X3 ||
                  p->form == MG_FORM_BF16X6;
  const size_t spec_room =
      (tc && p->spectral_model == MG_SPECTRUM_GAUSSIAN) ? MG_NOALLOC_SCRATCH_BYTES / 8 : 0;
  const size_t cap = MG_NOALLOC_SCRATCH_BYTES - spec_room;
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
  rc = mg_insert(p, ws, MG_NOALLOC_SCRATCH_BYTES, lo, cap_partial, stream);
  if (rc) return rc;
  rc = mg_check(ws, stream);
  if (rc == MG_ERR_WORKSPACE)
    mg::set_last_error(
        "mg_insert_noalloc: the built-in scratch (MG_NOALLOC_SCRATCH_BYTES = " +
        std::to_string((size_t)MG_NOALLOC_SCRATCH_BYTES) +
        " bytes) is too small for this problem's (tile, particle) pairs or split-K partial "
        "tiles (room for " + std::to_string(lo) + " pairs and " + std::to_string(cap_partial) +
        " partial tiles); use mg_insert with a workspace sized by mg_plan");
  return rc;
}
