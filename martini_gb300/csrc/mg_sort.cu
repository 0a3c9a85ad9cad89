// Device-wide exclusive scan and stable LSD radix sort of (key, value) pairs.
//
// Used by the footprint binning: (tile, particle) pairs are emitted in
// particle order and sorted by key = segment << cbits | kernel class | first
// channel of the particle's spectral support.  The sort is stable, so the
// order within a segment, class and channel is particle order and the
// binning is deterministic.
#include "mg_internal.cuh"

namespace mg {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;  // 2048

// Block-wide exclusive scan of one value per thread (returns the block total).
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* smem, T& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = lane < (int)(blockDim.x >> 5) ? smem[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    smem[lane] = w;
  }
  __syncthreads();
  const T warp_base = warp > 0 ? smem[warp - 1] : T(0);
  total = smem[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_base + x - v;
}

// Phase 1: per-block sums of int32 counts.
__global__ void k_scan_reduce(const int* __restrict__ in, long long n, long long* __restrict__ sums) {
  __shared__ long long sm[32];
  long long base = (long long)blockIdx.x * SCAN_TILE;
  long long s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    long long i = base + (long long)k * SCAN_THREADS + threadIdx.x;
    if (i < n) s += in[i];
  }
  long long tot;
  block_exclusive_scan<long long>(s, sm, tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// Phase 2: exclusive scan of the block sums in one block (any count).
__global__ void k_scan_top(long long* __restrict__ sums, long long nblocks, long long* __restrict__ total) {
  __shared__ long long sm[32];
  long long carry = 0;
  for (long long b0 = 0; b0 < nblocks; b0 += blockDim.x) {
    long long i = b0 + threadIdx.x;
    long long v = i < nblocks ? sums[i] : 0;
    long long tot;
    long long ex = block_exclusive_scan<long long>(v, sm, tot);
    if (i < nblocks) sums[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

// Phase 3: scan within each block plus the block's offset.
__global__ void k_scan_apply(const int* __restrict__ in, long long n, const long long* __restrict__ sums,
                             long long* __restrict__ out) {
  __shared__ long long sm[32];
  long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
  long long v[SCAN_ITEMS];
  long long s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    long long i = base + k;
    v[k] = i < n ? in[i] : 0;
    s += v[k];
  }
  long long tot;
  long long run = sums[blockIdx.x] + block_exclusive_scan<long long>(s, sm, tot);
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    long long i = base + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
}

long long scan_blocks(long long n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }

// Exclusive scan of n int32 counts into out (int64); total into *total.
// sums needs scan_blocks(n) entries.
void launch_scan(const int* in, long long n, long long* out, long long* sums, long long* total,
                 cudaStream_t s) {
  long long nb = scan_blocks(n);
  if (nb == 0) {
    k_scan_top<<<1, 1024, 0, s>>>(sums, 0, total);
    return;
  }
  k_scan_reduce<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, sums);
  k_scan_top<<<1, 1024, 0, s>>>(sums, nb, total);
  k_scan_apply<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, sums, out);
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits.  Each block owns RS_TILE consecutive
// elements; ranks within a block follow element order, so the sort is stable.
// ---------------------------------------------------------------------------

constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;  // 4096
constexpr int RS_WARPS = RS_THREADS / 32;

long long radix_blocks(long long n) { return (n + RS_TILE - 1) / RS_TILE; }

__global__ void k_radix_hist(const unsigned* __restrict__ keys, const long long* __restrict__ np,
                             long long cap, int shift, int* __restrict__ hist, long long nblocks_cap) {
  __shared__ int h[256];
  const long long n = min(*np, cap);
  const long long nb = (n + RS_TILE - 1) / RS_TILE;
  for (long long b = blockIdx.x; b < nblocks_cap; b += gridDim.x) {
    h[threadIdx.x] = 0;
    __syncthreads();
    if (b < nb) {
      const long long base = b * RS_TILE;
      for (int r = 0; r < RS_ROUNDS; ++r) {
        long long i = base + r * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1);
      }
    }
    __syncthreads();
    // digit-major layout: hist[d * nblocks_cap + b]
    hist[(long long)threadIdx.x * nblocks_cap + b] = h[threadIdx.x];
    __syncthreads();
  }
}

__global__ void k_radix_scatter(const unsigned* __restrict__ kin, const int* __restrict__ vin,
                                unsigned* __restrict__ kout, int* __restrict__ vout,
                                const long long* __restrict__ np, long long cap, int shift,
                                const long long* __restrict__ off, long long nblocks_cap) {
  __shared__ int running[256];
  __shared__ int wcnt[RS_WARPS][256];
  __shared__ long long base_off[256];
  const long long n = min(*np, cap);
  const long long nb = (n + RS_TILE - 1) / RS_TILE;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (long long b = blockIdx.x; b < nb; b += gridDim.x) {
    running[threadIdx.x] = 0;
    base_off[threadIdx.x] = off[(long long)threadIdx.x * nblocks_cap + b];
    for (int w = 0; w < RS_WARPS; ++w) wcnt[w][threadIdx.x] = 0;
    __syncthreads();
    const long long base = b * RS_TILE;
    for (int r = 0; r < RS_ROUNDS; ++r) {
      const long long i = base + r * RS_THREADS + threadIdx.x;
      const bool valid = i < n;
      unsigned key = valid ? kin[i] : 0u;
      int val = valid ? vin[i] : 0;
      // invalid lanes get digit 256 (never written)
      const int digit = valid ? (int)((key >> shift) & 255u) : 256;
      const unsigned peers = __match_any_sync(0xffffffffu, digit);
      const int rank_in_warp = __popc(peers & ((1u << lane) - 1u));
      const int leader = __ffs(peers) - 1;
      if (valid && lane == leader) wcnt[warp][digit] = __popc(peers);
      __syncthreads();
      if (valid) {
        int before = running[digit];
        for (int w = 0; w < warp; ++w) before += wcnt[w][digit];
        const long long dst = base_off[digit] + before + rank_in_warp;
        kout[dst] = key;
        vout[dst] = val;
      }
      __syncthreads();
      {
        int add = 0;
        for (int w = 0; w < RS_WARPS; ++w) {
          add += wcnt[w][threadIdx.x];
          wcnt[w][threadIdx.x] = 0;
        }
        running[threadIdx.x] += add;
      }
      __syncthreads();
    }
  }
}

// Sort n (<= cap; n read on the device) pairs in place (keys/values), using
// kt/vt as the second buffer; `bits` = significant key bits.  hist and off
// need 256 * radix_blocks(cap) entries, sums scan_blocks(256 * radix_blocks(cap)).
// After an odd number of passes the result is in kt/vt: returns true then.
bool launch_radix_sort(unsigned* keys, int* vals, unsigned* kt, int* vt, const long long* np,
                       long long cap, int bits, int* hist, long long* off, long long* sums,
                       int num_sms, cudaStream_t s) {
  const long long nbc = radix_blocks(cap);
  if (nbc == 0) return false;
  const int passes = (bits + 7) / 8;
  unsigned* ki = keys;
  int* vi = vals;
  unsigned* ko = kt;
  int* vo = vt;
  long long grid = nbc < (long long)num_sms * 8 ? nbc : (long long)num_sms * 8;
  for (int p = 0; p < passes; ++p) {
    const int shift = 8 * p;
    k_radix_hist<<<(unsigned)grid, RS_THREADS, 0, s>>>(ki, np, cap, shift, hist, nbc);
    launch_scan(hist, 256 * nbc, off, sums, nullptr, s);
    k_radix_scatter<<<(unsigned)grid, RS_THREADS, 0, s>>>(ki, vi, ko, vo, np, cap, shift, off, nbc);
    unsigned* tk = ki; ki = ko; ko = tk;
    int* tv = vi; vi = vo; vo = tv;
  }
  return (passes & 1) != 0;
}

}  // namespace mg
