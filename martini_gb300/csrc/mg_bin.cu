// Footprint binning: per-particle records, tile histograms, work-item plan and
// the tile-major particle list.
//
// The footprint of particle p is the reference's Chebyshev-box mask
// |i - x_p| <= r_p, |j - y_p| <= r_p (martini/martini.py:272-274) with
// r_p = ceil(sm_length * size_in_fwhm) (martini/sph_kernels.py:257-262).
// Its integer bounds are found here once per particle with the same FP64
// predicate, so the set of (pixel, particle) pairs equals the reference's.
#include <cmath>

#include "mg_internal.cuh"

namespace mg {

// Inclusive pixel range [lo, hi] of {i : |i - c| <= r}, clipped to [0, n).
__device__ __forceinline__ void box_bounds(double c, double r, int n, int& lo, int& hi) {
  if (!(r >= 0.0)) {  // NaN or negative range: empty
    lo = 0;
    hi = -1;
    return;
  }
  if (isinf(r)) {
    lo = 0;
    hi = n - 1;
    return;
  }
  double a = floor(c - r) - 1.0;
  double b = ceil(c + r) + 1.0;
  if (a < 0.0) a = 0.0;
  if (b > (double)(n - 1)) b = (double)(n - 1);
  if (a > b) {
    lo = 0;
    hi = -1;
    return;
  }
  int l = (int)a, h = (int)b;
  while (l <= h && !(fabs((double)l - c) <= r)) ++l;
  while (h >= l && !(fabs((double)h - c) <= r)) --h;
  lo = l;
  hi = h;
}

// Channel index range whose closed velocity interval meets [lo, hi].
__device__ __forceinline__ void channel_range(const double* e, int nc, int dec, double lo,
                                              double hi, int& c0, int& c1) {
  // E(k) = edges in increasing order
  auto E = [&](int k) { return dec ? e[nc - k] : e[k]; };
  // first c in [0, nc) with E(c + 1) >= lo
  int a = 0, b = nc;
  while (a < b) {
    int m = (a + b) >> 1;
    if (E(m + 1) >= lo) b = m; else a = m + 1;
  }
  int first = a;
  // last c in [0, nc) with E(c) <= hi  ->  (first c with E(c) > hi) - 1
  a = 0;
  b = nc;
  while (a < b) {
    int m = (a + b) >> 1;
    if (E(m) > hi) b = m; else a = m + 1;
  }
  int last = a - 1;
  if (first > last) {
    c0 = 1;
    c1 = 0;
    return;
  }
  if (dec) {
    c0 = nc - 1 - last;
    c1 = nc - 1 - first;
  } else {
    c0 = first;
    c1 = last;
  }
}


// One thread per particle: exact footprint, Dirac pixel, spectral support,
// packed record.  Tile coverage goes into a 2D difference array over the
// tile grid, (ntx + 1) x (nty + 1): +1 at the corners (tx0, ty0) and
// (tx1 + 1, ty1 + 1), -1 at (tx0, ty1 + 1) and (tx1 + 1, ty0), so four
// integer atomics per particle whatever its footprint; k_plan_tiles turns
// it into exact per-tile counts with prefix sums.  The array lives in
// shared memory when it fits (PREP_SMEM_DIFF) and is flushed once per block.
// The per-tile channel windows (needed only when a tile has several channel
// blocks) and the header maxima are reduced per block before their global
// atomics.
constexpr int PREP_THREADS = 256;
constexpr int PREP_SMEM_DIFF = 12288;

__global__ void __launch_bounds__(PREP_THREADS) k_prep(PrepArgs a, Geo g, Ws w) {
  extern __shared__ int s_diff[];  // the difference array when it fits
  __shared__ int s_wmax;
  __shared__ unsigned s_wb, s_sb;
  __shared__ unsigned long long s_spec;
  const int dw = g.nty + 1;
  const int ndiff = (g.ntx + 1) * dw;
  const bool smem_hist = ndiff <= PREP_SMEM_DIFF;
  int* const diff = smem_hist ? s_diff : w.tile_diff;
  const bool windows = w.ncb_seg > 1;
  if (smem_hist)
    for (int t = threadIdx.x; t < ndiff; t += blockDim.x) s_diff[t] = 0;
  if (threadIdx.x == 0) {
    s_wmax = 0;
    s_wb = s_sb = 0u;
    s_spec = 0ull;
  }
  __syncthreads();
  const int dec = w.hdr->edges_dec;
  int my_wmax = 0;
  unsigned my_wb = 0u, my_sb = 0u;
  unsigned my_spec = 0u;  // support channels of this thread's particles
  // every thread of a block runs the same number of iterations
  for (long long base = blockIdx.x * (long long)blockDim.x; base < a.n;
       base += (long long)gridDim.x * blockDim.x) {
    const long long p = base + threadIdx.x;
    if (p >= a.n) continue;
    PRec rec;
    rec.ilo = 0; rec.ihi = -1; rec.jlo = 0; rec.jhi = -1;
    rec.clo = 1; rec.chi = 0;
    rec.xi = rec.yi = 0;
    rec.xf = rec.yf = 0.f;
    rec.h = 1.f; rec.inv_h2 = 1.f;
    rec.vhi = rec.vlo = 0.f; rec.inv_s = 0.f; rec.amp = 0.f; rec.pad_ = 0;
    int ks = a.kidx ? (int)a.kidx[p] : 0;
    if (ks < 0 || ks >= g.n_kernels) ks = 0;  // -1: kernels[0] (sph_kernels.py:1360)
    rec.kslot = ks;
    double x = a.x[p], y = a.y[p], r = a.r[p];
    // |coordinate| > 2^30 px cannot reach the cube (and would overflow int)
    bool ok = isfinite(x) && isfinite(y) && fabs(x) < 1073741824.0 && fabs(y) < 1073741824.0;
    if (ok) {
      box_bounds(x, r, g.nx, rec.ilo, rec.ihi);
      box_bounds(y, r, g.ny, rec.jlo, rec.jhi);
      ok = rec.ilo <= rec.ihi && rec.jlo <= rec.jhi;
    }
    if (ok && g.ks[ks].type == MG_KERNEL_DIRAC) {
      // weight 1 iff |x - i| < 0.5 and |y - j| < 0.5 (sph_kernels.py:1165):
      // at most one pixel per axis, tested in FP64.
      int di = -1, dj = -1;
      double fx = floor(x), fy = floor(y);
      if (fabs(x - fx) < 0.5) di = (int)fx; else if (fabs(x - (fx + 1.0)) < 0.5) di = (int)fx + 1;
      if (fabs(y - fy) < 0.5) dj = (int)fy; else if (fabs(y - (fy + 1.0)) < 0.5) dj = (int)fy + 1;
      if (di < rec.ilo || di > rec.ihi || dj < rec.jlo || dj > rec.jhi) {
        ok = false;
      } else {
        rec.ilo = rec.ihi = di;
        rec.jlo = rec.jhi = dj;
      }
    }
    if (ok) {
      double fx = floor(x), fy = floor(y);
      rec.xi = (int)fx;
      rec.yi = (int)fy;
      rec.xf = (float)(x - fx);
      rec.yf = (float)(y - fy);
      float h = a.h ? a.h[p] : 1.f;
      rec.h = h;
      rec.inv_h2 = 1.f / (h * h);
      if (g.spectral_model == MG_SPECTRUM_TABLE) {
        rec.clo = 0;
        rec.chi = g.nc - 1;
        rec.amp = 1.f;
      } else {
        double v = a.v[p];
        double am = a.amp[p];
        rec.amp = (float)am;
        double vh = (double)(float)v;
        rec.vhi = (float)vh;
        rec.vlo = (float)(v - vh);
        if (g.spectral_model == MG_SPECTRUM_GAUSSIAN) {
          double s = a.sigma ? (double)a.sigma[p] : (double)g.sigma_const;
          rec.inv_s = (float)(1.0 / (1.4142135623730951 * s));
          // |u| <= 4.5: beyond it each wing holds erfc(4.5) / 2 = 1e-10 of
          // the line's flux
          double half = 4.5 * 1.4142135623730951 * s;
          channel_range(a.edges, g.nc, dec, v - half, v + half, rec.clo, rec.chi);
        } else {
          channel_range(a.edges, g.nc, dec, v, v, rec.clo, rec.chi);
        }
        if (am == 0.0 || !isfinite(v)) {
          rec.clo = 1;
          rec.chi = 0;
        }
      }
      ok = rec.clo <= rec.chi;
    }
    if (!ok) {
      rec.ilo = 0; rec.ihi = -1; rec.jlo = 0; rec.jhi = -1;
    }
    w.rec[p] = rec;
    int np = 0;
    if (ok) {
      int tx0 = rec.ilo / TILE_I, tx1 = rec.ihi / TILE_I;
      int ty0 = rec.jlo / TILE_J, ty1 = rec.jhi / TILE_J;
      np = (tx1 - tx0 + 1) * (ty1 - ty0 + 1);
      atomicAdd(&diff[tx0 * dw + ty0], 1);
      atomicAdd(&diff[tx0 * dw + ty1 + 1], -1);
      atomicAdd(&diff[(tx1 + 1) * dw + ty0], -1);
      atomicAdd(&diff[(tx1 + 1) * dw + ty1 + 1], 1);
      if (windows)
        for (int tx = tx0; tx <= tx1; ++tx)
          for (int ty = ty0; ty <= ty1; ++ty) {
            const int t = tx * g.nty + ty;
            atomicMin(&w.tile_wlo[t], rec.clo);
            atomicMax(&w.tile_whi[t], rec.chi);
          }
      my_wmax = max(my_wmax, rec.chi - rec.clo);
      my_spec += (unsigned)(rec.chi - rec.clo + 1);
      if (g.form == MG_FORM_F16X3) {
        // magnitude bounds for the scaled FP16 split (non-negative floats
        // order like their bit patterns)
        const KSpec k = g.ks[ks];
        float wb = weight_bound(k.type, rec.inv_h2, k.gnorm);
        my_wb = max(my_wb, __float_as_uint(wb));
        float sb = rec.amp;
        if (g.spectral_model == MG_SPECTRUM_TABLE) {
          sb = 0.f;
          for (int c = 0; c < g.nc; ++c) sb = fmaxf(sb, fabsf(a.spectra[p * g.nc + c]));
        }
        my_sb = max(my_sb, __float_as_uint(sb));
      }
    }
    w.npairs[p] = np;
  }
  my_wmax = __reduce_max_sync(0xffffffffu, my_wmax);
  my_wb = __reduce_max_sync(0xffffffffu, my_wb);
  my_sb = __reduce_max_sync(0xffffffffu, my_sb);
  my_spec = __reduce_add_sync(0xffffffffu, my_spec);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&s_wmax, my_wmax);
    atomicMax(&s_wb, my_wb);
    atomicMax(&s_sb, my_sb);
    atomicAdd(&s_spec, (unsigned long long)my_spec);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicMax(&w.hdr->wmax, s_wmax);
    if (g.spectral_model == MG_SPECTRUM_GAUSSIAN)
      atomicAdd(reinterpret_cast<unsigned long long*>(&w.hdr->spec_bound), s_spec);
    if (g.form == MG_FORM_F16X3) {
      atomicMax(&w.hdr->wbound_bits, s_wb);
      atomicMax(&w.hdr->sbound_bits, s_sb);
    }
  }
  if (smem_hist)
    for (int t = threadIdx.x; t < ndiff; t += blockDim.x)
      if (s_diff[t]) atomicAdd(&w.tile_diff[t], s_diff[t]);
}

__global__ void k_tile_init(Geo g, Ws w, long long cap_pairs, long long cap_partial) {
  const int ndiff = (g.ntx + 1) * (g.nty + 1);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ndiff; t += gridDim.x * blockDim.x) {
    w.tile_diff[t] = 0;
    if (t < g.ntiles) {
      w.tile_wlo[t] = 0x7fffffff;
      w.tile_whi[t] = -1;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    WsHeader* h = w.hdr;
    h->status = 0;
    h->item_counter = 0;
    h->reduce_counter = 0;
    h->edges_dec = 0;
    h->n_pairs = h->n_items = h->n_partial_items = h->partial_bound = 0;
    h->cap_pairs = cap_pairs;
    h->cap_partial_items = cap_partial;
    h->wmax = 0;
    h->wbound_bits = 0u;
    h->sbound_bits = 0u;
    h->invw_bits = 0u;
    h->spec_bound = 0;
    h->n_spec = 0;
    h->spec_ready = 0;
  }
}

// Single-block pass over tiles after the histogram: per-tile counts from the
// difference array (prefix sums along ty, then along tx; in shared memory
// when it fits in `smem_cap` ints, else in place), pair offsets of the
// tile-major list and an upper bound on split-K partial items (every segment
// of a tile holds at most the tile's count).
__global__ void k_plan_tiles(Geo g, Ws w, int smem_cap, int num_sms) {
  constexpr int NT = 1024;
  __shared__ long long s_a[NT], s_b[NT];
  extern __shared__ int s_d[];
  const int tid = threadIdx.x;
  {
    const int dw = g.nty + 1, dh = g.ntx + 1;
    const int ndiff = dw * dh;
    const bool in_smem = ndiff <= smem_cap;
    int* const d = in_smem ? s_d : w.tile_diff;
    if (in_smem)
      for (int e = tid; e < ndiff; e += NT) s_d[e] = w.tile_diff[e];
    __syncthreads();
    for (int r = tid; r < dh; r += NT) {
      int acc = 0;
      for (int c = 0; c < dw; ++c) {
        acc += d[r * dw + c];
        d[r * dw + c] = acc;
      }
    }
    __syncthreads();
    for (int c = tid; c < dw; c += NT) {
      int acc = 0;
      for (int r = 0; r < dh; ++r) {
        acc += d[r * dw + c];
        d[r * dw + c] = acc;
      }
    }
    __syncthreads();
    for (int t = tid; t < g.ntiles; t += NT) {
      const int tx = t / g.nty, ty = t - tx * g.nty;
      w.tile_count[t] = d[tx * dw + ty];
    }
    __syncthreads();
  }
  const int per = (g.ntiles + NT - 1) / NT;
  const int t0 = tid * per;
  const int t1 = min(g.ntiles, t0 + per);
  long long sa = 0, sb = 0;
  for (int t = t0; t < t1; ++t) sa += w.tile_count[t];
  s_a[tid] = sa;
  __syncthreads();
  for (int off = 1; off < NT; off <<= 1) {
    long long a = 0;
    if (tid >= off) a = s_a[tid - off];
    __syncthreads();
    s_a[tid] += a;
    __syncthreads();
  }
  // item size from the total, then the split-K bound with it
  const int kch = item_particles(s_a[NT - 1], num_sms);
  for (int t = t0; t < t1; ++t) {
    const int cnt = w.tile_count[t];
    const int nk = (cnt + kch - 1) / kch;
    if (nk > 1) sb += (long long)nk * w.ncb_seg;
  }
  s_b[tid] = sb;
  __syncthreads();
  for (int off = NT / 2; off > 0; off >>= 1) {
    if (tid < off) s_b[tid] += s_b[tid + off];
    __syncthreads();
  }
  long long ea = s_a[tid] - sa;
  for (int t = t0; t < t1; ++t) {
    w.tile_off[t] = ea;
    ea += w.tile_count[t];
  }
  if (tid == NT - 1) {
    w.tile_off[g.ntiles] = s_a[NT - 1];
    WsHeader* h = w.hdr;
    h->n_pairs = s_a[NT - 1];
    h->partial_bound = s_b[0];
    h->kch = kch;
    unsigned st = h->status & ST_EDGES;
    if (h->n_pairs > h->cap_pairs) st |= ST_PAIRS;
    h->status = st;
  }
}

// Pairs in particle order: key = tile << cbits | clo, value = particle id.
__global__ void k_emit(long long n, Geo g, Ws w, unsigned* __restrict__ keys, int* __restrict__ vals) {
  if (w.hdr->status & (ST_PAIRS | ST_EDGES)) return;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const PRec rec = w.rec[p];
    if (rec.ilo > rec.ihi) continue;
    long long o = w.pair_off[p];
    const int tx0 = rec.ilo / TILE_I, tx1 = rec.ihi / TILE_I;
    const int ty0 = rec.jlo / TILE_J, ty1 = rec.jhi / TILE_J;
    for (int tx = tx0; tx <= tx1; ++tx)
      for (int ty = ty0; ty <= ty1; ++ty) {
        const unsigned t = (unsigned)(tx * g.nty + ty);
        keys[o] = (t << w.cbits) | (unsigned)rec.clo;
        vals[o] = (int)p;
        ++o;
      }
  }
}

// First index in [lo, hi) of sorted keys with key >= k.
__device__ __forceinline__ long long lower_bound_keys(const unsigned* keys, long long lo,
                                                      long long hi, unsigned k) {
  while (lo < hi) {
    long long m = (lo + hi) >> 1;
    if (keys[m] < k) lo = m + 1; else hi = m;
  }
  return lo;
}

// One thread per segment (tile, channel block): the sorted-list range of the
// particles whose support [clo, chi] can meet the block (clo within
// [c0 - wmax, c0 + width)), its K chunks and its split-K partial items.
__global__ void k_segments(Geo g, Ws w) {
  const bool bad = (w.hdr->status & (ST_PAIRS | ST_EDGES)) != 0;
  const int wmax = w.hdr->wmax;
  const int kch = w.hdr->kch;
  const unsigned cmask_hi = (1u << w.cbits);
  for (int sg = blockIdx.x * blockDim.x + threadIdx.x; sg < w.nseg; sg += gridDim.x * blockDim.x) {
    const int t = sg / w.ncb_seg;
    const int cb = sg - t * w.ncb_seg;
    long long lo = w.tile_off[t], hi = w.tile_off[t + 1];
    int items = 0, part = 0;
    if (!bad && hi > lo) {
      if (w.ncb_seg > 1) {
        const int c0 = cb * w.seg_width;
        const int clo_min = c0 - wmax > 0 ? c0 - wmax : 0;
        const unsigned c_end = (unsigned)(c0 + w.seg_width);  // first clo past the block
        const unsigned tk = (unsigned)t << w.cbits;
        const long long a = lower_bound_keys(w.keys, lo, hi, tk | (unsigned)clo_min);
        const long long b = c_end >= cmask_hi ? hi : lower_bound_keys(w.keys, a, hi, tk | c_end);
        // skip blocks entirely outside the tile's channel window
        if (c0 > w.tile_whi[t] || c0 + w.seg_width <= w.tile_wlo[t]) {
          lo = hi = a;
        } else {
          lo = a;
          hi = b;
        }
      }
      const long long cnt = hi - lo;
      if (cnt > 0) {
        items = (int)((cnt + kch - 1) / kch);
        part = items > 1 ? items : 0;
      }
    }
    w.seg_lo[sg] = lo;
    w.seg_hi[sg] = hi;
    w.seg_items[sg] = items;
    w.seg_part[sg] = part;
  }
}

__global__ void k_check_partials(Ws w) {
  WsHeader* h = w.hdr;
  if (h->n_partial_items > h->cap_partial_items) h->status |= ST_PARTIALS;
}

// Channel edges as double-float pairs, inverse channel widths, edge
// direction and the strict-monotonicity check of spectral_models.py:180-187.
__global__ void k_edges(const double* e, int nc, Ws w) {
  const int dec = e[nc] < e[0];
  if (blockIdx.x == 0 && threadIdx.x == 0) w.hdr->edges_dec = dec;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= nc; k += gridDim.x * blockDim.x) {
    double v = e[k];
    float hi = (float)v;
    w.ehi[k] = hi;
    w.elo[k] = (float)(v - (double)hi);
    if (k < nc) {
      w.inv_w[k] = (float)(1.0 / fabs(e[k + 1] - e[k]));
      atomicMax(&w.hdr->invw_bits, __float_as_uint(w.inv_w[k]));
      bool mono = dec ? (e[k + 1] < e[k]) : (e[k + 1] > e[k]);
      if (!mono) atomicOr(&w.hdr->status, ST_EDGES);
    }
  }
}

static unsigned grid_for(long long n, int num_sms) {
  long long blocks = (n + 255) / 256;
  if (blocks > (long long)num_sms * 32) blocks = (long long)num_sms * 32;
  return (unsigned)(blocks > 0 ? blocks : 1);
}

// Records, tile histogram, per-particle pair offsets and the tile plan.
void launch_prep(const PrepArgs& a, const Geo& g, const Ws& w, int num_sms, cudaStream_t s,
                 long long cap_pairs, long long cap_partial) {
  k_tile_init<<<(g.ntiles + 255) / 256, 256, 0, s>>>(g, w, cap_pairs, cap_partial);
  k_edges<<<(g.nc + 256) / 256, 256, 0, s>>>(a.edges, g.nc, w);
  if (a.n > 0) {
    // with the histogram in shared memory every block flushes up to ntiles
    // counts: fewer, longer-lived blocks
    const size_t ndiff = (size_t)(g.ntx + 1) * (g.nty + 1);
    const bool smem_hist = ndiff <= (size_t)PREP_SMEM_DIFF;
    const size_t hist_bytes = smem_hist ? sizeof(int) * ndiff : 0;
    unsigned blocks = grid_for(a.n, num_sms);
    const unsigned per_sm = hist_bytes <= 16384 ? 8u : 4u;
    if (smem_hist && blocks > per_sm * (unsigned)num_sms) blocks = per_sm * (unsigned)num_sms;
    k_prep<<<blocks, PREP_THREADS, hist_bytes, s>>>(a, g, w);
  }
  launch_scan(w.npairs, a.n, w.pair_off, w.scan_sums, nullptr, s);
  // dynamic shared memory for the difference array: up to 200 KB
  // (the attribute is per device: set on every launch, a host-side call)
  constexpr int kPlanSmemCap = 50 * 1024;
  const long long ndiff_all = (long long)(g.ntx + 1) * (g.nty + 1);
  int cap = ndiff_all <= kPlanSmemCap ? (int)ndiff_all : 0;
  if (cap > 0 && cudaFuncSetAttribute(k_plan_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(sizeof(int) * kPlanSmemCap)) != cudaSuccess) {
    cudaGetLastError();  // fall back to the in-place prefix sums
    cap = 0;
  }
  k_plan_tiles<<<1, 1024, sizeof(int) * (size_t)cap, s>>>(g, w, cap, num_sms);
}

int sort_bits(const Geo& g, const Ws& w) {
  int tbits = 0;
  while ((1LL << tbits) < (long long)g.ntiles) ++tbits;
  return tbits + w.cbits;
}

// Tile-major list sorted by (tile, clo), then the segments with their
// work-item and partial offsets.  Pairs are emitted into the buffer from
// which an even/odd number of radix passes ends in w.keys / w.list.
void launch_sort_segments(const PrepArgs& a, const Geo& g, const Ws& w, long long cap_pairs,
                          int num_sms, cudaStream_t s) {
  const int passes = (sort_bits(g, w) + 7) / 8;
  unsigned* k0 = (passes & 1) ? w.keys_tmp : w.keys;
  int* v0 = (passes & 1) ? w.list_tmp : w.list;
  unsigned* k1 = (passes & 1) ? w.keys : w.keys_tmp;
  int* v1 = (passes & 1) ? w.list : w.list_tmp;
  if (a.n > 0) k_emit<<<grid_for(a.n, num_sms), 256, 0, s>>>(a.n, g, w, k0, v0);
  launch_radix_sort(k0, v0, k1, v1, &w.hdr->n_pairs, cap_pairs, sort_bits(g, w), w.rs_hist,
                    w.rs_off, w.scan_sums, num_sms, s);
  k_segments<<<(unsigned)((w.nseg + 255) / 256), 256, 0, s>>>(g, w);
  launch_scan(w.seg_items, w.nseg, w.item_off, w.scan_sums, &w.hdr->n_items, s);
  launch_scan(w.seg_part, w.nseg, w.part_off, w.scan_sums, &w.hdr->n_partial_items, s);
  k_check_partials<<<1, 1, 0, s>>>(w);
}

}  // namespace mg
