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

// ---------------------------------------------------------------------------
// The galaxy table: kernel parameters into the workspace (no host copy, so
// the insertion can be captured in a CUDA graph).
// ---------------------------------------------------------------------------

constexpr int GALS_PER_SET = 16;
struct GalChunk {
  Gal g[GALS_PER_SET];
};
static_assert(sizeof(GalChunk) <= 3584, "galaxy chunk must fit the 4 KB parameter space");

__global__ void k_set_gals(GalChunk c, int first, int count, Geo g, Ws w) {
  const int k = threadIdx.x;
  if (k < count) {
    const Gal& G = c.g[k];
    const int gi = first + k;
    w.gal[gi] = G;
    w.gp0[gi] = G.p0;
    w.gt0[gi] = G.tile0;
    w.gs0[gi] = G.seg0;
    w.ge0[gi] = G.edge0;
    w.gr0[gi] = G.row0;
  }
  if (k == 0 && first + count == g.ngal) {
    w.gp0[g.ngal] = g.n;
    w.gt0[g.ngal] = g.ntiles;
    w.gs0[g.ngal] = g.nseg;
    w.ge0[g.ngal] = (int)g.nedge;
    w.gr0[g.ngal] = g.nrows;
  }
}

void launch_set_gals(const Gal* gals, const Geo& g, const Ws& w, cudaStream_t s) {
  for (int first = 0; first < g.ngal; first += GALS_PER_SET) {
    GalChunk c;
    const int count = g.ngal - first < GALS_PER_SET ? g.ngal - first : GALS_PER_SET;
    for (int k = 0; k < count; ++k) c.g[k] = gals[first + k];
    k_set_gals<<<1, 32, 0, s>>>(c, first, count, g, w);
  }
}

// ---------------------------------------------------------------------------
// Records and tile coverage
// ---------------------------------------------------------------------------

// One thread per particle of the batch: exact footprint, Dirac pixel,
// spectral support, packed record.  Tile coverage goes into the cube's 2D
// difference array over its tile grid, (ntx + 1) x (nty + 1): +1 at the
// corners (tx0, ty0) and (tx1 + 1, ty1 + 1), -1 at (tx0, ty1 + 1) and
// (tx1 + 1, ty0), so four integer atomics per particle whatever its
// footprint; k_diff_prefix turns them into exact per-tile counts.  For a
// single cube whose array fits (PREP_SMEM_DIFF) the array lives in shared
// memory and is flushed once per block.  The per-tile channel windows (needed
// only when a tile has several channel blocks) use global atomics; the
// per-cube maxima are reduced over the warp when its particles share a cube.
constexpr int PREP_THREADS = 256;
constexpr int PREP_SMEM_DIFF = 12288;

__global__ void __launch_bounds__(PREP_THREADS) k_prep(Geo g, Ws w) {
  extern __shared__ int s_diff[];  // the difference array of a single cube when it fits
  __shared__ unsigned long long s_spec;
  const bool smem_hist = g.ngal == 1 && g.ndiff <= PREP_SMEM_DIFF;
  if (smem_hist)
    for (int t = threadIdx.x; t < (int)g.ndiff; t += blockDim.x) s_diff[t] = 0;
  if (threadIdx.x == 0) s_spec = 0ull;
  __syncthreads();
  unsigned my_spec = 0u;  // support channels of this thread's particles
  const int lane = threadIdx.x & 31;
  // every thread of a block runs the same number of iterations
  for (long long base = blockIdx.x * (long long)blockDim.x; base < g.n;
       base += (long long)gridDim.x * blockDim.x) {
    const long long P = base + threadIdx.x;
    const bool valid = P < g.n;
    const int gk = valid ? find_gal(w.gp0, g.ngal, P) : 0;
    const Gal& G = w.gal[gk];
    int wmax_v = 0;
    unsigned wb_v = 0u, sb_v = 0u;
    if (valid) {
      const long long p = P - G.p0;
      const int dec = w.gst[gk].dec;
      const double* edges = G.edges;
      PRec rec;
      rec.ilo = 0; rec.ihi = -1; rec.jlo = 0; rec.jhi = -1;
      rec.clo = 1; rec.chi = 0;
      rec.xi = rec.yi = 0;
      rec.xf = rec.yf = 0.f;
      rec.h = 1.f; rec.inv_h2 = 1.f;
      rec.vhi = rec.vlo = 0.f; rec.inv_s = 0.f; rec.amp = 0.f; rec.flags = 0;
      int ks = G.kidx ? (int)G.kidx[p] : 0;
      if (ks < 0 || ks >= g.n_kernels) ks = 0;  // -1: kernels[0] (sph_kernels.py:1360)
      rec.kslot = ks;
      double x = G.x[p], y = G.y[p], r = G.r[p];
      // |coordinate| > 2^30 px cannot reach the cube (and would overflow int)
      bool ok = isfinite(x) && isfinite(y) && fabs(x) < 1073741824.0 && fabs(y) < 1073741824.0;
      if (ok) {
        box_bounds(x, r, G.nx, rec.ilo, rec.ihi);
        box_bounds(y, r, G.ny, rec.jlo, rec.jhi);
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
        float h = G.h ? G.h[p] : 1.f;
        rec.h = h;
        rec.inv_h2 = 1.f / (h * h);
        if (g.ks[ks].type <= MG_KERNEL_QUARTIC_SPLINE) {
          // every table kernel reaches h px; rows outside the cube are never
          // stored.  Tested in FP32 with a margin well above its rounding
          // (coordinates below 2^30 px): a flag missed near the edge only
          // keeps the per-row box test
          const float xf32 = (float)x;
          const float reach = h * (1.f + 0x1p-18f) + 1e-6f * (fabsf(xf32) + 1.f);
          const bool lo_in = rec.ilo == 0 || xf32 - (float)(rec.ilo - 1) >= reach;
          const bool hi_in = rec.ihi == G.nx - 1 || (float)(rec.ihi + 1) - xf32 >= reach;
          if (lo_in && hi_in) rec.flags |= PREC_ROWS_COVER;
          const float yf32 = (float)y;
          const float reach_y = h * (1.f + 0x1p-18f) + 1e-6f * (fabsf(yf32) + 1.f);
          const bool lo_jn = rec.jlo == 0 || yf32 - (float)(rec.jlo - 1) >= reach_y;
          const bool hi_jn = rec.jhi == G.ny - 1 || (float)(rec.jhi + 1) - yf32 >= reach_y;
          if (lo_jn && hi_jn) rec.flags |= PREC_COLS_COVER;
        }
        if (g.spectral_model == MG_SPECTRUM_TABLE) {
          rec.clo = 0;
          rec.chi = G.nc - 1;
          rec.amp = 1.f;
        } else {
          double v = G.v[p];
          double am = G.amp[p];
          rec.amp = (float)am;
          double vh = (double)(float)v;
          rec.vhi = (float)vh;
          rec.vlo = (float)(v - vh);
          if (g.spectral_model == MG_SPECTRUM_GAUSSIAN) {
            double sg = G.sigma ? (double)G.sigma[p] : (double)G.sigma_const;
            rec.inv_s = 1.f / (float)(1.4142135623730951 * sg);  // FP32 division
            // |u| <= 4.5: beyond it each wing holds erfc(4.5) / 2 = 1e-10 of
            // the line's flux
            double half = 4.5 * 1.4142135623730951 * sg;
            channel_range(edges, G.nc, dec, v - half, v + half, rec.clo, rec.chi);
          } else {
            channel_range(edges, G.nc, dec, v, v, rec.clo, rec.chi);
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
      w.rec[P] = rec;
      int np = 0;
      if (ok) {
        const int tx0 = rec.ilo / TILE_I, tx1 = rec.ihi / TILE_I;
        const int ty0 = rec.jlo / TILE_J, ty1 = rec.jhi / TILE_J;
        // one pair per (tile, channel block) the line meets
        const int nb = G.ncb > 1 ? rec.chi / G.width - rec.clo / G.width + 1 : 1;
        np = (tx1 - tx0 + 1) * (ty1 - ty0 + 1) * nb;
        const int dw = G.nty + 1;
        int* const diff = smem_hist ? s_diff : w.tile_diff + G.diff0;
        atomicAdd(&diff[tx0 * dw + ty0], 1);
        atomicAdd(&diff[tx0 * dw + ty1 + 1], -1);
        atomicAdd(&diff[(tx1 + 1) * dw + ty0], -1);
        atomicAdd(&diff[(tx1 + 1) * dw + ty1 + 1], 1);
        wmax_v = rec.chi - rec.clo;
        my_spec += (unsigned)(rec.chi - rec.clo + 1);
        if (g.form == MG_FORM_F16X3) {
          // magnitude bounds for the scaled FP16 split (non-negative floats
          // order like their bit patterns)
          const KSpec k = g.ks[ks];
          wb_v = __float_as_uint(weight_bound(k.type, rec.inv_h2, k.gnorm));
          float sb = rec.amp;
          if (g.spectral_model == MG_SPECTRUM_TABLE) {
            sb = 0.f;
            for (int c = 0; c < G.nc; ++c) sb = fmaxf(sb, fabsf(G.spectra[p * G.nc + c]));
          }
          sb_v = __float_as_uint(sb);
        }
      }
      w.npairs[P] = np;
    }
    // per-cube maxima: one atomic per warp when its particles share a cube
    const int g0 = __shfl_sync(0xffffffffu, gk, 0);
    if (__all_sync(0xffffffffu, gk == g0)) {
      wmax_v = __reduce_max_sync(0xffffffffu, wmax_v);
      wb_v = __reduce_max_sync(0xffffffffu, wb_v);
      sb_v = __reduce_max_sync(0xffffffffu, sb_v);
      if (lane == 0) {
        if (wmax_v) atomicMax(&w.gst[g0].wmax, wmax_v);
        if (wb_v) atomicMax(&w.gst[g0].wbound_bits, wb_v);
        if (sb_v) atomicMax(&w.gst[g0].sbound_bits, sb_v);
      }
    } else if (valid) {
      if (wmax_v) atomicMax(&w.gst[gk].wmax, wmax_v);
      if (wb_v) atomicMax(&w.gst[gk].wbound_bits, wb_v);
      if (sb_v) atomicMax(&w.gst[gk].sbound_bits, sb_v);
    }
  }
  my_spec = __reduce_add_sync(0xffffffffu, my_spec);
  if (lane == 0) atomicAdd(&s_spec, (unsigned long long)my_spec);
  __syncthreads();
  if (threadIdx.x == 0 && g.spectral_model == MG_SPECTRUM_GAUSSIAN)
    atomicAdd(reinterpret_cast<unsigned long long*>(&w.hdr->spec_bound), s_spec);
  if (smem_hist)
    for (int t = threadIdx.x; t < (int)g.ndiff; t += blockDim.x)
      if (s_diff[t]) atomicAdd(&w.tile_diff[t], s_diff[t]);
}

__global__ void k_tile_init(Geo g, Ws w, long long cap_pairs, long long cap_partial) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < g.ndiff; t += stride)
    w.tile_diff[t] = 0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < g.ngal; k += stride) {
    GalState z;
    z.dec = 0;
    z.wmax = 0;
    z.wbound_bits = z.sbound_bits = z.invw_bits = 0u;
    z.pad_[0] = z.pad_[1] = z.pad_[2] = 0;
    w.gst[k] = z;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    WsHeader* h = w.hdr;
    h->status = 0;
    h->item_counter = 0;
    h->reduce_counter = 0;
    h->n_pairs = h->n_items = h->n_partial_items = h->partial_bound = 0;
    h->cap_pairs = cap_pairs;
    h->cap_partial_items = cap_partial;
    h->spec_bound = 0;
    h->n_spec = 0;
    h->spec_ready = 0;
    h->kch = KCH_MIN;
  }
}

// Channel edges of every cube as double-float pairs, inverse channel widths,
// edge direction and the strict-monotonicity check of
// spectral_models.py:180-187.  Batch-wide edge index e = edge0 + k.
__global__ void k_edges(Geo g, Ws w) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < g.nedge;
       e += (long long)gridDim.x * blockDim.x) {
    const int gk = find_gal(w.ge0, g.ngal, (int)e);
    const Gal& G = w.gal[gk];
    const int k = (int)e - G.edge0;
    const double* ed = G.edges;
    const int dec = ed[G.nc] < ed[0];
    if (k == 0) w.gst[gk].dec = dec;
    const double v = ed[k];
    const float hi = (float)v;
    w.ehi[e] = hi;
    w.elo[e] = (float)(v - (double)hi);
    if (k < G.nc) {
      const float iw = (float)(1.0 / fabs(ed[k + 1] - ed[k]));
      w.inv_w[e] = iw;
      atomicMax(&w.gst[gk].invw_bits, __float_as_uint(iw));
      const bool mono = dec ? (ed[k + 1] < ed[k]) : (ed[k + 1] > ed[k]);
      if (!mono) atomicOr(&w.hdr->status, ST_EDGES);
    } else {
      w.inv_w[e] = 0.f;
    }
  }
}

// One block per cube: exact per-tile counts from the cube's difference array
// (prefix sums along ty, then along tx; in shared memory when it fits in
// `smem_cap` ints, else in place).
__global__ void k_diff_prefix(Geo g, Ws w, int smem_cap) {
  extern __shared__ int s_d[];
  const Gal& G = w.gal[blockIdx.x];
  const int dw = G.nty + 1, dh = G.ntx + 1;
  const int nd = dw * dh;
  const bool in_smem = nd <= smem_cap;
  int* const d = in_smem ? s_d : w.tile_diff + G.diff0;
  const int* src = w.tile_diff + G.diff0;
  if (in_smem)
    for (int e = threadIdx.x; e < nd; e += blockDim.x) s_d[e] = src[e];
  __syncthreads();
  for (int r = threadIdx.x; r < dh; r += blockDim.x) {
    int acc = 0;
    for (int c = 0; c < dw; ++c) {
      acc += d[r * dw + c];
      d[r * dw + c] = acc;
    }
  }
  __syncthreads();
  for (int c = threadIdx.x; c < dw; c += blockDim.x) {
    int acc = 0;
    for (int r = 0; r < dh; ++r) {
      acc += d[r * dw + c];
      d[r * dw + c] = acc;
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < G.ntiles; t += blockDim.x) {
    const int tx = t / G.nty, ty = t - tx * G.nty;
    w.tile_count[G.tile0 + t] = d[tx * dw + ty];
  }
}

// After the scans of the pair counts (total in hdr->n_pairs) and the tile
// counts: the work item size from the total pairs, the split-K bound with it
// (every segment of a tile lists at most the tile's particles, each once)
// and the pair-capacity check.
__global__ void k_plan_finish(Geo g, Ws w, int num_sms) {
  __shared__ long long red[256];
  const long long total = w.hdr->n_pairs;
  const int kch = item_particles(total, num_sms, g.items_per_sm);
  long long sb = 0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < g.ntiles; t += gridDim.x * blockDim.x) {
    const long long cnt = w.tile_off[t + 1] - w.tile_off[t];
    const long long nk = (cnt + kch - 1) / kch;
    if (nk > 1) sb += nk * w.gal[find_gal(w.gt0, g.ngal, t)].ncb;
  }
  red[threadIdx.x] = sb;
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0 && red[0])
    atomicAdd(reinterpret_cast<unsigned long long*>(&w.hdr->partial_bound),
              (unsigned long long)red[0]);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    WsHeader* h = w.hdr;
    h->kch = kch;
    if (total > h->cap_pairs) atomicOr(&h->status, ST_PAIRS);
  }
}

// a / b for 0 <= a < 2^24, b >= 1, from a reciprocal estimate corrected to
// the exact quotient.
__device__ __forceinline__ int div_exact(int a, int b, float rb) {
  int q = (int)(((float)a + 0.5f) * rb);
  int r = a - q * b;
  while (r < 0) {
    --q;
    r += b;
  }
  while (r >= b) {
    ++q;
    r -= b;
  }
  return q;
}

// Pairs in particle order: key = global segment << cbits | class << (cbits -
// 2) | clo, class 0 for the table kernels, 1 for the Dirac kernel, 2 for the
// Gaussian and cubic-spline kernels (each class's particles then form
// stages of their own in each segment, which the tensor-core producers take
// on the class's own path) (one pair per
// tile and channel block the particle's line meets), value = particle.  A
// warp takes 32 particles, whose pairs are one contiguous range of the
// output (pair_off is the exclusive scan of the counts); each lane writes
// every 32nd pair of the range, finding its particle by a search over the
// lanes' first pairs, so every store of the warp is contiguous.  Pair e of
// a particle enumerates its tiles row-major over (tx, ty), then its channel
// blocks, at position pair_off[P] + e.
__global__ void k_emit(Geo g, Ws w, unsigned* __restrict__ keys, int* __restrict__ vals) {
  if (w.hdr->status & (ST_PAIRS | ST_EDGES)) return;
  const int lane = threadIdx.x & 31;
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long base = ((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5) * 32;
       base < g.n; base += nwarps * 32) {
    const long long P = base + lane;
    // this lane's particle: first pair, pair count and the parameters of its
    // tile / block ranges
    long long o = 0x7fffffffffffffffll;  // lanes past the end never match
    int np = 0, tx0 = 0, ty0 = 0, nty_span = 1, cb0 = 0, nb = 1, clo = 0, seg0 = 0, nty = 1,
        ncb = 1;
    unsigned cls = 0u;
    if (P < g.n) {
      o = w.pair_off[P];
      np = w.npairs[P];
      if (np > 0) {
        const PRec rec = w.rec[P];
        const Gal& G = w.gal[find_gal(w.gp0, g.ngal, P)];
        tx0 = rec.ilo / TILE_I;
        ty0 = rec.jlo / TILE_J;
        nty_span = rec.jhi / TILE_J - ty0 + 1;
        cb0 = G.ncb > 1 ? rec.clo / G.width : 0;
        nb = G.ncb > 1 ? rec.chi / G.width - cb0 + 1 : 1;
        clo = rec.clo;
        const int kt = g.ks[rec.kslot].type;
        cls = (kt == MG_KERNEL_GAUSSIAN || kt == MG_KERNEL_CUBIC_SPLINE) ? 2u
              : kt == MG_KERNEL_DIRAC                                     ? 1u
                                                                          : 0u;
        seg0 = G.seg0;
        nty = G.nty;
        ncb = G.ncb;
      }
    }
    const int last = (int)min(31ll, g.n - 1 - base);
    const long long start = __shfl_sync(0xffffffffu, o, 0);
    const long long end = __shfl_sync(0xffffffffu, o + np, last);
    for (long long f0 = start; f0 < end; f0 += 32) {  // warp-uniform
      const long long f = f0 + lane;
      // src = last lane whose first pair is <= f (offsets ascend over lanes;
      // an empty particle shares its offset with the next one)
      int src = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const long long ov = __shfl_sync(0xffffffffu, o, src + step);
        if (ov <= f) src += step;
      }
      const long long so = __shfl_sync(0xffffffffu, o, src);
      const int stx0 = __shfl_sync(0xffffffffu, tx0, src);
      const int sty0 = __shfl_sync(0xffffffffu, ty0, src);
      const int sspan = __shfl_sync(0xffffffffu, nty_span, src);
      const int scb0 = __shfl_sync(0xffffffffu, cb0, src);
      const int snb = __shfl_sync(0xffffffffu, nb, src);
      const int sclo = __shfl_sync(0xffffffffu, clo, src);
      const unsigned scls = __shfl_sync(0xffffffffu, cls, src);
      const int sseg0 = __shfl_sync(0xffffffffu, seg0, src);
      const int snty = __shfl_sync(0xffffffffu, nty, src);
      const int sncb = __shfl_sync(0xffffffffu, ncb, src);
      if (f < end) {
        const int e = (int)(f - so);
        int t = e, cb = scb0;
        if (snb > 1) {
          t = div_exact(e, snb, __frcp_rn((float)snb));
          cb = scb0 + (e - t * snb);
        }
        const int a = div_exact(t, sspan, __frcp_rn((float)sspan));
        const int tx = stx0 + a, ty = sty0 + (t - a * sspan);
        const unsigned sg = (unsigned)(sseg0 + (tx * snty + ty) * sncb + cb);
        keys[f] = (sg << g.cbits) | (scls << (g.cbits - 2)) | (unsigned)sclo;
        vals[f] = (int)(base + src);
      }
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

// One thread per segment (tile, channel block): its range of the sorted
// list (keys segment << cbits | clo, so the segment's particles are exactly
// the keys in [segment << cbits, (segment + 1) << cbits)), its K chunks and
// its split-K partial items.
__global__ void k_segments(Geo g, Ws w) {
  const bool bad = (w.hdr->status & (ST_PAIRS | ST_EDGES)) != 0;
  const int kch = w.hdr->kch;
  const long long n = w.hdr->n_pairs;
  for (int sg = blockIdx.x * blockDim.x + threadIdx.x; sg < g.nseg; sg += gridDim.x * blockDim.x) {
    long long lo = 0, hi = 0;
    int items = 0, part = 0;
    if (!bad && n > 0) {
      lo = lower_bound_keys(w.keys, 0, n, (unsigned)sg << g.cbits);
      hi = sg + 1 == g.nseg ? n
                            : lower_bound_keys(w.keys, lo, n, (unsigned)(sg + 1) << g.cbits);
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

// Work-queue keys: one thread per segment writes the keys of its items
// (item k of a segment holds min(kch, cnt - k kch) particles).  Estimated
// cost = particles x (2 TILE_PX + width): the kernel weights at the tile's
// pixels and the spectra and products over the segment's channel block.
// Key = 65535 - cost scaled to 16 bits, so that the stable ascending radix
// sort puts the largest items first and keeps segment order among equal
// ones: the persistent contraction then ends on the small items instead of
// leaving one large item to a single SM at the end.
__global__ void k_item_keys(Geo g, Ws w) {
  if (w.hdr->status & (ST_PAIRS | ST_EDGES)) return;
  const int kch = w.hdr->kch;
  const double cmax = (double)kch * (2.0 * TILE_PX + (double)g.max_width);
  for (int sg = blockIdx.x * blockDim.x + threadIdx.x; sg < g.nseg; sg += gridDim.x * blockDim.x) {
    const int n_it = w.seg_items[sg];
    if (n_it == 0) continue;
    const long long base = w.item_off[sg];
    const long long cnt = w.seg_hi[sg] - w.seg_lo[sg];
    const int width = w.gal[find_gal(w.gs0, g.ngal, sg)].width;
    for (int k = 0; k < n_it && base + k < w.cap_items; ++k) {
      const long long left = cnt - (long long)k * kch;
      const double lc = (double)(left < kch ? left : kch);
      double q = lc * (2.0 * TILE_PX + (double)width) / cmax * 65535.0 + 0.5;
      if (q > 65535.0) q = 65535.0;
      // all keys equal: the stable sort keeps segment order
      w.item_key[base + k] = g.cost_order ? 65535u - (unsigned)q : 0u;
      w.item_order[base + k] = (int)(base + k);
      w.item_seg[base + k] = sg;
    }
  }
}

__global__ void k_check_partials(Ws w) {
  WsHeader* h = w.hdr;
  if (h->n_partial_items > h->cap_partial_items) h->status |= ST_PARTIALS;
}

static unsigned grid_for(long long n, int num_sms) {
  long long blocks = (n + 255) / 256;
  if (blocks > (long long)num_sms * 32) blocks = (long long)num_sms * 32;
  return (unsigned)(blocks > 0 ? blocks : 1);
}

// Records, tile histograms, per-particle pair offsets and the tile plan.
void launch_prep(const Geo& g, const Ws& w, int num_sms, cudaStream_t s, long long cap_pairs,
                 long long cap_partial) {
  long long init_n = g.ndiff > g.ntiles ? g.ndiff : g.ntiles;
  if (g.ngal > init_n) init_n = g.ngal;
  k_tile_init<<<grid_for(init_n, num_sms), 256, 0, s>>>(g, w, cap_pairs, cap_partial);
  k_edges<<<grid_for(g.nedge, num_sms), 256, 0, s>>>(g, w);
  if (g.n > 0) {
    // with the histogram in shared memory every block flushes the array:
    // fewer, longer-lived blocks
    const bool smem_hist = g.ngal == 1 && g.ndiff <= PREP_SMEM_DIFF;
    const size_t hist_bytes = smem_hist ? sizeof(int) * (size_t)g.ndiff : 0;
    unsigned blocks = grid_for(g.n, num_sms);
    const unsigned per_sm = hist_bytes <= 16384 ? 8u : 4u;
    if (smem_hist && blocks > per_sm * (unsigned)num_sms) blocks = per_sm * (unsigned)num_sms;
    k_prep<<<blocks, PREP_THREADS, hist_bytes, s>>>(g, w);
  }
  launch_scan(w.npairs, g.n, w.pair_off, w.scan_sums, &w.hdr->n_pairs, s);
  // per-cube prefix sums of the difference arrays, in up to 200 KB of
  // dynamic shared memory (the attribute is per device: set on every launch)
  constexpr int kPlanSmemCap = 50 * 1024;
  int cap = g.max_diff <= kPlanSmemCap ? g.max_diff : 0;
  if (cap > 12 * 1024 &&
      cudaFuncSetAttribute(k_diff_prefix, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(sizeof(int) * kPlanSmemCap)) != cudaSuccess) {
    cudaGetLastError();  // fall back to the in-place prefix sums
    cap = 0;
  }
  k_diff_prefix<<<g.ngal, 256, sizeof(int) * (size_t)cap, s>>>(g, w, cap);
  launch_scan(w.tile_count, g.ntiles, w.tile_off, w.scan_sums, w.tile_off + g.ntiles, s);
  k_plan_finish<<<grid_for(g.ntiles, num_sms), 256, 0, s>>>(g, w, num_sms);
}

int sort_bits(const Geo& g) {
  int sbits = 0;
  while ((1LL << sbits) < (long long)g.nseg) ++sbits;
  return sbits + g.cbits;
}

// Tile-major list sorted by (tile, clo), then the segments with their
// work-item and partial offsets.  Pairs are emitted into the buffer from
// which an even/odd number of radix passes ends in w.keys / w.list.
void launch_sort_segments(const Geo& g, const Ws& w, long long cap_pairs, int num_sms,
                          cudaStream_t s) {
  const int passes = (sort_bits(g) + 7) / 8;
  unsigned* k0 = (passes & 1) ? w.keys_tmp : w.keys;
  int* v0 = (passes & 1) ? w.list_tmp : w.list;
  unsigned* k1 = (passes & 1) ? w.keys : w.keys_tmp;
  int* v1 = (passes & 1) ? w.list : w.list_tmp;
  if (g.n > 0) k_emit<<<grid_for(g.n, num_sms), 256, 0, s>>>(g, w, k0, v0);
  launch_radix_sort(k0, v0, k1, v1, &w.hdr->n_pairs, cap_pairs, sort_bits(g), w.rs_hist,
                    w.rs_off, w.scan_sums, num_sms, s);
  k_segments<<<(unsigned)((g.nseg + 255) / 256), 256, 0, s>>>(g, w);
  launch_scan(w.seg_items, g.nseg, w.item_off, w.scan_sums, &w.hdr->n_items, s);
  launch_scan(w.seg_part, g.nseg, w.part_off, w.scan_sums, &w.hdr->n_partial_items, s);
  // the work queue: items by estimated cost, largest first (16-bit keys: two
  // radix passes, the result back in item_key / item_order)
  k_item_keys<<<(unsigned)((g.nseg + 255) / 256), 256, 0, s>>>(g, w);
  launch_radix_sort(w.item_key, w.item_order, w.item_key_tmp, w.item_order_tmp, &w.hdr->n_items,
                    w.cap_items, 16, w.rs_hist, w.rs_off, w.scan_sums, num_sms, s);
  k_check_partials<<<1, 1, 0, s>>>(w);
}

}  // namespace mg
