// Plain FP32 contraction: for each work item (tile, particle chunk, channel
// block) the CTA builds W[32 particles][128 pixels] and S[32][64 channels] in
// shared memory and accumulates out[128][64] += W^T S on CUDA cores.
//
// This is the per-pixel sum of martini/martini.py:243-283 reorganised around
// output tiles: a pixel's spectrum is the sum over the particles whose
// footprint box contains it of weight * spectrum.
#include "mg_internal.cuh"

namespace mg {

constexpr int F32_THREADS = 256;
constexpr int F32_KC = 32;  // particles per shared-memory chunk
constexpr int F32_MASTER_BYTES = 32 * F32_THREADS * 4;  // master accumulators (dynamic)

struct ItemInfo {
  int seg, gal, tile, tx, ty, kc, nk;  // tile: within the cube
  int c0;            // first channel of this item's block
  long long lbeg;    // particle list range
  int lcount;
};

__device__ __forceinline__ ItemInfo decode_item(const Geo& g, const Ws& w, long long item,
                                                int kch) {
  ItemInfo it;
  const int sg = w.item_seg[item];
  it.seg = sg;
  it.gal = find_gal(w.gs0, g.ngal, sg);
  const Gal& G = w.gal[it.gal];
  const int ls = sg - G.seg0;
  it.tile = ls / G.ncb;
  const int cb = ls - it.tile * G.ncb;
  it.tx = it.tile / G.nty;
  it.ty = it.tile - it.tx * G.nty;
  it.nk = w.seg_items[sg];
  it.kc = (int)(item - w.item_off[sg]);
  it.c0 = cb * G.width;
  it.lbeg = w.seg_lo[sg] + (long long)it.kc * kch;
  const long long left = w.seg_hi[sg] - it.lbeg;
  it.lcount = (int)(left < kch ? left : kch);
  return it;
}

__global__ void __launch_bounds__(F32_THREADS, 2)
k_contract_fp32(Geo g, Ws w) {
  __shared__ __align__(16) float Ws_[F32_KC][TILE_PX];
  __shared__ __align__(16) float Ss_[F32_KC][CBLK];
  // Master accumulator: each F32_KC-particle chunk is summed from zero in
  // registers and added here (round to nearest).  One running FP32 sum over
  // an item's particles (up to ~10^6 on a dense tile) drops every product
  // below half an ulp of the sum, a loss that only grows with the count; a
  // chunk sum of 32 products meets the master far less often.  Laid out
  // [value][thread] in dynamic shared memory (F32_MASTER_BYTES): each
  // thread's slots are conflict-free.
  extern __shared__ float Ms_dyn[];
  float(*Ms_)[F32_THREADS] = reinterpret_cast<float(*)[F32_THREADS]>(Ms_dyn);
  __shared__ PRec recs[F32_KC];
  __shared__ int s_pid[F32_KC];
  __shared__ KSpec s_ks[MG_MAX_KERNELS];
  __shared__ long long s_item;

  const int tid = threadIdx.x;
  if (tid < MG_MAX_KERNELS) s_ks[tid] = g.ks[tid];
  const WsHeader* hdr = w.hdr;
  if (hdr->status) return;
  const long long n_items = hdr->n_items;
  const int kch = hdr->kch;
  const int tr = tid >> 4;  // pixel group: pixels tr*8 .. tr*8+7
  const int tc = tid & 15;  // channel group: channels tc*4 .. tc*4+3

  for (;;) {
    if (tid == 0) s_item = (long long)atomicAdd(&w.hdr->item_counter, 1u);
    __syncthreads();
    const long long item = s_item;
    __syncthreads();
    if (item >= n_items) break;
    // the queue runs over the items in cost order, largest first
    const ItemInfo it = decode_item(g, w, (long long)w.item_order[item], kch);
    const Gal& G = w.gal[it.gal];
    const int dec = w.gst[it.gal].dec;
    const int nc = G.nc;
    const float* ehi = w.ehi + G.edge0;
    const float* elo = w.elo + G.edge0;
    const float* inv_w = w.inv_w + G.edge0;
    const int i0 = it.tx * TILE_I, j0 = it.ty * TILE_J;

    float acc[8][4];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = 0.f;
#pragma unroll
    for (int v = 0; v < 32; ++v) Ms_[v][tid] = 0.f;

    for (int k0 = 0; k0 < it.lcount; k0 += F32_KC) {
      const int kn = min(F32_KC, it.lcount - k0);
      if (tid < F32_KC) {
        if (tid < kn) {
          int pid = w.list[it.lbeg + k0 + tid];
          recs[tid] = w.rec[pid];
          s_pid[tid] = pid;
        } else {
          PRec z;
          z.ilo = 0; z.ihi = -1; z.jlo = 0; z.jhi = -1; z.clo = 1; z.chi = 0;
          z.kslot = 0; z.flags = 0;
          recs[tid] = z;
          s_pid[tid] = 0;
        }
      }
      __syncthreads();
      {
        // W: particle q, tile row ii (16 pixels along j)
        const int q = tid >> 3, ii = tid & 7;
        const PRec r = recs[q];
        const int i = i0 + ii;
        // a particle listed for this block whose line misses it (the list
        // bound is conservative) contributes nothing: no weights
        const bool hit = r.chi >= it.c0 && r.clo < it.c0 + CBLK;
#pragma unroll 4
        for (int jj = 0; jj < TILE_J; ++jj)
          Ws_[q][ii * TILE_J + jj] = hit ? pixel_weight(r, s_ks, i, j0 + jj) : 0.f;
        // S: particle q, channels c0 + ii*8 .. +7
        for (int cc = ii * 8; cc < ii * 8 + 8; ++cc) {
          const int c = it.c0 + cc;
          float s = 0.f;
          if (c < nc && q < kn) {
            if (g.spectral_model == MG_SPECTRUM_TABLE) {
              s = G.spectra[((long long)s_pid[q] - G.p0) * nc + c];
            } else {
              s = channel_spectrum(r, g.spectral_model, c, dec, ehi, elo, inv_w);
            }
          }
          Ss_[q][cc] = s;
        }
      }
      __syncthreads();
#pragma unroll 8
      for (int k = 0; k < F32_KC; ++k) {
        const float4 wa = *reinterpret_cast<const float4*>(&Ws_[k][tr * 8]);
        const float4 wb = *reinterpret_cast<const float4*>(&Ws_[k][tr * 8 + 4]);
        const float4 s = *reinterpret_cast<const float4*>(&Ss_[k][tc * 4]);
        const float wv[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
#pragma unroll
        for (int a = 0; a < 8; ++a) {
          acc[a][0] = fmaf(wv[a], s.x, acc[a][0]);
          acc[a][1] = fmaf(wv[a], s.y, acc[a][1]);
          acc[a][2] = fmaf(wv[a], s.z, acc[a][2]);
          acc[a][3] = fmaf(wv[a], s.w, acc[a][3]);
        }
      }
      // chunk sum into the master, registers back to zero
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          Ms_[a * 4 + b][tid] += acc[a][b];
          acc[a][b] = 0.f;
        }
      __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = Ms_[a * 4 + b][tid];

    // epilogue: direct cube write (single K chunk) or split-K partial
    if (it.nk == 1) {
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        const int px = tr * 8 + a;
        const int i = i0 + px / TILE_J, j = j0 + px % TILE_J;
        if (i >= G.nx || j >= G.ny) continue;
        float* dst = G.cube + ((long long)i * G.ny + j) * nc;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int c = it.c0 + tc * 4 + b;
          if (c < nc) dst[c] = g.accumulate ? dst[c] + acc[a][b] : acc[a][b];
        }
      }
    } else {
      const long long slot = w.part_off[it.seg] + it.kc;
      float* dst = w.partial + slot * (long long)(TILE_PX * g.max_width);
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        const int px = tr * 8 + a;
        *reinterpret_cast<float4*>(&dst[px * CBLK + tc * 4]) =
            make_float4(acc[a][0], acc[a][1], acc[a][2], acc[a][3]);
      }
    }
  }
}

// Split-K reduction, shared by every form: a segment with nk > 1 work items
// left nk partial rows of TILE_PX x seg_width floats (pixel-major).  One
// block per (segment, chunk of RED_CHUNK floats): each thread sums four
// channels of one pixel over the rows in ascending row order, so the result
// does not depend on scheduling, with RED_ROWS float4 loads in flight.
constexpr int RED_THREADS = 256;
constexpr int RED_CHUNK = RED_THREADS * 4;
constexpr int RED_ROWS = 8;

__global__ void __launch_bounds__(RED_THREADS) k_reduce_partials(Geo g, Ws w) {
  if (w.hdr->status) return;
  const long long slot = (long long)TILE_PX * g.max_width;  // floats per partial row
  const int nchunk = (int)((slot + RED_CHUNK - 1) / RED_CHUNK);
  const long long units = (long long)g.nseg * nchunk;
  for (long long u = blockIdx.x; u < units; u += gridDim.x) {
    const int sg = (int)(u / nchunk);
    const int nk = w.seg_part[sg];
    if (nk == 0) continue;
    const int gk = find_gal(w.gs0, g.ngal, sg);
    const Gal& G = w.gal[gk];
    const int width = G.width;  // a multiple of 16 channels
    const int per_row = TILE_PX * width;
    const int e = (int)(u - (long long)sg * nchunk) * RED_CHUNK + threadIdx.x * 4;
    if (e >= per_row) continue;
    const float4* src =
        reinterpret_cast<const float4*>(w.partial + w.part_off[sg] * slot + e);
    const long long row4 = slot / 4;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k0 = 0; k0 < nk; k0 += RED_ROWS) {
      float4 v[RED_ROWS];
#pragma unroll
      for (int q = 0; q < RED_ROWS; ++q)
        if (k0 + q < nk) v[q] = __ldcs(src + (long long)(k0 + q) * row4);
#pragma unroll
      for (int q = 0; q < RED_ROWS; ++q)
        if (k0 + q < nk) {
          acc.x += v[q].x;
          acc.y += v[q].y;
          acc.z += v[q].z;
          acc.w += v[q].w;
        }
    }
    const int ls = sg - G.seg0;
    const int t = ls / G.ncb;
    const int cb = ls - t * G.ncb;
    const int tx = t / G.nty, ty = t - tx * G.nty;
    const int px = e / width, c = cb * width + (e - px * width);
    const int i = tx * TILE_I + px / TILE_J, j = ty * TILE_J + px % TILE_J;
    if (i >= G.nx || j >= G.ny) continue;
    const int nc = G.nc;
    float* dst = G.cube + ((long long)i * G.ny + j) * nc + c;
    if (g.accumulate) {
      if (c < nc) acc.x += dst[0];
      if (c + 1 < nc) acc.y += dst[1];
      if (c + 2 < nc) acc.z += dst[2];
      if (c + 3 < nc) acc.w += dst[3];
    }
    if (c < nc) dst[0] = acc.x;
    if (c + 1 < nc) dst[1] = acc.y;
    if (c + 2 < nc) dst[2] = acc.z;
    if (c + 3 < nc) dst[3] = acc.w;
  }
}

void launch_reduce_partials(const Geo& g, const Ws& w, int num_sms, cudaStream_t s) {
  k_reduce_partials<<<num_sms * 8, RED_THREADS, 0, s>>>(g, w);
}

// Flux sums over the unpadded region (martini/martini.py:367-392), in a
// fixed order: per pixel row (one block per row of the unpadded region, a
// thread per channel) in double-float, then the row sums in FP64 in row
// order.
constexpr int FLUX_ROWS = 1;  // pixel rows (axis 0) per chunk

// Double-float running sum (Knuth's TwoSum): hi carries the FP32 sum and lo
// the rounding errors of its additions, so hi + lo is the sum to ~n eps^2
// without FP64 arithmetic (FP64 units are few on this part).
struct DFloat {
  float hi, lo;
};

__device__ __forceinline__ void df_add(DFloat& a, float x) {
  const float t = __fadd_rn(a.hi, x);
  const float bp = __fadd_rn(t, -a.hi);
  const float e = __fadd_rn(__fadd_rn(a.hi, -__fadd_rn(t, -bp)), __fadd_rn(x, -bp));
  a.hi = t;
  a.lo = __fadd_rn(a.lo, e);
}

// Sum of one pixel row's voxels of channel c (stride nc), j in [j0, j1), in
// a fixed order: four interleaved double-float sums combined in FP64.
__device__ __forceinline__ double row_sum(const float* row, int j0, int j1, int nc) {
  DFloat a[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  int j = j0;
  for (; j + 4 <= j1; j += 4) {
    float x[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) x[u] = __ldcs(row + (long long)(j + u) * nc);
#pragma unroll
    for (int u = 0; u < 4; ++u) df_add(a[u], x[u]);
  }
  for (; j < j1; ++j) df_add(a[0], __ldcs(row + (long long)j * nc));
  double acc = 0.0;
#pragma unroll
  for (int u = 0; u < 4; ++u) acc += (double)a[u].hi + (double)a[u].lo;
  return acc;
}

__global__ void k_flux_partial(const float* __restrict__ cube, int nx, int ny, int nc, int padx,
                               int pady, double* __restrict__ part) {
  const int chunk = blockIdx.x;
  const int i0 = padx + chunk * FLUX_ROWS;
  const int i1 = min(nx - padx, i0 + FLUX_ROWS);
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    double acc = 0.0;
    for (int i = i0; i < i1; ++i) acc += row_sum(cube + ((long long)i * ny) * nc + c, pady, ny - pady, nc);
    part[(long long)chunk * nc + c] = acc;
  }
}

__global__ void k_flux_final(const double* __restrict__ part, int nchunks, int nc,
                             double* __restrict__ flux) {
  __shared__ double red[1024];
  double tot = 0.0;
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < nchunks; ++k) s += part[(long long)k * nc + c];
    flux[1 + c] = s;
    tot += s;
  }
  red[threadIdx.x] = tot;
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) flux[0] = red[0];
}

int flux_chunks(int nx, int padx) {
  int rows = nx - 2 * padx;
  if (rows < 1) rows = 1;
  return (rows + FLUX_ROWS - 1) / FLUX_ROWS;
}

void launch_flux(const float* cube, int nx, int ny, int nc, int padx, int pady, double* part,
                 double* flux, cudaStream_t s) {
  const int nch = flux_chunks(nx, padx);
  const int thr = nc < 256 ? ((nc + 31) / 32) * 32 : 256;
  k_flux_partial<<<nch, thr, 0, s>>>(cube, nx, ny, nc, padx, pady, part);
  k_flux_final<<<1, 1024, 0, s>>>(part, nch, nc, flux);
}

int launch_contract_fp32(const Geo& g, const Ws& w, int num_sms, cudaStream_t s) {
  // the dynamic shared-memory attribute is per device: set once on each
  // (host-side, before a graph capture by the first insertion on a device)
  constexpr int kMaxDev = 64;
  static bool attr_set[kMaxDev] = {false};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return MG_ERR_CUDA;
  if (!attr_set[dev]) {
    if (cudaFuncSetAttribute(k_contract_fp32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             F32_MASTER_BYTES) != cudaSuccess)
      return MG_ERR_CUDA;
    attr_set[dev] = true;
  }
  k_contract_fp32<<<num_sms * 2, F32_THREADS, F32_MASTER_BYTES, s>>>(g, w);
  launch_reduce_partials(g, w, num_sms, s);
  return MG_OK;
}

// Flux sums of every cube of a batch: one block per unpadded pixel row of
// all cubes, a thread per channel adding the row's voxels in a fixed order
// (four interleaved double-float sums, combined in FP64), then per cube and
// channel eight row groups (rows r = g mod 8) summed in FP64 and combined in
// group order, and one block per cube adding the channels.
__global__ void k_flux_rows(Geo g, Ws w) {
  const int gk = find_gal(w.gr0, g.ngal, (int)blockIdx.x);
  const Gal& G = w.gal[gk];
  if (!G.flux) return;
  const int r = blockIdx.x - G.row0;
  const int i = G.padx + r;
  const int nc = G.nc;
  const int j1 = G.ny - G.pady;
  for (int c = threadIdx.x; c < nc; c += blockDim.x)
    w.flux_part[G.fpart0 + (long long)r * nc + c] =
        row_sum(G.cube + ((long long)i * G.ny) * nc + c, G.pady, j1, nc);
}

constexpr int FLUX_CH = 32;  // channels per block of k_flux_channels
constexpr int FLUX_RG = 8;   // row groups per block: rows r = g (mod FLUX_RG)

__global__ void __launch_bounds__(FLUX_CH * FLUX_RG) k_flux_channels(Geo g, Ws w) {
  __shared__ double part[FLUX_RG][FLUX_CH];
  const Gal& G = w.gal[blockIdx.y];
  if (!G.flux) return;
  const int cl = threadIdx.x % FLUX_CH, rg = threadIdx.x / FLUX_CH;
  const int c = blockIdx.x * FLUX_CH + cl;
  const int rows = G.nx - 2 * G.padx;
  double s = 0.0;
  if (c < G.nc)
    for (int r = rg; r < rows; r += FLUX_RG) s += w.flux_part[G.fpart0 + (long long)r * G.nc + c];
  part[rg][cl] = s;
  __syncthreads();
  if (rg == 0 && c < G.nc) {
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < FLUX_RG; ++k) t += part[k][cl];
    G.flux[1 + c] = t;
  }
}

__global__ void k_flux_cubes(Geo g, Ws w) {
  __shared__ double red[256];
  const Gal& G = w.gal[blockIdx.x];
  if (!G.flux) return;
  double tot = 0.0;
  for (int c = threadIdx.x; c < G.nc; c += blockDim.x) tot += G.flux[1 + c];
  red[threadIdx.x] = tot;
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) G.flux[0] = red[0];
}

void launch_flux_batch(const Geo& g, const Ws& w, cudaStream_t s) {
  if (g.nrows <= 0) return;
  const int thr = g.max_nc < 256 ? ((g.max_nc + 31) / 32) * 32 : 256;
  k_flux_rows<<<g.nrows, thr, 0, s>>>(g, w);
  k_flux_channels<<<dim3((unsigned)((g.max_nc + FLUX_CH - 1) / FLUX_CH), (unsigned)g.ngal),
                    FLUX_CH * FLUX_RG, 0, s>>>(g, w);
  k_flux_cubes<<<g.ngal, 256, 0, s>>>(g, w);
}

}  // namespace mg
