// Internal device-side definitions shared by the martini_gb300 kernels.
//
// Cube tiles are TILE_I x TILE_J pixels (128 pixels: one tensor-core M tile)
// and contraction channel blocks are CBLK channels.  Particles are binned by
// the tiles their footprint box touches; each (tile, particle-chunk,
// channel-block) is one work item of the contraction kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/martini_gb300.h"
#include "mg_kernel_tables.h"

namespace mg {

constexpr int TILE_I = 8;    // pixels along axis 0 (RA index)
constexpr int TILE_J = 16;   // pixels along axis 1 (Dec index)
constexpr int TILE_PX = TILE_I * TILE_J;
constexpr int CBLK = 64;     // channels per FP32 work item
constexpr int KCH_MIN = 2048;     // fewest particles per work item (split-K granularity)
constexpr int ITEMS_PER_SM = 24;  // default target work items per SM when the pairs allow

// Particles per work item for a launch with `total_pairs` (tile, particle)
// pairs: about `items_per_sm` items per SM (1 .. ITEMS_PER_SM; the plan's
// split-K bound holds for every value up to the default), a multiple of 64,
// at least KCH_MIN.  Small problems keep fine items for load balance; large
// ones get items long enough that split-K partial tiles stay few.
__host__ __device__ inline int item_particles(long long total_pairs, int num_sms,
                                              int items_per_sm = ITEMS_PER_SM) {
  if (items_per_sm < 1 || items_per_sm > ITEMS_PER_SM) items_per_sm = ITEMS_PER_SM;
  const long long per = (long long)(num_sms > 0 ? num_sms : 1) * items_per_sm;
  long long t = (total_pairs + per - 1) / per;
  t = (t + 63) / 64 * 64;
  if (t < KCH_MIN) t = KCH_MIN;
  if (t > (1LL << 30)) t = 1LL << 30;
  return (int)t;
}

// Per-particle record written by the prep kernel (64 bytes).
struct PRec {
  int ilo, ihi, jlo, jhi;  // exact footprint box (inclusive), clipped; empty if ilo > ihi
  int xi, yi;              // floor(x), floor(y)
  float xf, yf;            // x - xi, y - yi in [0, 1)
  float h;                 // sm_length * rescale, px
  float inv_h2;            // 1 / h^2
  int kslot;               // resolved kernel table slot
  int clo, chi;            // channel support, inclusive; empty if clo > chi
  float vhi, vlo;          // velocity as a double-float pair, km/s
  float inv_s;             // 1 / (sqrt(2) sigma), km/s^-1
  float amp;               // mHI / D^2 / 2.36e5
  int flags;               // PREC_* bits
};

// The footprint's rows [ilo, ihi] hold every cube row within the kernel's
// support radius h of the particle (tested in FP64 with a 2^-20 margin, so
// the FP32 profile argument of any other row is past the support): a radial
// table kernel needs no per-row box test.
constexpr int PREC_ROWS_COVER = 1;
// The same for the footprint's columns [jlo, jhi] (axis 1).
constexpr int PREC_COLS_COVER = 2;

// Per-particle parameters of the tensor-core producers (64 bytes), written
// once per insertion by k_tc_params: the particle's position, the weight
// constants of its kernel with the cube's operand scale applied, its kind,
// footprint box, channel support and spectrum-store row.  The contraction
// copies one per tile visit (four 16-byte cp.async) and derives only the
// tile-relative fields.
struct TcPar {
  int xi, yi;              // floor(x), floor(y)
  float xf, yf;            // x - xi, y - yi
  float k2;                // table kernels: inv_h2 * cells per unit s; cubic spline: 4 inv_h2;
                           // Gaussian: 1 / (h sigma)
  float scale;             // weight scale with the cube's operand scale
  int kind;                // producer kind and flags, kernel slot << 8, type << 12 (0: none)
  int clo;                 // channel support [clo, chi]
  int ilo, ihi, jlo, jhi;  // footprint box (clipped to the cube)
  int chi;
  int pad_;
  long long soff;          // spectrum-store row of the particle
};
static_assert(sizeof(TcPar) == 64, "four 16-byte pieces");

struct KSpec {
  int type;
  float truncate;
  float gnorm;       // Gaussian truncation normalisation
  float pad_;
};

// One cube of a batch (mg_insert is a batch of one).  Written into the
// workspace by k_set_gals from kernel parameters, so an insertion needs no
// host-to-device copy and can be captured in a CUDA graph.  Offsets place the
// cube's particles, tiles, segments, edges and flux rows in the batch-wide
// arrays.
struct Gal {
  const double* x;
  const double* y;
  const double* r;
  const float* h;
  const int8_t* kidx;
  const double* v;
  const float* sigma;
  const double* amp;
  const float* spectra;
  const double* edges;
  float* cube;
  double* flux;
  long long p0;       // first particle in the batch
  long long n;        // particles
  long long diff0;    // first entry of the tile difference array
  long long fpart0;   // first FP64 flux partial (flux rows x nc)
  int nx, ny, nc, padx, pady;
  int ntx, nty, ntiles;
  int tile0;          // first global tile
  int seg0;           // first global segment
  int ncb, width;     // channel blocks per tile and channels per block
  int edge0;          // first channel edge (nc + 1 per cube)
  int row0;           // first flux row (unpadded rows of the cubes before)
  float sigma_const;
  int pad_;
};

// Per-cube values the kernels find on the device (reset by k_tile_init).
struct GalState {
  int dec;                 // channel edges decrease with index
  int wmax;                // max (chi - clo) over the cube's particles
  unsigned wbound_bits;    // max pixel weight bound (float bits, >= 0)
  unsigned sbound_bits;    // max spectrum bound (float bits, >= 0)
  unsigned invw_bits;      // max 1 / |channel width| (float bits)
  int pad_[3];
};

// Batch-wide constants (kernel parameters).  Every cube of a batch shares
// the kernel table, spectral model, contraction form and accumulate flag.
struct Geo {
  int ngal;
  int n_kernels;
  int spectral_model;
  int form;
  int accumulate;     // add into the cubes instead of overwriting them
  int ntiles;         // tiles of all cubes
  int nseg;           // segments of all cubes
  int max_width;      // widest channel block (partial slots hold TILE_PX x max_width)
  int max_nc;
  int cbits;          // key bits below the segment: two kernel-class bits, then the
                      // channel bits of the widest band
  int nrows;          // flux rows of all cubes
  int max_diff;       // largest difference array of one cube
  long long n;        // particles of all cubes
  long long ndiff;    // difference-array entries of all cubes
  long long nedge;    // channel edges of all cubes
  long long nfpart;   // FP64 flux partials of all cubes
  KSpec ks[MG_MAX_KERNELS];
  // launch shape (mg_tuning): particles per tensor-core stage (0: the
  // form's default), work items per SM, cost-ordered work queue
  int kc;
  int items_per_sm;
  int cost_order;
  int pad_tuning;
};

// Cube of a batch-wide index: the largest k < ngal with keys[k] <= v (cubes
// with no particles share their successor's start, and are skipped).
template <typename T>
__device__ __forceinline__ int find_gal(const T* keys, int ngal, T v) {
  int a = 0, b = ngal;
  while (b - a > 1) {
    const int m = (a + b) >> 1;
    if (keys[m] <= v) a = m; else b = m;
  }
  return a;
}

// Status bits of WsHeader::status.
constexpr unsigned ST_PAIRS = 1u;        // pairs exceed the list capacity
constexpr unsigned ST_PARTIALS = 2u;     // split-K partials exceed capacity
constexpr unsigned ST_EDGES = 4u;        // channel edges not strictly monotonic
constexpr unsigned ST_TIMEOUT = 8u;      // a bounded device-side wait expired

// Workspace header (device): status flags and scalar counters.
struct WsHeader {
  unsigned int status;           // ST_* bits
  unsigned int item_counter;     // dynamic scheduler cursor
  unsigned int reduce_counter;
  int pad0;
  long long n_pairs;
  long long n_items;
  long long n_partial_items;
  long long partial_bound;       // upper bound on partial items (from tile counts)
  long long cap_pairs;
  long long cap_partial_items;
  long long spec_bound;          // sum over particles of support channels (Gaussian)
  long long n_spec;              // values in the spectrum store (spectrum stage)
  int spec_ready;                // 1 once the store holds this binning's spectra
  int kch;                       // particles per work item (item_particles)
  long long pad1[1];
};

// Pointers into the workspace (host computes, passes by value).  Arrays run
// over the whole batch.  A "segment" is one (tile, channel block) of the
// contraction: Gal::ncb blocks per tile (FP32 form: ceil(nc / CBLK) blocks
// of CBLK channels; tensor-core forms: the band rounded to 16 in one block up
// to 256 channels, else blocks of 256).
struct Ws {
  WsHeader* hdr;
  Gal* gal;              // [ngal]
  GalState* gst;         // [ngal]
  long long* gp0;        // [ngal + 1] first particle of each cube
  int* gt0;              // [ngal + 1] first tile
  int* gs0;              // [ngal + 1] first segment
  int* ge0;              // [ngal + 1] first edge
  int* gr0;              // [ngal + 1] first flux row
  PRec* rec;             // [n]
  TcPar* tpar;           // [n] tensor-core forms only (else null)
  int* npairs;           // [n] tiles touched per particle
  long long* pair_off;   // [n] exclusive scan of npairs
  int* tile_count;       // [ntiles]
  int* tile_diff;        // [ndiff] per cube (ntx + 1) x (nty + 1) difference arrays
  long long* tile_off;   // [ntiles + 1] pair offsets (tile-major sorted list)
  float* ehi;            // [nedge] edges, double-float high part
  float* elo;            // [nedge] low part
  float* inv_w;          // [nedge] 1 / |channel width| (channel c of a cube at edge0 + c)
  unsigned* keys;        // [cap_pairs] sorted keys: segment << cbits | class | clo
  int* list;             // [cap_pairs] particle ids in sorted order
  unsigned* keys_tmp;    // [cap_pairs] radix-sort second buffer
  int* list_tmp;         // [cap_pairs]
  int* rs_hist;          // [256 * radix_blocks(cap_pairs)]
  long long* rs_off;     // [256 * radix_blocks(cap_pairs)]
  long long* scan_sums;  // [scan scratch]
  long long* seg_lo;     // [nseg] list range of each segment
  long long* seg_hi;     // [nseg]
  int* seg_items;        // [nseg] work items (K chunks) of each segment
  int* seg_part;         // [nseg] partial items of each segment
  long long* item_off;   // [nseg] exclusive scan of seg_items
  long long* part_off;   // [nseg] exclusive scan of seg_part
  float* partial;        // [cap_partial_items][TILE_PX][max_width]
  double* flux_part;     // [nfpart]
  unsigned* spec;        // [cap_spec] per-particle Gaussian spectra over [clo, chi], as the
                         // tensor-core form's scaled 16-bit hi | lo << 16 halves
  long long cap_spec;    // room in spec (the workspace beyond the fixed layout)
  // Work queue order: item_order[k] is the k-th item the contraction takes,
  // the items sorted by estimated cost, largest first (stable: equal costs
  // keep segment order).  item_key / item_*_tmp are the sort's buffers.
  int* item_order;       // [cap_items]
  unsigned* item_key;    // [cap_items]
  unsigned* item_key_tmp;
  int* item_order_tmp;
  int* item_seg;         // [cap_items] segment of each item (in item index order)
  long long cap_items;
};

// Upper bound on the work items of a binning with at most cap_pairs pairs:
// every item holds at least one pair, and a segment of cnt pairs has
// ceil(cnt / kch) <= 1 + cnt / KCH_MIN items.
__host__ __device__ inline long long items_bound(long long nseg, long long cap_pairs) {
  const long long b = nseg + cap_pairs / KCH_MIN + 1;
  return cap_pairs < b ? cap_pairs : b;
}

// Host-side launchers (all asynchronous on stream s).
void launch_set_gals(const Gal* gals, const Geo& g, const Ws& w, cudaStream_t s);
void launch_prep(const Geo& g, const Ws& w, int num_sms, cudaStream_t s, long long cap_pairs,
                 long long cap_partial);
void launch_sort_segments(const Geo& g, const Ws& w, long long cap_pairs, int num_sms,
                          cudaStream_t s);
int sort_bits(const Geo& g);
void launch_scan(const int* in, long long n, long long* out, long long* sums, long long* total,
                 cudaStream_t s);
long long scan_blocks(long long n);
long long radix_blocks(long long n);
bool launch_radix_sort(unsigned* keys, int* vals, unsigned* kt, int* vt, const long long* np,
                       long long cap, int bits, int* hist, long long* off, long long* sums,
                       int num_sms, cudaStream_t s);
int launch_contract_fp32(const Geo& g, const Ws& w, int num_sms, cudaStream_t s);
int launch_contract_bf16x3(const Geo& g, const Ws& w, int num_sms, cudaStream_t s);
void launch_reduce_partials(const Geo& g, const Ws& w, int num_sms, cudaStream_t s);
void launch_spec_store(const Geo& g, const Ws& w, int num_sms, cudaStream_t s);
void launch_flux_batch(const Geo& g, const Ws& w, cudaStream_t s);
void launch_flux(const float* cube, int nx, int ny, int nc, int padx, int pady, double* part,
                 double* flux, cudaStream_t s);
int flux_chunks(int nx, int padx);

// Footprint and channel support (FP64), shared by the binning and the
// global-profile kernels.
// |k - c| <= r as the reference evaluates it, in FP64.  For moderate
// coordinates (m = |c| + r + 1 < 1e6, k within r + 2 of c) the FP32
// difference decides whenever it clears r by 4e-7 m: c and r rounded to FP32
// and the FP32 subtraction are each off by at most 2^-24 of their magnitude,
// about 1.8e-7 m together, so beyond that band FP64 gives the same answer.
// Only tests inside the band run in FP64 (this part has few FP64 units).
struct AbsWithin {
  double c, r;
  float cf, rf, tol;
  bool fast;
  __device__ __forceinline__ AbsWithin(double c_, double r_) : c(c_), r(r_) {
    cf = (float)c_;
    rf = (float)r_;
    const float m = fabsf(cf) + rf + 1.f;
    fast = m < 1.0e6f;  // false for NaN too
    tol = 4.0e-7f * m;
  }
  __device__ __forceinline__ bool operator()(int k) const {
    if (fast) {
      const float d = fabsf((float)k - cf);
      if (d <= rf - tol) return true;
      if (d >= rf + tol) return false;
    }
    return fabs((double)k - c) <= r;
  }
};

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
  const AbsWithin in(c, r);
  // scan start points outside the answer on both sides: FP32 for moderate
  // coordinates (off by < 0.2 there, so one extra step of margin), FP64 else
  double a, b;
  if (in.fast) {
    a = (double)(floorf(in.cf - in.rf) - 2.f);
    b = (double)(ceilf(in.cf + in.rf) + 2.f);
  } else {
    a = floor(c - r) - 1.0;
    b = ceil(c + r) + 1.0;
  }
  if (a < 0.0) a = 0.0;
  if (b > (double)(n - 1)) b = (double)(n - 1);
  if (a > b) {
    lo = 0;
    hi = -1;
    return;
  }
  int l = (int)a, h = (int)b;
  while (l <= h && !in(l)) ++l;
  while (h >= l && !in(h)) --h;
  lo = l;
  hi = h;
}

// Smallest k in [0, n] with pred(k) (pred monotone false -> true over
// [0, n), pred(n) taken as true), searched from a guess: galloping steps to
// bracket the answer, then bisection.  Exact for any guess; a right guess
// costs two probes.
template <class P>
__device__ __forceinline__ int first_true(int n, int guess, P pred) {
  int lo, hi;  // answer in (lo, hi]: pred(hi) true or hi == n, pred(lo) false or lo == -1
  guess = min(max(guess, 0), n);
  if (guess == n || pred(guess)) {
    hi = guess;
    int step = 1;
    lo = guess - 1;
    while (lo >= 0 && pred(lo)) {
      hi = lo;
      lo -= step;
      step <<= 1;
    }
    if (lo < -1) lo = -1;
  } else {
    lo = guess;
    int step = 1;
    hi = guess + 1;
    while (hi < n && !pred(hi)) {
      lo = hi;
      hi += step;
      step <<= 1;
    }
    if (hi > n) hi = n;
  }
  while (hi - lo > 1) {
    const int m = lo + ((hi - lo) >> 1);
    if (pred(m)) hi = m; else lo = m;
  }
  return hi;
}

// Channel index range whose closed velocity interval meets [lo, hi].  The
// FP64 edge comparisons decide; a linear guess from the end edges (exact
// for uniform channels) starts each search.
__device__ __forceinline__ void channel_range(const double* e, int nc, int dec, double lo,
                                              double hi, int& c0, int& c1) {
  // E(k) = edges in increasing order
  auto E = [&](int k) { return dec ? e[nc - k] : e[k]; };
  const double e0 = E(0), en = E(nc);
  const float scale = (float)nc / (float)(en - e0);
  auto guess = [&](double v) {
    const float t = floorf((float)(v - e0) * scale);
    return t >= 0.f ? (t < (float)nc ? (int)t : nc) : 0;  // NaN -> 0
  };
  // first c in [0, nc) with E(c + 1) >= lo (nc if none)
  const int first = first_true(nc, guess(lo) - 1, [&](int c) { return E(c + 1) >= lo; });
  // last c in [0, nc) with E(c) <= hi  ->  (first c with E(c) > hi) - 1
  const int last = first_true(nc, guess(hi), [&](int c) { return E(c) > hi; }) - 1;
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

// ---------------------------------------------------------------------------
// Kernel pixel integrals (martini/sph_kernels.py).  dx, dy are particle minus
// pixel centre in px, h the rescaled smoothing length.  Each returns the
// integral over the pixel per unit pixel area (px^-2).
// ---------------------------------------------------------------------------

constexpr float kPi = 3.14159265358979323846f;

// Radial kernels (WendlandC2 sph_kernels.py:400-441, WendlandC6 :544-685,
// cubic spline :791-858, quartic spline :1486-1564): the pixel integral is
// scale * f(s) / h^2 with s = R^2 (offsets doubled for the cubic spline).
// f comes from cubic polynomials on uniform cells fitted in FP64 to the
// reference closed forms (mg_kernel_tables.h, made by gen_kernel_tables.py):
// a direct cell index, one float4 of coefficients and three FMAs, accurate
// to ~1e-7 of f(0) in FP32 (7e-7 for Wendland C6) where the closed forms
// lose up to 7e-4.
// floor(u) and t = u - floor(u) for 0 <= u < 2^23 without conversions:
// adding 2^23 rounded toward -inf leaves floor(u) in the low mantissa bits.
__device__ __forceinline__ int kt_floor(float u, float& t) {
  const float v = __fadd_rd(u, 8388608.f);
  t = u - (v - 8388608.f);
  return __float_as_int(v) - 0x4B000000;
}

__device__ __forceinline__ float kt_eval(int kt, float s) {
  const KTableInfo& inf = kt_info[kt];
  if (!(s < inf.smax)) return 0.f;
  const float R = s > 0.f ? s * rsqrtf(s) : 0.f;
  int r = 0;
  if (inf.nreg == 3) r = (s > 1.f) ? 2 : (R >= inf.split_r ? 1 : 0);
  const KRegion g = inf.reg[r];
  if (g.var == 2) {  // cells in s; s >= smax lands on the zero cell
    const float u = fminf(s * g.cells_per_unit, (float)g.ncell);
    float t;
    const int c = kt_floor(u, t);
    const float4 cf = __ldg(reinterpret_cast<const float4*>(kt_coef) + g.first + c);
    return fmaf(fmaf(fmaf(cf.w, t, cf.z), t, cf.y), t, cf.x);
  }
  const float a2 = fmaxf(1.f - s, 0.f);
  const float v = g.var ? (a2 > 0.f ? a2 * rsqrtf(a2) : 0.f) : R;
  const float u = (v - g.lo) * g.cells_per_unit;
  int c = (int)u;
  c = c < 0 ? 0 : (c >= g.ncell ? g.ncell - 1 : c);
  const float t = u - (float)c;
  static_assert(KT_DEG == 3, "one float4 of coefficients per cell");
  const float4 cf = __ldg(reinterpret_cast<const float4*>(kt_coef) + g.first + c);
  return fmaf(fmaf(fmaf(cf.w, t, cf.z), t, cf.y), t, cf.x);
}

__device__ __forceinline__ float w_radial(int kt, float r2, float inv_h2) {
  const float s = (kt == MG_KERNEL_CUBIC_SPLINE ? 4.f : 1.f) * r2 * inv_h2;
  return kt_eval(kt, s) * kt_info[kt].scale * inv_h2;
}

// Upper bound of a particle's pixel weight (per unit pixel area).
__device__ __forceinline__ float weight_bound(int type, float inv_h2, float gnorm) {
  if (type == MG_KERNEL_DIRAC) return 1.f;
  if (type == MG_KERNEL_GAUSSIAN) return 1.f / gnorm;
  return kt_eval(type, 0.f) * kt_info[type].scale * inv_h2;
}

// _GaussianKernel._kernel_integral, sph_kernels.py:994-1044.
__device__ __forceinline__ float w_gaussian(float dx, float dy, float h, float trunc,
                                            float gnorm) {
  // quotients by h sigma as products with one reciprocal (an ulp or two from
  // the quotients, without six divisions per pixel)
  const float inv_hs = 1.f / (h * 0.42466090014400953f);  // sigma = 1 / (2 sqrt(2 ln 2))
  const float dr = sqrtf(dx * dx + dy * dy);
  const float q = dr * inv_hs;
  if ((dr - 0.70710678118654752f) * inv_hs > trunc) return 0.f;
  const float zmax = trunc > q ? sqrtf(trunc * trunc - q * q) : 0.f;
  const float s = inv_hs * 0.70710678118654752f;  // 1 / (h sqrt(2) sigma)
  const float ex = erff((dx + 0.5f) * s) - erff((dx - 0.5f) * s);
  const float ey = erff((dy + 0.5f) * s) - erff((dy - 0.5f) * s);
  return 0.25f * erff(zmax * 0.70710678118654752f) * ex * ey * (1.f / gnorm);
}

// Weight of pixel (i, j) for a particle record; 0 outside the footprint box.
__device__ __forceinline__ float pixel_weight(const PRec& r, const KSpec* ks, int i, int j) {
  if (i < r.ilo || i > r.ihi || j < r.jlo || j > r.jhi) return 0.f;
  const KSpec k = ks[r.kslot];
  if (k.type == MG_KERNEL_DIRAC) return 1.f;  // footprint reduced to the one pixel
  float dx = (float)(r.xi - i) + r.xf;
  float dy = (float)(r.yi - j) + r.yf;
  float r2 = dx * dx + dy * dy;
  if (k.type == MG_KERNEL_GAUSSIAN) return w_gaussian(dx, dy, r.h, k.truncate, k.gnorm);
  return w_radial(k.type, r2, r.inv_h2);
}

// ---------------------------------------------------------------------------
// Channel spectra (martini/spectral_models.py)
// ---------------------------------------------------------------------------

// 0.5 [erf(b) - erf(a)] for b >= a, using erfc in the tails.
__device__ __forceinline__ float half_erf_diff(float a, float b) {
  if (a >= 0.f) return 0.5f * (erfcf(a) - erfcf(b));
  if (b <= 0.f) return 0.5f * (erfcf(-b) - erfcf(-a));
  return 0.5f * (erff(b) - erff(a));
}

// S_p(c) for one channel (GAUSSIAN / DIRAC), spectral_models.py:63-200.
// Edge e of the cube is (ehi[e] + elo[e]); the channel's lower/upper edges
// depend on the edge direction (spectral_models.py:180-187).
__device__ __forceinline__ float channel_spectrum(const PRec& r, int model, int c, int dec,
                                                  const float* ehi, const float* elo,
                                                  const float* inv_w) {
  if (c < r.clo || c > r.chi) return 0.f;
  if (model == MG_SPECTRUM_DIRAC) return r.amp * inv_w[c];
  int e_lo = dec ? c + 1 : c;
  int e_hi = dec ? c : c + 1;
  float a = ((ehi[e_lo] - r.vhi) + (elo[e_lo] - r.vlo)) * r.inv_s;
  float b = ((ehi[e_hi] - r.vhi) + (elo[e_hi] - r.vlo)) * r.inv_s;
  return r.amp * half_erf_diff(a, b) * inv_w[c];
}

}  // namespace mg
