// C ABI of the martini_gb300 library (declared in include/martini_gb300.h).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "mg_internal.cuh"

using namespace mg;

namespace mg {
void set_last_error(const std::string& msg);
}

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(MG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

bool known_form(int form) {
  return form == MG_FORM_FP32 || form == MG_FORM_BF16X3 || form == MG_FORM_F16X3 ||
         form == MG_FORM_BF16X6;
}

// Segment shape of a contraction form: channel blocks per tile and their
// width.  Tensor-core forms: the band (rounded to 16) in one block up to the
// form's block width, else blocks of that width: 256 for the pairs (a block
// and its master accumulator fill the 512 TMEM columns), 128 for bf16x6
// (two working accumulators and the master: its 64-particle stages).
void seg_shape(int form, int nc, int* ncb, int* width) {
  if (form == MG_FORM_BF16X3 || form == MG_FORM_F16X3 || form == MG_FORM_BF16X6) {
    const int bw = form == MG_FORM_BF16X6 ? 128 : 256;
    if (nc <= bw) {
      *ncb = 1;
      *width = (nc + 15) / 16 * 16;
    } else {
      *ncb = (nc + bw - 1) / bw;
      *width = bw;
    }
  } else {
    *ncb = (nc + CBLK - 1) / CBLK;
    *width = CBLK;
  }
}

int channel_bits(int nc) {
  int b = 0;
  while ((1 << b) < nc) ++b;
  return b;
}

struct Layout {
  size_t hdr, gal, gst, gp0, gt0, gs0, ge0, gr0, rec, tpar, npairs, pair_off, tile_count, tile_diff,
      tile_off, ehi, elo, inv_w, keys, list, keys_tmp, list_tmp, rs_hist,
      rs_off, scan_sums, seg_lo, seg_hi, seg_items, seg_part, item_off, part_off, partial,
      flux_part, item_order, item_key, item_key_tmp, item_order_tmp, item_seg, total;
  long long cap_items;
};

Layout layout(const Geo& g, long long cap_pairs, long long cap_partial) {
  Layout L;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o += align256(bytes > 0 ? bytes : 1);
    return at;
  };
  const size_t nn = (size_t)(g.n > 0 ? g.n : 1);
  const size_t ng1 = (size_t)g.ngal + 1;
  const size_t cp = (size_t)(cap_pairs > 0 ? cap_pairs : 1);
  const long long rb = radix_blocks(cap_pairs > 0 ? cap_pairs : 1);
  long long scan_n = g.n;
  if (256 * rb > scan_n) scan_n = 256 * rb;
  if (g.nseg > scan_n) scan_n = g.nseg;
  if (g.ntiles > scan_n) scan_n = g.ntiles;
  L.hdr = take(sizeof(WsHeader));
  L.gal = take(sizeof(Gal) * (size_t)g.ngal);
  L.gst = take(sizeof(GalState) * (size_t)g.ngal);
  L.gp0 = take(sizeof(long long) * ng1);
  L.gt0 = take(sizeof(int) * ng1);
  L.gs0 = take(sizeof(int) * ng1);
  L.ge0 = take(sizeof(int) * ng1);
  L.gr0 = take(sizeof(int) * ng1);
  L.rec = take(sizeof(PRec) * nn);
  const bool tc = g.form == MG_FORM_BF16X3 || g.form == MG_FORM_F16X3 || g.form == MG_FORM_BF16X6;
  L.tpar = tc ? take(sizeof(TcPar) * nn) : 0;
  L.npairs = take(sizeof(int) * nn);
  L.pair_off = take(sizeof(long long) * nn);
  L.tile_count = take(sizeof(int) * (size_t)g.ntiles);
  L.tile_diff = take(sizeof(int) * (size_t)g.ndiff);
  L.tile_off = take(sizeof(long long) * ((size_t)g.ntiles + 1));
  L.ehi = take(sizeof(float) * (size_t)g.nedge);
  L.elo = take(sizeof(float) * (size_t)g.nedge);
  L.inv_w = take(sizeof(float) * (size_t)g.nedge);
  L.keys = take(sizeof(unsigned) * cp);
  L.list = take(sizeof(int) * cp);
  L.keys_tmp = take(sizeof(unsigned) * cp);
  L.list_tmp = take(sizeof(int) * cp);
  L.rs_hist = take(sizeof(int) * 256 * (size_t)rb);
  L.rs_off = take(sizeof(long long) * 256 * (size_t)rb);
  L.scan_sums = take(sizeof(long long) * (size_t)(scan_blocks(scan_n) + 1));
  L.seg_lo = take(sizeof(long long) * (size_t)g.nseg);
  L.seg_hi = take(sizeof(long long) * (size_t)g.nseg);
  L.seg_items = take(sizeof(int) * (size_t)g.nseg);
  L.seg_part = take(sizeof(int) * (size_t)g.nseg);
  L.item_off = take(sizeof(long long) * (size_t)g.nseg);
  L.part_off = take(sizeof(long long) * (size_t)g.nseg);
  L.flux_part = take(sizeof(double) * (size_t)g.nfpart);
  L.cap_items = items_bound(g.nseg, cap_pairs > 0 ? cap_pairs : 0);
  const size_t ci = (size_t)(L.cap_items > 0 ? L.cap_items : 1);
  L.item_order = take(sizeof(int) * ci);
  L.item_key = take(sizeof(unsigned) * ci);
  L.item_key_tmp = take(sizeof(unsigned) * ci);
  L.item_order_tmp = take(sizeof(int) * ci);
  L.item_seg = take(sizeof(int) * ci);
  L.partial = take(sizeof(float) * (size_t)TILE_PX * g.max_width *
                   (size_t)(cap_partial > 0 ? cap_partial : 0));
  L.total = o;
  return L;
}

Ws make_ws(void* base, const Layout& L) {
  char* b = static_cast<char*>(base);
  Ws w;
  w.hdr = reinterpret_cast<WsHeader*>(b + L.hdr);
  w.gal = reinterpret_cast<Gal*>(b + L.gal);
  w.gst = reinterpret_cast<GalState*>(b + L.gst);
  w.gp0 = reinterpret_cast<long long*>(b + L.gp0);
  w.gt0 = reinterpret_cast<int*>(b + L.gt0);
  w.gs0 = reinterpret_cast<int*>(b + L.gs0);
  w.ge0 = reinterpret_cast<int*>(b + L.ge0);
  w.gr0 = reinterpret_cast<int*>(b + L.gr0);
  w.rec = reinterpret_cast<PRec*>(b + L.rec);
  w.tpar = L.tpar ? reinterpret_cast<TcPar*>(b + L.tpar) : nullptr;
  w.npairs = reinterpret_cast<int*>(b + L.npairs);
  w.pair_off = reinterpret_cast<long long*>(b + L.pair_off);
  w.tile_count = reinterpret_cast<int*>(b + L.tile_count);
  w.tile_diff = reinterpret_cast<int*>(b + L.tile_diff);
  w.tile_off = reinterpret_cast<long long*>(b + L.tile_off);
  w.ehi = reinterpret_cast<float*>(b + L.ehi);
  w.elo = reinterpret_cast<float*>(b + L.elo);
  w.inv_w = reinterpret_cast<float*>(b + L.inv_w);
  w.keys = reinterpret_cast<unsigned*>(b + L.keys);
  w.list = reinterpret_cast<int*>(b + L.list);
  w.keys_tmp = reinterpret_cast<unsigned*>(b + L.keys_tmp);
  w.list_tmp = reinterpret_cast<int*>(b + L.list_tmp);
  w.rs_hist = reinterpret_cast<int*>(b + L.rs_hist);
  w.rs_off = reinterpret_cast<long long*>(b + L.rs_off);
  w.scan_sums = reinterpret_cast<long long*>(b + L.scan_sums);
  w.seg_lo = reinterpret_cast<long long*>(b + L.seg_lo);
  w.seg_hi = reinterpret_cast<long long*>(b + L.seg_hi);
  w.seg_items = reinterpret_cast<int*>(b + L.seg_items);
  w.seg_part = reinterpret_cast<int*>(b + L.seg_part);
  w.item_off = reinterpret_cast<long long*>(b + L.item_off);
  w.part_off = reinterpret_cast<long long*>(b + L.part_off);
  w.partial = reinterpret_cast<float*>(b + L.partial);
  w.flux_part = reinterpret_cast<double*>(b + L.flux_part);
  w.spec = nullptr;
  w.cap_spec = 0;
  w.item_order = reinterpret_cast<int*>(b + L.item_order);
  w.item_key = reinterpret_cast<unsigned*>(b + L.item_key);
  w.item_key_tmp = reinterpret_cast<unsigned*>(b + L.item_key_tmp);
  w.item_order_tmp = reinterpret_cast<int*>(b + L.item_order_tmp);
  w.item_seg = reinterpret_cast<int*>(b + L.item_seg);
  w.cap_items = L.cap_items;
  return w;
}

double gaussian_norm(double t) {
  return std::erf(t / std::sqrt(2.0)) -
         2.0 * t / std::sqrt(2.0 * 3.14159265358979323846) * std::exp(-t * t / 2.0);
}

// Validate one problem (no device access: edge direction and monotonicity
// are resolved by the k_edges kernel).
int check_problem(const mg_problem* p) {
  if (!p) return fail(MG_ERR_INVALID_ARGUMENT, "null problem");
  if (p->nx <= 0 || p->ny <= 0 || p->nc <= 0)
    return fail(MG_ERR_INVALID_ARGUMENT, "cube dimensions must be positive");
  if (p->n < 0) return fail(MG_ERR_INVALID_ARGUMENT, "negative particle count");
  if (p->n_kernels < 1 || p->n_kernels > MG_MAX_KERNELS)
    return fail(MG_ERR_INVALID_ARGUMENT, "n_kernels must be 1..4");
  if (p->padx < 0 || p->pady < 0 || 2 * p->padx >= p->nx || 2 * p->pady >= p->ny)
    return fail(MG_ERR_INVALID_ARGUMENT, "invalid pad");
  if (!p->edges || !p->cube) return fail(MG_ERR_INVALID_ARGUMENT, "edges and cube are required");
  if (p->spectral_model == MG_SPECTRUM_TABLE) {
    if (p->n > 0 && !p->spectra)
      return fail(MG_ERR_INVALID_ARGUMENT, "TABLE spectral model needs spectra");
  } else if (p->spectral_model == MG_SPECTRUM_GAUSSIAN || p->spectral_model == MG_SPECTRUM_DIRAC) {
    if (p->n > 0 && (!p->v || !p->amp))
      return fail(MG_ERR_INVALID_ARGUMENT, "v and amp are required");
    if (p->n > 0 && p->spectral_model == MG_SPECTRUM_GAUSSIAN && !p->sigma &&
        !(p->sigma_const > 0.f))
      return fail(MG_ERR_INVALID_ARGUMENT, "Gaussian spectrum needs sigma > 0");
  } else {
    return fail(MG_ERR_INVALID_ARGUMENT, "unknown spectral model");
  }
  if (p->n > 0 && (!p->x || !p->y || !p->sm_range || !p->h_eff))
    return fail(MG_ERR_INVALID_ARGUMENT, "x, y, sm_range and h_eff are required");
  if (!known_form(p->form))
    return fail(MG_ERR_INVALID_ARGUMENT, "unknown contraction form");
  for (int k = 0; k < p->n_kernels; ++k) {
    const int t = p->kernels[k].type;
    if (t < MG_KERNEL_WENDLAND_C2 || t > MG_KERNEL_DIRAC)
      return fail(MG_ERR_INVALID_ARGUMENT, "unknown kernel type");
    if (t == MG_KERNEL_GAUSSIAN && !(p->kernels[k].truncate >= 2.f))
      return fail(MG_ERR_INVALID_ARGUMENT,
                  "GaussianKernel with truncation <2sigma will cause large errors in total mass.");
  }
  return MG_OK;
}

// Host description of a batch: the per-cube table and the batch constants.
struct Batch {
  std::vector<Gal> gal;
  Geo g;
};

// Validate a batch (every cube shares the kernel table, spectral model,
// contraction form and accumulate flag) and lay its cubes out in the
// batch-wide index spaces.  `shape_only` (workspace sizing) checks just
// what the layout depends on: sizes, pads and form.
int make_batch(const mg_problem* probs, int nprob, Batch* b, bool shape_only = false) {
  if (!probs || nprob < 1) return fail(MG_ERR_INVALID_ARGUMENT, "empty batch");
  if (nprob > 65535) return fail(MG_ERR_INVALID_ARGUMENT, "at most 65535 cubes in a batch");
  for (int k = 0; k < nprob; ++k) {
    const mg_problem& p = probs[k];
    int rc = MG_OK;
    if (!shape_only) {
      rc = check_problem(&p);
    } else if (p.nx <= 0 || p.ny <= 0 || p.nc <= 0 || p.n < 0) {
      rc = fail(MG_ERR_INVALID_ARGUMENT, "invalid problem dimensions");
    } else if (p.padx < 0 || p.pady < 0 || 2 * p.padx >= p.nx || 2 * p.pady >= p.ny) {
      rc = fail(MG_ERR_INVALID_ARGUMENT, "invalid pad");
    } else if (!known_form(p.form)) {
      rc = fail(MG_ERR_INVALID_ARGUMENT, "unknown contraction form");
    }
    if (rc) return rc;
  }
  const mg_problem& p0 = probs[0];
  for (int k = 1; k < nprob && !shape_only; ++k) {
    const mg_problem& p = probs[k];
    bool same = p.n_kernels == p0.n_kernels && p.spectral_model == p0.spectral_model &&
                p.form == p0.form && (p.accumulate != 0) == (p0.accumulate != 0);
    for (int j = 0; same && j < p0.n_kernels; ++j)
      same = p.kernels[j].type == p0.kernels[j].type &&
             p.kernels[j].truncate == p0.kernels[j].truncate;
    if (!same)
      return fail(MG_ERR_INVALID_ARGUMENT,
                  "the problems of a batch must share kernels, spectral model, form and "
                  "accumulate flag");
  }
  Geo& g = b->g;
  std::memset(&g, 0, sizeof(Geo));
  g.ngal = nprob;
  g.n_kernels = p0.n_kernels;
  g.spectral_model = p0.spectral_model;
  g.form = p0.form;
  g.accumulate = p0.accumulate != 0;
  for (int k = 0; k < p0.n_kernels && k < MG_MAX_KERNELS; ++k) {
    const int t = p0.kernels[k].type;
    g.ks[k].type = t;
    g.ks[k].truncate = p0.kernels[k].truncate;
    g.ks[k].gnorm = t == MG_KERNEL_GAUSSIAN ? (float)gaussian_norm(p0.kernels[k].truncate) : 1.f;
  }
  b->gal.assign(nprob, Gal());
  long long n = 0, ndiff = 0, nedge = 0, nfpart = 0, ntiles = 0, nseg = 0, nrows = 0;
  for (int k = 0; k < nprob; ++k) {
    const mg_problem& p = probs[k];
    Gal& G = b->gal[k];
    std::memset(&G, 0, sizeof(Gal));
    G.x = p.x;
    G.y = p.y;
    G.r = p.sm_range;
    G.h = p.h_eff;
    G.kidx = p.kernel_index;
    G.v = p.v;
    G.sigma = p.sigma;
    G.amp = p.amp;
    G.spectra = p.spectra;
    G.edges = p.edges;
    G.cube = p.cube;
    G.flux = p.flux;
    G.sigma_const = p.sigma_const;
    G.nx = p.nx;
    G.ny = p.ny;
    G.nc = p.nc;
    G.padx = p.padx;
    G.pady = p.pady;
    G.ntx = (p.nx + TILE_I - 1) / TILE_I;
    G.nty = (p.ny + TILE_J - 1) / TILE_J;
    const long long nt = (long long)G.ntx * G.nty;
    seg_shape(p.form, p.nc, &G.ncb, &G.width);
    G.p0 = n;
    G.n = p.n;
    G.tile0 = (int)ntiles;
    G.seg0 = (int)nseg;
    G.diff0 = ndiff;
    G.edge0 = (int)nedge;
    G.row0 = (int)nrows;
    G.fpart0 = nfpart;
    G.ntiles = (int)nt;
    const long long nd = (long long)(G.ntx + 1) * (G.nty + 1);
    const int rows = p.nx - 2 * p.padx;
    n += p.n;
    ntiles += nt;
    nseg += nt * G.ncb;
    ndiff += nd;
    nedge += p.nc + 1;
    nrows += rows;
    nfpart += (long long)rows * p.nc;
    if (ntiles > (1LL << 30) || nseg > (1LL << 30) || nedge > (1LL << 30) || nrows > (1LL << 30))
      return fail(MG_ERR_INVALID_ARGUMENT, "batch too large");
    if (G.width > g.max_width) g.max_width = G.width;
    if (p.nc > g.max_nc) g.max_nc = p.nc;
    if (nd > g.max_diff) g.max_diff = nd > (1LL << 30) ? (1 << 30) : (int)nd;
  }
  g.n = n;
  g.ntiles = (int)ntiles;
  g.nseg = (int)nseg;
  g.ndiff = ndiff;
  g.nedge = nedge;
  g.nrows = (int)nrows;
  g.nfpart = nfpart;
  // sort-key bits below the segment: two kernel-class bits above the channel
  g.cbits = channel_bits(g.max_nc) + 2;
  return MG_OK;
}

// SM count of the current device (cached per device).
int num_sms() {
  constexpr int kMaxDev = 64;
  static int sms[kMaxDev] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return 1;
  if (sms[dev] <= 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    sms[dev] = v > 0 ? v : 1;
  }
  return sms[dev];
}

bool tc_form(int form) {
  return form == MG_FORM_BF16X3 || form == MG_FORM_F16X3 || form == MG_FORM_BF16X6;
}

int workspace_view(const Geo& g, void* ws, size_t bytes, long long cap_pairs,
                   long long cap_partial, Ws* w) {
  Layout L = layout(g, cap_pairs, cap_partial);
  if (!ws || bytes < L.total)
    return fail(MG_ERR_WORKSPACE, "workspace too small: need " + std::to_string(L.total) +
                                      " bytes, have " + std::to_string(bytes));
  *w = make_ws(ws, L);
  if (sort_bits(g) > 32) return fail(MG_ERR_INVALID_ARGUMENT, "cube too large for the sort key");
  // the workspace beyond the fixed layout holds the spectrum store of the
  // tensor-core forms (Gaussian lines); without room they evaluate in-kernel
  if (tc_form(g.form) && g.spectral_model == MG_SPECTRUM_GAUSSIAN) {
    w->spec = reinterpret_cast<unsigned*>(static_cast<char*>(ws) + L.total);
    w->cap_spec = (long long)((bytes - L.total) / sizeof(unsigned));
  }
  return MG_OK;
}

// Zero the cubes of a batch (one block row per cube).
__global__ void k_clear_cubes(Geo g, Ws w) {
  const Gal& G = w.gal[blockIdx.y];
  const long long n = (long long)G.nx * G.ny * G.nc;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x)
    G.cube[k] = 0.f;
}

}  // namespace

void mg::set_last_error(const std::string& msg) { g_err = msg; }

extern "C" {

const char* mg_version(void) { return "martini_gb300 0.2 (sm_103a)"; }

const char* mg_last_error(void) { return g_err.c_str(); }

int mg_workspace_size_batched(const mg_problem* probs, int32_t nprob, int64_t max_pairs,
                              int64_t max_partial_items, size_t* bytes) {
  if (!probs || !bytes) return fail(MG_ERR_INVALID_ARGUMENT, "null argument");
  if (max_pairs < 0 || max_partial_items < 0)
    return fail(MG_ERR_INVALID_ARGUMENT, "negative capacity");
  Batch b;
  int rc = make_batch(probs, nprob, &b, true);
  if (rc) return rc;
  *bytes = layout(b.g, max_pairs, max_partial_items).total;
  return MG_OK;
}

int mg_workspace_size(const mg_problem* p, int64_t max_pairs, int64_t max_partial_items,
                      size_t* bytes) {
  if (!p || !bytes) return fail(MG_ERR_INVALID_ARGUMENT, "null argument");
  if (p->nx <= 0 || p->ny <= 0 || p->nc <= 0 || p->n < 0)
    return fail(MG_ERR_INVALID_ARGUMENT, "invalid problem dimensions");
  return mg_workspace_size_batched(p, 1, max_pairs, max_partial_items, bytes);
}

}  // extern "C"

namespace {

// ---------------------------------------------------------------------------
// Launch shapes: validation, the per-class cache and the problem class key
// ---------------------------------------------------------------------------

bool shape_ok(int form, const mg_tuning& t) {
  if (t.items_per_sm < 0 || t.items_per_sm > ITEMS_PER_SM) return false;
  if (t.cost_order != 0 && t.cost_order != 1) return false;
  if (t.kc == 0) return true;
  if (form == MG_FORM_FP32) return false;
  return t.kc == 32 || t.kc == 64;
}

// The launch shape into the batch constants.  A plan (no particle list)
// bins with the default items per SM: its split-K bound then holds for
// every shape, whose items per SM never exceed the default.
void apply_shape(const mg_tuning* t, bool scatter, Geo* g) {
  mg_tuning d;
  mg_tuning_default(&d);
  const mg_tuning& u = (t && shape_ok(g->form, *t)) ? *t : d;
  g->kc = u.kc;
  g->items_per_sm = (scatter && u.items_per_sm > 0) ? u.items_per_sm : ITEMS_PER_SM;
  g->cost_order = u.cost_order;
}

std::mutex g_tune_mu;
std::map<std::string, mg_tuning> g_tune_cache;

int floor_log2(double v) { return v >= 1.0 ? (int)std::floor(std::log2(v)) : -1; }

// Problem class: form, kernel table, spectral model, cubes (octave), widest
// band, particles (octave), pairs per tile (half octave).
std::string class_key(const Batch& b, long long max_pairs) {
  const Geo& g = b.g;
  std::string k = "f" + std::to_string(g.form) + " m" + std::to_string(g.spectral_model);
  for (int i = 0; i < g.n_kernels; ++i)
    k += " k" + std::to_string(g.ks[i].type) + ":" + std::to_string((int)(g.ks[i].truncate * 16));
  const double ppt = g.ntiles > 0 ? (double)max_pairs / (double)g.ntiles : 0.0;
  k += " g" + std::to_string(floor_log2((double)g.ngal)) + " c" + std::to_string(g.max_nc) +
       " n" + std::to_string(floor_log2((double)g.n + 1.0)) + " t" +
       std::to_string((int)std::floor(2.0 * std::log2(ppt + 1.0)));
  return k;
}

// The stages of an insertion (MG_STAGE_* bits; `scatter` adds the particle
// list to the binning stage); all asynchronous on stream s.
int run(const mg_problem* probs, int nprob, void* ws, size_t bytes, cudaStream_t s,
        long long cap_pairs, long long cap_partial, int stages, bool scatter, Ws* wout,
        Batch* bout, const mg_tuning* shape) {
  Batch& b = *bout;
  int rc = make_batch(probs, nprob, &b);
  if (rc) return rc;
  apply_shape(shape, scatter, &b.g);
  const Geo& g = b.g;
  if (cap_pairs < 0 || cap_partial < 0) return fail(MG_ERR_INVALID_ARGUMENT, "negative capacity");
  Ws w;
  rc = workspace_view(g, ws, bytes, cap_pairs, cap_partial, &w);
  if (rc) return rc;
  launch_set_gals(b.gal.data(), g, w, s);
  if (stages & MG_STAGE_BIN) {
    launch_prep(g, w, num_sms(), s, cap_pairs, cap_partial);
    if (scatter) launch_sort_segments(g, w, cap_pairs, num_sms(), s);
  }
  if ((stages & MG_STAGE_SPEC) && tc_form(g.form)) launch_spec_store(g, w, num_sms(), s);
  cudaError_t e;
  if (stages & MG_STAGE_CONTRACT) {
    e = cudaSuccess;
    if (!g.accumulate) {
      if (g.ngal == 1) {
        const Gal& G = b.gal[0];
        e = cudaMemsetAsync(G.cube, 0, sizeof(float) * (size_t)G.nx * G.ny * G.nc, s);
      } else {
        k_clear_cubes<<<dim3(64, (unsigned)g.ngal), 256, 0, s>>>(g, w);
      }
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(&w.hdr->item_counter, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return cuda_fail(e, "cube clear");
    if (tc_form(g.form)) {
      rc = launch_contract_bf16x3(g, w, num_sms(), s);
      if (rc == MG_ERR_CUDA) return cuda_fail(cudaGetLastError(), "tensor-core kernel set-up");
      if (rc) return fail(rc, "tensor-core form does not support this cube (band too wide)");
    } else {
      rc = launch_contract_fp32(g, w, num_sms(), s);
      if (rc) return cuda_fail(cudaGetLastError(), "FP32 contraction set-up");
    }
  }
  if (stages & MG_STAGE_FLUX) {
    bool any = false;
    for (const Gal& G : b.gal) any = any || G.flux != nullptr;
    if (any) launch_flux_batch(g, w, s);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
  *wout = w;
  return MG_OK;
}

}  // namespace

extern "C" {

int mg_plan_batched(const mg_problem* probs, int32_t nprob, void* workspace,
                    size_t workspace_bytes, void* stream, mg_plan_info* info) {
  if (!info) return fail(MG_ERR_INVALID_ARGUMENT, "null info");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Ws w{};
  Batch b;
  int rc = run(probs, nprob, workspace, workspace_bytes, s, 0, 0, MG_STAGE_BIN, false, &w, &b,
               nullptr);
  if (rc) return rc;
  WsHeader h;
  cudaError_t e = cudaMemcpyAsync(&h, w.hdr, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "mg_plan readback");
  if (h.status & ST_EDGES) return fail(MG_ERR_NOT_MONOTONIC, "Channel edges are not monotonic sequence.");
  info->n_pairs = h.n_pairs;
  info->n_items = 0;
  info->n_partial_items = h.partial_bound;
  info->n_tiles = b.g.ntiles;
  size_t spec_bytes = 0;
  if (tc_form(b.g.form) && b.g.spectral_model == MG_SPECTRUM_GAUSSIAN)
    // one 32-bit word per support channel: packed hi | lo halves, or the FP32
    // value the three-piece BF16 split is taken from
    spec_bytes = align256(sizeof(unsigned) * (size_t)h.spec_bound);
  info->workspace_bytes = layout(b.g, h.n_pairs, h.partial_bound).total + spec_bytes;
  return MG_OK;
}

int mg_plan(const mg_problem* p, void* workspace, size_t workspace_bytes, void* stream,
            mg_plan_info* info) {
  return mg_plan_batched(p, 1, workspace, workspace_bytes, stream, info);
}

int mg_insert_stages_batched(const mg_problem* probs, int32_t nprob, void* workspace,
                             size_t workspace_bytes, int64_t max_pairs, int64_t max_partial_items,
                             int32_t stages, void* stream) {
  if (stages & ~MG_STAGE_ALL) return fail(MG_ERR_INVALID_ARGUMENT, "unknown stage bits");
  Ws w;
  Batch b;
  // the launch shape cached for this problem's class, if any
  mg_tuning shape;
  mg_tuning_lookup(probs, nprob, max_pairs, &shape);
  return run(probs, nprob, workspace, workspace_bytes, static_cast<cudaStream_t>(stream),
             max_pairs, max_partial_items, stages, true, &w, &b, &shape);
}

int mg_insert_batched(const mg_problem* probs, int32_t nprob, void* workspace,
                      size_t workspace_bytes, int64_t max_pairs, int64_t max_partial_items,
                      void* stream) {
  return mg_insert_stages_batched(probs, nprob, workspace, workspace_bytes, max_pairs,
                                  max_partial_items, MG_STAGE_ALL, stream);
}

int mg_insert(const mg_problem* p, void* workspace, size_t workspace_bytes, int64_t max_pairs,
              int64_t max_partial_items, void* stream) {
  return mg_insert_stages_batched(p, 1, workspace, workspace_bytes, max_pairs, max_partial_items,
                                  MG_STAGE_ALL, stream);
}

int mg_insert_stages(const mg_problem* p, void* workspace, size_t workspace_bytes,
                     int64_t max_pairs, int64_t max_partial_items, int32_t stages, void* stream) {
  return mg_insert_stages_batched(p, 1, workspace, workspace_bytes, max_pairs, max_partial_items,
                                  stages, stream);
}

int mg_check(void* workspace, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!workspace) return fail(MG_ERR_INVALID_ARGUMENT, "null workspace");
  WsHeader h;
  cudaError_t e = cudaMemcpyAsync(&h, workspace, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "mg_check");
  if (h.status & ST_EDGES)
    return fail(MG_ERR_NOT_MONOTONIC, "Channel edges are not monotonic sequence.");
  if (h.status & ST_TIMEOUT)
    return fail(MG_ERR_TIMEOUT, "a device-side pipeline wait expired (results invalid)");
  if (h.status)
    return fail(MG_ERR_WORKSPACE, "workspace capacity exceeded (pairs " +
                                      std::to_string(h.n_pairs) + ", partial items " +
                                      std::to_string(h.n_partial_items) + ")");
  return MG_OK;
}

int mg_flux(const float* cube, int32_t nx, int32_t ny, int32_t nc, int32_t padx, int32_t pady,
            double* flux, void* workspace, size_t workspace_bytes, void* stream) {
  if (!cube || !flux || nx <= 0 || ny <= 0 || nc <= 0 || padx < 0 || pady < 0 ||
      2 * padx >= nx || 2 * pady >= ny)
    return fail(MG_ERR_INVALID_ARGUMENT, "invalid mg_flux arguments");
  size_t need = sizeof(double) * (size_t)flux_chunks(nx, padx) * nc;
  if (!workspace || workspace_bytes < need)
    return fail(MG_ERR_WORKSPACE, "mg_flux workspace too small: need " + std::to_string(need));
  launch_flux(cube, nx, ny, nc, padx, pady, static_cast<double*>(workspace), flux,
              static_cast<cudaStream_t>(stream));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "mg_flux launch");
  return MG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// mg_spectra: materialised spectra (the reference's spectral_model.spectra)
// ---------------------------------------------------------------------------

namespace mg {

__global__ void k_spectra(long long n, int nc, int model, const double* __restrict__ v,
                          const float* __restrict__ sigma, float sigma_const,
                          const double* __restrict__ amp, const double* __restrict__ edges,
                          float* __restrict__ out) {
  const long long total = n * nc;
  const int dec = edges[nc] < edges[0];
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    const long long p = k / nc;
    const int c = (int)(k - p * nc);
    const double vp = v[p];
    const double lo = dec ? edges[c + 1] : edges[c];
    const double hi = dec ? edges[c] : edges[c + 1];
    const float inv_w = (float)(1.0 / fabs(edges[c + 1] - edges[c]));
    float phi;
    if (model == MG_SPECTRUM_DIRAC) {
      phi = (vp >= lo && vp <= hi) ? 1.f : 0.f;  // H(0) = 1 (spectral_models.py:544-570)
    } else {
      const double s = sigma ? (double)sigma[p] : (double)sigma_const;
      const float is = (float)(1.0 / (1.4142135623730951 * s));
      const float vh = (float)vp, vl = (float)(vp - (double)vh);
      const float lh = (float)lo, ll = (float)(lo - (double)lh);
      const float hh = (float)hi, hl = (float)(hi - (double)hh);
      phi = half_erf_diff(((lh - vh) + (ll - vl)) * is, ((hh - vh) + (hl - vl)) * is);
    }
    out[k] = (float)amp[p] * phi * inv_w;
  }
}

}  // namespace mg

extern "C" int mg_spectra(const mg_problem* p, float* out, void* stream) {
  if (!p || !out) return fail(MG_ERR_INVALID_ARGUMENT, "null argument");
  if (p->spectral_model != MG_SPECTRUM_GAUSSIAN && p->spectral_model != MG_SPECTRUM_DIRAC)
    return fail(MG_ERR_INVALID_ARGUMENT, "mg_spectra needs a GAUSSIAN or DIRAC model");
  if (p->nc <= 0 || p->n < 0 || !p->edges) return fail(MG_ERR_INVALID_ARGUMENT, "invalid problem");
  if (p->n == 0) return MG_OK;
  if (!p->v || !p->amp) return fail(MG_ERR_INVALID_ARGUMENT, "v and amp are required");
  long long total = p->n * (long long)p->nc;
  long long blocks = (total + 255) / 256;
  if (blocks > (long long)num_sms() * 64) blocks = (long long)num_sms() * 64;
  k_spectra<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      p->n, p->nc, p->spectral_model, p->v, p->sigma, p->sigma_const,
      p->amp, p->edges, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "mg_spectra launch");
  return MG_OK;
}

// ---------------------------------------------------------------------------
// Launch-shape autotuner (declared in include/martini_gb300.h)
// ---------------------------------------------------------------------------

extern "C" {

void mg_tuning_default(mg_tuning* out) {
  if (!out) return;
  out->kc = 0;
  // the autotuner's choice on the single-cube disc workloads; plans keep
  // ITEMS_PER_SM for their split-K bounds
  out->items_per_sm = ITEMS_PER_SM / 4;
  out->cost_order = 1;
  out->reserved = 0;
}

int mg_tuning_candidates(int32_t form, mg_tuning* out, int32_t cap) {
  std::vector<mg_tuning> c;
  const bool tc = form == MG_FORM_BF16X3 || form == MG_FORM_F16X3 || form == MG_FORM_BF16X6;
  const int kcs[2] = {0, 32};
  const int ipss[3] = {ITEMS_PER_SM, ITEMS_PER_SM / 2, ITEMS_PER_SM / 4};
  for (int kc : kcs) {
    if (kc && !tc) continue;
    for (int ips : ipss)
      for (int order = 1; order >= 0; --order) {
        mg_tuning t;
        t.kc = kc;
        t.items_per_sm = ips;
        t.cost_order = order;
        t.reserved = 0;
        c.push_back(t);
      }
  }
  for (int i = 0; out && i < cap && i < (int)c.size(); ++i) out[i] = c[i];
  return (int)c.size();
}

int mg_tuning_lookup(const mg_problem* probs, int32_t nprob, int64_t max_pairs, mg_tuning* out) {
  mg_tuning_default(out);
  Batch b;
  if (make_batch(probs, nprob, &b, true)) return 0;
  const std::string key = class_key(b, max_pairs);
  std::lock_guard<std::mutex> lock(g_tune_mu);
  const auto it = g_tune_cache.find(key);
  if (it == g_tune_cache.end()) return 0;
  if (out) *out = it->second;
  return 1;
}

int mg_tuning_store(const mg_problem* probs, int32_t nprob, int64_t max_pairs,
                    const mg_tuning* t) {
  if (!t) return fail(MG_ERR_INVALID_ARGUMENT, "null tuning");
  Batch b;
  int rc = make_batch(probs, nprob, &b, true);
  if (rc) return rc;
  if (!shape_ok(b.g.form, *t))
    return fail(MG_ERR_INVALID_ARGUMENT, "launch shape not supported by this form");
  const std::string key = class_key(b, max_pairs);
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune_cache[key] = *t;
  return MG_OK;
}

void mg_tuning_reset(void) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune_cache.clear();
}

int mg_tune_batched(const mg_problem* probs, int32_t nprob, void* workspace,
                    size_t workspace_bytes, int64_t max_pairs, int64_t max_partial_items,
                    int32_t reps, void* stream, mg_tuning* best, float* best_ms) {
  if (!probs || nprob < 1 || !best) return fail(MG_ERR_INVALID_ARGUMENT, "null argument");
  if (reps < 1) reps = 1;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the tuning runs overwrite the cubes: accumulate off
  std::vector<mg_problem> pv(probs, probs + nprob);
  for (mg_problem& p : pv) p.accumulate = 0;
  mg_tuning cand[16];
  const int nc = std::min(16, mg_tuning_candidates(pv[0].form, cand, 16));
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return cuda_fail(cudaGetLastError(), "mg_tune");
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return cuda_fail(cudaGetLastError(), "mg_tune");
  }
  int rc = MG_OK;
  float best_t = 0.f;
  int best_i = -1;
  for (int c = 0; c < nc && rc == MG_OK; ++c) {
    Ws w;
    Batch b;
    rc = run(pv.data(), nprob, workspace, workspace_bytes, s, max_pairs, max_partial_items,
             MG_STAGE_BIN | MG_STAGE_SPEC, true, &w, &b, &cand[c]);
    if (rc) break;
    rc = mg_check(workspace, stream);
    if (rc) break;
    std::vector<float> ms;
    for (int r = 0; r < reps && rc == MG_OK; ++r) {
      cudaEventRecord(e0, s);
      rc = run(pv.data(), nprob, workspace, workspace_bytes, s, max_pairs, max_partial_items,
               MG_STAGE_CONTRACT, true, &w, &b, &cand[c]);
      cudaEventRecord(e1, s);
      if (rc) break;
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        rc = cuda_fail(cudaGetLastError(), "mg_tune timing");
        break;
      }
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      ms.push_back(t);
    }
    if (rc) break;
    rc = mg_check(workspace, stream);
    if (rc) break;
    std::sort(ms.begin(), ms.end());
    const float med = ms[ms.size() / 2];
    if (best_i < 0 || med < best_t) {
      best_t = med;
      best_i = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  *best = cand[best_i];
  if (best_ms) *best_ms = best_t;
  return mg_tuning_store(probs, nprob, max_pairs, best);
}

int mg_tune(const mg_problem* p, void* workspace, size_t workspace_bytes, int64_t max_pairs,
            int64_t max_partial_items, int32_t reps, void* stream, mg_tuning* best,
            float* best_ms) {
  return mg_tune_batched(p, 1, workspace, workspace_bytes, max_pairs, max_partial_items, reps,
                         stream, best, best_ms);
}

}  // extern "C"
