// GPU set-up: projection, smoothing lengths, kernel choice, pruning and
// compaction, in FP64 (what Martini.__init__ does on the host).
//
// One thread per particle follows the host steps in the same order:
//   sky position and velocity    martini/sources/sph_source.py:265-326
//   TAN projection, spectral px   sph_source.py:328-362 (datacube.py:438-486)
//   smoothing length in px        martini/sph_kernels.py:235-262
//   adaptive kernel choice        sph_kernels.py:1241-1274
//   footprint range               sph_kernels.py:257-262
//   amplitude, thermal width      spectral_models.py:127-145, :465-485
//   pruning                       martini/martini.py:168-241
// Pass 1 writes keep flags; their scan gives each kept particle its slot;
// pass 2 repeats the arithmetic and writes the kept particles in order.
#include <cmath>
#include <string>

#include "mg_internal.cuh"

namespace mg {
void set_last_error(const std::string& msg);  // mg_api.cu
}

namespace {

using namespace mg;

constexpr double kPiD = 3.14159265358979323846;
constexpr double kDeg = kPiD / 180.0;      // numpy deg2rad factor
constexpr double kRad2Deg = 180.0 / kPiD;  // numpy rad2deg factor
constexpr double kKB = 1.380649e-23;           // J/K (CODATA 2018)
constexpr double kMP = 1.67262192369e-27;      // kg (CODATA 2018)
constexpr double kCkms = 299792.458;           // km/s
constexpr double kHIfreq = 1420405751.768;     // Hz
constexpr double kMHItoJy = 2.36e5;

// Host-computed constants of one set-up (kernel parameters).
struct SetupArgs {
  mg_source src;
  mg_grid grid;
  mg_kernel_choice kc;
  double rot[9];     // R_y(dec) R_z(-ra) applied to row vectors: pos = xyz . rot
  double unit[3];    // direction of (ra, dec)
  int model;
  float sigma_const;
  int prune;
};

struct Derived {
  double x, y, z, v, dist_mpc, h_px, sigma_kms;
  int kidx;
  double size, rescale;
  bool keep;
};

__device__ Derived derive(const SetupArgs& a, long long p) {
  const mg_source& s = a.src;
  const mg_grid& gr = a.grid;
  Derived o;
  const double x0 = s.xyz[3 * p], x1 = s.xyz[3 * p + 1], x2 = s.xyz[3 * p + 2];
  const double u0 = s.vxyz[3 * p], u1 = s.vxyz[3 * p + 1], u2 = s.vxyz[3 * p + 2];
  const double dk = s.distance * 1e3;
  double pos[3], vel[3];
  for (int j = 0; j < 3; ++j) {
    pos[j] = x0 * a.rot[j] + x1 * a.rot[3 + j] + x2 * a.rot[6 + j] + a.unit[j] * dk;
  }
  const double hf = s.h * 100.0 * 1e-3;
  for (int j = 0; j < 3; ++j) {
    vel[j] = u0 * a.rot[j] + u1 * a.rot[3 + j] + u2 * a.rot[6 + j] + hf * pos[j] +
             a.unit[j] * s.vpeculiar;
  }
  const double d = sqrt(pos[0] * pos[0] + pos[1] * pos[1] + pos[2] * pos[2]);
  const double vlos = (pos[0] * vel[0] + pos[1] * vel[1] + pos[2] * vel[2]) / d;
  const double dec_p = asin(pos[2] / d) * kRad2Deg;
  double ra_p = fmod(atan2(pos[1], pos[0]) * kRad2Deg, 360.0);
  if (ra_p < 0.0) ra_p += 360.0;
  o.v = vlos;
  o.dist_mpc = d * 1e-3;
  // TAN projection about the cube's reference point
  const double ar = ra_p * kDeg, dr = dec_p * kDeg;
  const double a0 = gr.crval[0] * kDeg, d0 = gr.crval[1] * kDeg;
  const double cda = cos(ar - a0);
  const double cosc = sin(dr) * sin(d0) + cos(dr) * cos(d0) * cda;
  const double xi = (cos(dr) * sin(ar - a0) / cosc) * kRad2Deg;
  const double eta = ((sin(dr) * cos(d0) - cos(dr) * sin(d0) * cda) / cosc) * kRad2Deg;
  o.x = gr.crpix[0] - 1.0 + xi / gr.cdelt[0];
  o.y = gr.crpix[1] - 1.0 + eta / gr.cdelt[1];
  if (!(cosc > 0.0)) o.x = o.y = nan("");  // behind the projection plane
  const double world = gr.freq_mode ? kHIfreq * (1.0 - vlos / kCkms) : vlos;
  o.z = (gr.crpix[2] - 1.0) + (world - gr.crval[2]) / gr.cdelt[2];
  // smoothing length in pixels and the kernel of the adaptive tuple
  const double hs = s.hsm ? s.hsm[p] : 0.0;
  o.h_px = (atan(hs / (o.dist_mpc * 1e3)) * kRad2Deg) * 3600.0 / gr.px_size_arcsec;
  const mg_kernel_choice& kc = a.kc;
  int idx = 0;
  if (kc.adaptive) {
    idx = -1;
    for (int k = 0; k < kc.n_kernels && idx < 0; ++k) {
      const double hv = o.h_px * kc.rescale[k];
      const bool ok = kc.upper[k] ? (hv <= kc.threshold[k]) : (hv >= kc.threshold[k]);
      if (ok) idx = k;
    }
  }
  o.kidx = idx;
  const int ks = idx < 0 ? 0 : idx;
  o.size = kc.size_in_fwhm[ks];
  o.rescale = kc.rescale[ks];
  // line width (km/s)
  double hw = 0.0;
  o.sigma_kms = 0.0;
  if (a.model == MG_SPECTRUM_GAUSSIAN) {
    o.sigma_kms = s.T ? sqrt(kKB * s.T[p] / kMP) / 1e3 : (double)a.sigma_const;
    hw = o.sigma_kms;
  }
  // pruning (martini/martini.py:168-241)
  const double r = ceil(o.h_px * o.size);
  bool reject = false;
  if (a.prune & MG_PRUNE_SPATIAL) {
    reject = reject || (o.x + r < 0.0) || (o.y + r < 0.0);
    reject = reject || (o.x - r > (double)gr.nx) || (o.y - r > (double)gr.ny);
    reject = reject || isnan(o.x) || isnan(o.y);
  }
  if (a.prune & MG_PRUNE_SPECTRAL) {
    const double hwc = hw / gr.max_channel_width;
    reject = reject || (o.z + 4.0 * hwc < 0.0) || (o.z - 4.0 * hwc > (double)gr.nc);
  }
  if (a.prune & MG_PRUNE_MASS) reject = reject || (s.mHI[p] == 0.0);
  o.keep = !reject;
  return o;
}

__global__ void k_setup_flags(SetupArgs a, int* __restrict__ keep) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < a.src.n;
       p += (long long)gridDim.x * blockDim.x)
    keep[p] = derive(a, p).keep ? 1 : 0;
}

__global__ void k_setup_write(SetupArgs a, const int* __restrict__ keep,
                              const long long* __restrict__ slot, mg_particles out) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < a.src.n;
       p += (long long)gridDim.x * blockDim.x) {
    if (!keep[p]) continue;
    const Derived o = derive(a, p);
    const long long q = slot[p];
    out.x[q] = o.x;
    out.y[q] = o.y;
    out.sm_range[q] = ceil(o.h_px * o.size);
    out.h_eff[q] = (float)(o.h_px * o.rescale);
    if (out.kernel_index) out.kernel_index[q] = (int8_t)o.kidx;
    out.v[q] = o.v;
    if (out.sigma) out.sigma[q] = (float)o.sigma_kms;
    out.amp[q] = a.src.mHI[p] * pow(o.dist_mpc, -2.0) / kMHItoJy;
  }
}

}  // namespace

extern "C" size_t mg_setup_workspace_size(int64_t n) {
  const long long nn = n > 0 ? n : 1;
  size_t b = ((sizeof(int) * (size_t)nn + 255) & ~size_t(255));
  b += ((sizeof(long long) * (size_t)nn + 255) & ~size_t(255));
  b += sizeof(long long) * (size_t)(scan_blocks(nn) + 1);
  return b;
}

extern "C" int mg_setup(const mg_source* src, const mg_grid* grid, const mg_kernel_choice* kc,
                        int32_t spectral_model, float sigma_const, int32_t prune,
                        const mg_particles* out, void* workspace, size_t workspace_bytes,
                        void* stream) {
  if (!src || !grid || !kc || !out) {
    mg::set_last_error("mg_setup: null argument");
    return MG_ERR_INVALID_ARGUMENT;
  }
  if (src->n < 0 || (src->n > 0 && (!src->xyz || !src->vxyz || !src->hsm || !src->mHI)) ||
      kc->n_kernels < 1 || kc->n_kernels > 4 || grid->nx <= 0 || grid->ny <= 0 || grid->nc <= 0 ||
      !(grid->px_size_arcsec > 0.0) || !(grid->max_channel_width > 0.0) || !out->n_kept ||
      (src->n > 0 && (!out->x || !out->y || !out->sm_range || !out->h_eff || !out->v ||
                      !out->amp))) {
    mg::set_last_error("mg_setup: invalid arguments");
    return MG_ERR_INVALID_ARGUMENT;
  }
  if (spectral_model != MG_SPECTRUM_GAUSSIAN && spectral_model != MG_SPECTRUM_DIRAC) {
    mg::set_last_error("mg_setup: GAUSSIAN or DIRAC spectral model");
    return MG_ERR_INVALID_ARGUMENT;
  }
  if (spectral_model == MG_SPECTRUM_GAUSSIAN && !src->T && !(sigma_const > 0.f)) {
    mg::set_last_error("mg_setup: Gaussian lines need T or sigma_const > 0");
    return MG_ERR_INVALID_ARGUMENT;
  }
  const size_t need = mg_setup_workspace_size(src->n);
  if (!workspace || workspace_bytes < need) {
    mg::set_last_error("mg_setup: workspace too small: need " + std::to_string(need));
    return MG_ERR_WORKSPACE;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  SetupArgs a;
  a.src = *src;
  a.grid = *grid;
  a.kc = *kc;
  a.model = spectral_model;
  a.sigma_const = sigma_const;
  a.prune = prune;
  // R_y(dec) R_z(-ra) on row vectors and the unit vector of (ra, dec), in
  // the host's FP64 so every particle uses the same constants
  const double ra = src->ra * kDeg, dec = src->dec * kDeg;
  const double cr = std::cos(ra), sr = std::sin(ra), cd = std::cos(dec), sd = std::sin(dec);
  const double A[9] = {cd, 0.0, sd, 0.0, 1.0, 0.0, -sd, 0.0, cd};
  const double B[9] = {cr, sr, 0.0, -sr, cr, 0.0, 0.0, 0.0, 1.0};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double acc = 0.0;
      for (int k = 0; k < 3; ++k) acc += A[3 * i + k] * B[3 * k + j];
      a.rot[3 * i + j] = acc;
    }
  a.unit[0] = cd * cr;
  a.unit[1] = cd * sr;
  a.unit[2] = sd;
  char* b = static_cast<char*>(workspace);
  const long long nn = src->n > 0 ? src->n : 1;
  int* keep = reinterpret_cast<int*>(b);
  long long* slot = reinterpret_cast<long long*>(b + ((sizeof(int) * (size_t)nn + 255) &
                                                      ~size_t(255)));
  long long* sums = reinterpret_cast<long long*>(
      reinterpret_cast<char*>(slot) + ((sizeof(long long) * (size_t)nn + 255) & ~size_t(255)));
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long blocks = (src->n + 255) / 256;
  if (blocks > (long long)sms * 16) blocks = (long long)sms * 16;
  if (blocks < 1) blocks = 1;
  if (src->n > 0) k_setup_flags<<<(unsigned)blocks, 256, 0, s>>>(a, keep);
  launch_scan(keep, src->n, slot, sums, reinterpret_cast<long long*>(out->n_kept), s);
  if (src->n > 0) k_setup_write<<<(unsigned)blocks, 256, 0, s>>>(a, keep, slot, *out);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    mg::set_last_error(std::string("mg_setup launch: ") + cudaGetErrorString(e));
    return MG_ERR_CUDA;
  }
  return MG_OK;
}
