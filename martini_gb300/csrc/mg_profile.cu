// Global profile: the spatially integrated spectrum of a source
// (GlobalProfile.insert_source_in_spectrum, martini/martini.py:1551-1596).
//
// The reference inserts every particle that survives spectral and mass
// pruning into a one-pixel cube with a DiracDeltaKernel of infinite range at
// pixel (0, 0), so each particle's weight is 1 and the spectrum in Jy is
// spectrum[c] = sum_p S_p(c).  Here that sum is formed directly: one pass
// writes each particle's line record (channel support by the same FP64
// search as the cube path), then blocks own contiguous particle ranges and a
// thread per channel adds S_p(c) in FP64 in particle order; the block
// partials are summed in block order, so the result is deterministic.
#include <string>

#include "mg_internal.cuh"

namespace mg {
void set_last_error(const std::string& msg);  // mg_api.cu
}

namespace {

using namespace mg;

constexpr int PROF_THREADS = 256;
constexpr int PROF_MAX_BLOCKS = 1024;

struct ProfRec {
  float vhi, vlo, inv_s, amp;
  int clo, chi;
};

struct ProfWs {
  WsHeader* hdr;
  float* ehi;
  float* elo;
  float* inv_w;
  int* dec;
  ProfRec* rec;
  double* part;
};

size_t al(size_t x) { return (x + 255) & ~size_t(255); }

int prof_blocks(long long n) {
  long long b = (n + 2047) / 2048;
  if (b > PROF_MAX_BLOCKS) b = PROF_MAX_BLOCKS;
  return (int)(b > 0 ? b : 1);
}

size_t prof_layout(long long n, int nc, size_t* off) {
  size_t o = 0;
  off[0] = o; o += al(sizeof(WsHeader));
  off[1] = o; o += al(sizeof(float) * (size_t)(nc + 1));
  off[2] = o; o += al(sizeof(float) * (size_t)(nc + 1));
  off[3] = o; o += al(sizeof(float) * (size_t)(nc + 1));
  off[4] = o; o += al(sizeof(int));
  off[5] = o; o += al(sizeof(ProfRec) * (size_t)(n > 0 ? n : 1));
  off[6] = o; o += al(sizeof(double) * (size_t)prof_blocks(n) * nc);
  return o;
}

__global__ void k_profile_edges(const double* __restrict__ e, int nc, ProfWs w) {
  const int dec = e[nc] < e[0];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    w.hdr->status = 0;
    *w.dec = dec;
  }
  __syncthreads();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= nc; k += gridDim.x * blockDim.x) {
    const double v = e[k];
    const float hi = (float)v;
    w.ehi[k] = hi;
    w.elo[k] = (float)(v - (double)hi);
    if (k < nc) {
      w.inv_w[k] = (float)(1.0 / fabs(e[k + 1] - e[k]));
      const bool mono = dec ? (e[k + 1] < e[k]) : (e[k + 1] > e[k]);
      if (!mono) atomicOr(&w.hdr->status, ST_EDGES);
    }
  }
}

__global__ void k_profile_rec(long long n, int nc, int model, const double* __restrict__ v,
                              const float* __restrict__ sigma, float sigma_const,
                              const double* __restrict__ amp, const double* __restrict__ edges,
                              ProfWs w) {
  const int dec = *w.dec;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    ProfRec r;
    const double vp = v[p], am = amp[p];
    const double vh = (double)(float)vp;
    r.vhi = (float)vh;
    r.vlo = (float)(vp - vh);
    r.amp = (float)am;
    r.inv_s = 0.f;
    if (model == MG_SPECTRUM_GAUSSIAN) {
      const double s = sigma ? (double)sigma[p] : (double)sigma_const;
      r.inv_s = (float)(1.0 / (1.4142135623730951 * s));
      const double half = 4.5 * 1.4142135623730951 * s;
      channel_range(edges, nc, dec, vp - half, vp + half, r.clo, r.chi);
    } else {
      channel_range(edges, nc, dec, vp, vp, r.clo, r.chi);
    }
    if (am == 0.0 || !isfinite(vp)) {  // mass pruning (martini.py:168-241)
      r.clo = 1;
      r.chi = 0;
    }
    w.rec[p] = r;
  }
}

__global__ void __launch_bounds__(PROF_THREADS) k_profile_sum(long long n, int nc, int model,
                                                              ProfWs w) {
  if (w.hdr->status) return;
  const int dec = *w.dec;
  const long long per = (n + gridDim.x - 1) / gridDim.x;
  const long long p0 = (long long)blockIdx.x * per;
  const long long p1 = p0 + per < n ? p0 + per : n;
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    double acc = 0.0;
    for (long long p = p0; p < p1; ++p) {
      const ProfRec q = w.rec[p];
      if (c < q.clo || c > q.chi) continue;
      PRec r;
      r.clo = q.clo;
      r.chi = q.chi;
      r.vhi = q.vhi;
      r.vlo = q.vlo;
      r.inv_s = q.inv_s;
      r.amp = q.amp;
      acc += (double)channel_spectrum(r, model, c, dec, w.ehi, w.elo, w.inv_w);
    }
    w.part[(long long)blockIdx.x * nc + c] = acc;
  }
}

__global__ void k_profile_final(int nblocks, int nc, ProfWs w, double* __restrict__ spectrum) {
  if (w.hdr->status) return;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += w.part[(long long)b * nc + c];
    spectrum[c] = s;
  }
}

}  // namespace

extern "C" size_t mg_global_profile_workspace_size(int64_t n, int32_t nc) {
  size_t off[7];
  return prof_layout(n, nc > 0 ? nc : 1, off);
}

extern "C" int mg_global_profile(const mg_problem* p, double* spectrum, void* workspace,
                                 size_t workspace_bytes, void* stream) {
  if (!p || !spectrum || !p->edges || p->nc <= 0 || p->n < 0) {
    mg::set_last_error("mg_global_profile: invalid arguments");
    return MG_ERR_INVALID_ARGUMENT;
  }
  if (p->spectral_model != MG_SPECTRUM_GAUSSIAN && p->spectral_model != MG_SPECTRUM_DIRAC) {
    mg::set_last_error("mg_global_profile: GAUSSIAN or DIRAC spectral model");
    return MG_ERR_INVALID_ARGUMENT;
  }
  if (p->n > 0 && (!p->v || !p->amp ||
                   (p->spectral_model == MG_SPECTRUM_GAUSSIAN && !p->sigma &&
                    !(p->sigma_const > 0.f)))) {
    mg::set_last_error("mg_global_profile: v, amp and (Gaussian) sigma are required");
    return MG_ERR_INVALID_ARGUMENT;
  }
  size_t off[7];
  const size_t need = prof_layout(p->n, p->nc, off);
  if (!workspace || workspace_bytes < need) {
    mg::set_last_error("mg_global_profile: workspace too small: need " + std::to_string(need));
    return MG_ERR_WORKSPACE;
  }
  char* b = static_cast<char*>(workspace);
  ProfWs w;
  w.hdr = reinterpret_cast<WsHeader*>(b + off[0]);
  w.ehi = reinterpret_cast<float*>(b + off[1]);
  w.elo = reinterpret_cast<float*>(b + off[2]);
  w.inv_w = reinterpret_cast<float*>(b + off[3]);
  w.dec = reinterpret_cast<int*>(b + off[4]);
  w.rec = reinterpret_cast<ProfRec*>(b + off[5]);
  w.part = reinterpret_cast<double*>(b + off[6]);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(w.hdr, 0, sizeof(WsHeader), s);
  if (e != cudaSuccess) {
    mg::set_last_error(std::string("mg_global_profile: ") + cudaGetErrorString(e));
    return MG_ERR_CUDA;
  }
  // one block, so the edge direction is known before the range checks
  k_profile_edges<<<1, 256, 0, s>>>(p->edges, p->nc, w);
  const int nb = prof_blocks(p->n);
  if (p->n > 0) {
    long long rb = (p->n + 255) / 256;
    if (rb > 4096) rb = 4096;
    k_profile_rec<<<(unsigned)rb, 256, 0, s>>>(p->n, p->nc, p->spectral_model, p->v, p->sigma,
                                               p->sigma_const, p->amp, p->edges, w);
    k_profile_sum<<<nb, PROF_THREADS, 0, s>>>(p->n, p->nc, p->spectral_model, w);
  } else {
    cudaMemsetAsync(w.part, 0, sizeof(double) * (size_t)nb * p->nc, s);
  }
  k_profile_final<<<(p->nc + 255) / 256, 256, 0, s>>>(nb, p->nc, w, spectrum);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    mg::set_last_error(std::string("mg_global_profile launch: ") + cudaGetErrorString(e));
    return MG_ERR_CUDA;
  }
  return MG_OK;
}
