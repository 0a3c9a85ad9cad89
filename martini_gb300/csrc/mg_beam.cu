// Beam convolution of the inserted cube (Martini.convolve_beam,
// martini/martini.py:863-901): every channel of the padded cube convolved
// with the beam image in "same" mode, the pad dropped, and the result scaled
// from Jy/arcsec^2 to Jy/beam by the beam area.
//
// The reference convolves each spatial slice with scipy's fftconvolve; the
// direct form here gives the same sums in FP32:
//   out[i][j] = scale * sum_{a,b} in[i + hx - a][j + hy - b] * K[a][b],
// hx = (kx - 1) / 2, hy = (ky - 1) / 2, zero outside the padded cube, for the
// unpadded pixels only.  A block computes 8 x 16 output pixels of 32
// channels (the cube's channel axis is the fastest, so a warp's lanes read 32
// consecutive floats): the input halo tile and the beam image are staged in
// shared memory; each thread accumulates one output row of 16 pixels for its
// channel.  Beams whose halo tile does not fit read the cube through the
// cache instead.
#include <string>

#include "mg_internal.cuh"

namespace mg {
void set_last_error(const std::string& msg);  // mg_api.cu
}

namespace {

constexpr int BT_I = 8;   // output rows per block (one per warp)
constexpr int BT_J = 16;  // output columns per thread
constexpr int BC = 32;    // channels per block (one per lane)
constexpr size_t kBeamSmemMax = 200 * 1024;

size_t beam_smem(int kx, int ky) {
  return sizeof(float) * ((size_t)(BT_I + kx - 1) * (BT_J + ky - 1) * BC + (size_t)kx * ky);
}

__global__ void __launch_bounds__(BT_I * 32) k_beam_conv(const float* __restrict__ in, int nx,
                                                         int ny, int nc, int px, int py,
                                                         const float* __restrict__ kern, int kx,
                                                         int ky, float scale,
                                                         float* __restrict__ out) {
  extern __shared__ float sm[];
  const int hi = BT_I + kx - 1, hj = BT_J + ky - 1;
  float* s_in = sm;
  float* s_k = sm + (size_t)hi * hj * BC;
  const int hx = (kx - 1) / 2, hy = (ky - 1) / 2;
  const int i0 = px + blockIdx.y * BT_I, j0 = py + blockIdx.x * BT_J, c0 = blockIdx.z * BC;
  const int rb = i0 - hx, cb = j0 - hy;
  const int tid = threadIdx.x;
  const int total = hi * hj * BC;
  for (int e = tid; e < total; e += blockDim.x) {
    const int c = e % BC;
    const int pc = e / BC;
    const int r = pc / hj, q = pc - (pc / hj) * hj;
    const int gi = rb + r, gj = cb + q, gc = c0 + c;
    float v = 0.f;
    if (gi >= 0 && gi < nx && gj >= 0 && gj < ny && gc < nc)
      v = __ldg(in + ((long long)gi * ny + gj) * nc + gc);
    s_in[e] = v;
  }
  for (int t = tid; t < kx * ky; t += blockDim.x) s_k[t] = kern[t];
  __syncthreads();
  const int lane = tid & 31, w = tid >> 5;
  const int i = i0 + w;
  if (i >= nx - px) return;
  float acc[BT_J];
#pragma unroll
  for (int u = 0; u < BT_J; ++u) acc[u] = 0.f;
  for (int a = 0; a < kx; ++a) {
    const float* row = s_in + (size_t)(w + kx - 1 - a) * hj * BC + lane;
    for (int b = 0; b < ky; ++b) {
      const float kv = s_k[a * ky + b];
      const float* col = row + (size_t)(ky - 1 - b) * BC;
#pragma unroll
      for (int u = 0; u < BT_J; ++u) acc[u] = fmaf(col[u * BC], kv, acc[u]);
    }
  }
  const int c = c0 + lane;
  if (c >= nc) return;
  const int nyo = ny - 2 * py;
#pragma unroll
  for (int u = 0; u < BT_J; ++u) {
    const int j = j0 + u;
    if (j < ny - py) out[((long long)(i - px) * nyo + (j - py)) * nc + c] = acc[u] * scale;
  }
}

// Large beams: one output voxel per thread, input through the cache.
__global__ void k_beam_conv_direct(const float* __restrict__ in, int nx, int ny, int nc, int px,
                                   int py, const float* __restrict__ kern, int kx, int ky,
                                   float scale, float* __restrict__ out) {
  const int nxo = nx - 2 * px, nyo = ny - 2 * py;
  const long long total = (long long)nxo * nyo * nc;
  const int hx = (kx - 1) / 2, hy = (ky - 1) / 2;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(e % nc);
    const long long pix = e / nc;
    const int i = px + (int)(pix / nyo), j = py + (int)(pix % nyo);
    float acc = 0.f;
    for (int a = 0; a < kx; ++a) {
      const int gi = i + hx - a;
      if (gi < 0 || gi >= nx) continue;
      for (int b = 0; b < ky; ++b) {
        const int gj = j + hy - b;
        if (gj < 0 || gj >= ny) continue;
        acc = fmaf(__ldg(in + ((long long)gi * ny + gj) * nc + c), __ldg(kern + a * ky + b), acc);
      }
    }
    out[e] = acc * scale;
  }
}

}  // namespace

extern "C" int mg_convolve_beam(const float* cube, int32_t nx, int32_t ny, int32_t nc,
                                int32_t padx, int32_t pady, const float* kernel, int32_t kx,
                                int32_t ky, float scale, float* out, void* stream) {
  if (!cube || !kernel || !out || nx <= 0 || ny <= 0 || nc <= 0 || kx <= 0 || ky <= 0 ||
      (kx % 2) == 0 || (ky % 2) == 0 || padx < 0 || pady < 0 || 2 * padx >= nx ||
      2 * pady >= ny) {
    mg::set_last_error("mg_convolve_beam: invalid arguments (odd kernel sizes, pads < half size)");
    return MG_ERR_INVALID_ARGUMENT;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t smem = beam_smem(kx, ky);
  if (smem <= kBeamSmemMax) {
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_beam_conv, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kBeamSmemMax) != cudaSuccess) {
      mg::set_last_error("mg_convolve_beam: shared memory attribute");
      return MG_ERR_CUDA;
    }
    const dim3 grid((unsigned)((ny - 2 * pady + BT_J - 1) / BT_J),
                    (unsigned)((nx - 2 * padx + BT_I - 1) / BT_I), (unsigned)((nc + BC - 1) / BC));
    k_beam_conv<<<grid, BT_I * 32, smem, s>>>(cube, nx, ny, nc, padx, pady, kernel, kx, ky, scale,
                                              out);
  } else {
    k_beam_conv_direct<<<4096, 256, 0, s>>>(cube, nx, ny, nc, padx, pady, kernel, kx, ky, scale,
                                            out);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    mg::set_last_error(std::string("mg_convolve_beam launch: ") + cudaGetErrorString(e));
    return MG_ERR_CUDA;
  }
  return MG_OK;
}
