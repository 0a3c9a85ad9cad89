// Split-precision tensor-core contraction (tcgen05, sm_103a).
//
// One persistent CTA (16 warps) per SM walks the work items (tile, K chunk).
// For each stage of KC particles of the tile's list (sorted by kernel class,
// then first channel) the warps build in shared memory
//   A = W[128 pixels][KC particles]        (kernel pixel integrals)
//   B = S[Nw channels][KC particles]       (spectra over the stage's window)
// each split into 16-bit pieces: a hi + lo pair (bf16, or fp16 after exact
// power-of-two scaling), or the exact three-piece BF16 split hi + mid + lo of
// the FP32 value.  The pieces are stored K-major in the no-swizzle canonical
// layout (8-row x 16-byte core matrices; K-direction stride 128 B, row-group
// stride 256 B).  One thread of the MMA warp issues the products per
// 16-particle step -- three for a pair (W_hi S_hi + W_hi S_lo + W_lo S_hi),
// six for three pieces (every cross term down to 2^-16 relative: hh, hm, mh,
// mm, hl, lh) -- as tcgen05.mma (kind::f16, FP32 accumulate) into a TMEM
// accumulator holding the tile's block (128 lanes = pixels, columns =
// channels), at the stage's column window.
//
// Roles: every warp computes one weight task per stage; the build warps also
// copy the next stage's particle parameters (cp.async) and turn them into
// stage parameters; the other warps take the spectrum tasks and the drains.
// Stages are handed over by mbarriers, not block barriers: each warp arrives
// on the stage's mbarrier when its part is written, the MMA thread waits for
// all of them, and tcgen05.commit arrives on the stage buffer's mbarrier when
// the buffer may be written again.  Two shared-memory stage buffers
// alternate; stage parameters rotate over three.
//
// Every stage (three pieces) or every two (pairs) the working accumulator is
// drained (round to nearest) into a master accumulator in the other half of
// TMEM, as the last step of the next stage.  The epilogue reads TMEM with
// tcgen05.ld and writes 128-byte channel runs of each pixel to the cube, or
// to a split-K partial buffer.
//
// Every mbarrier wait has an iteration limit: on expiry the kernel sets
// ST_TIMEOUT, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "mg_internal.cuh"

namespace mg {

constexpr int TC_THREADS = 512;
constexpr int TC_TMEM_COLS = 512;  // whole TMEM: one CTA per SM
constexpr unsigned TC_SPIN_LIMIT = 1u << 26;
// The tensor core's FP32 accumulation does not round to nearest: summing
// many MMAs into one accumulator drifts low (~2^-26 per MMA, relative).  When
// the band fits in half of TMEM the working accumulator is drained every
// TC_DRAIN stages (every stage for the three-piece split) into a master
// accumulator in the other half with round-to-nearest FP32 adds, which bounds
// that drift to the MMAs of one interval; within it the small cross terms
// are issued before the hi x hi products.
constexpr int TC_DRAIN = 2;
// Radial tables up to this many cells (one float4 each, zero cells
// included: every table of mg_kernel_tables.h) are copied to shared memory.
constexpr int KT_SMEM_CELLS = 1025;
constexpr int TC_MASTER_COL = 256;
// 64-particle stages of the three-piece split keep a second working
// accumulator here (blocks of at most 128 channels): K-steps 0-1 accumulate
// at column 0, K-steps 2-3 at this column, so each sees the MMA sequence of
// a 32-particle stage before the drain
constexpr int TC_WB_COL = 128;

// Operand splits: a hi + lo pair of FP16 (scaled) or BF16 pieces, or three
// BF16 pieces hi + mid + lo that represent the FP32 value exactly.
constexpr int SPLIT_F16_2 = 0;
constexpr int SPLIT_BF16_2 = 1;
constexpr int SPLIT_BF16_3 = 2;
__host__ __device__ constexpr int split_parts(int split) { return split == SPLIT_BF16_3 ? 3 : 2; }
__host__ __device__ constexpr bool split_bf16(int split) { return split != SPLIT_F16_2; }
// Particles per stage: 64 by default, 32 as a launch-shape choice.  The
// three-piece split's 64-particle stages fit with blocks of 128 channels.

// Shared memory at the widest band: two stages of A and B pieces plus the
// static arrays must fit in the 227 KB of a CTA.
constexpr size_t tc_stage_bytes(int split, int kc, int nw) {
  return (size_t)split_parts(split) * (kc / 16) * (4096 + 32 * (size_t)nw);
}
constexpr size_t tc_static_bytes(int kc) {
  return (KT_SMEM_CELLS + 257) * 16 + 2 * kc * (sizeof(PRec) + sizeof(int) + sizeof(long long)) +
         4096;
}
static_assert(2 * tc_stage_bytes(SPLIT_F16_2, 64, TC_MASTER_COL) + tc_static_bytes(64) <=
                  227 * 1024,
              "tensor-core kernel shared memory (pairs)");
static_assert(2 * tc_stage_bytes(SPLIT_BF16_3, 32, TC_MASTER_COL) + tc_static_bytes(32) <=
                  227 * 1024,
              "tensor-core kernel shared memory (three pieces)");
static_assert(2 * tc_stage_bytes(SPLIT_BF16_3, 64, TC_WB_COL) + tc_static_bytes(64) <= 227 * 1024,
              "tensor-core kernel shared memory (three pieces, 64-particle stages)");

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ void mbar_arrive(unsigned bar) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(bar)
      : "memory");
}

// Bounded wait; returns false on timeout.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  for (unsigned i = 0; i < TC_SPIN_LIMIT; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// one TcPar (64 bytes: four 16-byte pieces), piece k to dst + k * stride
// bytes (all addresses 16-byte aligned)
__device__ __forceinline__ void cp_async_tpar(void* dst, unsigned stride, const void* src) {
#pragma unroll
  for (int k = 0; k < 4; ++k)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                     smem_u32(dst) + k * stride),
                 "l"(static_cast<const char*>(src) + 16 * k)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major, no swizzle (layout type 0),
// descriptor version 1; lbo = byte stride between the two K core matrices,
// sbo = byte stride between 8-row groups.
__device__ __forceinline__ unsigned long long sdesc(unsigned saddr, unsigned lbo, unsigned sbo) {
  unsigned long long d = 0;
  d |= (unsigned long long)((saddr & 0x3FFFFu) >> 4);
  d |= (unsigned long long)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (unsigned long long)((sbo >> 4) & 0x3FFFu) << 32;
  d |= 1ull << 46;
  return d;
}

// Instruction descriptor, kind::f16: D FP32; A, B both BF16 (format 1) or
// both FP16 (format 0); both K-major; N >> 3 at bit 17, M >> 4 at bit 24.
__device__ __forceinline__ unsigned idesc_f16kind(int M, int N, bool bf16) {
  const unsigned fmt = bf16 ? 1u : 0u;
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((unsigned)(N >> 3) << 17) |
         ((unsigned)(M >> 4) << 24);
}

__device__ __forceinline__ void umma(unsigned d_tmem, unsigned long long a, unsigned long long b,
                                     unsigned idesc, unsigned acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void umma_commit(unsigned bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}

__device__ __forceinline__ void tmem_ld32(unsigned taddr, unsigned (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
      "%28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_st32_zero(unsigned taddr) {
  const unsigned z = 0u;
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
      "%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
      "%1};" ::"r"(taddr),
      "r"(z)
      : "memory");
}

__device__ __forceinline__ void tmem_ld16(unsigned taddr, unsigned (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_st16(unsigned taddr, const unsigned (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15, %16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
      "r"(r[15])
      : "memory");
}

__device__ __forceinline__ void tmem_st16_zero(unsigned taddr) {
  const unsigned z = 0u;
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
      "%1, %1, %1, %1, %1, %1};" ::"r"(taddr),
      "r"(z)
      : "memory");
}

__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// hi + lo split of a float into two 16-bit floats.
template <bool BF16>
__device__ __forceinline__ void split2(float v, unsigned short& hi, unsigned short& lo) {
  if (BF16) {
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    hi = __bfloat16_as_ushort(h);
    lo = __bfloat16_as_ushort(__float2bfloat16_rn(v - __bfloat162float(h)));
  } else {
    const __half h = __float2half_rn(v);
    hi = __half_as_ushort(h);
    lo = __half_as_ushort(__float2half_rn(v - __half2float(h)));
  }
}

__device__ __forceinline__ TcPar empty_tpar() {
  TcPar z;
  z.xi = z.yi = 0;
  z.xf = z.yf = z.k2 = z.scale = 0.f;
  z.kind = 0;
  z.clo = 1;
  z.chi = 0;
  z.ilo = 0; z.ihi = -1; z.jlo = 0; z.jhi = -1;
  z.pad_ = 0;
  z.soff = 0;
  return z;
}

struct ItemTC {
  int seg, gal, tile, tx, ty, kc, nk;  // tile: within the cube
  int c0;  // first channel of the segment's block
  long long lbeg;
  int lcount;
};

__device__ __forceinline__ ItemTC decode_tc(const Geo& g, const Ws& w, long long item, int kch) {
  const int a = w.item_seg[item];
  ItemTC it;
  it.seg = a;
  it.gal = find_gal(w.gs0, g.ngal, a);
  const Gal& G = w.gal[it.gal];
  const int ls = a - G.seg0;
  it.tile = ls / G.ncb;
  it.c0 = (ls - it.tile * G.ncb) * G.width;
  it.tx = it.tile / G.nty;
  it.ty = it.tile - it.tx * G.nty;
  it.nk = w.seg_items[a];
  it.kc = (int)(item - w.item_off[a]);
  it.lbeg = w.seg_lo[a] + (long long)it.kc * kch;
  const long long left = w.seg_hi[a] - it.lbeg;
  it.lcount = (int)(left < kch ? left : kch);
  return it;
}

__device__ __forceinline__ PRec empty_rec() {
  PRec z;
  z.ilo = 0; z.ihi = -1; z.jlo = 0; z.jhi = -1; z.clo = 1; z.chi = 0;
  z.kslot = 0; z.xi = z.yi = 0; z.xf = z.yf = 0.f; z.h = 1.f; z.inv_h2 = 1.f;
  z.vhi = z.vlo = 0.f; z.inv_s = 0.f; z.amp = 0.f; z.flags = 0;
  return z;
}

// Cubic-spline profile f(s), s = R^2 (doubled offsets), from its cells in R
// and A = sqrt(1 - R^2) (same cells and coefficients as kt_eval), written
// without branches so that the four pixels of a lane evaluate in parallel.
// Returns 0 outside the support.
__device__ __forceinline__ float kt_eval_cubic(const KTableInfo& inf,
                                               const float4* __restrict__ tab, float s) {
  const float R = s * rsqrtf(fmaxf(s, 1e-30f));
  const int r = (s > 1.f) ? 2 : (R >= inf.split_r ? 1 : 0);
  const KRegion g = inf.reg[r];
  const float a2 = fmaxf(1.f - s, 0.f);
  const float v = g.var ? a2 * rsqrtf(fmaxf(a2, 1e-30f)) : R;
  const float u = (v - g.lo) * g.cells_per_unit;
  const int c = min(max(__float2int_rz(u), 0), g.ncell - 1);
  const float t = u - (float)c;
  static_assert(KT_DEG == 3, "one float4 of coefficients per cell");
  const float4 cf = tab[g.first + c];
  const float f = fmaf(fmaf(fmaf(cf.w, t, cf.z), t, cf.y), t, cf.x);
  return s < inf.smax ? f : 0.f;
}

// 16-bit hi/lo halves of two values packed as (first | second << 16).
template <bool BF16>
// Packed conversions round each element as the scalar ones do (same bits
// as split2 per value), with one conversion per pair.
__device__ __forceinline__ void split_pair(float a, float b, unsigned& hi, unsigned& lo) {
  if (BF16) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const unsigned*>(&h);
    lo = *reinterpret_cast<const unsigned*>(&l);
  } else {
    const __half2 h = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const unsigned*>(&h);
    lo = *reinterpret_cast<const unsigned*>(&l);
  }
}

// Exact three-piece BF16 split of two FP32 values, packed as (first |
// second << 16) per piece.  hi keeps the top 16 bits of the float (sign,
// exponent and 7 stored mantissa bits: a BF16 by truncation); r = v - hi is
// exact (same sign and binade) and holds the remaining 16 mantissa bits; mid
// is r truncated the same way and lo = r - mid is exact with at most 8
// significant bits, so it is a BF16 too.  hi + mid + lo == v for every
// normal float (the pieces carry the exponent range of FP32).
__device__ __forceinline__ void split3_pair(float a, float b, unsigned& hi, unsigned& mid,
                                            unsigned& lo) {
  const unsigned ua = __float_as_uint(a), ub = __float_as_uint(b);
  hi = __byte_perm(ua, ub, 0x7632);
  const float ra = a - __uint_as_float(ua & 0xFFFF0000u);
  const float rb = b - __uint_as_float(ub & 0xFFFF0000u);
  const unsigned ura = __float_as_uint(ra), urb = __float_as_uint(rb);
  mid = __byte_perm(ura, urb, 0x7632);
  const float la = ra - __uint_as_float(ura & 0xFFFF0000u);
  const float lb = rb - __uint_as_float(urb & 0xFFFF0000u);
  lo = __byte_perm(__float_as_uint(la), __float_as_uint(lb), 0x7632);
}

// The pieces of two values (particles q, q + 1) stored at byte offset off of
// each piece's tile; piece k's tile starts at base + k * piece_bytes.
template <int SPLIT>
__device__ __forceinline__ void store_split(float a, float b, unsigned char* base,
                                            unsigned piece_bytes, unsigned off) {
  if constexpr (SPLIT == SPLIT_BF16_3) {
    unsigned h, m, l;
    split3_pair(a, b, h, m, l);
    *reinterpret_cast<unsigned*>(base + off) = h;
    *reinterpret_cast<unsigned*>(base + piece_bytes + off) = m;
    *reinterpret_cast<unsigned*>(base + 2 * piece_bytes + off) = l;
  } else {
    unsigned h, l;
    split_pair<split_bf16(SPLIT)>(a, b, h, l);
    *reinterpret_cast<unsigned*>(base + off) = h;
    *reinterpret_cast<unsigned*>(base + piece_bytes + off) = l;
  }
}

// Coefficients of table cell floor(u) (u >= 0) from shared memory, and the
// fraction t: base32 is the shared address of the table minus 2^23 cells,
// so the sum of 2^23 and floor(u) left in the float's bits by kt_floor's
// rounded add indexes the cell directly (32-bit shared-window arithmetic).
__device__ __forceinline__ float4 kt_cell_smem(unsigned base32, float u, float& t) {
  const float v = __fadd_rd(u, 8388608.f);
  t = u - (v - 8388608.f);
  float4 c;
  asm("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
      : "=f"(c.x), "=f"(c.y), "=f"(c.z), "=f"(c.w)
      : "r"(base32 + (__float_as_uint(v) << 4)));
  return c;
}

__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// One value's 16-bit hi and lo halves packed as hi | lo << 16 (the same
// roundings as split_pair).
template <bool BF16>
__device__ __forceinline__ unsigned split_one(float a) {
  unsigned hi, lo;
  split_pair<BF16>(a, 0.f, hi, lo);
  return (hi & 0xFFFFu) | (lo << 16);
}

// Exact power-of-two scale of one cube's spectra in the FP16 split form:
// the largest |S| bound -> 2^14.
__device__ __forceinline__ float spec_scale(const GalState& gs, int model) {
  const float sb = __uint_as_float(gs.sbound_bits) *
                   (model == MG_SPECTRUM_TABLE ? 1.f : __uint_as_float(gs.invw_bits));
  return sb > 0.f ? exp2f(14.f - ceilf(log2f(sb))) : 1.f;
}

// erfc(z) for z >= 0 by the Chebyshev-fitted form of Press, Teukolsky,
// Vetterling & Flannery, Numerical Recipes (2nd ed., section 6.2, "erfcc"):
// erfc(z) = t exp(-z^2 + P(t)), t = 1 / (1 + z / 2), fractional error below
// 1.2e-7 for all z >= 0.  Cheaper than the library erfcf on the producer
// path; the FP32 contraction form keeps erff/erfcf.
__device__ __forceinline__ float erfc_nr(float z) {
  const float t = __frcp_rn(fmaf(0.5f, z, 1.f));
  float p = 0.17087277f;
  p = fmaf(p, t, -0.82215223f);
  p = fmaf(p, t, 1.48851587f);
  p = fmaf(p, t, -1.13520398f);
  p = fmaf(p, t, 0.27886807f);
  p = fmaf(p, t, -0.18628806f);
  p = fmaf(p, t, 0.09678418f);
  p = fmaf(p, t, 0.37409196f);
  p = fmaf(p, t, 1.00002368f);
  p = fmaf(p, t, -1.26551223f);
  return t * __expf(fmaf(-z, z, p));
}

// erfc(|u|) and sign of u at channel edge ge for a Gaussian line.
__device__ __forceinline__ void edge_term(const PRec& r, int ge, const float* ehi,
                                          const float* elo, float& cval, bool& pos) {
  const float u = ((ehi[ge] - r.vhi) + (elo[ge] - r.vlo)) * r.inv_s;
  pos = u >= 0.f;
  cval = erfc_nr(fabsf(u));
}

// 0.5 [erf(b) - erf(a)] (a < b) from erfc(|a|), erfc(|b|) and the signs.
__device__ __forceinline__ float half_diff_from_c(float ca, bool pa, float cb, bool pb) {
  const float both = 0.5f * (pa ? ca - cb : cb - ca);
  return (pa || !pb) ? both : fmaf(-0.5f, ca + cb, 1.f);
}

// B = S for particles (q, q + 1) over the window channels, lines evaluated
// here (no spectrum store).  A Gaussian line needs erfc at every window edge
// once: in step m lane l evaluates edge 31 m + l and channel 31 m + l
// (l < 31) takes its upper index edge from lane l + 1, so each step covers
// 31 channels with no repeated evaluation.
template <int SPLIT>
__device__ __forceinline__ void produce_s_pair(const PRec& r0, const PRec& r1, bool v0, bool v1,
                                               int q, int w0, int nw, int nc, int dec, int model,
                                               const float* ehi, const float* elo,
                                               const float* inv_w, const float* spectra,
                                               int pid0, int pid1, int lane, float ss,
                                               unsigned char* b0, unsigned b_bytes) {
  const unsigned qoff = (unsigned)(q >> 4) * ((unsigned)nw * 32u) +
                        (unsigned)((q >> 3) & 1) * 128u + (unsigned)(q & 7) * 2u;
  const bool gauss = model == MG_SPECTRUM_GAUSSIAN;
  const int step = gauss ? 31 : 32;
  for (int base = 0; base < nw; base += step) {  // warp-uniform
    const int n = base + lane;
    const int c = w0 + n;
    float s0 = 0.f, s1 = 0.f;
    if (gauss) {
      float ca0 = 0.f, ca1 = 0.f;
      bool pa0 = true, pa1 = true;
      if (n <= nw && c <= nc) {
        if (v0) edge_term(r0, c, ehi, elo, ca0, pa0);
        if (v1) edge_term(r1, c, ehi, elo, ca1, pa1);
      }
      const float cb0 = __shfl_down_sync(0xffffffffu, ca0, 1);
      const float cb1 = __shfl_down_sync(0xffffffffu, ca1, 1);
      const bool pb0 = __shfl_down_sync(0xffffffffu, (int)pa0, 1) != 0;
      const bool pb1 = __shfl_down_sync(0xffffffffu, (int)pa1, 1) != 0;
      if (lane < 31 && n < nw && c < nc) {
        const float iw = inv_w[c] * ss;
        // edge c is the channel's lower edge for increasing edges, the upper
        // one for decreasing edges
        const float phi0 = dec ? half_diff_from_c(cb0, pb0, ca0, pa0)
                               : half_diff_from_c(ca0, pa0, cb0, pb0);
        const float phi1 = dec ? half_diff_from_c(cb1, pb1, ca1, pa1)
                               : half_diff_from_c(ca1, pa1, cb1, pb1);
        s0 = (v0 && c >= r0.clo && c <= r0.chi) ? r0.amp * iw * phi0 : 0.f;
        s1 = (v1 && c >= r1.clo && c <= r1.chi) ? r1.amp * iw * phi1 : 0.f;
      }
    } else if (n < nw && c < nc) {
      if (model == MG_SPECTRUM_DIRAC) {
        if (v0 && c >= r0.clo && c <= r0.chi) s0 = r0.amp * inv_w[c] * ss;
        if (v1 && c >= r1.clo && c <= r1.chi) s1 = r1.amp * inv_w[c] * ss;
      } else {
        if (v0 && c >= r0.clo && c <= r0.chi) s0 = spectra[(long long)pid0 * nc + c] * ss;
        if (v1 && c >= r1.clo && c <= r1.chi) s1 = spectra[(long long)pid1 * nc + c] * ss;
      }
    }
    if (n < nw && (!gauss || lane < 31)) {
      const unsigned off = qoff + (unsigned)(n >> 3) * 256u + (unsigned)(n & 7) * 16u;
      store_split<SPLIT>(s0, s1, b0, b_bytes, off);
    }
  }
}

// Row lengths of the spectrum store: support channels of each particle
// that reaches the cube (0 otherwise).  Written over the per-particle pair
// counts, which the binning stage no longer needs.
__global__ void k_spec_count(Geo g, Ws w) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.n;
       p += (long long)gridDim.x * blockDim.x) {
    const PRec& r = w.rec[p];
    const int ilo = r.ilo, ihi = r.ihi, clo = r.clo, chi = r.chi;
    w.npairs[p] = ilo <= ihi ? chi - clo + 1 : 0;
  }
}

// Gaussian line of each particle over its support, once per particle (the
// producer would otherwise evaluate it at every tile the particle touches):
// one warp per particle, the same shared-edge arithmetic as the producer, so
// the contraction gives the same bits with or without the store.  Row p
// starts at pair_off[p] (exclusive scan of the row lengths).
// What k_spec_eval needs of one particle (independent loads by index, so
// the next particle's are in flight while this one's line is evaluated).
struct SpecIn {
  int cnt, clo;
  long long off;
  float vhi, vlo, inv_s, amp;
};

__device__ __forceinline__ SpecIn spec_in(const Ws& w, long long p) {
  SpecIn q;
  q.cnt = w.npairs[p];
  q.off = w.pair_off[p];
  const PRec& r = w.rec[p];
  q.clo = r.clo;
  q.vhi = r.vhi;
  q.vlo = r.vlo;
  q.inv_s = r.inv_s;
  q.amp = r.amp;
  return q;
}

__global__ void k_spec_eval(Geo g, Ws w) {
  const bool form_bf16 = g.form == MG_FORM_BF16X3;
  const bool form_fp32 = g.form == MG_FORM_BF16X6;  // the contraction splits the FP32 value
  const bool fits = w.hdr->n_spec <= w.cap_spec;
  // read by the contraction, which runs after this whole kernel
  if (blockIdx.x == 0 && threadIdx.x == 0) w.hdr->spec_ready = fits ? 1 : 0;
  if (!fits) return;
  const int lane = threadIdx.x & 31;
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  long long p = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  if (p >= g.n) return;
  SpecIn cur = spec_in(w, p);
  // the cube of the warp's particles: its edges, direction and scale, reloaded
  // only when the cube changes (a cube's particles are contiguous and p only
  // grows)
  int gk_c = -1, dec = 0, nc = 0;
  long long gp1 = -1;  // first particle past cube gk_c
  const float *ehi = nullptr, *elo = nullptr, *inv_w = nullptr;
  float ss = 1.f;
  for (; p < g.n; p += nwarps) {
    const long long pn = p + nwarps;
    SpecIn nxt;
    if (pn < g.n) nxt = spec_in(w, pn);  // warp-uniform
    if (cur.cnt > 0) {                    // warp-uniform
      const int cnt = cur.cnt;
      if (gk_c < 0 || p >= gp1) {
        gk_c = find_gal(w.gp0, g.ngal, p);
        const Gal& G = w.gal[gk_c];
        gp1 = w.gp0[gk_c + 1];
        dec = w.gst[gk_c].dec;
        nc = G.nc;
        ehi = w.ehi + G.edge0;
        elo = w.elo + G.edge0;
        inv_w = w.inv_w + G.edge0;
        ss = (form_bf16 || form_fp32) ? 1.f : spec_scale(w.gst[gk_c], g.spectral_model);
      }
      PRec r;
      r.vhi = cur.vhi;
      r.vlo = cur.vlo;
      r.inv_s = cur.inv_s;
      unsigned* out = w.spec + cur.off;
      for (int base = 0; base < cnt; base += 31) {
        const int m = base + lane;
        const int c = cur.clo + m;
        float ca = 0.f;
        bool pa = true;
        if (m <= cnt && c <= nc) edge_term(r, c, ehi, elo, ca, pa);
        const float cb = __shfl_down_sync(0xffffffffu, ca, 1);
        const bool pb = __shfl_down_sync(0xffffffffu, (int)pa, 1) != 0;
        if (lane < 31 && m < cnt) {
          const float phi =
              dec ? half_diff_from_c(cb, pb, ca, pa) : half_diff_from_c(ca, pa, cb, pb);
          const float val = (cur.amp * inv_w[c] * phi) * ss;
          out[m] = form_fp32   ? __float_as_uint(val)
                   : form_bf16 ? split_one<true>(val)
                               : split_one<false>(val);
        }
      }
    }
    cur = nxt;
  }
}

// ---------------------------------------------------------------------------
// Stage parameters and the operand producers.
//
// When a stage's records arrive, the record warps turn each particle into a
// compact StagePar (tile-relative position, kernel constants, footprint box)
// and SPar (its spectrum-store row).  The producers read these as warp-wide
// broadcasts and write operand rows of 8 particles (16 bytes per piece), so
// a quarter-warp stores 128 contiguous bytes: no shared-memory bank
// conflicts.
//
// Weights: warp w takes particle group g8 = w % (KC / 8) (8 particles) and
// pixel group pg = w / (KC / 8); lane l holds PXL = KC / 32 pixels,
// m = 32 (pg PXL + k) + l, i.e. tile row 2 (pg PXL + k) + l / 16 and column
// l % 16.  A particle whose footprint rows miss the warp's 2 PXL rows is
// skipped by the whole warp (exact: the reference weighs only pixels in the
// box).  Spectra: one task per (32-channel chunk of the stage window,
// 8-particle group); lane l takes window channel 32 chunk + l.
// ---------------------------------------------------------------------------

constexpr int WK_NONE = 0;   // contributes nothing to this segment
constexpr int WK_TAB = 1;    // radial kernel, s-cells in shared memory
constexpr int WK_TABG = 2;   // radial kernel, s-cells in global memory
constexpr int WK_CUBIC = 3;  // cubic spline (cells in R and sqrt(1 - R^2))
constexpr int WK_GAUSS = 4;
constexpr int WK_DIRAC = 5;
constexpr int WK_COVER = 8;  // the box holds the support in rows and columns: no box test

struct StagePar {
  float dxr, xf;  // xi - i0 (exact), x - xi
  float dyr, yf;  // yi - j0 (exact), y - yi
  float k2;       // TAB/TABG: inv_h2 * cells per unit s; CUBIC: 4 inv_h2; GAUSS: 1 / (h sigma)
  float scale;    // TAB/TABG/CUBIC: table scale * inv_h2 * sw; GAUSS: 0.25 / gnorm * sw;
                  // DIRAC: sw
  int kind;       // WK_* | WK_COVER, kernel slot << 8, kernel type << 12
  int mask;       // footprint box within the tile: row bits 0-7, column bits 8-23 (all set
                  // when the box holds the support: no test needed; none for WK_NONE)
};
static_assert(sizeof(StagePar) == 32, "two 16-byte broadcasts per particle");

struct SPar {
  long long soff;  // spectrum-store row of the particle (cp.async target)
  int clo;         // first support channel
  unsigned n;      // support channels in the row; 0: contributes nothing
};

// The tile-independent parameters of one particle (k_tc_params): kernel
// kind and constants with the cube's operand scale sw, position, box,
// support.  A particle that reaches no pixel or no channel gets kind 0.
__device__ __forceinline__ TcPar tc_param(const PRec& r, const KSpec* ks, int ktab_type, float sw,
                                          long long soff) {
  const bool valid = r.ilo <= r.ihi && r.jlo <= r.jhi && r.clo <= r.chi;
  const KSpec kk = ks[r.kslot];
  const int t = kk.type;
  int kind = WK_NONE;
  float k2 = 0.f, scale = 0.f;
  if (valid) {
    if (t == MG_KERNEL_DIRAC) {
      kind = WK_DIRAC;
      scale = sw;
    } else if (t == MG_KERNEL_GAUSSIAN) {
      kind = WK_GAUSS;
      k2 = 1.f / (r.h * 0.42466090014400953f);  // 1 / (h sigma_FWHM)
      scale = 0.25f / kk.gnorm * sw;
    } else {
      const KTableInfo& inf = kt_info[t];
      if (t == MG_KERNEL_CUBIC_SPLINE) {
        kind = WK_CUBIC;
        k2 = 4.f * r.inv_h2;
      } else {
        kind = t == ktab_type ? WK_TAB : WK_TABG;
        k2 = r.inv_h2 * inf.reg[0].cells_per_unit;
      }
      scale = inf.scale * r.inv_h2 * sw;
      if ((r.flags & PREC_ROWS_COVER) && (r.flags & PREC_COLS_COVER)) kind |= WK_COVER;
    }
  }
  TcPar q;
  q.xi = r.xi;
  q.yi = r.yi;
  q.xf = r.xf;
  q.yf = r.yf;
  q.k2 = k2;
  q.scale = scale;
  q.kind = kind == WK_NONE ? 0 : (kind | (r.kslot << 8) | (t << 12));
  q.clo = r.clo;
  q.ilo = r.ilo;
  q.ihi = r.ihi;
  q.jlo = r.jlo;
  q.jhi = r.jhi;
  q.chi = r.chi;
  q.pad_ = 0;
  q.soff = soff;
  return q;
}

// StagePar / SPar of one particle of a stage, tile-relative (listed: in this
// stage; a particle whose line misses the segment's block contributes
// nothing).  Returns the WK_* kind and flags.
__device__ __forceinline__ int build_stage(const TcPar& t, bool listed, int i0, int j0, int cb0,
                                           int cb1, StagePar& P, SPar& S) {
  const bool valid = listed && t.kind != 0 && t.chi >= cb0 && t.clo <= cb1;
  const int kind = valid ? t.kind : 0;
  P.dxr = (float)(t.xi - i0);
  P.xf = t.xf;
  P.dyr = (float)(t.yi - j0);
  P.yf = t.yf;
  // an empty slot: zero k2 and scale (u = 0 and a zero weight in every path)
  P.k2 = valid ? t.k2 : 0.f;
  P.scale = valid ? t.scale : 0.f;
  P.kind = kind;
  // box rows / columns within the tile as bit masks
  unsigned rows = 0u, cols = 0u;
  if (valid) {
    const int a = max(t.ilo - i0, 0), b = min(t.ihi - i0, TILE_I - 1);
    const int c = max(t.jlo - j0, 0), d = min(t.jhi - j0, TILE_J - 1);
    if (a <= b) rows = ((2u << b) - 1u) & ~((1u << a) - 1u);
    if (c <= d) cols = ((2u << d) - 1u) & ~((1u << c) - 1u);
    if (kind & WK_COVER) {
      // rows outside the box still need no test (the table's zero cell), but
      // the warps whose rows miss the box skip it: keep the row bits
      cols = 0xFFFFu;
    }
  }
  P.mask = (int)(rows | cols << 8);
  S.soff = t.soff;
  S.clo = t.clo;
  S.n = valid ? (unsigned)(t.chi - t.clo + 1) : 0u;
  return kind;
}

// Group paths of the weight producers.
constexpr int GP_GENERAL = 0;  // each particle takes its kind's path
constexpr int GP_MIXED = 1;    // table / Dirac / empty: one branch-free block with box tests
constexpr int GP_COVERED = 2;  // table kernels whose boxes hold their supports, or empty
constexpr int GP_GAUSS = 3;    // Gaussian kernels or empty: one branch-free block
constexpr int GP_DIRAC = 4;    // Dirac kernels or empty: the box test picks the scale

__device__ __forceinline__ float horner3(const float4& cf, float t) {
  return fmaf(fmaf(fmaf(cf.w, t, cf.z), t, cf.y), t, cf.x);
}

// GaussianKernel pixel integral (sph_kernels.py:994-1044):
// 0.25 erf(zmax / sqrt 2) (erf(x1) - erf(x0)) (erf(y1) - erf(y0)) / norm.
// gauss_factor: the erf difference of lane's line of pixels -- column `lane`
// for lanes 0-15, row wr0 + (lane - 16) mod 2 PXL for lanes 16 and up -- to
// be shared by shuffles (an empty slot, k2 = 0, gives 0).
template <int PXL>
__device__ __forceinline__ float gauss_factor(const StagePar& P, int wr0, int lane) {
  const float sc = P.k2 * 0.70710678118654752f;  // 1 / (h sqrt(2) sigma)
  const float d = lane < 16 ? (P.dyr - (float)lane) + P.yf
                            : (P.dxr - (float)(wr0 + ((lane - 16) & (2 * PXL - 1)))) + P.xf;
  return erff((d + 0.5f) * sc) - erff((d - 0.5f) * sc);
}
// The truncation factor erf(zmax / sqrt 2) at squared offset q2 (pixel units)
// from its cubic cells in zmax, in shared memory at gtab_s32 (minus 2^23
// cells, as kt_cell_smem takes it); t2 = truncate^2, ihs2 = 1 / (h sigma)^2.
__device__ __forceinline__ float gauss_trunc(unsigned gtab_s32, float q2, float ihs2, float t2) {
  const float z2 = fmaxf(fmaf(-q2, ihs2, t2), 0.f);  // truncate^2 - q^2
  const float u = fminf(sqrt_approx(z2) * GT_CELLS_PER_UNIT, (float)GT_NCELL);
  float t;
  const float4 cf = kt_cell_smem(gtab_s32, u, t);
  return horner3(cf, t);
}

// Weights of one stage particle at a lane's PXL pixels (tile rows il[k],
// column jl).  Warp-uniform: every lane takes the same branch.
template <int PXL>
__device__ __forceinline__ void w_particle(const StagePar& P, const KSpec* ks, unsigned ktab_s32,
                                           unsigned gtab_s32, float ucap, int wr0, const int (&il)[PXL],
                                           const float (&ilf)[PXL], int jl, float jlf, int lane,
                                           float (&w)[PXL]) {
#pragma unroll
  for (int k = 0; k < PXL; ++k) w[k] = 0.f;
  const int kind = P.kind & 7;
  const unsigned rows = (unsigned)P.mask & 0xFFu;
  // the warp's rows are wr0 .. wr0 + 2 PXL - 1
  if (kind == WK_NONE || ((rows >> wr0) & ((1u << (2 * PXL)) - 1u)) == 0u) return;
  const bool jin = ((unsigned)P.mask >> (8 + jl)) & 1u;
  bool in[PXL];
#pragma unroll
  for (int k = 0; k < PXL; ++k) in[k] = jin && ((rows >> il[k]) & 1u);
  const float dy = (P.dyr - jlf) + P.yf;
  float dx[PXL];
#pragma unroll
  for (int k = 0; k < PXL; ++k) dx[k] = (P.dxr - ilf[k]) + P.xf;
  if (kind == WK_TAB) {
    // cells in s = R^2 in shared memory; u clamped onto the zero cell past
    // the support, so a covered particle needs no box test
    const float dy2k = dy * dy * P.k2;
    const bool cover = (P.kind & WK_COVER) != 0;
    const unsigned base32 = ktab_s32 - (0x4B000000u << 4);
#pragma unroll
    for (int k = 0; k < PXL; ++k) {
      float u = fminf(fmaf(dx[k] * P.k2, dx[k], dy2k), ucap);
      if (!cover && !in[k]) u = ucap;
      float t;
      const float4 cf = kt_cell_smem(base32, u, t);
      w[k] = horner3(cf, t) * P.scale;
    }
    return;
  }
  if (kind == WK_GAUSS) {
    // column factors from lanes 0-15, the warp's row factors from lanes
    // 16 .. 16 + 2 PXL - 1, shared by shuffles
    const float e = gauss_factor<PXL>(P, wr0, lane);
    const float ey = __shfl_sync(0xffffffffu, e, jl);
    const KSpec kk = ks[(P.kind >> 8) & 0xF];
    const float t2 = kk.truncate * kk.truncate;
    const float ihs2 = P.k2 * P.k2;
    const float dy2 = dy * dy;
    const float c = ey * P.scale;
#pragma unroll
    for (int k = 0; k < PXL; ++k) {
      const float ex = __shfl_sync(0xffffffffu, e, 16 + (il[k] - wr0));
      const float T = gauss_trunc(gtab_s32, fmaf(dx[k], dx[k], dy2), ihs2, t2);
      w[k] = in[k] ? T * ex * c : 0.f;
    }
    return;
  }
  if (kind == WK_DIRAC) {
#pragma unroll
    for (int k = 0; k < PXL; ++k) w[k] = in[k] ? P.scale : 0.f;
    return;
  }
  const int type = (P.kind >> 12) & 0xF;
  const KTableInfo& inf = kt_info[type];
  const bool cover = (P.kind & WK_COVER) != 0;
  if (kind == WK_CUBIC) {
    const float4* tab = reinterpret_cast<const float4*>(kt_coef);
    const float dy2 = dy * dy;
#pragma unroll
    for (int k = 0; k < PXL; ++k) {
      const float f = kt_eval_cubic(inf, tab, fmaf(dx[k], dx[k], dy2) * P.k2);
      w[k] = (cover || in[k]) ? f * P.scale : 0.f;
    }
    return;
  }
  // WK_TABG: another radial kernel's s-cells from global memory
  const float4* tab = reinterpret_cast<const float4*>(kt_coef) + inf.reg[0].first;
  const float gcap = (float)inf.reg[0].ncell;
  const float dy2k = dy * dy * P.k2;
#pragma unroll
  for (int k = 0; k < PXL; ++k) {
    float u = fminf(fmaf(dx[k] * P.k2, dx[k], dy2k), gcap);
    if (!cover && !in[k]) u = gcap;
    float t;
    const int cell = kt_floor(u, t);
    w[k] = horner3(__ldg(tab + cell), t) * P.scale;
  }
}

// Pieces of 8 consecutive particles' values (one core-matrix row), stored as
// one 16-byte row per piece at byte offset off of each piece's tile.
template <int SPLIT>
__device__ __forceinline__ void store_row8(unsigned char* base, unsigned piece_bytes,
                                           unsigned off, const float (&v)[8]) {
  if constexpr (SPLIT == SPLIT_BF16_3) {
    uint4 h, m, l;
    split3_pair(v[0], v[1], h.x, m.x, l.x);
    split3_pair(v[2], v[3], h.y, m.y, l.y);
    split3_pair(v[4], v[5], h.z, m.z, l.z);
    split3_pair(v[6], v[7], h.w, m.w, l.w);
    *reinterpret_cast<uint4*>(base + off) = h;
    *reinterpret_cast<uint4*>(base + piece_bytes + off) = m;
    *reinterpret_cast<uint4*>(base + 2 * piece_bytes + off) = l;
  } else {
    uint4 h, l;
    split_pair<split_bf16(SPLIT)>(v[0], v[1], h.x, l.x);
    split_pair<split_bf16(SPLIT)>(v[2], v[3], h.y, l.y);
    split_pair<split_bf16(SPLIT)>(v[4], v[5], h.z, l.z);
    split_pair<split_bf16(SPLIT)>(v[6], v[7], h.w, l.w);
    *reinterpret_cast<uint4*>(base + off) = h;
    *reinterpret_cast<uint4*>(base + piece_bytes + off) = l;
  }
}

// A = W of one 8-particle group over the warp's pixel group.  `path`
// GP_COVERED: every particle is empty or a table kernel whose box holds its
// support, so the 8 x PXL weights are one branch-free block of independent
// chains with no box test (an empty slot has zero k2 and scale: u = 0 and a
// zero weight).  GP_MIXED adds Dirac particles and box tests (an empty
// slot's mask is empty, so u lands on the table's zero cell; DIRAC: the box
// test picks sw).  GP_DIRAC: Dirac kernels (or empty), the box test alone.
// GP_GAUSS: Gaussian kernels (or empty), their erf
// factors as 8 independent chains.  GP_GENERAL: each particle takes its
// kind's path.
template <int SPLIT, int PXL>
__device__ __forceinline__ void produce_w_task(const StagePar* par, int path, const KSpec* ks,
                                               unsigned ktab_s32, unsigned gtab_s32, float ucap,
                                               int g8, int pg,
                                               int lane, unsigned char* a0, unsigned a_bytes) {
  const int jl = lane & 15;
  const float jlf = (float)jl;
  const int wr0 = 2 * pg * PXL;
  int il[PXL];
  float ilf[PXL];
#pragma unroll
  for (int k = 0; k < PXL; ++k) {
    il[k] = wr0 + 2 * k + (lane >> 4);
    ilf[k] = (float)il[k];
  }
  float w[8][PXL];
  if (path == GP_COVERED) {
    const unsigned base32 = ktab_s32 - (0x4B000000u << 4);
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const StagePar P = par[e];
      const float dy = (P.dyr - jlf) + P.yf;
      const float dy2k = dy * dy * P.k2;
#pragma unroll
      for (int k = 0; k < PXL; ++k) {
        const float dx = (P.dxr - ilf[k]) + P.xf;
        const float u = fminf(fmaf(dx * P.k2, dx, dy2k), ucap);
        float t;
        const float4 cf = kt_cell_smem(base32, u, t);
        w[e][k] = horner3(cf, t) * P.scale;
      }
    }
  } else if (path == GP_MIXED) {
    const unsigned base32 = ktab_s32 - (0x4B000000u << 4);
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const StagePar P = par[e];
      const unsigned msk = (unsigned)P.mask;
      const bool jin = (msk >> (8 + jl)) & 1u;
      const bool cover = (P.kind & WK_COVER) != 0;
      const bool dirac = (P.kind & 7) == WK_DIRAC;
      const float dy = (P.dyr - jlf) + P.yf;
      const float dy2k = dy * dy * P.k2;
#pragma unroll
      for (int k = 0; k < PXL; ++k) {
        const float dx = (P.dxr - ilf[k]) + P.xf;
        const bool in = jin && ((msk >> il[k]) & 1u);
        float u = fminf(fmaf(dx * P.k2, dx, dy2k), ucap);
        u = (cover || in) ? u : ucap;
        float t;
        const float4 cf = kt_cell_smem(base32, u, t);
        const float wt = horner3(cf, t) * P.scale;
        w[e][k] = dirac ? (in ? P.scale : 0.f) : wt;
      }
    }
  } else if (path == GP_DIRAC) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const StagePar P = par[q];
      const unsigned msk = (unsigned)P.mask;
      const bool jin = (msk >> (8 + jl)) & 1u;
#pragma unroll
      for (int k = 0; k < PXL; ++k) w[q][k] = jin && ((msk >> il[k]) & 1u) ? P.scale : 0.f;
    }
  } else if (path == GP_GAUSS) {
    // two particles' erf factors at a time (independent chains; more would
    // spill registers), then their pixels' truncation factors and box tests
#pragma unroll
    for (int h = 0; h < 8; h += 2) {
      float e[2];
#pragma unroll
      for (int r = 0; r < 2; ++r) e[r] = gauss_factor<PXL>(par[h + r], wr0, lane);
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const StagePar P = par[h + r];
        const unsigned msk = (unsigned)P.mask;
        const bool jin = (msk >> (8 + jl)) & 1u;
        const float ey = __shfl_sync(0xffffffffu, e[r], jl);
        const float tr = ks[(P.kind >> 8) & 0xF].truncate;
        const float ihs2 = P.k2 * P.k2;
        const float dy = (P.dyr - jlf) + P.yf;
        const float dy2 = dy * dy;
        const float c = ey * P.scale;
#pragma unroll
        for (int k = 0; k < PXL; ++k) {
          const float ex = __shfl_sync(0xffffffffu, e[r], 16 + (il[k] - wr0));
          const float dx = (P.dxr - ilf[k]) + P.xf;
          const float T = gauss_trunc(gtab_s32, fmaf(dx, dx, dy2), ihs2, tr * tr);
          const bool in = jin && ((msk >> il[k]) & 1u);
          w[h + r][k] = in ? T * ex * c : 0.f;
        }
      }
    }
  } else {
#pragma unroll
    for (int e = 0; e < 8; ++e)
      w_particle<PXL>(par[e], ks, ktab_s32, gtab_s32, ucap, wr0, il, ilf, jl, jlf, lane, w[e]);
  }
  const unsigned goff = (unsigned)(g8 >> 1) * 4096u + (unsigned)(g8 & 1) * 128u;
#pragma unroll
  for (int k = 0; k < PXL; ++k) {
    const int m = 32 * (pg * PXL + k) + lane;
    const float v[8] = {w[0][k], w[1][k], w[2][k], w[3][k], w[4][k], w[5][k], w[6][k], w[7][k]};
    store_row8<SPLIT>(a0, a_bytes, goff + (unsigned)(m >> 3) * 256u + (unsigned)(m & 7) * 16u,
                      v);
  }
}

// Spectrum-store values of one S task (8 particles at the lane's window
// channel), loaded ahead of their store.
__device__ __forceinline__ void s_task_load(const SPar* sp, const unsigned* spec, int wa, int n,
                                            unsigned (&v)[8]) {
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const SPar q = sp[e];
    const unsigned d = (unsigned)(wa + n - q.clo);  // below clo wraps past n
    v[e] = d < q.n ? __ldg(spec + q.soff + d) : 0u;
  }
}

// B = S of one 8-particle group at window channel n (n < nw), from values
// as the spectrum store keeps them: hi | lo << 16 halves (pairs), or the
// FP32 value (three pieces).
template <int SPLIT>
__device__ __forceinline__ void s_task_store(const unsigned (&v)[8], int g8, int n, int nw,
                                             unsigned char* b0, unsigned b_bytes) {
  const unsigned off = (unsigned)(g8 >> 1) * ((unsigned)nw * 32u) + (unsigned)(g8 & 1) * 128u +
                       (unsigned)(n >> 3) * 256u + (unsigned)(n & 7) * 16u;
  if constexpr (SPLIT == SPLIT_BF16_3) {
    const float f[8] = {__uint_as_float(v[0]), __uint_as_float(v[1]), __uint_as_float(v[2]),
                        __uint_as_float(v[3]), __uint_as_float(v[4]), __uint_as_float(v[5]),
                        __uint_as_float(v[6]), __uint_as_float(v[7])};
    store_row8<SPLIT>(b0, b_bytes, off, f);
  } else {
    const uint4 h = make_uint4(__byte_perm(v[0], v[1], 0x5410), __byte_perm(v[2], v[3], 0x5410),
                               __byte_perm(v[4], v[5], 0x5410), __byte_perm(v[6], v[7], 0x5410));
    const uint4 l = make_uint4(__byte_perm(v[0], v[1], 0x7632), __byte_perm(v[2], v[3], 0x7632),
                               __byte_perm(v[4], v[5], 0x7632), __byte_perm(v[6], v[7], 0x7632));
    *reinterpret_cast<uint4*>(b0 + off) = h;
    *reinterpret_cast<uint4*>(b0 + b_bytes + off) = l;
  }
}

// Prefetch into L2 the part of a listed particle's spectrum-store row that
// falls in the block [cb0, cb1] (one prefetch per 128-byte line): the
// spectrum tasks of its stage read it a stage later.
__device__ __forceinline__ void prefetch_row(const unsigned* spec, const TcPar& t, bool listed,
                                             int cb0, int cb1) {
  if (spec == nullptr || !listed || t.kind == 0) return;
  const int a = max(t.clo, cb0), b = min(t.chi, cb1);
  if (a > b) return;
  const char* p = reinterpret_cast<const char*>(spec + t.soff + (a - t.clo));
  const char* e = reinterpret_cast<const char*>(spec + t.soff + (b - t.clo));
  for (; p < e; p += 128) asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
  asm volatile("prefetch.global.L2 [%0];" ::"l"(e));
}

// What a build warp tells the others about its 32 particles of a stage:
// the union of their supports and the path of each of its 8-particle groups.
// Lane l holds particle l (kind 0 for an empty slot).
__device__ __forceinline__ void build_summary(int clo, int chi, int kind, int lane, int2* win,
                                              int* gp) {
  clo = __reduce_min_sync(0xffffffffu, clo);
  chi = __reduce_max_sync(0xffffffffu, chi);
  const int k = kind & 7;
  const unsigned cov =
      __ballot_sync(0xffffffffu, k == WK_NONE || (k == WK_TAB && (kind & WK_COVER)));
  const unsigned mix = __ballot_sync(0xffffffffu, k == WK_NONE || k == WK_TAB || k == WK_DIRAC);
  const unsigned gau = __ballot_sync(0xffffffffu, k == WK_NONE || k == WK_GAUSS);
  const unsigned dir = __ballot_sync(0xffffffffu, k == WK_NONE || k == WK_DIRAC);
  if (lane == 0) *win = make_int2(clo, chi);
  if (lane < 4) {
    const unsigned c8 = (cov >> (8 * lane)) & 0xffu, m8 = (mix >> (8 * lane)) & 0xffu;
    const unsigned g8 = (gau >> (8 * lane)) & 0xffu, d8 = (dir >> (8 * lane)) & 0xffu;
    gp[lane] = d8 == 0xffu   ? GP_DIRAC
               : c8 == 0xffu ? GP_COVERED
               : m8 == 0xffu ? GP_MIXED
               : g8 == 0xffu ? GP_GAUSS
                             : GP_GENERAL;
  }
}

template <int SPLIT, int KC>
__global__ void __launch_bounds__(TC_THREADS, 1)
k_contract_tc(Geo g, Ws w, int nwmax) {
  static_assert(KC == 32 || KC == 64, "stage size");
  static_assert(KC == 32 || KC == 64, "records of a stage: one per lane of KC / 32 warps");
  constexpr bool BF16 = split_bf16(SPLIT);
  constexpr int NP = split_parts(SPLIT);  // 16-bit pieces per operand
  // Roles of the warps in a stage.  Every warp computes one weight task.
  // The last NB = KC / 32 warps (build warps) also copy the next stage's
  // particle parameters and turn them into stage parameters, one particle
  // per lane (slot bq); lane 0 of the warp before them issues the MMAs
  // after the stage barrier; the other NSW warps take the spectrum tasks.
  constexpr int NWARP = TC_THREADS / 32;
  constexpr int NB = KC / 32;
  constexpr int MMA_WARP = NWARP - NB - 1;
  constexpr int NSW = MMA_WARP;
  // stages between drains: TC_DRAIN for pairs (24 MMAs), every stage for
  // three pieces (the same 24 MMAs, over half the particles)
  constexpr int DRAIN_STAGES = NP == 3 ? 1 : TC_DRAIN;
  // two working accumulators (K halves of a 64-particle stage, three pieces)
  constexpr bool TWO_ACC = NP == 3 && KC == 64;
  constexpr int KSTEPS = KC / 16;
  extern __shared__ __align__(1024) unsigned char smem[];
  // the next stage's particles (cp.async targets; only the build warps touch
  // them, each its own slot: copied at a stage's start, read at its end),
  // piece k of slot q at s_tp[k][q], so that a warp's 16-byte reads of one
  // piece are contiguous
  __shared__ __align__(16) uint4 s_tp[4][KC];
  // Stage parameters rotate over three buffers (stage ch in buffer ch % 3
  // of its item): the build warps write a stage's while the warps still
  // finishing the stage before the previous one read theirs.
  __shared__ int s_pid[3][KC];
  __shared__ int2 s_win[3][NB];    // support union [clo, chi] per build warp (window)
  __shared__ int s_gp[3][KC / 8];  // path of each 8-particle group (GP_*)
  __shared__ __align__(16) StagePar s_par[3][KC];  // weight producers' view of a stage
  __shared__ __align__(16) SPar s_spar[3][KC];     // spectrum producers' view
  __shared__ KSpec s_ks[MG_MAX_KERNELS];
  __shared__ float4 s_ktab[KT_SMEM_CELLS];
  __shared__ float4 s_gtab[GT_NCELL + 1];  // Gaussian truncation cells
  __shared__ __align__(8) unsigned long long bars[2];
  // s_full[b]: every warp has produced its part of the stage in buffer b
  // (the MMA warp then issues it); s_parb[b]: the build warps have written
  // the parameters of the stage in buffer b
  __shared__ __align__(8) unsigned long long s_full[2], s_parb[3];
  __shared__ unsigned s_tmem;
  __shared__ long long s_item;
  __shared__ int s_abort;

  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const bool bld = warp >= NWARP - NB;         // a build warp
  const int bq = (warp - (NWARP - NB)) * 32 + lane;  // its particle slot
  if (w.hdr->status) return;
  const long long n_items = w.hdr->n_items;
  const int kch = w.hdr->kch;
  // Gaussian lines come from the spectrum store when it was filled
  const unsigned* spec = (g.spectral_model == MG_SPECTRUM_GAUSSIAN && w.cap_spec > 0 &&
                       w.hdr->spec_ready)
                          ? w.spec
                          : nullptr;

  const unsigned a_bytes = KSTEPS * 4096u;                 // one piece of A
  const unsigned b_bytes = KSTEPS * (unsigned)nwmax * 32u;  // one piece of B
  const unsigned st_bytes = NP * (a_bytes + b_bytes);
  const unsigned sbase = smem_u32(smem);

  if (tid < MG_MAX_KERNELS) s_ks[tid] = g.ks[tid];
  // the table of the launch's radial kernel (at most one per kernel tuple)
  int ktab_type = -1;
  for (int k = 0; k < g.n_kernels; ++k)
    if (g.ks[k].type <= MG_KERNEL_QUARTIC_SPLINE) ktab_type = g.ks[k].type;
  if (ktab_type >= 0) {
    const KTableInfo& inf = kt_info[ktab_type];
    const int ncell = inf.ncoef;
    if (ncell <= KT_SMEM_CELLS) {
      const float4* src = reinterpret_cast<const float4*>(kt_coef) + inf.reg[0].first;
      for (int e = tid; e < ncell; e += TC_THREADS) s_ktab[e] = src[e];
    } else {
      ktab_type = -1;
    }
  }
  for (int e = tid; e <= GT_NCELL; e += TC_THREADS)
    s_gtab[e] = reinterpret_cast<const float4*>(gt_coef)[e];
  const unsigned gtab_s32 = smem_u32(s_gtab) - (0x4B000000u << 4);
  // the zero cell past the support of the shared-memory table
  const float ucap = ktab_type >= 0 ? (float)kt_info[ktab_type].reg[0].ncell : 0.f;
  if (tid == 0) {
    mbar_init(smem_u32(&bars[0]), 1);
    mbar_init(smem_u32(&bars[1]), 1);
    mbar_init(smem_u32(&s_full[0]), NWARP);
    mbar_init(smem_u32(&s_full[1]), NWARP);
    mbar_init(smem_u32(&s_parb[0]), NB);
    mbar_init(smem_u32(&s_parb[1]), NB);
    mbar_init(smem_u32(&s_parb[2]), NB);
    s_abort = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&s_tmem)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = s_tmem;
  const int quarter = warp & 3;    // TMEM lane quarter of this warp
  const int colgrp = warp >> 2;    // 4 warps share a quarter: 32-column groups
  const unsigned lane_base = (unsigned)(quarter * 32) << 16;
  int ncols = g.max_width;  // channels of the item's block held in TMEM (<= 256)

  const bool drain = ncols <= TC_MASTER_COL;  // master accumulator fits
  // Columns [lo, hi) of both accumulators that MMAs may have written since
  // they were last zeroed (32-column chunk granularity, warp-uniform tests);
  // TMEM is zero everywhere else.
  auto chunk_in = [](int c, int lo, int hi) { return c < hi && c + 32 > lo; };
  auto zero_tmem = [&](int lo, int hi) {
    for (int c = colgrp * 32; c < ncols; c += 128) {
      if (!chunk_in(c, lo, hi)) continue;
      tmem_st32_zero(tmem + lane_base + c);
      if (TWO_ACC) tmem_st32_zero(tmem + lane_base + TC_WB_COL + c);
      if (drain) tmem_st32_zero(tmem + lane_base + TC_MASTER_COL + c);
    }
    tmem_wait_st();
  };
  // master += working (round to nearest), working = 0 over the columns
  // written since the last drain; no MMA in flight
  // The drain of columns [lo, hi): the warps of a lane quarter take its
  // 16-column pieces round robin (a column past what the MMAs wrote is zero
  // and adds nothing).  The MMA and build warps (column group 3 of the last
  // quarters) leave their quarters' pieces to the other three.
  const int dwarps = quarter >= MMA_WARP - 12 ? 3 : 4;
  auto drain_tmem = [&](int lo, int hi) {
    if (colgrp >= dwarps) return;
    for (int c = (lo & ~15) + 16 * colgrp; c < hi; c += 16 * dwarps) {
      unsigned a[16], b[16];
      tmem_ld16(tmem + lane_base + c, a);
      tmem_ld16(tmem + lane_base + TC_MASTER_COL + c, b);
      if constexpr (TWO_ACC) {
        unsigned a2[16];
        tmem_ld16(tmem + lane_base + TC_WB_COL + c, a2);
        tmem_wait_ld();
#pragma unroll
        for (int v = 0; v < 16; ++v)
          a[v] = __float_as_uint(__uint_as_float(a[v]) + __uint_as_float(a2[v]));
        tmem_st16_zero(tmem + lane_base + TC_WB_COL + c);
      } else {
        tmem_wait_ld();
      }
#pragma unroll
      for (int v = 0; v < 16; ++v)
        b[v] = __float_as_uint(__uint_as_float(a[v]) + __uint_as_float(b[v]));
      tmem_st16(tmem + lane_base + TC_MASTER_COL + c, b);
      tmem_st16_zero(tmem + lane_base + c);
    }
    tmem_wait_st();
  };
  zero_tmem(0, ncols);
  tc_fence_before();
  __syncthreads();

  // per stage buffer s: bit s of phase_bits is its mbarrier parity, bit s
  // of pending_bits says MMAs reading it are in flight (registers, not a
  // dynamically indexed array)
  unsigned phase_bits = 0u, pending_bits = 0u;
  // bit b: parity of the next phase of s_full[b] / s_parb[b] to complete
  unsigned full_par = 0u, parb_par = 0u;
  int stage = 0;
  int since_drain = 0;
  // thread 0 takes the next item from the queue while this one runs (the
  // atomic's round trip is off the item switch)
  long long next_item = tid == 0 ? (long long)atomicAdd(&w.hdr->item_counter, 1u) : 0;

  for (;;) {
    if (tid == 0) s_item = next_item;
    __syncthreads();
    const long long item = s_item;
    if (item >= n_items || s_abort) break;
    if (tid == 0) next_item = (long long)atomicAdd(&w.hdr->item_counter, 1u);
    // the queue runs over the items in cost order, largest first
    const ItemTC it = decode_tc(g, w, (long long)w.item_order[item], kch);
    const Gal& G = w.gal[it.gal];
    const GalState& gs = w.gst[it.gal];
    const int dec = gs.dec;
    const int nc = G.nc;
    ncols = G.width;
    // exact power-of-two operand scales of this cube (FP16 form): largest
    // |W|, |S| -> 2^14
    float sw = 1.f, ss = 1.f;
    if (!BF16) {
      const float wb = __uint_as_float(gs.wbound_bits);
      if (wb > 0.f) sw = exp2f(14.f - ceilf(log2f(wb)));
      ss = spec_scale(gs, g.spectral_model);
    }
    const float unscale = 1.f / (sw * ss);
    const int i0 = it.tx * TILE_I, j0 = it.ty * TILE_J;
    const int nchunk = (it.lcount + KC - 1) / KC;
    int d_lo = 0x7fffffff, d_hi = 0;  // columns written since the last drain
    // a drain scheduled after a stage's MMAs runs as the last step of the
    // next stage's production, once those MMAs have completed (the next
    // stage's MMAs wait for every warp's arrival, drains included), over
    // columns [p_lo, p_hi)
    bool drain_due = false;
    int p_lo = 0, p_hi = 0;
    int t_lo = 0x7fffffff, t_hi = 0;  // columns written by this item

    // records of the first stage; the list entry of the second
    int pid_ahead = 0;
    const int cb0 = it.c0, cb1 = it.c0 + ncols - 1;  // the segment's channel block
    if (bld) {
      const bool listed = bq < it.lcount;
      TcPar t = empty_tpar();
      if (listed) {
        const int pid = w.list[it.lbeg + bq];
        t = w.tpar[pid];
        s_pid[0][bq] = pid;
      } else {
        s_pid[0][bq] = 0;
      }
      if (KC + bq < it.lcount) pid_ahead = w.list[it.lbeg + KC + bq];
      const int kind = build_stage(t, listed, i0, j0, cb0, cb1, s_par[0][bq], s_spar[0][bq]);
      prefetch_row(spec, t, listed, cb0, cb1);
      build_summary(listed ? t.clo : 0x7fffffff, listed ? t.chi : -1, kind, lane,
                    &s_win[0][bq >> 5], &s_gp[0][(bq >> 5) * 4]);
      if (KC + bq < it.lcount) asm volatile("prefetch.global.L2 [%0];" ::"l"(w.tpar + pid_ahead));
    }
    __syncthreads();

    for (int ch = 0; ch < nchunk; ++ch) {
      const int buf = ch % 3;              // this stage's parameters
      const int nbuf = buf == 2 ? 0 : buf + 1;  // the next stage's
      const int k0 = ch * KC;
      const int kn = min(KC, it.lcount - k0);
      // the stage must be free: every thread waits for the MMAs that last read it
      if ((pending_bits >> stage) & 1u) {
        if (!mbar_wait(smem_u32(&bars[stage]), (phase_bits >> stage) & 1u)) s_abort = 1;
        phase_bits ^= 1u << stage;
        pending_bits &= ~(1u << stage);
      }
      // the stage's parameters: built at the item's start for its first
      // stage, else by the build warps during the previous stage
      if (ch > 0) {
        if (!mbar_wait(smem_u32(&s_parb[buf]), (parb_par >> buf) & 1u)) s_abort = 1;
        parb_par ^= 1u << buf;
      }
      // the next stage's records travel global -> shared by cp.async while
      // this one is produced (its list entry was read a stage earlier); the
      // list entry of the stage after is read now
      const bool has_next = ch + 1 < nchunk;
      int npid = 0;
      if (has_next && bld) {
        if (k0 + KC + bq < it.lcount) {
          npid = pid_ahead;
          cp_async_tpar(&s_tp[0][bq], KC * 16u, w.tpar + npid);
        } else {
          const TcPar z = empty_tpar();
#pragma unroll
          for (int k = 0; k < 4; ++k) s_tp[k][bq] = reinterpret_cast<const uint4*>(&z)[k];
        }
        cp_async_commit();
        if (k0 + 2 * KC + bq < it.lcount) pid_ahead = w.list[it.lbeg + k0 + 2 * KC + bq];
      }
      // stage channel window [w0, w0 + nw): min clo, max chi
      int w0, nw;
      {
        // the extremes of the stage's listed particles' supports
        int2 lh = s_win[buf][0];
        if (NB > 1) {
          const int2 u = s_win[buf][NB - 1];
          lh = make_int2(min(lh.x, u.x), max(lh.y, u.y));
        }
        int lo = lh.x, hi = lh.y;
        // relative to the segment's block [c0, c0 + ncols)
        lo = max(lo, it.c0) - it.c0;
        hi = min(hi, it.c0 + ncols - 1) - it.c0;
        if (hi < lo) lo = hi = 0;  // no support in this block: zeros
        w0 = lo & ~15;
        nw = ((hi + 1 - w0) + 15) & ~15;
        if (nw < 16) nw = 16;
        if (nw > nwmax) nw = nwmax;
        if (w0 + nw > ncols) w0 = ncols - nw;
        if (w0 < 0) w0 = 0;
        d_lo = min(d_lo, w0);
        d_hi = max(d_hi, w0 + nw);
        t_lo = min(t_lo, w0);
        t_hi = max(t_hi, w0 + nw);
      }
      unsigned char* const sa = smem + stage * st_bytes;  // NP pieces of A, then of B
      unsigned char* const sb = sa + NP * a_bytes;
      // drain of the previous interval: the MMAs of the previous stage are
      // waited for, then the working accumulator is added into the master
      // (a warp with no pieces to drain does not wait: the stage's buffer
      // stays pending until the warp next needs it)
      auto drain_now = [&]() {
        drain_due = false;
        if (colgrp >= dwarps) return;
        const int sp = stage ^ 1;  // the previous stage's buffer
        if (!mbar_wait(smem_u32(&bars[sp]), (phase_bits >> sp) & 1u)) s_abort = 1;
        phase_bits ^= 1u << sp;
        pending_bits &= ~(1u << sp);
        tc_fence_after();
        drain_tmem(p_lo, p_hi);
        tc_fence_before();
      };
      // ---- A = W: one 8-particle group x pixel group per warp
      constexpr int PXL = KC / 32;  // pixels per lane
      constexpr int NG8 = KC / 8;   // particle groups of a stage
      const int wa = it.c0 + w0;    // first window channel (absolute)
      // Spectrum tasks go to warps 0 .. NSW - 1 in rounds of NSW, every
      // other round in reverse order, so that the warps' counts differ by
      // one at most and the extra tasks do not pile up on the same warps.
      // The loads of a warp's first task are in flight during its weights.
      const int n_chunks = (nw + 31) >> 5;
      const int n_stasks = spec ? n_chunks * NG8 : 0;
      const int t0 = warp < NSW ? warp : n_stasks;
      unsigned sv[8];
      if (t0 < n_stasks)
        s_task_load(s_spar[buf] + 8 * (t0 % NG8), spec, wa, 32 * (t0 / NG8) + lane, sv);
      // the table paths need the launch's table in shared memory
      int path = s_gp[buf][warp % NG8];
      if (ktab_type < 0 && (path == GP_COVERED || path == GP_MIXED)) path = GP_GENERAL;
      produce_w_task<SPLIT, PXL>(s_par[buf] + 8 * (warp % NG8), path, s_ks,
                                 smem_u32(s_ktab), gtab_s32, ucap, warp % NG8, warp / NG8, lane, sa,
                                 a_bytes);
      // ---- B = S
      if (spec) {
        // Gaussian lines from the spectrum store: tasks of (32-channel
        // chunk, 8-particle group), round robin over the warps
        for (int t = t0, r = 0; t < n_stasks;
             ++r, t = r * NSW + ((r & 1) ? NSW - 1 - warp : warp)) {
          const int g8 = t % NG8, n = 32 * (t / NG8) + lane;
          if (t != t0) s_task_load(s_spar[buf] + 8 * g8, spec, wa, n, sv);
          if (n < nw) s_task_store<SPLIT>(sv, g8, n, nw, sb, b_bytes);
        }
      } else {
        // lines evaluated here (Dirac lines, tabulated spectra, or no room
        // for the store): warp w takes particles w * PPW .. + PPW - 1 in pairs
        constexpr int PPW = KC / (TC_THREADS / 32);
#pragma unroll
        for (int pp = 0; pp < PPW; pp += 2) {
          const int q = warp * PPW + pp;
          const PRec r0 = q < kn ? w.rec[s_pid[buf][q]] : empty_rec();
          const PRec r1 = q + 1 < kn ? w.rec[s_pid[buf][q + 1]] : empty_rec();
          // a particle listed for this block whose line misses the block
          // (the list bound is conservative) contributes nothing
          const bool v0 = q < kn && r0.chi >= cb0 && r0.clo <= cb1;
          const bool v1 = q + 1 < kn && r1.chi >= cb0 && r1.clo <= cb1;
          produce_s_pair<SPLIT>(r0, r1, v0, v1, q, wa, nw, nc, dec, g.spectral_model,
                                w.ehi + G.edge0, w.elo + G.edge0, w.inv_w + G.edge0, G.spectra,
                                (int)(s_pid[buf][q] - G.p0), (int)(s_pid[buf][q + 1] - G.p0),
                                lane, ss, sb, b_bytes);
        }
      }
      if (has_next && bld) {
        // the next stage's buffer of parameters was last read two stages
        // ago: every warp must have finished that stage (s_full[stage]'s
        // phase before the current one)
        if (ch > 1 &&
            !mbar_wait(smem_u32(&s_full[stage]), ((full_par >> stage) & 1u) ^ 1u))
          s_abort = 1;
        s_pid[nbuf][bq] = npid;
        cp_async_wait_all();
        const bool listed = k0 + KC + bq < it.lcount;
        TcPar t;
#pragma unroll
        for (int k = 0; k < 4; ++k) reinterpret_cast<uint4*>(&t)[k] = s_tp[k][bq];
        const int kind = build_stage(t, listed, i0, j0, cb0, cb1, s_par[nbuf][bq],
                                     s_spar[nbuf][bq]);
        prefetch_row(spec, t, listed, cb0, cb1);
        build_summary(listed ? t.clo : 0x7fffffff, listed ? t.chi : -1, kind, lane,
                      &s_win[nbuf][bq >> 5], &s_gp[nbuf][(bq >> 5) * 4]);
        // the particle of the stage after next into L2: its cp.async, at the
        // next stage's start, then misses HBM no more
        if (k0 + 2 * KC + bq < it.lcount)
          asm volatile("prefetch.global.L2 [%0];" ::"l"(w.tpar + pid_ahead));
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&s_parb[nbuf]));
      }
      // the drain of the previous interval, last: its MMAs have had the
      // whole production of this stage to complete
      if (drain_due) drain_now();
      // hand the stage over: operands to the async proxy, drains before the
      // next MMAs, then one arrival per warp; no warp waits for the others
      fence_proxy_async();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&s_full[stage]));
      const unsigned fpar = (full_par >> stage) & 1u;
      full_par ^= 1u << stage;
      if (tid == MMA_WARP * 32) {
        if (!mbar_wait(smem_u32(&s_full[stage]), fpar)) s_abort = 1;
        tc_fence_after();
        // nw <= nwmax <= 256: one MMA spans the window.  The descriptors'
        // start-address field (bits 0-13, address / 16) steps by adding the
        // K-step offsets: every stage address is below 256 KB, so no carry.
        const unsigned base = sbase + stage * st_bytes;
        const unsigned id = idesc_f16kind(128, nw, BF16);
        // pieces: hi, lo (pairs) or hi, mid, lo (three), a_bytes / b_bytes apart
        const unsigned long long a_hi = sdesc(base, 128, 256);
        const unsigned long long a_2 = a_hi + (a_bytes >> 4);
        const unsigned long long b_hi = sdesc(base + NP * a_bytes, 128, 256);
        const unsigned long long b_2 = b_hi + (b_bytes >> 4);
        const unsigned bstep = (unsigned)nw * 2u;  // K step of B: nw * 32 bytes
        const unsigned d = tmem + (unsigned)w0;
        // Smallest terms first: the tensor core's FP32 accumulation truncates
        // each MMA's sum to the accumulator's precision, so every MMA loses up
        // to an ulp of the accumulator.  Issued into the working accumulator
        // the last drain left at zero, the cross terms (2^-8 .. 2^-16 of the
        // hi products) lose ulps of their own small sums; only the hi x hi
        // products, last, meet the full-size accumulator.
        // the accumulator of K-step ks: the second working one for the
        // upper half of a 64-particle three-piece stage
        auto dk = [&](int ks) { return TWO_ACC && ks >= 2 ? d + (unsigned)TC_WB_COL : d; };
        if constexpr (NP == 3) {
          const unsigned long long a_3 = a_2 + (a_bytes >> 4);
          const unsigned long long b_3 = b_2 + (b_bytes >> 4);
#pragma unroll
          for (int ks = 0; ks < KSTEPS; ++ks) {
            const unsigned ao = (unsigned)ks * 256u, bo = (unsigned)ks * bstep;
            umma(dk(ks), a_2 + ao, b_2 + bo, id, 1u);   // mid mid
            umma(dk(ks), a_hi + ao, b_3 + bo, id, 1u);  // hi lo
            umma(dk(ks), a_3 + ao, b_hi + bo, id, 1u);  // lo hi
          }
        }
#pragma unroll
        for (int ks = 0; ks < KSTEPS; ++ks) {
          const unsigned ao = (unsigned)ks * 256u, bo = (unsigned)ks * bstep;
          umma(dk(ks), a_hi + ao, b_2 + bo, id, 1u);  // hi lo (pair) / hi mid
          umma(dk(ks), a_2 + ao, b_hi + bo, id, 1u);  // lo hi (pair) / mid hi
        }
#pragma unroll
        for (int ks = 0; ks < KSTEPS; ++ks)
          umma(dk(ks), a_hi + (unsigned)ks * 256u, b_hi + (unsigned)ks * bstep, id, 1u);
        umma_commit(smem_u32(&bars[stage]));
      }
      if (s_abort) break;
      pending_bits |= 1u << stage;
      stage ^= 1;
      if (drain && ++since_drain == DRAIN_STAGES && ch + 1 < nchunk) {
        // drain the interval's columns during the next stage (its commit
        // covers every earlier MMA)
        drain_due = true;
        p_lo = d_lo;
        p_hi = d_hi;
        d_lo = 0x7fffffff;
        d_hi = 0;
        since_drain = 0;
      }
    }
    since_drain = 0;

    // all MMAs of the item complete (a commit covers every earlier MMA)
    for (int s = 0; s < 2; ++s) {
      if ((pending_bits >> s) & 1u) {
        if (!mbar_wait(smem_u32(&bars[s]), (phase_bits >> s) & 1u)) s_abort = 1;
        phase_bits ^= 1u << s;
        pending_bits &= ~(1u << s);
      }
    }
    __syncthreads();
    if (s_abort) {
      if (tid == 0) atomicOr(&w.hdr->status, ST_TIMEOUT);
      break;
    }
    tc_fence_after();
    // ---- epilogue: TMEM -> registers -> cube or partial
    {
      const int p = quarter * 32 + lane;
      const int i = i0 + p / TILE_J, j = j0 + p % TILE_J;
      const bool inside = i < G.nx && j < G.ny;
      float* dst;
      int limit;
      bool vec;
      if (it.nk == 1) {
        dst = G.cube + ((long long)i * G.ny + j) * nc + it.c0;
        limit = min(ncols, nc - it.c0);
        vec = (nc & 3) == 0 && (limit & 3) == 0;  // 16-byte aligned rows
      } else {
        const long long slot = w.part_off[it.seg] + it.kc;
        dst = w.partial + slot * (long long)(TILE_PX * g.max_width) + (long long)p * ncols;
        limit = ncols;
        vec = true;
      }
      for (int c = colgrp * 32; c < ncols; c += 128) {
        unsigned r[32];
        if (!chunk_in(c, t_lo, t_hi)) {
          // never written: zero (already in a cleared or accumulated cube)
          if (it.nk == 1) continue;
#pragma unroll
          for (int v = 0; v < 32; ++v) r[v] = 0u;
        } else {
          tmem_ld32(tmem + lane_base + (unsigned)c, r);
          tmem_wait_ld();
          if (TWO_ACC) {
            for (int h = 0; h < 32; h += 16) {
              unsigned m[16];
              tmem_ld16(tmem + lane_base + TC_WB_COL + (unsigned)(c + h), m);
              tmem_wait_ld();
#pragma unroll
              for (int v = 0; v < 16; ++v)
                r[h + v] = __float_as_uint(__uint_as_float(r[h + v]) + __uint_as_float(m[v]));
            }
          }
          if (drain) {
            for (int h = 0; h < 32; h += 16) {
              unsigned m[16];
              tmem_ld16(tmem + lane_base + TC_MASTER_COL + (unsigned)(c + h), m);
              tmem_wait_ld();
#pragma unroll
              for (int v = 0; v < 16; ++v)
                r[h + v] = __float_as_uint(__uint_as_float(r[h + v]) + __uint_as_float(m[v]));
            }
          }
        }
        if (inside || it.nk != 1) {
          // cube writes add to the contents in accumulate mode (one writer
          // per voxel: this item, or the split-K reduction)
          const bool add = g.accumulate && it.nk == 1;
          if (vec && c + 32 <= limit) {
#pragma unroll
            for (int v = 0; v < 8; ++v) {
              float4 o = make_float4(
                  __uint_as_float(r[4 * v]) * unscale, __uint_as_float(r[4 * v + 1]) * unscale,
                  __uint_as_float(r[4 * v + 2]) * unscale,
                  __uint_as_float(r[4 * v + 3]) * unscale);
              if (add) {
                const float4 p4 = *reinterpret_cast<const float4*>(dst + c + 4 * v);
                o.x += p4.x;
                o.y += p4.y;
                o.z += p4.z;
                o.w += p4.w;
              }
              *reinterpret_cast<float4*>(dst + c + 4 * v) = o;
            }
          } else {
#pragma unroll
            for (int v = 0; v < 32; ++v)
              if (c + v < limit) {
                const float o = __uint_as_float(r[v]) * unscale;
                dst[c + v] = add ? dst[c + v] + o : o;
              }
          }
        }
      }
    }
    zero_tmem(t_lo, t_hi);
    tc_fence_before();
    __syncthreads();
  }

  __syncthreads();
  tc_fence_after();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TC_TMEM_COLS)
                 : "memory");
  }
}

template <int SPLIT, int KC>
int launch_tc(const Geo& g, const Ws& w, int num_sms, cudaStream_t s, int nwmax) {
  size_t smem = 2 * tc_stage_bytes(SPLIT, KC, nwmax);
  // at least 116 KB so that one CTA (and its 512 TMEM columns) fits per SM
  if (smem < 118784) smem = 118784;
  // the shared-memory attribute is per device: set once on each (host-side
  // calls, made before a graph capture by the first insertion on a device)
  constexpr int kMaxDev = 64;
  static int attr_bytes[kMaxDev] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return MG_ERR_CUDA;
  if (attr_bytes[dev] <= 0) {
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, k_contract_tc<SPLIT, KC>) != cudaSuccess) return MG_ERR_CUDA;
    const int bytes = 227 * 1024 - (int)fa.sharedSizeBytes;
    if (cudaFuncSetAttribute(k_contract_tc<SPLIT, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             bytes) != cudaSuccess)
      return MG_ERR_CUDA;
    attr_bytes[dev] = bytes;
  }
  if ((int)smem > attr_bytes[dev]) return MG_ERR_UNSUPPORTED;
  k_contract_tc<SPLIT, KC><<<num_sms, TC_THREADS, smem, s>>>(g, w, nwmax);
  return MG_OK;
}

// Spectrum store of the tensor-core forms (Gaussian lines): row lengths,
// their scan into row offsets, the rows.
void launch_spec_store(const Geo& g, const Ws& w, int num_sms, cudaStream_t s) {
  const long long n = g.n;
  if (g.spectral_model != MG_SPECTRUM_GAUSSIAN || w.cap_spec <= 0 || n <= 0) return;
  const unsigned blocks = (unsigned)std::min<long long>((n + 255) / 256, (long long)num_sms * 16);
  k_spec_count<<<blocks, 256, 0, s>>>(g, w);
  launch_scan(w.npairs, n, w.pair_off, w.scan_sums, &w.hdr->n_spec, s);
  // a warp per particle, many warps in flight (each particle's work is a
  // short dependent chain: record, offsets, erfc)
  const unsigned eblocks = (unsigned)std::min<long long>((n + 7) / 8, (long long)num_sms * 64);
  k_spec_eval<<<eblocks, 256, 0, s>>>(g, w);
}

// The tensor-core producers' per-particle parameters (TcPar), once per
// insertion: the launch's radial kernel type (its table sits in shared
// memory in the contraction), each cube's operand scale sw, the spectrum-
// store row (pair_off holds the store's row offsets after the SPEC stage).
__global__ void k_tc_params(Geo g, Ws w) {
  __shared__ KSpec s_ks[MG_MAX_KERNELS];
  if (threadIdx.x < MG_MAX_KERNELS) s_ks[threadIdx.x] = g.ks[threadIdx.x];
  __syncthreads();
  int ktab_type = -1;
  for (int k = 0; k < g.n_kernels; ++k)
    if (g.ks[k].type <= MG_KERNEL_QUARTIC_SPLINE) ktab_type = g.ks[k].type;
  if (ktab_type >= 0 && kt_info[ktab_type].ncoef > KT_SMEM_CELLS) ktab_type = -1;
  const bool f16 = g.form == MG_FORM_F16X3;
  int gk = -1;
  long long gp1 = -1;
  float sw = 1.f;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.n;
       p += (long long)gridDim.x * blockDim.x) {
    if (gk < 0 || p >= gp1) {
      gk = find_gal(w.gp0, g.ngal, p);
      gp1 = w.gp0[gk + 1];
      sw = 1.f;
      if (f16) {
        const float wb = __uint_as_float(w.gst[gk].wbound_bits);
        if (wb > 0.f) sw = exp2f(14.f - ceilf(log2f(wb)));
      }
    }
    w.tpar[p] = tc_param(w.rec[p], s_ks, ktab_type, sw, w.pair_off[p]);
  }
}

int launch_contract_bf16x3(const Geo& g, const Ws& w, int num_sms, cudaStream_t s) {
  const int nwmax = g.max_width;  // a stage window never exceeds the widest block
  if (nwmax > TC_MASTER_COL) return MG_ERR_UNSUPPORTED;
  if (g.n > 0) {
    const unsigned blocks =
        (unsigned)std::min<long long>((g.n + 255) / 256, (long long)num_sms * 16);
    k_tc_params<<<blocks, 256, 0, s>>>(g, w);
  }
  // stage size: the form's default unless the launch shape asks for 32
  const bool kc32 = g.kc == 32;
  int rc;
  if (g.form == MG_FORM_BF16X6) {
    // 64-particle stages hold two working accumulators of 128 columns
    if (!kc32 && nwmax > TC_WB_COL) return MG_ERR_UNSUPPORTED;
    rc = kc32 ? launch_tc<SPLIT_BF16_3, 32>(g, w, num_sms, s, nwmax)
              : launch_tc<SPLIT_BF16_3, 64>(g, w, num_sms, s, nwmax);
  }
  else if (g.form == MG_FORM_BF16X3)
    rc = kc32 ? launch_tc<SPLIT_BF16_2, 32>(g, w, num_sms, s, nwmax)
              : launch_tc<SPLIT_BF16_2, 64>(g, w, num_sms, s, nwmax);
  else
    rc = kc32 ? launch_tc<SPLIT_F16_2, 32>(g, w, num_sms, s, nwmax)
              : launch_tc<SPLIT_F16_2, 64>(g, w, num_sms, s, nwmax);
  if (rc) return rc;
  launch_reduce_partials(g, w, num_sms, s);
  return MG_OK;
}

}  // namespace mg
