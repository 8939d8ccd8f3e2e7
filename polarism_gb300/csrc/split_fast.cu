// Split-step passes for FP32 rows and columns of 1024 sites: register-resident four-step FFTs.
//
// A 1024-point transform is 1024 = 32 x 32 (n = n2 + 32 n1, k = k1 + 32 k2):
//   X[k1 + 32 k2] = sum_n2 W_32^{n2 k2} W_1024^{n2 k1} sum_n1 x[n2 + 32 n1] W_32^{n1 k1}.
// A thread holds the 32 values x[n2 + 32 n1] of its n2 (n1 = register index), does the inner
// 32-point DFT in registers, multiplies by W_1024^{n2 k1}, exchanges once through shared
// memory so that it holds the 32 values of one k1, and does the outer 32-point DFT: it ends
// with X[k1 + 32 k2] (k2 = register index), the same layout it started from, so the kinetic
// factor and the local step apply in place.  One exchange per transform replaces the generic
// kernel's five barrier-separated radix-4 passes through shared memory (split.cu).
//
// Rows: a warp per row (lane = n2), the exchange within the warp.  Columns: a block per panel
// of eight columns (thread = (column, n2)), the exchange across the block, and between the
// inverse and forward transforms the local step (split_local.cuh) runs over the panel in
// shared memory as a plain loop, so its code exists once.
//
// Precision: every twiddle that is not +-1 or +-i is applied as a rounded value plus its
// remainder (the 32-point constants and the table W_1024^{n2 k1}), as the generic FP32 passes
// do: rounded factors alone carry a per-step amplitude bias that drifts the norm over long runs.
#include <cmath>

#include "ifrk_internal.h"
#include "ifrk_sites.cuh"
#include "split_local.cuh"

namespace pg {
namespace {

constexpr int kN = 1024;
constexpr int kRowsPerWarp = 4;             // rows a warp transforms in turn (row pass)
constexpr int kRowWarps = 8;                // warps a block (row pass)
constexpr int kPanel = 8;                   // columns a block (column pass)
constexpr int kXStride = 33;                // padded row of the 32 x 32 exchange
constexpr int kPanelStride = 32 * 33 + 4;   // one column's exchange block (elements = 4 mod 16)

// W_32^e = exp(-2 pi i e / 32) = c - i s for e = 1..15 (not 8) as {c, s} rounded to FP32 and
// the remainders {c - c_fp32, s - s_fp32}, from the double-precision cos and sin; e is a
// constant once the DFT loops are unrolled, so the switch folds to immediates.
__device__ __forceinline__ float4 w32(int e) {
  switch (e) {
    case 1: return make_float4(0.9807852506637573f, 0.19509032368659973f, 2.9739473106360492e-08f, -1.6704715388726754e-09f);
    case 2: return make_float4(0.9238795042037964f, 0.3826834261417389f, 2.830748968563057e-08f, 6.2233507236442165e-09f);
    case 3: return make_float4(0.8314695954322815f, 0.5555702447891235f, 1.687026340846387e-08f, -1.1769521357507529e-08f);
    case 4: return make_float4(0.7071067690849304f, 0.7071067690849304f, 1.2101617485882343e-08f, 1.2101617485882343e-08f);
    case 5: return make_float4(0.5555702447891235f, 0.8314695954322815f, -1.1769521357507529e-08f, 1.687026340846387e-08f);
    case 6: return make_float4(0.3826834261417389f, 0.9238795042037964f, 6.2233507236442165e-09f, 2.830748968563057e-08f);
    case 7: return make_float4(0.19509032368659973f, 0.9807852506637573f, -1.670471427850373e-09f, 2.9739473106360492e-08f);
    case 9: return make_float4(-0.19509032368659973f, 0.9807852506637573f, 1.6704715388726754e-09f, 2.9739473106360492e-08f);
    case 10: return make_float4(-0.3826834261417389f, 0.9238795042037964f, -6.2233507236442165e-09f, 2.830748968563057e-08f);
    case 11: return make_float4(-0.5555702447891235f, 0.8314695954322815f, 1.1769521357507529e-08f, 1.687026340846387e-08f);
    case 12: return make_float4(-0.7071067690849304f, 0.7071067690849304f, -1.2101617485882343e-08f, 1.2101617485882343e-08f);
    case 13: return make_float4(-0.8314695954322815f, 0.5555702447891235f, -1.687026340846387e-08f, -1.1769521357507529e-08f);
    case 14: return make_float4(-0.9238795042037964f, 0.3826834261417389f, -2.830748968563057e-08f, 6.223351167733426e-09f);
    case 15: return make_float4(-0.9807852506637573f, 0.19509032368659973f, -2.9739473106360492e-08f, -1.6704710947834656e-09f);
    default: return make_float4(1.0f, 0.0f, 0.0f, 0.0f);
  }
}

__host__ __device__ constexpr int brev5(int i) {
  return ((i & 1) << 4) | ((i & 2) << 2) | (i & 4) | ((i & 8) >> 2) | ((i & 16) >> 4);
}

// x * W_32^e (forward) or x * conj(W_32^e) (inverse); e is a constant once unrolled.
template <bool INV>
__device__ __forceinline__ float2 w32mul(float2 x, int e) {
  if (e == 0) return x;
  if (e == 8) return INV ? make_float2(-x.y, x.x) : make_float2(x.y, -x.x);
  const float4 w = w32(e);
  const float ch = w.x, sh = w.y, cl = w.z, sl = w.w;
  // forward: (x.x c + x.y s) + i (x.y c - x.x s); inverse: (x.x c - x.y s) + i (x.y c + x.x s)
  const float ys = INV ? -x.y : x.y;
  const float xs = INV ? x.x : -x.x;
  const float re = fmaf(x.x, ch, fmaf(ys, sh, fmaf(x.x, cl, ys * sl)));
  const float im = fmaf(x.y, ch, fmaf(xs, sh, fmaf(x.y, cl, xs * sl)));
  return make_float2(re, im);
}

// In-register 32-point DFT (radix 2, decimation in time; the bit-reversed read is a renaming).
template <bool INV>
__device__ __forceinline__ void dft32(float2 (&v)[32]) {
  float2 a[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) a[i] = v[brev5(i)];
#pragma unroll
  for (int s = 1; s <= 5; ++s) {
#pragma unroll
    for (int b = 0; b < 16; ++b) {  // the 16 butterflies of stage s (span m = 2^s)
      const int h = 1 << (s - 1);
      const int j = b & (h - 1);
      const int lo = ((b >> (s - 1)) << s) + j;
      const float2 u = a[lo];
      const float2 t = w32mul<INV>(a[lo + h], j << (5 - s));
      a[lo] = make_float2(u.x + t.x, u.y + t.y);
      a[lo + h] = make_float2(u.x - t.x, u.y - t.y);
    }
  }
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = a[i];
}

// conj of the 32 values: an inverse transform is the forward transform of the conjugate,
// conjugated, so each kernel carries one copy of the transform's code (an instruction-cache
// working set half as large; the kernels were stalled on instruction fetch).
__device__ __forceinline__ void conj32(float2 (&v)[32]) {
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i].y = -v[i].y;
}

// Inner DFT and the W_1024^{n2 k1} factors (tw4[k1][n2]: rounded value and remainder).
template <bool INV>
__device__ __forceinline__ void four_step_first(float2 (&v)[32], int n2, const float4* tw4) {
  dft32<INV>(v);
#pragma unroll
  for (int k1 = 1; k1 < 32; ++k1) {
    const float4 w = tw4[k1 * 32 + n2];
    v[k1] = INV ? cmulc2f(v[k1], make_float2(w.x, w.y), make_float2(w.z, w.w))
                : cmul2f(v[k1], make_float2(w.x, w.y), make_float2(w.z, w.w));
  }
}

// A forward 1024-point transform of a row held by a warp (lane = n2, buf: 32 x kXStride
// values).
__device__ __forceinline__ void fft1024_warp(float2 (&v)[32], int lane, float2* buf,
                                             const float4* tw4) {
  four_step_first<false>(v, lane, tw4);
#pragma unroll
  for (int k1 = 0; k1 < 32; ++k1) buf[k1 * kXStride + lane] = v[k1];
  __syncwarp();
#pragma unroll
  for (int n2 = 0; n2 < 32; ++n2) v[n2] = buf[lane * kXStride + n2];
  __syncwarp();
  dft32<false>(v);
}

// ------------------------------------------------------------------ row pass
__global__ void __launch_bounds__(kRowWarps * 32, 2)
    row_fast_kernel(float2* __restrict__ data, const float4* __restrict__ tw4_g,
                    const float2* __restrict__ px, const float2* __restrict__ py,
                    const RowPassArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.halt != nullptr && __ldcg(a.halt) != 0) return;  // steady-state monitor halted the run
  float4* tw4 = reinterpret_cast<float4*>(smem_raw);                     // [32][32]
  float2* xb = reinterpret_cast<float2*>(tw4 + kN);                      // [warps][32][33]
  for (int i = threadIdx.x; i < kN; i += blockDim.x) tw4[i] = tw4_g[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int member = blockIdx.z;
  float2* buf = xb + warp * 32 * kXStride;
  const float2* pxm = px + static_cast<long long>(member) * a.table_stride;
  const float2* pym = py + static_cast<long long>(member) * a.table_stride;
  const float scale = static_cast<float>(a.scale);
  const long long plane = static_cast<long long>(kN) * a.ny;
#pragma unroll 1
  for (int q = 0; q < kRowsPerWarp; ++q) {
    const int row = (blockIdx.x * kRowWarps + warp) * kRowsPerWarp + q;
    float2* d = data + member * plane + static_cast<long long>(row) * kN;
    float2 v[32];
#pragma unroll
    for (int t = 0; t < 32; ++t) v[t] = d[lane + 32 * t];
    // Phase 0: forward transform and kick; phase 1: the inverse transform (conj32).
#pragma unroll 1
    for (int ph = 0; ph < 2; ++ph) {
      if (ph == 0 ? a.forward : a.inverse) {
        if (ph == 1) conj32(v);
        fft1024_warp(v, lane, buf, tw4);
        if (ph == 1) conj32(v);
      }
      if (ph == 0 && a.multiply) {
        // psi (1 + dx) (1 + dy) scale, the factor differences stored (see split.cu)
        const float2 dy = pym[row];
#pragma unroll
        for (int r = 0; r < 32; ++r) {
          const float2 dx = pxm[lane + 32 * r];
          const float2 dxy = cmul(dx, dy);
          const float2 f1 = make_float2(dx.x + dy.x + dxy.x, dx.y + dy.y + dxy.y);
          const float2 vf = cmul(v[r], f1);
          v[r] = make_float2((v[r].x + vf.x) * scale, (v[r].y + vf.y) * scale);
        }
      }
    }
#pragma unroll
    for (int t = 0; t < 32; ++t) d[lane + 32 * t] = v[t];
  }
}

// ------------------------------------------------------------------ IFRK row pass
// ifrk_row_kernel (ifrk.cu) for FP32 rows of 1024 sites of a one-component field: the row's
// forward transform, the stage spectrum saved, the Lawson combination
// sum_t coef_t Ex_t[kx] Ey_t[ky] src_t (src_t: this row's spectrum, or a stored one), the
// inverse transform; a warp per row, as row_fast_kernel.
__global__ void __launch_bounds__(kRowWarps * 32, 2)
    ifrk_row_fast_kernel(const float2* __restrict__ in, float2* __restrict__ save,
                         float2* __restrict__ out, const float2* __restrict__ tables,
                         const float4* __restrict__ tw4_g, const IfrkRowArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // The twiddle table through L1, as in the IFRK column pass (no block barrier either).
  const float4* tw4 = tw4_g;                                             // [32][32]
  float2* xb = reinterpret_cast<float2*>(smem_raw);                      // [warps][32][33]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int member = blockIdx.z;
  float2* buf = xb + warp * 32 * kXStride;
  const long long table_stride = static_cast<long long>(a.members) * (kN + a.ny);
#pragma unroll 1
  for (int q = 0; q < kRowsPerWarp; ++q) {
    const int row = (blockIdx.x * kRowWarps + warp) * kRowsPerWarp + q;
    const long long moff = member * a.member_stride + static_cast<long long>(row) * kN;
    float2 v[32];
#pragma unroll
    for (int t = 0; t < 32; ++t) v[t] = in ? in[moff + lane + 32 * t] : make_float2(0.f, 0.f);
    // Phase 0: forward transform, save, combination; phase 1: the inverse transform (conj32).
#pragma unroll 1
    for (int ph = 0; ph < 2; ++ph) {
      if (ph == 0 ? a.forward : a.inverse) {
        if (ph == 1) conj32(v);
        fft1024_warp(v, lane, buf, tw4);
        if (ph == 1) conj32(v);
      }
      if (ph == 1) continue;
      if (save) {
#pragma unroll
        for (int r = 0; r < 32; ++r) save[moff + lane + 32 * r] = v[r];
      }
      // The term on this row's own spectrum (src null; at most one) first, in place, then the
      // stored spectra, a term at a time so that the row stays the only array in registers.
      int own = -1;
      for (int s = 0; s < a.terms; ++s)
        if (a.src[s] == nullptr) own = s;
      const float2* tabs = tables + static_cast<long long>(member) * (kN + a.ny);
      if (own >= 0) {
        const float2* tab = tabs + a.table[own] * table_stride;
        const float2 ey = tab[kN + row];
        const float c = static_cast<float>(a.coef[own]);
#pragma unroll
        for (int r = 0; r < 32; ++r) {
          const float2 ev = cmul(cmul(tab[lane + 32 * r], ey), v[r]);
          v[r] = make_float2(c * ev.x, c * ev.y);
        }
      } else {
#pragma unroll
        for (int r = 0; r < 32; ++r) v[r] = make_float2(0.f, 0.f);
      }
#pragma unroll 1
      for (int s = 0; s < a.terms; ++s) {
        if (s == own) continue;
        const float2* tab = tabs + a.table[s] * table_stride;
        const float2* src = static_cast<const float2*>(a.src[s]) + moff;
        const float2 ey = tab[kN + row];
        const float c = static_cast<float>(a.coef[s]);
#pragma unroll
        for (int r = 0; r < 32; ++r) {
          const float2 ev = cmul(cmul(tab[lane + 32 * r], ey), src[lane + 32 * r]);
          v[r].x += c * ev.x;
          v[r].y += c * ev.y;
        }
      }
    }
#pragma unroll
    for (int t = 0; t < 32; ++t) out[moff + lane + 32 * t] = v[t];
  }
}

// ------------------------------------------------------------------ column pass
// A forward 1024-point transform of the block's eight columns (thread = (column c, n2 = p));
// pan is the panel's exchange buffer ([c][k1][n2], columns kPanelStride apart).
__device__ __forceinline__ void fft1024_panel(float2 (&v)[32], int p, int c, float2* pan,
                                              const float4* tw4) {
  four_step_first<false>(v, p, tw4);
  __syncthreads();  // every earlier read of pan is done
#pragma unroll
  for (int k1 = 0; k1 < 32; ++k1) pan[c * kPanelStride + k1 * kXStride + p] = v[k1];
  __syncthreads();
#pragma unroll
  for (int n2 = 0; n2 < 32; ++n2) v[n2] = pan[c * kPanelStride + p * kXStride + n2];
  dft32<false>(v);
}

// The local step of the single case (LocalStep::single) over a panel in site order
// ([row][column] in pan), kSiteBatch sites a thread at a time: the reservoir and envelope
// loads of the whole batch are issued before the first site's arithmetic.  One site at a time,
// a site's reservoir store would come before the next site's loads, which the compiler may not
// move above it (the same array), so a thread would keep one site's loads in flight.
constexpr int kSiteBatch = 4;  // 8 measured slightly slower
template <int OP, bool NOISE>
__device__ __forceinline__ void panel_local_single(const LocalStep<float>& local, float2* pan,
                                                   int nx, int x0) {
  const int threads = static_cast<int>(blockDim.x);
  for (int e0 = threadIdx.x; e0 < kPanel * kN; e0 += kSiteBatch * threads) {
    int o[kSiteBatch];
    bool ok[kSiteBatch];
    float2 x[kSiteBatch];
    float n[kSiteBatch], P[kSiteBatch];
#pragma unroll
    for (int u = 0; u < kSiteBatch; ++u) {
      const int e = e0 + u * threads;
      ok[u] = e < kPanel * kN;
      const int ee = ok[u] ? e : e0;  // a site of the panel: loads stay in bounds
      o[u] = (ee / kPanel) * nx + x0 + ee % kPanel;
      x[u] = pan[ee];
      n[u] = local.rm[o[u]];
      P[u] = local.pm[o[u]];
    }
#pragma unroll
    for (int u = 0; u < kSiteBatch; ++u)
      n[u] = local.template step_single<OP, NOISE>(x[u], n[u], P[u], o[u]);
#pragma unroll
    for (int u = 0; u < kSiteBatch; ++u) {
      if (!ok[u]) continue;
      pan[e0 + u * threads] = x[u];
      if (OP != SPLIT_OP_NONLINEAR) local.rm[o[u]] = n[u];
    }
  }
}

__global__ void __launch_bounds__(kPanel * 32, 2)
    col_fast_kernel(float2* __restrict__ data, float* __restrict__ res, const float* __restrict__ pump,
                    const float* __restrict__ potential, const float4* __restrict__ tw4_g,
                    const SplitConst<float>* __restrict__ consts, const float* __restrict__ scales,
                    const unsigned long long* __restrict__ step_base, const ColPassArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.halt != nullptr && __ldcg(a.halt) != 0) return;  // steady-state monitor halted the run
  float4* tw4 = reinterpret_cast<float4*>(smem_raw);  // [32][32]
  float2* pan = reinterpret_cast<float2*>(tw4 + kN);  // exchange, or [row][c] for the local step
  for (int i = threadIdx.x; i < kN; i += blockDim.x) tw4[i] = tw4_g[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c = lane & (kPanel - 1);
  const int p = warp * 4 + (lane >> 3);  // n2: 0..31
  const int member = blockIdx.z;
  const int x0 = blockIdx.x * kPanel;
  const long long plane = static_cast<long long>(a.nx) * kN;
  float2* d = data + member * plane + x0 + c;
  float2 v[32];
#pragma unroll
  for (int t = 0; t < 32; ++t) v[t] = d[static_cast<long long>(p + 32 * t) * a.nx];
  // Phase 0: the inverse transform (conj32 around the forward one) and the local step;
  // phase 1: the forward transform.
#pragma unroll 1
  for (int ph = 0; ph < 2; ++ph) {
    if (ph == 0 ? a.inverse : a.forward) {
      if (ph == 0) conj32(v);
      fft1024_panel(v, p, c, pan, tw4);
      if (ph == 0) conj32(v);
    }
    if (ph == 1 || a.op == SPLIT_OP_NONE) continue;
    // Through shared memory in site order, so that the local step is one loop.
    __syncthreads();
#pragma unroll
    for (int t = 0; t < 32; ++t) pan[(p + 32 * t) * kPanel + c] = v[t];
    __syncthreads();
    const LocalStep<float> local(a, member, res, pump, potential, consts, scales, step_base);
    if (local.single()) {
      const int nx = a.nx;
      switch (a.op * 2 + (a.noise ? 1 : 0)) {
#define PG_SPLIT_SINGLE(OP, NOISE)             \
  case OP * 2 + NOISE:                         \
    panel_local_single<OP, NOISE>(local, pan, nx, x0); \
    break;
        PG_SPLIT_SINGLE(SPLIT_OP_KOUTER, 1)
        PG_SPLIT_SINGLE(SPLIT_OP_KOUTER, 0)
        PG_SPLIT_SINGLE(SPLIT_OP_NONLINEAR, 1)
        PG_SPLIT_SINGLE(SPLIT_OP_NONLINEAR, 0)
        PG_SPLIT_SINGLE(SPLIT_OP_RES_START, 1)
        PG_SPLIT_SINGLE(SPLIT_OP_RES_START, 0)
        PG_SPLIT_SINGLE(SPLIT_OP_RES_END, 1)
        PG_SPLIT_SINGLE(SPLIT_OP_RES_END, 0)
        PG_SPLIT_SINGLE(SPLIT_OP_RES_END_START, 1)
        PG_SPLIT_SINGLE(SPLIT_OP_RES_END_START, 0)
#undef PG_SPLIT_SINGLE
        default:
          break;
      }
    } else {
#pragma unroll 2
      for (int e = threadIdx.x; e < kPanel * kN; e += blockDim.x) {
        const int row = e / kPanel, col = e % kPanel;
        float2 x = pan[e];
        local.apply(x, static_cast<long long>(row) * a.nx + x0 + col);
        pan[e] = x;
      }
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < 32; ++t) v[t] = pan[(p + 32 * t) * kPanel + c];
  }
#pragma unroll
  for (int t = 0; t < 32; ++t) d[static_cast<long long>(p + 32 * t) * a.nx] = v[t];
}

// ------------------------------------------------------------------ IFRK column pass
// ifrk_col_kernel (ifrk.cu) for FP32 columns of 1024 sites of a one-component field: the
// forward-only pass that forms W (mode 3, any reservoir), and the stage and step-end passes
// (modes 0 and 1) for one single reservoir and one laser (ifrk_sites_batched).  An eight-column
// panel, the inverse transform, the site step over the panel in shared memory in site order
// (ifrk_sites.cuh, kIfrkBatch sites a thread at a stage, kIfrkEndBatch at the step end), the
// forward transform.  The error norm (mode 2) stays on the generic pass.
constexpr int kIfrkBatch = 8;     // 4 / 2 measured 4 % slower
constexpr int kIfrkEndBatch = 4;
__global__ void __launch_bounds__(kPanel * 32, 2)
    ifrk_col_fast_kernel(float2* __restrict__ psi, const float* __restrict__ n0,
                         float* __restrict__ dn_out, float* __restrict__ n_out,
                         float2* __restrict__ psi_start, float2* __restrict__ psi_new,
                         const float* __restrict__ pump, const float* __restrict__ potential,
                         const float4* __restrict__ tw4_g,
                         const SplitConst<float>* __restrict__ consts,
                         const float* __restrict__ scales,
                         const unsigned long long* __restrict__ step_base, const IfrkColArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // The twiddle table is read through L1 rather than staged in shared memory: two blocks an
  // SM then leave the driver a larger L1 for the site step's loads (+4.5 % on the step; the
  // split-step column pass, with fewer loads a site, gains nothing from it).
  const float4* tw4 = tw4_g;                          // [32][32]
  float2* pan = reinterpret_cast<float2*>(smem_raw);  // exchange, or [row][c] for the site step
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c = lane & (kPanel - 1);
  const int p = warp * 4 + (lane >> 3);  // n2: 0..31
  const int member = blockIdx.z;
  const int x0 = blockIdx.x * kPanel;
  const long long plane = static_cast<long long>(a.nx) * kN;
  float2* d = psi + member * plane + x0 + c;
  float2 v[32];
#pragma unroll
  for (int t = 0; t < 32; ++t) v[t] = d[static_cast<long long>(p + 32 * t) * a.nx];
  // Phase 0: the inverse transform (conj32 around the forward one) and the site step;
  // phase 1: the forward transform (one copy of the transform's code).
#pragma unroll 1
  for (int ph = 0; ph < 2; ++ph) {
    if (ph == 0 ? a.inverse : a.forward) {
      if (ph == 0) conj32(v);
      fft1024_panel(v, p, c, pan, tw4);
      if (ph == 0) conj32(v);
    }
    if (ph == 1 || a.mode == 3) continue;
    __syncthreads();
#pragma unroll
    for (int t = 0; t < 32; ++t) pan[(p + 32 * t) * kPanel + c] = v[t];
    __syncthreads();
    {
      const SplitConst<float> k = consts[member];
      const float s0 = scales ? scales[static_cast<long long>(a.scale_index) * a.members + member]
                              : 0.f;
      const float* pm = pump + member * a.pump_stride;
      const float* vm =
          potential ? potential + member * a.pot_stride * (a.potential == 2 ? 2 : 1) : nullptr;
      const unsigned long long step = a.noise ? step_base[0] + a.step_offset : 0ull;
      const PhiloxCellPrefix prefix = philox_cell_prefix(
          static_cast<uint32_t>(step), static_cast<uint32_t>(step >> 32), 1u,
          static_cast<uint32_t>(k.seed), static_cast<uint32_t>(k.seed >> 32));
      ifrk_sites_run<float, kIfrkBatch, kIfrkEndBatch>(pan, kPanel, 3, kN, a, k, x0,
                                                       member * plane, n0, dn_out, n_out,
                                                       psi_start, psi_new, pm, vm, s0, prefix);
    }
    __syncthreads();
    if (a.mode == 1 && !a.forward) return;
#pragma unroll
    for (int t = 0; t < 32; ++t) v[t] = pan[(p + 32 * t) * kPanel + c];
  }
#pragma unroll
  for (int t = 0; t < 32; ++t) d[static_cast<long long>(p + 32 * t) * a.nx] = v[t];
}

size_t row_fast_smem() { return kN * sizeof(float4) + kRowWarps * 32 * kXStride * sizeof(float2); }
size_t col_fast_smem() { return kN * sizeof(float4) + kPanel * kPanelStride * sizeof(float2); }
size_t ifrk_col_fast_smem() { return kPanel * kPanelStride * sizeof(float2); }
size_t ifrk_row_fast_smem() { return kRowWarps * 32 * kXStride * sizeof(float2); }

}  // namespace

bool split_fast_row(int nx, int ny) { return nx == kN && ny % (kRowWarps * kRowsPerWarp) == 0; }
bool split_fast_col(int nx, int ny) { return ny == kN && nx % kPanel == 0; }

void split_fast_twiddles(float* out) {
  // tw4[k1][n2] = W_1024^{n2 k1}: rounded value and remainder, from double precision.
  const double pi = 3.141592653589793238462643383279502884;
  for (int k1 = 0; k1 < 32; ++k1)
    for (int n2 = 0; n2 < 32; ++n2) {
      const double ang = -2.0 * pi * static_cast<double>((n2 * k1) % kN) / kN;
      const double cr = std::cos(ang), ci = std::sin(ang);
      float* o = out + 4 * (k1 * 32 + n2);
      o[0] = static_cast<float>(cr);
      o[1] = static_cast<float>(ci);
      o[2] = static_cast<float>(cr - static_cast<double>(o[0]));
      o[3] = static_cast<float>(ci - static_cast<double>(o[1]));
    }
}

cudaError_t configure_split_fast() {
  cudaError_t e = cudaFuncSetAttribute(row_fast_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(row_fast_smem()));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(ifrk_row_fast_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(ifrk_row_fast_smem()));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(ifrk_col_fast_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(ifrk_col_fast_smem()));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(col_fast_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(col_fast_smem()));
}

cudaError_t launch_row_fast(float* data, const float* tw4, const float* px, const float* py,
                            const RowPassArgs& a, int members, cudaStream_t stream) {
  const dim3 grid(a.ny / (kRowWarps * kRowsPerWarp), 1, members);
  row_fast_kernel<<<grid, kRowWarps * 32, row_fast_smem(), stream>>>(
      reinterpret_cast<float2*>(data), reinterpret_cast<const float4*>(tw4),
      reinterpret_cast<const float2*>(px), reinterpret_cast<const float2*>(py), a);
  return cudaGetLastError();
}

bool ifrk_fast_row(const IfrkRowArgs& a) {
  return a.comps == 1 && !a.spinor && a.nx == kN && a.ny % (kRowWarps * kRowsPerWarp) == 0;
}

cudaError_t launch_ifrk_row_fast(const float* in, float* save, float* out, const float* tables,
                                 const float* tw4, const IfrkRowArgs& a, cudaStream_t stream) {
  const dim3 grid(a.ny / (kRowWarps * kRowsPerWarp), 1, a.members);
  ifrk_row_fast_kernel<<<grid, kRowWarps * 32, ifrk_row_fast_smem(), stream>>>(
      reinterpret_cast<const float2*>(in), reinterpret_cast<float2*>(save),
      reinterpret_cast<float2*>(out), reinterpret_cast<const float2*>(tables),
      reinterpret_cast<const float4*>(tw4), a);
  return cudaGetLastError();
}

bool ifrk_fast_col(const IfrkColArgs& a) {
  return a.comps == 1 && a.ny == kN && a.nx % kPanel == 0 &&
         static_cast<long long>(a.nx) * kN <= 0x7fffffffLL &&
         (a.mode == 3 || ifrk_sites_batched(a));
}

cudaError_t launch_ifrk_col_fast(float* psi, const float* n0, float* dn_out, float* n_out,
                                 const float* psi_start, const float* psi_new, const float* pump,
                                 const float* potential, const float* tw4,
                                 const SplitConst<float>* consts, const float* scales,
                                 const unsigned long long* step_base, const IfrkColArgs& a,
                                 cudaStream_t stream) {
  const dim3 grid(a.nx / kPanel, 1, a.members);
  ifrk_col_fast_kernel<<<grid, kPanel * 32, ifrk_col_fast_smem(), stream>>>(
      reinterpret_cast<float2*>(psi), n0, dn_out, n_out,
      reinterpret_cast<float2*>(const_cast<float*>(psi_start)),
      reinterpret_cast<float2*>(const_cast<float*>(psi_new)), pump, potential,
      reinterpret_cast<const float4*>(tw4), consts, scales, step_base, a);
  return cudaGetLastError();
}

cudaError_t launch_col_fast(float* data, float* res, const float* pump, const float* potential,
                            const float* tw4, const SplitConst<float>* consts, const float* scales,
                            const unsigned long long* step_base, const ColPassArgs& a,
                            cudaStream_t stream) {
  const dim3 grid(a.nx / kPanel, 1, a.members);
  col_fast_kernel<<<grid, kPanel * 32, col_fast_smem(), stream>>>(
      reinterpret_cast<float2*>(data), res, pump, potential, reinterpret_cast<const float4*>(tw4),
      consts, scales, step_base, a);
  return cudaGetLastError();
}

}  // namespace pg
