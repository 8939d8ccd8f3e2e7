// The site step of the IFRK column passes for the common configuration (device code shared by
// the generic column pass in ifrk.cu and the 1024-point register-resident column pass in
// split_fast.cu): one field component, one single reservoir, one laser.  Math as
// polarism/solver/ifrk_fft_cuda_solver.py:128-142 (right-hand side) and :148-241 (stage
// reservoir n0 + sum_j coef_j dn_j, single-reservoir derivative, step-end clamp and Wigner
// increment), restated from the generic loop of ifrk_col_kernel, which covers every other
// configuration.
#pragma once
#include "fft.cuh"
#include "ifrk_internal.h"
#include "philox.cuh"
#include "pg_internal.h"

namespace pg {
namespace {

__device__ __forceinline__ float mul_rn_i(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn_i(double a, double b) { return __dmul_rn(a, b); }

// Whether the column pass's site step has the batched form: one component, one single
// reservoir, one laser, a stage (mode 0, up to five terms) or the step end (mode 1, one to five
// terms).  Lawson RK4 and Dormand-Prince 5 have at most five nonzero terms in a tableau row.
__host__ __device__ inline bool ifrk_sites_batched(const IfrkColArgs& a) {
  const bool base = a.comps == 1 && a.res_fields == 1 && a.res_comps == 1 && a.pump_terms <= 1;
  return base && ((a.mode == 0 && a.terms <= 5) || (a.mode == 1 && a.terms >= 1 && a.terms <= 5));
}

// A stage (MODE 0) or step end (MODE 1) over a panel of C columns held in buf as [row][column]
// (C = 2^lc; ny rows; panel's first column x0; the member's plane at mbase).  Each thread takes
// U sites at a time and issues every global load of the batch (reservoir, the TERMS stage
// derivatives, envelope, potential) before it forms the first result, so U sites' loads are
// in flight; one site at a time, a site's stores would come before the next site's loads,
// which the compiler may not move above them.  The arithmetic is the generic loop's,
// expression for expression and in the same order.
template <typename T, int MODE, int TERMS, int U>
__device__ __forceinline__ void ifrk_sites_single(
    typename C2T<T>::type* buf, int C, int lc, int ny, const IfrkColArgs& a,
    const SplitConst<T>& k, int x0, long long mbase, const T* __restrict__ n0,
    T* __restrict__ dn_out, T* __restrict__ n_out, typename C2T<T>::type* __restrict__ psi_start,
    typename C2T<T>::type* __restrict__ psi_new, const T* __restrict__ pm,
    const T* __restrict__ vm, T s0, const PhiloxCellPrefix& prefix) {
  using C2 = typename C2T<T>::type;
  const int count = C * ny;
  const T* dn[TERMS > 0 ? TERMS : 1];
  T cf[TERMS > 0 ? TERMS : 1];
#pragma unroll
  for (int j = 0; j < TERMS; ++j) {
    dn[j] = static_cast<const T*>(a.dn[j]) + mbase;
    cf[j] = static_cast<T>(a.coef[j]);
  }
  const T* nm = n0 + mbase;
  const int stride = U * static_cast<int>(blockDim.x);
  for (int e0 = threadIdx.x; e0 < count; e0 += stride) {
    int o[U], bi[U];
    bool ok[U];
    C2 v[U];
    T nv[U], acc[U], pp[U], vre[U], vim[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int e = e0 + u * static_cast<int>(blockDim.x);
      ok[u] = e < count;
      const int ee = ok[u] ? e : e0;  // a site of the panel: loads stay in bounds
      const int c = ee & (C - 1), i = ee >> lc;
      o[u] = i * a.nx + x0 + c;
      bi[u] = i * C + c;
      v[u] = buf[bi[u]];
      nv[u] = nm[o[u]];
      acc[u] = T(0);
      if (MODE == 0) {
        pp[u] = pm[o[u]];
        vre[u] = T(0);
        vim[u] = T(0);
        if (vm) {
          vre[u] = a.potential == 2 ? vm[2 * static_cast<long long>(o[u])] : vm[o[u]];
          vim[u] = a.potential == 2 ? vm[2 * static_cast<long long>(o[u]) + 1] : T(0);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < TERMS; ++j)
#pragma unroll
      for (int u = 0; u < U; ++u) acc[u] += cf[j] * dn[j][o[u]];
    if (MODE == 0) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (!ok[u]) continue;
        const T nval = nv[u] + acc[u];
        const C2 x = v[u];
        const T rho = x.x * x.x + x.y * x.y;
        if (psi_start) psi_start[mbase + o[u]] = x;
        const T eff = vre[u] + k.g_C * rho + k.g_R * nval;
        const T e_over = eff * k.inv_hbar;
        const T g = T(0.5) * (k.R * nval - k.gamma_C) + vim[u] * k.inv_hbar;
        buf[bi[u]] = C2{g * x.x + e_over * x.y, g * x.y - e_over * x.x};
        const T P = mul_rn_i(s0, pp[u]);
        dn_out[mbase + o[u]] = P - (k.gamma_R + k.R * rho) * nval;
      }
    } else {
      Words4 w[U];
      if (a.noise) {
        uint32_t cell[U];
#pragma unroll
        for (int u = 0; u < U; ++u) cell[u] = static_cast<uint32_t>(o[u]);
        philox_cells(cell, prefix, w);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (!ok[u]) continue;
        T nval = nv[u] + acc[u];
        nval = nval > T(0) ? nval : T(0);
        n_out[mbase + o[u]] = nval;
        C2 x = v[u];
        if (a.noise) {
          WignerDraw<T>::apply(w[u], k.noise_a + k.noise_b * nval, x.x, x.y);
          buf[bi[u]] = x;
        }
        psi_new[mbase + o[u]] = x;
      }
    }
  }
}

// ifrk_sites_single for the launch's mode and term count (ifrk_sites_batched(a) holds); U0 /
// U1 sites a batch at a stage / the step end.
template <typename T, int U0, int U1>
__device__ __forceinline__ void ifrk_sites_run(
    typename C2T<T>::type* buf, int C, int lc, int ny, const IfrkColArgs& a,
    const SplitConst<T>& k, int x0, long long mbase, const T* n0, T* dn_out, T* n_out,
    typename C2T<T>::type* psi_start, typename C2T<T>::type* psi_new, const T* pm, const T* vm,
    T s0, const PhiloxCellPrefix& prefix) {
  switch (a.mode * 8 + a.terms) {
#define PG_IFRK_SITES(MODE, TERMS, U)                                                         \
  case MODE * 8 + TERMS:                                                                      \
    ifrk_sites_single<T, MODE, TERMS, U>(buf, C, lc, ny, a, k, x0, mbase, n0, dn_out, n_out, \
                                         psi_start, psi_new, pm, vm, s0, prefix);             \
    break;
    PG_IFRK_SITES(0, 0, U0)
    PG_IFRK_SITES(0, 1, U0)
    PG_IFRK_SITES(0, 2, U0)
    PG_IFRK_SITES(0, 3, U0)
    PG_IFRK_SITES(0, 4, U0)
    PG_IFRK_SITES(0, 5, U0)
    PG_IFRK_SITES(1, 1, U1)
    PG_IFRK_SITES(1, 2, U1)
    PG_IFRK_SITES(1, 3, U1)
    PG_IFRK_SITES(1, 4, U1)
    PG_IFRK_SITES(1, 5, U1)
#undef PG_IFRK_SITES
    default:
      break;
  }
}

}  // namespace
}  // namespace pg
