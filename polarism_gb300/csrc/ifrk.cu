// Lawson integrating-factor RK (IFRK) passes on the Stockham FFT building blocks.
//
// Math follows polarism/solver/ifrk_fft_cuda_solver.py:96-109 (Lawson factor
// exp(i (-hbar/2m) tau k^2)), :128-142 (nonlinear right-hand side), :148-241 (stage
// combination psi_hat_i = E(c_i h) psi_hat_0 + h sum_j a_ij E((c_i - c_j) h) f_hat_j,
// stage-coupled reservoir n_i = n_0 + h sum_j a_ij dn_j, final reservoir clamp) and
// :243-293 (embedded error norm: RMS of |e| / (atol + rtol max(|y0|, |y1|)) over the
// condensate and the reservoir, accumulated here in FP64).  The fused kernels of
// polarism/solver/ifrk_cuda_fused.py:10-108 (combine_k / stage_rhs / finish_res) map onto
// one row pass and one column pass per stage.
#include <algorithm>

#include "fft.cuh"
#include "ifrk_internal.h"
#include "ifrk_sites.cuh"
#include "philox.cuh"
#include "pg_internal.h"

namespace pg {
namespace {

constexpr double kTwoPi = 6.283185307179586476925286766559;

// sin and cos of an FP64 phase angle in the working precision: FP32 takes the angle reduced
// to [-pi, pi] in FP64 first, so the only FP32 error is that of the reduced angle.
__device__ __forceinline__ void sincos_angle(double a, float* s, float* c) {
  const double n = rint(a * (1.0 / kTwoPi));
  sincosf(static_cast<float>(fma(-n, kTwoPi, a)), s, c);
}
__device__ __forceinline__ void sincos_angle(double a, double* s, double* c) { sincos(a, s, c); }

// sin and cos of (r_hi + r_lo)(t_hi + t_lo): the product is formed as p + t with the exact
// rounding error of p = r_hi t_hi (an FMA) and the cross terms, reduced by 2 pi split into two
// floats (Cody and Waite's method), so the reduced angle carries an absolute error of a few
// 1e-7 for any angle below 2^24 turns -- the accuracy of the FP64 reduction rounded to FP32.
__device__ __forceinline__ void sincos_product(float r_hi, float r_lo, float t_hi, float t_lo,
                                               float* s, float* c) {
  constexpr float kTwoPiHi = 6.28318548202514648f;        // float(2 pi)
  constexpr float kTwoPiLo = -1.74845553146951617e-07f;   // 2 pi - kTwoPiHi
  constexpr float kInvTwoPi = 0.159154943091895336f;
  const float p = r_hi * t_hi;
  const float e = fmaf(r_hi, t_hi, -p);
  const float t = fmaf(r_hi, t_lo, fmaf(r_lo, t_hi, e));
  const float n = rintf(p * kInvTwoPi);
  const float d = fmaf(-n, kTwoPiLo, fmaf(-n, kTwoPiHi, p)) + t;
  sincosf(d, s, c);
}

// Per-mode FP32 table of the two-component Lawson factor, formed once in FP64.
__global__ void spin_mode_table_kernel(float* __restrict__ table, const SpinorConst* __restrict__ consts,
                                       int nx, int ny, double kx_unit, double ky_unit) {
  const int member = blockIdx.y;
  const long long plane = static_cast<long long>(nx) * ny;
  const SpinorConst sc = consts[member];
  float* tm = table + static_cast<long long>(member) * kSpinModeFields * plane;
  for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < plane;
       e += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int j = static_cast<int>(e % nx);
    const int i = static_cast<int>(e / nx);
    const double kx = kx_unit * static_cast<double>(j < (nx >> 1) ? j : j - nx);
    const double ky = ky_unit * static_cast<double>(i < (ny >> 1) ? i : i - ny);
    const double k2 = kx * kx + ky * ky;
    const double rate_e = sc.rate * k2;
    const double bk2 = sc.beta * k2;
    const double omega = sqrt(sc.half_z * sc.half_z + bk2 * bk2);
    const double rate_w = omega * sc.inv_hbar;
    const float re_hi = static_cast<float>(rate_e), rw_hi = static_cast<float>(rate_w);
    tm[0 * plane + e] = re_hi;
    tm[1 * plane + e] = static_cast<float>(rate_e - static_cast<double>(re_hi));
    tm[2 * plane + e] = rw_hi;
    tm[3 * plane + e] = static_cast<float>(rate_w - static_cast<double>(rw_hi));
    tm[4 * plane + e] = static_cast<float>(sc.beta * (kx * kx - ky * ky));
    tm[5 * plane + e] = static_cast<float>(-2.0 * sc.beta * kx * ky);
    tm[6 * plane + e] = omega > 0.0 ? static_cast<float>(1.0 / omega) : 0.0f;
  }
}

template <typename T>
__global__ void __launch_bounds__(1024) ifrk_row_kernel(const typename C2T<T>::type* __restrict__ in,
                                                        typename C2T<T>::type* __restrict__ save,
                                                        typename C2T<T>::type* __restrict__ out,
                                                        const typename C2T<T>::type* __restrict__ tables,
                                                        const typename C2T<T>::type* __restrict__ tw,
                                                        const IfrkRowArgs a) {
  using C2 = typename C2T<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2* tws = reinterpret_cast<C2*>(smem_raw);
  C2* buf = tws + a.nx;  // [component][row][x]
  const int member = blockIdx.z;
  const int row0 = blockIdx.x * a.rows;
  const int count = a.rows * a.nx;  // values per component
  const int comps = a.comps;
  const long long plane = static_cast<long long>(a.nx) * a.ny;
  const long long moff = member * a.member_stride + static_cast<long long>(row0) * a.nx;
  const int all = count * comps;
  for (int k = threadIdx.x; k < a.nx; k += blockDim.x) tws[k] = tw[k];
  if (in) {
    for (int e = threadIdx.x; e < all; e += blockDim.x) {
      const int c = e >= count ? 1 : 0;
      buf[e] = in[moff + c * plane + (e - c * count)];
    }
  }
  __syncthreads();
  const int log2batch = a.log2rows + (comps == 2 ? 1 : 0);
  if (a.forward) smem_fft<T, false, false>(buf, tws, a.log2nx, log2batch, 1, a.nx);
  if (save) {
    for (int e = threadIdx.x; e < all; e += blockDim.x) {
      const int c = e >= count ? 1 : 0;
      save[moff + c * plane + (e - c * count)] = buf[e];
    }
  }
  if (!a.spinor) {
    const long long table_stride = static_cast<long long>(a.members) * (a.nx + a.ny);
    for (int e = threadIdx.x; e < count; e += blockDim.x) {
      const int r = e >> a.log2nx;
      const int j = e & (a.nx - 1);
      const int i = row0 + r;
      C2 acc{T(0), T(0)};
#pragma unroll
      for (int t = 0; t < kIfrkMaxTerms; ++t) {
        if (t >= a.terms) break;
        const C2* tab = tables + a.table[t] * table_stride + static_cast<long long>(member) * (a.nx + a.ny);
        const C2 E = cmul(tab[j], tab[a.nx + i]);
        const C2 v = a.src[t] ? static_cast<const C2*>(a.src[t])[moff + e] : buf[e];
        const C2 ev = cmul(E, v);
        const T c = static_cast<T>(a.coef[t]);
        acc.x += c * ev.x;
        acc.y += c * ev.y;
      }
      buf[e] = acc;
    }
  } else {
    // Two components: out = sum_t coef_t / N exp(-i H(k) tau_t / hbar) src_t with
    // exp(-i H t) = exp(-i E t) [[cos - i s z, -i s u], [-i s u*, cos + i s z]],
    // s = sin(w t) / w, w = sqrt(z^2 + |u|^2), u = beta (kx - i ky)^2 (dispersion.py:66-83).
    const SpinorConst sc = static_cast<const SpinorConst*>(a.spin)[member];
    const T zf = static_cast<T>(sc.half_z);
    if constexpr (sizeof(T) == 4) {
      // FP32 state: the per-mode quantities come from the table and the angles are formed in
      // compensated FP32 (sincos_product); the arithmetic after the angles is the same.
      const float inv_hbar_f = static_cast<float>(sc.inv_hbar);
      const long long mplane = static_cast<long long>(a.nx) * a.ny;
      const float* tm = a.modes + static_cast<long long>(member) * kSpinModeFields * mplane +
                        static_cast<long long>(row0) * a.nx;
      for (int e = threadIdx.x; e < count; e += blockDim.x) {
        const float re_hi = tm[e], re_lo = tm[mplane + e];
        const float rw_hi = tm[2 * mplane + e], rw_lo = tm[3 * mplane + e];
        const float ure = tm[4 * mplane + e], uim = tm[5 * mplane + e];
        const float inv_om = tm[6 * mplane + e];
        C2 acc0{T(0), T(0)}, acc1{T(0), T(0)};
#pragma unroll 1
        for (int t = 0; t < a.terms; ++t) {
          T se, ce, sw, cw;
          sincos_product(re_hi, re_lo, a.tau_hi[t], a.tau_lo[t], &se, &ce);
          sincos_product(rw_hi, rw_lo, a.tau_hi[t], a.tau_lo[t], &sw, &cw);
          const T so = inv_om > 0.0f ? sw * inv_om : a.tau_hi[t] * inv_hbar_f;
          C2 s0, s1;
          if (a.src[t]) {
            const C2* src = static_cast<const C2*>(a.src[t]) + moff;
            s0 = src[e];
            s1 = src[plane + e];
          } else {
            s0 = buf[e];
            s1 = buf[count + e];
          }
          const T sz = so * zf;
          const C2 a0{cw * s0.x + sz * s0.y + so * (uim * s1.x + ure * s1.y),
                      cw * s0.y - sz * s0.x + so * (uim * s1.y - ure * s1.x)};
          const C2 a1{cw * s1.x - sz * s1.y + so * (ure * s0.y - uim * s0.x),
                      cw * s1.y + sz * s1.x - so * (ure * s0.x + uim * s0.y)};
          const T w = static_cast<T>(a.coef[t] * a.inv_n);
          acc0.x += w * (ce * a0.x + se * a0.y);
          acc0.y += w * (ce * a0.y - se * a0.x);
          acc1.x += w * (ce * a1.x + se * a1.y);
          acc1.y += w * (ce * a1.y - se * a1.x);
        }
        buf[e] = acc0;
        buf[count + e] = acc1;
      }
    } else
    for (int e = threadIdx.x; e < count; e += blockDim.x) {
      const int j = e & (a.nx - 1);
      const int i = row0 + (e >> a.log2nx);
      const double kx = a.kx_unit * static_cast<double>(j < (a.nx >> 1) ? j : j - a.nx);
      const double ky = a.ky_unit * static_cast<double>(i < (a.ny >> 1) ? i : i - a.ny);
      const double k2 = kx * kx + ky * ky;
      const double rate_e = sc.rate * k2;                 // E(k) / hbar
      const double bk2 = sc.beta * k2;
      const double omega = sqrt(sc.half_z * sc.half_z + bk2 * bk2);
      const double rate_w = omega * sc.inv_hbar;
      const T ure = static_cast<T>(sc.beta * (kx * kx - ky * ky));
      const T uim = static_cast<T>(-2.0 * sc.beta * kx * ky);
      const T om = static_cast<T>(omega);
      C2 acc0{T(0), T(0)}, acc1{T(0), T(0)};
#pragma unroll 1
      for (int t = 0; t < a.terms; ++t) {
        const double tau = a.tau[t];
        T se, ce, sw, cw;
        sincos_angle(rate_e * tau, &se, &ce);
        sincos_angle(rate_w * tau, &sw, &cw);
        const T so = omega > 0.0 ? sw / om : static_cast<T>(tau * sc.inv_hbar);
        C2 s0, s1;
        if (a.src[t]) {
          const C2* src = static_cast<const C2*>(a.src[t]) + moff;
          s0 = src[e];
          s1 = src[plane + e];
        } else {
          s0 = buf[e];
          s1 = buf[count + e];
        }
        const T sz = so * zf;
        // (cos - i s z) s0 + (-i s u) s1  and  (-i s u*) s0 + (cos + i s z) s1
        const C2 a0{cw * s0.x + sz * s0.y + so * (uim * s1.x + ure * s1.y),
                    cw * s0.y - sz * s0.x + so * (uim * s1.y - ure * s1.x)};
        const C2 a1{cw * s1.x - sz * s1.y + so * (ure * s0.y - uim * s0.x),
                    cw * s1.y + sz * s1.x - so * (ure * s0.x + uim * s0.y)};
        const T w = static_cast<T>(a.coef[t] * a.inv_n);
        // phase exp(-i E t) = (ce, -se)
        acc0.x += w * (ce * a0.x + se * a0.y);
        acc0.y += w * (ce * a0.y - se * a0.x);
        acc1.x += w * (ce * a1.x + se * a1.y);
        acc1.y += w * (ce * a1.y - se * a1.x);
      }
      buf[e] = acc0;
      buf[count + e] = acc1;
    }
  }
  __syncthreads();
  if (a.inverse) smem_fft<T, true, false>(buf, tws, a.log2nx, log2batch, 1, a.nx);
  for (int e = threadIdx.x; e < all; e += blockDim.x) {
    const int c = e >= count ? 1 : 0;
    out[moff + c * plane + (e - c * count)] = buf[e];
  }
}

template <typename T>
__device__ __forceinline__ T scaled_square(T mag, T scale) {
  // (mag / scale)^2 with the reference's handling of a zero scale.
  if (scale > T(0)) {
    const T r = mag / scale;
    return r * r;
  }
  return mag == T(0) ? T(0) : T(INFINITY);
}

// Column pass over a panel of `cols` columns of every component of one member.  Reservoir
// planes are laid out [field][member][reservoir component][y][x]; with one reservoir
// component per field component each component feeds its own reservoirs with its own
// density and pump share, otherwise one shared set sees the summed density
// (ifrk_fft_cuda_solver.py:118-126; single_reservoir.py:81-98; double_reservoir.py:106-130).
template <typename T>
__global__ void __launch_bounds__(1024) ifrk_col_kernel(typename C2T<T>::type* __restrict__ psi,
                                                        const T* __restrict__ n0,
                                                        T* __restrict__ dn_out,
                                                        T* __restrict__ n_out,
                                                        typename C2T<T>::type* __restrict__ psi_start,
                                                        typename C2T<T>::type* __restrict__ psi_new,
                                                        const T* __restrict__ pump,
                                                        const T* __restrict__ potential,
                                                        const typename C2T<T>::type* __restrict__ tw,
                                                        const SplitConst<T>* __restrict__ consts,
                                                        const T* __restrict__ scales,
                                                        const unsigned long long* __restrict__ step_base,
                                                        double* __restrict__ partials,
                                                        const IfrkColArgs a) {
  using C2 = typename C2T<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2* tws = reinterpret_cast<C2*>(smem_raw);
  C2* buf = tws + a.ny;  // [y][component][column]
  __shared__ double red[32];
  const int member = blockIdx.z;
  const int x0 = blockIdx.x * a.cols;
  const int C = a.cols;
  const int comps = a.comps;
  const int lcc = a.log2cols + a.log2comps;
  const int CC = 1 << lcc;  // panel columns over all components
  const long long plane = static_cast<long long>(a.nx) * a.ny;
  const long long fbase = static_cast<long long>(member) * comps * plane;
  C2* d = psi + fbase;
  for (int k = threadIdx.x; k < a.ny; k += blockDim.x) tws[k] = tw[k];
  const int count = C * a.ny;  // sites of the panel
  const int all = count * comps;
  for (int e = threadIdx.x; e < all; e += blockDim.x) {
    const int c2 = e & (CC - 1), i = e >> lcc;
    const int comp = c2 >> a.log2cols, c = c2 & (C - 1);
    buf[i * CC + c2] = d[comp * plane + static_cast<long long>(i) * a.nx + x0 + c];
  }
  __syncthreads();
  if (a.inverse) smem_fft<T, true, true>(buf, tws, a.log2ny, lcc, CC, 1);
  double local = 0.0;
  if (a.mode != 3) {
    const SplitConst<T> k = consts[member];
    const int L = a.pump_terms > 1 ? a.pump_terms : 1;
    const T* cs = scales ? scales + static_cast<long long>(a.scale_index * L) * a.members + member
                         : nullptr;
    const T s0 = cs ? cs[0] : T(0);
    const T* pm = pump + member * a.pump_stride;
    const T* vm = potential ? potential + member * a.pot_stride * (a.potential == 2 ? 2 : 1) : nullptr;
    const unsigned long long step = a.noise ? step_base[0] + a.step_offset : 0ull;
    // Philox rounds that depend only on (step, stream, key), per component stream 1 + comp.
    const PhiloxCellPrefix prefix[2] = {
        philox_cell_prefix(static_cast<uint32_t>(step), static_cast<uint32_t>(step >> 32), 1u,
                           static_cast<uint32_t>(k.seed), static_cast<uint32_t>(k.seed >> 32)),
        philox_cell_prefix(static_cast<uint32_t>(step), static_cast<uint32_t>(step >> 32), 2u,
                           static_cast<uint32_t>(k.seed), static_cast<uint32_t>(k.seed >> 32))};
    const int F = a.res_fields, Cr = a.res_comps;
    const int NQ = F * Cr;
    const long long qstride = static_cast<long long>(Cr) * plane;      // reservoir member stride
    const long long fstride = static_cast<long long>(a.members) * qstride;  // field stride
    // The common configuration in batches of sites a thread (ifrk_sites.cuh): three at a stage
    // and two at the step end (FP64: two and one) are the most that stay within the 64
    // registers of 1024-thread blocks without spilling.
    const bool batched = ifrk_sites_batched(a) && plane <= 0x7fffffffLL;
    if (batched)
      ifrk_sites_run<T, sizeof(T) == 4 ? 3 : 2, sizeof(T) == 4 ? 2 : 1>(
          buf, C, a.log2cols, a.ny, a, k, x0, static_cast<long long>(member) * plane, n0, dn_out,
          n_out, psi_start, psi_new, pm, vm, s0, prefix[0]);
    // Every other configuration: a site at a time.
    if (!batched)
    for (int e = threadIdx.x; e < count; e += blockDim.x) {
      const int c = e & (C - 1), i = e >> a.log2cols;
      const long long o = static_cast<long long>(i) * a.nx + x0 + c;
      C2 v[2];
      v[0] = buf[i * CC + c];
      v[1] = comps == 2 ? buf[i * CC + C + c] : C2{T(0), T(0)};
      // Stage (or final) reservoir values n0 + sum coef_j dn_j; the sum alone is the error term.
      T nval[4] = {T(0), T(0), T(0), T(0)}, dsum[4] = {T(0), T(0), T(0), T(0)};
      long long ridx[4] = {0, 0, 0, 0};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (q >= NQ) break;
        const int f = Cr == 2 ? (q >> 1) : q, cr = Cr == 2 ? (q & 1) : 0;
        ridx[q] = f * fstride + member * qstride + cr * plane + o;
        T acc = T(0);
#pragma unroll
        for (int j = 0; j < kIfrkMaxStages; ++j) {
          if (j >= a.terms) break;
          acc += static_cast<T>(a.coef[j]) * static_cast<const T*>(a.dn[j])[ridx[q]];
        }
        dsum[q] = acc;
        nval[q] = n0[ridx[q]] + acc;
      }
      if (a.mode == 0) {
        T rho[2];
#pragma unroll
        for (int comp = 0; comp < 2; ++comp) {
          rho[comp] = v[comp].x * v[comp].x + v[comp].y * v[comp].y;
          if (comp < comps && psi_start) psi_start[fbase + comp * plane + o] = v[comp];
        }
        T vre = T(0), vim = T(0);
        if (vm) {
          vre = a.potential == 2 ? vm[2 * o] : vm[o];
          vim = a.potential == 2 ? vm[2 * o + 1] : T(0);
        }
#pragma unroll
        for (int comp = 0; comp < 2; ++comp) {
          if (comp >= comps) break;
          const int ra = Cr == comps ? comp : 0;
          const T nA = F >= 1 ? nval[ra] : T(0);
          const T nI = F == 2 ? nval[Cr + ra] : T(0);
          // rhs = (-i/hbar) (V_re + g_C rho + alpha_2 rho_other + g_R n_A + g_I n_I) psi
          //       + (R n_A - gamma_C)/2 psi + (V_im / hbar) psi
          T eff = vre + k.g_C * rho[comp] + k.g_R * nA;
          if (comps == 2) eff += k.alpha_2 * rho[1 - comp];
          if (F == 2) eff += k.g_I * nI;
          const T e_over = eff * k.inv_hbar;
          const T g = T(0.5) * (k.R * nA - k.gamma_C) + vim * k.inv_hbar;
          buf[i * CC + comp * C + c] = C2{g * v[comp].x + e_over * v[comp].y, g * v[comp].y - e_over * v[comp].x};
        }
        if (F >= 1) {
          const T p_site = L > 1 && cs ? pump_terms_value(pm, a.pump_term_stride, cs, a.members, L, o)
                                       : mul_rn_i(s0, pm[o]);
#pragma unroll
          for (int cr = 0; cr < 2; ++cr) {
            if (cr >= Cr) break;
            const T rr = Cr == comps ? rho[cr] : (comps == 2 ? rho[0] + rho[1] : rho[0]);
            const T P = Cr == 2 ? mul_rn_i(p_site, k.weight[cr]) : p_site;
            if (F == 1) {
              dn_out[ridx[cr]] = P - (k.gamma_R + k.R * rr) * nval[cr];
            } else if (a.res_kind == PG_RES_QDOUBLE) {
              // quadratic_double_reservoir.py:13-14: n_R fed by kappa n_I^2.
              const T nR = nval[cr], nI = nval[Cr + cr];
              const T transfer = k.kappa * nI * nI;
              dn_out[ridx[cr]] = transfer - k.gamma_R * nR - k.R * nR * rr;
              dn_out[ridx[Cr + cr]] = P - transfer - k.gamma_I * nI;
            } else {
              const T nA = nval[cr], nI = nval[Cr + cr];
              dn_out[ridx[Cr + cr]] = P - (k.gamma_I + k.R_IA) * nI + k.R_AI * nA;
              dn_out[ridx[cr]] = k.R_IA * nI - (k.gamma_A + k.R_AI + k.R * rr) * nA;
            }
          }
        }
      } else if (a.mode == 1) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (q >= NQ) break;
          nval[q] = nval[q] > T(0) ? nval[q] : T(0);
          n_out[ridx[q]] = nval[q];
        }
#pragma unroll
        for (int comp = 0; comp < 2; ++comp) {
          if (comp >= comps) break;
          C2 w = v[comp];
          if (a.noise) {
            const T nA = F >= 1 ? nval[Cr == comps ? comp : 0] : T(0);
            const uint32_t cell[1] = {static_cast<uint32_t>(o)};
            Words4 w1[1];
            philox_cells(cell, prefix[comp], w1);
            const Words4 words = w1[0];
            WignerDraw<T>::apply(words, k.noise_a + k.noise_b * nA, w.x, w.y);
            buf[i * CC + comp * C + c] = w;
          }
          psi_new[fbase + comp * plane + o] = w;
        }
      } else {  // mode 2: error norm, v = condensate error, dsum = reservoir error
#pragma unroll
        for (int comp = 0; comp < 2; ++comp) {
          if (comp >= comps) break;
          const C2 y0 = psi_start[fbase + comp * plane + o];
          const C2 y1 = psi_new[fbase + comp * plane + o];
          const T a0 = sqrt(y0.x * y0.x + y0.y * y0.y), a1 = sqrt(y1.x * y1.x + y1.y * y1.y);
          const T scale = static_cast<T>(a.atol) + static_cast<T>(a.rtol) * (a0 > a1 ? a0 : a1);
          local += static_cast<double>(
              scaled_square(sqrt(v[comp].x * v[comp].x + v[comp].y * v[comp].y), scale));
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (q >= NQ) break;
          const T r0 = fabs(n0[ridx[q]]), r1 = fabs(n_out[ridx[q]]);
          const T rs = static_cast<T>(a.atol) + static_cast<T>(a.rtol) * (r0 > r1 ? r0 : r1);
          local += static_cast<double>(scaled_square(fabs(dsum[q]), rs));
        }
      }
    }
    __syncthreads();
  }
  if (a.mode == 2) {
    // Block reduction of the FP64 partial sums; one value per (member, panel).
    for (int off = 16; off > 0; off >>= 1) local += __shfl_down_sync(0xffffffffu, local, off);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = local;
    __syncthreads();
    if (warp == 0) {
      const int nw = (blockDim.x + 31) >> 5;
      double v = lane < nw ? red[lane] : 0.0;
      for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
      if (lane == 0) partials[member * gridDim.x + blockIdx.x] = v;
    }
    return;
  }
  if (a.forward) smem_fft<T, false, true>(buf, tws, a.log2ny, lcc, CC, 1);
  if (a.mode == 1 && !a.forward) return;
  for (int e = threadIdx.x; e < all; e += blockDim.x) {
    const int c2 = e & (CC - 1), i = e >> lcc;
    const int comp = c2 >> a.log2cols, c = c2 & (C - 1);
    d[comp * plane + static_cast<long long>(i) * a.nx + x0 + c] = buf[i * CC + c2];
  }
}

}  // namespace

template <typename T>
cudaError_t launch_ifrk_row(const T* in, T* save, T* out, const T* tables, const IfrkRowArgs& a,
                            const T* twiddle, cudaStream_t stream) {
  using C2 = typename C2T<T>::type;
  const int blocks = a.ny / a.rows;
  const size_t smem = sizeof(C2) * (static_cast<size_t>(a.nx) + static_cast<size_t>(a.rows) * a.nx * a.comps);
  ifrk_row_kernel<T><<<dim3(blocks, 1, a.members), a.threads, smem, stream>>>(
      reinterpret_cast<const C2*>(in), reinterpret_cast<C2*>(save), reinterpret_cast<C2*>(out),
      reinterpret_cast<const C2*>(tables), reinterpret_cast<const C2*>(twiddle), a);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_ifrk_col(T* psi, const T* n0, T* dn_out, T* n_out, const T* psi_start,
                            const T* psi_new, const T* pump, const T* potential, const T* twiddle,
                            const SplitConst<T>* consts, const T* scales,
                            const unsigned long long* step_base, double* partials,
                            const IfrkColArgs& a, cudaStream_t stream) {
  using C2 = typename C2T<T>::type;
  const int blocks = a.nx / a.cols;
  const size_t smem = sizeof(C2) * (static_cast<size_t>(a.ny) + static_cast<size_t>(a.cols) * a.ny * a.comps);
  ifrk_col_kernel<T><<<dim3(blocks, 1, a.members), a.threads, smem, stream>>>(
      reinterpret_cast<C2*>(psi), n0, dn_out, n_out,
      reinterpret_cast<C2*>(const_cast<T*>(psi_start)), reinterpret_cast<C2*>(const_cast<T*>(psi_new)),
      pump, potential, reinterpret_cast<const C2*>(twiddle), consts, scales, step_base, partials, a);
  return cudaGetLastError();
}

template <typename T>
cudaError_t configure_ifrk_kernels(size_t max_smem) {
  cudaError_t e = cudaFuncSetAttribute(ifrk_row_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(max_smem));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(ifrk_col_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(max_smem));
}

template cudaError_t launch_ifrk_row<float>(const float*, float*, float*, const float*,
                                            const IfrkRowArgs&, const float*, cudaStream_t);
template cudaError_t launch_ifrk_row<double>(const double*, double*, double*, const double*,
                                             const IfrkRowArgs&, const double*, cudaStream_t);
template cudaError_t launch_ifrk_col<float>(float*, const float*, float*, float*, const float*,
                                            const float*, const float*, const float*, const float*,
                                            const SplitConst<float>*, const float*,
                                            const unsigned long long*, double*, const IfrkColArgs&,
                                            cudaStream_t);
template cudaError_t launch_ifrk_col<double>(double*, const double*, double*, double*, const double*,
                                             const double*, const double*, const double*,
                                             const double*, const SplitConst<double>*,
                                             const double*, const unsigned long long*, double*,
                                             const IfrkColArgs&, cudaStream_t);
template cudaError_t configure_ifrk_kernels<float>(size_t);
template cudaError_t configure_ifrk_kernels<double>(size_t);

cudaError_t launch_spin_mode_table(float* table, const SpinorConst* consts, int nx, int ny,
                                   int members, double kx_unit, double ky_unit, cudaStream_t stream) {
  const long long plane = static_cast<long long>(nx) * ny;
  const int blocks = static_cast<int>(std::min<long long>(1024, (plane + 255) / 256));
  spin_mode_table_kernel<<<dim3(blocks, members), 256, 0, stream>>>(table, consts, nx, ny, kx_unit,
                                                                     ky_unit);
  return cudaGetLastError();
}

}  // namespace pg
