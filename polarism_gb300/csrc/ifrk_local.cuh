// The per-site part of the Lawson IFRK column pass (ifrk.cu), shared by the generic pass and
// the register-resident 1024-site pass (split_fast.cu): stage reservoir values, the
// right-hand side of the stage (mode 0: psi gets its derivative, dn_j written), the step end
// (mode 1: clamped reservoir, Wigner increment, psi_new written), the embedded error norm
// (mode 2: the FP64 sum of scaled squares grows).  Math as ifrk_fft_cuda_solver.py:118-293.
#pragma once
#include "fft.cuh"
#include "ifrk_internal.h"
#include "philox.cuh"
#include "pg_internal.h"

namespace pg {

template <typename T>
__device__ __forceinline__ T scaled_square(T mag, T scale) {
  // (mag / scale)^2 with the reference's handling of a zero scale.
  if (scale > T(0)) {
    const T r = mag / scale;
    return r * r;
  }
  return mag == T(0) ? T(0) : T(INFINITY);
}

__device__ __forceinline__ float mul_rn_i(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn_i(double a, double b) { return __dmul_rn(a, b); }

template <typename T>
struct IfrkLocal {
  using C2 = typename C2T<T>::type;
  const IfrkColArgs& a;
  int member, comps;
  long long plane, fbase;
  const T* n0;
  T* dn_out;
  T* n_out;
  C2* psi_start;
  C2* psi_new;
  SplitConst<T> k;
  int L;
  const T* cs;
  T s0;
  const T* pm;
  const T* vm;
  PhiloxCellPrefix prefix[2];
  int F, Cr, NQ;
  long long qstride, fstride;

  __device__ __forceinline__ IfrkLocal(const IfrkColArgs& args, int member_, const T* n0_, T* dn_out_,
                                       T* n_out_, C2* psi_start_, C2* psi_new_, const T* pump,
                                       const T* potential, const SplitConst<T>* consts,
                                       const T* scales, const unsigned long long* step_base)
      : a(args), member(member_), comps(args.comps),
        plane(static_cast<long long>(args.nx) * args.ny),
        fbase(static_cast<long long>(member_) * args.comps * plane), n0(n0_), dn_out(dn_out_),
        n_out(n_out_), psi_start(psi_start_), psi_new(psi_new_) {
    k = consts[member];
    L = a.pump_terms > 1 ? a.pump_terms : 1;
    cs = scales ? scales + static_cast<long long>(a.scale_index * L) * a.members + member : nullptr;
    s0 = cs ? cs[0] : T(0);
    pm = pump + member * a.pump_stride;
    vm = potential ? potential + member * a.pot_stride * (a.potential == 2 ? 2 : 1) : nullptr;
    const unsigned long long step = a.noise ? step_base[0] + a.step_offset : 0ull;
    // Philox rounds that depend only on (step, stream, key), per component stream 1 + comp.
    prefix[0] = philox_cell_prefix(static_cast<uint32_t>(step), static_cast<uint32_t>(step >> 32), 1u,
                                   static_cast<uint32_t>(k.seed), static_cast<uint32_t>(k.seed >> 32));
    prefix[1] = philox_cell_prefix(static_cast<uint32_t>(step), static_cast<uint32_t>(step >> 32), 2u,
                                   static_cast<uint32_t>(k.seed), static_cast<uint32_t>(k.seed >> 32));
    F = a.res_fields;
    Cr = a.res_comps;
    NQ = F * Cr;
    qstride = static_cast<long long>(Cr) * plane;      // reservoir member stride
    fstride = static_cast<long long>(a.members) * qstride;  // field stride
  }

  // Site o (offset within the member's plane) with its field values v (both components).
  __device__ __forceinline__ void site(C2 (&v)[2], long long o, double& local) const {
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
        v[comp] = C2{g * v[comp].x + e_over * v[comp].y, g * v[comp].y - e_over * v[comp].x};
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
          v[comp] = w;
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
};

}  // namespace pg
