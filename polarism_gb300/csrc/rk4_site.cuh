// FP32 site arithmetic shared by the full-width RK4 kernel and the uneven-size sweep
// kernel: the right-hand side of polarism/model.py:89-127 with the single reservoir of
// polarism/reservoir/single_reservoir.py:81-98 at one site, on packed FP32x2 values.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "pg_internal.h"

namespace pg {

struct Pair {
  float2 a, b;  // complex values of the thread's two columns
};

struct WideConst {
  float2 nax, nay;      // (-ax, -ax), (-ay, -ay)
  float w0, gc, gr, half_R, half_gC, R, gamma_R, noise_a, noise_b;
  float inv_hbar, eta;  // potential scale and kinetic relaxation (general variant)
  uint64_t seed;
};

__device__ __forceinline__ WideConst wide_const(const RhsConst<float>& kk) {
  WideConst k;
  k.nax = make_float2(-kk.ax, -kk.ax);
  k.nay = make_float2(-kk.ay, -kk.ay);
  k.w0 = kk.w0;
  k.gc = kk.gc;
  k.gr = kk.gr;
  k.half_R = kk.half_R;
  k.half_gC = kk.half_gC;
  k.R = kk.R;
  k.gamma_R = kk.gamma_R;
  k.noise_a = kk.noise_a;
  k.noise_b = kk.noise_b;
  k.inv_hbar = kk.inv_hbar;
  k.eta = kk.eta_a;
  k.seed = kk.seed;
  return k;
}

// Right-hand side at one site: c centre, (lt, rt, up, dn) neighbours.  Writes
// d = dpsi/dt and returns dn/dt.
__device__ __forceinline__ float site_rhs(float2 c, float2 lt, float2 rt, float2 up, float2 dn,
                                          float n, float sP, const WideConst& k, float2& d) {
  const float2 sx = __fadd2_rn(lt, rt);
  const float2 sy = __fadd2_rn(up, dn);
  const float2 nl = __ffma2_rn(k.nay, sy, __fmul2_rn(k.nax, sx));  // -a (lap without centre)
  const float rho = fmaf(c.x, c.x, c.y * c.y);
  const float w = fmaf(k.gr, n, fmaf(k.gc, rho, k.w0));
  const float gl = fmaf(k.half_R, n, -k.half_gC);
  const float2 u = __ffma2_rn(make_float2(w, w), c, nl);  // w c - a lap_neighbours
  d.x = fmaf(gl, c.x, u.y);
  d.y = fmaf(gl, c.y, -u.x);
  return fmaf(-fmaf(k.R, rho, k.gamma_R), n, sP);
}

// site_rhs with a potential V = vre + i vim (polarism/model.py:89-127: -i V psi / hbar) and,
// when relax, the kinetic-relaxation term + eta n_A (hbar / 2m) Laplacian psi of the general
// right-hand side; the Laplacian with its centre weight is -(w0 c + nl).
__device__ __forceinline__ float site_rhs_general(float2 c, float2 lt, float2 rt, float2 up,
                                                  float2 dn, float n, float sP, const WideConst& k,
                                                  float vre, float vim, bool relax, float2& d) {
  const float2 sx = __fadd2_rn(lt, rt);
  const float2 sy = __fadd2_rn(up, dn);
  const float2 nl = __ffma2_rn(k.nay, sy, __fmul2_rn(k.nax, sx));
  const float rho = fmaf(c.x, c.x, c.y * c.y);
  const float w = fmaf(vre, k.inv_hbar, fmaf(k.gr, n, fmaf(k.gc, rho, k.w0)));
  const float gl = fmaf(vim, k.inv_hbar, fmaf(k.half_R, n, -k.half_gC));
  const float2 u = __ffma2_rn(make_float2(w, w), c, nl);
  d.x = fmaf(gl, c.x, u.y);
  d.y = fmaf(gl, c.y, -u.x);
  if (relax) {
    const float en = k.eta * n;
    const float2 t = __ffma2_rn(make_float2(k.w0, k.w0), c, nl);
    d.x = fmaf(-en, t.x, d.x);
    d.y = fmaf(-en, t.y, d.y);
  }
  return fmaf(-fmaf(k.R, rho, k.gamma_R), n, sP);
}

__device__ __forceinline__ float2 axpy2(float h, float2 d, float2 y) {
  return __ffma2_rn(make_float2(h, h), d, y);
}

// site_rhs at two adjacent sites a (left) and b (right) of one row: L is a's left neighbour,
// R is b's right neighbour.  The per-site scalars (nonlinear frequency, gain, reservoir
// derivative) of the two sites run as packed FP32x2 instructions, each lane the same FP32
// operation with the same rounding as site_rhs, so the results are bitwise those of two
// site_rhs calls.  n2 and sp2 hold (a, b) reservoir values and pump products; returns the
// (a, b) reservoir derivatives.
__device__ __forceinline__ float2 pair_rhs(float2 ca, float2 cb, float2 L, float2 R, float2 upa,
                                           float2 upb, float2 dna, float2 dnb, float2 n2,
                                           float2 sp2, const WideConst& k, float2& da, float2& db) {
  const float2 nla = __ffma2_rn(k.nay, __fadd2_rn(upa, dna), __fmul2_rn(k.nax, __fadd2_rn(L, cb)));
  const float2 nlb = __ffma2_rn(k.nay, __fadd2_rn(upb, dnb), __fmul2_rn(k.nax, __fadd2_rn(ca, R)));
  const float2 rho = make_float2(fmaf(ca.x, ca.x, ca.y * ca.y), fmaf(cb.x, cb.x, cb.y * cb.y));
  const float2 w = __ffma2_rn(make_float2(k.gr, k.gr), n2,
                              __ffma2_rn(make_float2(k.gc, k.gc), rho, make_float2(k.w0, k.w0)));
  const float2 gl = __ffma2_rn(make_float2(k.half_R, k.half_R), n2,
                               make_float2(-k.half_gC, -k.half_gC));
  const float2 ua = __ffma2_rn(make_float2(w.x, w.x), ca, nla);
  const float2 ub = __ffma2_rn(make_float2(w.y, w.y), cb, nlb);
  da.x = fmaf(gl.x, ca.x, ua.y);
  da.y = fmaf(gl.x, ca.y, -ua.x);
  db.x = fmaf(gl.y, cb.x, ub.y);
  db.y = fmaf(gl.y, cb.y, -ub.x);
  // -(R rho + gamma_R) n + sP with the negation folded into the constants (exact).
  return __ffma2_rn(__ffma2_rn(make_float2(-k.R, -k.R), rho, make_float2(-k.gamma_R, -k.gamma_R)),
                    n2, sp2);
}

}  // namespace pg
