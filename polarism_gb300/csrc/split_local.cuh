// The split-step's local operations at one site (device code shared by the generic column
// pass in split.cu and the 1024-point register-resident column pass in split_fast.cu): the
// reservoir half steps, the exact nonlinear step and the Wigner increment, for every
// SplitOp.
#pragma once
#include "fft.cuh"
#include "philox.cuh"
#include "pg_internal.h"
#include "split_internal.h"

namespace pg {
namespace {

__device__ __forceinline__ float mul_rn_t(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn_t(double a, double b) { return __dmul_rn(a, b); }

// Midpoint RK2 reservoir half step at frozen |psi|^2 with the final clamp
// (polarism/reservoir/single_reservoir.py:100-111).
template <typename T>
__device__ __forceinline__ T reservoir_half(T n, T rho, T pump, T h, const SplitConst<T>& k) {
  const T loss = k.gamma_R + k.R * rho;
  const T k1 = pump - loss * n;
  const T mid = n + T(0.5) * h * k1;
  const T k2 = pump - loss * mid;
  const T out = n + h * k2;
  return out > T(0) ? out : T(0);
}

// Right-hand sides of the two-field reservoirs, state (active, inactive): the double
// reservoir (polarism/reservoir/double_reservoir.py:106-130) and the quadratic-double one,
// fed by kappa n_I^2 (polarism/reservoir/quadratic_double_reservoir.py:13-14).
template <typename T>
__device__ __forceinline__ void two_field_rhs(T a, T b, T rho, T pump, bool quadratic,
                                              const SplitConst<T>& k, T& da, T& db) {
  if (quadratic) {
    const T transfer = k.kappa * b * b;
    da = transfer - k.gamma_R * a - k.R * a * rho;
    db = pump - transfer - k.gamma_I * b;
  } else {
    da = k.R_IA * b - (k.gamma_A + k.R_AI + k.R * rho) * a;
    db = pump - (k.gamma_I + k.R_IA) * b + k.R_AI * a;
  }
}

// The same midpoint half step for both fields of a two-field reservoir, each clamped at 0.
template <typename T>
__device__ __forceinline__ void reservoir_half2(T& a, T& b, T rho, T pump, T h, bool quadratic,
                                                const SplitConst<T>& k) {
  T da, db;
  two_field_rhs(a, b, rho, pump, quadratic, k, da, db);
  T da2, db2;
  two_field_rhs(a + T(0.5) * h * da, b + T(0.5) * h * db, rho, pump, quadratic, k, da2, db2);
  const T na = a + h * da2, nb = b + h * db2;
  a = na > T(0) ? na : T(0);
  b = nb > T(0) ? nb : T(0);
}

// (exp(x) - 1) / x, exp(x) - 1 and (sin, cos - 1) of the local step.  FP64 follows the
// reference (expm1 with its three-term series below 1e-6, library sincos).  FP32 uses
// five-term series for |x| < 2^-5 (truncation x^5/720 < 5e-11 relative) and Taylor
// polynomials for |phi| < 1/8 (truncation below 1e-13), the library functions outside: the
// per-step arguments are that small at the time steps the split-step solvers run with, and
// the polynomials are cheaper than the library's range reduction.
__device__ __forceinline__ double phase_time_factor(double x) {
  return fabs(x) < 1e-6 ? 1.0 + x * 0.5 + x * x / 6.0 : expm1(x) / x;
}
__device__ __forceinline__ float phase_time_factor(float x) {
  if (fabsf(x) < 0.03125f)
    return 1.0f + x * (0.5f + x * (1.0f / 6.0f + x * (1.0f / 24.0f + x * (1.0f / 120.0f))));
  return expm1f(x) / x;
}
__device__ __forceinline__ double local_expm1(double x) { return expm1(x); }
__device__ __forceinline__ float local_expm1(float x) {
  if (fabsf(x) < 0.03125f)
    return x * (1.0f + x * (0.5f + x * (1.0f / 6.0f + x * (1.0f / 24.0f + x * (1.0f / 120.0f)))));
  return expm1f(x);
}
__device__ __forceinline__ void local_sincos_m1(double x, double* s, double* cm1) {
  double c;
  sincos(x, s, &c);
  *cm1 = c - 1.0;
}
__device__ __forceinline__ void local_sincos_m1(float x, float* s, float* cm1) {
  if (fabsf(x) < 0.125f) {
    const float x2 = x * x;
    *s = x * (1.0f - x2 * (1.0f / 6.0f) * (1.0f - x2 * (1.0f / 20.0f) * (1.0f - x2 * (1.0f / 42.0f))));
    *cm1 = -x2 * 0.5f * (1.0f - x2 * (1.0f / 12.0f) * (1.0f - x2 * (1.0f / 30.0f) * (1.0f - x2 * (1.0f / 56.0f))));
  } else {
    float c;
    sincosf(x, s, &c);
    *cm1 = c - 1.0f;  // |phi| >= 1/8: |c - 1| >= 0.0078, so c - 1 keeps c's precision
  }
}

// Exact local step psi * exp(g dt - i phi) (split_step_fft_solver.py:121-139); n2 is the
// inactive reservoir (0 without one), which enters the phase through g_I.  Applied as
// psi + psi D with D = exp(g dt - i phi) - 1 = (e + c1 + e c1) - i (1 + e) s, e = exp(g dt) - 1,
// c1 = cos phi - 1: the factor itself sits next to 1 at these step sizes, where its rounding
// would repeat step after step (a rounded exp(g dt) there carries up to 6e-8 of bias a step).
template <typename T>
__device__ __forceinline__ void nonlinear(T& re, T& im, T n, T n2, bool two, T vre, T vim, T dt,
                                          const SplitConst<T>& k) {
  const T rho = re * re + im * im;
  const T gain = (k.R * n - k.gamma_C) * T(0.5) + vim * k.inv_hbar;
  const T x = T(2) * gain * dt;
  const T phase_time = dt * phase_time_factor(x);
  T pot = vre + k.g_R * n;
  if (two) pot += k.g_I * n2;
  const T phase = (pot * dt + k.g_C * rho * phase_time) * k.inv_hbar;
  const T e = local_expm1(gain * dt);
  T s, c1;
  local_sincos_m1(phase, &s, &c1);
  const T dre = e + c1 + e * c1;
  const T dim = -(s + e * s);
  const T r = re, i = im;
  re = r + (r * dre - i * dim);
  im = i + (r * dim + i * dre);
}


// Everything the local step of one column-pass launch needs for a member, and the step at
// one site (flat index o within the member's plane).
template <typename T>
struct LocalStep {
  using C2 = typename C2T<T>::type;
  SplitConst<T> k;
  // The launch's settings, copied (a pointer to the kernel's parameter would move it to local
  // memory and make every read a local load).
  int op, reservoir, noise, pot_kind;
  long long pump_term_stride;
  int m_count, L;
  const T* c0;
  const T* c1;
  T s0, s1;
  const T* pm;
  const T* vm;
  T* rm;
  T* rm2;
  bool two, quadratic;
  T dt, h;
  PhiloxCellPrefix prefix;

  __device__ __forceinline__ LocalStep(const ColPassArgs& args, int member, T* res, const T* pump,
                                       const T* potential, const SplitConst<T>* consts,
                                       const T* scales, const unsigned long long* step_base) {
    op = args.op;
    reservoir = args.reservoir;
    noise = args.noise;
    pot_kind = args.potential;
    pump_term_stride = args.pump_term_stride;
    k = consts[member];
    m_count = args.members;
    // Coefficients [k][sample][term][member]; the term axis exists only with several lasers.
    L = args.pump_terms > 1 ? args.pump_terms : 1;
    c0 = scales + static_cast<long long>((args.scale_offset + 0) * L) * m_count + member;
    c1 = scales + static_cast<long long>((args.scale_offset + 1) * L) * m_count + member;
    s0 = c0[0];
    s1 = c1[0];
    const long long plane = static_cast<long long>(args.nx) * args.ny;
    pm = pump + member * args.pump_stride;
    vm = potential ? potential + member * args.pot_stride * (args.potential == 2 ? 2 : 1) : nullptr;
    rm = res + member * plane;
    // Second reservoir field (inactive) one field after the first: [field][member][y][x].
    two = args.res_kind >= 2;
    quadratic = args.res_kind == 3;
    rm2 = two ? rm + static_cast<long long>(args.members) * plane : nullptr;
    dt = args.template dt_of<T>();
    h = dt * T(0.5);
    const unsigned long long step = args.noise ? step_base[0] + args.step_offset : 0ull;
    // Philox rounds that depend only on (step, stream, key), formed once per launch and member.
    prefix = philox_cell_prefix(static_cast<uint32_t>(step), static_cast<uint32_t>(step >> 32), 1u,
                                static_cast<uint32_t>(k.seed), static_cast<uint32_t>(k.seed >> 32));
  }

  // One reservoir half step at the given pump value on the chosen reservoir model.
  __device__ __forceinline__ void res_half(T& n, T& n2, T rho, T pump_value) const {
    if (two) {
      reservoir_half2(n, n2, rho, pump_value, h, quadratic, k);
    } else if (reservoir) {
      n = reservoir_half(n, rho, pump_value, h, k);
    }
  }

  // Whether step_single covers this launch: one reservoir field, one laser and no potential
  // (the common case, without the general code's branches).
  __device__ __forceinline__ bool single() const {
    return reservoir && !two && L == 1 && vm == nullptr;
  }

  // apply() for that case with the operation known at compile time, on values already
  // loaded: the reservoir n and the envelope P at site o (32-bit site offsets: a member holds
  // fewer than 2^31 sites).  The same operations, in the same order; returns the new n, which
  // the caller stores unless OP is SPLIT_OP_NONLINEAR.
  template <int OP, bool NOISE>
  __device__ __forceinline__ T step_single(C2& v, T n, T P, int o) const {
    if (OP == SPLIT_OP_KOUTER) {
      n = reservoir_half(n, v.x * v.x + v.y * v.y, mul_rn_t(s0, P), h, k);
      nonlinear(v.x, v.y, n, T(0), false, T(0), T(0), dt, k);
      n = reservoir_half(n, v.x * v.x + v.y * v.y, mul_rn_t(s1, P), h, k);
    } else if (OP == SPLIT_OP_RES_START || OP == SPLIT_OP_RES_END) {
      n = reservoir_half(n, v.x * v.x + v.y * v.y, mul_rn_t(s0, P), h, k);
    } else if (OP == SPLIT_OP_RES_END_START) {
      const T rho = v.x * v.x + v.y * v.y;
      n = reservoir_half(n, rho, mul_rn_t(s0, P), h, k);
      n = reservoir_half(n, rho, mul_rn_t(s1, P), h, k);
    } else if (OP == SPLIT_OP_NONLINEAR) {
      nonlinear(v.x, v.y, n, T(0), false, T(0), T(0), dt, k);
    }
    if (NOISE && (OP == SPLIT_OP_KOUTER || OP == SPLIT_OP_NONLINEAR)) {
      const uint32_t cell[1] = {static_cast<uint32_t>(o)};
      Words4 w[1];
      philox_cells(cell, prefix, w);
      WignerDraw<T>::apply(w[0], k.noise_a + k.noise_b * n, v.x, v.y);
    }
    return n;
  }

  __device__ __forceinline__ void apply(C2& v, long long o) const {
    T n = (reservoir || two) ? rm[o] : T(0);
    T n2 = two ? rm2[o] : T(0);
    T Pa, Pb;  // pump at the first and the second coefficient sample
    if (L > 1) {
      Pa = pump_terms_value(pm, pump_term_stride, c0, m_count, L, o);
      Pb = pump_terms_value(pm, pump_term_stride, c1, m_count, L, o);
    } else {
      const T P = pm[o];
      Pa = mul_rn_t(s0, P);
      Pb = mul_rn_t(s1, P);
    }
    T vre = T(0), vim = T(0);
    if (vm) {
      vre = pot_kind == 2 ? vm[2 * o] : vm[o];
      vim = pot_kind == 2 ? vm[2 * o + 1] : T(0);
    }
    bool add_noise = false;
    switch (op) {
      case SPLIT_OP_KOUTER:
        res_half(n, n2, v.x * v.x + v.y * v.y, Pa);
        nonlinear(v.x, v.y, n, n2, two, vre, vim, dt, k);
        res_half(n, n2, v.x * v.x + v.y * v.y, Pb);
        add_noise = noise != 0;
        break;
      case SPLIT_OP_RES_START:
        res_half(n, n2, v.x * v.x + v.y * v.y, Pa);
        break;
      case SPLIT_OP_RES_END_START: {
        const T rho = v.x * v.x + v.y * v.y;
        res_half(n, n2, rho, Pa);
        res_half(n, n2, rho, Pb);
        break;
      }
      case SPLIT_OP_NONLINEAR:
        nonlinear(v.x, v.y, n, n2, two, vre, vim, dt, k);
        add_noise = noise != 0;
        break;
      case SPLIT_OP_RES_END:
        res_half(n, n2, v.x * v.x + v.y * v.y, Pa);
        break;
      default:
        break;
    }
    if (add_noise) {
      const uint32_t cell[1] = {static_cast<uint32_t>(o)};
      Words4 w[1];
      philox_cells(cell, prefix, w);
      WignerDraw<T>::apply(w[0], k.noise_a + k.noise_b * n, v.x, v.y);
    }
    if (reservoir || two) rm[o] = n;
    if (two) rm2[o] = n2;
  }
};

}  // namespace
}  // namespace pg
