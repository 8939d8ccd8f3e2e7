// Split-step Fourier stepping: hand-written shared-memory Stockham FFT passes with
// the kinetic propagator and the local (reservoir / nonlinear / Wigner) step fused in.
//
// A 2-D transform is split into a row pass (FFT along x of C contiguous rows) and a
// column pass (FFT along y of a panel of C adjacent columns).  Both run in place on
// the state array, each block owning disjoint rows / panels.
//
//   row pass:    [F_x] -> x (px[j] py[i])  -> [F_x^-1]        (propagator is separable:
//                 exp(-i hbar (kx^2+ky^2) tau / 2m) = exp(-i c kx^2) exp(-i c ky^2))
//   column pass: [F_y^-1] -> local op at each site -> [F_y]
//
// Orderings built from these passes (polarism/solver/split_step_fft_cuda_solver.py:
// 106-184,1144-1325 for K(dt/2)[R(dt/2) N(dt) R(dt/2)]K(dt/2) with the spectrum kept
// between steps; polarism/solver/split_step_fft_solver.py:97-159 for
// R/2 K/2 N K/2 R/2) are sequenced by the host in api_split.cu.
//
// The Stockham passes follow the autosort recurrence
//   y[q + s (R p + r)] = w_N^{p r s} * sum_t x[q + s (p + m t)] w_R^{r t}
// with radix 4 (plus one radix-2 pass when log2 N is odd), executed in place with the
// inputs of every butterfly staged in registers between two barriers.
#include "philox.cuh"
#include "pg_internal.h"
#include "split_internal.h"
#include "fft.cuh"

namespace pg {
namespace {

// Element loops are unrolled so several global loads are in flight per thread.
constexpr int kUnrollIO = 4;
constexpr int kUnrollLocal = 2;

// ------------------------------------------------------------------ row pass
template <typename T>
__global__ void __launch_bounds__(1024) row_pass_kernel(typename C2T<T>::type* __restrict__ data,
                                                        const typename C2T<T>::type* __restrict__ tw,
                                                        const typename C2T<T>::type* __restrict__ px,
                                                        const typename C2T<T>::type* __restrict__ py,
                                                        const RowPassArgs a) {
  using C2 = typename C2T<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr bool COMP = sizeof(T) == 4;  // FP32: twiddles as rounded value + remainder
  C2* tws = reinterpret_cast<C2*>(smem_raw);
  C2* buf = tws + (COMP ? 2 : 1) * a.nx;
  const int member = blockIdx.z;
  const int row0 = blockIdx.x * a.rows;
  const int rows = a.rows;
  const long long plane = static_cast<long long>(a.nx) * a.ny;
  C2* d = data + member * plane + static_cast<long long>(row0) * a.nx;
  for (int k = threadIdx.x; k < (COMP ? 2 : 1) * a.nx; k += blockDim.x) tws[k] = tw[k];
  const int count = rows * a.nx;
  #pragma unroll kUnrollIO
  for (int e = threadIdx.x; e < count; e += blockDim.x) buf[e] = d[e];
  __syncthreads();
  if (a.forward) smem_fft<T, false, false, COMP>(buf, tws, a.log2nx, a.log2rows, 1, a.nx);
  if (a.multiply) {
    // psi (1 + dx[j]) (1 + dy[i]) scale = (psi + psi (dx + dy + dx dy)) scale, with the factor
    // differences d stored in place of the factors (see setup_tables) and scale a power of two.
    const C2* pxm = px + static_cast<long long>(member) * a.table_stride;
    const C2* pym = py + static_cast<long long>(member) * a.table_stride;
    const T scale = static_cast<T>(a.scale);
    for (int e = threadIdx.x; e < count; e += blockDim.x) {
      const int r = e >> a.log2nx;
      const int j = e & (a.nx - 1);
      const C2 dx = pxm[j], dy = pym[row0 + r];
      const C2 dxy = cmul(dx, dy);
      const C2 f1{dx.x + dy.x + dxy.x, dx.y + dy.y + dxy.y};
      const C2 v = buf[e];
      const C2 vf = cmul(v, f1);
      buf[e] = C2{(v.x + vf.x) * scale, (v.y + vf.y) * scale};
    }
    __syncthreads();
  }
  if (a.inverse) smem_fft<T, true, false, COMP>(buf, tws, a.log2nx, a.log2rows, 1, a.nx);
  #pragma unroll kUnrollIO
  for (int e = threadIdx.x; e < count; e += blockDim.x) d[e] = buf[e];
}

// ------------------------------------------------------------------ local operations
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

// ------------------------------------------------------------------ column pass
template <typename T>
__global__ void __launch_bounds__(1024) col_pass_kernel(typename C2T<T>::type* __restrict__ data,
                                                        T* __restrict__ res,
                                                        const T* __restrict__ pump,
                                                        const T* __restrict__ potential,
                                                        const typename C2T<T>::type* __restrict__ tw,
                                                        const SplitConst<T>* __restrict__ consts,
                                                        const T* __restrict__ scales,
                                                        const unsigned long long* __restrict__ step_base,
                                                        const ColPassArgs a) {
  using C2 = typename C2T<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr bool COMP = sizeof(T) == 4;  // FP32: twiddles as rounded value + remainder
  C2* tws = reinterpret_cast<C2*>(smem_raw);
  C2* buf = tws + (COMP ? 2 : 1) * a.ny;
  const int member = blockIdx.z;
  const int x0 = blockIdx.x * a.cols;
  const int C = a.cols;
  const long long plane = static_cast<long long>(a.nx) * a.ny;
  C2* d = data + member * plane;
  for (int k = threadIdx.x; k < (COMP ? 2 : 1) * a.ny; k += blockDim.x) tws[k] = tw[k];
  const int count = C * a.ny;
  #pragma unroll kUnrollIO
  for (int e = threadIdx.x; e < count; e += blockDim.x) {
    const int c = e & (C - 1), i = e >> a.log2cols;
    buf[i * C + c] = d[static_cast<long long>(i) * a.nx + x0 + c];
  }
  __syncthreads();
  if (a.inverse) smem_fft<T, true, true, COMP>(buf, tws, a.log2ny, a.log2cols, a.cols, 1);
  if (a.op != SPLIT_OP_NONE) {
    const SplitConst<T> k = consts[member];
    const int m_count = a.members;
    // Coefficients [k][sample][term][member]; the term axis exists only with several lasers.
    const int L = a.pump_terms > 1 ? a.pump_terms : 1;
    const T* c0 = scales + static_cast<long long>((a.scale_offset + 0) * L) * m_count + member;
    const T* c1 = scales + static_cast<long long>((a.scale_offset + 1) * L) * m_count + member;
    const T s0 = c0[0], s1 = c1[0];
    const T* pm = pump + member * a.pump_stride;
    const T* vm = potential ? potential + member * a.pot_stride * (a.potential == 2 ? 2 : 1) : nullptr;
    T* rm = res + member * plane;
    // Second reservoir field (inactive) one field after the first: [field][member][y][x].
    const bool two = a.res_kind >= 2;
    const bool quadratic = a.res_kind == 3;
    T* rm2 = two ? rm + static_cast<long long>(a.members) * plane : nullptr;
    const T dt = a.template dt_of<T>();
    const T h = dt * T(0.5);
    const unsigned long long step = a.noise ? step_base[0] + a.step_offset : 0ull;
    // Philox rounds that depend only on (step, stream, key), formed once for the block.
    const PhiloxCellPrefix prefix =
        philox_cell_prefix(static_cast<uint32_t>(step), static_cast<uint32_t>(step >> 32), 1u,
                           static_cast<uint32_t>(k.seed), static_cast<uint32_t>(k.seed >> 32));
    // One reservoir half step at the given pump coefficient on the chosen model.
    auto res_half = [&](T& n, T& n2, T rho, T pump_value) {
      if (two) {
        reservoir_half2(n, n2, rho, pump_value, h, quadratic, k);
      } else if (a.reservoir) {
        n = reservoir_half(n, rho, pump_value, h, k);
      }
    };
    #pragma unroll kUnrollLocal
    for (int e = threadIdx.x; e < count; e += blockDim.x) {
      const int c = e & (C - 1), i = e >> a.log2cols;
      const long long o = static_cast<long long>(i) * a.nx + x0 + c;
      C2 v = buf[i * C + c];
      T n = (a.reservoir || two) ? rm[o] : T(0);
      T n2 = two ? rm2[o] : T(0);
      T Pa, Pb;  // pump at the first and the second coefficient sample
      if (L > 1) {
        Pa = pump_terms_value(pm, a.pump_term_stride, c0, m_count, L, o);
        Pb = pump_terms_value(pm, a.pump_term_stride, c1, m_count, L, o);
      } else {
        const T P = pm[o];
        Pa = mul_rn_t(s0, P);
        Pb = mul_rn_t(s1, P);
      }
      T vre = T(0), vim = T(0);
      if (vm) {
        vre = a.potential == 2 ? vm[2 * o] : vm[o];
        vim = a.potential == 2 ? vm[2 * o + 1] : T(0);
      }
      bool add_noise = false;
      switch (a.op) {
        case SPLIT_OP_KOUTER:
          res_half(n, n2, v.x * v.x + v.y * v.y, Pa);
          nonlinear(v.x, v.y, n, n2, two, vre, vim, dt, k);
          res_half(n, n2, v.x * v.x + v.y * v.y, Pb);
          add_noise = a.noise != 0;
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
          add_noise = a.noise != 0;
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
      buf[i * C + c] = v;
      if (a.reservoir || two) rm[o] = n;
      if (two) rm2[o] = n2;
    }
    __syncthreads();
  }
  if (a.forward) smem_fft<T, false, true, COMP>(buf, tws, a.log2ny, a.log2cols, a.cols, 1);
  #pragma unroll kUnrollIO
  for (int e = threadIdx.x; e < count; e += blockDim.x) {
    const int c = e & (C - 1), i = e >> a.log2cols;
    d[static_cast<long long>(i) * a.nx + x0 + c] = buf[i * C + c];
  }
}

}  // namespace

template <typename T>
cudaError_t launch_row_pass(T* data, const T* tw, const T* px, const T* py, const RowPassArgs& a,
                            int members, cudaStream_t stream) {
  using C2 = typename C2T<T>::type;
  const int blocks = (a.ny + a.rows - 1) / a.rows;
  const size_t tw_values = static_cast<size_t>(a.nx) * (sizeof(T) == 4 ? 2 : 1);
  const size_t smem = sizeof(C2) * (tw_values + static_cast<size_t>(a.rows) * a.nx);
  row_pass_kernel<T><<<dim3(blocks, 1, members), a.threads, smem, stream>>>(
      reinterpret_cast<C2*>(data), reinterpret_cast<const C2*>(tw), reinterpret_cast<const C2*>(px),
      reinterpret_cast<const C2*>(py), a);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_col_pass(T* data, T* res, const T* pump, const T* potential, const T* tw,
                            const SplitConst<T>* consts, const T* scales,
                            const unsigned long long* step_base, const ColPassArgs& a,
                            cudaStream_t stream) {
  using C2 = typename C2T<T>::type;
  const int blocks = (a.nx + a.cols - 1) / a.cols;
  const size_t tw_values = static_cast<size_t>(a.ny) * (sizeof(T) == 4 ? 2 : 1);
  const size_t smem = sizeof(C2) * (tw_values + static_cast<size_t>(a.cols) * a.ny);
  col_pass_kernel<T><<<dim3(blocks, 1, a.members), a.threads, smem, stream>>>(
      reinterpret_cast<C2*>(data), res, pump, potential, reinterpret_cast<const C2*>(tw), consts,
      scales, step_base, a);
  return cudaGetLastError();
}

template <typename T>
cudaError_t configure_split_kernels(size_t max_smem) {
  cudaError_t e = cudaFuncSetAttribute(row_pass_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(max_smem));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(col_pass_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(max_smem));
}

template cudaError_t launch_row_pass<float>(float*, const float*, const float*, const float*,
                                            const RowPassArgs&, int, cudaStream_t);
template cudaError_t launch_row_pass<double>(double*, const double*, const double*, const double*,
                                             const RowPassArgs&, int, cudaStream_t);
template cudaError_t launch_col_pass<float>(float*, float*, const float*, const float*, const float*,
                                            const SplitConst<float>*, const float*,
                                            const unsigned long long*, const ColPassArgs&,
                                            cudaStream_t);
template cudaError_t launch_col_pass<double>(double*, double*, const double*, const double*,
                                             const double*, const SplitConst<double>*, const double*,
                                             const unsigned long long*, const ColPassArgs&,
                                             cudaStream_t);
int split_max_vals(bool is_double) { return is_double ? MaxVals<double>::value : MaxVals<float>::value; }

template cudaError_t configure_split_kernels<float>(size_t);
template cudaError_t configure_split_kernels<double>(size_t);

}  // namespace pg
