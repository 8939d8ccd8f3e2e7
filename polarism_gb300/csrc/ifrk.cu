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
#include "fft.cuh"
#include "ifrk_internal.h"
#include "philox.cuh"
#include "pg_internal.h"

namespace pg {
namespace {

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
  C2* buf = tws + a.nx;
  const int member = blockIdx.z;
  const int row0 = blockIdx.x * a.rows;
  const int count = a.rows * a.nx;
  const long long moff = member * a.member_stride + static_cast<long long>(row0) * a.nx;
  for (int k = threadIdx.x; k < a.nx; k += blockDim.x) tws[k] = tw[k];
  if (in) {
    for (int e = threadIdx.x; e < count; e += blockDim.x) buf[e] = in[moff + e];
  }
  __syncthreads();
  if (a.forward) smem_fft<T, false, false>(buf, tws, a.log2nx, a.log2rows, 1, a.nx);
  if (save) {
    for (int e = threadIdx.x; e < count; e += blockDim.x) save[moff + e] = buf[e];
  }
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
  __syncthreads();
  if (a.inverse) smem_fft<T, true, false>(buf, tws, a.log2nx, a.log2rows, 1, a.nx);
  for (int e = threadIdx.x; e < count; e += blockDim.x) out[moff + e] = buf[e];
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

__device__ __forceinline__ float mul_rn_i(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn_i(double a, double b) { return __dmul_rn(a, b); }

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
  C2* buf = tws + a.ny;
  __shared__ double red[32];
  const int member = blockIdx.z;
  const int x0 = blockIdx.x * a.cols;
  const int C = a.cols;
  const long long plane = static_cast<long long>(a.nx) * a.ny;
  C2* d = psi + member * plane;
  for (int k = threadIdx.x; k < a.ny; k += blockDim.x) tws[k] = tw[k];
  const int count = C * a.ny;
  for (int e = threadIdx.x; e < count; e += blockDim.x) {
    const int c = e & (C - 1), i = e >> a.log2cols;
    buf[i * C + c] = d[static_cast<long long>(i) * a.nx + x0 + c];
  }
  __syncthreads();
  if (a.inverse) smem_fft<T, true, true>(buf, tws, a.log2ny, a.log2cols, a.cols, 1);
  double local = 0.0;
  if (a.mode != 3) {
    const SplitConst<T> k = consts[member];
    const T s0 = scales ? scales[a.scale_index * a.members + member] : T(0);
    const T* pm = pump + member * a.pump_stride;
    const T* vm = potential ? potential + member * a.pot_stride * (a.potential == 2 ? 2 : 1) : nullptr;
    const unsigned long long step = a.noise ? step_base[0] + a.step_offset : 0ull;
    for (int e = threadIdx.x; e < count; e += blockDim.x) {
      const int c = e & (C - 1), i = e >> a.log2cols;
      const long long o = static_cast<long long>(i) * a.nx + x0 + c;
      const long long mo = member * plane + o;
      C2 v = buf[i * C + c];
      // Stage (or final) reservoir: n0 + sum coef_j dn_j (the sum alone is the error term).
      T n = T(0), dsum = T(0);
      if (a.reservoir) {
#pragma unroll
        for (int j = 0; j < kIfrkMaxStages; ++j) {
          if (j >= a.terms) break;
          dsum += static_cast<T>(a.coef[j]) * static_cast<const T*>(a.dn[j])[mo];
        }
        n = n0[mo] + dsum;
      }
      if (a.mode == 0) {
        if (psi_start) psi_start[mo] = v;
        const T rho = v.x * v.x + v.y * v.y;
        T vre = T(0), vim = T(0);
        if (vm) {
          vre = a.potential == 2 ? vm[2 * o] : vm[o];
          vim = a.potential == 2 ? vm[2 * o + 1] : T(0);
        }
        // rhs = (-i/hbar) (V_re + g_C rho + g_R n) psi + (R n - gamma_C)/2 psi + (V_im/hbar) psi
        const T e_over = (vre + k.g_C * rho + k.g_R * n) * k.inv_hbar;
        const T g = T(0.5) * (k.R * n - k.gamma_C) + vim * k.inv_hbar;
        buf[i * C + c] = C2{g * v.x + e_over * v.y, g * v.y - e_over * v.x};
        if (a.reservoir) dn_out[mo] = mul_rn_i(s0, pm[o]) - (k.gamma_R + k.R * rho) * n;
      } else if (a.mode == 1) {
        n = n > T(0) ? n : T(0);
        if (a.reservoir) n_out[mo] = n;
        if (a.noise) {
          const Words4 w = wigner_words(static_cast<uint32_t>(o), step, 1u, k.seed);
          WignerDraw<T>::apply(w, k.noise_a + k.noise_b * n, v.x, v.y);
          buf[i * C + c] = v;
        }
        psi_new[mo] = v;
      } else {  // mode 2: error norm, v = condensate error, n = reservoir error
        const C2 y0 = psi_start[mo];
        const C2 y1 = psi_new[mo];
        const T a0 = sqrt(y0.x * y0.x + y0.y * y0.y), a1 = sqrt(y1.x * y1.x + y1.y * y1.y);
        const T scale = static_cast<T>(a.atol) + static_cast<T>(a.rtol) * (a0 > a1 ? a0 : a1);
        local += static_cast<double>(scaled_square(sqrt(v.x * v.x + v.y * v.y), scale));
        if (a.reservoir) {
          const T en = dsum;  // h sum_j (b_j - bhat_j) dn_j
          const T r0 = fabs(n0[mo]), r1 = fabs(n_out[mo]);
          const T rs = static_cast<T>(a.atol) + static_cast<T>(a.rtol) * (r0 > r1 ? r0 : r1);
          local += static_cast<double>(scaled_square(fabs(en), rs));
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
  if (a.forward) smem_fft<T, false, true>(buf, tws, a.log2ny, a.log2cols, a.cols, 1);
  if (a.mode == 1 && !a.forward) return;
  for (int e = threadIdx.x; e < count; e += blockDim.x) {
    const int c = e & (C - 1), i = e >> a.log2cols;
    d[static_cast<long long>(i) * a.nx + x0 + c] = buf[i * C + c];
  }
}

}  // namespace

template <typename T>
cudaError_t launch_ifrk_row(const T* in, T* save, T* out, const T* tables, const IfrkRowArgs& a,
                            const T* twiddle, cudaStream_t stream) {
  using C2 = typename C2T<T>::type;
  const int blocks = a.ny / a.rows;
  const size_t smem = sizeof(C2) * (static_cast<size_t>(a.nx) + static_cast<size_t>(a.rows) * a.nx);
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
  const size_t smem = sizeof(C2) * (static_cast<size_t>(a.ny) + static_cast<size_t>(a.cols) * a.ny);
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

}  // namespace pg
