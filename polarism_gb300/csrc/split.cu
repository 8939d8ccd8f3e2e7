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
#include "split_local.cuh"

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
  if (a.halt != nullptr && __ldcg(a.halt) != 0) return;  // steady-state monitor halted the run
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
  if (a.halt != nullptr && __ldcg(a.halt) != 0) return;  // steady-state monitor halted the run
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
    const LocalStep<T> local(a, member, res, pump, potential, consts, scales, step_base);
    #pragma unroll kUnrollLocal
    for (int e = threadIdx.x; e < count; e += blockDim.x) {
      const int c = e & (C - 1), i = e >> a.log2cols;
      const long long o = static_cast<long long>(i) * a.nx + x0 + c;
      C2 v = buf[i * C + c];
      local.apply(v, o);
      buf[i * C + c] = v;
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
