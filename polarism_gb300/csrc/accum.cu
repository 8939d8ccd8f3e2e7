// FP64 observables of the device-resident state.
//
// * Density moments sum |psi|^2 and sum |psi|^4 per site (polarism/results/accumulators.py:
//   134-172, G2Accumulator.update), accumulated in FP64 from the working precision.
// * Momentum distribution sum |FFT2 psi|^2 per mode (accumulators.py:95-131,
//   MomentumDistribution.update): one column pass (F_y) into a scratch spectrum and one row
//   pass (F_x) whose epilogue squares and accumulates in FP64.
// * Per-member norm sum |psi|^2 dV (polarism/simulation_controller.py:92-103) and the
//   steady-state comparison of simulation_controller.py:710-734 (relative density and norm
//   changes against the previous check), reduced in FP64 through per-block partial sums.
// * The device-resident steady-state monitor (pg_steady_update / _poll / _results): the
//   partial sums here, then the decision of steady_monitor.cu (comparison, per-member stop
//   decision and first stop step of simulation_controller.py:698-734), so the chunk loop of
//   simulation_controller.py:1063-1130 needs no host round trip per check.  Once every member
//   has stopped the solver's halt word is set: RK4 and split-step launches queued after that
//   return at once, so the run ends on the step of the deciding check as the reference's
//   loop does.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "fft.cuh"
#include "ifrk_internal.h"
#include "pg_internal.h"
#include "solver.h"
#include "steady_monitor.h"

namespace pg {
namespace {

template <typename T>
__global__ void density_moments_kernel(const typename C2T<T>::type* __restrict__ psi,
                                       double* __restrict__ sum_rho, double* __restrict__ sum_rho2,
                                       long long n, const int* __restrict__ halt) {
  if (halt != nullptr && __ldcg(halt) != 0) return;  // a sample after the run halted: none
  for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < n;
       e += static_cast<long long>(gridDim.x) * blockDim.x) {
    const auto v = psi[e];
    const double re = static_cast<double>(v.x), im = static_cast<double>(v.y);
    // Rounded as the reference's NumPy sums are: each product and each sum on its own (no
    // fused multiply-add), so FP64 sums of an FP32 or FP64 field are bitwise the reference's.
    const double rho = __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im));
    sum_rho[e] = __dadd_rn(sum_rho[e], rho);
    sum_rho2[e] = __dadd_rn(sum_rho2[e], __dmul_rn(rho, rho));
  }
}

// Row pass: F_x of the F_y-transformed field, |.|^2 accumulated in FP64 per mode.
template <typename T>
__global__ void __launch_bounds__(1024) spectrum_power_row_kernel(const typename C2T<T>::type* __restrict__ half,
                                                                  const typename C2T<T>::type* __restrict__ tw,
                                                                  double* __restrict__ sum_k, int nx,
                                                                  int ny, int log2nx, int rows,
                                                                  int log2rows, const int* __restrict__ halt) {
  using C2 = typename C2T<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (halt != nullptr && __ldcg(halt) != 0) return;  // a sample after the run halted: none
  C2* tws = reinterpret_cast<C2*>(smem_raw);
  C2* buf = tws + nx;
  const int member = blockIdx.z;
  const long long off = static_cast<long long>(member) * nx * ny + static_cast<long long>(blockIdx.x) * rows * nx;
  for (int k = threadIdx.x; k < nx; k += blockDim.x) tws[k] = tw[k];
  const int count = rows * nx;
  for (int e = threadIdx.x; e < count; e += blockDim.x) buf[e] = half[off + e];
  __syncthreads();
  smem_fft<T, false, false>(buf, tws, log2nx, log2rows, 1, nx);
  for (int e = threadIdx.x; e < count; e += blockDim.x) {
    const double re = static_cast<double>(buf[e].x), im = static_cast<double>(buf[e].y);
    sum_k[off + e] = __dadd_rn(sum_k[off + e], __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im)));
  }
}

// Per-(member, block) FP64 partial sums of |psi|^2 over a member's sites.
template <typename T>
__global__ void norm_partials_kernel(const typename C2T<T>::type* __restrict__ psi, long long sites,
                                     double* __restrict__ partials) {
  __shared__ double red[32];
  const int member = blockIdx.y;
  const auto* p = psi + static_cast<long long>(member) * sites;
  double local = 0.0;
  for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < sites;
       e += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double re = static_cast<double>(p[e].x), im = static_cast<double>(p[e].y);
    local += re * re + im * im;
  }
  for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) partials[static_cast<long long>(member) * gridDim.x + blockIdx.x] = v;
  }
}

// out[m] = scale * sum of member m's partials (one warp per member).
__global__ void finalize_partials_kernel(const double* __restrict__ partials, int per_member,
                                         double scale, double* __restrict__ out) {
  const int member = blockIdx.x;
  double v = 0.0;
  for (int b = threadIdx.x; b < per_member; b += 32) v += partials[static_cast<long long>(member) * per_member + b];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (threadIdx.x == 0) out[member] = scale * v;
}

// Steady-state partials: sum (rho - rho_old)^2, sum rho_old^2, sum rho; rho_old <- rho.
// With two components the density is summed over them (simulation_controller.py:714-716).
template <typename T>
__global__ void steady_partials_kernel(const typename C2T<T>::type* __restrict__ psi,
                                       T* __restrict__ rho_old, long long sites, int comps,
                                       int have_old, double* __restrict__ partials,
                                       const int* __restrict__ halt) {
  __shared__ double red[3][32];
  if (halt != nullptr && __ldcg(halt) != 0) return;  // the state no longer advances
  const int member = blockIdx.y;
  const long long base = static_cast<long long>(member) * sites;
  double d2 = 0.0, o2 = 0.0, n = 0.0;
  for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < sites;
       e += static_cast<long long>(gridDim.x) * blockDim.x) {
    const auto v = psi[base * comps + e];
    T rho = v.x * v.x + v.y * v.y;
    if (comps == 2) {
      const auto w = psi[base * comps + sites + e];
      rho += w.x * w.x + w.y * w.y;
    }
    if (have_old) {
      const double old = static_cast<double>(rho_old[base + e]);
      const double diff = static_cast<double>(rho) - old;
      d2 += diff * diff;
      o2 += old * old;
    }
    n += static_cast<double>(rho);
    rho_old[base + e] = rho;
  }
  double vals[3] = {d2, o2, n};
  for (int q = 0; q < 3; ++q) {
    double v = vals[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    for (int q = 0; q < 3; ++q) {
      double v = threadIdx.x < (blockDim.x >> 5) ? red[q][threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (threadIdx.x == 0) partials[(static_cast<long long>(member) * gridDim.x + blockIdx.x) * 3 + q] = v;
    }
  }
}

struct AccumBuffers {
  double* sum_rho = nullptr;
  double* sum_rho2 = nullptr;
  double* sum_k = nullptr;
  void* half = nullptr;      // scratch spectrum for the momentum distribution
  void* rho_old = nullptr;   // density at the previous steady-state check
  double* partials = nullptr;
  int partial_blocks = 0;    // per member
  double* out = nullptr;     // device results (members)
  long long samples_rho = 0, samples_k = 0;
  SteadyMonitor mon;                 // device steady-state monitor (its have_old: rho_old holds a check)
};

constexpr int kReduceThreads = 256;

int reduce_blocks(long long sites) {
  const long long b = (sites + kReduceThreads * 8 - 1) / (kReduceThreads * 8);
  return static_cast<int>(std::max<long long>(1, std::min<long long>(b, 256)));
}

AccumBuffers& acc(pg_solver* s) { return *static_cast<AccumBuffers*>(s->accum); }

int ensure_accum(pg_solver* s) {
  if (s->accum) return PG_OK;
  AccumBuffers* a = new AccumBuffers();
  s->accum = a;
  a->partial_blocks = reduce_blocks(s->plane);
  PG_CUDA(cudaMalloc(&a->partials, sizeof(double) * 3 * a->partial_blocks * s->cfg.members));
  PG_CUDA(cudaMalloc(&a->out, sizeof(double) * s->cfg.members));
  return PG_OK;
}

template <typename T>
cudaError_t launch_norm(const void* psi, long long sites, int members, double scale,
                        double* partials, int blocks, double* out, cudaStream_t stream) {
  using C2 = typename C2T<T>::type;
  norm_partials_kernel<T><<<dim3(blocks, members), kReduceThreads, 0, stream>>>(
      static_cast<const C2*>(psi), sites, partials);
  finalize_partials_kernel<<<members, 32, 0, stream>>>(partials, blocks, scale, out);
  return cudaGetLastError();
}

}  // namespace

void accum_release(pg_solver* s) {
  if (!s->accum) return;
  AccumBuffers* a = static_cast<AccumBuffers*>(s->accum);
  cudaFree(a->sum_rho);
  cudaFree(a->sum_rho2);
  cudaFree(a->sum_k);
  cudaFree(a->half);
  cudaFree(a->rho_old);
  cudaFree(a->partials);
  cudaFree(a->out);
  steady_monitor_free(a->mon);
  delete a;
  s->accum = nullptr;
}

}  // namespace pg

extern "C" {

int pg_accumulate(pg_solver* s, int32_t kinds) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_accumulate: null solver");
  PG_CHECK((kinds & ~3) == 0 && kinds != 0, PG_ERR_INVALID,
           "pg_accumulate: kinds is a mask of 1 (density moments) and 2 (momentum distribution)");
  PG_CHECK(!s->spectral, PG_ERR_INVALID, "pg_accumulate: the state holds a spectrum");
  int rc = pg::ensure_accum(s);
  if (rc != PG_OK) return rc;
  pg::AccumBuffers& a = pg::acc(s);
  const bool dbl = s->cfg.precision == PG_DOUBLE;
  // Two-component fields accumulate per component (accumulators.py:103-113, 142-148).
  const long long values = s->field_values;
  const int planes = s->cfg.members * s->comps;
  const size_t dbytes = static_cast<size_t>(values) * sizeof(double);
  if (kinds & 1) {
    if (!a.sum_rho) {
      PG_CUDA(cudaMalloc(&a.sum_rho, dbytes));
      PG_CUDA(cudaMalloc(&a.sum_rho2, dbytes));
      PG_CUDA(cudaMemsetAsync(a.sum_rho, 0, dbytes, s->stream));
      PG_CUDA(cudaMemsetAsync(a.sum_rho2, 0, dbytes, s->stream));
    }
    const int blocks = static_cast<int>(std::min<long long>(4096, (values + 255) / 256));
    if (dbl)
      pg::density_moments_kernel<double><<<blocks, 256, 0, s->stream>>>(
          static_cast<const double2*>(s->psi[s->cur]), a.sum_rho, a.sum_rho2, values, s->halt);
    else
      pg::density_moments_kernel<float><<<blocks, 256, 0, s->stream>>>(
          static_cast<const float2*>(s->psi[s->cur]), a.sum_rho, a.sum_rho2, values, s->halt);
    PG_CUDA(cudaGetLastError());
    a.samples_rho += 1;
  }
  if (kinds & 2) {
    rc = pg::split_ensure(s);
    if (rc != PG_OK) return rc;
    const size_t cbytes = static_cast<size_t>(values) * 2 * s->real_size;
    if (!a.sum_k) {
      PG_CUDA(cudaMalloc(&a.sum_k, dbytes));
      PG_CUDA(cudaMemsetAsync(a.sum_k, 0, dbytes, s->stream));
    }
    if (!a.half) PG_CUDA(cudaMalloc(&a.half, cbytes));
    PG_CUDA(cudaMemcpyAsync(a.half, s->psi[s->cur], cbytes, cudaMemcpyDeviceToDevice, s->stream));
    // Column pass F_y (in place on the scratch copy), then the squaring row pass.
    pg::IfrkColArgs c{};
    const int mv = pg::split_max_vals(dbl);
    const size_t csize = dbl ? 16 : 8;
    const int nx = s->cfg.nx, ny = s->cfg.ny;
    auto ilog2 = [](int n) {
      int l = 0;
      while ((1 << l) < n) ++l;
      return l;
    };
    c.nx = nx;
    c.ny = ny;
    c.log2ny = ilog2(ny);
    int cols = 1;
    while (cols * 2 <= nx && cols * 2 <= 16 && cols * 2 * ny * csize <= 160 * 1024 && cols * 2 * ny <= mv * 1024)
      cols *= 2;
    c.cols = cols;
    c.log2cols = ilog2(cols);
    c.threads = std::max(32, (((cols * ny + mv - 1) / mv + 31) / 32) * 32);
    c.members = planes;
    c.comps = 1;
    c.mode = 3;
    c.forward = 1;
    if (dbl) {
      PG_CUDA(pg::configure_ifrk_kernels<double>(200 * 1024));
      PG_CUDA(pg::launch_ifrk_col<double>(static_cast<double*>(a.half), nullptr, nullptr, nullptr,
                                          nullptr, nullptr, nullptr, nullptr,
                                          static_cast<const double*>(s->tw_y), nullptr, nullptr,
                                          nullptr, nullptr, c, s->stream));
    } else {
      PG_CUDA(pg::configure_ifrk_kernels<float>(200 * 1024));
      PG_CUDA(pg::launch_ifrk_col<float>(static_cast<float*>(a.half), nullptr, nullptr, nullptr,
                                         nullptr, nullptr, nullptr, nullptr,
                                         static_cast<const float*>(s->tw_y), nullptr, nullptr,
                                         nullptr, nullptr, c, s->stream));
    }
    int rows = 1;
    while (rows * 2 <= ny && rows * 2 * nx <= 4096) rows *= 2;
    const int threads = std::max(32, (((rows * nx + mv - 1) / mv + 31) / 32) * 32);
    const size_t smem = csize * (static_cast<size_t>(nx) + static_cast<size_t>(rows) * nx);
    if (dbl) {
      cudaFuncSetAttribute(pg::spectrum_power_row_kernel<double>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      pg::spectrum_power_row_kernel<double><<<dim3(ny / rows, 1, planes), threads, smem, s->stream>>>(
          static_cast<const double2*>(a.half), static_cast<const double2*>(s->tw_x), a.sum_k, nx, ny,
          ilog2(nx), rows, ilog2(rows), s->halt);
    } else {
      cudaFuncSetAttribute(pg::spectrum_power_row_kernel<float>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      pg::spectrum_power_row_kernel<float><<<dim3(ny / rows, 1, planes), threads, smem, s->stream>>>(
          static_cast<const float2*>(a.half), static_cast<const float2*>(s->tw_x), a.sum_k, nx, ny,
          ilog2(nx), rows, ilog2(rows), s->halt);
    }
    PG_CUDA(cudaGetLastError());
    a.samples_k += 1;
  }
  return PG_OK;
}

int pg_accumulator_sums(pg_solver* s, int32_t kind, double* out, int64_t* samples) {
  PG_CHECK(s && out && samples, PG_ERR_INVALID, "pg_accumulator_sums: null argument");
  PG_CHECK(s->accum, PG_ERR_INVALID, "pg_accumulator_sums: nothing accumulated");
  pg::AccumBuffers& a = pg::acc(s);
  const size_t bytes = static_cast<size_t>(s->field_values) * sizeof(double);
  double* src = kind == 0 ? a.sum_rho : kind == 1 ? a.sum_rho2 : kind == 2 ? a.sum_k : nullptr;
  PG_CHECK(src, PG_ERR_INVALID, "pg_accumulator_sums: kind 0 sum rho, 1 sum rho^2, 2 sum |psi_k|^2");
  PG_CUDA(cudaMemcpyAsync(out, src, bytes, cudaMemcpyDeviceToHost, s->stream));
  PG_CUDA(pg::stream_sync(s));
  *samples = kind == 2 ? a.samples_k : a.samples_rho;
  return PG_OK;
}

int pg_accumulator_load(pg_solver* s, int32_t kind, const double* sums, int64_t samples) {
  PG_CHECK(s && sums && samples >= 0, PG_ERR_INVALID, "pg_accumulator_load: bad argument");
  PG_CHECK(kind >= 0 && kind <= 2, PG_ERR_INVALID,
           "pg_accumulator_load: kind 0 sum rho, 1 sum rho^2, 2 sum |psi_k|^2");
  int rc = pg::ensure_accum(s);
  if (rc != PG_OK) return rc;
  pg::AccumBuffers& a = pg::acc(s);
  const size_t bytes = static_cast<size_t>(s->field_values) * sizeof(double);
  double** dst = kind == 0 ? &a.sum_rho : kind == 1 ? &a.sum_rho2 : &a.sum_k;
  if (kind < 2 && !a.sum_rho) {  // the two density sums live and die together
    PG_CUDA(cudaMalloc(&a.sum_rho, bytes));
    PG_CUDA(cudaMalloc(&a.sum_rho2, bytes));
    PG_CUDA(cudaMemsetAsync(a.sum_rho, 0, bytes, s->stream));
    PG_CUDA(cudaMemsetAsync(a.sum_rho2, 0, bytes, s->stream));
  }
  if (!*dst) PG_CUDA(cudaMalloc(dst, bytes));
  PG_CUDA(cudaMemcpyAsync(*dst, sums, bytes, cudaMemcpyHostToDevice, s->stream));
  PG_CUDA(pg::stream_sync(s));
  if (kind == 2)
    a.samples_k = samples;
  else
    a.samples_rho = samples;
  return PG_OK;
}

int pg_steady_export(pg_solver* s, void* density, double* norms, int64_t* stop_steps,
                     int32_t* have_reference) {
  PG_CHECK(s && have_reference, PG_ERR_INVALID, "pg_steady_export: null argument");
  *have_reference = 0;
  if (!s->accum || !pg::acc(s).mon.norm_old) {
    if (stop_steps)
      for (int m = 0; m < s->cfg.members; ++m) stop_steps[m] = -1;
    return PG_OK;
  }
  pg::AccumBuffers& a = pg::acc(s);
  const int m = s->cfg.members;
  PG_CUDA(pg::stream_sync(s));
  if (a.mon.have_old) {
    if (density)
      PG_CUDA(cudaMemcpy(density, a.rho_old, static_cast<size_t>(s->sites) * s->real_size,
                         cudaMemcpyDeviceToHost));
    if (norms) PG_CUDA(cudaMemcpy(norms, a.mon.norm_old, sizeof(double) * m, cudaMemcpyDeviceToHost));
    *have_reference = 1;
  }
  if (stop_steps)
    PG_CUDA(cudaMemcpy(stop_steps, a.mon.stop_step, sizeof(long long) * m, cudaMemcpyDeviceToHost));
  return PG_OK;
}

int pg_steady_import(pg_solver* s, const void* density, const double* norms,
                     const int64_t* stop_steps, int32_t have_reference) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_steady_import: null solver");
  PG_CHECK(!have_reference || (density && norms), PG_ERR_INVALID,
           "pg_steady_import: a reference needs the density and the norms");
  int rc = pg_steady_reset(s);
  if (rc != PG_OK) return rc;
  pg::AccumBuffers& a = pg::acc(s);
  const int m = s->cfg.members;
  if (have_reference || stop_steps) ++s->host_syncs;  // blocking copies
  if (have_reference) {
    PG_CUDA(cudaMemcpy(a.rho_old, density, static_cast<size_t>(s->sites) * s->real_size,
                       cudaMemcpyHostToDevice));
    PG_CUDA(cudaMemcpy(a.mon.norm_old, norms, sizeof(double) * m, cudaMemcpyHostToDevice));
    a.mon.have_old = true;
  }
  if (stop_steps)
    PG_CUDA(cudaMemcpy(a.mon.stop_step, stop_steps, sizeof(long long) * m, cudaMemcpyHostToDevice));
  return PG_OK;
}

int pg_accumulator_zero(pg_solver* s) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_accumulator_zero: null solver");
  if (!s->accum) return PG_OK;
  pg::AccumBuffers& a = pg::acc(s);
  const size_t bytes = static_cast<size_t>(s->field_values) * sizeof(double);
  if (a.sum_rho) PG_CUDA(cudaMemsetAsync(a.sum_rho, 0, bytes, s->stream));
  if (a.sum_rho2) PG_CUDA(cudaMemsetAsync(a.sum_rho2, 0, bytes, s->stream));
  if (a.sum_k) PG_CUDA(cudaMemsetAsync(a.sum_k, 0, bytes, s->stream));
  a.samples_rho = a.samples_k = 0;
  return PG_OK;
}

int pg_accumulator_reset(pg_solver* s) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_accumulator_reset: null solver");
  if (!s->accum) return PG_OK;
  pg::AccumBuffers& a = pg::acc(s);
  const size_t bytes = static_cast<size_t>(s->field_values) * sizeof(double);
  if (a.sum_rho) PG_CUDA(cudaMemsetAsync(a.sum_rho, 0, bytes, s->stream));
  if (a.sum_rho2) PG_CUDA(cudaMemsetAsync(a.sum_rho2, 0, bytes, s->stream));
  if (a.sum_k) PG_CUDA(cudaMemsetAsync(a.sum_k, 0, bytes, s->stream));
  a.samples_rho = a.samples_k = 0;
  a.mon.have_old = false;
  PG_CUDA(pg::stream_sync(s));
  return PG_OK;
}

int pg_norms(pg_solver* s, double* out) {
  PG_CHECK(s && out, PG_ERR_INVALID, "pg_norms: null argument");
  PG_CHECK(!s->spectral, PG_ERR_INVALID, "pg_norms: the state holds a spectrum");
  int rc = pg::ensure_accum(s);
  if (rc != PG_OK) return rc;
  pg::AccumBuffers& a = pg::acc(s);
  const double cell = s->cfg.dx * s->cfg.dy;
  const cudaError_t e =
      s->cfg.precision == PG_DOUBLE
          ? pg::launch_norm<double>(s->psi[s->cur], s->plane * s->comps, s->cfg.members, cell,
                                    a.partials, a.partial_blocks, a.out, s->stream)
          : pg::launch_norm<float>(s->psi[s->cur], s->plane * s->comps, s->cfg.members, cell,
                                   a.partials, a.partial_blocks, a.out, s->stream);
  PG_CUDA(e);
  PG_CUDA(cudaMemcpyAsync(out, a.out, sizeof(double) * s->cfg.members, cudaMemcpyDeviceToHost, s->stream));
  PG_CUDA(pg::stream_sync(s));
  return PG_OK;
}

int pg_steady_reset(pg_solver* s) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_steady_reset: null solver");
  int rc = pg::ensure_accum(s);
  if (rc != PG_OK) return rc;
  pg::AccumBuffers& a = pg::acc(s);
  PG_CUDA(pg::steady_monitor_alloc(a.mon, s->cfg.members));
  if (!a.rho_old) PG_CUDA(cudaMalloc(&a.rho_old, static_cast<size_t>(s->sites) * s->real_size));
  // Stream ordered, without a host wait (steady_monitor_reset).
  PG_CUDA(pg::steady_monitor_reset(a.mon, s->halt, s->stream));
  return PG_OK;
}

int pg_steady_update(pg_solver* s, int64_t step, int32_t record, double rtol,
                     int32_t halt_when_all_stopped) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_steady_update: null solver");
  PG_CHECK(!s->spectral, PG_ERR_INVALID, "pg_steady_update: the state holds a spectrum");
  PG_CHECK(rtol >= 0.0, PG_ERR_INVALID, "pg_steady_update: negative rtol");
  int rc = pg::ensure_accum(s);
  if (rc != PG_OK) return rc;
  pg::AccumBuffers& a = pg::acc(s);
  if (!a.mon.norm_old) {
    rc = pg_steady_reset(s);
    if (rc != PG_OK) return rc;
  }
  const int blocks = a.partial_blocks;
  const int m = s->cfg.members;
  if (s->cfg.precision == PG_DOUBLE)
    pg::steady_partials_kernel<double><<<dim3(blocks, m), 256, 0, s->stream>>>(
        static_cast<const double2*>(s->psi[s->cur]), static_cast<double*>(a.rho_old), s->plane,
        s->comps, a.mon.have_old ? 1 : 0, a.partials, s->halt);
  else
    pg::steady_partials_kernel<float><<<dim3(blocks, m), 256, 0, s->stream>>>(
        static_cast<const float2*>(s->psi[s->cur]), static_cast<float*>(a.rho_old), s->plane,
        s->comps, a.mon.have_old ? 1 : 0, a.partials, s->halt);
  PG_CUDA(cudaGetLastError());
  PG_CUDA(pg::steady_monitor_decide(a.mon, a.partials, blocks, nullptr, s->cfg.dx * s->cfg.dy,
                                    record ? 1 : 0, rtol, static_cast<long long>(step), s->flips,
                                    halt_when_all_stopped ? 1 : 0, s->halt, s->stream));
  return PG_OK;
}

int pg_steady_poll(pg_solver* s, int32_t* stopped, int64_t* updates_done) {
  PG_CHECK(s && stopped && updates_done, PG_ERR_INVALID, "pg_steady_poll: null argument");
  if (!s->accum) {
    *stopped = 0;
    *updates_done = 0;
    return PG_OK;
  }
  pg::steady_monitor_poll(pg::acc(s).mon, stopped, updates_done);
  return PG_OK;
}

int pg_steady_results(pg_solver* s, double* rel_density, double* rel_norm, double* norms,
                      int64_t* stop_steps, int64_t* halt_step) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_steady_results: null solver");
  PG_CHECK(s->accum && pg::acc(s).mon.norm_old, PG_ERR_INVALID,
           "pg_steady_results: no steady-state check has been made");
  pg::AccumBuffers& a = pg::acc(s);
  const int m = s->cfg.members;
  std::vector<double> res(static_cast<size_t>(3) * m);
  std::vector<long long> stops(m);
  long long hs[2] = {-1, -1};  // step and flips of the halting check
  int halted = 0;
  PG_CUDA(pg::steady_monitor_fetch(a.mon, s->halt, res.data(), stops.data(), &halted, hs, s->stream));
  PG_CUDA(pg::stream_sync(s));
  for (int mm = 0; mm < m; ++mm) {
    if (rel_density) rel_density[mm] = res[mm];
    if (rel_norm) rel_norm[mm] = res[m + mm];
    if (norms) norms[mm] = res[2 * m + mm];
    if (stop_steps) stop_steps[mm] = stops[mm];
  }
  if (halted) {
    // RK4 launches after the halt returned without writing, yet the host swapped the
    // ping-pong buffers for each of them: the state of the halt step is under the parity it
    // had then (split steps, in place, swap nothing).  Clear the halt so that the solver
    // steps again.
    s->cur ^= static_cast<int>((s->flips - hs[1]) & 1);
    s->flips = hs[1];
    s->parity_step = hs[0];
    PG_CUDA(cudaMemsetAsync(s->halt, 0, sizeof(int), s->stream));
    PG_CUDA(pg::stream_sync(s));
  }
  if (halt_step) *halt_step = halted ? hs[0] : -1;
  return PG_OK;
}

int pg_steady_check(pg_solver* s, double* rel_density, double* rel_norm, double* norms) {
  PG_CHECK(s && rel_density && rel_norm && norms, PG_ERR_INVALID, "pg_steady_check: null argument");
  int rc = pg_steady_update(s, -1, 0, 0.0, 0);
  if (rc != PG_OK) return rc;
  return pg_steady_results(s, rel_density, rel_norm, norms, nullptr, nullptr);
}

// Stand-alone FP64 norms of caller-owned device fields; scratch for the per-block partial
// sums is allocated for the call.
int pg_field_norms(const void* psi, int32_t precision, int32_t members, int64_t sites_per_member,
                   double cell, double* norms_out, void* stream) {
  PG_CHECK(psi && norms_out && members >= 1 && sites_per_member >= 1, PG_ERR_INVALID,
           "pg_field_norms: bad argument");
  PG_CHECK(precision == PG_SINGLE || precision == PG_DOUBLE, PG_ERR_INVALID,
           "pg_field_norms: bad precision");
  const int blocks = pg::reduce_blocks(sites_per_member);
  double* partials = nullptr;
  PG_CUDA(cudaMalloc(&partials, sizeof(double) * static_cast<size_t>(blocks) * members));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = precision == PG_DOUBLE
                      ? pg::launch_norm<double>(psi, sites_per_member, members, cell, partials, blocks,
                                                norms_out, st)
                      : pg::launch_norm<float>(psi, sites_per_member, members, cell, partials, blocks,
                                               norms_out, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(partials);
  if (e != cudaSuccess) {
    pg::set_error(std::string("pg_field_norms: ") + cudaGetErrorString(e));
    return PG_ERR_CUDA;
  }
  return PG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Allocation-free FP64 norms.
//
// Some callers of this library must not allocate device memory: an application whose
// device memory is owned by another framework's pooling allocator (a PyTorch or JAX
// process that reserved it), or a stepping loop that cannot pay for the device-wide
// synchronisation cudaMalloc and cudaFree imply.  pg_field_norms_noalloc serves them: the
// per-block partial sums live in the fixed device array below instead of memory allocated
// per call.
//
// The array holds kNoAllocPartials doubles (64 KiB) on every GPU that loads the library,
// until the process exits.  All calls share it; each call overwrites the partials it uses
// before reading them, so nothing has to start at zero, but calls whose kernels overlap on
// the GPU (different streams or host threads) race on it and must be serialised by the
// caller.  The first call on each device looks up the array's device address
// (cudaGetSymbolAddress) with that device current; make that first call before any stream
// capture.  The address is cached per device for the life of the process: after
// cudaDeviceReset (which unloads this module's device copy) the cache is stale, so a process
// that resets a device must not call this entry point on it again.  Two host threads making
// their first call on the same device at once both look the address up and store the same
// value, so the unsynchronised cache write is harmless.
namespace pg {
namespace {

constexpr int kNoAllocPartials = 8192;
static __device__ __align__(256) double g_noalloc_partials[kNoAllocPartials];

constexpr int kMaxDevices = 64;
double* g_noalloc_ptr[kMaxDevices] = {};

}  // namespace
}  // namespace pg

extern "C" int pg_field_norms_noalloc(const void* psi, int32_t precision, int32_t members,
                                      int64_t sites_per_member, double cell, double* norms_out,
                                      void* stream) {
  PG_CHECK(psi && norms_out && members >= 1 && sites_per_member >= 1, PG_ERR_INVALID,
           "pg_field_norms_noalloc: bad argument");
  PG_CHECK(precision == PG_SINGLE || precision == PG_DOUBLE, PG_ERR_INVALID,
           "pg_field_norms_noalloc: bad precision");
  PG_CHECK(members <= pg::kNoAllocPartials, PG_ERR_INVALID,
           "pg_field_norms_noalloc: at most 8192 members fit the fixed scratch array");
  int dev = 0;
  PG_CUDA(cudaGetDevice(&dev));
  PG_CHECK(dev >= 0 && dev < pg::kMaxDevices, PG_ERR_UNSUPPORTED,
           "pg_field_norms_noalloc: device index beyond the supported 64");
  if (!pg::g_noalloc_ptr[dev]) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, pg::g_noalloc_partials);
    if (e != cudaSuccess) {
      pg::set_error(std::string("pg_field_norms_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return PG_ERR_CUDA;
    }
    pg::g_noalloc_ptr[dev] = static_cast<double*>(ptr);
  }
  // Blocks per member, bounded so members * blocks fits the array.
  const int blocks = std::max(1, std::min(pg::reduce_blocks(sites_per_member), pg::kNoAllocPartials / members));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const cudaError_t e =
      precision == PG_DOUBLE
          ? pg::launch_norm<double>(psi, sites_per_member, members, cell, pg::g_noalloc_ptr[dev], blocks,
                                    norms_out, st)
          : pg::launch_norm<float>(psi, sites_per_member, members, cell, pg::g_noalloc_ptr[dev], blocks,
                                   norms_out, st);
  if (e != cudaSuccess) {
    pg::set_error(std::string("pg_field_norms_noalloc: ") + cudaGetErrorString(e));
    return PG_ERR_CUDA;
  }
  return PG_OK;
}
