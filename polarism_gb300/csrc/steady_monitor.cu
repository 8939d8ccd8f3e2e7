// The device-resident steady-state monitor (steady_monitor.h).
#include <cmath>

#include "steady_monitor.h"

namespace pg {
namespace {

// Per-member decision of one steady-state check from the partial sums (one block): relative
// density and norm changes, the stop criterion of simulation_controller.py:728-729 and the
// first stop step (_record_stops, :698-708).
__global__ void steady_decide_kernel(const double* __restrict__ partials, int blocks, int members,
                                     const double* __restrict__ cells, double cell, int have_old,
                                     int record, double rtol, long long step, long long swaps,
                                     int halt_when_all, double* __restrict__ norm_old,
                                     long long* __restrict__ stop_step, double* __restrict__ results,
                                     int* __restrict__ halt, long long* __restrict__ halt_step,
                                     unsigned long long* __restrict__ host_word,
                                     unsigned int update_index) {
  __shared__ int stopped;
  if (halt != nullptr && __ldcg(halt) != 0) return;  // already halted: nothing has changed
  if (threadIdx.x == 0) stopped = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
  for (int m = warp; m < members; m += warps) {
    double v[3] = {0.0, 0.0, 0.0};
    for (int b = lane; b < blocks; b += 32)
      for (int q = 0; q < 3; ++q) v[q] += partials[(static_cast<long long>(m) * blocks + b) * 3 + q];
    for (int q = 0; q < 3; ++q)
      for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
    if (lane == 0) {
      const double norm = v[2] * (cells != nullptr ? cells[m] : cell);
      double rd = INFINITY, rn = INFINITY;
      if (have_old) {
        rd = sqrt(v[0]) / fmax(sqrt(v[1]), 1e-30);
        rn = fabs(norm - norm_old[m]) / fmax(norm_old[m], 1e-30);
        const bool reached = norm < 1e-30 || (rn < rtol && rd < rtol);
        if (record && reached && stop_step[m] < 0) stop_step[m] = step;
      }
      results[m] = rd;
      results[members + m] = rn;
      results[2 * members + m] = norm;
      norm_old[m] = norm;
      if (stop_step[m] >= 0) atomicAdd(&stopped, 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (halt_when_all && stopped == members && halt != nullptr) {
      *halt = 1;
      halt_step[0] = step;
      halt_step[1] = swaps;
    }
    *reinterpret_cast<volatile unsigned long long*>(host_word) =
        (static_cast<unsigned long long>(update_index) << 32) | static_cast<unsigned int>(stopped);
    __threadfence_system();
  }
}

}  // namespace

cudaError_t steady_monitor_alloc(SteadyMonitor& mon, int members) {
  if (mon.norm_old) return cudaSuccess;
  cudaError_t e;
  if ((e = cudaMalloc(&mon.norm_old, sizeof(double) * members)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&mon.stop_step, sizeof(long long) * members)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&mon.results, sizeof(double) * 3 * members)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&mon.halt_step, 2 * sizeof(long long))) != cudaSuccess) return e;
  if ((e = cudaHostAlloc(&mon.host_word, sizeof(unsigned long long), cudaHostAllocMapped)) !=
      cudaSuccess)
    return e;
  *reinterpret_cast<volatile unsigned long long*>(mon.host_word) = 0ull;
  if ((e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&mon.dev_word), mon.host_word, 0)) !=
      cudaSuccess)
    return e;
  mon.members = members;
  return cudaSuccess;
}

void steady_monitor_free(SteadyMonitor& mon) {
  cudaFree(mon.norm_old);
  cudaFree(mon.stop_step);
  cudaFree(mon.results);
  cudaFree(mon.halt_step);
  if (mon.host_word) cudaFreeHost(mon.host_word);
  mon = SteadyMonitor{};
}

cudaError_t steady_monitor_reset(SteadyMonitor& mon, int* halt, cudaStream_t stream) {
  const int m = mon.members;
  cudaError_t e;
  if ((e = cudaMemsetAsync(mon.norm_old, 0, sizeof(double) * m, stream)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(mon.stop_step, 0xff, sizeof(long long) * m, stream)) != cudaSuccess)
    return e;  // -1
  if ((e = cudaMemsetAsync(mon.halt_step, 0xff, 2 * sizeof(long long), stream)) != cudaSuccess)
    return e;
  if (halt != nullptr && (e = cudaMemsetAsync(halt, 0, sizeof(int), stream)) != cudaSuccess) return e;
  mon.have_old = false;
  mon.reset_base = mon.updates;
  return cudaSuccess;
}

cudaError_t steady_monitor_decide(SteadyMonitor& mon, const double* partials, int blocks,
                                  const double* cells, double cell, int record, double rtol,
                                  long long step, long long swaps, int halt_when_all, int* halt,
                                  cudaStream_t stream) {
  mon.updates += 1;
  steady_decide_kernel<<<1, 256, 0, stream>>>(
      partials, blocks, mon.members, cells, cell, mon.have_old ? 1 : 0, record, rtol, step, swaps,
      halt_when_all, mon.norm_old, mon.stop_step, mon.results, halt, mon.halt_step, mon.dev_word,
      mon.updates);
  mon.have_old = true;
  return cudaGetLastError();
}

void steady_monitor_poll(const SteadyMonitor& mon, int32_t* stopped, int64_t* updates_done) {
  if (!mon.host_word) {
    *stopped = 0;
    *updates_done = 0;
    return;
  }
  const unsigned long long w = *reinterpret_cast<volatile unsigned long long*>(mon.host_word);
  const unsigned int done = static_cast<unsigned int>(w >> 32) - mon.reset_base;
  // A word from before the last reset (or none yet) reads as no check finished.
  const bool current = done != 0 && done <= mon.updates - mon.reset_base;
  *stopped = current ? static_cast<int32_t>(w & 0xffffffffull) : 0;
  *updates_done = current ? static_cast<int64_t>(done) : 0;
}

cudaError_t steady_monitor_fetch(const SteadyMonitor& mon, const int* halt, double* results,
                                 long long* stops, int* halted, long long* halt_record,
                                 cudaStream_t stream) {
  const int m = mon.members;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(results, mon.results, sizeof(double) * 3 * m, cudaMemcpyDeviceToHost,
                           stream)) != cudaSuccess)
    return e;
  if ((e = cudaMemcpyAsync(stops, mon.stop_step, sizeof(long long) * m, cudaMemcpyDeviceToHost,
                           stream)) != cudaSuccess)
    return e;
  if ((e = cudaMemcpyAsync(halted, halt, sizeof(int), cudaMemcpyDeviceToHost, stream)) != cudaSuccess)
    return e;
  return cudaMemcpyAsync(halt_record, mon.halt_step, 2 * sizeof(long long), cudaMemcpyDeviceToHost,
                         stream);
}

}  // namespace pg
