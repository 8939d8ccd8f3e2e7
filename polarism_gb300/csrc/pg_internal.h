// Internal declarations shared by the CUDA translation units of libpolarism_gb300.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/polarism_gb300.h"

namespace pg {

// Thread-local last error; every C-ABI entry point clears it on success.
void set_error(const std::string& msg);
const char* last_error();

#define PG_CUDA(call)                                                                 \
  do {                                                                                \
    cudaError_t _e = (call);                                                          \
    if (_e != cudaSuccess) {                                                          \
      ::pg::set_error(std::string(#call) + ": " + cudaGetErrorString(_e));            \
      return PG_ERR_CUDA;                                                             \
    }                                                                                 \
  } while (0)

#define PG_CHECK(cond, code, msg)                                                     \
  do {                                                                                \
    if (!(cond)) {                                                                    \
      ::pg::set_error(msg);                                                           \
      return (code);                                                                  \
    }                                                                                 \
  } while (0)

// Per-member constants of the finite-difference right-hand side, pre-divided so the
// stage arithmetic is a short chain of FMAs.  a = hbar / (2 m_eff).
template <typename T>
struct RhsConst {
  T ax, ay;          // a / dx^2, a / dy^2
  T w0;              // 2 (ax + ay): the Laplacian's centre weight
  T gc, gr, gi;      // g_C / hbar, g_R / hbar, g_I / hbar
  T inv_hbar;        // 1 / hbar (potential)
  T half_R, half_gC; // R / 2, gamma_C / 2
  T R, gamma_R;      // reservoir loss
  T eta_a;           // kinetic relaxation eta (multiplies n_A * a * Laplacian)
  T noise_a, noise_b;// sigma^2 = noise_a + noise_b * n_A  (strength (gamma_C + R n) dt / (4 dV))
  T pad_;
  unsigned long long seed;
  // Two-field reservoirs: double (active n_A, inactive n_I) and quadratic-double (n_R, n_I).
  T gamma_I, gamma_A, R_IA, R_AI, kappa, pad2_;
};

// Geometry of one RK4 launch (one time step over every member).
struct RK4Geom {
  int nx, ny, members;
  int tile_w;        // useful columns per block
  int strip_h;       // output rows per block
  int wrap;          // 1: the block spans the full periodic row (no x halo)
  long long pump_stride;   // 0: shared envelope; nx*ny: one envelope per member
  long long pot_stride;    // 0: shared potential; nx*ny: per member
  const int* halt = nullptr;  // when non-null and set, the launch returns at once
  long long pump_term_stride = 0;  // reals between consecutive pump terms' envelopes
};

struct RK4Features {
  int potential;     // 0 none, 1 real, 2 complex
  int relax;         // kinetic relaxation term on
  int reservoir;     // PG_RES_*: 0 none, 1 single, 2 double, 3 quadratic-double
  int pump_terms;    // separable pump terms L (> 1 only on the general variant)
};

// Pump value of L separable terms at element o of the member's first envelope:
// sum_t c[t * cstride] E_t[o], each product and each partial sum rounded separately (the
// reference's combiner is compiled without FMA contraction, polarism/solver/cuda_pump.py:7-19).
__device__ __forceinline__ float pump_mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double pump_mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float pump_add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double pump_add_rn(double a, double b) { return __dadd_rn(a, b); }
template <typename T>
__device__ __forceinline__ T pump_terms_value(const T* env, long long term_stride, const T* c,
                                              int cstride, int terms, long long o) {
  T v = pump_mul_rn(c[0], env[o]);
  for (int t = 1; t < terms; ++t)
    v = pump_add_rn(v, pump_mul_rn(c[static_cast<long long>(t) * cstride], env[t * term_stride + o]));
  return v;
}

// Launch one fused whole-step RK4 update; scales points at [3][members] pump
// coefficients (device memory) and step_base at the global step counter (device).
// With a two-field reservoir n_in/n_out hold the active field of every member followed by
// the inactive field of every member.
template <typename T>
cudaError_t launch_rk4_step(const T* psi_in, const T* n_in, const T* pump, const T* potential,
                            T* psi_out, T* n_out, const RhsConst<T>* consts,
                            const T* scales, const unsigned long long* step_base,
                            int step_offset, T dt, bool noise, const RK4Geom& g,
                            const RK4Features& f, cudaStream_t stream);

// Choose the tile width / strip height for a grid (deterministic heuristic,
// overridable through the autotuner table).
void choose_rk4_geometry(int nx, int ny, int members, int precision, int sm_count,
                         RK4Geom* g);

int philox_words_device(const uint32_t* counters, uint64_t key, uint32_t* out, int64_t n,
                        cudaStream_t stream);

}  // namespace pg
