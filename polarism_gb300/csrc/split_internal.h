// Internal declarations of the split-step (Stockham FFT) passes.
#pragma once
#include <cuda_runtime.h>

namespace pg {

enum SplitOp {
  SPLIT_OP_NONE = 0,
  SPLIT_OP_KOUTER = 1,         // R(dt/2) at P(t+dt/4), N(dt), R(dt/2) at P(t+3dt/4), Wigner
  SPLIT_OP_RES_START = 2,      // R(dt/2) at P(t+dt/4)
  SPLIT_OP_RES_END_START = 3,  // R(dt/2) at P(t-dt/4) of the previous step, then at P(t+dt/4)
  SPLIT_OP_NONLINEAR = 4,      // N(dt), then Wigner with the current n_R
  SPLIT_OP_RES_END = 5,        // R(dt/2) at P(t+3dt/4)
};

// Per-member constants of the local split-step operations.
template <typename T>
struct SplitConst {
  T inv_hbar, g_C, g_R, R, gamma_C, gamma_R;
  T noise_a, noise_b;
  unsigned long long seed;
  // Inactive-reservoir coupling, cross-spin term, two-field reservoir rates and the pump
  // share of each component (the cross-spin term and the shares are read by the IFRK
  // passes only).
  T g_I, alpha_2, gamma_I, gamma_A, R_IA, R_AI;
  T weight[2];
  T kappa;
};

struct RowPassArgs {
  int nx, ny, log2nx;
  int rows, log2rows;   // rows per block (power of two)
  int threads;
  int forward, inverse, multiply;
  int table_stride;     // complex values between consecutive members' propagator factors
  double scale;         // power-of-two factor of the kick: psi (1 + d) * scale
  const int* halt;      // steady-state monitor's halt word: when set the pass returns at once
};

struct ColPassArgs {
  int nx, ny, log2ny;
  int cols, log2cols;   // columns per block (power of two)
  int threads;
  int members;
  int forward, inverse;
  int op;               // SplitOp
  int reservoir;        // single reservoir present
  int res_kind;         // PG_RES_*: 2 double, 3 quadratic-double use the second field
  int potential;        // 0 none, 1 real, 2 complex
  int noise;
  long long pump_stride, pot_stride;
  int pump_terms;       // separable pump terms L
  long long pump_term_stride;  // reals between consecutive terms' envelopes
  int scale_offset;     // coefficient sample ([k][sample][term][member]) of the first coefficient
  int step_offset;      // noise step = step_base[0] + step_offset
  double dt_d;
  float dt_f;
  const int* halt;      // as RowPassArgs::halt
  // dt in the working precision is read through dt_of<T>().
  template <typename T>
  __host__ __device__ T dt_of() const;
};

template <>
inline __host__ __device__ float ColPassArgs::dt_of<float>() const { return dt_f; }
template <>
inline __host__ __device__ double ColPassArgs::dt_of<double>() const { return dt_d; }

template <typename T>
cudaError_t launch_row_pass(T* data, const T* tw, const T* px, const T* py, const RowPassArgs& a,
                            int members, cudaStream_t stream);

template <typename T>
cudaError_t launch_col_pass(T* data, T* res, const T* pump, const T* potential, const T* tw,
                            const SplitConst<T>* consts, const T* scales,
                            const unsigned long long* step_base, const ColPassArgs& a,
                            cudaStream_t stream);

template <typename T>
cudaError_t configure_split_kernels(size_t max_smem);

// Register-resident four-step passes for FP32 rows / columns of 1024 sites (split_fast.cu):
// whether they apply, their W_1024^{n2 k1} table (1024 float4: rounded value, remainder),
// attribute set-up and launches (arguments as launch_row_pass / launch_col_pass).
bool split_fast_row(int nx, int ny);
bool split_fast_col(int nx, int ny);
void split_fast_twiddles(float* out);
cudaError_t configure_split_fast();
cudaError_t launch_row_fast(float* data, const float* tw4, const float* px, const float* py,
                            const RowPassArgs& a, int members, cudaStream_t stream);
cudaError_t launch_col_fast(float* data, float* res, const float* pump, const float* potential,
                            const float* tw4, const SplitConst<float>* consts, const float* scales,
                            const unsigned long long* step_base, const ColPassArgs& a,
                            cudaStream_t stream);

// The IFRK row pass on the same transforms (FP32, one component, rows of 1024 sites): whether
// it applies and its launch (arguments as launch_ifrk_row; tw4 as above).
struct IfrkRowArgs;
struct IfrkColArgs;
bool ifrk_fast_row(const IfrkRowArgs& a);
// The IFRK column pass likewise (one component, columns of 1024 sites, eight-column panels):
// the forward-only pass, and stages and step ends with one single reservoir and one laser.
bool ifrk_fast_col(const IfrkColArgs& a);
cudaError_t launch_ifrk_col_fast(float* psi, const float* n0, float* dn_out, float* n_out,
                                 const float* psi_start, const float* psi_new, const float* pump,
                                 const float* potential, const float* tw4,
                                 const SplitConst<float>* consts, const float* scales,
                                 const unsigned long long* step_base, const IfrkColArgs& a,
                                 cudaStream_t stream);
cudaError_t launch_ifrk_row_fast(const float* in, float* save, float* out, const float* tables,
                                 const float* tw4, const IfrkRowArgs& a, cudaStream_t stream);

// Complex values one thread stages per FFT pass: blocks need N * C <= this * threads.
int split_max_vals(bool is_double);

}  // namespace pg
