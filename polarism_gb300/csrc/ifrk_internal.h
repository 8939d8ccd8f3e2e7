// Internal declarations of the Lawson IFRK passes.
#pragma once
#include <cuda_runtime.h>

#include "split_internal.h"

namespace pg {

constexpr int kIfrkMaxTerms = 8;   // psi0_hat plus up to 7 stage spectra
constexpr int kIfrkMaxStages = 7;  // dp5

// Row pass: [F_x of `in` (+ store to `save`)] -> out_hat = sum_t coef_t E_t src_t ->
// [F_x^-1] -> out.  A source pointer equal to nullptr selects the freshly transformed row.
struct IfrkRowArgs {
  int nx, ny, log2nx, rows, log2rows, threads, members;
  int comps;                   // field components (1, or 2 for the spinor)
  int forward;                 // transform `in` along x first
  int inverse;                 // F_x^-1 before writing `out`
  int terms;
  const void* src[kIfrkMaxTerms];   // full spectra (member-major), or nullptr = this row
  double coef[kIfrkMaxTerms];       // h a_ij (1 for psi0_hat)
  int table[kIfrkMaxTerms];         // index of the separable factor table (nx + ny complex)
  long long member_stride;          // complex values per member of a spectrum
  // Spinor: the 2x2 Lawson factor exp(-i H(k) tau / hbar) is evaluated per mode from the
  // per-member constants (FP64 phase angles) instead of separable tables.
  int spinor;
  double tau[kIfrkMaxTerms];        // tau of each term
  double kx_unit, ky_unit;          // 2 pi / (n d) along x and y
  double inv_n;                     // 1 / (nx ny): normalisation of the inverse transforms
  const void* spin;                 // SpinorConst per member
  // FP32 state: per-mode table (see kSpinModeFields) and each tau as a float pair
  // tau_hi + tau_lo, so the phase angles are formed in compensated FP32 instead of FP64.
  const float* modes;
  float tau_hi[kIfrkMaxTerms], tau_lo[kIfrkMaxTerms];
};


// Per-member constants of the two-component Lawson factor (polarism/dispersion.py:34-83).
struct SpinorConst {
  double rate;      // hbar / 2m: E(k) / hbar = rate k^2
  double half_z;    // Zeeman splitting / 2 (meV)
  double beta;      // TE-TM coefficient
  double inv_hbar;
};

// Per-mode fields of the FP32 spinor table, [member][field][mode]: E(k)/hbar and w(k)/hbar as
// float pairs (hi + lo of the FP64 value), Re u and Im u of u = beta (kx - i ky)^2, and 1 / w
// (0 where w = 0).
constexpr int kSpinModeFields = 7;
cudaError_t launch_spin_mode_table(float* table, const SpinorConst* consts, int nx, int ny,
                                   int members, double kx_unit, double ky_unit, cudaStream_t stream);

// Column pass of one stage: F_y^-1 -> psi_i; n_i = n0 + sum coef_j dn_j; rhs_i; dn_i -> F_y.
struct IfrkColArgs {
  int nx, ny, log2ny, cols, log2cols, threads, members;
  int comps, log2comps;        // field components
  int res_fields;              // 0 none, 1 single, 2 active + inactive
  int res_comps;               // reservoir planes per field (1 shared or comps)
  int res_kind;                // PG_RES_*: two fields are double (2) or quadratic-double (3)
  int mode;                    // 0 stage RHS, 1 step end, 2 error norm, 3 forward only
  int inverse, forward;
  int reservoir;               // any reservoir present
  int potential;               // 0 none, 1 real, 2 complex
  int noise;                   // Wigner increment at the step end (mode 1)
  int terms;
  const void* dn[kIfrkMaxStages];   // stage reservoir derivatives
  double coef[kIfrkMaxStages];      // h a_ij (stage) or h b_j (step end) or h (b_j - bhat_j)
  long long pump_stride, pot_stride;
  int scale_index;             // pump coefficient sample of `scales` ([k][term][member])
  int pump_terms;              // separable pump terms L
  long long pump_term_stride;  // reals between consecutive terms' envelopes
  int step_offset;
  double rtol, atol;
};

template <typename T>
cudaError_t launch_ifrk_row(const T* in, T* save, T* out, const T* tables, const IfrkRowArgs& a,
                            const T* twiddle, cudaStream_t stream);

// Column pass.  psi: in/out panel array; n0/n_out/dn_out: reservoir arrays; start/extra:
// mode-dependent (step start psi for the error norm; new psi output of the step end).
template <typename T>
cudaError_t launch_ifrk_col(T* psi, const T* n0, T* dn_out, T* n_out, const T* psi_start,
                            const T* psi_new, const T* pump, const T* potential, const T* twiddle,
                            const SplitConst<T>* consts, const T* scales,
                            const unsigned long long* step_base, double* partials,
                            const IfrkColArgs& a, cudaStream_t stream);

template <typename T>
cudaError_t configure_ifrk_kernels(size_t max_smem);

}  // namespace pg
