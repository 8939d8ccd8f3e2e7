// Internal declarations of the full-width FP32 RK4 kernel.
#pragma once
#include <cuda_runtime.h>

#include "pg_internal.h"

namespace pg {

struct WideGeom {
  int nx, ny, members;
  int blocks;              // persistent grid size
  long long pump_stride;   // 0: shared envelope; nx*ny: one per member
  int pump_terms = 1;      // separable lasers: 1, or 2 on rows of at most 1024 sites
  long long pump_term_stride = 0;  // reals between consecutive lasers' envelopes
  const int* halt = nullptr;  // when non-null and set, the launch returns at once
  // General variant: potential (0 none, 1 real, 2 complex; shared or per member) and the
  // kinetic-relaxation term.
  const float* pot = nullptr;
  long long pot_stride = 0;
  int pot_kind = 0;
  int relax = 0;
  // 0: the give-up setting (each block's first row copy is withheld, so its waits run out);
  // otherwise the normal path.  Every wait polls up to kWaitPolls (tma.cuh).
  int wait_limit = 100000;
};

bool wide_rk4_supported(int nx, int ny);
size_t wide_rk4_smem(int nx);
cudaError_t configure_wide_rk4();
// Grid of the full-width kernel for this shape: persistent blocks (or, for rows of 2048 to
// 8192 sites, whole clusters of nx / 1024 CTAs), at least 16 rows of work each.
int wide_rk4_grid(int nx, int ny, int members, int sm_count, int terms = 1);
cudaError_t launch_rk4_wide(const float* psi_in, const float* n_in, const float* pump,
                            float* psi_out, float* n_out, const RhsConst<float>* consts,
                            const float* scales, const unsigned long long* step_base,
                            int step_offset, float dt, bool noise, const WideGeom& g,
                            int* err_flag, cudaStream_t stream);
// Four sites a thread (rk4_quad.cu): rows of 512 or 1024 sites without a potential or
// kinetic relaxation; bitwise the same results as launch_rk4_wide.
bool quad_rk4_supported(int nx, int ny);
cudaError_t configure_quad_rk4();
int quad_rk4_grid(int nx, int ny, int members, int sm_count);
cudaError_t launch_rk4_quad(const float* psi_in, const float* n_in, const float* pump,
                            float* psi_out, float* n_out, const RhsConst<float>* consts,
                            const float* scales, const unsigned long long* step_base,
                            int step_offset, float dt, bool noise, const WideGeom& g,
                            int* err_flag, cudaStream_t stream);
// The general variant runs when the geometry asks for a potential or kinetic relaxation.
inline bool wide_general(const WideGeom& g) { return g.pot_kind != 0 || g.relax != 0; }

}  // namespace pg
