// Definition of the opaque pg_solver handle shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <tuple>
#include <vector>

#include "pg_internal.h"

namespace pg {
constexpr int kChunk = 64;         // steps per staged chunk / CUDA graph
constexpr int kStagingSlots = 4;   // pinned staging ring depth
}  // namespace pg

struct pg_solver {
  pg_config cfg{};
  std::vector<pg_physics> physics;
  cudaStream_t stream = nullptr;
  int sm_count = 0;
  size_t real_size = 4;
  long long plane = 0;     // nx * ny
  long long sites = 0;     // members * plane
  int comps = 1;           // field components (2: circular-basis spinor)
  int res_fields = 1;      // 0 none, 1 single reservoir, 2 active + inactive
  int res_comps = 1;       // reservoir planes per field: 1 shared or = comps
  long long field_values = 0;  // complex values of the state: members * comps * plane
  long long res_values = 0;    // reals of the reservoir: res_fields * members * res_comps * plane
  void* psi[2] = {nullptr, nullptr};
  void* res[2] = {nullptr, nullptr};
  void* pump = nullptr;
  void* potential = nullptr;
  void* consts = nullptr;
  void* scales = nullptr;  // kChunk * 3 * pump_terms * members reals
  int pump_terms = 1;      // separable pump terms L
  long long pump_term_stride = 0;  // reals between consecutive terms' envelopes
  unsigned long long* step_base = nullptr;
  int cur = 0;
  bool noise = false;
  std::vector<uint64_t> seeds;
  std::vector<double> noise_gamma, noise_R, noise_strength;
  double dt_over_4dv = 0.0;
  pg::RK4Geom geom{};
  // Pinned staging ring for chunk scales and the step base.
  struct Slot {
    void* host = nullptr;
    cudaEvent_t done = nullptr;
  } staging[pg::kStagingSlots];
  int next_slot = 0;
  std::map<std::pair<int, int>, cudaGraphExec_t> graphs;  // (length, parity) -> graph
  int* err_flag = nullptr;   // set by kernels whose bounded waits gave up
  int wait_limit = 100000;   // 0: bounded waits give up at once (pg_set_wait_limit)
  // Device halt word of the steady-state monitor: once it is set every RK4 and split-step
  // launch returns at once, so steps queued after the last member stopped leave the state
  // as it was.
  int* halt = nullptr;
  long long parity_step = 0;  // absolute step whose state sits under `cur` after pg_rk4_advance
  long long flips = 0;        // swaps of `cur` by RK4 steps so far (split steps work in place)
  int rk4_kernel = 0;        // 0 auto, 1 tiled streaming kernel, 2 full-width kernel,
                             // 3 full-width kernel with four sites a thread
  int wide_blocks = 0;       // persistent grid of the full-width kernel
  int quad_blocks = 0;       // persistent grid of its four-sites-a-thread form
  // Split-step state.
  bool spectral = false;      // psi holds the unnormalised 2-D spectrum instead of psi(x, y)
  bool split_ready = false;
  void* tw_x = nullptr;       // exp(-2 pi i k / nx), k < nx
  void* tw_y = nullptr;
  void* prop = nullptr;       // [table][member][nx + ny] propagator factors
  void* tw4 = nullptr;        // FP32 1024-point four-step factors W_1024^{n2 k1} (split_fast.cu)
  void* split_consts = nullptr;
  std::map<std::tuple<int, int, int>, cudaGraphExec_t> split_graphs;  // (ordering, len, parity)
  void* ifrk = nullptr;       // IFRK stage buffers (created on first use)
  void* accum = nullptr;      // FP64 observable sums (created on first use)
  long long last_launches = 0;
  // Graph capture failures: graph_failure (a test hook) makes the next capture (1) or
  // instantiation (2) fail as a failing CUDA call would; graph_fallbacks counts the chunks
  // that ran as plain launches after a capture or instantiation failed.
  int graph_failure = 0;
  long long graph_fallbacks = 0;
  // Host waits (pg_sync_counts): host_syncs counts every wait of the library for the
  // solver's stream to drain, throttle_waits the staging-ring waits that found the slot's
  // earlier copy still queued (the host had run kStagingSlots chunks ahead of the device).
  long long host_syncs = 0;
  long long throttle_waits = 0;
};

namespace pg {
// Wait for everything queued on the solver's stream (counted in host_syncs).
inline cudaError_t stream_sync(pg_solver* s) {
  ++s->host_syncs;
  return cudaStreamSynchronize(s->stream);
}
}  // namespace pg


namespace pg {
int split_release(pg_solver* s);
int split_ensure(pg_solver* s);
void ifrk_release(pg_solver* s);
void ifrk_invalidate(pg_solver* s);
void accum_release(pg_solver* s);
int split_refresh_consts(pg_solver* s);
// Stage a chunk's per-step coefficients (per_step * members doubles per step) and the step base.
int stage_coefficients(pg_solver* s, const double* coeffs, int len, int per_step, int64_t step);
}  // namespace pg
