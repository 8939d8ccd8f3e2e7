// The device-resident steady-state monitor shared by the solver handle and the sweep handle.
//
// One check compares the density with the previous check's (partial sums made by the
// caller's kernel: sum (rho - rho_old)^2, sum rho_old^2, sum rho per member and block) and
// decides in a one-block kernel, as polarism/simulation_controller.py:710-734 does on the
// host: relative density and norm changes, the criterion norm < 1e-30 or both below rtol,
// the first stop step of each member (_record_stops, :698-708).  The kernel publishes
// (update index, members stopped) in a 64-bit word of mapped host memory, which the host
// reads without waiting, and, when asked, sets the caller's halt word once every member has
// stopped, recording the check's step and the caller's buffer-swap count at that check.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace pg {

struct SteadyMonitor {
  int members = 0;
  double* norm_old = nullptr;        // device, members
  long long* stop_step = nullptr;    // device, members (-1: not stopped)
  double* results = nullptr;         // device, 3 * members: rel_density | rel_norm | norm
  long long* halt_step = nullptr;    // device: [step, swaps] of the halting check
  unsigned long long* host_word = nullptr;  // mapped host memory: (update index << 32) | stopped
  unsigned long long* dev_word = nullptr;   // its device alias
  unsigned int updates = 0;          // checks queued (never reset: the progress word's index)
  unsigned int reset_base = 0;       // updates at the last reset
  bool have_old = false;             // a previous check's density is held
};

// Buffers for `members` (once; a no-op when they exist).
cudaError_t steady_monitor_alloc(SteadyMonitor& mon, int members);
void steady_monitor_free(SteadyMonitor& mon);

// Stream ordered, without a host wait: checks of an earlier run still queued finish before
// these writes, and the progress words they publish carry update indices at or below
// reset_base, which steady_monitor_poll reads as "no check finished yet".  Clears `halt`.
cudaError_t steady_monitor_reset(SteadyMonitor& mon, int* halt, cudaStream_t stream);

// Queue the decision of one check from partials[(member * blocks + block) * 3 + q]; the cell
// area is cells[member] when cells is non-null, else `cell`.  Returns at once when `halt` is
// already set.
cudaError_t steady_monitor_decide(SteadyMonitor& mon, const double* partials, int blocks,
                                  const double* cells, double cell, int record, double rtol,
                                  long long step, long long swaps, int halt_when_all, int* halt,
                                  cudaStream_t stream);

// Members stopped and checks finished since the last reset, read without waiting.
void steady_monitor_poll(const SteadyMonitor& mon, int32_t* stopped, int64_t* updates_done);

// Queue copies of the results, stop steps, halt word and halt record into host memory
// (results: 3 * members doubles; stops: members; halt_record: 2).  The caller waits.
cudaError_t steady_monitor_fetch(const SteadyMonitor& mon, const int* halt, double* results,
                                 long long* stops, int* halted, long long* halt_record,
                                 cudaStream_t stream);

}  // namespace pg
