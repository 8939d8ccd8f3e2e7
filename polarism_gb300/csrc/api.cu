// C ABI of libpolarism_gb300: solver lifecycle, state transfer, RK4 advance with
// CUDA-graph chunks, and the Philox test hook.
//
// The advance loop mirrors polarism/solver/rk4_cuda_solver.py:3451-3642: per-stage
// pump scales for a chunk of up to 64 steps are copied to a device array and the
// global step base is set before the chunk runs (rk4_cuda_solver.py:3564-3586);
// chunks of even length keep the ping-pong buffers on the same parity.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "philox.cuh"
#include "pg_internal.h"
#include "solver.h"
#include "tma.cuh"
#include "wide_internal.h"

namespace pg {

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }
const char* last_error() { return g_last_error.c_str(); }

namespace {

__global__ void philox_words_kernel(const uint4* __restrict__ counters, uint4* __restrict__ out,
                                    uint32_t k0, uint32_t k1, long long n) {
  const long long j = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const uint4 c = counters[j];
  const Words4 w = philox4x32_10(Words4{c.x, c.y, c.z, c.w}, k0, k1);
  out[j] = make_uint4(w.a, w.b, w.c, w.d);
}

template <typename T>
__global__ void wigner_normals_kernel(const uint4* __restrict__ counters, T* __restrict__ out,
                                      uint32_t k0, uint32_t k1, long long n) {
  const long long j = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const uint4 c = counters[j];
  const Words4 w = philox4x32_10(Words4{c.x, c.y, c.z, c.w}, k0, k1);
  T re = T(0), im = T(0);
  WignerDraw<T>::apply(w, T(1), re, im);
  out[2 * j] = re;
  out[2 * j + 1] = im;
}

}  // namespace

int philox_words_device(const uint32_t* counters, uint64_t key, uint32_t* out, int64_t n,
                        cudaStream_t stream) {
  if (n <= 0) return PG_OK;
  const int threads = 256;
  const long long blocks = (n + threads - 1) / threads;
  philox_words_kernel<<<static_cast<unsigned>(blocks), threads, 0, stream>>>(
      reinterpret_cast<const uint4*>(counters), reinterpret_cast<uint4*>(out),
      static_cast<uint32_t>(key), static_cast<uint32_t>(key >> 32), n);
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

}  // namespace pg

namespace pg {

// Copy a chunk's per-step coefficients and its step base into the device arrays
// (stream ordered, through a ring of pinned staging buffers).
int stage_coefficients(pg_solver* s, const double* coeffs, int len, int per_step, int64_t step) {
  pg_solver::Slot& slot = s->staging[s->next_slot];
  s->next_slot = (s->next_slot + 1) % kStagingSlots;
  if (cudaEventQuery(slot.done) == cudaErrorNotReady) ++s->throttle_waits;
  PG_CUDA(cudaEventSynchronize(slot.done));
  const int m = s->cfg.members;
  const size_t count = static_cast<size_t>(len) * per_step * m;
  unsigned char* host = static_cast<unsigned char*>(slot.host);
  if (s->cfg.precision == PG_DOUBLE) {
    std::memcpy(host, coeffs, count * sizeof(double));
  } else {
    float* h = reinterpret_cast<float*>(host);
    for (size_t i = 0; i < count; ++i) h[i] = static_cast<float>(coeffs[i]);
  }
  const size_t bytes = count * s->real_size;
  const size_t base_off = static_cast<size_t>(kChunk) * 3 * s->pump_terms * m * 8;
  unsigned long long b = static_cast<unsigned long long>(step);
  std::memcpy(host + base_off, &b, sizeof(b));
  if (bytes) PG_CUDA(cudaMemcpyAsync(s->scales, host, bytes, cudaMemcpyHostToDevice, s->stream));
  PG_CUDA(cudaMemcpyAsync(s->step_base, host + base_off, sizeof(b), cudaMemcpyHostToDevice,
                          s->stream));
  PG_CUDA(cudaEventRecord(slot.done, s->stream));
  return PG_OK;
}

}  // namespace pg

namespace {

using pg::kChunk;
using pg::kStagingSlots;

template <typename T>
void build_consts(const pg_solver* s, std::vector<pg::RhsConst<T>>& out) {
  const pg_config& c = s->cfg;
  out.resize(c.members);
  for (int m = 0; m < c.members; ++m) {
    const pg_physics& p = s->physics[m];
    const double a = p.hbar / (2.0 * p.m_eff);
    pg::RhsConst<T>& k = out[m];
    k.ax = static_cast<T>(a / (c.dx * c.dx));
    k.ay = static_cast<T>(a / (c.dy * c.dy));
    k.w0 = static_cast<T>(2.0 * (a / (c.dx * c.dx) + a / (c.dy * c.dy)));
    k.gc = static_cast<T>(p.g_C / p.hbar);
    k.gr = static_cast<T>(p.g_R / p.hbar);
    k.gi = static_cast<T>(p.g_I / p.hbar);
    k.inv_hbar = static_cast<T>(1.0 / p.hbar);
    k.half_R = static_cast<T>(0.5 * p.R);
    k.half_gC = static_cast<T>(0.5 * p.gamma_C);
    k.R = static_cast<T>(p.R);
    k.gamma_R = static_cast<T>(p.gamma_R);
    k.eta_a = static_cast<T>(p.kinetic_relaxation_eta);
    k.pad_ = T(0);
    k.gamma_I = static_cast<T>(p.gamma_I);
    k.gamma_A = static_cast<T>(p.gamma_A);
    k.R_IA = static_cast<T>(p.R_IA);
    k.R_AI = static_cast<T>(p.R_AI);
    k.kappa = static_cast<T>(p.kappa);
    k.pad2_ = T(0);
    if (s->noise) {
      k.noise_a = static_cast<T>(s->noise_strength[m] * s->noise_gamma[m] * s->dt_over_4dv);
      k.noise_b = static_cast<T>(s->noise_strength[m] * s->noise_R[m] * s->dt_over_4dv);
      k.seed = s->seeds[m];
    } else {
      k.noise_a = k.noise_b = T(0);
      k.seed = 0ull;
    }
  }
}

int upload_consts(pg_solver* s) {
  if (s->cfg.precision == PG_DOUBLE) {
    std::vector<pg::RhsConst<double>> v;
    build_consts(s, v);
    PG_CUDA(cudaMemcpyAsync(s->consts, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice,
                            s->stream));
  } else {
    std::vector<pg::RhsConst<float>> v;
    build_consts(s, v);
    PG_CUDA(cudaMemcpyAsync(s->consts, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice,
                            s->stream));
  }
  PG_CUDA(pg::stream_sync(s));
  return PG_OK;
}

void free_graphs(pg_solver* s) {
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  s->graphs.clear();
}

pg::RK4Features features(const pg_solver* s) {
  pg::RK4Features f{};
  f.potential = s->cfg.potential;
  f.reservoir = s->cfg.reservoir;
  f.pump_terms = s->pump_terms;
  f.relax = 0;
  for (const auto& p : s->physics)
    if (p.kinetic_relaxation_eta != 0.0) f.relax = 1;
  return f;
}

// The full-width kernel takes one laser, or two on rows of at most 1024 sites (their
// envelopes stream as extra ring rows; wider rows' bands have no room for them).
bool wide_lasers_ok(int terms, int nx) { return terms == 1 || (terms == 2 && nx <= 1024); }

bool use_wide(const pg_solver* s) {
  const pg::RK4Features f = features(s);
  // FP32, single reservoir, one laser (two on rows up to 1024 sites); a potential, kinetic
  // relaxation or a second laser selects the full-width kernel's general variant.
  const bool eligible = s->cfg.precision == PG_SINGLE && f.reservoir == 1 &&
                        wide_lasers_ok(f.pump_terms, s->cfg.nx) &&
                        pg::wide_rk4_supported(s->cfg.nx, s->cfg.ny);
  if (s->rk4_kernel == 1) return false;
  return eligible;
}

// The full-width kernel's four-sites-a-thread form (kernel kind 3): rows of 512 or 1024 sites
// without a potential or relaxation.  At 1024 x 1024 x 32 with Wigner noise it measured 124.7 G
// site-updates/s against 130.8 for the two-site form (eight warps an SM leave its dependency
// chains exposed), so the two-site form is the default.
bool use_quad(const pg_solver* s, const pg::WideGeom& w) {
  return s->rk4_kernel == 3 && s->quad_blocks > 0 && !pg::wide_general(w) &&
         pg::quad_rk4_supported(s->cfg.nx, s->cfg.ny);
}

// Launch one RK4 step reading buffers of parity `from`; step_offset indexes the chunk scales.
cudaError_t launch_step(pg_solver* s, int from, int step_offset) {
  const int to = 1 - from;
  const pg::RK4Features f = features(s);
  if (use_wide(s)) {
    pg::WideGeom w{};
    w.nx = s->cfg.nx;
    w.ny = s->cfg.ny;
    w.members = s->cfg.members;
    w.blocks = s->wide_blocks;
    w.pump_stride = s->cfg.pump_per_member ? s->plane : 0;
    w.pump_terms = f.pump_terms;
    w.pump_term_stride = s->pump_term_stride;
    w.halt = s->halt;
    w.pot = static_cast<const float*>(s->potential);
    w.pot_stride = s->cfg.potential_per_member ? s->plane : 0;
    w.pot_kind = f.potential;
    w.relax = f.relax;
    w.wait_limit = s->wait_limit;
    if (use_quad(s, w)) {
      w.blocks = s->quad_blocks;
      return pg::launch_rk4_quad(static_cast<const float*>(s->psi[from]),
                                 static_cast<const float*>(s->res[from]),
                                 static_cast<const float*>(s->pump), static_cast<float*>(s->psi[to]),
                                 static_cast<float*>(s->res[to]),
                                 static_cast<const pg::RhsConst<float>*>(s->consts),
                                 static_cast<const float*>(s->scales), s->step_base, step_offset,
                                 static_cast<float>(s->cfg.dt), s->noise, w, s->err_flag, s->stream);
    }
    return pg::launch_rk4_wide(static_cast<const float*>(s->psi[from]),
                               static_cast<const float*>(s->res[from]),
                               static_cast<const float*>(s->pump), static_cast<float*>(s->psi[to]),
                               static_cast<float*>(s->res[to]),
                               static_cast<const pg::RhsConst<float>*>(s->consts),
                               static_cast<const float*>(s->scales), s->step_base, step_offset,
                               static_cast<float>(s->cfg.dt), s->noise, w, s->err_flag, s->stream);
  }
  pg::RK4Geom g = s->geom;
  g.pump_stride = s->cfg.pump_per_member ? s->plane : 0;
  g.pot_stride = s->cfg.potential_per_member ? s->plane : 0;
  g.halt = s->halt;
  g.pump_term_stride = s->pump_term_stride;
  if (s->cfg.precision == PG_DOUBLE) {
    return pg::launch_rk4_step<double>(
        static_cast<const double*>(s->psi[from]), static_cast<const double*>(s->res[from]),
        static_cast<const double*>(s->pump), static_cast<const double*>(s->potential),
        static_cast<double*>(s->psi[to]), static_cast<double*>(s->res[to]),
        static_cast<const pg::RhsConst<double>*>(s->consts), static_cast<const double*>(s->scales),
        s->step_base, step_offset, s->cfg.dt, s->noise, g, f, s->stream);
  }
  return pg::launch_rk4_step<float>(
      static_cast<const float*>(s->psi[from]), static_cast<const float*>(s->res[from]),
      static_cast<const float*>(s->pump), static_cast<const float*>(s->potential),
      static_cast<float*>(s->psi[to]), static_cast<float*>(s->res[to]),
      static_cast<const pg::RhsConst<float>*>(s->consts), static_cast<const float*>(s->scales),
      s->step_base, step_offset, static_cast<float>(s->cfg.dt), s->noise, g, f, s->stream);
}

int graph_for(pg_solver* s, int len, int parity, cudaGraphExec_t* out) {
  auto key = std::make_pair(len, parity);
  auto it = s->graphs.find(key);
  if (it != s->graphs.end()) {
    *out = it->second;
    return PG_OK;
  }
  const int forced = s->graph_failure;  // test hook: fail as the real call would
  s->graph_failure = 0;
  cudaGraph_t graph = nullptr;
  PG_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t launch_err = cudaSuccess;
  for (int k = 0; k < len && launch_err == cudaSuccess; ++k)
    launch_err = launch_step(s, (parity + k) & 1, k);
  cudaError_t end_err = cudaStreamEndCapture(s->stream, &graph);
  if (forced == 1 && end_err == cudaSuccess) end_err = cudaErrorStreamCaptureInvalidated;
  if (launch_err != cudaSuccess || end_err != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    pg::set_error(std::string("graph capture failed: ") +
                  cudaGetErrorString(launch_err != cudaSuccess ? launch_err : end_err));
    return PG_ERR_CUDA;
  }
  cudaGraphExec_t exec = nullptr;
  cudaError_t inst = forced == 2 ? cudaErrorInvalidValue : cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (inst != cudaSuccess) {
    pg::set_error(std::string("graph instantiate failed: ") + cudaGetErrorString(inst));
    return PG_ERR_CUDA;
  }
  s->graphs[key] = exec;
  *out = exec;
  return PG_OK;
}

void release(pg_solver* s) {
  if (!s) return;
  free_graphs(s);
  pg::split_release(s);
  pg::ifrk_release(s);
  pg::accum_release(s);
  for (auto& slot : s->staging) {
    if (slot.host) cudaFreeHost(slot.host);
    if (slot.done) cudaEventDestroy(slot.done);
  }
  for (int i = 0; i < 2; ++i) {
    cudaFree(s->psi[i]);
    cudaFree(s->res[i]);
  }
  cudaFree(s->pump);
  cudaFree(s->potential);
  cudaFree(s->consts);
  cudaFree(s->scales);
  cudaFree(s->step_base);
  cudaFree(s->err_flag);
  cudaFree(s->halt);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

}  // namespace

extern "C" {

const char* pg_last_error(void) { return pg::last_error(); }

int pg_version(void) { return 1; }

int pg_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int pg_create(const pg_config* cfg, const pg_physics* physics, pg_solver** out) {
  PG_CHECK(cfg && physics && out, PG_ERR_INVALID, "pg_create: null argument");
  PG_CHECK(cfg->nx >= 4 && cfg->ny >= 4, PG_ERR_INVALID, "pg_create: grid must be at least 4x4");
  PG_CHECK(cfg->members >= 1, PG_ERR_INVALID, "pg_create: members must be >= 1");
  PG_CHECK(cfg->precision == PG_SINGLE || cfg->precision == PG_DOUBLE, PG_ERR_INVALID,
           "pg_create: precision must be PG_SINGLE or PG_DOUBLE");
  PG_CHECK(cfg->reservoir >= PG_RES_NONE && cfg->reservoir <= PG_RES_QDOUBLE, PG_ERR_UNSUPPORTED,
           "pg_create: reservoir must be PG_RES_NONE, PG_RES_SINGLE, PG_RES_DOUBLE or PG_RES_QDOUBLE");
  PG_CHECK(cfg->pump_terms >= 0 && cfg->pump_terms <= 16, PG_ERR_INVALID,
           "pg_create: pump_terms must be between 1 and 16 (0 means 1)");
  PG_CHECK(cfg->components >= 0 && cfg->components <= 2, PG_ERR_INVALID,
           "pg_create: components must be 1 or 2");
  const int comps = cfg->components == 0 ? 1 : cfg->components;
  const int res_comps = cfg->reservoir_components == 0 ? comps : cfg->reservoir_components;
  PG_CHECK(res_comps == 1 || res_comps == comps, PG_ERR_INVALID,
           "pg_create: reservoir_components must be 1 or equal to components");
  PG_CHECK(cfg->potential >= PG_POT_NONE && cfg->potential <= PG_POT_COMPLEX, PG_ERR_INVALID,
           "pg_create: bad potential kind");
  PG_CHECK(cfg->dx > 0 && cfg->dy > 0 && cfg->dt > 0, PG_ERR_INVALID,
           "pg_create: dx, dy and dt must be positive");
  PG_CHECK(static_cast<long long>(cfg->nx) * cfg->ny < (1ll << 31), PG_ERR_INVALID,
           "pg_create: one member must hold fewer than 2^31 sites");
  *out = nullptr;
  pg_solver* s = new pg_solver();
  s->cfg = *cfg;
  s->physics.assign(physics, physics + cfg->members);
  s->real_size = cfg->precision == PG_DOUBLE ? 8 : 4;
  s->plane = static_cast<long long>(cfg->nx) * cfg->ny;
  s->sites = s->plane * cfg->members;
  s->comps = comps;
  s->res_fields = cfg->reservoir >= PG_RES_DOUBLE ? 2 : cfg->reservoir;
  s->res_comps = res_comps;
  s->field_values = s->sites * comps;
  s->pump_terms = cfg->pump_terms <= 0 ? 1 : cfg->pump_terms;
  s->pump_term_stride = cfg->pump_per_member ? s->sites : s->plane;
  s->res_values = s->sites * s->res_fields * res_comps;
  int dev = 0;
  auto fail = [&](cudaError_t e, const char* what) {
    pg::set_error(std::string("pg_create: ") + what + ": " + cudaGetErrorString(e));
    release(s);
    return PG_ERR_CUDA;
  };
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(e, "cudaGetDevice");
  e = cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return fail(e, "device attribute");
  e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(e, "stream");
  const size_t field_bytes = static_cast<size_t>(s->field_values) * 2 * s->real_size;
  const size_t res_bytes = static_cast<size_t>(std::max<long long>(1, s->res_values)) * s->real_size;
  for (int i = 0; i < 2; ++i) {
    if ((e = cudaMalloc(&s->psi[i], field_bytes)) != cudaSuccess) return fail(e, "psi buffers");
    if ((e = cudaMalloc(&s->res[i], res_bytes)) != cudaSuccess) return fail(e, "reservoir buffers");
    cudaMemsetAsync(s->psi[i], 0, field_bytes, s->stream);
    cudaMemsetAsync(s->res[i], 0, res_bytes, s->stream);
  }
  const size_t pump_bytes = static_cast<size_t>(s->pump_term_stride) * s->pump_terms * s->real_size;
  if ((e = cudaMalloc(&s->pump, pump_bytes)) != cudaSuccess) return fail(e, "pump buffer");
  cudaMemsetAsync(s->pump, 0, pump_bytes, s->stream);
  if (cfg->potential != PG_POT_NONE) {
    const size_t pot_bytes = static_cast<size_t>(cfg->potential_per_member ? s->sites : s->plane) *
                             s->real_size * (cfg->potential == PG_POT_COMPLEX ? 2 : 1);
    if ((e = cudaMalloc(&s->potential, pot_bytes)) != cudaSuccess) return fail(e, "potential buffer");
    cudaMemsetAsync(s->potential, 0, pot_bytes, s->stream);
  }
  const size_t const_bytes = static_cast<size_t>(cfg->members) *
                             (cfg->precision == PG_DOUBLE ? sizeof(pg::RhsConst<double>)
                                                          : sizeof(pg::RhsConst<float>));
  if ((e = cudaMalloc(&s->consts, const_bytes)) != cudaSuccess) return fail(e, "constants");
  const size_t scale_bytes =
      static_cast<size_t>(kChunk) * 3 * s->pump_terms * cfg->members * s->real_size;
  if ((e = cudaMalloc(&s->scales, scale_bytes)) != cudaSuccess) return fail(e, "scales");
  if ((e = cudaMalloc(&s->step_base, sizeof(unsigned long long))) != cudaSuccess)
    return fail(e, "step base");
  cudaMemsetAsync(s->step_base, 0, sizeof(unsigned long long), s->stream);
  if ((e = cudaMalloc(&s->err_flag, sizeof(int))) != cudaSuccess) return fail(e, "error flag");
  cudaMemsetAsync(s->err_flag, 0, sizeof(int), s->stream);
  if ((e = cudaMalloc(&s->halt, sizeof(int))) != cudaSuccess) return fail(e, "halt word");
  cudaMemsetAsync(s->halt, 0, sizeof(int), s->stream);
  if (cfg->precision == PG_SINGLE && pg::wide_rk4_supported(cfg->nx, cfg->ny)) {
    if ((e = pg::configure_wide_rk4()) != cudaSuccess) return fail(e, "wide kernel attributes");
    s->wide_blocks = pg::wide_rk4_grid(cfg->nx, cfg->ny, cfg->members, s->sm_count,
                                       s->pump_terms == 2 && cfg->nx <= 1024 ? 2 : 1);
    if (pg::quad_rk4_supported(cfg->nx, cfg->ny)) {
      if ((e = pg::configure_quad_rk4()) != cudaSuccess) return fail(e, "quad kernel attributes");
      s->quad_blocks = pg::quad_rk4_grid(cfg->nx, cfg->ny, cfg->members, s->sm_count);
    }
  }
  const size_t staging_bytes = static_cast<size_t>(kChunk) * 3 * s->pump_terms * cfg->members * 8 + 64;
  for (auto& slot : s->staging) {
    if ((e = cudaMallocHost(&slot.host, staging_bytes)) != cudaSuccess) return fail(e, "staging");
    if ((e = cudaEventCreateWithFlags(&slot.done, cudaEventDisableTiming)) != cudaSuccess)
      return fail(e, "staging event");
  }
  pg::choose_rk4_geometry(cfg->nx, cfg->ny, cfg->members, cfg->precision, s->sm_count, &s->geom);
  int rc = upload_consts(s);
  if (rc != PG_OK) {
    release(s);
    return rc;
  }
  *out = s;
  return PG_OK;
}

void pg_destroy(pg_solver* s) {
  if (s && s->stream) pg::stream_sync(s);
  release(s);
}

void* pg_stream(pg_solver* s) { return s ? static_cast<void*>(s->stream) : nullptr; }

namespace {
// Read (and clear) the device error flag after a synchronisation point.
int check_device_flag(pg_solver* s) {
  int flag = 0;
  PG_CUDA(cudaMemcpyAsync(&flag, s->err_flag, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  PG_CUDA(pg::stream_sync(s));
  if (flag) {
    cudaMemsetAsync(s->err_flag, 0, sizeof(int), s->stream);
    pg::stream_sync(s);
    pg::set_error("a bounded device wait timed out; results of the last advance are invalid");
    return PG_ERR_TIMEOUT;
  }
  return PG_OK;
}
}  // namespace

int pg_synchronize(pg_solver* s) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_synchronize: null solver");
  PG_CUDA(pg::stream_sync(s));
  return check_device_flag(s);
}

int pg_set_state(pg_solver* s, const void* psi, const void* res, int on_device) {
  PG_CHECK(s && psi, PG_ERR_INVALID, "pg_set_state: null argument");
  PG_CHECK(s->cfg.reservoir == PG_RES_NONE || res, PG_ERR_INVALID,
           "pg_set_state: reservoir array required");
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  pg::ifrk_invalidate(s);
  PG_CUDA(cudaMemcpyAsync(s->psi[s->cur], psi, static_cast<size_t>(s->field_values) * 2 * s->real_size,
                          kind, s->stream));
  if (s->cfg.reservoir != PG_RES_NONE)
    PG_CUDA(cudaMemcpyAsync(s->res[s->cur], res, static_cast<size_t>(s->res_values) * s->real_size,
                            kind, s->stream));
  PG_CUDA(pg::stream_sync(s));
  return PG_OK;
}

int pg_get_state(pg_solver* s, void* psi, void* res, int on_device) {
  PG_CHECK(s && psi, PG_ERR_INVALID, "pg_get_state: null argument");
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  PG_CUDA(cudaMemcpyAsync(psi, s->psi[s->cur], static_cast<size_t>(s->field_values) * 2 * s->real_size,
                          kind, s->stream));
  if (res && s->cfg.reservoir != PG_RES_NONE)
    PG_CUDA(cudaMemcpyAsync(res, s->res[s->cur], static_cast<size_t>(s->res_values) * s->real_size,
                            kind, s->stream));
  PG_CUDA(pg::stream_sync(s));
  return check_device_flag(s);
}

int pg_rk4_set_kernel(pg_solver* s, int32_t kind) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_rk4_set_kernel: null solver");
  PG_CHECK(kind >= 0 && kind <= 3, PG_ERR_INVALID,
           "pg_rk4_set_kernel: kind must be 0, 1, 2 or 3");
  if (kind == 3)
    PG_CHECK(pg::quad_rk4_supported(s->cfg.nx, s->cfg.ny) && s->cfg.potential == PG_POT_NONE,
             PG_ERR_UNSUPPORTED,
             "pg_rk4_set_kernel: the four-sites-a-thread form needs nx in {512, 1024} and no "
             "potential");
  if (kind >= 2) {
    const pg::RK4Features f = features(s);
    PG_CHECK(s->cfg.precision == PG_SINGLE && f.reservoir == 1 &&
                 wide_lasers_ok(f.pump_terms, s->cfg.nx) && (kind == 2 || f.pump_terms == 1) &&
                 pg::wide_rk4_supported(s->cfg.nx, s->cfg.ny),
             PG_ERR_UNSUPPORTED,
             "pg_rk4_set_kernel: the full-width kernel needs FP32, a single reservoir, one laser "
             "(two on rows of at most 1024 sites) and nx in {128, 256, 512, 1024} or a multiple "
             "of 1024 up to 16384");
  }
  s->rk4_kernel = kind;
  free_graphs(s);
  return PG_OK;
}

int pg_set_wait_limit(pg_solver* s, int32_t polls) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_set_wait_limit: null solver");
  PG_CHECK(polls == 0 || polls == pg::kWaitPolls, PG_ERR_INVALID,
           "pg_set_wait_limit: polls must be 0 (the give-up setting: every wait gives up at once) "
           "or 100000 (the kernels' compiled bound)");
  PG_CUDA(pg::stream_sync(s));
  s->wait_limit = polls;
  free_graphs(s);  // captured launches carry the old limit
  return PG_OK;
}

int pg_test_fail_next_graph(pg_solver* s, int32_t what) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_test_fail_next_graph: null solver");
  PG_CHECK(what >= 0 && what <= 2, PG_ERR_INVALID,
           "pg_test_fail_next_graph: 0 (none), 1 (capture) or 2 (instantiation)");
  s->graph_failure = what;
  free_graphs(s);  // the next chunk must capture anew
  return PG_OK;
}

int64_t pg_graph_fallbacks(pg_solver* s) { return s ? s->graph_fallbacks : -1; }

int pg_sync_counts(pg_solver* s, int64_t* host_syncs, int64_t* throttle_waits) {
  PG_CHECK(s && host_syncs && throttle_waits, PG_ERR_INVALID, "pg_sync_counts: null argument");
  *host_syncs = s->host_syncs;
  *throttle_waits = s->throttle_waits;
  return PG_OK;
}

int pg_rk4_prepare(pg_solver* s, int32_t n_steps) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_rk4_prepare: null solver");
  PG_CHECK(n_steps >= 0, PG_ERR_INVALID, "pg_rk4_prepare: negative step count");
  // The chunks pg_rk4_advance would cut n_steps into (graphs of even length up to kChunk; a
  // chunk keeps the buffer parity), for either starting parity.
  int done = 0;
  while (done < n_steps) {
    int len = std::min(kChunk, n_steps - done);
    if (len >= 2 && (len & 1)) len -= 1;
    if (len >= 2) {
      for (int parity = 0; parity < 2; ++parity) {
        cudaGraphExec_t exec = nullptr;
        const int rc = graph_for(s, len, parity, &exec);
        if (rc != PG_OK) return rc;
      }
    }
    done += len;
  }
  return PG_OK;
}

int pg_rk4_get_kernel(pg_solver* s, int32_t* kind) {
  PG_CHECK(s && kind, PG_ERR_INVALID, "pg_rk4_get_kernel: null argument");
  *kind = !use_wide(s) ? 1 : s->rk4_kernel == 3 ? 3 : 2;
  return PG_OK;
}

int pg_state_pointers(pg_solver* s, void** psi, void** res) {
  PG_CHECK(s && psi && res, PG_ERR_INVALID, "pg_state_pointers: null argument");
  *psi = s->psi[s->cur];
  *res = s->cfg.reservoir != PG_RES_NONE ? s->res[s->cur] : nullptr;
  return PG_OK;
}

int pg_set_pump(pg_solver* s, const void* envelope, int on_device) {
  PG_CHECK(s && envelope, PG_ERR_INVALID, "pg_set_pump: null argument");
  const size_t bytes = static_cast<size_t>(s->pump_term_stride) * s->pump_terms * s->real_size;
  PG_CUDA(cudaMemcpyAsync(s->pump, envelope, bytes,
                          on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s->stream));
  PG_CUDA(pg::stream_sync(s));
  return PG_OK;
}

int pg_set_potential(pg_solver* s, const void* potential, int on_device) {
  PG_CHECK(s && potential, PG_ERR_INVALID, "pg_set_potential: null argument");
  PG_CHECK(s->cfg.potential != PG_POT_NONE, PG_ERR_INVALID,
           "pg_set_potential: solver was created without a potential");
  const size_t bytes = static_cast<size_t>(s->cfg.potential_per_member ? s->sites : s->plane) *
                       s->real_size * (s->cfg.potential == PG_POT_COMPLEX ? 2 : 1);
  PG_CUDA(cudaMemcpyAsync(s->potential, potential, bytes,
                          on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s->stream));
  PG_CUDA(pg::stream_sync(s));
  return PG_OK;
}

int pg_set_noise(pg_solver* s, const uint64_t* seeds, const double* gamma, const double* scattering,
                 const double* strength, double dt_over_4dv) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_set_noise: null solver");
  if (!seeds) {
    s->noise = false;
  } else {
    PG_CHECK(gamma && scattering && strength, PG_ERR_INVALID, "pg_set_noise: null member arrays");
    const int m = s->cfg.members;
    s->seeds.assign(seeds, seeds + m);
    s->noise_gamma.assign(gamma, gamma + m);
    s->noise_R.assign(scattering, scattering + m);
    s->noise_strength.assign(strength, strength + m);
    s->dt_over_4dv = dt_over_4dv;
    s->noise = true;
  }
  free_graphs(s);
  int rc = upload_consts(s);
  if (rc != PG_OK) return rc;
  return s->split_ready ? pg::split_refresh_consts(s) : PG_OK;
}

int pg_rk4_set_geometry(pg_solver* s, int32_t tile_w, int32_t strip_h) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_rk4_set_geometry: null solver");
  PG_CHECK(strip_h >= 4 && strip_h % 4 == 0, PG_ERR_INVALID,
           "pg_rk4_set_geometry: strip height must be a positive multiple of 4");
  const int max_threads = s->cfg.precision == PG_DOUBLE ? 288 : 544;
  const int nx = s->cfg.nx;
  if (tile_w >= nx) {
    PG_CHECK(((nx + 31) / 32) * 32 <= max_threads, PG_ERR_INVALID,
             "pg_rk4_set_geometry: row too wide for a full-width block");
    s->geom.wrap = 1;
    s->geom.tile_w = nx;
  } else {
    PG_CHECK(tile_w >= 8 && ((tile_w + 8 + 31) / 32) * 32 <= max_threads, PG_ERR_INVALID,
             "pg_rk4_set_geometry: tile width out of range");
    s->geom.wrap = 0;
    s->geom.tile_w = tile_w;
  }
  s->geom.strip_h = strip_h;
  free_graphs(s);
  return PG_OK;
}

int pg_rk4_get_geometry(pg_solver* s, int32_t* tile_w, int32_t* strip_h) {
  PG_CHECK(s && tile_w && strip_h, PG_ERR_INVALID, "pg_rk4_get_geometry: null argument");
  *tile_w = s->geom.tile_w;
  *strip_h = s->geom.strip_h;
  return PG_OK;
}

int pg_rk4_advance(pg_solver* s, int64_t start_step, int32_t n_steps, const double* stage_scales,
                   int use_graphs) {
  PG_CHECK(s && stage_scales, PG_ERR_INVALID, "pg_rk4_advance: null argument");
  PG_CHECK(n_steps >= 0, PG_ERR_INVALID, "pg_rk4_advance: negative step count");
  PG_CHECK(!s->spectral, PG_ERR_INVALID,
           "pg_rk4_advance: the state holds a spectrum; set real-space psi first");
  PG_CHECK(s->comps == 1, PG_ERR_UNSUPPORTED,
           "pg_rk4_advance: two-component fields run on the IFRK path");
  PG_CHECK(s->res_comps == 1, PG_ERR_UNSUPPORTED,
           "pg_rk4_advance: one reservoir plane per field");
  s->last_launches = 0;
  pg::ifrk_invalidate(s);
  const int m = s->cfg.members;
  int done = 0;
  while (done < n_steps) {
    const int remaining = n_steps - done;
    int len = std::min(kChunk, remaining);
    const bool graph = use_graphs && len >= 2;
    if (graph && (len & 1)) len -= 1;
    int rc = pg::stage_coefficients(s, stage_scales + static_cast<size_t>(done) * 3 * s->pump_terms * m, len,
                                    3 * s->pump_terms,
                                    start_step + done);
    if (rc != PG_OK) return rc;
    cudaGraphExec_t exec = nullptr;
    // A chunk whose graph cannot be captured or instantiated runs as plain launches: capture
    // only records (nothing of the chunk has run), so the state buffers are as before it, the
    // role of the reference's pre-chunk copy and restore (rk4_cuda_solver.py:3591-3602).
    if (graph && graph_for(s, len, s->cur, &exec) != PG_OK) {
      cudaGetLastError();
      ++s->graph_fallbacks;
      exec = nullptr;
    }
    if (exec != nullptr) {
      PG_CUDA(cudaGraphLaunch(exec, s->stream));
      s->cur = (s->cur + len) & 1;
      s->flips += len;
    } else {
      for (int k = 0; k < len; ++k) {
        PG_CUDA(launch_step(s, s->cur, k));
        s->cur ^= 1;
        ++s->flips;
      }
    }
    s->last_launches += len;
    done += len;
  }
  s->parity_step = start_step + n_steps;
  return PG_OK;
}

int64_t pg_last_launch_count(pg_solver* s) { return s ? s->last_launches : -1; }

int pg_wigner_normals(const uint32_t* counters, uint64_t key, int32_t precision, void* out,
                      int64_t n) {
  PG_CHECK(counters && out && n >= 0, PG_ERR_INVALID, "pg_wigner_normals: bad argument");
  PG_CHECK(precision == PG_SINGLE || precision == PG_DOUBLE, PG_ERR_INVALID,
           "pg_wigner_normals: bad precision");
  if (n == 0) return PG_OK;
  const size_t esize = precision == PG_DOUBLE ? 8 : 4;
  void* dc = nullptr;
  void* dout = nullptr;
  PG_CUDA(cudaMalloc(&dc, static_cast<size_t>(n) * 16));
  cudaError_t e = cudaMalloc(&dout, static_cast<size_t>(n) * 2 * esize);
  if (e == cudaSuccess) e = cudaMemcpy(dc, counters, static_cast<size_t>(n) * 16, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    const int threads = 256;
    const unsigned blocks = static_cast<unsigned>((n + threads - 1) / threads);
    if (precision == PG_DOUBLE)
      pg::wigner_normals_kernel<double><<<blocks, threads>>>(
          static_cast<const uint4*>(dc), static_cast<double*>(dout), static_cast<uint32_t>(key),
          static_cast<uint32_t>(key >> 32), n);
    else
      pg::wigner_normals_kernel<float><<<blocks, threads>>>(
          static_cast<const uint4*>(dc), static_cast<float*>(dout), static_cast<uint32_t>(key),
          static_cast<uint32_t>(key >> 32), n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, dout, static_cast<size_t>(n) * 2 * esize, cudaMemcpyDeviceToHost);
  cudaFree(dc);
  cudaFree(dout);
  if (e != cudaSuccess) {
    pg::set_error(std::string("pg_wigner_normals: ") + cudaGetErrorString(e));
    return PG_ERR_CUDA;
  }
  return PG_OK;
}

int pg_philox_words(const uint32_t* counters, uint64_t key, uint32_t* out, int64_t n) {
  PG_CHECK(counters && out && n >= 0, PG_ERR_INVALID, "pg_philox_words: bad argument");
  if (n == 0) return PG_OK;
  void* dc = nullptr;
  void* dout = nullptr;
  const size_t bytes = static_cast<size_t>(n) * 16;
  PG_CUDA(cudaMalloc(&dc, bytes));
  cudaError_t e = cudaMalloc(&dout, bytes);
  if (e != cudaSuccess) {
    cudaFree(dc);
    pg::set_error(std::string("pg_philox_words: ") + cudaGetErrorString(e));
    return PG_ERR_CUDA;
  }
  int rc = PG_OK;
  if ((e = cudaMemcpy(dc, counters, bytes, cudaMemcpyHostToDevice)) != cudaSuccess) {
    pg::set_error(std::string("pg_philox_words: ") + cudaGetErrorString(e));
    rc = PG_ERR_CUDA;
  }
  if (rc == PG_OK) rc = pg::philox_words_device(static_cast<const uint32_t*>(dc), key,
                                                static_cast<uint32_t*>(dout), n, nullptr);
  if (rc == PG_OK && (e = cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost)) != cudaSuccess) {
    pg::set_error(std::string("pg_philox_words: ") + cudaGetErrorString(e));
    rc = PG_ERR_CUDA;
  }
  cudaFree(dc);
  cudaFree(dout);
  return rc;
}

}  // extern "C"
