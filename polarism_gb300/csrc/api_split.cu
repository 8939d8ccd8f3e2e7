// Host sequencing of the split-step orderings on top of the Stockham passes (split.cu).
//
// K-outer ordering (split-step-fft-cuda; polarism/solver/split_step_fft_cuda_solver.py:
// 1144-1325): the spectrum is kept between steps; per step one column pass does
// F_y^-1, the local step R(dt/2) N(dt) R(dt/2) with the Wigner increment, and F_y, and
// one row pass does F_x, the full kinetic factor / N and F_x^-1.  The half kick at
// entry and exit of an advance is folded into the first and last row passes.
//
// CPU ordering (split-step-fft; polarism/solver/split_step_fft_solver.py:97-159):
// R/2 K/2 N K/2 R/2 with psi in real space at step boundaries; the reservoir half
// steps ending one step and starting the next are fused into one column pass.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "pg_internal.h"
#include "solver.h"
#include "split_internal.h"

namespace pg {
namespace {

constexpr double kPi = 3.141592653589793238462643383279502884;

enum PropTable { PROP_HALF_N = 0, PROP_FULL_N = 1, PROP_EXIT = 2, PROP_COUNT = 3 };

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
int ilog2(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return l;
}

double fft_wavenumber(int j, int n, double d) {
  const int k = j < (n + 1) / 2 ? j : j - n;  // numpy.fft.fftfreq ordering
  return 2.0 * kPi * static_cast<double>(k) / (static_cast<double>(n) * d);
}

template <typename T>
int setup_tables(pg_solver* s) {
  const pg_config& c = s->cfg;
  const int nx = c.nx, ny = c.ny, m = c.members;
  // Twiddles w_N^k = exp(-2 pi i k / N), computed in double precision.  FP32 tables hold a
  // second block of N values after the first: the remainder w - round(w), so that the
  // split-step passes multiply by hi + lo.  A rounded table alone misses |w| = 1 by ~3e-8
  // with a non-zero mean; applied ~15 times a site and step, always with the same rounding,
  // that bias drifts the norm by ~1e-4 over 1000 steps.  Other passes read the first block.
  const int tw_blocks = sizeof(T) == 4 ? 2 : 1;
  std::vector<T> twx(2 * nx * tw_blocks), twy(2 * ny * tw_blocks);
  auto fill_twiddles = [&](std::vector<T>& tw, int n) {
    for (int k = 0; k < n; ++k) {
      const double a = -2.0 * kPi * k / n;
      const double cr = std::cos(a), ci = std::sin(a);
      tw[2 * k] = static_cast<T>(cr);
      tw[2 * k + 1] = static_cast<T>(ci);
      if (tw_blocks == 2) {
        tw[2 * (n + k)] = static_cast<T>(cr - static_cast<double>(tw[2 * k]));
        tw[2 * (n + k) + 1] = static_cast<T>(ci - static_cast<double>(tw[2 * k + 1]));
      }
    }
  };
  fill_twiddles(twx, nx);
  fill_twiddles(twy, ny);
  // Separable propagators exp(-i hbar k^2 tau / 2m) = (1 + dx[j]) (1 + dy[i]), stored as the
  // differences d = exp(-i theta) - 1 = (-2 sin^2(theta / 2), -sin theta), which keep their
  // relative precision at small theta (a rounded exp(-i theta) there has |f| > 1: its cosine
  // rounds to 1).  The power-of-two scale of each table is applied apart (RowPassArgs::scale).
  const size_t per = static_cast<size_t>(nx + ny);
  std::vector<T> prop(static_cast<size_t>(PROP_COUNT) * m * per * 2);
  for (int table = 0; table < PROP_COUNT; ++table) {
    for (int mm = 0; mm < m; ++mm) {
      const pg_physics& p = s->physics[mm];
      // The last row pass left F_x^-1 (Psi full / N); F_x of it is nx Psi full / N, so
      // ny conj(half) turns it into Psi half.
      const double tau = table == PROP_HALF_N ? 0.5 * c.dt : table == PROP_FULL_N ? c.dt : -0.5 * c.dt;
      const double cf = p.hbar * tau / (2.0 * p.m_eff);
      T* base = prop.data() + ((static_cast<size_t>(table) * m + mm) * per) * 2;
      auto store = [&](int idx, double k) {
        const double theta = cf * k * k;
        const double sh = std::sin(0.5 * theta);
        base[2 * idx] = static_cast<T>(-2.0 * sh * sh);
        base[2 * idx + 1] = static_cast<T>(-std::sin(theta));
      };
      for (int j = 0; j < nx; ++j) store(j, fft_wavenumber(j, nx, c.dx));
      for (int i = 0; i < ny; ++i) store(nx + i, fft_wavenumber(i, ny, c.dy));
    }
  }
  PG_CUDA(cudaMalloc(&s->tw_x, twx.size() * sizeof(T)));
  PG_CUDA(cudaMalloc(&s->tw_y, twy.size() * sizeof(T)));
  PG_CUDA(cudaMalloc(&s->prop, prop.size() * sizeof(T)));
  PG_CUDA(cudaMalloc(&s->split_consts, static_cast<size_t>(m) * sizeof(SplitConst<T>)));
  PG_CUDA(cudaMemcpyAsync(s->tw_x, twx.data(), twx.size() * sizeof(T), cudaMemcpyHostToDevice,
                          s->stream));
  PG_CUDA(cudaMemcpyAsync(s->tw_y, twy.data(), twy.size() * sizeof(T), cudaMemcpyHostToDevice,
                          s->stream));
  PG_CUDA(cudaMemcpyAsync(s->prop, prop.data(), prop.size() * sizeof(T), cudaMemcpyHostToDevice,
                          s->stream));
  PG_CUDA(configure_split_kernels<T>(200 * 1024));
  if (sizeof(T) == 4 && (split_fast_row(nx, ny) || split_fast_col(nx, ny))) {
    std::vector<float> tw4(4 * 1024);
    split_fast_twiddles(tw4.data());
    PG_CUDA(cudaMalloc(&s->tw4, tw4.size() * sizeof(float)));
    PG_CUDA(cudaMemcpyAsync(s->tw4, tw4.data(), tw4.size() * sizeof(float), cudaMemcpyHostToDevice,
                            s->stream));
    PG_CUDA(configure_split_fast());
    PG_CUDA(pg::stream_sync(s));  // the host tables go out of scope
  }
  PG_CUDA(pg::stream_sync(s));
  return PG_OK;
}

template <typename T>
int upload_split_consts(pg_solver* s) {
  const int m = s->cfg.members;
  std::vector<SplitConst<T>> v(m);
  for (int i = 0; i < m; ++i) {
    const pg_physics& p = s->physics[i];
    SplitConst<T>& k = v[i];
    k.inv_hbar = static_cast<T>(1.0 / p.hbar);
    k.g_C = static_cast<T>(p.g_C);
    k.g_R = static_cast<T>(p.g_R);
    k.R = static_cast<T>(p.R);
    k.gamma_C = static_cast<T>(p.gamma_C);
    k.gamma_R = static_cast<T>(p.gamma_R);
    k.g_I = static_cast<T>(p.g_I);
    k.alpha_2 = static_cast<T>(p.alpha_2);
    k.gamma_I = static_cast<T>(p.gamma_I);
    k.gamma_A = static_cast<T>(p.gamma_A);
    k.R_IA = static_cast<T>(p.R_IA);
    k.R_AI = static_cast<T>(p.R_AI);
    k.weight[0] = static_cast<T>(p.pump_weight_plus);
    k.weight[1] = static_cast<T>(p.pump_weight_minus);
    k.kappa = static_cast<T>(p.kappa);
    if (s->noise) {
      k.noise_a = static_cast<T>(s->noise_strength[i] * s->noise_gamma[i] * s->dt_over_4dv);
      k.noise_b = static_cast<T>(s->noise_strength[i] * s->noise_R[i] * s->dt_over_4dv);
      k.seed = s->seeds[i];
    } else {
      k.noise_a = k.noise_b = T(0);
      k.seed = 0ull;
    }
  }
  PG_CUDA(cudaMemcpyAsync(s->split_consts, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice,
                          s->stream));
  PG_CUDA(pg::stream_sync(s));
  return PG_OK;
}

int ensure_split(pg_solver* s) {
  if (s->split_ready) return PG_OK;
  const pg_config& c = s->cfg;
  PG_CHECK(is_pow2(c.nx) && is_pow2(c.ny) && c.nx >= 4 && c.ny >= 4 && c.nx <= 4096 &&
               c.ny <= 4096,
           PG_ERR_UNSUPPORTED, "split-step: nx and ny must be powers of two between 4 and 4096");
  int rc = c.precision == PG_DOUBLE ? setup_tables<double>(s) : setup_tables<float>(s);
  if (rc != PG_OK) return rc;
  rc = c.precision == PG_DOUBLE ? upload_split_consts<double>(s) : upload_split_consts<float>(s);
  if (rc != PG_OK) return rc;
  s->split_ready = true;
  return PG_OK;
}

struct PassPlan {
  RowPassArgs row;
  ColPassArgs col;
};

PassPlan plan(const pg_solver* s) {
  const pg_config& c = s->cfg;
  const bool dbl = c.precision == PG_DOUBLE;
  const int mv = split_max_vals(dbl);
  const size_t csize = dbl ? 16 : 8;
  PassPlan p{};
  RowPassArgs& r = p.row;
  r.nx = c.nx;
  r.ny = c.ny;
  r.log2nx = ilog2(c.nx);
  int rows = 1;
  while (rows * 2 <= c.ny && rows * 2 * c.nx <= 4096) rows *= 2;
  r.rows = rows;
  r.log2rows = ilog2(rows);
  // mv values a thread, or down to four when the grid would not fill the GPU otherwise.
  const long long resident = 1024LL * std::max(1, s->sm_count);
  auto block_threads = [&](long long blocks, int values) {
    int th = (values + mv - 1) / mv;
    if (blocks * th < resident) th = std::min(1024, std::max(th, (values + 3) / 4));
    return std::max(32, ((th + 31) / 32) * 32);
  };
  int threads = block_threads(static_cast<long long>(c.ny / rows) * c.members, rows * c.nx);
  r.threads = threads;
  r.table_stride = c.nx + c.ny;
  r.halt = s->halt;
  ColPassArgs& k = p.col;
  k.nx = c.nx;
  k.ny = c.ny;
  k.log2ny = ilog2(c.ny);
  // Four columns a block (a 32-byte row segment of FP32 complex): several blocks then share
  // an SM and one block's loads and stores overlap another's transforms.  At 1024^2 this ran
  // 10% faster than sixteen-column blocks of 1024 threads (one block per SM); two columns
  // (half a DRAM sector a row) ran 30% slower.
  int cols = 1;
  while (cols * 2 <= c.nx && cols * 2 <= 4 && cols * 2 * c.ny * csize <= 160 * 1024 &&
         cols * 2 * c.ny <= mv * 1024)
    cols *= 2;
  k.cols = cols;
  k.log2cols = ilog2(cols);
  k.threads = block_threads(static_cast<long long>(c.nx / cols) * c.members, cols * c.ny);
  k.members = c.members;
  k.reservoir = c.reservoir == PG_RES_SINGLE;
  k.res_kind = c.reservoir;
  k.potential = c.potential;
  k.noise = s->noise ? 1 : 0;
  k.pump_stride = c.pump_per_member ? s->plane : 0;
  k.pump_terms = s->pump_terms;
  k.pump_term_stride = s->pump_term_stride;
  k.pot_stride = c.potential_per_member ? s->plane : 0;
  k.dt_d = c.dt;
  k.dt_f = static_cast<float>(c.dt);
  k.halt = s->halt;
  return p;
}

template <typename T>
cudaError_t row_launch(pg_solver* s, const PassPlan& p, int forward, int table, int inverse) {
  RowPassArgs a = p.row;
  a.forward = forward;
  a.inverse = inverse;
  a.multiply = table >= 0;
  // Scale of the table: 1/N for the kicks between transforms, ny for the exit half kick
  // (powers of two, so applying it apart rounds nothing).
  a.scale = table == PROP_EXIT ? static_cast<double>(s->cfg.ny)
                               : 1.0 / (static_cast<double>(s->cfg.nx) * s->cfg.ny);
  const size_t per = static_cast<size_t>(s->cfg.nx + s->cfg.ny);
  const T* px = static_cast<const T*>(s->prop) +
                (static_cast<size_t>(table < 0 ? 0 : table) * s->cfg.members * per) * 2;
  const T* py = px + static_cast<size_t>(s->cfg.nx) * 2;
  // Member m's factors start at px + m * (nx + ny) complex values (py follows its px).
  if (sizeof(T) == 4 && s->tw4 != nullptr && split_fast_row(s->cfg.nx, s->cfg.ny))
    return launch_row_fast(static_cast<float*>(s->psi[s->cur]), static_cast<const float*>(s->tw4),
                           reinterpret_cast<const float*>(px), reinterpret_cast<const float*>(py),
                           a, s->cfg.members, s->stream);
  return launch_row_pass<T>(static_cast<T*>(s->psi[s->cur]), static_cast<const T*>(s->tw_x), px,
                            py, a, s->cfg.members, s->stream);
}

template <typename T>
cudaError_t col_launch(pg_solver* s, const PassPlan& p, int inverse, int op, int forward,
                       int scale_offset, int step_offset) {
  ColPassArgs a = p.col;
  a.inverse = inverse;
  a.forward = forward;
  a.op = op;
  a.scale_offset = scale_offset;
  a.step_offset = step_offset;
  if (sizeof(T) == 4 && s->tw4 != nullptr && split_fast_col(s->cfg.nx, s->cfg.ny))
    return launch_col_fast(static_cast<float*>(s->psi[s->cur]), static_cast<float*>(s->res[s->cur]),
                           static_cast<const float*>(s->pump), static_cast<const float*>(s->potential),
                           static_cast<const float*>(s->tw4),
                           static_cast<const SplitConst<float>*>(s->split_consts),
                           static_cast<const float*>(s->scales), s->step_base, a, s->stream);
  return launch_col_pass<T>(static_cast<T*>(s->psi[s->cur]), static_cast<T*>(s->res[s->cur]),
                            static_cast<const T*>(s->pump), static_cast<const T*>(s->potential),
                            static_cast<const T*>(s->tw_y),
                            static_cast<const SplitConst<T>*>(s->split_consts),
                            static_cast<const T*>(s->scales), s->step_base, a, s->stream);
}

// The launches of one chunk of `len` steps (scales already staged).
template <typename T>
cudaError_t chunk_launches(pg_solver* s, const PassPlan& p, int ordering, int len) {
  cudaError_t e = cudaSuccess;
  if (ordering == 1) {
    for (int k = 0; k < len && e == cudaSuccess; ++k) {
      e = col_launch<T>(s, p, 1, SPLIT_OP_KOUTER, 1, 2 * k, k);
      if (e == cudaSuccess) e = row_launch<T>(s, p, 1, PROP_FULL_N, 1);
    }
    return e;
  }
  for (int k = 0; k < len && e == cudaSuccess; ++k) {
    if (k == 0)
      e = col_launch<T>(s, p, 0, SPLIT_OP_RES_START, 1, 0, 0);
    else
      e = col_launch<T>(s, p, 1, SPLIT_OP_RES_END_START, 1, 2 * k - 1, k);
    if (e == cudaSuccess) e = row_launch<T>(s, p, 1, PROP_HALF_N, 1);
    if (e == cudaSuccess) e = col_launch<T>(s, p, 1, SPLIT_OP_NONLINEAR, 1, 0, k);
    if (e == cudaSuccess) e = row_launch<T>(s, p, 1, PROP_HALF_N, 1);
  }
  if (e == cudaSuccess) e = col_launch<T>(s, p, 1, SPLIT_OP_RES_END, 0, 2 * (len - 1) + 1, len - 1);
  return e;
}

// The graph of one chunk of `len` steps of the ordering, captured and instantiated on first
// use (test hook: graph_failure makes the capture (1) or instantiation (2) fail).
template <typename T>
int split_graph_for(pg_solver* s, const PassPlan& p, int ordering, int len, cudaGraphExec_t* out) {
  auto key = std::make_tuple(ordering, len, 0);
  auto it = s->split_graphs.find(key);
  if (it != s->split_graphs.end()) {
    *out = it->second;
    return PG_OK;
  }
  const int forced = s->graph_failure;
  s->graph_failure = 0;
  cudaGraph_t graph = nullptr;
  PG_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t le = chunk_launches<T>(s, p, ordering, len);
  cudaError_t ee = cudaStreamEndCapture(s->stream, &graph);
  if (forced == 1 && ee == cudaSuccess) ee = cudaErrorStreamCaptureInvalidated;
  cudaGraphExec_t exec = nullptr;
  cudaError_t ie = cudaSuccess;
  if (le == cudaSuccess && ee == cudaSuccess)
    ie = forced == 2 ? cudaErrorInvalidValue : cudaGraphInstantiate(&exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (le != cudaSuccess || ee != cudaSuccess || ie != cudaSuccess) {
    set_error(std::string("split-step graph capture failed: ") +
              cudaGetErrorString(le != cudaSuccess ? le : ee != cudaSuccess ? ee : ie));
    return PG_ERR_CUDA;
  }
  s->split_graphs[key] = exec;
  *out = exec;
  return PG_OK;
}

template <typename T>
int split_prepare_t(pg_solver* s, int ordering, int n_steps) {
  const PassPlan p = plan(s);
  for (int done = 0; done < n_steps;) {
    const int len = std::min(kChunk, n_steps - done);
    cudaGraphExec_t exec = nullptr;
    if (len >= 2) {
      const int rc = split_graph_for<T>(s, p, ordering, len, &exec);
      if (rc != PG_OK) return rc;
    }
    done += len;
  }
  return PG_OK;
}

template <typename T>
int split_advance_t(pg_solver* s, int ordering, int64_t start_step, int n_steps,
                    const double* scales, int use_graphs) {
  const PassPlan p = plan(s);
  s->last_launches = 0;
  if (ordering == 1) {
    // Entry: spectrum (or FFT2 of psi) times the half kick, then F_x^-1.
    if (!s->spectral) {
      PG_CUDA(col_launch<T>(s, p, 0, SPLIT_OP_NONE, 1, 0, 0));
      PG_CUDA(row_launch<T>(s, p, 1, PROP_HALF_N, 1));
      s->last_launches += 2;
    } else {
      PG_CUDA(row_launch<T>(s, p, 0, PROP_HALF_N, 1));
      s->last_launches += 1;
    }
    s->spectral = false;
  } else {
    PG_CHECK(!s->spectral, PG_ERR_INVALID,
             "split-step-fft (R/2 K/2 N K/2 R/2) needs psi in real space; the state holds a "
             "spectrum");
  }
  const int m = s->cfg.members;
  int done = 0;
  while (done < n_steps) {
    const int len = std::min(kChunk, n_steps - done);
    int rc = stage_coefficients(s, scales + static_cast<size_t>(done) * 2 * s->pump_terms * m, len,
                                2 * s->pump_terms, start_step + done);
    if (rc != PG_OK) return rc;
    cudaGraphExec_t exec = nullptr;
    if (use_graphs && len >= 2 && split_graph_for<T>(s, p, ordering, len, &exec) != PG_OK) {
      // A failed capture or instantiation has run nothing of the chunk (capture only records):
      // the chunk runs as plain launches (see pg_rk4_advance).
      cudaGetLastError();
      ++s->graph_fallbacks;
      exec = nullptr;
    }
    if (exec != nullptr) {
      PG_CUDA(cudaGraphLaunch(exec, s->stream));
    } else {
      PG_CUDA(chunk_launches<T>(s, p, ordering, len));
    }
    s->last_launches += ordering == 1 ? 2 * len : 4 * len + 1;
    done += len;
  }
  if (ordering == 1) {
    // Exit: F_x, then ny conj(half) turns the last full kick into the closing half kick.
    PG_CUDA(row_launch<T>(s, p, 1, PROP_EXIT, 0));
    s->last_launches += 1;
    s->spectral = true;
  }
  return PG_OK;
}

}  // namespace

int split_ensure(pg_solver* s) { return ensure_split(s); }

int split_release(pg_solver* s) {
  for (auto& kv : s->split_graphs) cudaGraphExecDestroy(kv.second);
  s->split_graphs.clear();
  cudaFree(s->tw_x);
  cudaFree(s->tw_y);
  cudaFree(s->tw4);
  s->tw4 = nullptr;
  cudaFree(s->prop);
  cudaFree(s->split_consts);
  s->tw_x = s->tw_y = s->prop = s->split_consts = nullptr;
  s->split_ready = false;
  return PG_OK;
}

int split_refresh_consts(pg_solver* s) {
  for (auto& kv : s->split_graphs) cudaGraphExecDestroy(kv.second);
  s->split_graphs.clear();
  return s->cfg.precision == PG_DOUBLE ? upload_split_consts<double>(s)
                                       : upload_split_consts<float>(s);
}

}  // namespace pg

extern "C" {

int pg_split_advance(pg_solver* s, int32_t ordering, int64_t start_step, int32_t n_steps,
                     const double* half_scales, int use_graphs) {
  PG_CHECK(s && half_scales, PG_ERR_INVALID, "pg_split_advance: null argument");
  PG_CHECK(ordering == 0 || ordering == 1, PG_ERR_INVALID,
           "pg_split_advance: ordering must be 0 (R/2 K/2 N K/2 R/2) or 1 (K/2 [R/2 N R/2] K/2)");
  PG_CHECK(n_steps >= 0, PG_ERR_INVALID, "pg_split_advance: negative step count");
  PG_CHECK(s->comps == 1 && s->res_comps == 1, PG_ERR_UNSUPPORTED,
           "pg_split_advance: two-component fields run on the IFRK path");
  if (n_steps == 0) return PG_OK;
  pg::ifrk_invalidate(s);
  int rc = pg::ensure_split(s);
  if (rc != PG_OK) return rc;
  return s->cfg.precision == PG_DOUBLE
             ? pg::split_advance_t<double>(s, ordering, start_step, n_steps, half_scales, use_graphs)
             : pg::split_advance_t<float>(s, ordering, start_step, n_steps, half_scales, use_graphs);
}

int pg_split_prepare(pg_solver* s, int32_t ordering, int32_t n_steps) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_split_prepare: null solver");
  PG_CHECK(ordering == 0 || ordering == 1, PG_ERR_INVALID, "pg_split_prepare: ordering must be 0 or 1");
  PG_CHECK(n_steps >= 0, PG_ERR_INVALID, "pg_split_prepare: negative step count");
  PG_CHECK(s->comps == 1 && s->res_comps == 1, PG_ERR_UNSUPPORTED,
           "pg_split_prepare: two-component fields run on the IFRK path");
  int rc = pg::ensure_split(s);
  if (rc != PG_OK) return rc;
  return s->cfg.precision == PG_DOUBLE ? pg::split_prepare_t<double>(s, ordering, n_steps)
                                       : pg::split_prepare_t<float>(s, ordering, n_steps);
}

int pg_set_state_kind(pg_solver* s, int32_t spectral) {
  PG_CHECK(s, PG_ERR_INVALID, "pg_set_state_kind: null solver");
  s->spectral = spectral != 0;
  return PG_OK;
}

int pg_get_state_kind(pg_solver* s, int32_t* spectral) {
  PG_CHECK(s && spectral, PG_ERR_INVALID, "pg_get_state_kind: null argument");
  *spectral = s->spectral ? 1 : 0;
  return PG_OK;
}

}  // extern "C"
