// Host sequencing of the Lawson IFRK step (fixed step and adaptive DP5 trials).
//
// Per stage i: one row pass (F_x of the previous stage's half-transformed right-hand
// side, stored as f_hat_{i-1}; the Lawson combination; F_x^-1) and one column pass
// (F_y^-1; right-hand side and reservoir derivative of stage i; F_y).  The step ends
// with the b-weighted combination (row pass) and the clamped reservoir, the Wigner
// increment and the new field (column pass).  Adaptive trials add the error combination
// and an FP64 error norm reduced per block (polarism/solver/ifrk_fft_cuda_solver.py:
// 148-293; the accept/retry decision and the PI control stay on the host as in
// polarism/solver/step_controller.py:48-81).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "ifrk_internal.h"
#include "pg_internal.h"
#include "solver.h"

namespace pg {
namespace {

constexpr double kPi2 = 3.141592653589793238462643383279502884;

// Butcher tableaus (published Dormand-Prince 5(4) and the classic RK4), as in
// polarism/solver/tableaus.py:34-60.
struct Tableau {
  int stages;
  double A[7][7];
  double b[7];
  double c[7];
  double bhat[7];
  bool embedded;
};

const Tableau& tableau(int which) {
  static const Tableau rk4 = {
      4,
      {{0, 0, 0, 0}, {0.5, 0, 0, 0}, {0, 0.5, 0, 0}, {0, 0, 1.0, 0}},
      {1.0 / 6, 1.0 / 3, 1.0 / 3, 1.0 / 6},
      {0, 0.5, 0.5, 1.0},
      {0},
      false};
  static const Tableau dp5 = {
      7,
      {{0},
       {1.0 / 5},
       {3.0 / 40, 9.0 / 40},
       {44.0 / 45, -56.0 / 15, 32.0 / 9},
       {19372.0 / 6561, -25360.0 / 2187, 64448.0 / 6561, -212.0 / 729},
       {9017.0 / 3168, -355.0 / 33, 46732.0 / 5247, 49.0 / 176, -5103.0 / 18656},
       {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84}},
      {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84, 0},
      {0, 1.0 / 5, 3.0 / 10, 4.0 / 5, 8.0 / 9, 1.0, 1.0},
      {5321.0 / 57600, 0, 7429.0 / 16695, 1321.0 / 1920, -126603.0 / 339200, 121.0 / 700,
       -1.0 / 40},
      true};
  return which == 1 ? dp5 : rk4;
}

bool is_pow2i(int n) { return n > 0 && (n & (n - 1)) == 0; }
int ilog2i(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return l;
}
double wavenumber(int j, int n, double d) {
  const int k = j < (n + 1) / 2 ? j : j - n;
  return 2.0 * kPi2 * static_cast<double>(k) / (static_cast<double>(n) * d);
}

struct IfrkBuffers {
  size_t csize = 0;
  void* W = nullptr;
  void* psi0_hat = nullptr;
  void* fhat[kIfrkMaxStages] = {};
  void* ehat = nullptr;
  void* psi_new = nullptr;
  void* psi_start = nullptr;
  void* n_new = nullptr;
  void* dn[kIfrkMaxStages] = {};
  void* tables = nullptr;
  size_t table_capacity = 0;  // number of (members x (nx + ny)) tables
  double* partials = nullptr;
  int partial_blocks = 0;
  std::vector<double> host_partials;
  bool w_valid = false;  // W holds F_y of the current state
  SpinorConst* spin = nullptr;  // two-component Lawson constants per member
  float* spin_modes = nullptr;  // FP32 state: per-mode table of the two-component factor
};

IfrkBuffers& bufs(pg_solver* s) { return *static_cast<IfrkBuffers*>(s->ifrk); }

int ensure_ifrk(pg_solver* s) {
  if (s->ifrk) return PG_OK;
  const pg_config& c = s->cfg;
  PG_CHECK(is_pow2i(c.nx) && is_pow2i(c.ny) && c.nx >= 4 && c.ny >= 4 && c.nx <= 4096 && c.ny <= 4096,
           PG_ERR_UNSUPPORTED, "IFRK: nx and ny must be powers of two between 4 and 4096");
  for (const auto& p : s->physics)
    PG_CHECK(p.kinetic_relaxation_eta == 0.0, PG_ERR_UNSUPPORTED,
             "IFRK: the kinetic relaxation term is not implemented on the GPU path");
  // The split-step set-up provides twiddles and the per-member constants.
  int rc = split_ensure(s);
  if (rc != PG_OK) return rc;
  IfrkBuffers* b = new IfrkBuffers();
  s->ifrk = b;
  const size_t cbytes = static_cast<size_t>(s->field_values) * 2 * s->real_size;
  const size_t rbytes = static_cast<size_t>(std::max<long long>(1, s->res_values)) * s->real_size;
  b->csize = cbytes;
  PG_CUDA(cudaMalloc(&b->W, cbytes));
  PG_CUDA(cudaMalloc(&b->psi0_hat, cbytes));
  for (int i = 0; i < kIfrkMaxStages; ++i) {
    PG_CUDA(cudaMalloc(&b->fhat[i], cbytes));
    PG_CUDA(cudaMalloc(&b->dn[i], rbytes));
  }
  PG_CUDA(cudaMalloc(&b->ehat, cbytes));
  PG_CUDA(cudaMalloc(&b->psi_new, cbytes));
  PG_CUDA(cudaMalloc(&b->psi_start, cbytes));
  PG_CUDA(cudaMalloc(&b->n_new, rbytes));
  const int cols_blocks = c.nx;  // upper bound on column panels per member
  b->partial_blocks = cols_blocks;
  PG_CUDA(cudaMalloc(&b->partials, sizeof(double) * static_cast<size_t>(cols_blocks) * c.members));
  b->host_partials.resize(static_cast<size_t>(cols_blocks) * c.members);
  if (s->comps == 2) {
    std::vector<SpinorConst> host(c.members);
    for (int m = 0; m < c.members; ++m) {
      const pg_physics& p = s->physics[m];
      host[m] = SpinorConst{p.hbar / (2.0 * p.m_eff), 0.5 * p.zeeman, p.te_tm, 1.0 / p.hbar};
    }
    PG_CUDA(cudaMalloc(&b->spin, host.size() * sizeof(SpinorConst)));
    PG_CUDA(cudaMemcpyAsync(b->spin, host.data(), host.size() * sizeof(SpinorConst),
                            cudaMemcpyHostToDevice, s->stream));
    PG_CUDA(pg::stream_sync(s));
    if (c.precision == PG_SINGLE) {
      PG_CUDA(cudaMalloc(&b->spin_modes, sizeof(float) * kSpinModeFields * static_cast<size_t>(s->plane) *
                                             c.members));
      PG_CUDA(launch_spin_mode_table(b->spin_modes, b->spin, c.nx, c.ny, c.members,
                                     2.0 * kPi2 / (static_cast<double>(c.nx) * c.dx),
                                     2.0 * kPi2 / (static_cast<double>(c.ny) * c.dy), s->stream));
      PG_CUDA(pg::stream_sync(s));
    }
  }
  const size_t esize = s->real_size;
  if (c.precision == PG_DOUBLE)
    PG_CUDA(configure_ifrk_kernels<double>(200 * 1024));
  else
    PG_CUDA(configure_ifrk_kernels<float>(200 * 1024));
  (void)esize;
  return PG_OK;
}

// Upload the separable Lawson factors E(tau)/N for a list of tau values.
template <typename T>
int upload_tables(pg_solver* s, const std::vector<double>& taus) {
  IfrkBuffers& b = bufs(s);
  const pg_config& c = s->cfg;
  const size_t per = static_cast<size_t>(c.nx + c.ny);
  const size_t ntab = taus.size();
  if (ntab > b.table_capacity) {
    cudaFree(b.tables);
    b.tables = nullptr;
    PG_CUDA(cudaMalloc(&b.tables, ntab * c.members * per * 2 * sizeof(T)));
    b.table_capacity = ntab;
  }
  std::vector<T> host(ntab * c.members * per * 2);
  const double N = static_cast<double>(c.nx) * c.ny;
  for (size_t t = 0; t < ntab; ++t) {
    for (int m = 0; m < c.members; ++m) {
      const pg_physics& p = s->physics[m];
      const double rate = -p.hbar / (2.0 * p.m_eff);
      T* base = host.data() + ((t * c.members + m) * per) * 2;
      for (int j = 0; j < c.nx; ++j) {
        const double k = wavenumber(j, c.nx, c.dx);
        const std::complex<double> v = std::exp(std::complex<double>(0.0, rate * taus[t] * k * k)) / N;
        base[2 * j] = static_cast<T>(v.real());
        base[2 * j + 1] = static_cast<T>(v.imag());
      }
      for (int i = 0; i < c.ny; ++i) {
        const double k = wavenumber(i, c.ny, c.dy);
        const std::complex<double> v = std::exp(std::complex<double>(0.0, rate * taus[t] * k * k));
        base[2 * (c.nx + i)] = static_cast<T>(v.real());
        base[2 * (c.nx + i) + 1] = static_cast<T>(v.imag());
      }
    }
  }
  PG_CUDA(cudaMemcpyAsync(b.tables, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice,
                          s->stream));
  PG_CUDA(pg::stream_sync(s));
  return PG_OK;
}

struct Plan {
  IfrkRowArgs row;
  IfrkColArgs col;
};

Plan make_plan(const pg_solver* s) {
  const pg_config& c = s->cfg;
  const bool dbl = c.precision == PG_DOUBLE;
  const int mv = split_max_vals(dbl);
  const size_t csize = dbl ? 16 : 8;
  Plan p{};
  IfrkRowArgs& r = p.row;
  r.nx = c.nx;
  r.ny = c.ny;
  r.log2nx = ilog2i(c.nx);
  const int comps = s->comps;
  // Fill the GPU first: stop growing the tiles once fewer than two blocks per SM would remain
  // (a single 512^2 spinor otherwise runs on 32 column blocks); columns stay at least one
  // 32-byte sector wide so the panel loads remain coalesced.
  const long long want_blocks = 2LL * std::max(1, s->sm_count);
  int rows = 1;
  while (rows * 2 <= c.ny && rows * 2 * c.nx * comps <= 4096 &&
         static_cast<long long>(c.ny / (rows * 2)) * c.members >= want_blocks)
    rows *= 2;
  r.rows = rows;
  r.log2rows = ilog2i(rows);
  // Threads per block: mv values each, unless the whole grid would then hold fewer threads
  // than the GPU runs at once (a single 512^2 spinor gives about 7 warps per SM); then down to
  // four values a thread, which the Stockham passes handle with one butterfly per thread.
  const long long resident = 1024LL * std::max(1, s->sm_count);
  auto block_threads = [&](long long blocks, int values) {
    int th = (values + mv - 1) / mv;
    if (blocks * th < resident) th = std::min(1024, std::max(th, (values + 3) / 4));
    return std::max(32, ((th + 31) / 32) * 32);
  };
  int threads = block_threads(static_cast<long long>(c.ny / rows) * c.members, rows * c.nx * comps);
  r.threads = threads;
  r.members = c.members;
  r.comps = comps;
  r.member_stride = s->plane * comps;
  r.spinor = comps == 2 ? 1 : 0;
  r.kx_unit = 2.0 * kPi2 / (static_cast<double>(c.nx) * c.dx);
  r.ky_unit = 2.0 * kPi2 / (static_cast<double>(c.ny) * c.dy);
  r.inv_n = 1.0 / (static_cast<double>(c.nx) * c.ny);
  r.spin = s->ifrk ? static_cast<const void*>(static_cast<IfrkBuffers*>(s->ifrk)->spin) : nullptr;
  r.modes = s->ifrk ? static_cast<IfrkBuffers*>(s->ifrk)->spin_modes : nullptr;
  IfrkColArgs& k = p.col;
  k.nx = c.nx;
  k.ny = c.ny;
  k.log2ny = ilog2i(c.ny);
  const int min_cols = static_cast<int>(std::min<size_t>(static_cast<size_t>(c.nx), 32 / csize));
  int cols = 1;
  // At most four columns a block, as the split-step column pass: several blocks share an SM
  // (fixed-step IFRK4 at 1024^2 x 16 members: +7% over sixteen-column blocks).
  while (cols * 2 <= c.nx && cols * 2 <= 4 && cols * 2 * comps * c.ny * csize <= 160 * 1024 &&
         cols * 2 * comps * c.ny <= mv * 1024 &&
         (cols < min_cols || static_cast<long long>(c.nx / (cols * 2)) * c.members >= want_blocks))
    cols *= 2;
  k.cols = cols;
  k.log2cols = ilog2i(cols);
  k.threads = block_threads(static_cast<long long>(c.nx / cols) * c.members, cols * comps * c.ny);
  k.members = c.members;
  k.comps = comps;
  k.log2comps = comps == 2 ? 1 : 0;
  k.res_fields = s->res_fields;
  k.res_kind = s->cfg.reservoir;
  k.res_comps = s->res_comps;
  k.reservoir = s->res_fields > 0;
  k.potential = c.potential;
  k.pump_stride = c.pump_per_member ? s->plane : 0;
  k.pump_terms = s->pump_terms;
  k.pump_term_stride = s->pump_term_stride;
  k.pot_stride = c.potential_per_member ? s->plane : 0;
  return p;
}

// Table bookkeeping: index of tau in the list (appended when new).
int tau_index(std::vector<double>& taus, double tau) {
  for (size_t i = 0; i < taus.size(); ++i)
    if (taus[i] == tau) return static_cast<int>(i);
  taus.push_back(tau);
  return static_cast<int>(taus.size() - 1);
}

struct StepTables {
  std::vector<double> taus;
  // stage combine: [stage][term] table index; term 0 = psi0_hat
  int stage_tab[kIfrkMaxStages][kIfrkMaxTerms];
  int final_tab[kIfrkMaxTerms];
  int err_tab[kIfrkMaxTerms];
};

StepTables build_tables(const Tableau& tb, double h) {
  StepTables st{};
  for (int i = 0; i < tb.stages; ++i) {
    st.stage_tab[i][0] = tau_index(st.taus, tb.c[i] * h);
    for (int j = 0; j < i; ++j) st.stage_tab[i][1 + j] = tau_index(st.taus, (tb.c[i] - tb.c[j]) * h);
  }
  st.final_tab[0] = tau_index(st.taus, h);
  for (int j = 0; j < tb.stages; ++j) {
    st.final_tab[1 + j] = tau_index(st.taus, (1.0 - tb.c[j]) * h);
    st.err_tab[j] = st.final_tab[1 + j];
  }
  return st;
}

// The spinor row pass evaluates its Lawson factors from tau instead of the tables.
void set_taus(IfrkRowArgs& r, const StepTables& st) {
  for (int t = 0; t < r.terms; ++t) {
    r.tau[t] = st.taus[r.table[t]];
    r.tau_hi[t] = static_cast<float>(r.tau[t]);
    r.tau_lo[t] = static_cast<float>(r.tau[t] - static_cast<double>(r.tau_hi[t]));
  }
}

// A row pass: the register-resident four-step form for FP32 one-component rows of 1024 sites,
// the generic Stockham pass otherwise.
template <typename T>
cudaError_t ifrk_row(pg_solver* s, const T* in, T* save, T* out, const T* tables,
                     const IfrkRowArgs& a, const T* tw) {
  if constexpr (sizeof(T) == 4) {
    if (s->tw4 != nullptr && ifrk_fast_row(a))
      return launch_ifrk_row_fast(in, save, out, tables, static_cast<const float*>(s->tw4), a,
                                  s->stream);
  }
  return launch_ifrk_row<T>(in, save, out, tables, a, tw, s->stream);
}

// A column pass: the register-resident form for FP32 one-component columns of 1024 sites
// (the forward-only pass, and stages and step ends with one single reservoir and one laser),
// the generic Stockham pass otherwise.
template <typename T>
cudaError_t ifrk_col(pg_solver* s, T* psi, const T* n0, T* dn_out, T* n_out, const T* psi_start,
                     const T* psi_new, const T* tw, const SplitConst<T>* consts, const T* scales,
                     const IfrkColArgs& a) {
  if constexpr (sizeof(T) == 4) {
    if (s->tw4 != nullptr && ifrk_fast_col(a))
      return launch_ifrk_col_fast(psi, n0, dn_out, n_out, psi_start, psi_new,
                                  static_cast<const float*>(s->pump),
                                  static_cast<const float*>(s->potential),
                                  static_cast<const float*>(s->tw4), consts, scales, s->step_base,
                                  a, s->stream);
  }
  return launch_ifrk_col<T>(psi, n0, dn_out, n_out, psi_start, psi_new,
                            static_cast<const T*>(s->pump), static_cast<const T*>(s->potential), tw,
                            consts, scales, s->step_base, nullptr, a, s->stream);
}

template <typename T>
int run_step(pg_solver* s, const Plan& p, const Tableau& tb, const StepTables& st, double h,
             int scale_base, int step_offset, bool noise, bool adaptive, double rtol, double atol,
             double* err_out) {
  IfrkBuffers& b = bufs(s);
  T* state = static_cast<T*>(s->psi[s->cur]);
  T* n0 = static_cast<T*>(s->res[s->cur]);
  T* W = static_cast<T*>(b.W);
  const T* tw_x = static_cast<const T*>(s->tw_x);
  const T* tw_y = static_cast<const T*>(s->tw_y);
  const T* tables = static_cast<const T*>(b.tables);
  const auto* consts = static_cast<const SplitConst<T>*>(s->split_consts);
  const T* scales = static_cast<const T*>(s->scales);
  if (!b.w_valid) {
    PG_CUDA(cudaMemcpyAsync(W, state, b.csize, cudaMemcpyDeviceToDevice, s->stream));
    IfrkColArgs a = p.col;
    a.mode = 3;
    a.inverse = 0;
    a.forward = 1;
    PG_CUDA(ifrk_col<T>(s, W, n0, nullptr, nullptr, nullptr, nullptr, tw_y, consts, nullptr, a));
    b.w_valid = true;
    s->last_launches += 1;
  }
  for (int i = 0; i < tb.stages; ++i) {
    IfrkRowArgs r = p.row;
    r.forward = 1;
    r.inverse = 1;
    r.terms = 0;
    // psi0_hat: the fresh row at stage 0, the stored spectrum afterwards.
    r.src[r.terms] = i == 0 ? nullptr : b.psi0_hat;
    r.coef[r.terms] = 1.0;
    r.table[r.terms] = st.stage_tab[i][0];
    ++r.terms;
    for (int j = 0; j < i; ++j) {
      if (tb.A[i][j] == 0.0) continue;
      r.src[r.terms] = j == i - 1 ? nullptr : b.fhat[j];
      r.coef[r.terms] = h * tb.A[i][j];
      r.table[r.terms] = st.stage_tab[i][1 + j];
      ++r.terms;
    }
    T* save = static_cast<T*>(i == 0 ? b.psi0_hat : b.fhat[i - 1]);
    set_taus(r, st);
    PG_CUDA(ifrk_row<T>(s, W, save, W, tables, r, tw_x));
    IfrkColArgs a = p.col;
    a.mode = 0;
    a.inverse = 1;
    a.forward = 1;
    a.terms = 0;
    for (int j = 0; j < i; ++j) {
      if (tb.A[i][j] == 0.0) continue;
      a.dn[a.terms] = b.dn[j];
      a.coef[a.terms] = h * tb.A[i][j];
      ++a.terms;
    }
    a.scale_index = scale_base + i;
    PG_CUDA(ifrk_col<T>(s, W, n0, static_cast<T*>(b.dn[i]), nullptr,
                        adaptive && i == 0 ? static_cast<T*>(b.psi_start) : nullptr, nullptr, tw_y,
                        consts, scales, a));
    s->last_launches += 2;
  }
  // Final combination.
  {
    IfrkRowArgs r = p.row;
    r.forward = 1;
    r.inverse = 1;
    r.terms = 0;
    r.src[r.terms] = b.psi0_hat;
    r.coef[r.terms] = 1.0;
    r.table[r.terms] = st.final_tab[0];
    ++r.terms;
    for (int j = 0; j < tb.stages; ++j) {
      if (tb.b[j] == 0.0) continue;
      r.src[r.terms] = j == tb.stages - 1 ? nullptr : b.fhat[j];
      r.coef[r.terms] = h * tb.b[j];
      r.table[r.terms] = st.final_tab[1 + j];
      ++r.terms;
    }
    set_taus(r, st);
    PG_CUDA(ifrk_row<T>(s, W, static_cast<T*>(b.fhat[tb.stages - 1]), W, tables, r, tw_x));
    IfrkColArgs a = p.col;
    a.mode = 1;
    a.inverse = 1;
    a.forward = 1;
    a.noise = noise ? 1 : 0;
    a.step_offset = step_offset;
    a.terms = 0;
    for (int j = 0; j < tb.stages; ++j) {
      if (tb.b[j] == 0.0) continue;
      a.dn[a.terms] = b.dn[j];
      a.coef[a.terms] = h * tb.b[j];
      ++a.terms;
    }
    PG_CUDA(ifrk_col<T>(s, W, n0, nullptr, static_cast<T*>(b.n_new), nullptr,
                        static_cast<T*>(b.psi_new), tw_y, consts, scales, a));
    s->last_launches += 2;
  }
  if (adaptive) {
    IfrkRowArgs r = p.row;
    r.forward = 0;
    r.inverse = 1;
    r.terms = 0;
    for (int j = 0; j < tb.stages; ++j) {
      const double w = tb.b[j] - tb.bhat[j];
      if (w == 0.0) continue;
      r.src[r.terms] = b.fhat[j];
      r.coef[r.terms] = h * w;
      r.table[r.terms] = st.err_tab[j];
      ++r.terms;
    }
    set_taus(r, st);
    PG_CUDA(ifrk_row<T>(s, static_cast<const T*>(nullptr), static_cast<T*>(nullptr),
                        static_cast<T*>(b.ehat), tables, r, tw_x));
    IfrkColArgs a = p.col;
    a.mode = 2;
    a.inverse = 1;
    a.forward = 0;
    a.rtol = rtol;
    a.atol = atol;
    a.terms = 0;
    for (int j = 0; j < tb.stages; ++j) {
      const double w = tb.b[j] - tb.bhat[j];
      if (w == 0.0) continue;
      a.dn[a.terms] = b.dn[j];
      a.coef[a.terms] = h * w;
      ++a.terms;
    }
    PG_CUDA(launch_ifrk_col<T>(static_cast<T*>(b.ehat), n0, nullptr, static_cast<T*>(b.n_new),
                               static_cast<T*>(b.psi_start), static_cast<T*>(b.psi_new),
                               static_cast<const T*>(s->pump), static_cast<const T*>(s->potential),
                               tw_y, consts, scales, s->step_base, b.partials, a, s->stream));
    s->last_launches += 2;
    const int panels = s->cfg.nx / p.col.cols;
    const size_t count = static_cast<size_t>(panels) * s->cfg.members;
    PG_CUDA(cudaMemcpyAsync(b.host_partials.data(), b.partials, count * sizeof(double),
                            cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA(pg::stream_sync(s));
    // Values per member entering the RMS: every field component and reservoir plane.
    const double sites = static_cast<double>(s->plane) * (s->comps + s->res_fields * s->res_comps);
    double err = 0.0;
    for (int m = 0; m < s->cfg.members; ++m) {
      double sum = 0.0;
      for (int q = 0; q < panels; ++q) sum += b.host_partials[static_cast<size_t>(m) * panels + q];
      const double e = std::sqrt(sum / sites);
      err = std::max(err, std::isnan(e) ? INFINITY : e);
    }
    *err_out = err;
  }
  return PG_OK;
}

// Accept the step: the new field and reservoir become the state.
void commit(pg_solver* s) {
  IfrkBuffers& b = bufs(s);
  std::swap(s->psi[s->cur], b.psi_new);
  std::swap(s->res[s->cur], b.n_new);
}

template <typename T>
int ifrk_advance_t(pg_solver* s, int tab, int64_t start_step, int n_steps, const double* scales) {
  const Tableau& tb = tableau(tab);
  const Plan p = make_plan(s);
  const double h = s->cfg.dt;
  StepTables st = build_tables(tb, h);
  int rc = s->comps == 1 ? upload_tables<T>(s, st.taus) : PG_OK;
  if (rc != PG_OK) return rc;
  IfrkBuffers& b = bufs(s);
  b.w_valid = false;
  s->last_launches = 0;
  const int m = s->cfg.members;
  const int per_chunk = std::max(1, (kChunk * 3) / tb.stages);
  int done = 0;
  while (done < n_steps) {
    const int len = std::min(per_chunk, n_steps - done);
    rc = stage_coefficients(s, scales + static_cast<size_t>(done) * tb.stages * s->pump_terms * m, len,
                            tb.stages * s->pump_terms,
                            start_step + done);
    if (rc != PG_OK) return rc;
    for (int k = 0; k < len; ++k) {
      rc = run_step<T>(s, p, tb, st, h, k * tb.stages, k, s->noise, false, 0, 0, nullptr);
      if (rc != PG_OK) return rc;
      commit(s);
    }
    done += len;
  }
  return PG_OK;
}

template <typename T>
int ifrk_trial_t(pg_solver* s, int tab, double h, const double* scales, double rtol, double atol,
                 double* err, int* accepted) {
  const Tableau& tb = tableau(tab);
  PG_CHECK(tb.embedded, PG_ERR_INVALID, "pg_ifrk_trial: the tableau has no embedded pair");
  const Plan p = make_plan(s);
  StepTables st = build_tables(tb, h);
  int rc = s->comps == 1 ? upload_tables<T>(s, st.taus) : PG_OK;
  if (rc != PG_OK) return rc;
  rc = stage_coefficients(s, scales, 1, tb.stages * s->pump_terms, 0);
  if (rc != PG_OK) return rc;
  s->last_launches = 0;
  rc = run_step<T>(s, p, tb, st, h, 0, 0, false, true, rtol, atol, err);
  if (rc != PG_OK) return rc;
  IfrkBuffers& b = bufs(s);
  if (*err <= 1.0) {
    commit(s);
    *accepted = 1;
  } else {
    b.w_valid = false;  // W was advanced; rebuild it from the unchanged state
    *accepted = 0;
  }
  return PG_OK;
}

}  // namespace

void ifrk_release(pg_solver* s) {
  if (!s->ifrk) return;
  IfrkBuffers* b = static_cast<IfrkBuffers*>(s->ifrk);
  cudaFree(b->W);
  cudaFree(b->psi0_hat);
  for (int i = 0; i < kIfrkMaxStages; ++i) {
    cudaFree(b->fhat[i]);
    cudaFree(b->dn[i]);
  }
  cudaFree(b->ehat);
  cudaFree(b->psi_new);
  cudaFree(b->psi_start);
  cudaFree(b->n_new);
  cudaFree(b->tables);
  cudaFree(b->partials);
  cudaFree(b->spin);
  cudaFree(b->spin_modes);
  delete b;
  s->ifrk = nullptr;
}

void ifrk_invalidate(pg_solver* s) {
  if (s->ifrk) bufs(s).w_valid = false;
}

}  // namespace pg

extern "C" {

int pg_ifrk_advance(pg_solver* s, int32_t tab, int64_t start_step, int32_t n_steps,
                    const double* stage_scales) {
  PG_CHECK(s && stage_scales, PG_ERR_INVALID, "pg_ifrk_advance: null argument");
  PG_CHECK(tab == 0 || tab == 1, PG_ERR_INVALID, "pg_ifrk_advance: tableau must be 0 (rk4) or 1 (dp5)");
  PG_CHECK(n_steps >= 0, PG_ERR_INVALID, "pg_ifrk_advance: negative step count");
  PG_CHECK(!s->spectral, PG_ERR_INVALID, "pg_ifrk_advance: the state holds a spectrum");
  if (n_steps == 0) return PG_OK;
  int rc = pg::ensure_ifrk(s);
  if (rc != PG_OK) return rc;
  return s->cfg.precision == PG_DOUBLE
             ? pg::ifrk_advance_t<double>(s, tab, start_step, n_steps, stage_scales)
             : pg::ifrk_advance_t<float>(s, tab, start_step, n_steps, stage_scales);
}

int pg_ifrk_trial(pg_solver* s, int32_t tab, double h, const double* stage_scales, double rtol,
                  double atol, double* err_out, int32_t* accepted) {
  PG_CHECK(s && stage_scales && err_out && accepted, PG_ERR_INVALID, "pg_ifrk_trial: null argument");
  PG_CHECK(tab == 1, PG_ERR_INVALID, "pg_ifrk_trial: adaptive trials need the dp5 tableau (1)");
  PG_CHECK(h > 0 && rtol > 0 && atol >= 0, PG_ERR_INVALID, "pg_ifrk_trial: bad step or tolerances");
  PG_CHECK(!s->spectral, PG_ERR_INVALID, "pg_ifrk_trial: the state holds a spectrum");
  int rc = pg::ensure_ifrk(s);
  if (rc != PG_OK) return rc;
  int acc = 0;
  rc = s->cfg.precision == PG_DOUBLE
           ? pg::ifrk_trial_t<double>(s, tab, h, stage_scales, rtol, atol, err_out, &acc)
           : pg::ifrk_trial_t<float>(s, tab, h, stage_scales, rtol, atol, err_out, &acc);
  *accepted = acc;
  return rc;
}

}  // extern "C"
