// Fused whole-step RK4 kernel for the driven-dissipative GPE (finite differences).
//
// Math follows polarism/model.py:89-127 (right-hand side), polarism/reservoir/
// single_reservoir.py:81-98 (reservoir derivative), polarism/solver/
// rk4_fdm_solver.py:36-82 (stage-coupled RK4 with the reservoir advanced through
// the same stages) and the reservoir clamp of single_reservoir.py:70-73.  The
// pump product is rounded on its own (__fmul_rn / __dmul_rn) as in
// polarism/solver/rk4_cuda_solver.py:884-888, and the Wigner increment uses the
// post-step clamped reservoir and the pre-step counter (rk4_cuda_solver.py:518-532).
//
// Schedule (one launch = one RK4 step of every member).  A block owns a column
// window of the grid and a strip of rows.  Each thread owns one column and
// streams down the strip: on iteration i it receives row r of psi0/n0 and
// evaluates stage 1 on row r-1, stage 2 on r-2, stage 3 on r-3, stage 4 plus the
// final combine on r-4.  Every stage's vertical neighbours are in the thread's
// own registers (ring of four rows); horizontal neighbours come from one
// shared-memory exchange per row, double-buffered so one __syncthreads per row
// suffices.  HBM traffic is one read of psi, n and the pump envelope and one
// write of psi and n per site (28 B/site in FP32) plus the strip/tile halos.
#include "philox.cuh"
#include "pg_internal.h"

namespace pg {
namespace {

template <typename T>
struct Cplx;
template <>
struct Cplx<float> {
  using type = float2;
};
template <>
struct Cplx<double> {
  using type = double2;
};

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

template <typename T>
struct MaxThreads;
template <>
struct MaxThreads<float> {
  static constexpr int value = 544;
};
template <>
struct MaxThreads<double> {
  static constexpr int value = 288;
};

// One right-hand-side evaluation at a site.  c is the centre, (lt, rt, up, dn) the
// four neighbours, n the active reservoir density, sP the scaled pump.
// n2 is the inactive reservoir of the two-field reservoirs (double: n_I feeding n_A,
// polarism/reservoir/double_reservoir.py:106-130; quadratic-double: n_I feeding n_R through
// kappa n_I^2, quadratic_double_reservoir.py:13-14); dn2 its derivative.
template <typename T, bool GENERAL, bool TWO>
__device__ __forceinline__ void site_rhs(const typename Cplx<T>::type c,
                                         const typename Cplx<T>::type lt,
                                         const typename Cplx<T>::type rt,
                                         const typename Cplx<T>::type up,
                                         const typename Cplx<T>::type dn, const T n, const T sP,
                                         const RhsConst<T>& k, const T vre, const T vim,
                                         const RK4Features& f, T& dre, T& dim, T& dnr,
                                         const T n2, T& dn2) {
  const T rho = c.x * c.x + c.y * c.y;
  const T lre = k.ax * (lt.x + rt.x) + k.ay * (up.x + dn.x);
  const T lim = k.ax * (lt.y + rt.y) + k.ay * (up.y + dn.y);
  T w = k.w0 + k.gc * rho + k.gr * n;
  T gl = k.half_R * n - k.half_gC;
  if (GENERAL) {
    w += vre * k.inv_hbar;
    gl += vim * k.inv_hbar;
    if (TWO) w += k.gi * n2;
  }
  dre = gl * c.x + w * c.y - lim;
  dim = gl * c.y - w * c.x + lre;
  if (GENERAL && f.relax) {
    const T en = k.eta_a * n;
    dre += en * (lre - k.w0 * c.x);
    dim += en * (lim - k.w0 * c.y);
  }
  dnr = sP - (k.gamma_R + k.R * rho) * n;
  dn2 = T(0);
  if (GENERAL) {
    if (f.reservoir == 0) {
      dnr = T(0);
    } else if (TWO && f.reservoir == 2) {
      dn2 = sP - (k.gamma_I + k.R_IA) * n2 + k.R_AI * n;
      dnr = k.R_IA * n2 - (k.gamma_A + k.R_AI + k.R * rho) * n;
    } else if (TWO && f.reservoir == 3) {
      const T transfer = k.kappa * n2 * n2;
      dnr = transfer - k.gamma_R * n - k.R * n * rho;
      dn2 = sP - transfer - k.gamma_I * n2;
    }
  }
}

template <typename T, bool NOISE, bool GENERAL, bool TWO>
__global__ void __launch_bounds__(MaxThreads<T>::value, 1)
    rk4_stream_kernel(const typename Cplx<T>::type* __restrict__ psi_in,
                      const T* __restrict__ n_in, const T* __restrict__ pump,
                      const T* __restrict__ potential, typename Cplx<T>::type* __restrict__ psi_out,
                      T* __restrict__ n_out, const RhsConst<T>* __restrict__ consts,
                      const T* __restrict__ scales, const unsigned long long* __restrict__ step_base,
                      const int step_offset, const T dt, const RK4Geom g, const RK4Features f) {
  using C2 = typename Cplx<T>::type;
  if (g.halt != nullptr && __ldcg(g.halt) != 0) return;  // steady-state monitor halted the run
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2* xbuf = reinterpret_cast<C2*>(smem_raw);  // [2 parities][4 stage rows][blockDim]

  const int tid = threadIdx.x;
  const int nthreads = blockDim.x;
  const int member = blockIdx.z;
  const int nx = g.nx, ny = g.ny;
  const long long plane = static_cast<long long>(nx) * ny;

  // Column owned by this thread, and its horizontal neighbours in the exchange buffer.
  int gx, lt_i, rt_i;
  bool col_writes;
  if (g.wrap) {
    gx = tid < nx ? tid : nx - 1;
    lt_i = tid < nx ? (tid == 0 ? nx - 1 : tid - 1) : tid;
    rt_i = tid < nx ? (tid == nx - 1 ? 0 : tid + 1) : tid;
    col_writes = tid < nx;
  } else {
    const int x0 = blockIdx.x * g.tile_w;
    int x = (x0 - 4 + tid) % nx;
    if (x < 0) x += nx;
    gx = x;
    lt_i = tid > 0 ? tid - 1 : 0;
    rt_i = tid < nthreads - 1 ? tid + 1 : nthreads - 1;
    const int w_eff = min(g.tile_w, nx - x0);
    col_writes = tid >= 4 && tid < 4 + w_eff;
  }

  const RhsConst<T> k = consts[member];
  const int m_count = g.members;
  // Coefficients [step][stage][term][member]; the term axis exists only with several lasers.
  const int L = GENERAL ? f.pump_terms : 1;
  const T* c0 = scales + static_cast<long long>((step_offset * 3 + 0) * L) * m_count + member;
  const T* c1 = scales + static_cast<long long>((step_offset * 3 + 1) * L) * m_count + member;
  const T* c2 = scales + static_cast<long long>((step_offset * 3 + 2) * L) * m_count + member;
  const T s0 = c0[0], s1 = c1[0], s2 = c2[0];
  const bool multi = GENERAL && L > 1;  // several separable lasers: sum the terms per site
  const T hh = dt * T(0.5), h6 = dt / T(6), h3 = dt / T(3);

  const C2* psi_m = psi_in + member * plane;
  const T* n_m = n_in + member * plane;
  constexpr bool two = GENERAL && TWO;  // a second (inactive) reservoir field
  const long long field2 = static_cast<long long>(g.members) * plane;  // offset of the inactive field
  const T* n2_m = n_m + field2;
  const T* pump_m = pump + member * g.pump_stride;
  const T* pot_m = potential ? potential + member * g.pot_stride * (f.potential == 2 ? 2 : 1) : nullptr;

  const int y0 = blockIdx.y * g.strip_h;
  const int h_eff = min(g.strip_h, ny - y0);
  const int n_iter = (h_eff + 8 + 3) & ~3;

  // Ring registers indexed by row & 3.
  C2 p0[4], q1[4], q2[4], q3[4], acc[4];
  T n0[4], m1[4], m2[4], m3[4], accn[4], P[4];
  T u0[4], v1[4], v2[4], v3[4], accu[4];  // the inactive field's ring (two-field reservoirs)
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    p0[s] = q1[s] = q2[s] = q3[s] = acc[s] = C2{T(0), T(0)};
    n0[s] = m1[s] = m2[s] = m3[s] = accn[s] = P[s] = T(0);
    u0[s] = v1[s] = v2[s] = v3[s] = accu[s] = T(0);
  }
  for (int s = tid; s < 8 * nthreads; s += nthreads) xbuf[s] = C2{T(0), T(0)};

  // Row counters (wrapped): rload = row of psi0 received this iteration, rpump = rload - 1,
  // rout = rload - 4.
  int row_load = ((y0 - 4) % ny + ny) % ny;
  int row_pump = ((y0 - 5) % ny + ny) % ny;
  int row_out = ((y0 - 8) % ny + ny) % ny;

  // Prefetch distance of two rows.
  C2 pf_psi[2];
  T pf_n[2], pf_p[2], pf_u[2];
  {
    int rl = row_load, rp = row_pump;
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      const long long o = static_cast<long long>(rl) * nx + gx;
      pf_psi[d] = psi_m[o];
      pf_n[d] = f.reservoir ? n_m[o] : T(0);
      pf_u[d] = two ? n2_m[o] : T(0);
      pf_p[d] = pump_m[static_cast<long long>(rp) * nx + gx];
      rl = rl + 1 == ny ? 0 : rl + 1;
      rp = rp + 1 == ny ? 0 : rp + 1;
    }
  }
  int row_pf = row_load + 2;
  while (row_pf >= ny) row_pf -= ny;
  int row_pf_pump = row_pump + 2;
  while (row_pf_pump >= ny) row_pf_pump -= ny;
  __syncthreads();

  const unsigned long long noise_step = NOISE ? step_base[0] + step_offset : 0ull;
  // Philox rounds that depend only on (step, stream, key), formed once for the block.
  const PhiloxCellPrefix prefix =
      philox_cell_prefix(static_cast<uint32_t>(noise_step), static_cast<uint32_t>(noise_step >> 32),
                         1u, static_cast<uint32_t>(k.seed), static_cast<uint32_t>(k.seed >> 32));

  for (int i0 = 0; i0 < n_iter; i0 += 4) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int i = i0 + j;
      const int sa = (j + 3) & 3;  // row r-1
      const int sb = (j + 2) & 3;  // row r-2
      const int sc = (j + 1) & 3;  // row r-3
      const int sd = j;            // row r-4 (and row r)
      // Receive row r (psi0, n0) and pump row r-1; refill the prefetch slot.
      p0[j] = pf_psi[j & 1];
      n0[j] = pf_n[j & 1];
      u0[j] = pf_u[j & 1];
      P[sa] = pf_p[j & 1];
      {
        const long long o = static_cast<long long>(row_pf) * nx + gx;
        pf_psi[j & 1] = psi_m[o];
        pf_n[j & 1] = f.reservoir ? n_m[o] : T(0);
        pf_u[j & 1] = two ? n2_m[o] : T(0);
        pf_p[j & 1] = pump_m[static_cast<long long>(row_pf_pump) * nx + gx];
        row_pf = row_pf + 1 == ny ? 0 : row_pf + 1;
        row_pf_pump = row_pf_pump + 1 == ny ? 0 : row_pf_pump + 1;
      }
      const C2* xin = xbuf + ((j + 1) & 1) * 4 * nthreads;
      T vre = T(0), vim = T(0);
      // The Philox words of this iteration's output site, drawn in the straight-line code of
      // the four stages so the integer work fills their issue gaps.
      Words4 wz{0u, 0u, 0u, 0u};
      if (NOISE) {
        const uint32_t cell[1] = {static_cast<uint32_t>(static_cast<long long>(row_out) * nx + gx)};
        Words4 w1[1];
        philox_cells(cell, prefix, w1);
        wz = w1[0];
      }

      // Stage 1 at row r-1: k1 = f(psi0).
      {
        const int ra = row_load == 0 ? ny - 1 : row_load - 1;
        if (GENERAL && f.potential) {
          const long long o = static_cast<long long>(ra) * nx + gx;
          vre = f.potential == 2 ? pot_m[2 * o] : pot_m[o];
          vim = f.potential == 2 ? pot_m[2 * o + 1] : T(0);
        }
        T dre, dim, dnr, du;
        const T sP = multi ? pump_terms_value(pump_m, g.pump_term_stride, c0, m_count, L,
                                              static_cast<long long>(ra) * nx + gx)
                           : mul_rn(s0, P[sa]);
        site_rhs<T, GENERAL, TWO>(p0[sa], xin[lt_i], xin[rt_i], p0[sb], p0[j], n0[sa],
                             sP, k, vre, vim, f, dre, dim, dnr, u0[sa], du);
        q1[sa] = C2{p0[sa].x + hh * dre, p0[sa].y + hh * dim};
        m1[sa] = n0[sa] + hh * dnr;
        acc[sa] = C2{p0[sa].x + h6 * dre, p0[sa].y + h6 * dim};
        accn[sa] = n0[sa] + h6 * dnr;
        if (two) {
          v1[sa] = u0[sa] + hh * du;
          accu[sa] = u0[sa] + h6 * du;
        }
      }
      // Stage 2 at row r-2: k2 = f(psi1).
      {
        if (GENERAL && f.potential) {
          int rb = row_load - 2;
          if (rb < 0) rb += ny;
          const long long o = static_cast<long long>(rb) * nx + gx;
          vre = f.potential == 2 ? pot_m[2 * o] : pot_m[o];
          vim = f.potential == 2 ? pot_m[2 * o + 1] : T(0);
        }
        T dre, dim, dnr, du;
        const C2* xr = xin + nthreads;
        T sP = mul_rn(s1, P[sb]);
        if (multi) {
          int rb = row_load - 2;
          if (rb < 0) rb += ny;
          sP = pump_terms_value(pump_m, g.pump_term_stride, c1, m_count, L,
                                static_cast<long long>(rb) * nx + gx);
        }
        site_rhs<T, GENERAL, TWO>(q1[sb], xr[lt_i], xr[rt_i], q1[sc], q1[sa], m1[sb],
                             sP, k, vre, vim, f, dre, dim, dnr, v1[sb], du);
        q2[sb] = C2{p0[sb].x + hh * dre, p0[sb].y + hh * dim};
        m2[sb] = n0[sb] + hh * dnr;
        acc[sb] = C2{acc[sb].x + h3 * dre, acc[sb].y + h3 * dim};
        accn[sb] = accn[sb] + h3 * dnr;
        if (two) {
          v2[sb] = u0[sb] + hh * du;
          accu[sb] = accu[sb] + h3 * du;
        }
      }
      // Stage 3 at row r-3: k3 = f(psi2).
      {
        if (GENERAL && f.potential) {
          int rc = row_load - 3;
          if (rc < 0) rc += ny;
          const long long o = static_cast<long long>(rc) * nx + gx;
          vre = f.potential == 2 ? pot_m[2 * o] : pot_m[o];
          vim = f.potential == 2 ? pot_m[2 * o + 1] : T(0);
        }
        T dre, dim, dnr, du;
        const C2* xr = xin + 2 * nthreads;
        T sP = mul_rn(s1, P[sc]);
        if (multi) {
          int rc = row_load - 3;
          if (rc < 0) rc += ny;
          sP = pump_terms_value(pump_m, g.pump_term_stride, c1, m_count, L,
                                static_cast<long long>(rc) * nx + gx);
        }
        site_rhs<T, GENERAL, TWO>(q2[sc], xr[lt_i], xr[rt_i], q2[sd], q2[sb], m2[sc],
                             sP, k, vre, vim, f, dre, dim, dnr, v2[sc], du);
        q3[sc] = C2{p0[sc].x + dt * dre, p0[sc].y + dt * dim};
        m3[sc] = n0[sc] + dt * dnr;
        acc[sc] = C2{acc[sc].x + h3 * dre, acc[sc].y + h3 * dim};
        accn[sc] = accn[sc] + h3 * dnr;
        if (two) {
          v3[sc] = u0[sc] + dt * du;
          accu[sc] = accu[sc] + h3 * du;
        }
      }
      // Stage 4 at row r-4: k4 = f(psi3), final combine, clamp, Wigner increment.
      {
        if (GENERAL && f.potential) {
          const long long o = static_cast<long long>(row_out) * nx + gx;
          vre = f.potential == 2 ? pot_m[2 * o] : pot_m[o];
          vim = f.potential == 2 ? pot_m[2 * o + 1] : T(0);
        }
        T dre, dim, dnr, du;
        const C2* xr = xin + 3 * nthreads;
        const T sP = multi ? pump_terms_value(pump_m, g.pump_term_stride, c2, m_count, L,
                                              static_cast<long long>(row_out) * nx + gx)
                           : mul_rn(s2, P[sd]);
        site_rhs<T, GENERAL, TWO>(q3[sd], xr[lt_i], xr[rt_i], q3[sa], q3[sc], m3[sd],
                             sP, k, vre, vim, f, dre, dim, dnr, v3[sd], du);
        T ore = acc[sd].x + h6 * dre;
        T oim = acc[sd].y + h6 * dim;
        T on = accn[sd] + h6 * dnr;
        on = on < T(0) ? T(0) : on;
        T ou = two ? accu[sd] + h6 * du : T(0);
        ou = ou < T(0) ? T(0) : ou;
        if (i >= 8 && i - 8 < h_eff && col_writes) {
          const long long o = static_cast<long long>(row_out) * nx + gx;
          if (NOISE) {
            WignerDraw<T>::apply(wz, k.noise_a + k.noise_b * on, ore, oim);
          }
          psi_out[member * plane + o] = C2{ore, oim};
          if (!GENERAL || f.reservoir) n_out[member * plane + o] = on;
          if (two) n_out[field2 + member * plane + o] = ou;
        }
      }
      // Publish this iteration's stage inputs for the horizontal neighbours.
      {
        C2* xo = xbuf + (j & 1) * 4 * nthreads;
        xo[tid] = p0[j];
        xo[nthreads + tid] = q1[sa];
        xo[2 * nthreads + tid] = q2[sb];
        xo[3 * nthreads + tid] = q3[sc];
      }
      row_load = row_load + 1 == ny ? 0 : row_load + 1;
      row_out = row_out + 1 == ny ? 0 : row_out + 1;
      __syncthreads();
    }
  }
}

template <typename T, bool NOISE, bool GENERAL, bool TWO>
cudaError_t launch_variant(const T* psi_in, const T* n_in, const T* pump, const T* potential,
                           T* psi_out, T* n_out, const RhsConst<T>* consts, const T* scales,
                           const unsigned long long* step_base, int step_offset, T dt,
                           const RK4Geom& g, const RK4Features& f, cudaStream_t stream) {
  using C2 = typename Cplx<T>::type;
  const int threads = g.wrap ? ((g.nx + 31) / 32) * 32 : ((g.tile_w + 8 + 31) / 32) * 32;
  if (threads > MaxThreads<T>::value) return cudaErrorInvalidConfiguration;
  const int ntx = g.wrap ? 1 : (g.nx + g.tile_w - 1) / g.tile_w;
  const int nstrips = (g.ny + g.strip_h - 1) / g.strip_h;
  const size_t smem = sizeof(C2) * 8 * static_cast<size_t>(threads);
  auto kern = rk4_stream_kernel<T, NOISE, GENERAL, TWO>;
  kern<<<dim3(ntx, nstrips, g.members), threads, smem, stream>>>(
      reinterpret_cast<const C2*>(psi_in), n_in, pump, potential, reinterpret_cast<C2*>(psi_out),
      n_out, consts, scales, step_base, step_offset, dt, g, f);
  return cudaGetLastError();
}

}  // namespace

template <typename T>
cudaError_t launch_rk4_step(const T* psi_in, const T* n_in, const T* pump, const T* potential,
                            T* psi_out, T* n_out, const RhsConst<T>* consts, const T* scales,
                            const unsigned long long* step_base, int step_offset, T dt, bool noise,
                            const RK4Geom& g, const RK4Features& f, cudaStream_t stream) {
  const bool general = f.potential != 0 || f.relax != 0 || f.reservoir != 1 || f.pump_terms > 1;
  const bool two = f.reservoir >= 2;
#define PG_RK4_VARIANT(N, G, W)                                                                  \
  launch_variant<T, N, G, W>(psi_in, n_in, pump, potential, psi_out, n_out, consts, scales,     \
                             step_base, step_offset, dt, g, f, stream)
  if (noise) {
    if (two) return PG_RK4_VARIANT(true, true, true);
    return general ? PG_RK4_VARIANT(true, true, false) : PG_RK4_VARIANT(true, false, false);
  }
  if (two) return PG_RK4_VARIANT(false, true, true);
  return general ? PG_RK4_VARIANT(false, true, false) : PG_RK4_VARIANT(false, false, false);
#undef PG_RK4_VARIANT
}

template cudaError_t launch_rk4_step<float>(const float*, const float*, const float*, const float*,
                                            float*, float*, const RhsConst<float>*, const float*,
                                            const unsigned long long*, int, float, bool,
                                            const RK4Geom&, const RK4Features&, cudaStream_t);
template cudaError_t launch_rk4_step<double>(const double*, const double*, const double*,
                                             const double*, double*, double*,
                                             const RhsConst<double>*, const double*,
                                             const unsigned long long*, int, double, bool,
                                             const RK4Geom&, const RK4Features&, cudaStream_t);

void choose_rk4_geometry(int nx, int ny, int members, int precision, int sm_count, RK4Geom* g) {
  const int max_wrap = precision == PG_DOUBLE ? 256 : 512;
  g->nx = nx;
  g->ny = ny;
  g->members = members;
  if (nx <= max_wrap) {
    g->wrap = 1;
    g->tile_w = nx;
  } else {
    g->wrap = 0;
    g->tile_w = precision == PG_DOUBLE ? 256 : 512;
  }
  const int threads = g->wrap ? ((nx + 31) / 32) * 32 : ((g->tile_w + 8 + 31) / 32) * 32;
  const int ntx = g->wrap ? 1 : (nx + g->tile_w - 1) / g->tile_w;
  // Resident blocks per SM bounded by the register file (about 96 registers per thread
  // in FP32, 192 in FP64) and by 2048 threads.
  const int regs = precision == PG_DOUBLE ? 192 : 96;
  int per_sm = 65536 / (regs * threads);
  per_sm = per_sm < 1 ? 1 : per_sm;
  if (per_sm * threads > 2048) per_sm = 2048 / threads;
  const long long slots = static_cast<long long>(sm_count > 0 ? sm_count : 152) * per_sm;
  // Pick the strip height (multiple of 4, >= 16) minimising waves * (strip + 8).
  int best_h = ny;
  double best_cost = 1e300;
  for (int h = 16; h <= ny + 3; h += 4) {
    const long long blocks = static_cast<long long>(ntx) * members * ((ny + h - 1) / h);
    const long long waves = (blocks + slots - 1) / slots;
    const double cost = static_cast<double>(waves) * (h + 8);
    if (cost < best_cost - 1e-9) {
      best_cost = cost;
      best_h = h;
    }
  }
  g->strip_h = best_h;
  g->pump_stride = 0;
  g->pot_stride = 0;
}

}  // namespace pg
