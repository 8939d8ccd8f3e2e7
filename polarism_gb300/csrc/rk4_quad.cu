// Full-width fused RK4 step for FP32 rows of 512 or 1024 sites with four adjacent sites per
// thread: the four-site form of the full-width kernel in rk4_wide.cu, chosen with RK4 kernel
// kind 3.  It executes about 27% fewer instructions per site than the two-site form but keeps
// only eight warps on an SM (four sites need ~230 registers a thread), which leaves the stage
// chains' latencies exposed: 124.7 against 130.8 G site-updates/s at 1024^2 x 32 with Wigner
// noise, so the two-site form is the default.
//
// Same mathematics and, site by site, the same operation order as rk4_wide.cu and rk4.cu
// (polarism/model.py:89-127, polarism/solver/rk4_fdm_solver.py:36-82,
// single_reservoir.py:70-98, Wigner increment of rk4_cuda_solver.py:518-532), so its results
// are bitwise those of the two-site form.  What changes is the mapping onto the SM:
//
// * A thread owns four adjacent columns, so a 1024-site row is 256 threads (8 warps).  Two of
//   each site's four horizontal neighbours of a stage are in the thread's own registers; only
//   the two edge columns go through the shared-memory exchange, and the per-row costs (the
//   ring and exchange barriers, the loop and address arithmetic, the Philox key schedule)
//   are shared by four sites instead of two.
// * The per-site scalars (density, nonlinear frequency, gain, reservoir derivative, pump
//   product, reservoir stage updates) of two sites are computed as one packed FP32x2
//   instruction; each lane is the same FP32 operation with the same rounding as the scalar
//   form.
// * Everything else follows rk4_wide.cu: rows of psi0, n0 and the pump envelope stream into an
//   8-row shared-memory ring through 1-D bulk copies three rows ahead, the four stages run
//   on rows r-1 .. r-4 of a register-streamed pipeline, a split arrive/wait mbarrier orders
//   the exchange, blocks are persistent over the member-major row space, and every wait is
//   bounded.
#include <algorithm>

#include "philox.cuh"
#include "pg_internal.h"
#include "rk4_site.cuh"
#include "tma.cuh"
#include "wide_internal.h"

namespace pg {
namespace {

constexpr int kQRing = 8;  // rows resident: r-4 .. r plus three in flight

template <int NX>
struct QuadShape {
  static constexpr int THREADS = NX / 4;
  // Ring (psi 8 B + n 4 B + pump 4 B per site and row), exchange [parity][stage][thread]
  // of float4 (the thread's first and last site), the ring barriers and the exchange barrier,
  // and one word of thread 0's (its feed mode; see feed) with padding.
  static constexpr size_t SMEM = static_cast<size_t>(kQRing) * NX * 16 +
                                 static_cast<size_t>(2) * 3 * THREADS * 16 +
                                 (kQRing + 2) * sizeof(uint64_t);
};

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 dup(float a) { return make_float2(a, a); }

// Right-hand side at the thread's four sites, site_rhs of rk4_site.cuh with the per-site
// scalars of sites (0, 1) and (2, 3) paired into FP32x2 instructions.  c: centre values,
// L / R: the left neighbour of site 0 and the right neighbour of site 3, up / dn: the rows
// above and below, n01 / n23: reservoir, sp01 / sp23: pump products.  Writes d = dpsi/dt and
// returns dn/dt in dn01 / dn23.
__device__ __forceinline__ void quad_rhs(const float2 (&c)[4], float2 L, float2 R,
                                         const float2 (&up)[4], const float2 (&dn)[4], float2 n01,
                                         float2 n23, float2 sp01, float2 sp23, const WideConst& k,
                                         float2 (&d)[4], float2& dn01, float2& dn23) {
  float2 nl[4];
  float rho[4];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const float2 lt = s == 0 ? L : c[s - 1];
    const float2 rt = s == 3 ? R : c[s + 1];
    const float2 sx = __fadd2_rn(lt, rt);
    const float2 sy = __fadd2_rn(up[s], dn[s]);
    nl[s] = __ffma2_rn(k.nay, sy, __fmul2_rn(k.nax, sx));
    rho[s] = fmaf(c[s].x, c[s].x, c[s].y * c[s].y);
  }
  const float2 rho01 = f2(rho[0], rho[1]), rho23 = f2(rho[2], rho[3]);
  const float2 w01 = __ffma2_rn(dup(k.gr), n01, __ffma2_rn(dup(k.gc), rho01, dup(k.w0)));
  const float2 w23 = __ffma2_rn(dup(k.gr), n23, __ffma2_rn(dup(k.gc), rho23, dup(k.w0)));
  const float2 gl01 = __ffma2_rn(dup(k.half_R), n01, dup(-k.half_gC));
  const float2 gl23 = __ffma2_rn(dup(k.half_R), n23, dup(-k.half_gC));
  const float w[4] = {w01.x, w01.y, w23.x, w23.y};
  const float gl[4] = {gl01.x, gl01.y, gl23.x, gl23.y};
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const float2 u = __ffma2_rn(dup(w[s]), c[s], nl[s]);  // w c - a lap_neighbours
    d[s].x = fmaf(gl[s], c[s].x, u.y);
    d[s].y = fmaf(gl[s], c[s].y, -u.x);
  }
  // -(R rho + gamma_R) n + sP with the negation folded into the constants (exact).
  dn01 = __ffma2_rn(__ffma2_rn(dup(-k.R), rho01, dup(-k.gamma_R)), n01, sp01);
  dn23 = __ffma2_rn(__ffma2_rn(dup(-k.R), rho23, dup(-k.gamma_R)), n23, sp23);
}

__device__ __forceinline__ void load4(const float2* p, float2 (&v)[4]) {
  const float4 a = *reinterpret_cast<const float4*>(p);
  const float4 b = *reinterpret_cast<const float4*>(p + 2);
  v[0] = f2(a.x, a.y);
  v[1] = f2(a.z, a.w);
  v[2] = f2(b.x, b.y);
  v[3] = f2(b.z, b.w);
}

__device__ __forceinline__ void load_pairs(const float* p, float2& lo, float2& hi) {
  const float4 a = *reinterpret_cast<const float4*>(p);
  lo = f2(a.x, a.y);
  hi = f2(a.z, a.w);
}

template <int NX, bool NOISE>
__global__ void __launch_bounds__(QuadShape<NX>::THREADS, 1)
    rk4_quad_kernel(const float2* __restrict__ psi_in, const float* __restrict__ n_in,
                    const float* __restrict__ pump, float2* __restrict__ psi_out,
                    float* __restrict__ n_out, const RhsConst<float>* __restrict__ consts,
                    const float* __restrict__ scales,
                    const unsigned long long* __restrict__ step_base, const int step_offset,
                    const float dt, const WideGeom g, int* __restrict__ err_flag) {
  constexpr int T = QuadShape<NX>::THREADS;
  if (g.halt != nullptr && __ldcg(g.halt) != 0) return;  // steady-state monitor halted the run
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float2* ring_psi = reinterpret_cast<float2*>(smem_raw);           // [kQRing][NX]
  float* ring_n = reinterpret_cast<float*>(ring_psi + kQRing * NX);  // [kQRing][NX]
  float* ring_p = ring_n + kQRing * NX;                              // [kQRing][NX]
  float4* xbuf = reinterpret_cast<float4*>(ring_p + kQRing * NX);    // [2][3][T]
  uint64_t* mbar = reinterpret_cast<uint64_t*>(xbuf + 6 * T);        // [kQRing + 1]
  const uint32_t xbar = smem_u32(&mbar[kQRing]);
  volatile int* feed_mode = reinterpret_cast<volatile int*>(&mbar[kQRing + 1]);

  const int ny = g.ny;
  const int t = threadIdx.x;
  const int col0 = 4 * t;
  const int lcol = t == 0 ? NX - 1 : col0 - 1;
  const int rcol = t == T - 1 ? 0 : col0 + 4;
  const int lthr = t == 0 ? T - 1 : t - 1;
  const int rthr = t == T - 1 ? 0 : t + 1;
  const long long plane = static_cast<long long>(NX) * ny;
  constexpr uint32_t kRowBytes = NX * 16u;

  if (t == 0) {
    for (int s = 0; s < kQRing; ++s) mbar_init(smem_u32(&mbar[s]), 1);
    mbar_init(xbar, T);
    fence_mbar_init();
    *feed_mode = 0;
  }
  __syncthreads();

  const long long total_rows = static_cast<long long>(g.members) * ny;
  const long long r_begin = total_rows * blockIdx.x / gridDim.x;
  const long long r_end = total_rows * (blockIdx.x + 1) / gridDim.x;
  const float hh = 0.5f * dt, h6 = dt / 6.0f, h3 = dt / 3.0f;
  unsigned it = 0;  // ring uses so far; a multiple of kQRing at every segment start
  bool timed_out = false;

  long long gr = r_begin;
  while (gr < r_end) {
    const int member = static_cast<int>(gr / ny);
    const int ya = static_cast<int>(gr - static_cast<long long>(member) * ny);
    const int yb = static_cast<int>(min(static_cast<long long>(ny), ya + (r_end - gr)));
    gr += yb - ya;
    const int h_rows = yb - ya;
    const int n_iter = (h_rows + 8 + kQRing - 1) & ~(kQRing - 1);

    const RhsConst<float> kk = consts[member];
    const WideConst k = wide_const(kk);
    const uint32_t key0 = static_cast<uint32_t>(kk.seed), key1 = static_cast<uint32_t>(kk.seed >> 32);
    const float s0 = scales[(step_offset * 3 + 0) * g.members + member];
    const float s1 = scales[(step_offset * 3 + 1) * g.members + member];
    const float s2 = scales[(step_offset * 3 + 2) * g.members + member];
    const unsigned long long noise_step = NOISE ? step_base[0] + step_offset : 0ull;
    const PhiloxCellPrefix prefix =
        philox_cell_prefix(static_cast<uint32_t>(noise_step), static_cast<uint32_t>(noise_step >> 32),
                           1u, key0, key1);
    const float2* psi_m = psi_in + member * plane;
    const float* n_m = n_in + member * plane;
    const float* p_m = pump + member * g.pump_stride;
    float2* out_psi_m = psi_out + member * plane + col0;
    float* out_n_m = n_out + member * plane + col0;
    int row_first = (ya - 4) % ny;
    if (row_first < 0) row_first += ny;

    // Bulk copies of iteration i (row ya - 4 + i) into ring slot i % kQRing.
    auto issue = [&](int i) {
      const int slot = i & (kQRing - 1);
      int row = row_first + i;
      while (row >= ny) row -= ny;
      const uint32_t bar = smem_u32(&mbar[slot]);
      mbar_arrive_expect_tx(bar, kRowBytes);
      const long long ro = static_cast<long long>(row) * NX;
      bulk_g2s(smem_u32(ring_psi + slot * NX), psi_m + ro, NX * 8u, bar);
      bulk_g2s(smem_u32(ring_n + slot * NX), n_m + ro, NX * 4u, bar);
      bulk_g2s(smem_u32(ring_p + slot * NX), p_m + ro, NX * 4u, bar);
    };
    // Thread 0 feeds ring use it + i: the row copies, or, once one of its own waits has given
    // up (tested at the barrier of the use it has just waited for), an empty arrival; the
    // give-up setting withholds and later settles the block's first use, as in rk4_wide.cu.
    auto feed = [&](int i) {
      const unsigned u = it + i;
      int mode = *feed_mode;
      if (mode == 0 && i >= 3) {
        // the use thread 0 has just waited for: open means its wait gave up
        const unsigned w = u - 3;
        if (!mbar_test(smem_u32(&mbar[w & (kQRing - 1)]), (w / kQRing) & 1u)) *feed_mode = mode = 1;
      }
      if (g.wait_limit == 0) {
        if (u == 0) return;
        if (u == kQRing) mbar_arrive(smem_u32(&mbar[0]));
      }
      if (mode == 0) {
        issue(i);
        return;
      }
      mbar_fill_empty(smem_u32(&mbar[i & (kQRing - 1)]), u, kQRing);
    };
    if (t == 0) {
      for (int i = 0; i < 3 && i < n_iter; ++i) feed(i);
    }

    // Register rings [row slot][site] (complex) and [row slot] of site pairs (reservoir).
    float2 q1[4][4], q2[4][4], q3[4][4], acc[4][4];
    float2 m1[4][2], m2[4][2], m3[4][2], accn[4][2];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
#pragma unroll
      for (int s = 0; s < 4; ++s) q1[r][s] = q2[r][s] = q3[r][s] = acc[r][s] = f2(0.f, 0.f);
#pragma unroll
      for (int p = 0; p < 2; ++p) m1[r][p] = m2[r][p] = m3[r][p] = accn[r][p] = f2(0.f, 0.f);
    }
    int row_out = (ya - 8) % ny;
    if (row_out < 0) row_out += ny;

    // Four iterations per unrolled body (the register rings have four slots); the ring slot of
    // row r is (i0 + j) % kQRing with i0 % kQRing in {0, 4}.
    for (int i0 = 0; i0 < n_iter; i0 += 4) {
      const int base = i0 & (kQRing - 1);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int i = i0 + j;
        const int ja = (j + 3) & 3, jb = (j + 2) & 3, jc = (j + 1) & 3, jd = j & 3;
        const int slot0 = base + j;                                // row r
        const int slot1 = (base + j + kQRing - 1) & (kQRing - 1);  // row r-1
        const int slot2 = (base + j + kQRing - 2) & (kQRing - 1);  // row r-2
        const int slot3 = (base + j + kQRing - 3) & (kQRing - 1);  // row r-3
        const int slot4 = (base + j + kQRing - 4) & (kQRing - 1);  // row r-4
        const uint32_t parity = ((it + i) / kQRing) & 1u;
        if (!mbar_wait_bounded(smem_u32(&mbar[slot0]), parity, kWaitPolls)) timed_out = true;

        // Philox words and the variance-free part of the Box-Muller draw of this
        // iteration's output row (four cells), interleaved with the stages by the compiler.
        float r2[4] = {0.f, 0.f, 0.f, 0.f}, sn[4] = {0.f, 0.f, 0.f, 0.f}, cs[4] = {0.f, 0.f, 0.f, 0.f};
        if (NOISE) {
          const uint32_t cell = static_cast<uint32_t>(row_out * NX + col0);
          const uint32_t cells[4] = {cell, cell + 1u, cell + 2u, cell + 3u};
          Words4 w[4];
          philox_cells(cells, prefix, w);
#pragma unroll
          for (int s = 0; s < 4; ++s) WignerDraw<float>::prepare(w[s], r2[s], sn[s], cs[s]);
        }

        // Stage 1 at row r-1 from the ring: k1 = f(psi0).
        float2 c[4], u[4], dv[4], d[4];
        load4(ring_psi + slot1 * NX + col0, c);
        load4(ring_psi + slot2 * NX + col0, u);   // psi0 at row r-2 (stage 2 needs it too)
        load4(ring_psi + slot0 * NX + col0, dv);
        {
          const float2 L = ring_psi[slot1 * NX + lcol], R = ring_psi[slot1 * NX + rcol];
          float2 n01, n23, p01, p23, dn01, dn23;
          load_pairs(ring_n + slot1 * NX + col0, n01, n23);
          load_pairs(ring_p + slot1 * NX + col0, p01, p23);
          quad_rhs(c, L, R, u, dv, n01, n23, __fmul2_rn(dup(s0), p01), __fmul2_rn(dup(s0), p23),
                   k, d, dn01, dn23);
#pragma unroll
          for (int s = 0; s < 4; ++s) {
            q1[ja][s] = axpy2(hh, d[s], c[s]);
            acc[ja][s] = axpy2(h6, d[s], c[s]);
          }
          m1[ja][0] = __ffma2_rn(dup(hh), dn01, n01);
          m1[ja][1] = __ffma2_rn(dup(hh), dn23, n23);
          accn[ja][0] = __ffma2_rn(dup(h6), dn01, n01);
          accn[ja][1] = __ffma2_rn(dup(h6), dn23, n23);
        }
        // Split barrier: every thread has published its stage values of iteration i-1 and
        // finished every read of it (the exchange half written below, and the ring slot of
        // row r-5 that the copy of row r+3 reuses).
        {
          const unsigned gi = it + i;
          if (gi > 0 && !mbar_wait_bounded(xbar, (gi - 1) & 1u, kWaitPolls)) timed_out = true;
          if (t == 0 && i + 3 < n_iter) feed(i + 3);
        }
        const float4* xin = xbuf + ((j + 1) & 1) * 3 * T;
        // Stage 2 at row r-2: k2 = f(psi1).
        {
          const float2 L = make_float2(xin[lthr].z, xin[lthr].w);
          const float2 R = make_float2(xin[rthr].x, xin[rthr].y);
          float2 n0a, n0b, p01, p23, dn01, dn23;
          load_pairs(ring_p + slot2 * NX + col0, p01, p23);
          load_pairs(ring_n + slot2 * NX + col0, n0a, n0b);
          quad_rhs(q1[jb], L, R, q1[jc], q1[ja], m1[jb][0], m1[jb][1], __fmul2_rn(dup(s1), p01),
                   __fmul2_rn(dup(s1), p23), k, d, dn01, dn23);
#pragma unroll
          for (int s = 0; s < 4; ++s) {
            q2[jb][s] = axpy2(hh, d[s], u[s]);
            acc[jb][s] = axpy2(h3, d[s], acc[jb][s]);
          }
          m2[jb][0] = __ffma2_rn(dup(hh), dn01, n0a);
          m2[jb][1] = __ffma2_rn(dup(hh), dn23, n0b);
          accn[jb][0] = __ffma2_rn(dup(h3), dn01, accn[jb][0]);
          accn[jb][1] = __ffma2_rn(dup(h3), dn23, accn[jb][1]);
        }
        // Stage 3 at row r-3: k3 = f(psi2).
        {
          const float2 L = make_float2(xin[T + lthr].z, xin[T + lthr].w);
          const float2 R = make_float2(xin[T + rthr].x, xin[T + rthr].y);
          float2 n0a, n0b, p01, p23, dn01, dn23, p0[4];
          load_pairs(ring_p + slot3 * NX + col0, p01, p23);
          load_pairs(ring_n + slot3 * NX + col0, n0a, n0b);
          load4(ring_psi + slot3 * NX + col0, p0);
          quad_rhs(q2[jc], L, R, q2[jd], q2[jb], m2[jc][0], m2[jc][1], __fmul2_rn(dup(s1), p01),
                   __fmul2_rn(dup(s1), p23), k, d, dn01, dn23);
#pragma unroll
          for (int s = 0; s < 4; ++s) {
            q3[jc][s] = axpy2(dt, d[s], p0[s]);
            acc[jc][s] = axpy2(h3, d[s], acc[jc][s]);
          }
          m3[jc][0] = __ffma2_rn(dup(dt), dn01, n0a);
          m3[jc][1] = __ffma2_rn(dup(dt), dn23, n0b);
          accn[jc][0] = __ffma2_rn(dup(h3), dn01, accn[jc][0]);
          accn[jc][1] = __ffma2_rn(dup(h3), dn23, accn[jc][1]);
        }
        // Stage 4 at row r-4: k4 = f(psi3), final combine, clamp, Wigner increment.
        {
          const float2 L = make_float2(xin[2 * T + lthr].z, xin[2 * T + lthr].w);
          const float2 R = make_float2(xin[2 * T + rthr].x, xin[2 * T + rthr].y);
          float2 p01, p23, dn01, dn23;
          load_pairs(ring_p + slot4 * NX + col0, p01, p23);
          quad_rhs(q3[jd], L, R, q3[ja], q3[jc], m3[jd][0], m3[jd][1], __fmul2_rn(dup(s2), p01),
                   __fmul2_rn(dup(s2), p23), k, d, dn01, dn23);
          float2 o[4];
#pragma unroll
          for (int s = 0; s < 4; ++s) o[s] = axpy2(h6, d[s], acc[jd][s]);
          const float2 na01 = __ffma2_rn(dup(h6), dn01, accn[jd][0]);
          const float2 na23 = __ffma2_rn(dup(h6), dn23, accn[jd][1]);
          float nv[4] = {na01.x, na01.y, na23.x, na23.y};
#pragma unroll
          for (int s = 0; s < 4; ++s) nv[s] = nv[s] < 0.f ? 0.f : nv[s];
          if (i >= 8 && i - 8 < h_rows) {
            const long long o_row = static_cast<long long>(row_out) * NX;
            if (NOISE) {
#pragma unroll
              for (int s = 0; s < 4; ++s)
                WignerDraw<float>::add(fmaf(k.noise_b, nv[s], k.noise_a), r2[s], sn[s], cs[s],
                                       o[s].x, o[s].y);
            }
            float4* po = reinterpret_cast<float4*>(out_psi_m + o_row);
            po[0] = make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
            po[1] = make_float4(o[2].x, o[2].y, o[3].x, o[3].y);
            *reinterpret_cast<float4*>(out_n_m + o_row) = make_float4(nv[0], nv[1], nv[2], nv[3]);
          }
        }
        // Publish the edge sites' stage inputs for the neighbouring threads.
        {
          float4* xo = xbuf + (j & 1) * 3 * T;
          xo[t] = make_float4(q1[ja][0].x, q1[ja][0].y, q1[ja][3].x, q1[ja][3].y);
          xo[T + t] = make_float4(q2[jb][0].x, q2[jb][0].y, q2[jb][3].x, q2[jb][3].y);
          xo[2 * T + t] = make_float4(q3[jc][0].x, q3[jc][0].y, q3[jc][3].x, q3[jc][3].y);
        }
        row_out = row_out + 1 == ny ? 0 : row_out + 1;
        mbar_arrive(xbar);
      }
    }
    it += n_iter;
  }
  // After a wait of thread 0's gave up: copies it issued may still be in flight in the last
  // ring uses; a use it filled empty completes at once.
  if (t == 0 && (timed_out || *feed_mode != 0)) drain_ring(mbar, kQRing, it >= kQRing ? it - kQRing : 0u, it);
  if (timed_out) atomicOr(err_flag, 1);
}

template <int NX>
cudaError_t configure_quad_shape() {
  const int smem = static_cast<int>(QuadShape<NX>::SMEM);
  cudaError_t e = cudaFuncSetAttribute(rk4_quad_kernel<NX, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(rk4_quad_kernel<NX, false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  return e;
}

template <int NX>
int quad_blocks_per_sm() {
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, rk4_quad_kernel<NX, true>,
                                                    QuadShape<NX>::THREADS,
                                                    QuadShape<NX>::SMEM) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return blocks < 1 ? 1 : blocks;
}

template <int NX>
cudaError_t launch_quad_shape(const float* psi_in, const float* n_in, const float* pump,
                              float* psi_out, float* n_out, const RhsConst<float>* consts,
                              const float* scales, const unsigned long long* step_base,
                              int step_offset, float dt, bool noise, const WideGeom& g,
                              int* err_flag, cudaStream_t stream) {
  const float2* pin = reinterpret_cast<const float2*>(psi_in);
  float2* pout = reinterpret_cast<float2*>(psi_out);
  constexpr int threads = QuadShape<NX>::THREADS;
  constexpr size_t smem = QuadShape<NX>::SMEM;
  if (noise)
    rk4_quad_kernel<NX, true><<<g.blocks, threads, smem, stream>>>(
        pin, n_in, pump, pout, n_out, consts, scales, step_base, step_offset, dt, g, err_flag);
  else
    rk4_quad_kernel<NX, false><<<g.blocks, threads, smem, stream>>>(
        pin, n_in, pump, pout, n_out, consts, scales, step_base, step_offset, dt, g, err_flag);
  return cudaGetLastError();
}

}  // namespace

bool quad_rk4_supported(int nx, int ny) { return (nx == 512 || nx == 1024) && ny >= 4; }

cudaError_t configure_quad_rk4() {
  cudaError_t e = configure_quad_shape<512>();
  if (e == cudaSuccess) e = configure_quad_shape<1024>();
  return e;
}

int quad_rk4_grid(int nx, int ny, int members, int sm_count) {
  const int per_sm = nx == 512 ? quad_blocks_per_sm<512>() : quad_blocks_per_sm<1024>();
  const long long rows = static_cast<long long>(members) * ny;
  const long long blocks = static_cast<long long>(per_sm) * std::max(1, sm_count);
  return static_cast<int>(std::min(blocks, std::max<long long>(1, rows / 16)));
}

cudaError_t launch_rk4_quad(const float* psi_in, const float* n_in, const float* pump,
                            float* psi_out, float* n_out, const RhsConst<float>* consts,
                            const float* scales, const unsigned long long* step_base,
                            int step_offset, float dt, bool noise, const WideGeom& g,
                            int* err_flag, cudaStream_t stream) {
  if (g.nx == 1024)
    return launch_quad_shape<1024>(psi_in, n_in, pump, psi_out, n_out, consts, scales, step_base,
                                   step_offset, dt, noise, g, err_flag, stream);
  if (g.nx == 512)
    return launch_quad_shape<512>(psi_in, n_in, pump, psi_out, n_out, consts, scales, step_base,
                                  step_offset, dt, noise, g, err_flag, stream);
  return cudaErrorInvalidValue;
}

}  // namespace pg
