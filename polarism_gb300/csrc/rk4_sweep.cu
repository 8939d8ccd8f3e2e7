// Uneven-size sweep: members of different power-of-two grids stepped by one persistent
// launch per RK4 step.
//
// Polarism runs each grid size of a sweep as its own batch (polarism/sweep.py:98-324:
// grid.* overrides are non-batchable, so members are grouped and every group goes through
// its own SimulationController); within a batch the per-member constants are indexed by
// member (rk4_cuda_solver.py:1482-1536, config/batch_physics.py:17-60).  Here every member
// of every size lives in one packed set of arrays and one kernel advances all of them.
//
// Work decomposition.  A block covers LANES columns (LANES/2 threads, two columns each).  A
// work item is a horizontal stack of LANES/W strips of W-wide members (W = the members' nx):
// each strip is `h` consecutive rows of one member, and the strips of an item advance in
// lock step through the same register-streaming RK4 schedule as the full-width kernel
// (stage s on row r-s, an 8-row TMA ring, one shared exchange and one barrier per row).
// Every item therefore costs LANES x (h + 8) site-stages whatever W is, so equal strip
// heights give equal items; persistent blocks walk the item list with a stride of the grid
// size.  The host chooses LANES and the strip height (the autotuner times the candidates).
//
// The arithmetic per site is the full-width kernel's (rk4_site.cuh), in the same order, so a
// member's result is bitwise identical to stepping it alone with that kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "philox.cuh"
#include "pg_internal.h"
#include "rk4_site.cuh"
#include "steady_monitor.h"
#include "tma.cuh"

namespace pg {
namespace {

constexpr int kRing = 8;
constexpr int kMaxStrips = 8;      // strips per item: LANES / W <= 8
constexpr int kSweepChunk = 64;    // steps per staged chunk / CUDA graph
constexpr int kSweepSlots = 4;     // pinned staging ring depth

struct SweepMember {
  long long offset;  // first site of the member in the packed arrays
  int nx, ny;
};

struct SweepStrip {
  int member, y0;
};

struct SweepItem {
  int wl2;    // log2 of the strips' width W
  int h;      // rows per strip
  int count;  // strips in use (the rest repeat strip 0 and store nothing)
  int pad;
  SweepStrip strip[kMaxStrips];
};

template <int LANES, bool NOISE>
__global__ void __launch_bounds__(LANES / 2, (LANES >= 1024 ? 1 : 2))
    rk4_sweep_kernel(const float2* __restrict__ psi_in, const float* __restrict__ n_in,
                     const float* __restrict__ pump, float2* __restrict__ psi_out,
                     float* __restrict__ n_out, const RhsConst<float>* __restrict__ consts,
                     const SweepMember* __restrict__ members, const SweepItem* __restrict__ items,
                     const int n_items, const int n_members, const float* __restrict__ scales,
                     const unsigned long long* __restrict__ step_base, const int step_offset,
                     const float dt, const int wait_limit, int* __restrict__ err_flag,
                     const int* __restrict__ halt) {
  if (halt != nullptr && __ldcg(halt) != 0) return;  // steady-state monitor halted the sweep
  constexpr int HALF = LANES / 2;
  // One block per SM (1024 lanes): a split arrive/wait barrier lets its warps drift apart
  // by up to a row, which measured faster; with two blocks per SM the blocks already
  // interleave and a block-wide barrier is cheaper.
  constexpr bool kSplit = LANES >= 1024;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float2* ring_psi = reinterpret_cast<float2*>(smem_raw);             // [kRing][LANES]
  float* ring_n = reinterpret_cast<float*>(ring_psi + kRing * LANES); // [kRing][LANES]
  float* ring_p = ring_n + kRing * LANES;                             // [kRing][LANES]
  float4* xbuf = reinterpret_cast<float4*>(ring_p + kRing * LANES);   // [2][3][HALF]
  uint64_t* mbar = reinterpret_cast<uint64_t*>(xbuf + 6 * HALF);  // [kRing] + exchange barrier
  const uint32_t xbar = smem_u32(&mbar[kRing]);

  const int t = threadIdx.x;
  const int col0 = 2 * t;  // ring column of the thread's first site
  if (t == 0) {
    for (int s = 0; s < kRing; ++s) mbar_init(smem_u32(&mbar[s]), 1);
    if (kSplit) mbar_init(xbar, LANES / 2);
    fence_mbar_init();
  }
  __syncthreads();

  const float hh = 0.5f * dt, h6 = dt / 6.0f, h3 = dt / 3.0f;
  unsigned it = 0;  // ring uses so far; a multiple of kRing at every item start
  bool timed_out = false;

  for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
    const int wl2 = items[item].wl2;
    const int h_rows = items[item].h;
    const int count = items[item].count;
    const int W = 1 << wl2;
    const int hw = W >> 1;                 // threads per strip
    const int sub = t >> (wl2 - 1);        // the thread's strip
    const int lt = t & (hw - 1);
    const int lc = 2 * lt;                 // member-local column of the first site
    const int base = sub << wl2;           // first ring column of the strip
    const int lcol = base + (lc == 0 ? W - 1 : lc - 1);
    const int rcol = base + (lc + 2 == W ? 0 : lc + 2);
    const int lthr = sub * hw + (lt == 0 ? hw - 1 : lt - 1);
    const int rthr = sub * hw + (lt + 1 == hw ? 0 : lt + 1);
    const bool writer = sub < count;
    const SweepStrip st = items[item].strip[writer ? sub : 0];
    const SweepMember mem = members[st.member];
    const int ny = mem.ny;

    const RhsConst<float> kk = consts[st.member];
    const WideConst k = wide_const(kk);
    const uint32_t key0 = static_cast<uint32_t>(kk.seed), key1 = static_cast<uint32_t>(kk.seed >> 32);
    const float s0 = scales[(step_offset * 3 + 0) * n_members + st.member];
    const float s1 = scales[(step_offset * 3 + 1) * n_members + st.member];
    const float s2 = scales[(step_offset * 3 + 2) * n_members + st.member];
    const unsigned long long noise_step = NOISE ? step_base[0] + step_offset : 0ull;
    const PhiloxCellPrefix prefix =
        philox_cell_prefix(static_cast<uint32_t>(noise_step), static_cast<uint32_t>(noise_step >> 32),
                           1u, key0, key1);
    const float2* psi_m = psi_in + mem.offset;
    const float* n_m = n_in + mem.offset;
    const float* p_m = pump + mem.offset;
    float2* out_psi_m = psi_out + mem.offset + lc;
    float* out_n_m = n_out + mem.offset + lc;
    int row_first = (st.y0 - 4) % ny;
    if (row_first < 0) row_first += ny;
    const int n_iter = (h_rows + 8 + kRing - 1) & ~(kRing - 1);

    // Thread 0 arms the slot's barrier for the whole row (LANES * 16 bytes) before the
    // strips' leaders issue their bulk copies, so the expected bytes are always registered
    // first.
    // The give-up setting (wait_limit 0) withholds the block's first ring use (no arming, no
    // copies), so that every thread's wait for it runs out on a healthy GPU, and settles it with
    // an arrival just before its slot is armed again.  This kernel keeps no other failure
    // state in its rows: each wait is bounded (kWaitPolls), and the completion of later ring
    // slots without copies that the full-width kernel uses after a failure measured 4-6%
    // slower here, where the block barrier waits for thread 0 every row.
    auto arm = [&](int i) {
      const unsigned u = it + i;
      if (wait_limit == 0) {
        if (u == 0) return;
        if (u == kRing) mbar_arrive(smem_u32(&mbar[0]));
      }
      mbar_arrive_expect_tx(smem_u32(&mbar[i & (kRing - 1)]), LANES * 16u);
    };
    auto issue = [&](int i) {
      if (wait_limit == 0 && it + i == 0) return;
      const int slot = i & (kRing - 1);
      int row = row_first + i;
      while (row >= ny) row -= ny;
      const uint32_t bar = smem_u32(&mbar[slot]);
      const long long src = static_cast<long long>(row) << wl2;
      bulk_g2s(smem_u32(ring_psi + slot * LANES + base), psi_m + src, W * 8u, bar);
      bulk_g2s(smem_u32(ring_n + slot * LANES + base), n_m + src, W * 4u, bar);
      bulk_g2s(smem_u32(ring_p + slot * LANES + base), p_m + src, W * 4u, bar);
    };
    if (t == 0) {
      for (int i = 0; i < (kSplit ? 4 : 3) && i < n_iter; ++i) arm(i);
    }
    __syncthreads();
    if (lt == 0) {
      for (int i = 0; i < 3 && i < n_iter; ++i) issue(i);
    }

    Pair q1[4], q2[4], q3[4], acc[4];
    float2 m1[4], m2[4], m3[4], accn[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      q1[s] = q2[s] = q3[s] = acc[s] = Pair{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
      m1[s] = m2[s] = m3[s] = accn[s] = make_float2(0.f, 0.f);
    }
    int row_out = (st.y0 - 8) % ny;
    if (row_out < 0) row_out += ny;

    for (int i0 = 0; i0 < n_iter; i0 += kRing) {
      const uint32_t parity = ((it + i0) / kRing) & 1u;
#pragma unroll
      for (int j = 0; j < kRing; ++j) {
        const int i = i0 + j;
        const int ja = (j + 3) & 3, jb = (j + 2) & 3, jc = (j + 1) & 3, jd = j & 3;
        const int slot0 = j;
        const int slot1 = (j + kRing - 1) % kRing;
        const int slot2 = (j + kRing - 2) % kRing;
        const int slot3 = (j + kRing - 3) % kRing;
        const int slot4 = (j + kRing - 4) % kRing;
        if (!mbar_wait_bounded(smem_u32(&mbar[slot0]), parity, kWaitPolls)) timed_out = true;
        // Philox words and the variance-free part of the Box-Muller draw for this
        // iteration's output row, in the same straight-line code as the four stages so
        // that the integer and SFU work fills the stencil's issue gaps.
        float r2a = 0.f, sna = 0.f, csa = 0.f, r2b = 0.f, snb = 0.f, csb = 0.f;
        if (NOISE) {
          const uint32_t cell = static_cast<uint32_t>((row_out << wl2) + lc);
          const uint32_t cells[2] = {cell, cell + 1u};
          Words4 w[2];
          philox_cells(cells, prefix, w);
          WignerDraw<float>::prepare(w[0], r2a, sna, csa);
          WignerDraw<float>::prepare(w[1], r2b, snb, csb);
        }
        const float4* xin = xbuf + ((j + 1) & 1) * 3 * HALF;

        // Stage 1 at row r-1 from the ring.
        const float2* R1 = ring_psi + slot1 * LANES;
        const float4 c4 = *reinterpret_cast<const float4*>(R1 + col0);
        const float4 u4 = *reinterpret_cast<const float4*>(ring_psi + slot2 * LANES + col0);
        const float4 d4 = *reinterpret_cast<const float4*>(ring_psi + slot0 * LANES + col0);
        const float2 lt1 = R1[lcol], rt1 = R1[rcol];
        const float2 c0 = make_float2(c4.x, c4.y), c1 = make_float2(c4.z, c4.w);
        const float2 up0 = make_float2(u4.x, u4.y), up1 = make_float2(u4.z, u4.w);
        const float2 dn0 = make_float2(d4.x, d4.y), dn1 = make_float2(d4.z, d4.w);
        const float2 n1v = *reinterpret_cast<const float2*>(ring_n + slot1 * LANES + col0);
        const float2 P1 = *reinterpret_cast<const float2*>(ring_p + slot1 * LANES + col0);
        {
          float2 da, db;
          const float dna = site_rhs(c0, lt1, c1, up0, dn0, n1v.x, __fmul_rn(s0, P1.x), k, da);
          const float dnb = site_rhs(c1, c0, rt1, up1, dn1, n1v.y, __fmul_rn(s0, P1.y), k, db);
          q1[ja] = Pair{axpy2(hh, da, c0), axpy2(hh, db, c1)};
          acc[ja] = Pair{axpy2(h6, da, c0), axpy2(h6, db, c1)};
          m1[ja] = make_float2(fmaf(hh, dna, n1v.x), fmaf(hh, dnb, n1v.y));
          accn[ja] = make_float2(fmaf(h6, dna, n1v.x), fmaf(h6, dnb, n1v.y));
        }
        if (kSplit) {
          // Split barrier: wait until every thread has arrived at the end of iteration
          // i-1 (published its stage values, finished reading the exchange buffer written
          // below and the ring slot of row r-5 that the copy of row r+3 reuses).  Thread 0
          // armed that slot's barrier before arriving, so the copies follow the arming.
          const unsigned g = it + i;
          if (g > 0 && !mbar_wait_bounded(xbar, (g - 1) & 1u, kWaitPolls)) timed_out = true;
          if (lt == 0 && i + 3 < n_iter) issue(i + 3);
        }
        // Stage 2 at row r-2.
        {
          const float4 L = xin[lthr], Rr = xin[rthr];
          const float2 lt2 = make_float2(L.z, L.w), rt2 = make_float2(Rr.x, Rr.y);
          const float2 P2 = *reinterpret_cast<const float2*>(ring_p + slot2 * LANES + col0);
          const float2 n0 = *reinterpret_cast<const float2*>(ring_n + slot2 * LANES + col0);
          const Pair c = q1[jb];
          float2 da, db;
          const float dna = site_rhs(c.a, lt2, c.b, q1[jc].a, q1[ja].a, m1[jb].x,
                                     __fmul_rn(s1, P2.x), k, da);
          const float dnb = site_rhs(c.b, c.a, rt2, q1[jc].b, q1[ja].b, m1[jb].y,
                                     __fmul_rn(s1, P2.y), k, db);
          q2[jb] = Pair{axpy2(hh, da, up0), axpy2(hh, db, up1)};
          m2[jb] = make_float2(fmaf(hh, dna, n0.x), fmaf(hh, dnb, n0.y));
          acc[jb] = Pair{axpy2(h3, da, acc[jb].a), axpy2(h3, db, acc[jb].b)};
          accn[jb] = make_float2(fmaf(h3, dna, accn[jb].x), fmaf(h3, dnb, accn[jb].y));
        }
        // Stage 3 at row r-3.
        {
          const float4 L = xin[HALF + lthr], Rr = xin[HALF + rthr];
          const float2 lt3 = make_float2(L.z, L.w), rt3 = make_float2(Rr.x, Rr.y);
          const float2 P3 = *reinterpret_cast<const float2*>(ring_p + slot3 * LANES + col0);
          const float2 n0 = *reinterpret_cast<const float2*>(ring_n + slot3 * LANES + col0);
          const float4 p4 = *reinterpret_cast<const float4*>(ring_psi + slot3 * LANES + col0);
          const Pair c = q2[jc];
          float2 da, db;
          const float dna = site_rhs(c.a, lt3, c.b, q2[jd].a, q2[jb].a, m2[jc].x,
                                     __fmul_rn(s1, P3.x), k, da);
          const float dnb = site_rhs(c.b, c.a, rt3, q2[jd].b, q2[jb].b, m2[jc].y,
                                     __fmul_rn(s1, P3.y), k, db);
          q3[jc] = Pair{axpy2(dt, da, make_float2(p4.x, p4.y)), axpy2(dt, db, make_float2(p4.z, p4.w))};
          m3[jc] = make_float2(fmaf(dt, dna, n0.x), fmaf(dt, dnb, n0.y));
          acc[jc] = Pair{axpy2(h3, da, acc[jc].a), axpy2(h3, db, acc[jc].b)};
          accn[jc] = make_float2(fmaf(h3, dna, accn[jc].x), fmaf(h3, dnb, accn[jc].y));
        }
        // Stage 4 at row r-4, final combine, clamp, Wigner increment.
        {
          const float4 L = xin[2 * HALF + lthr], Rr = xin[2 * HALF + rthr];
          const float2 lt4 = make_float2(L.z, L.w), rt4 = make_float2(Rr.x, Rr.y);
          const float2 P4 = *reinterpret_cast<const float2*>(ring_p + slot4 * LANES + col0);
          const Pair c = q3[jd];
          float2 da, db;
          const float dna = site_rhs(c.a, lt4, c.b, q3[ja].a, q3[jc].a, m3[jd].x,
                                     __fmul_rn(s2, P4.x), k, da);
          const float dnb = site_rhs(c.b, c.a, rt4, q3[ja].b, q3[jc].b, m3[jd].y,
                                     __fmul_rn(s2, P4.y), k, db);
          float2 oa = axpy2(h6, da, acc[jd].a);
          float2 ob = axpy2(h6, db, acc[jd].b);
          float na = fmaf(h6, dna, accn[jd].x);
          float nb = fmaf(h6, dnb, accn[jd].y);
          na = na < 0.f ? 0.f : na;
          nb = nb < 0.f ? 0.f : nb;
          if (writer && i >= 8 && i - 8 < h_rows) {
            const long long o = static_cast<long long>(row_out) << wl2;
            if (NOISE) {
              WignerDraw<float>::add(fmaf(k.noise_b, na, k.noise_a), r2a, sna, csa, oa.x, oa.y);
              WignerDraw<float>::add(fmaf(k.noise_b, nb, k.noise_a), r2b, snb, csb, ob.x, ob.y);
            }
            *reinterpret_cast<float4*>(out_psi_m + o) = make_float4(oa.x, oa.y, ob.x, ob.y);
            *reinterpret_cast<float2*>(out_n_m + o) = make_float2(na, nb);
          }
        }
        {
          float4* xo = xbuf + (j & 1) * 3 * HALF;
          xo[t] = make_float4(q1[ja].a.x, q1[ja].a.y, q1[ja].b.x, q1[ja].b.y);
          xo[HALF + t] = make_float4(q2[jb].a.x, q2[jb].a.y, q2[jb].b.x, q2[jb].b.y);
          xo[2 * HALF + t] = make_float4(q3[jc].a.x, q3[jc].a.y, q3[jc].b.x, q3[jc].b.y);
        }
        row_out = row_out + 1 == ny ? 0 : row_out + 1;
        if (kSplit) {
          // Arm the slot the next iteration's copies fill (its last phase, row r-4, has
          // completed), then arrive on the exchange barrier.
          if (t == 0 && i + 4 < n_iter) arm(i + 4);
          mbar_arrive(xbar);
        } else {
          // The slot of row r+3 held row r-5, last read by stage 4 of the previous
          // iteration.
          if (t == 0 && i + 3 < n_iter) arm(i + 3);
          __syncthreads();
          if (lt == 0 && i + 3 < n_iter) issue(i + 3);
        }
      }
    }
    it += n_iter;
  }
  // After a timeout: copies of the last ring uses may still be in flight (a use whose copies
  // landed returns at once).
  if (t == 0 && timed_out) drain_ring(mbar, kRing, it >= kRing ? it - kRing : 0u, it);
  if (timed_out) atomicOr(err_flag, 1);
}

size_t sweep_smem(int lanes) {
  return static_cast<size_t>(kRing) * lanes * 16 + static_cast<size_t>(6) * (lanes / 2) * 16 +
         (kRing + 1) * sizeof(uint64_t);
}

template <int LANES>
cudaError_t configure_lanes() {
  cudaError_t e = cudaFuncSetAttribute(rk4_sweep_kernel<LANES, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(sweep_smem(LANES)));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(rk4_sweep_kernel<LANES, false>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(sweep_smem(LANES)));
}

template <int LANES>
int blocks_per_sm(bool noise) {
  int blocks = 0;
  cudaError_t e = noise ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                              &blocks, rk4_sweep_kernel<LANES, true>, LANES / 2, sweep_smem(LANES))
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                              &blocks, rk4_sweep_kernel<LANES, false>, LANES / 2, sweep_smem(LANES));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return blocks < 1 ? 1 : blocks;
}

// Steady-state partials per (block, member) over the packed layout: sum (rho - rho_old)^2,
// sum rho_old^2, sum rho; rho_old <- rho (polarism/simulation_controller.py:710-734).
__global__ void sweep_steady_partials_kernel(const float2* __restrict__ psi, float* __restrict__ rho_old,
                                             const SweepMember* __restrict__ members, int have_old,
                                             double* __restrict__ partials,
                                             const int* __restrict__ halt) {
  __shared__ double red[3][32];
  if (halt != nullptr && __ldcg(halt) != 0) return;  // the state no longer advances
  const SweepMember mem = members[blockIdx.y];
  const long long sites = static_cast<long long>(mem.nx) * mem.ny;
  double d2 = 0.0, o2 = 0.0, n = 0.0;
  for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < sites;
       e += static_cast<long long>(gridDim.x) * blockDim.x) {
    const float2 v = psi[mem.offset + e];
    const float rho = v.x * v.x + v.y * v.y;
    if (have_old) {
      const double old = static_cast<double>(rho_old[mem.offset + e]);
      const double diff = static_cast<double>(rho) - old;
      d2 += diff * diff;
      o2 += old * old;
    }
    n += static_cast<double>(rho);
    rho_old[mem.offset + e] = rho;
  }
  double vals[3] = {d2, o2, n};
  for (int q = 0; q < 3; ++q) {
    double v = vals[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    for (int q = 0; q < 3; ++q) {
      double v = threadIdx.x < (blockDim.x >> 5) ? red[q][threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (threadIdx.x == 0)
        partials[(static_cast<long long>(blockIdx.y) * gridDim.x + blockIdx.x) * 3 + q] = v;
    }
  }
}

constexpr int kSteadyBlocks = 64;

}  // namespace
}  // namespace pg

struct pg_sweep {
  int members = 0;
  std::vector<pg_sweep_grid> grids;
  std::vector<pg_physics> physics;
  double dt = 0.0;
  std::vector<long long> offsets;  // members + 1
  long long sites = 0;
  cudaStream_t stream = nullptr;
  int sm_count = 0;
  float* psi[2] = {nullptr, nullptr};
  float* res[2] = {nullptr, nullptr};
  float* pump = nullptr;
  pg::RhsConst<float>* consts = nullptr;
  pg::SweepMember* dmembers = nullptr;
  pg::SweepItem* ditems = nullptr;
  int item_capacity = 0;
  int n_items = 0;
  int blocks = 0;
  int lanes = 0;
  int strip_rows = 0;
  std::vector<uint8_t> active;
  float* scales = nullptr;
  unsigned long long* step_base = nullptr;
  int* err_flag = nullptr;
  int wait_limit = 100000;  // 0: the give-up setting (pg_sweep_set_wait_limit)
  int cur = 0;
  bool noise = false;
  std::vector<uint64_t> seeds;
  std::vector<double> noise_gamma, noise_R, noise_strength;
  struct Slot {
    void* host = nullptr;
    cudaEvent_t done = nullptr;
  } staging[pg::kSweepSlots];
  int next_slot = 0;
  std::map<std::pair<int, int>, cudaGraphExec_t> graphs;
  cudaEvent_t t_begin = nullptr, t_end = nullptr;
  bool timed = false;
  long long last_launches = 0;
  // Steady-state check.
  float* rho_old = nullptr;
  double* partials = nullptr;
  bool have_old = false;
  std::vector<double> norm_old;
  // Device steady-state monitor (pg_sweep_steady_update): decisions, halt word (every sweep
  // launch returns at once while it is set), per-member cell areas, and the buffer swaps so
  // far (the parity of the halting check's state).
  pg::SteadyMonitor mon;
  int* halt = nullptr;
  double* cells = nullptr;
  long long flips = 0;
  // Host waits (pg_sweep_sync_counts), as the solver handle counts them.
  long long host_syncs = 0;
  long long throttle_waits = 0;
};

namespace {

using pg::SweepItem;
using pg::SweepMember;

// Wait for everything queued on the sweep's stream (counted in host_syncs).
cudaError_t sweep_sync(pg_sweep* w) {
  ++w->host_syncs;
  return cudaStreamSynchronize(w->stream);
}

bool is_pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

int ilog2(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}

void sweep_free_graphs(pg_sweep* w) {
  for (auto& kv : w->graphs) cudaGraphExecDestroy(kv.second);
  w->graphs.clear();
}

void sweep_release(pg_sweep* w) {
  if (!w) return;
  sweep_free_graphs(w);
  for (auto& slot : w->staging) {
    if (slot.host) cudaFreeHost(slot.host);
    if (slot.done) cudaEventDestroy(slot.done);
  }
  for (int i = 0; i < 2; ++i) {
    cudaFree(w->psi[i]);
    cudaFree(w->res[i]);
  }
  cudaFree(w->pump);
  cudaFree(w->consts);
  cudaFree(w->dmembers);
  cudaFree(w->ditems);
  cudaFree(w->scales);
  cudaFree(w->step_base);
  cudaFree(w->err_flag);
  cudaFree(w->rho_old);
  cudaFree(w->partials);
  pg::steady_monitor_free(w->mon);
  cudaFree(w->halt);
  cudaFree(w->cells);
  if (w->t_begin) cudaEventDestroy(w->t_begin);
  if (w->t_end) cudaEventDestroy(w->t_end);
  if (w->stream) cudaStreamDestroy(w->stream);
  delete w;
}

int upload_sweep_consts(pg_sweep* w) {
  std::vector<pg::RhsConst<float>> v(w->members);
  for (int m = 0; m < w->members; ++m) {
    const pg_physics& p = w->physics[m];
    const pg_sweep_grid& g = w->grids[m];
    const double a = p.hbar / (2.0 * p.m_eff);
    pg::RhsConst<float>& k = v[m];
    std::memset(&k, 0, sizeof(k));
    k.ax = static_cast<float>(a / (g.dx * g.dx));
    k.ay = static_cast<float>(a / (g.dy * g.dy));
    k.w0 = static_cast<float>(2.0 * (a / (g.dx * g.dx) + a / (g.dy * g.dy)));
    k.gc = static_cast<float>(p.g_C / p.hbar);
    k.gr = static_cast<float>(p.g_R / p.hbar);
    k.gi = static_cast<float>(p.g_I / p.hbar);
    k.inv_hbar = static_cast<float>(1.0 / p.hbar);
    k.half_R = static_cast<float>(0.5 * p.R);
    k.half_gC = static_cast<float>(0.5 * p.gamma_C);
    k.R = static_cast<float>(p.R);
    k.gamma_R = static_cast<float>(p.gamma_R);
    if (w->noise) {
      const double dt_over_4dv = w->dt / (4.0 * g.dx * g.dy);
      k.noise_a = static_cast<float>(w->noise_strength[m] * w->noise_gamma[m] * dt_over_4dv);
      k.noise_b = static_cast<float>(w->noise_strength[m] * w->noise_R[m] * dt_over_4dv);
      k.seed = w->seeds[m];
    }
  }
  PG_CUDA(cudaMemcpyAsync(w->consts, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice,
                          w->stream));
  PG_CUDA(sweep_sync(w));
  return PG_OK;
}

int lanes_blocks_per_sm(int lanes, bool noise) {
  return lanes == 1024 ? pg::blocks_per_sm<1024>(noise) : pg::blocks_per_sm<512>(noise);
}

// Rebuild the item list for (lanes, strip_rows) over the active members.  Strips of equal
// width and height are packed lanes / W to an item; items are ordered tallest first so the
// strided walk of the persistent blocks spreads the heavy ones.
int build_items(pg_sweep* w, int lanes, int strip_rows) {
  std::map<std::pair<int, int>, std::vector<pg::SweepStrip>> groups;  // (wl2, h) -> strips
  for (int m = 0; m < w->members; ++m) {
    if (!w->active[m]) continue;
    const int nx = w->grids[m].nx, ny = w->grids[m].ny;
    const int wl2 = ilog2(nx);
    for (int y0 = 0; y0 < ny; y0 += strip_rows)
      groups[{wl2, std::min(strip_rows, ny - y0)}].push_back(pg::SweepStrip{m, y0});
  }
  std::vector<SweepItem> items;
  for (auto& kv : groups) {
    const int wl2 = kv.first.first, h = kv.first.second;
    const int per_item = lanes >> wl2;
    const auto& strips = kv.second;
    for (size_t b = 0; b < strips.size(); b += per_item) {
      SweepItem it{};
      it.wl2 = wl2;
      it.h = h;
      it.count = static_cast<int>(std::min<size_t>(per_item, strips.size() - b));
      for (int q = 0; q < pg::kMaxStrips; ++q)
        it.strip[q] = q < it.count ? strips[b + q] : strips[b];
      items.push_back(it);
    }
  }
  std::stable_sort(items.begin(), items.end(),
                   [](const SweepItem& a, const SweepItem& b) { return a.h > b.h; });
  if (static_cast<int>(items.size()) > w->item_capacity) {
    cudaFree(w->ditems);
    w->ditems = nullptr;
    w->item_capacity = 0;
    PG_CUDA(cudaMalloc(&w->ditems, std::max<size_t>(1, items.size()) * sizeof(SweepItem)));
    w->item_capacity = static_cast<int>(std::max<size_t>(1, items.size()));
  }
  if (!items.empty())
    PG_CUDA(cudaMemcpyAsync(w->ditems, items.data(), items.size() * sizeof(SweepItem),
                            cudaMemcpyHostToDevice, w->stream));
  PG_CUDA(sweep_sync(w));
  w->n_items = static_cast<int>(items.size());
  const long long resident = static_cast<long long>(lanes_blocks_per_sm(lanes, true)) * w->sm_count;
  w->blocks = static_cast<int>(std::max<long long>(1, std::min<long long>(resident, w->n_items)));
  w->lanes = lanes;
  w->strip_rows = strip_rows;
  sweep_free_graphs(w);
  return PG_OK;
}

int check_tiling(const pg_sweep* w, int lanes, int strip_rows) {
  PG_CHECK(lanes == 512 || lanes == 1024, PG_ERR_INVALID, "pg_sweep_set_tiling: lanes must be 512 or 1024");
  PG_CHECK(strip_rows >= 8 && strip_rows <= (1 << 20), PG_ERR_INVALID,
           "pg_sweep_set_tiling: strip_rows must be at least 8");
  for (int m = 0; m < w->members; ++m) {
    const int nx = w->grids[m].nx;
    PG_CHECK(nx <= lanes && nx * pg::kMaxStrips >= lanes, PG_ERR_INVALID,
             "pg_sweep_set_tiling: every member's nx must lie in [lanes / 8, lanes]");
  }
  return PG_OK;
}

// Default tiling before any measurement: the narrowest lanes that hold every member, and
// the strip height whose modelled time (waves of equal items x rows per item incl. the
// 8-row pipeline fill) is smallest.
void default_tiling(const pg_sweep* w, int* lanes, int* strip_rows) {
  int max_nx = 0, max_ny = 0;
  for (const auto& g : w->grids) {
    max_nx = std::max(max_nx, g.nx);
    max_ny = std::max(max_ny, g.ny);
  }
  *lanes = max_nx <= 512 ? 512 : 1024;
  const long long resident = static_cast<long long>(lanes_blocks_per_sm(*lanes, true)) * w->sm_count;
  double best = 1e300;
  int best_h = 8;
  for (int h = 8; h <= std::max(8, max_ny); h *= 2) {
    std::map<std::pair<int, int>, long long> strips;
    for (const auto& g : w->grids)
      for (int y0 = 0; y0 < g.ny; y0 += h) strips[{g.nx, std::min(h, g.ny - y0)}] += 1;
    double rows = 0.0;
    long long items = 0;
    for (const auto& kv : strips) {
      const long long per = *lanes / kv.first.first;
      const long long n = (kv.second + per - 1) / per;
      items += n;
      rows += static_cast<double>(n) * (((kv.first.second + 8 + 7) / 8) * 8);
    }
    const double waves = std::ceil(static_cast<double>(items) / static_cast<double>(resident));
    const double per_item = rows / std::max<long long>(1, items);
    const double cost = waves * per_item;
    if (cost < best) {
      best = cost;
      best_h = h;
    }
  }
  *strip_rows = best_h;
}

cudaError_t launch_sweep_step(pg_sweep* w, int from, int step_offset) {
  const int to = 1 - from;
  if (w->n_items == 0) return cudaSuccess;
  const size_t smem = pg::sweep_smem(w->lanes);
  const float dt = static_cast<float>(w->dt);
#define PG_SWEEP_LAUNCH(L, N)                                                                   \
  pg::rk4_sweep_kernel<L, N><<<w->blocks, L / 2, smem, w->stream>>>(                            \
      reinterpret_cast<const float2*>(w->psi[from]), w->res[from], w->pump,                    \
      reinterpret_cast<float2*>(w->psi[to]), w->res[to], w->consts, w->dmembers, w->ditems,     \
      w->n_items, w->members, w->scales, w->step_base, step_offset, dt, w->wait_limit,           \
      w->err_flag, w->halt)
  if (w->lanes == 1024) {
    if (w->noise) PG_SWEEP_LAUNCH(1024, true); else PG_SWEEP_LAUNCH(1024, false);
  } else {
    if (w->noise) PG_SWEEP_LAUNCH(512, true); else PG_SWEEP_LAUNCH(512, false);
  }
#undef PG_SWEEP_LAUNCH
  return cudaGetLastError();
}

int sweep_graph_for(pg_sweep* w, int len, int parity, cudaGraphExec_t* out) {
  auto key = std::make_pair(len, parity);
  auto it = w->graphs.find(key);
  if (it != w->graphs.end()) {
    *out = it->second;
    return PG_OK;
  }
  cudaGraph_t graph = nullptr;
  PG_CUDA(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t launch_err = cudaSuccess;
  for (int k = 0; k < len && launch_err == cudaSuccess; ++k)
    launch_err = launch_sweep_step(w, (parity + k) & 1, k);
  cudaError_t end_err = cudaStreamEndCapture(w->stream, &graph);
  if (launch_err != cudaSuccess || end_err != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    pg::set_error(std::string("sweep graph capture failed: ") +
                  cudaGetErrorString(launch_err != cudaSuccess ? launch_err : end_err));
    return PG_ERR_CUDA;
  }
  cudaGraphExec_t exec = nullptr;
  cudaError_t inst = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (inst != cudaSuccess) {
    pg::set_error(std::string("sweep graph instantiate failed: ") + cudaGetErrorString(inst));
    return PG_ERR_CUDA;
  }
  w->graphs[key] = exec;
  *out = exec;
  return PG_OK;
}

int stage_sweep_coefficients(pg_sweep* w, const double* coeffs, int len, int64_t step) {
  pg_sweep::Slot& slot = w->staging[w->next_slot];
  w->next_slot = (w->next_slot + 1) % pg::kSweepSlots;
  if (cudaEventQuery(slot.done) == cudaErrorNotReady) ++w->throttle_waits;
  PG_CUDA(cudaEventSynchronize(slot.done));
  const size_t count = static_cast<size_t>(len) * 3 * w->members;
  float* h = static_cast<float*>(slot.host);
  for (size_t i = 0; i < count; ++i) h[i] = static_cast<float>(coeffs[i]);
  const size_t base_off = static_cast<size_t>(pg::kSweepChunk) * 3 * w->members * 4;
  unsigned char* host = static_cast<unsigned char*>(slot.host);
  const unsigned long long b = static_cast<unsigned long long>(step);
  std::memcpy(host + base_off, &b, sizeof(b));
  if (count) PG_CUDA(cudaMemcpyAsync(w->scales, host, count * 4, cudaMemcpyHostToDevice, w->stream));
  PG_CUDA(cudaMemcpyAsync(w->step_base, host + base_off, sizeof(b), cudaMemcpyHostToDevice, w->stream));
  PG_CUDA(cudaEventRecord(slot.done, w->stream));
  return PG_OK;
}

int sweep_check_flag(pg_sweep* w) {
  int flag = 0;
  PG_CUDA(cudaMemcpyAsync(&flag, w->err_flag, sizeof(int), cudaMemcpyDeviceToHost, w->stream));
  PG_CUDA(sweep_sync(w));
  if (flag) {
    cudaMemsetAsync(w->err_flag, 0, sizeof(int), w->stream);
    sweep_sync(w);
    pg::set_error("a bounded device wait timed out; results of the last advance are invalid");
    return PG_ERR_TIMEOUT;
  }
  return PG_OK;
}

}  // namespace

extern "C" {

int pg_sweep_create(int32_t members, const pg_sweep_grid* grids, const pg_physics* physics,
                    double dt, pg_sweep** out) {
  PG_CHECK(grids && physics && out, PG_ERR_INVALID, "pg_sweep_create: null argument");
  PG_CHECK(members >= 1, PG_ERR_INVALID, "pg_sweep_create: members must be >= 1");
  PG_CHECK(dt > 0, PG_ERR_INVALID, "pg_sweep_create: dt must be positive");
  for (int m = 0; m < members; ++m) {
    const pg_sweep_grid& g = grids[m];
    PG_CHECK(is_pow2(g.nx) && g.nx >= 64 && g.nx <= 1024, PG_ERR_UNSUPPORTED,
             "pg_sweep_create: every member's nx must be a power of two in [64, 1024]");
    PG_CHECK(g.ny >= 4 && static_cast<long long>(g.nx) * g.ny < (1ll << 31), PG_ERR_INVALID,
             "pg_sweep_create: ny must be >= 4 and a member below 2^31 sites");
    PG_CHECK(g.dx > 0 && g.dy > 0, PG_ERR_INVALID, "pg_sweep_create: dx and dy must be positive");
  }
  *out = nullptr;
  pg_sweep* w = new pg_sweep();
  w->members = members;
  w->grids.assign(grids, grids + members);
  w->physics.assign(physics, physics + members);
  w->dt = dt;
  w->active.assign(members, 1);
  w->offsets.resize(members + 1);
  w->offsets[0] = 0;
  for (int m = 0; m < members; ++m)
    w->offsets[m + 1] = w->offsets[m] + static_cast<long long>(grids[m].nx) * grids[m].ny;
  w->sites = w->offsets[members];
  auto fail = [&](cudaError_t e, const char* what) {
    pg::set_error(std::string("pg_sweep_create: ") + what + ": " + cudaGetErrorString(e));
    sweep_release(w);
    return PG_ERR_CUDA;
  };
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(e, "cudaGetDevice");
  if ((e = cudaDeviceGetAttribute(&w->sm_count, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return fail(e, "device attribute");
  if ((e = cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return fail(e, "stream");
  const size_t sites = static_cast<size_t>(w->sites);
  for (int i = 0; i < 2; ++i) {
    if ((e = cudaMalloc(&w->psi[i], sites * 8)) != cudaSuccess) return fail(e, "psi buffers");
    if ((e = cudaMalloc(&w->res[i], sites * 4)) != cudaSuccess) return fail(e, "reservoir buffers");
    cudaMemsetAsync(w->psi[i], 0, sites * 8, w->stream);
    cudaMemsetAsync(w->res[i], 0, sites * 4, w->stream);
  }
  if ((e = cudaMalloc(&w->pump, sites * 4)) != cudaSuccess) return fail(e, "pump buffer");
  cudaMemsetAsync(w->pump, 0, sites * 4, w->stream);
  if ((e = cudaMalloc(&w->consts, members * sizeof(pg::RhsConst<float>))) != cudaSuccess)
    return fail(e, "constants");
  if ((e = cudaMalloc(&w->dmembers, members * sizeof(SweepMember))) != cudaSuccess)
    return fail(e, "member table");
  std::vector<SweepMember> table(members);
  for (int m = 0; m < members; ++m) table[m] = SweepMember{w->offsets[m], grids[m].nx, grids[m].ny};
  if ((e = cudaMemcpyAsync(w->dmembers, table.data(), members * sizeof(SweepMember),
                           cudaMemcpyHostToDevice, w->stream)) != cudaSuccess)
    return fail(e, "member table upload");
  if ((e = cudaMalloc(&w->scales, static_cast<size_t>(pg::kSweepChunk) * 3 * members * 4)) != cudaSuccess)
    return fail(e, "scales");
  if ((e = cudaMalloc(&w->step_base, sizeof(unsigned long long))) != cudaSuccess)
    return fail(e, "step base");
  cudaMemsetAsync(w->step_base, 0, sizeof(unsigned long long), w->stream);
  if ((e = cudaMalloc(&w->err_flag, sizeof(int))) != cudaSuccess) return fail(e, "error flag");
  cudaMemsetAsync(w->err_flag, 0, sizeof(int), w->stream);
  if ((e = cudaMalloc(&w->halt, sizeof(int))) != cudaSuccess) return fail(e, "halt word");
  cudaMemsetAsync(w->halt, 0, sizeof(int), w->stream);
  std::vector<double> cells(members);
  for (int m = 0; m < members; ++m) cells[m] = grids[m].dx * grids[m].dy;
  if ((e = cudaMalloc(&w->cells, members * sizeof(double))) != cudaSuccess) return fail(e, "cells");
  if ((e = cudaMemcpyAsync(w->cells, cells.data(), members * sizeof(double), cudaMemcpyHostToDevice,
                           w->stream)) != cudaSuccess)
    return fail(e, "cells upload");
  if ((e = pg::configure_lanes<512>()) != cudaSuccess) return fail(e, "kernel attributes");
  if ((e = pg::configure_lanes<1024>()) != cudaSuccess) return fail(e, "kernel attributes");
  const size_t staging_bytes = static_cast<size_t>(pg::kSweepChunk) * 3 * members * 4 + 64;
  for (auto& slot : w->staging) {
    if ((e = cudaMallocHost(&slot.host, staging_bytes)) != cudaSuccess) return fail(e, "staging");
    if ((e = cudaEventCreateWithFlags(&slot.done, cudaEventDisableTiming)) != cudaSuccess)
      return fail(e, "staging event");
  }
  if ((e = cudaEventCreate(&w->t_begin)) != cudaSuccess) return fail(e, "timing event");
  if ((e = cudaEventCreate(&w->t_end)) != cudaSuccess) return fail(e, "timing event");
  int rc = upload_sweep_consts(w);
  int lanes = 0, rows = 0;
  default_tiling(w, &lanes, &rows);
  if (rc == PG_OK && check_tiling(w, lanes, rows) != PG_OK) {
    pg::set_error("pg_sweep_create: with a 1024-wide member every member needs nx >= 128");
    rc = PG_ERR_UNSUPPORTED;
  }
  if (rc == PG_OK) rc = build_items(w, lanes, rows);
  if (rc != PG_OK) {
    sweep_release(w);
    return rc;
  }
  *out = w;
  return PG_OK;
}

void pg_sweep_destroy(pg_sweep* w) {
  if (w && w->stream) cudaStreamSynchronize(w->stream);
  sweep_release(w);
}

void* pg_sweep_stream(pg_sweep* w) { return w ? static_cast<void*>(w->stream) : nullptr; }

int64_t pg_sweep_total_sites(pg_sweep* w) { return w ? w->sites : -1; }

int pg_sweep_offsets(pg_sweep* w, int64_t* offsets) {
  PG_CHECK(w && offsets, PG_ERR_INVALID, "pg_sweep_offsets: null argument");
  for (int m = 0; m <= w->members; ++m) offsets[m] = w->offsets[m];
  return PG_OK;
}

int pg_sweep_set_state(pg_sweep* w, const void* psi, const void* res, int on_device) {
  PG_CHECK(w && psi && res, PG_ERR_INVALID, "pg_sweep_set_state: null argument");
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  PG_CUDA(cudaMemcpyAsync(w->psi[w->cur], psi, static_cast<size_t>(w->sites) * 8, kind, w->stream));
  PG_CUDA(cudaMemcpyAsync(w->res[w->cur], res, static_cast<size_t>(w->sites) * 4, kind, w->stream));
  PG_CUDA(sweep_sync(w));
  return PG_OK;
}

int pg_sweep_get_state(pg_sweep* w, void* psi, void* res, int on_device) {
  PG_CHECK(w && psi, PG_ERR_INVALID, "pg_sweep_get_state: null argument");
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  PG_CUDA(cudaMemcpyAsync(psi, w->psi[w->cur], static_cast<size_t>(w->sites) * 8, kind, w->stream));
  if (res)
    PG_CUDA(cudaMemcpyAsync(res, w->res[w->cur], static_cast<size_t>(w->sites) * 4, kind, w->stream));
  PG_CUDA(sweep_sync(w));
  return sweep_check_flag(w);
}

int pg_sweep_state_pointers(pg_sweep* w, void** psi, void** res) {
  PG_CHECK(w && psi && res, PG_ERR_INVALID, "pg_sweep_state_pointers: null argument");
  *psi = w->psi[w->cur];
  *res = w->res[w->cur];
  return PG_OK;
}

int pg_sweep_set_pump(pg_sweep* w, const void* envelope, int on_device) {
  PG_CHECK(w && envelope, PG_ERR_INVALID, "pg_sweep_set_pump: null argument");
  PG_CUDA(cudaMemcpyAsync(w->pump, envelope, static_cast<size_t>(w->sites) * 4,
                          on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, w->stream));
  PG_CUDA(sweep_sync(w));
  return PG_OK;
}

int pg_sweep_set_noise(pg_sweep* w, const uint64_t* seeds, const double* gamma,
                       const double* scattering, const double* strength) {
  PG_CHECK(w, PG_ERR_INVALID, "pg_sweep_set_noise: null sweep");
  if (!seeds) {
    w->noise = false;
  } else {
    PG_CHECK(gamma && scattering && strength, PG_ERR_INVALID, "pg_sweep_set_noise: null member arrays");
    const int m = w->members;
    w->seeds.assign(seeds, seeds + m);
    w->noise_gamma.assign(gamma, gamma + m);
    w->noise_R.assign(scattering, scattering + m);
    w->noise_strength.assign(strength, strength + m);
    w->noise = true;
  }
  sweep_free_graphs(w);
  return upload_sweep_consts(w);
}

int pg_sweep_set_tiling(pg_sweep* w, int32_t lanes, int32_t strip_rows) {
  PG_CHECK(w, PG_ERR_INVALID, "pg_sweep_set_tiling: null sweep");
  int rc = check_tiling(w, lanes, strip_rows);
  if (rc != PG_OK) return rc;
  PG_CUDA(sweep_sync(w));
  return build_items(w, lanes, strip_rows);
}

int pg_sweep_set_wait_limit(pg_sweep* w, int32_t polls) {
  PG_CHECK(w, PG_ERR_INVALID, "pg_sweep_set_wait_limit: null sweep");
  PG_CHECK(polls == 0 || polls == pg::kWaitPolls, PG_ERR_INVALID,
           "pg_sweep_set_wait_limit: polls must be 0 (the give-up setting: every wait gives up at "
           "once) or 100000 (the kernel's compiled bound)");
  PG_CUDA(sweep_sync(w));
  w->wait_limit = polls;
  sweep_free_graphs(w);  // captured launches carry the old setting
  return PG_OK;
}

int pg_sweep_get_tiling(pg_sweep* w, int32_t* lanes, int32_t* strip_rows, int32_t* items,
                        int32_t* blocks) {
  PG_CHECK(w && lanes && strip_rows && items && blocks, PG_ERR_INVALID,
           "pg_sweep_get_tiling: null argument");
  *lanes = w->lanes;
  *strip_rows = w->strip_rows;
  *items = w->n_items;
  *blocks = w->blocks;
  return PG_OK;
}

int pg_sweep_set_active(pg_sweep* w, const uint8_t* active) {
  PG_CHECK(w, PG_ERR_INVALID, "pg_sweep_set_active: null sweep");
  PG_CUDA(sweep_sync(w));
  for (int m = 0; m < w->members; ++m) w->active[m] = active ? (active[m] ? 1 : 0) : 1;
  // An inactive member keeps its state: copy it into the other parity buffer now, since
  // the ping-pong buffers of active members swap every step and the state of an
  // inactive one must be found under the current parity at every later step.
  for (int m = 0; m < w->members; ++m) {
    if (w->active[m]) continue;
    const size_t off = static_cast<size_t>(w->offsets[m]);
    const size_t n = static_cast<size_t>(w->offsets[m + 1] - w->offsets[m]);
    PG_CUDA(cudaMemcpyAsync(w->psi[1 - w->cur] + 2 * off, w->psi[w->cur] + 2 * off, n * 8,
                            cudaMemcpyDeviceToDevice, w->stream));
    PG_CUDA(cudaMemcpyAsync(w->res[1 - w->cur] + off, w->res[w->cur] + off, n * 4,
                            cudaMemcpyDeviceToDevice, w->stream));
  }
  return build_items(w, w->lanes, w->strip_rows);
}

int pg_sweep_advance(pg_sweep* w, int64_t start_step, int32_t n_steps, const double* stage_scales,
                     int use_graphs) {
  PG_CHECK(w && stage_scales, PG_ERR_INVALID, "pg_sweep_advance: null argument");
  PG_CHECK(n_steps >= 0, PG_ERR_INVALID, "pg_sweep_advance: negative step count");
  w->last_launches = 0;
  PG_CUDA(cudaEventRecord(w->t_begin, w->stream));
  int done = w->n_items == 0 ? n_steps : 0;  // every member frozen: nothing to launch
  while (done < n_steps) {
    int len = std::min(pg::kSweepChunk, n_steps - done);
    const bool graph = use_graphs && len >= 2;
    if (graph && (len & 1)) len -= 1;
    int rc = stage_sweep_coefficients(w, stage_scales + static_cast<size_t>(done) * 3 * w->members,
                                      len, start_step + done);
    if (rc != PG_OK) return rc;
    if (graph) {
      cudaGraphExec_t exec = nullptr;
      rc = sweep_graph_for(w, len, w->cur, &exec);
      if (rc != PG_OK) return rc;
      PG_CUDA(cudaGraphLaunch(exec, w->stream));
    } else {
      for (int k = 0; k < len; ++k) PG_CUDA(launch_sweep_step(w, (w->cur + k) & 1, k));
    }
    w->cur = (w->cur + len) & 1;
    w->flips += len;
    w->last_launches += w->n_items ? len : 0;
    done += len;
  }
  PG_CUDA(cudaEventRecord(w->t_end, w->stream));
  w->timed = true;
  return PG_OK;
}

int pg_sweep_last_time_ms(pg_sweep* w, float* ms) {
  PG_CHECK(w && ms, PG_ERR_INVALID, "pg_sweep_last_time_ms: null argument");
  PG_CHECK(w->timed, PG_ERR_INVALID, "pg_sweep_last_time_ms: no advance call yet");
  PG_CUDA(cudaEventSynchronize(w->t_end));
  PG_CUDA(cudaEventElapsedTime(ms, w->t_begin, w->t_end));
  return sweep_check_flag(w);
}

int64_t pg_sweep_last_launch_count(pg_sweep* w) { return w ? w->last_launches : -1; }

int pg_sweep_synchronize(pg_sweep* w) {
  PG_CHECK(w, PG_ERR_INVALID, "pg_sweep_synchronize: null sweep");
  PG_CUDA(sweep_sync(w));
  return sweep_check_flag(w);
}

int pg_sweep_steady_check(pg_sweep* w, double* rel_density, double* rel_norm, double* norms) {
  PG_CHECK(w && rel_density && rel_norm && norms, PG_ERR_INVALID, "pg_sweep_steady_check: null argument");
  const int m = w->members;
  if (!w->rho_old) PG_CUDA(cudaMalloc(&w->rho_old, static_cast<size_t>(w->sites) * 4));
  if (!w->partials)
    PG_CUDA(cudaMalloc(&w->partials, static_cast<size_t>(m) * pg::kSteadyBlocks * 3 * sizeof(double)));
  pg::sweep_steady_partials_kernel<<<dim3(pg::kSteadyBlocks, m), 256, 0, w->stream>>>(
      reinterpret_cast<const float2*>(w->psi[w->cur]), w->rho_old, w->dmembers, w->have_old ? 1 : 0,
      w->partials, nullptr);
  PG_CUDA(cudaGetLastError());
  std::vector<double> host(static_cast<size_t>(3) * pg::kSteadyBlocks * m);
  PG_CUDA(cudaMemcpyAsync(host.data(), w->partials, host.size() * sizeof(double),
                          cudaMemcpyDeviceToHost, w->stream));
  PG_CUDA(sweep_sync(w));
  if (w->norm_old.size() != static_cast<size_t>(m)) w->norm_old.assign(m, 0.0);
  for (int mm = 0; mm < m; ++mm) {
    double d2 = 0, o2 = 0, n = 0;
    for (int b = 0; b < pg::kSteadyBlocks; ++b) {
      const double* p = &host[(static_cast<size_t>(mm) * pg::kSteadyBlocks + b) * 3];
      d2 += p[0];
      o2 += p[1];
      n += p[2];
    }
    const double norm = n * w->grids[mm].dx * w->grids[mm].dy;
    norms[mm] = norm;
    if (w->have_old) {
      rel_density[mm] = std::sqrt(d2) / std::max(std::sqrt(o2), 1e-30);
      rel_norm[mm] = std::fabs(norm - w->norm_old[mm]) / std::max(w->norm_old[mm], 1e-30);
    } else {
      rel_density[mm] = rel_norm[mm] = INFINITY;
    }
    w->norm_old[mm] = norm;
  }
  w->have_old = true;
  return sweep_check_flag(w);
}

int pg_sweep_steady_reset(pg_sweep* w) {
  PG_CHECK(w, PG_ERR_INVALID, "pg_sweep_steady_reset: null sweep");
  const int m = w->members;
  if (!w->rho_old) PG_CUDA(cudaMalloc(&w->rho_old, static_cast<size_t>(w->sites) * 4));
  if (!w->partials)
    PG_CUDA(cudaMalloc(&w->partials, static_cast<size_t>(m) * pg::kSteadyBlocks * 3 * sizeof(double)));
  PG_CUDA(pg::steady_monitor_alloc(w->mon, m));
  PG_CUDA(pg::steady_monitor_reset(w->mon, w->halt, w->stream));
  w->have_old = false;
  return PG_OK;
}

int pg_sweep_steady_update(pg_sweep* w, int64_t step, int32_t record, double rtol,
                           int32_t halt_when_all_stopped) {
  PG_CHECK(w, PG_ERR_INVALID, "pg_sweep_steady_update: null sweep");
  PG_CHECK(rtol >= 0.0, PG_ERR_INVALID, "pg_sweep_steady_update: negative rtol");
  if (!w->mon.norm_old) {
    const int rc = pg_sweep_steady_reset(w);
    if (rc != PG_OK) return rc;
  }
  pg::sweep_steady_partials_kernel<<<dim3(pg::kSteadyBlocks, w->members), 256, 0, w->stream>>>(
      reinterpret_cast<const float2*>(w->psi[w->cur]), w->rho_old, w->dmembers,
      w->mon.have_old ? 1 : 0, w->partials, w->halt);
  PG_CUDA(cudaGetLastError());
  PG_CUDA(pg::steady_monitor_decide(w->mon, w->partials, pg::kSteadyBlocks, w->cells, 0.0,
                                    record ? 1 : 0, rtol, static_cast<long long>(step), w->flips,
                                    halt_when_all_stopped ? 1 : 0, w->halt, w->stream));
  return PG_OK;
}

int pg_sweep_steady_poll(pg_sweep* w, int32_t* stopped, int64_t* updates_done) {
  PG_CHECK(w && stopped && updates_done, PG_ERR_INVALID, "pg_sweep_steady_poll: null argument");
  pg::steady_monitor_poll(w->mon, stopped, updates_done);
  return PG_OK;
}

int pg_sweep_steady_results(pg_sweep* w, double* rel_density, double* rel_norm, double* norms,
                            int64_t* stop_steps, int64_t* halt_step) {
  PG_CHECK(w, PG_ERR_INVALID, "pg_sweep_steady_results: null sweep");
  PG_CHECK(w->mon.norm_old, PG_ERR_INVALID, "pg_sweep_steady_results: no steady-state check has been made");
  const int m = w->members;
  std::vector<double> res(static_cast<size_t>(3) * m);
  std::vector<long long> stops(m);
  long long hs[2] = {-1, -1};  // step and buffer swaps of the halting check
  int halted = 0;
  PG_CUDA(pg::steady_monitor_fetch(w->mon, w->halt, res.data(), stops.data(), &halted, hs, w->stream));
  PG_CUDA(sweep_sync(w));
  for (int mm = 0; mm < m; ++mm) {
    if (rel_density) rel_density[mm] = res[mm];
    if (rel_norm) rel_norm[mm] = res[m + mm];
    if (norms) norms[mm] = res[2 * m + mm];
    if (stop_steps) stop_steps[mm] = stops[mm];
  }
  if (halted) {
    // Sweep launches after the halt returned without writing while the host swapped the
    // buffers for each: the halting check's state is under the parity it had then.  Clear
    // the halt so that the sweep steps again.
    w->cur ^= static_cast<int>((w->flips - hs[1]) & 1);
    w->flips = hs[1];
    PG_CUDA(cudaMemsetAsync(w->halt, 0, sizeof(int), w->stream));
    PG_CUDA(sweep_sync(w));
  }
  if (halt_step) *halt_step = halted ? hs[0] : -1;
  return sweep_check_flag(w);
}

int pg_sweep_sync_counts(pg_sweep* w, int64_t* host_syncs, int64_t* throttle_waits) {
  PG_CHECK(w && host_syncs && throttle_waits, PG_ERR_INVALID, "pg_sweep_sync_counts: null argument");
  *host_syncs = w->host_syncs;
  *throttle_waits = w->throttle_waits;
  return PG_OK;
}

}  // extern "C"
