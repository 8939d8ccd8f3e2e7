// Full-width fused RK4 step for FP32 rows of 128 to 1024 sites, and of multiples of 1024 sites
// up to 16384 as 1024-site bands (2048-8192: one band per CTA of a thread-block cluster).
//
// Same mathematics and operation order as rk4.cu (polarism/model.py:89-127,
// polarism/solver/rk4_fdm_solver.py:36-82, single_reservoir.py:70-98, Wigner
// increment of rk4_cuda_solver.py:518-532), mapped differently onto the SM:
//
// * A block spans the whole periodic row (2 columns per thread, nx/2 threads), so
//   there is no horizontal halo and 1024-wide rows use 16 balanced warps.  Wider rows
//   split into 1024-column bands: a cluster of CTAs per row range (one band each, the two
//   edge columns of stages 2-4 pushed to the neighbouring CTA's shared memory with
//   st.async), or past the portable cluster size, independent blocks that recompute a
//   four-column halo.
// * Rows of psi0, n0 and the pump envelope stream into an 8-row shared-memory ring
//   through 1-D bulk copies (TMA) that complete on per-slot mbarriers, three rows
//   ahead of use.  Stage 1 reads its whole stencil straight from the ring; stages 2-4
//   get vertical neighbours from per-thread register rings and horizontal ones from
//   one double-buffered shared exchange per row, ordered (for 1024-site rows) by a
//   split arrive/wait mbarrier rather than a block-wide barrier, so warps drift apart
//   by up to a row.
// * Complex arithmetic uses packed FP32x2 instructions (__ffma2_rn and friends), and so do the
//   per-site scalars of a thread's two sites (pair_rhs: density terms, gain, reservoir
//   derivative, pump products, reservoir stage updates), lane for lane the scalar operations.
// * The exchange holds each thread's two columns in two arrays, so a stage is published with
//   two 8-byte stores straight from the register pairs the packed arithmetic produced.
// * Blocks are persistent: block c advances rows [c R / G, (c+1) R / G) of the
//   member-major row space (R = members * ny rows; BAND: members * bands * ny; CLUSTER:
//   c and G count clusters), restarting the 4-row pipeline fill whenever it crosses into
//   the next member (or band).
#include <algorithm>

#include "philox.cuh"
#include "pg_internal.h"
#include "rk4_site.cuh"
#include "tma.cuh"
#include "wide_internal.h"

namespace pg {
namespace {

constexpr int kRing = 8;          // rows resident: r-4..r plus three in flight

// At least 512 resident threads per SM for every row width (128 registers a thread).
// Threads of a block: two sites each over the shared-memory row.  Rows wider than NX = 1024
// sites go in 1024-column bands whose shared-memory rows carry four halo columns on each side:
// BAND recomputes the halo (a block owns the band alone; the four stages each reach one
// column further, so 516 threads rounded up to whole warps), CLUSTER gives each band of a row
// to one CTA of a thread-block cluster (NX / 2 threads) and exchanges the two edge columns of
// each stage through distributed shared memory.
template <int NX, bool BAND, bool CLUSTER = false>
struct WideShape {
  static constexpr int W = (BAND || CLUSTER) ? NX + 8 : NX;  // sites per shared-memory row
  static constexpr int ACTIVE = BAND ? W / 2 : NX / 2;      // threads that own two sites
  static constexpr int THREADS = BAND ? ((ACTIVE + 31) / 32) * 32 : NX / 2;
};
// Barriers after the ring's: the row exchange, then (CLUSTER) the left and right
// neighbours' edge deliveries, two of each by iteration parity.
constexpr int kBars = kRing + 5;
// CLUSTER inboxes after the barriers: [from left, from right][parity][stage] edge values,
// then thread 0's feed mode (0 copies, 1 empty arrivals; see feed) and padding.
constexpr int kInbox = 2 * 2 * 3;
constexpr int kFailWords = 2;
constexpr uint32_t kEdgeBytes = 3 * 8;  // one iteration's delivery: three stage values

// TERMS: separable lasers whose envelopes stream beside psi and n_R (one ring row each); the
// pump of a stage is sum_l c_l E_l with products and partial sums rounded apart, as the tiled
// kernel forms it.  Several lasers run on rows of at most 1024 sites.
template <int NX, bool NOISE, bool GENERAL, bool BAND, bool CLUSTER = false, int TERMS = 1>
__global__ void __launch_bounds__(WideShape<NX, BAND, CLUSTER>::THREADS, (NX >= 1024 ? 1 : 1024 / NX))
    rk4_wide_kernel(const float2* __restrict__ psi_in, const float* __restrict__ n_in,
                    const float* __restrict__ pump, float2* __restrict__ psi_out,
                    float* __restrict__ n_out, const RhsConst<float>* __restrict__ consts,
                    const float* __restrict__ scales,
                    const unsigned long long* __restrict__ step_base, const int step_offset,
                    const float dt, const WideGeom g, int* __restrict__ err_flag) {
  constexpr int W = WideShape<NX, BAND, CLUSTER>::W;
  constexpr int ACTIVE = WideShape<NX, BAND, CLUSTER>::ACTIVE;
  constexpr int HALF = WideShape<NX, BAND, CLUSTER>::THREADS;  // exchange-buffer stride
  constexpr bool HALO = BAND || CLUSTER;  // shared-memory rows carry the band's halo
  static_assert(TERMS == 1 || !HALO, "several lasers run on rows of at most 1024 sites");
  // One block per SM (1024-site rows): a split arrive/wait barrier lets its warps drift
  // apart by up to a row, which measured faster; with several blocks per SM the blocks
  // already interleave and a block-wide barrier is cheaper.
  constexpr bool kSplit = NX >= 1024;
  if (g.halt != nullptr && __ldcg(g.halt) != 0) return;  // steady-state monitor halted the run
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float2* ring_psi = reinterpret_cast<float2*>(smem_raw);          // [kRing][W]
  float* ring_n = reinterpret_cast<float*>(ring_psi + kRing * W);  // [kRing][W]
  float* ring_p = ring_n + kRing * W;                              // [kRing][TERMS][W]
  // Exchange: each thread's first (xa) and second (xb) column of the three stage inputs,
  // [parity][stage][thread]; two 8-byte stores a stage keep the values in the register pairs
  // the packed arithmetic produced them in.
  float2* xa = reinterpret_cast<float2*>(ring_p + kRing * TERMS * W);  // [2][3][HALF]
  float2* xb = xa + 6 * HALF;                                  // [2][3][HALF]
  uint64_t* mbar = reinterpret_cast<uint64_t*>(xb + 6 * HALF);  // [kBars]
  const uint32_t xbar = smem_u32(&mbar[kRing]);
  // CLUSTER: at the end of each iteration the left neighbour's thread HALF-1 pushes its
  // right column's three stage values into in_left[parity] with st.async, completing on
  // from_left[parity]; the right neighbour's thread 0 pushes its left column into in_right.
  // Only this CTA's edge threads (0 and HALF-1) read them, after arming and waiting.
  const uint32_t from_left = smem_u32(&mbar[kRing + 1]);
  const uint32_t from_right = smem_u32(&mbar[kRing + 3]);
  float2* in_left = reinterpret_cast<float2*>(mbar + kBars);  // [2][3]
  float2* in_right = in_left + 6;                              // [2][3]
  volatile int* feed_mode = reinterpret_cast<volatile int*>(in_right + 6);

  const int ny = g.ny;
  const int t = threadIdx.x;
  // BAND: threads past the band's sites repeat the last active thread's work and write
  // nothing; the halo columns have no left / right neighbour in the band (their results are
  // not written either).
  const int tc = BAND ? min(t, ACTIVE - 1) : t;
  const bool owner = !BAND || t < ACTIVE;
  // Shared-memory column of the thread's first site (CLUSTER: past the left halo).
  const int col0 = CLUSTER ? 2 * tc + 4 : 2 * tc;
  const int lcol = CLUSTER ? col0 - 1
                 : BAND    ? (col0 == 0 ? 0 : col0 - 1)
                           : (col0 == 0 ? NX - 1 : col0 - 1);
  const int rcol = CLUSTER ? col0 + 2
                 : BAND    ? (col0 + 2 >= W ? col0 + 1 : col0 + 2)
                           : (col0 + 2 == NX ? 0 : col0 + 2);
  // Owners of lcol / rcol in the exchange (CLUSTER: the edge threads' neighbours are the
  // neighbouring CTAs' edge threads, read through distributed shared memory).
  const int lthr = BAND ? max(tc - 1, 0) : (t == 0 ? HALF - 1 : t - 1);
  const int rthr = BAND ? min(tc + 1, ACTIVE - 1) : (t + 1 == HALF ? 0 : t + 1);
  const int gnx = HALO ? g.nx : NX;  // sites per grid row
  const int bands = HALO ? g.nx / NX : 1;
  // CLUSTER: the CTA's band is its rank; clusters share out the rows.
  const int rank = CLUSTER ? static_cast<int>(cluster_ctarank()) : 0;
  const int unit_id = CLUSTER ? static_cast<int>(blockIdx.x) / bands : static_cast<int>(blockIdx.x);
  const int units = CLUSTER ? static_cast<int>(gridDim.x) / bands : static_cast<int>(gridDim.x);
  const uint32_t left_rank = CLUSTER ? static_cast<uint32_t>((rank + bands - 1) % bands) : 0u;
  const uint32_t right_rank = CLUSTER ? static_cast<uint32_t>((rank + 1) % bands) : 0u;
  const long long plane = static_cast<long long>(gnx) * ny;
  constexpr uint32_t kRowBytes = W * (12u + 4u * TERMS);

  if (t == 0) {
    for (int s = 0; s < kRing; ++s) mbar_init(smem_u32(&mbar[s]), 1);
    if (kSplit) mbar_init(xbar, HALF);
    if (CLUSTER)
      for (int s = kRing + 1; s < kBars; ++s) mbar_init(smem_u32(&mbar[s]), 1);
    fence_mbar_init();
    *feed_mode = 0;
  }
  // CLUSTER: every CTA's barriers exist before any neighbour arrives on them.
  if (CLUSTER) cluster_sync_all(); else __syncthreads();
  // Neighbour addresses (CLUSTER): the inbox and barrier each edge thread delivers to.
  const uint32_t left_inbox = CLUSTER ? map_shared_rank(smem_u32(in_right), left_rank) : 0u;
  const uint32_t left_bar = CLUSTER ? map_shared_rank(from_right, left_rank) : 0u;
  const uint32_t right_inbox = CLUSTER ? map_shared_rank(smem_u32(in_left), right_rank) : 0u;
  const uint32_t right_bar = CLUSTER ? map_shared_rank(from_left, right_rank) : 0u;
  // Horizontal neighbours of stage s (0..2) from the exchange of parity `xb`: the left
  // neighbour's right column and the right neighbour's left column.
  auto xchg = [&](int par, int s, float2& lt, float2& rt) {
    const int o = (par * 3 + s) * HALF;
    lt = CLUSTER && t == 0 ? in_left[par * 3 + s] : xb[o + lthr];
    rt = CLUSTER && t == HALF - 1 ? in_right[par * 3 + s] : xa[o + rthr];
  };
  // CLUSTER edge threads: arm and wait for the neighbours' delivery of iteration g.
  auto receive = [&](unsigned g) {
    const uint32_t q = g & 1u, par = (g >> 1) & 1u;
    bool ok = true;
    if (t == 0) {
      mbar_arrive_expect_tx(from_left + 8u * q, kEdgeBytes);
      ok = mbar_wait_bounded(from_left + 8u * q, par, kWaitPolls);
    }
    if (t == HALF - 1) {
      mbar_arrive_expect_tx(from_right + 8u * q, kEdgeBytes);
      ok = mbar_wait_bounded(from_right + 8u * q, par, kWaitPolls);
    }
    return ok;
  };

  const long long total_rows = static_cast<long long>(g.members) * (CLUSTER ? 1 : bands) * ny;
  const long long r_begin = total_rows * unit_id / units;
  const long long r_end = total_rows * (unit_id + 1) / units;
  const float hh = 0.5f * dt, h6 = dt / 6.0f, h3 = dt / 3.0f;
  unsigned it = 0;  // ring uses so far; always a multiple of kRing at a segment start
  bool timed_out = false;

  long long gr = r_begin;
  while (gr < r_end) {
    // Row space [member][band][row]; a segment stays within one (member, band).
    const long long unit = gr / ny;
    const int member = CLUSTER ? static_cast<int>(unit) : static_cast<int>(unit / bands);
    const int band = CLUSTER ? rank : static_cast<int>(unit % bands);
    const int ya = static_cast<int>(gr - unit * ny);
    const int yb = static_cast<int>(min(static_cast<long long>(ny), ya + (r_end - gr)));
    gr += yb - ya;
    const int h_rows = yb - ya;
    const int n_iter = (h_rows + 8 + kRing - 1) & ~(kRing - 1);

    const RhsConst<float> kk = consts[member];
    const WideConst k = wide_const(kk);
    const uint32_t key0 = static_cast<uint32_t>(kk.seed), key1 = static_cast<uint32_t>(kk.seed >> 32);
    // Coefficient sample q of laser l: scales[[step][q][l][member]].  With one laser the
    // stage multiplies s_q by the envelope; with several, pump_pair forms sum_l c_ql E_l and
    // the stage's factor is 1 (a multiply by 1 rounds nothing).
    float cs[3][TERMS];
#pragma unroll
    for (int q = 0; q < 3; ++q)
#pragma unroll
      for (int l = 0; l < TERMS; ++l)
        cs[q][l] = scales[(static_cast<long long>(step_offset * 3 + q) * TERMS + l) * g.members + member];
    const float s0 = TERMS == 1 ? cs[0][0] : 1.f;
    const float s1 = TERMS == 1 ? cs[1][0] : 1.f;
    const float s2 = TERMS == 1 ? cs[2][0] : 1.f;
    const unsigned long long noise_step = NOISE ? step_base[0] + step_offset : 0ull;
    const PhiloxCellPrefix prefix =
        philox_cell_prefix(static_cast<uint32_t>(noise_step), static_cast<uint32_t>(noise_step >> 32),
                           1u, key0, key1);
    // Grid column of shared-memory column c: the band starts four columns left of its first
    // written column.
    const int gc0 = HALO ? band * NX - 4 : 0;
    const int gcol0 = gc0 + col0;                                    // may lie outside [0, gnx)
    const int gcol0w = gcol0 < 0 ? gcol0 + gnx : (gcol0 >= gnx ? gcol0 - gnx : gcol0);
    const bool writes = owner && (!HALO || (col0 >= 4 && col0 < 4 + NX));
    const float2* psi_m = psi_in + member * plane;
    const float* n_m = n_in + member * plane;
    const float* p_m = pump + member * g.pump_stride;
    const float* pot_m = GENERAL && g.pot_kind != 0
                             ? g.pot + member * g.pot_stride * (g.pot_kind == 2 ? 2 : 1)
                             : nullptr;
    // General variant: the potential of the thread's two sites on `row` as (Re, Im) pairs.
    auto pot_at = [&](int row, float2& va, float2& vb) {
      va = vb = make_float2(0.f, 0.f);
      if (GENERAL && pot_m != nullptr) {
        const long long o = static_cast<long long>(row) * gnx + gcol0w;
        if (g.pot_kind == 2) {
          const float4 v = *reinterpret_cast<const float4*>(pot_m + 2 * o);
          va = make_float2(v.x, v.y);
          vb = make_float2(v.z, v.w);
        } else {
          const float2 v = *reinterpret_cast<const float2*>(pot_m + o);
          va.x = v.x;
          vb.x = v.y;
        }
      }
    };
    // Right-hand side at the thread's two sites (a, b): L / R the outer neighbours, up / dn
    // the rows above and below, n2 the reservoir pair, sP = s P the pump products, va / vb the
    // potential (general variant); returns the reservoir derivatives.
    auto rhs2 = [&](float2 ca, float2 cb, float2 L, float2 R, float2 upa, float2 upb, float2 dna,
                    float2 dnb, float2 n2, float s, float2 P, float2 va, float2 vb, float2& da,
                    float2& db) -> float2 {
      if (GENERAL) {
        const bool rl = g.relax != 0;
        const float x = site_rhs_general(ca, L, cb, upa, dna, n2.x, __fmul_rn(s, P.x), k, va.x,
                                         va.y, rl, da);
        const float y = site_rhs_general(cb, ca, R, upb, dnb, n2.y, __fmul_rn(s, P.y), k, vb.x,
                                         vb.y, rl, db);
        return make_float2(x, y);
      }
      return pair_rhs(ca, cb, L, R, upa, upb, dna, dnb, n2, __fmul2_rn(make_float2(s, s), P), k,
                      da, db);
    };
    // The pump envelope pair of ring slot `slot` (one laser), or the stage pump of coefficient
    // sample q (several).
    auto pump_pair = [&](int slot, int q) -> float2 {
      const float* base = ring_p + slot * TERMS * W + col0;
      const float2 e0 = *reinterpret_cast<const float2*>(base);
      if (TERMS == 1) return e0;
      float2 v = make_float2(__fmul_rn(cs[q][0], e0.x), __fmul_rn(cs[q][0], e0.y));
#pragma unroll
      for (int l = 1; l < TERMS; ++l) {
        const float2 e = *reinterpret_cast<const float2*>(base + l * W);
        v = make_float2(__fadd_rn(v.x, __fmul_rn(cs[q][l], e.x)),
                        __fadd_rn(v.y, __fmul_rn(cs[q][l], e.y)));
      }
      return v;
    };
    float2* out_psi_m = psi_out + member * plane + gcol0w;
    float* out_n_m = n_out + member * plane + gcol0w;
    int row_first = (ya - 4) % ny;
    if (row_first < 0) row_first += ny;

    // Issue the bulk copies of iteration `i` (row ya - 4 + i) into ring slot i % kRing.
    auto issue = [&](int i) {
      const int slot = i & (kRing - 1);
      int row = row_first + i;
      while (row >= ny) row -= ny;
      const uint32_t bar = smem_u32(&mbar[slot]);
      mbar_arrive_expect_tx(bar, kRowBytes);
      const long long ro = static_cast<long long>(row) * gnx;
      if (!HALO) {
        bulk_g2s(smem_u32(ring_psi + slot * W), psi_m + ro, NX * 8u, bar);
        bulk_g2s(smem_u32(ring_n + slot * W), n_m + ro, NX * 4u, bar);
#pragma unroll
        for (int l = 0; l < TERMS; ++l)
          bulk_g2s(smem_u32(ring_p + (slot * TERMS + l) * W), p_m + l * g.pump_term_stride + ro,
                   NX * 4u, bar);
      } else {
        // Columns [gc0, gc0 + W) of the periodic row: one copy, or two where the band wraps
        // (the first band starts at gnx - 4, the last one ends past gnx).  Every piece is a
        // multiple of four columns, so every copy starts and ends on 16 bytes.
        const int first = gc0 < 0 ? 4 : (gc0 + W > gnx ? gnx - gc0 : W);
        const int src0 = gc0 < 0 ? gnx - 4 : gc0;
        bulk_g2s(smem_u32(ring_psi + slot * W), psi_m + ro + src0, first * 8u, bar);
        bulk_g2s(smem_u32(ring_n + slot * W), n_m + ro + src0, first * 4u, bar);
        bulk_g2s(smem_u32(ring_p + slot * W), p_m + ro + src0, first * 4u, bar);
        if (first < W) {  // the rest continues from column 0 of the row
          bulk_g2s(smem_u32(ring_psi + slot * W + first), psi_m + ro, (W - first) * 8u, bar);
          bulk_g2s(smem_u32(ring_n + slot * W + first), n_m + ro, (W - first) * 4u, bar);
          bulk_g2s(smem_u32(ring_p + slot * W + first), p_m + ro, (W - first) * 4u, bar);
        }
      }
    };
    // Thread 0 feeds ring use it + i: the row copies, or, once one of its own waits has given
    // up, an empty arrival (see tma.cuh).  It tells the two apart at the barrier: feeding use
    // u (u >= it + 3) it tests, without waiting, the use it has just waited for, u - 3, whose
    // slot is not yet fed again (so the test cannot mistake a later phase for it).  Reading
    // timed_out in the loop instead, even once per kRing rows, measured 6% slower.  The give-up
    // setting (wait_limit 0) withholds the block's first use, so that every thread's wait for
    // it runs out, and settles it just before its slot is fed again.
    auto feed = [&](int i) {
      const unsigned u = it + i;
      int mode = *feed_mode;
      if (mode == 0 && i >= 3) {
        // the use thread 0 has just waited for: open means its wait gave up
        const unsigned w = u - 3;
        if (!mbar_test(smem_u32(&mbar[w & (kRing - 1)]), (w / kRing) & 1u)) *feed_mode = mode = 1;
      }
      if (g.wait_limit == 0) {
        if (u == 0) return;
        if (u == kRing) mbar_arrive(smem_u32(&mbar[0]));
      }
      if (mode == 0) {
        issue(i);
        return;
      }
      mbar_fill_empty(smem_u32(&mbar[i & (kRing - 1)]), u, kRing);
    };
    if (t == 0) {
      for (int i = 0; i < 3 && i < n_iter; ++i) feed(i);
    }

    Pair q1[4], q2[4], q3[4], acc[4];
    float2 m1[4], m2[4], m3[4], accn[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      q1[s] = q2[s] = q3[s] = acc[s] = Pair{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
      m1[s] = m2[s] = m3[s] = accn[s] = make_float2(0.f, 0.f);
    }
    int row_out = (ya - 8) % ny;
    if (row_out < 0) row_out += ny;

    for (int i0 = 0; i0 < n_iter; i0 += kRing) {
      const uint32_t parity = ((it + i0) / kRing) & 1u;
#pragma unroll
      for (int j = 0; j < kRing; ++j) {
        const int i = i0 + j;
        const int ja = (j + 3) & 3, jb = (j + 2) & 3, jc = (j + 1) & 3, jd = j & 3;
        const int slot0 = j;                        // row r
        const int slot1 = (j + kRing - 1) % kRing;  // row r-1
        const int slot2 = (j + kRing - 2) % kRing;  // row r-2
        const int slot3 = (j + kRing - 3) % kRing;  // row r-3
        const int slot4 = (j + kRing - 4) % kRing;  // row r-4
        if (!mbar_wait_bounded(smem_u32(&mbar[slot0]), parity, kWaitPolls)) timed_out = true;
        // Stage 1 at row r-1 from the ring: k1 = f(psi0).
        const float2* R1 = ring_psi + slot1 * W;
        const float4 c4 = *reinterpret_cast<const float4*>(R1 + col0);
        const float4 u4 = *reinterpret_cast<const float4*>(ring_psi + slot2 * W + col0);
        const float4 d4 = *reinterpret_cast<const float4*>(ring_psi + slot0 * W + col0);
        const float2 lt = R1[lcol], rt = R1[rcol];
        const float2 c0 = make_float2(c4.x, c4.y), c1 = make_float2(c4.z, c4.w);
        const float2 up0 = make_float2(u4.x, u4.y), up1 = make_float2(u4.z, u4.w);
        const float2 dn0 = make_float2(d4.x, d4.y), dn1 = make_float2(d4.z, d4.w);
        const float2 n1v = *reinterpret_cast<const float2*>(ring_n + slot1 * W + col0);
        const float2 P1 = pump_pair(slot1, 0);
        // Rows of the four stages (general variant only: the potential is read per stage).
        int srow[4] = {0, 0, 0, 0};
        if (GENERAL) {
          srow[3] = row_out;
#pragma unroll
          for (int q = 2; q >= 0; --q) srow[q] = srow[q + 1] + 1 == ny ? 0 : srow[q + 1] + 1;
        }
        {
          float2 da, db, va, vb;
          pot_at(srow[0], va, vb);
          const float2 dn2 = rhs2(c0, c1, lt, rt, up0, up1, dn0, dn1, n1v, s0, P1, va, vb, da, db);
          q1[ja] = Pair{axpy2(hh, da, c0), axpy2(hh, db, c1)};
          acc[ja] = Pair{axpy2(h6, da, c0), axpy2(h6, db, c1)};
          m1[ja] = axpy2(hh, dn2, n1v);
          accn[ja] = axpy2(h6, dn2, n1v);
        }
        if (kSplit) {
          // Split barrier: wait until every thread has arrived at the end of iteration
          // i-1, i.e. published its stage values there and finished every read of
          // iteration i-1 (the exchange buffer written below and the ring slot of row
          // r-5, which the copy of row r+3 reuses).  The wait sits after stage 1 so that
          // the draw and stage 1 overlap with the slower warps of the previous row.
          const unsigned g = it + i;
          if (g > 0 && !mbar_wait_bounded(xbar, (g - 1) & 1u, kWaitPolls)) timed_out = true;
          // The edge threads also wait for the neighbouring CTAs' edge values of iteration
          // i-1.  A neighbour delivers into the same inbox again only at the end of iteration
          // i+1, after it has received this thread's own delivery of iteration i.
          if (CLUSTER && g > 0 && !receive(g - 1)) timed_out = true;
          if (t == 0 && i + 3 < n_iter) feed(i + 3);
        }
        // Philox words and the variance-free part of the Box-Muller draw for this
        // iteration's output row, in the same straight-line code as stages 2-4 (after the
        // exchange wait) so that the integer and SFU work fills their issue gaps.
        float r2a = 0.f, sna = 0.f, csa = 0.f, r2b = 0.f, snb = 0.f, csb = 0.f;
        if (NOISE) {
          const uint32_t cell = static_cast<uint32_t>(row_out * gnx + gcol0w);
          const uint32_t cells[2] = {cell, cell + 1u};
          Words4 w[2];
          philox_cells(cells, prefix, w);
          WignerDraw<float>::prepare(w[0], r2a, sna, csa);
          WignerDraw<float>::prepare(w[1], r2b, snb, csb);
        }

        // Stage 2 at row r-2: k2 = f(psi1).
        {
          float2 lt2, rt2;
          xchg((j + 1) & 1, 0, lt2, rt2);
          const float2 P2 = pump_pair(slot2, 1);
          const float2 n0 = *reinterpret_cast<const float2*>(ring_n + slot2 * W + col0);
          const Pair c = q1[jb];
          float2 da, db, va, vb;
          pot_at(srow[1], va, vb);
          const float2 dn2 = rhs2(c.a, c.b, lt2, rt2, q1[jc].a, q1[jc].b, q1[ja].a, q1[ja].b,
                                  m1[jb], s1, P2, va, vb, da, db);
          q2[jb] = Pair{axpy2(hh, da, up0), axpy2(hh, db, up1)};  // psi0 at row r-2
          m2[jb] = axpy2(hh, dn2, n0);
          acc[jb] = Pair{axpy2(h3, da, acc[jb].a), axpy2(h3, db, acc[jb].b)};
          accn[jb] = axpy2(h3, dn2, accn[jb]);
        }
        // Stage 3 at row r-3: k3 = f(psi2).
        {
          float2 lt3, rt3;
          xchg((j + 1) & 1, 1, lt3, rt3);
          const float2 P3 = pump_pair(slot3, 1);
          const float2 n0 = *reinterpret_cast<const float2*>(ring_n + slot3 * W + col0);
          const float4 p4 = *reinterpret_cast<const float4*>(ring_psi + slot3 * W + col0);
          const Pair c = q2[jc];
          float2 da, db, va, vb;
          pot_at(srow[2], va, vb);
          const float2 dn2 = rhs2(c.a, c.b, lt3, rt3, q2[jd].a, q2[jd].b, q2[jb].a, q2[jb].b,
                                  m2[jc], s1, P3, va, vb, da, db);
          q3[jc] = Pair{axpy2(dt, da, make_float2(p4.x, p4.y)), axpy2(dt, db, make_float2(p4.z, p4.w))};
          m3[jc] = axpy2(dt, dn2, n0);
          acc[jc] = Pair{axpy2(h3, da, acc[jc].a), axpy2(h3, db, acc[jc].b)};
          accn[jc] = axpy2(h3, dn2, accn[jc]);
        }
        // Stage 4 at row r-4: k4 = f(psi3), final combine, clamp, Wigner increment.
        {
          float2 lt4, rt4;
          xchg((j + 1) & 1, 2, lt4, rt4);
          const float2 P4 = pump_pair(slot4, 2);
          const Pair c = q3[jd];
          float2 da, db, va, vb;
          pot_at(srow[3], va, vb);
          const float2 dn2 = rhs2(c.a, c.b, lt4, rt4, q3[ja].a, q3[ja].b, q3[jc].a, q3[jc].b,
                                  m3[jd], s2, P4, va, vb, da, db);
          float2 oa = axpy2(h6, da, acc[jd].a);
          float2 ob = axpy2(h6, db, acc[jd].b);
          const float2 nab = axpy2(h6, dn2, accn[jd]);
          float na = nab.x, nb = nab.y;
          na = na < 0.f ? 0.f : na;
          nb = nb < 0.f ? 0.f : nb;
          if (writes && i >= 8 && i - 8 < h_rows) {
            const long long o = static_cast<long long>(row_out) * gnx;
            if (NOISE) {
              WignerDraw<float>::add(fmaf(k.noise_b, na, k.noise_a), r2a, sna, csa, oa.x, oa.y);
              WignerDraw<float>::add(fmaf(k.noise_b, nb, k.noise_a), r2b, snb, csb, ob.x, ob.y);
            }
            *reinterpret_cast<float4*>(out_psi_m + o) = make_float4(oa.x, oa.y, ob.x, ob.y);
            *reinterpret_cast<float2*>(out_n_m + o) = make_float2(na, nb);
          }
        }
        // Publish stage inputs for the horizontal neighbours.
        {
          const int o = (j & 1) * 3 * HALF + t;
          xa[o] = q1[ja].a;
          xb[o] = q1[ja].b;
          xa[o + HALF] = q2[jb].a;
          xb[o + HALF] = q2[jb].b;
          xa[o + 2 * HALF] = q3[jc].a;
          xb[o + 2 * HALF] = q3[jc].b;
        }
        row_out = row_out + 1 == ny ? 0 : row_out + 1;
        if (CLUSTER) {
          // Deliver the edge column's three stage values to the neighbour that needs them.
          const uint32_t q = (it + i) & 1u;
          if (t == 0) {
            const uint32_t dst = left_inbox + q * kEdgeBytes;
            st_async_f2(dst, q1[ja].a, left_bar + 8u * q);
            st_async_f2(dst + 8u, q2[jb].a, left_bar + 8u * q);
            st_async_f2(dst + 16u, q3[jc].a, left_bar + 8u * q);
          }
          if (t == HALF - 1) {
            const uint32_t dst = right_inbox + q * kEdgeBytes;
            st_async_f2(dst, q1[ja].b, right_bar + 8u * q);
            st_async_f2(dst + 8u, q2[jb].b, right_bar + 8u * q);
            st_async_f2(dst + 16u, q3[jc].b, right_bar + 8u * q);
          }
        }
        if (kSplit) {
          mbar_arrive(xbar);
        } else {
          __syncthreads();
          // Slot of row r+3 held row r-5, last read by stage 4 of the previous iteration.
          if (t == 0 && i + 3 < n_iter) feed(i + 3);
        }
      }
    }
    it += n_iter;
  }
  // CLUSTER: take the neighbours' last deliveries, so that no store into this CTA's shared
  // memory is still in flight when it exits, then leave together.
  if (CLUSTER && it > 0 && !receive(it - 1)) timed_out = true;
  // After a wait of thread 0's gave up: copies it issued may still be in flight in the last
  // ring uses (every earlier one it waited for); a use it filled empty completes at once.
  if (t == 0 && (timed_out || *feed_mode != 0)) drain_ring(mbar, kRing, it >= kRing ? it - kRing : 0u, it);
  if (timed_out) atomicOr(err_flag, 1);
  if (CLUSTER) cluster_sync_all();
}

}  // namespace

bool wide_rk4_supported(int nx, int ny) {
  const bool full = nx == 128 || nx == 256 || nx == 512 || nx == 1024;
  const bool band = nx > 1024 && nx % 1024 == 0 && nx <= 16384;
  return (full || band) && ny >= 4;
}

namespace {

// Rows of 2048 .. 8192 sites run as clusters of nx / 1024 CTAs (the portable cluster size
// limit is 8); wider rows as independent bands.
bool use_cluster(int nx) { return nx > 1024 && nx % 1024 == 0 && nx / 1024 <= 8; }

template <int NX, bool BAND, bool CLUSTER, int TERMS = 1>
size_t smem_for() {
  using S = WideShape<NX, BAND, CLUSTER>;
  return static_cast<size_t>(kRing) * S::W * (12 + 4 * TERMS) + static_cast<size_t>(6) * S::THREADS * 16 +
         kBars * sizeof(uint64_t) + kInbox * sizeof(float2) + kFailWords * sizeof(int);
}

template <int NX, bool BAND, bool CLUSTER>
cudaError_t configure_shape() {
  const int smem = static_cast<int>(smem_for<NX, BAND, CLUSTER>());
  cudaError_t e = cudaFuncSetAttribute(rk4_wide_kernel<NX, true, false, BAND, CLUSTER>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(rk4_wide_kernel<NX, false, false, BAND, CLUSTER>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(rk4_wide_kernel<NX, true, true, BAND, CLUSTER>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(rk4_wide_kernel<NX, false, true, BAND, CLUSTER>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  return e;
}

// Two lasers (the general variant, rows of at most 1024 sites).
template <int NX>
cudaError_t configure_two_lasers() {
  const int smem = static_cast<int>(smem_for<NX, false, false, 2>());
  cudaError_t e = cudaFuncSetAttribute(rk4_wide_kernel<NX, true, true, false, false, 2>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(rk4_wide_kernel<NX, false, true, false, false, 2>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  return e;
}

template <int NX, bool BAND>
int blocks_shape(bool noise, int terms = 1) {
  int blocks = 0;
  const int threads = WideShape<NX, BAND>::THREADS;
  cudaError_t e =
      terms == 2 && !BAND
          ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &blocks, rk4_wide_kernel<NX, true, true, false, false, 2>, threads,
                smem_for<NX, false, false, 2>())
      : noise ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                  &blocks, rk4_wide_kernel<NX, true, false, BAND>, threads, smem_for<NX, BAND, false>())
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                  &blocks, rk4_wide_kernel<NX, false, false, BAND>, threads, smem_for<NX, BAND, false>());
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return blocks < 1 ? 1 : blocks;
}

// Clusters of `size` CTAs of the 1024-column cluster kernel that fit on the GPU at once.
int active_clusters(int size, bool noise) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = size;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(size, 1, 1);
  cfg.blockDim = dim3(WideShape<1024, false, true>::THREADS, 1, 1);
  cfg.dynamicSmemBytes = smem_for<1024, false, true>();
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  const cudaError_t e =
      noise ? cudaOccupancyMaxActiveClusters(&n, rk4_wide_kernel<1024, true, false, false, true>, &cfg)
            : cudaOccupancyMaxActiveClusters(&n, rk4_wide_kernel<1024, false, false, false, true>, &cfg);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

template <int NX, bool BAND>
cudaError_t launch_shape(const float* psi_in, const float* n_in, const float* pump, float* psi_out,
                         float* n_out, const RhsConst<float>* consts, const float* scales,
                         const unsigned long long* step_base, int step_offset, float dt, bool noise,
                         const WideGeom& g, int* err_flag, cudaStream_t stream) {
  const size_t smem = smem_for<NX, BAND, false>();
  const int threads = WideShape<NX, BAND>::THREADS;
  const float2* pin = reinterpret_cast<const float2*>(psi_in);
  float2* pout = reinterpret_cast<float2*>(psi_out);
  const bool general = wide_general(g);
  if (!BAND && g.pump_terms == 2) {
    const size_t smem2 = smem_for<NX, false, false, 2>();
    if (noise)
      rk4_wide_kernel<NX, true, true, false, false, 2><<<g.blocks, threads, smem2, stream>>>(
          pin, n_in, pump, pout, n_out, consts, scales, step_base, step_offset, dt, g, err_flag);
    else
      rk4_wide_kernel<NX, false, true, false, false, 2><<<g.blocks, threads, smem2, stream>>>(
          pin, n_in, pump, pout, n_out, consts, scales, step_base, step_offset, dt, g, err_flag);
    return cudaGetLastError();
  }
  if (g.pump_terms != 1) return cudaErrorInvalidValue;
  if (noise && general) {
    rk4_wide_kernel<NX, true, true, BAND><<<g.blocks, threads, smem, stream>>>(
        pin, n_in, pump, pout, n_out, consts, scales, step_base, step_offset, dt, g, err_flag);
  } else if (noise) {
    rk4_wide_kernel<NX, true, false, BAND><<<g.blocks, threads, smem, stream>>>(
        pin, n_in, pump, pout, n_out, consts, scales, step_base, step_offset, dt, g, err_flag);
  } else if (general) {
    rk4_wide_kernel<NX, false, true, BAND><<<g.blocks, threads, smem, stream>>>(
        pin, n_in, pump, pout, n_out, consts, scales, step_base, step_offset, dt, g, err_flag);
  } else {
    rk4_wide_kernel<NX, false, false, BAND><<<g.blocks, threads, smem, stream>>>(
        pin, n_in, pump, pout, n_out, consts, scales, step_base, step_offset, dt, g, err_flag);
  }
  return cudaGetLastError();
}

// Cluster launch: g.blocks CTAs in clusters of nx / 1024.
cudaError_t launch_cluster(const float* psi_in, const float* n_in, const float* pump,
                           float* psi_out, float* n_out, const RhsConst<float>* consts,
                           const float* scales, const unsigned long long* step_base,
                           int step_offset, float dt, bool noise, const WideGeom& g, int* err_flag,
                           cudaStream_t stream) {
  const int size = g.nx / 1024;
  if (g.blocks < size || g.blocks % size != 0) return cudaErrorInvalidValue;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = size;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(g.blocks, 1, 1);
  cfg.blockDim = dim3(WideShape<1024, false, true>::THREADS, 1, 1);
  cfg.dynamicSmemBytes = smem_for<1024, false, true>();
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const float2* pin = reinterpret_cast<const float2*>(psi_in);
  float2* pout = reinterpret_cast<float2*>(psi_out);
  const bool general = wide_general(g);
  if (noise && general)
    return cudaLaunchKernelEx(&cfg, rk4_wide_kernel<1024, true, true, false, true>, pin, n_in, pump,
                              pout, n_out, consts, scales, step_base, step_offset, dt, g, err_flag);
  if (noise)
    return cudaLaunchKernelEx(&cfg, rk4_wide_kernel<1024, true, false, false, true>, pin, n_in,
                              pump, pout, n_out, consts, scales, step_base, step_offset, dt, g,
                              err_flag);
  if (general)
    return cudaLaunchKernelEx(&cfg, rk4_wide_kernel<1024, false, true, false, true>, pin, n_in,
                              pump, pout, n_out, consts, scales, step_base, step_offset, dt, g,
                              err_flag);
  return cudaLaunchKernelEx(&cfg, rk4_wide_kernel<1024, false, false, false, true>, pin, n_in, pump,
                            pout, n_out, consts, scales, step_base, step_offset, dt, g, err_flag);
}

}  // namespace

size_t wide_rk4_smem(int nx) {
  switch (nx) {
    case 128: return smem_for<128, false, false>();
    case 256: return smem_for<256, false, false>();
    case 512: return smem_for<512, false, false>();
    case 1024: return smem_for<1024, false, false>();
    default: return use_cluster(nx) ? smem_for<1024, false, true>() : smem_for<1024, true, false>();
  }
}

cudaError_t configure_wide_rk4() {
  cudaError_t e = configure_shape<128, false, false>();
  if (e == cudaSuccess) e = configure_shape<256, false, false>();
  if (e == cudaSuccess) e = configure_shape<512, false, false>();
  if (e == cudaSuccess) e = configure_shape<1024, false, false>();
  if (e == cudaSuccess) e = configure_shape<1024, true, false>();
  if (e == cudaSuccess) e = configure_shape<1024, false, true>();
  if (e == cudaSuccess) e = configure_two_lasers<128>();
  if (e == cudaSuccess) e = configure_two_lasers<256>();
  if (e == cudaSuccess) e = configure_two_lasers<512>();
  if (e == cudaSuccess) e = configure_two_lasers<1024>();
  return e;
}

int wide_rk4_grid(int nx, int ny, int members, int sm_count, int terms) {
  if (use_cluster(nx)) {
    // Whole clusters, as many as fit at once, and at least 16 rows a cluster.
    const int size = nx / 1024;
    const long long rows = static_cast<long long>(members) * ny;
    const long long fit = std::max(1, active_clusters(size, true));
    const long long clusters = std::max<long long>(1, std::min(fit, rows / 16));
    return static_cast<int>(clusters * size);
  }
  int per_sm = 1;
  switch (nx) {
    case 128: per_sm = blocks_shape<128, false>(true, terms); break;
    case 256: per_sm = blocks_shape<256, false>(true, terms); break;
    case 512: per_sm = blocks_shape<512, false>(true, terms); break;
    case 1024: per_sm = blocks_shape<1024, false>(true, terms); break;
    default: per_sm = blocks_shape<1024, true>(true); break;
  }
  // Rows wider than 1024 sites (BAND) are separate 1024-site bands, each its own row stream.
  const long long bands = nx > 1024 ? nx / 1024 : 1;
  const long long rows = static_cast<long long>(members) * bands * ny;
  const long long blocks = static_cast<long long>(per_sm) * std::max(1, sm_count);
  return static_cast<int>(std::min(blocks, std::max<long long>(1, rows / 16)));
}

cudaError_t launch_rk4_wide(const float* psi_in, const float* n_in, const float* pump,
                            float* psi_out, float* n_out, const RhsConst<float>* consts,
                            const float* scales, const unsigned long long* step_base,
                            int step_offset, float dt, bool noise, const WideGeom& g,
                            int* err_flag, cudaStream_t stream) {
  switch (g.nx) {
    case 128:
      return launch_shape<128, false>(psi_in, n_in, pump, psi_out, n_out, consts, scales, step_base,
                                      step_offset, dt, noise, g, err_flag, stream);
    case 256:
      return launch_shape<256, false>(psi_in, n_in, pump, psi_out, n_out, consts, scales, step_base,
                                      step_offset, dt, noise, g, err_flag, stream);
    case 512:
      return launch_shape<512, false>(psi_in, n_in, pump, psi_out, n_out, consts, scales, step_base,
                                      step_offset, dt, noise, g, err_flag, stream);
    case 1024:
      return launch_shape<1024, false>(psi_in, n_in, pump, psi_out, n_out, consts, scales, step_base,
                                       step_offset, dt, noise, g, err_flag, stream);
    default:
      if (g.pump_terms != 1) return cudaErrorInvalidValue;
      if (use_cluster(g.nx))
        return launch_cluster(psi_in, n_in, pump, psi_out, n_out, consts, scales, step_base,
                              step_offset, dt, noise, g, err_flag, stream);
      if (g.nx > 1024 && g.nx % 1024 == 0)
        return launch_shape<1024, true>(psi_in, n_in, pump, psi_out, n_out, consts, scales,
                                        step_base, step_offset, dt, noise, g, err_flag, stream);
      return cudaErrorInvalidValue;
  }
}

}  // namespace pg
