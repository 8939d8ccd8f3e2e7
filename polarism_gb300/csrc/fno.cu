// Kernels of the learned warm start: a BF16 tensor-core GEMM with FP32 accumulation and the
// elementwise, mode-mixing and optimiser kernels of a Fourier neural operator.
//
// Every linear map of the network -- the pointwise channel mixes, the truncated DFTs along x
// and y that replace the FFTs of the spectral convolution, and their adjoints in the backward
// pass -- is a (batched, strided, optionally transposed) GEMM C = alpha op(A) op(B) + beta C
// with BF16 operands and FP32 accumulators.  The per-mode complex mixing of the spectral
// layer is a small batched contraction done in FP32 on the CUDA cores.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "pg_internal.h"
#include "tma.cuh"

namespace pg {
namespace {

constexpr int kBM = 64, kBN = 64, kBK = 32, kPad = 8;

struct GemmArgs {
  const __nv_bfloat16* A;
  const __nv_bfloat16* B;
  float* C;
  int M, N, K, lda, ldb, ldc, transA, transB;
  float alpha, beta;
  long long sA, sB, sC;       // outer batch strides
  int inner;                  // inner batch count: blockIdx.z = outer * inner + inner index
  long long sA2, sB2, sC2;    // inner batch strides
  int vecA, vecB;             // operand rows start on 16-byte boundaries: stage 8 values at once
};

__device__ __forceinline__ void batch_offsets(const GemmArgs& g, long long& oa, long long& ob, long long& oc) {
  const long long z = blockIdx.z;
  const long long outer = z / g.inner, in = z % g.inner;
  oa = outer * g.sA + in * g.sA2;
  ob = outer * g.sB + in * g.sB2;
  oc = outer * g.sC + in * g.sC2;
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// 64x64 output tile per block of 4 warps (2x2, 32x32 each); K staged 32 at a time through
// shared memory as [row][k] for A and [col][k] for B (k contiguous), the operand orders of
// the m16n8k16 fragments.  Out-of-range elements are staged as zero.
__global__ void __launch_bounds__(128) gemm_bf16_kernel(const GemmArgs g) {
  __shared__ __align__(16) __nv_bfloat16 As[kBM][kBK + kPad];
  __shared__ __align__(16) __nv_bfloat16 Bs[kBN][kBK + kPad];
  long long oa, ob, oc;
  batch_offsets(g, oa, ob, oc);
  const __nv_bfloat16* A = g.A + oa;
  const __nv_bfloat16* B = g.B + ob;
  float* C = g.C + oc;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int gq = lane >> 2, tq = lane & 3;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
  for (int k0 = 0; k0 < g.K; k0 += kBK) {
    for (int e = tid; e < kBM * kBK; e += 128) {
      int m, k;
      if (!g.transA) {
        m = e / kBK;
        k = e % kBK;
      } else {
        k = e / kBM;
        m = e % kBM;
      }
      const int gm = m0 + m, gk = k0 + k;
      __nv_bfloat16 v = zero;
      if (gm < g.M && gk < g.K)
        v = g.transA ? A[static_cast<long long>(gk) * g.lda + gm] : A[static_cast<long long>(gm) * g.lda + gk];
      As[m][k] = v;
    }
    for (int e = tid; e < kBN * kBK; e += 128) {
      int n, k;
      if (g.transB) {
        n = e / kBK;
        k = e % kBK;
      } else {
        k = e / kBN;
        n = e % kBN;
      }
      const int gn = n0 + n, gk = k0 + k;
      __nv_bfloat16 v = zero;
      if (gn < g.N && gk < g.K)
        v = g.transB ? B[static_cast<long long>(gn) * g.ldb + gk] : B[static_cast<long long>(gk) * g.ldb + gn];
      Bs[n][k] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; kk += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm + i * 16 + gq;
        af[i][0] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 2 * tq]);
        af[i][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 2 * tq]);
        af[i][2] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 2 * tq + 8]);
        af[i][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 2 * tq + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = wn + j * 8 + gq;
        bfr[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[c][kk + 2 * tq]);
        bfr[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[c][kk + 2 * tq + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = m0 + wm + i * 16 + gq + 8 * h;
        if (r >= g.M) continue;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int c = n0 + wn + j * 8 + 2 * tq + q;
          if (c >= g.N) continue;
          float* dst = C + static_cast<long long>(r) * g.ldc + c;
          const float v = g.alpha * acc[i][j][2 * h + q];
          *dst = g.beta == 0.f ? v : v + g.beta * *dst;
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------------------
// The same GEMM on the 5th-generation tensor cores: tcgen05.mma (kind::f16, BF16 operands,
// FP32 accumulators in tensor memory), issued by one thread per CTA.
//
// A CTA computes a 128 x 64 tile of C.  Per 64-wide K slab the 128 threads stage A (128 x 64)
// and B (64 x 64, as N x K) into shared memory in the canonical K-major layout without
// swizzle: 8-row x 16-byte core matrices, core matrix (row group g, k group j) at byte
// offset g * 1024 + j * 128 (so the K-direction stride between core matrices -- the leading
// byte offset -- is 128 and the 8-row-group stride -- the stride byte offset -- is 1024).
// After a proxy fence and a barrier, thread 0 issues four M128 N64 K16 MMAs (the descriptor
// start address advances 256 bytes per K16 step) and commits them to an mbarrier every thread
// waits on (bounded) before the slab is overwritten.  The accumulators (128 lanes x 64
// columns) are read back with tcgen05.ld (warp w owns lanes 32w..32w+31) for the epilogue.
// ---------------------------------------------------------------------------------------
constexpr int kTcM = 128, kTcN = 64, kTcK = 64;
constexpr uint32_t kTcCols = 64;                         // TMEM columns (power of two >= 32)
constexpr int kTcSmemA = kTcM * kTcK * 2;                // 16 KB
constexpr int kTcSmemB = kTcN * kTcK * 2;                // 8 KB
// 28 KB per CTA keeps at most 8 CTAs (8 x 64 TMEM columns = 512) on an SM.
constexpr int kTcSmem = 28 * 1024;
constexpr int kTcWaitLimit = 200000;

__device__ __forceinline__ uint64_t tc_smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr & 0x3FFFF) >> 4);            // start address
  d |= static_cast<uint64_t>(128 >> 4) << 16;                    // leading byte offset (K)
  d |= static_cast<uint64_t>(1024 >> 4) << 32;                   // stride byte offset (8 rows)
  d |= static_cast<uint64_t>(1) << 46;                           // descriptor version
  return d;                                                      // base offset 0, no swizzle
}

// kind::f16 instruction descriptor: D = F32, A = B = BF16, both K-major, N = 64, M = 128.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(kTcN >> 3) << 17) |
                              (static_cast<uint32_t>(kTcM >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, int accumulate) {
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

// One K slab of an operand into the canonical K-major layout: ROWS rows (M or N) x 64 k.
// kmajor: element (r, k) at X[r * ld + k], else at X[k * ld + r].  With vec, rows start on
// 16-byte boundaries and eight consecutive values along the contiguous index load at once:
// along k they are one 16-byte chunk of the layout, along r they go to eight chunks.
template <int ROWS>
__device__ __forceinline__ void stage_slab(__nv_bfloat16* S, const __nv_bfloat16* X, int ld, int kmajor,
                                           int vec, int r0, int R, int k0, int K, int tid) {
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  if (vec) {
    if (kmajor) {
      for (int e = tid; e < ROWS * (kTcK / 8); e += 128) {
        const int r = e >> 3, kv = (e & 7) * 8;
        const int gr = r0 + r, gk = k0 + kv;
        uint4 val = make_uint4(0u, 0u, 0u, 0u);
        if (gr < R) {
          const __nv_bfloat16* src = X + static_cast<long long>(gr) * ld + gk;
          if (gk + 8 <= K) {
            val = *reinterpret_cast<const uint4*>(src);
          } else {
            __nv_bfloat16 t[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) t[q] = gk + q < K ? src[q] : zero;
            val = *reinterpret_cast<const uint4*>(t);
          }
        }
        *reinterpret_cast<uint4*>(S + ((r >> 3) * 8 + (kv >> 3)) * 64 + (r & 7) * 8) = val;
      }
    } else {
      // Eight k rows x eight contiguous r values per thread: eight 16-byte loads, a transpose
      // in registers (byte permutes pairing the 16-bit halves of two k rows), eight 16-byte
      // stores, one per r, each the k-contiguous row of a core matrix.
      for (int blk = tid; blk < (ROWS / 8) * (kTcK / 8); blk += 128) {
        const int rb = blk % (ROWS / 8), kb = blk / (ROWS / 8);
        const int gr = r0 + rb * 8, gk0 = k0 + kb * 8;
        uint32_t w[8][4];
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
          const int gk = gk0 + kk;
          uint4 val = make_uint4(0u, 0u, 0u, 0u);
          if (gk < K) {
            const __nv_bfloat16* src = X + static_cast<long long>(gk) * ld + gr;
            if (gr + 8 <= R) {
              val = *reinterpret_cast<const uint4*>(src);
            } else {
              __nv_bfloat16 t[8];
#pragma unroll
              for (int q = 0; q < 8; ++q) t[q] = gr + q < R ? src[q] : zero;
              val = *reinterpret_cast<const uint4*>(t);
            }
          }
          w[kk][0] = val.x;
          w[kk][1] = val.y;
          w[kk][2] = val.z;
          w[kk][3] = val.w;
        }
        __nv_bfloat16* dst = S + (rb * 8 + kb) * 64;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          uint4 lo, hi;  // r = 2j and 2j + 1: k pairs (2i, 2i + 1) in word i
          lo.x = __byte_perm(w[0][j], w[1][j], 0x5410);
          hi.x = __byte_perm(w[0][j], w[1][j], 0x7632);
          lo.y = __byte_perm(w[2][j], w[3][j], 0x5410);
          hi.y = __byte_perm(w[2][j], w[3][j], 0x7632);
          lo.z = __byte_perm(w[4][j], w[5][j], 0x5410);
          hi.z = __byte_perm(w[4][j], w[5][j], 0x7632);
          lo.w = __byte_perm(w[6][j], w[7][j], 0x5410);
          hi.w = __byte_perm(w[6][j], w[7][j], 0x7632);
          *reinterpret_cast<uint4*>(dst + (2 * j) * 8) = lo;
          *reinterpret_cast<uint4*>(dst + (2 * j + 1) * 8) = hi;
        }
      }
    }
    return;
  }
  for (int e = tid; e < ROWS * kTcK; e += 128) {
    int r, k;
    if (kmajor) { r = e / kTcK; k = e % kTcK; } else { k = e / ROWS; r = e % ROWS; }
    const int gr = r0 + r, gk = k0 + k;
    __nv_bfloat16 v = zero;
    if (gr < R && gk < K)
      v = kmajor ? X[static_cast<long long>(gr) * ld + gk] : X[static_cast<long long>(gk) * ld + gr];
    S[((r >> 3) * 8 + (k >> 3)) * 64 + (r & 7) * 8 + (k & 7)] = v;
  }
}

__global__ void __launch_bounds__(128, 1) gemm_bf16_tc05_kernel(const GemmArgs g, int* err_flag) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  __nv_bfloat16* As = reinterpret_cast<__nv_bfloat16*>(tc_smem);
  __nv_bfloat16* Bs = reinterpret_cast<__nv_bfloat16*>(tc_smem + kTcSmemA);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(tc_smem + kTcSmemA + kTcSmemB);
  uint32_t* taddr_slot = reinterpret_cast<uint32_t*>(tc_smem + kTcSmemA + kTcSmemB + 16);
  long long oa, ob, oc;
  batch_offsets(g, oa, ob, oc);
  const __nv_bfloat16* A = g.A + oa;
  const __nv_bfloat16* B = g.B + ob;
  float* C = g.C + oc;
  const int m0 = blockIdx.y * kTcM, n0 = blockIdx.x * kTcN;
  const int tid = threadIdx.x, warp = tid >> 5;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(taddr_slot)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(smem_u32(mbar), 1);
    fence_mbar_init();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *taddr_slot;
  const uint32_t a_base = smem_u32(As), b_base = smem_u32(Bs);
  bool ok = true;
  uint32_t phase = 0;
  int slab = 0;
  for (int k0 = 0; k0 < g.K; k0 += kTcK, ++slab) {
    // Stage the slabs in the canonical layout: element (r, k) of a [rows][64] slab lives at
    // ((r / 8) * 8 + k / 8) * 64 + (r % 8) * 8 + k % 8 (elements).
    stage_slab<kTcM>(As, A, g.lda, !g.transA, g.vecA, m0, g.M, k0, g.K, tid);  // A is M x K unless transA
    stage_slab<kTcN>(Bs, B, g.ldb, g.transB, g.vecB, n0, g.N, k0, g.K, tid);   // B is K x N unless transB
    // Make the generic-proxy stores visible to the tensor core's async proxy.
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int s = 0; s < kTcK / 16; ++s)
        tc_mma(tmem, tc_smem_desc(a_base + 256 * s), tc_smem_desc(b_base + 256 * s), kTcIdesc,
               (slab > 0 || s > 0) ? 1 : 0);
      tc_commit(smem_u32(mbar));
    }
    // Every thread waits for the MMAs before the slab is restaged (or the result is read).
    if (!mbar_wait_bounded(smem_u32(mbar), phase, kTcWaitLimit)) ok = false;
    phase ^= 1u;
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // Epilogue: thread t of warp w holds row 32 w + lane of the tile, 64 FP32 columns.
  uint32_t v[64];
  const uint32_t lane_addr = tmem + (static_cast<uint32_t>(warp * 32) << 16);
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x64.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,"
      "%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,"
      "%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31]),
        "=r"(v[32]), "=r"(v[33]), "=r"(v[34]), "=r"(v[35]), "=r"(v[36]), "=r"(v[37]), "=r"(v[38]), "=r"(v[39]),
        "=r"(v[40]), "=r"(v[41]), "=r"(v[42]), "=r"(v[43]), "=r"(v[44]), "=r"(v[45]), "=r"(v[46]), "=r"(v[47]),
        "=r"(v[48]), "=r"(v[49]), "=r"(v[50]), "=r"(v[51]), "=r"(v[52]), "=r"(v[53]), "=r"(v[54]), "=r"(v[55]),
        "=r"(v[56]), "=r"(v[57]), "=r"(v[58]), "=r"(v[59]), "=r"(v[60]), "=r"(v[61]), "=r"(v[62]), "=r"(v[63])
      : "r"(lane_addr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  // Write the tile through shared memory (the slab area; every MMA has completed) so each warp
  // stores whole 128-byte row segments: 64 rows at a time, row stride 65 floats (no bank
  // conflicts on either side).
  float* stage = reinterpret_cast<float*>(tc_smem);
#pragma unroll 1
  for (int half = 0; half < 2; ++half) {
    __syncthreads();
    if ((warp >> 1) == half) {
      const int r = tid - 64 * half;
#pragma unroll
      for (int j = 0; j < 64; ++j) stage[r * 65 + j] = __uint_as_float(v[j]);
    }
    __syncthreads();
    const int c = n0 + (tid & 63);
    if (ok && g.K > 0 && c < g.N) {
#pragma unroll 4
      for (int q = 0; q < 32; ++q) {
        const int r = 2 * q + (tid >> 6);
        const int row = m0 + 64 * half + r;
        if (row < g.M) {
          float* dst = C + static_cast<long long>(row) * g.ldc + c;
          const float x = g.alpha * stage[r * 65 + (tid & 63)];
          *dst = g.beta == 0.f ? x : x + g.beta * *dst;
        }
      }
    }
  }
  if (!ok && tid == 0) atomicOr(err_flag, 1);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
  }
}

// out (+)= sum of `count` consecutive slices of n floats (fixed order: deterministic).
__global__ void sum_slices_kernel(const float* __restrict__ parts, float* __restrict__ out, long long n,
                                  int count, int accumulate) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    float s = accumulate ? out[i] : 0.f;
    for (int c = 0; c < count; ++c) s += parts[static_cast<long long>(c) * n + i];
    out[i] = s;
  }
}

__global__ void to_bf16_kernel(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, long long n) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    y[i] = __float2bfloat16_rn(x[i]);
}

constexpr float kGeluC = 0.7978845608028654f;  // sqrt(2 / pi)

__device__ __forceinline__ float gelu_f(float x) {
  return 0.5f * x * (1.f + tanhf(kGeluC * (x + 0.044715f * x * x * x)));
}

__device__ __forceinline__ float gelu_grad_f(float x) {
  const float t = tanhf(kGeluC * (x + 0.044715f * x * x * x));
  return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * kGeluC * (1.f + 3.f * 0.044715f * x * x);
}

// u[b, c, p] += bias[c]; act = gelu(u) (or u) in FP32 and, optionally, in BF16.
__global__ void bias_act_kernel(float* __restrict__ u, const float* __restrict__ bias,
                                float* __restrict__ act, __nv_bfloat16* __restrict__ act_bf,
                                int C, long long plane, long long n, int gelu) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int c = static_cast<int>((i / plane) % C);
    const float v = u[i] + (bias ? bias[c] : 0.f);
    u[i] = v;
    const float a = gelu ? gelu_f(v) : v;
    if (act) act[i] = a;
    if (act_bf) act_bf[i] = __float2bfloat16_rn(a);
  }
}

// g_pre = g_act * gelu'(pre), also in BF16.
__global__ void gelu_back_kernel(const float* __restrict__ pre, const float* __restrict__ g_act,
                                 float* __restrict__ g_pre, __nv_bfloat16* __restrict__ g_bf, long long n) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const float v = g_act[i] * gelu_grad_f(pre[i]);
    if (g_pre) g_pre[i] = v;
    if (g_bf) g_bf[i] = __float2bfloat16_rn(v);
  }
}

// out[c] = (accumulate ? out[c] : 0) + sum over b, p of x[b, c, p]; one block per channel.
__global__ void channel_sum_kernel(const float* __restrict__ x, float* __restrict__ out, int B, int C,
                                   long long plane, int accumulate) {
  __shared__ float red[32];
  const int c = blockIdx.x;
  float s = 0.f;
  for (int b = 0; b < B; ++b) {
    const float* p = x + (static_cast<long long>(b) * C + c) * plane;
    for (long long i = threadIdx.x; i < plane; i += blockDim.x) s += p[i];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) out[c] = (accumulate ? out[c] : 0.f) + v;
  }
}

// Spectra are stored [b][channel][ky (2m)][kx re (m) | kx im (m)]; weights [ky][kx][in][out].
__global__ void mode_mix_kernel(const float* __restrict__ y, const __nv_bfloat16* __restrict__ wre,
                                const __nv_bfloat16* __restrict__ wim, float* __restrict__ out,
                                int B, int cin, int cout, int m) {
  const long long total = static_cast<long long>(B) * cout * 2 * m * m;
  const int mm = 2 * m * m;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int mode = static_cast<int>(t % mm);
    const int o = static_cast<int>((t / mm) % cout);
    const int b = static_cast<int>(t / (static_cast<long long>(mm) * cout));
    const int ky = mode / m, kx = mode % m;
    float re = 0.f, im = 0.f;
    const float* yb = y + static_cast<long long>(b) * cin * 4 * m * m + ky * 2 * m;
    const long long wbase = (static_cast<long long>(ky) * m + kx) * cin * cout + o;
    for (int i = 0; i < cin; ++i) {
      const float a = yb[static_cast<long long>(i) * 4 * m * m + kx];
      const float c = yb[static_cast<long long>(i) * 4 * m * m + m + kx];
      const float r = __bfloat162float(wre[wbase + static_cast<long long>(i) * cout]);
      const float s = __bfloat162float(wim[wbase + static_cast<long long>(i) * cout]);
      re += a * r - c * s;
      im += a * s + c * r;
    }
    float* ob = out + (static_cast<long long>(b) * cout + o) * 4 * m * m + ky * 2 * m;
    ob[kx] = re;
    ob[m + kx] = im;
  }
}

// dY[b, i] = sum_o dO[b, o] conj(W[i, o]) per mode.
__global__ void mode_mix_back_input_kernel(const float* __restrict__ dout, const __nv_bfloat16* __restrict__ wre,
                                           const __nv_bfloat16* __restrict__ wim, float* __restrict__ dy,
                                           int B, int cin, int cout, int m) {
  const long long total = static_cast<long long>(B) * cin * 2 * m * m;
  const int mm = 2 * m * m;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int mode = static_cast<int>(t % mm);
    const int i = static_cast<int>((t / mm) % cin);
    const int b = static_cast<int>(t / (static_cast<long long>(mm) * cin));
    const int ky = mode / m, kx = mode % m;
    float re = 0.f, im = 0.f;
    const float* gb = dout + static_cast<long long>(b) * cout * 4 * m * m + ky * 2 * m;
    const long long wbase = ((static_cast<long long>(ky) * m + kx) * cin + i) * cout;
    for (int o = 0; o < cout; ++o) {
      const float gr = gb[static_cast<long long>(o) * 4 * m * m + kx];
      const float gi = gb[static_cast<long long>(o) * 4 * m * m + m + kx];
      const float r = __bfloat162float(wre[wbase + o]);
      const float s = __bfloat162float(wim[wbase + o]);
      re += gr * r + gi * s;
      im += gi * r - gr * s;
    }
    float* db = dy + (static_cast<long long>(b) * cin + i) * 4 * m * m + ky * 2 * m;
    db[kx] = re;
    db[m + kx] = im;
  }
}

// dW[i, o] = sum_b conj(Y[b, i]) dO[b, o] per mode (overwrites).
__global__ void mode_mix_back_weight_kernel(const float* __restrict__ y, const float* __restrict__ dout,
                                            float* __restrict__ dwre, float* __restrict__ dwim,
                                            int B, int cin, int cout, int m) {
  const long long total = static_cast<long long>(2 * m) * m * cin * cout;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int o = static_cast<int>(t % cout);
    const int i = static_cast<int>((t / cout) % cin);
    const int mode = static_cast<int>(t / (static_cast<long long>(cout) * cin));
    const int ky = mode / m, kx = mode % m;
    float re = 0.f, im = 0.f;
    for (int b = 0; b < B; ++b) {
      const float* yb = y + (static_cast<long long>(b) * cin + i) * 4 * m * m + ky * 2 * m;
      const float* gb = dout + (static_cast<long long>(b) * cout + o) * 4 * m * m + ky * 2 * m;
      const float a = yb[kx], c = yb[m + kx];
      const float gr = gb[kx], gi = gb[m + kx];
      re += a * gr + c * gi;
      im += a * gi - c * gr;
    }
    dwre[t] = re;
    dwim[t] = im;
  }
}

// Adam on FP32 master weights; the BF16 copy the GEMMs read is refreshed in the same pass.
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m1,
                            float* __restrict__ m2, __nv_bfloat16* __restrict__ w_bf, long long n,
                            float lr, float b1, float b2, float eps, float c1, float c2, float decay) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const float gi = g[i] + decay * w[i];
    const float a = b1 * m1[i] + (1.f - b1) * gi;
    const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    const float v = w[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    w[i] = v;
    if (w_bf) w_bf[i] = __float2bfloat16_rn(v);
  }
}

// Weighted squared error: grad = 2 w (pred - target) / count, per-block FP64 partial sums.
__global__ void mse_kernel(const float* __restrict__ pred, const float* __restrict__ target,
                           const float* __restrict__ weight, int C, long long plane,
                           float* __restrict__ grad, __nv_bfloat16* __restrict__ grad_bf,
                           double* __restrict__ partial, long long n, float scale) {
  __shared__ double red[32];
  double s = 0.0;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const float wc = weight ? weight[(i / plane) % C] : 1.f;
    const float d = pred[i] - target[i];
    s += static_cast<double>(wc) * d * d;
    const float gv = 2.f * wc * d * scale;
    if (grad) grad[i] = gv;
    if (grad_bf) grad_bf[i] = __float2bfloat16_rn(gv);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) partial[blockIdx.x] = v;
  }
}

__device__ int g_gemm_timeouts = 0;  // set when a tcgen05 GEMM's bounded wait gave up
int g_gemm_engine = 0;                // 0: tcgen05 (default), 1: mma.sync

int grid_for(long long n) {
  const long long b = (n + 255) / 256;
  return static_cast<int>(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

}  // namespace
}  // namespace pg

extern "C" {

int pg_gemm_bf16_2d(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K, int32_t lda,
                    int32_t ldb, int32_t ldc, int32_t transA, int32_t transB, float alpha, float beta,
                    int32_t batch, int64_t strideA, int64_t strideB, int64_t strideC, int32_t inner,
                    int64_t strideA2, int64_t strideB2, int64_t strideC2, void* stream) {
  PG_CHECK(A && B && C, PG_ERR_INVALID, "pg_gemm_bf16: null operand");
  PG_CHECK(M >= 0 && N >= 0 && K >= 0 && batch >= 1 && inner >= 1, PG_ERR_INVALID, "pg_gemm_bf16: bad sizes");
  PG_CHECK(lda >= (transA ? M : K) && ldb >= (transB ? K : N) && ldc >= N, PG_ERR_INVALID,
           "pg_gemm_bf16: leading dimension smaller than the row");
  PG_CHECK(static_cast<long long>(batch) * inner <= 65535 && (M + pg::kBM - 1) / pg::kBM <= 65535,
           PG_ERR_INVALID, "pg_gemm_bf16: grid too large");
  if (M == 0 || N == 0) return PG_OK;
  batch *= inner;
  // Vector staging needs every operand row (and batch slice) to start on a 16-byte boundary.
  auto aligned = [](const void* p, long long ld, long long s1, long long s2) {
    return (reinterpret_cast<uintptr_t>(p) & 15u) == 0 && ld % 8 == 0 && s1 % 8 == 0 && s2 % 8 == 0;
  };
  pg::GemmArgs g{static_cast<const __nv_bfloat16*>(A), static_cast<const __nv_bfloat16*>(B), C, M, N, K,
                 lda, ldb, ldc, transA ? 1 : 0, transB ? 1 : 0, alpha, beta, strideA, strideB, strideC,
                 inner, strideA2, strideB2, strideC2, aligned(A, lda, strideA, strideA2) ? 1 : 0,
                 aligned(B, ldb, strideB, strideB2) ? 1 : 0};
  if (pg::g_gemm_engine == 0 && K > 0) {
    PG_CHECK((M + pg::kTcM - 1) / pg::kTcM <= 65535, PG_ERR_INVALID, "pg_gemm_bf16: grid too large");
    int* flag = nullptr;
    PG_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&flag), pg::g_gemm_timeouts));
    dim3 grid((N + pg::kTcN - 1) / pg::kTcN, (M + pg::kTcM - 1) / pg::kTcM, batch);
    pg::gemm_bf16_tc05_kernel<<<grid, 128, pg::kTcSmem, static_cast<cudaStream_t>(stream)>>>(g, flag);
  } else {
    dim3 grid((N + pg::kBN - 1) / pg::kBN, (M + pg::kBM - 1) / pg::kBM, batch);
    pg::gemm_bf16_kernel<<<grid, 128, 0, static_cast<cudaStream_t>(stream)>>>(g);
  }
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

int pg_gemm_bf16(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K, int32_t lda,
                 int32_t ldb, int32_t ldc, int32_t transA, int32_t transB, float alpha, float beta,
                 int32_t batch, int64_t strideA, int64_t strideB, int64_t strideC, void* stream) {
  return pg_gemm_bf16_2d(A, B, C, M, N, K, lda, ldb, ldc, transA, transB, alpha, beta, batch, strideA,
                         strideB, strideC, 1, 0, 0, 0, stream);
}

int pg_fno_sum_slices(const float* parts, float* out, int64_t n, int32_t count, int32_t accumulate,
                      void* stream) {
  PG_CHECK(parts && out && n >= 0 && count >= 1, PG_ERR_INVALID, "pg_fno_sum_slices: bad argument");
  if (n == 0) return PG_OK;
  pg::sum_slices_kernel<<<pg::grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(parts, out, n, count,
                                                                                          accumulate);
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

int pg_gemm_set_engine(int32_t engine) {
  PG_CHECK(engine == 0 || engine == 1, PG_ERR_INVALID,
           "pg_gemm_set_engine: 0 (tcgen05 tensor cores) or 1 (mma.sync)");
  pg::g_gemm_engine = engine;
  return PG_OK;
}

int pg_gemm_timeouts(int32_t* count, int32_t clear) {
  PG_CHECK(count, PG_ERR_INVALID, "pg_gemm_timeouts: null argument");
  int v = 0;
  PG_CUDA(cudaMemcpyFromSymbol(&v, pg::g_gemm_timeouts, sizeof(int)));
  if (clear) {
    const int zero = 0;
    PG_CUDA(cudaMemcpyToSymbol(pg::g_gemm_timeouts, &zero, sizeof(int)));
  }
  *count = v;
  return PG_OK;
}

int pg_fno_to_bf16(const float* x, void* y, int64_t n, void* stream) {
  PG_CHECK(x && y && n >= 0, PG_ERR_INVALID, "pg_fno_to_bf16: bad argument");
  if (n == 0) return PG_OK;
  pg::to_bf16_kernel<<<pg::grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      x, static_cast<__nv_bfloat16*>(y), n);
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

int pg_fno_bias_act(float* u, const float* bias, float* act, void* act_bf16, int32_t C, int64_t plane,
                    int64_t n, int32_t gelu, void* stream) {
  PG_CHECK(u && C > 0 && plane > 0 && n >= 0, PG_ERR_INVALID, "pg_fno_bias_act: bad argument");
  if (n == 0) return PG_OK;
  pg::bias_act_kernel<<<pg::grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      u, bias, act, static_cast<__nv_bfloat16*>(act_bf16), C, plane, n, gelu);
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

int pg_fno_gelu_backward(const float* pre, const float* grad_act, float* grad_pre, void* grad_bf16,
                         int64_t n, void* stream) {
  PG_CHECK(pre && grad_act && n >= 0, PG_ERR_INVALID, "pg_fno_gelu_backward: bad argument");
  if (n == 0) return PG_OK;
  pg::gelu_back_kernel<<<pg::grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      pre, grad_act, grad_pre, static_cast<__nv_bfloat16*>(grad_bf16), n);
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

int pg_fno_channel_sum(const float* x, float* out, int32_t B, int32_t C, int64_t plane, int32_t accumulate,
                       void* stream) {
  PG_CHECK(x && out && B > 0 && C > 0 && plane > 0, PG_ERR_INVALID, "pg_fno_channel_sum: bad argument");
  pg::channel_sum_kernel<<<C, 256, 0, static_cast<cudaStream_t>(stream)>>>(x, out, B, C, plane, accumulate);
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

int pg_fno_mode_mix(const float* y, const void* wre, const void* wim, float* out, int32_t B, int32_t cin,
                    int32_t cout, int32_t modes, void* stream) {
  PG_CHECK(y && wre && wim && out && B > 0 && cin > 0 && cout > 0 && modes > 0, PG_ERR_INVALID,
           "pg_fno_mode_mix: bad argument");
  const long long total = static_cast<long long>(B) * cout * 2 * modes * modes;
  pg::mode_mix_kernel<<<pg::grid_for(total), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      y, static_cast<const __nv_bfloat16*>(wre), static_cast<const __nv_bfloat16*>(wim), out, B, cin, cout, modes);
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

int pg_fno_mode_mix_backward(const float* y, const float* dout, const void* wre, const void* wim, float* dy,
                             float* dwre, float* dwim, int32_t B, int32_t cin, int32_t cout, int32_t modes,
                             void* stream) {
  PG_CHECK(y && dout && wre && wim && B > 0 && cin > 0 && cout > 0 && modes > 0, PG_ERR_INVALID,
           "pg_fno_mode_mix_backward: bad argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dy) {
    const long long total = static_cast<long long>(B) * cin * 2 * modes * modes;
    pg::mode_mix_back_input_kernel<<<pg::grid_for(total), 256, 0, st>>>(
        dout, static_cast<const __nv_bfloat16*>(wre), static_cast<const __nv_bfloat16*>(wim), dy, B, cin, cout,
        modes);
  }
  if (dwre && dwim) {
    const long long total = static_cast<long long>(2 * modes) * modes * cin * cout;
    pg::mode_mix_back_weight_kernel<<<pg::grid_for(total), 256, 0, st>>>(y, dout, dwre, dwim, B, cin, cout,
                                                                         modes);
  }
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

int pg_fno_adam(float* w, const float* g, float* m1, float* m2, void* w_bf16, int64_t n, float lr,
                float beta1, float beta2, float eps, int64_t step, float decay, void* stream) {
  PG_CHECK(w && g && m1 && m2 && n >= 0 && step >= 1, PG_ERR_INVALID, "pg_fno_adam: bad argument");
  if (n == 0) return PG_OK;
  const float c1 = 1.f - std::pow(beta1, static_cast<float>(step));
  const float c2 = 1.f - std::pow(beta2, static_cast<float>(step));
  pg::adam_kernel<<<pg::grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      w, g, m1, m2, static_cast<__nv_bfloat16*>(w_bf16), n, lr, beta1, beta2, eps, c1, c2, decay);
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

int pg_fno_mse(const float* pred, const float* target, const float* weight, int32_t C, int64_t plane,
               float* grad, void* grad_bf16, double* partials, int32_t max_partials, int64_t n, float scale,
               int32_t* blocks_used, void* stream) {
  PG_CHECK(pred && target && partials && blocks_used && n > 0 && C > 0 && plane > 0, PG_ERR_INVALID,
           "pg_fno_mse: bad argument");
  int blocks = pg::grid_for(n);
  if (blocks > max_partials) blocks = max_partials;
  PG_CHECK(blocks >= 1, PG_ERR_INVALID, "pg_fno_mse: no partial slots");
  pg::mse_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      pred, target, weight, C, plane, grad, static_cast<__nv_bfloat16*>(grad_bf16), partials, n, scale);
  PG_CUDA(cudaGetLastError());
  *blocks_used = blocks;
  return PG_OK;
}

}  // extern "C"
