// Shared-memory Stockham FFT building blocks (device code shared by the split-step and
// IFRK passes).
//
// The in-place Stockham autosort pass follows the recurrence
//   y[q + s (R p + r)] = w_N^{p r s} * sum_t x[q + s (p + m t)] w_R^{r t}
// (s: product of the radices already done, m = N / (R s)), radix 4 with one radix-2 pass
// when log2 N is odd; every butterfly's inputs are staged in registers between two barriers.
#pragma once
#include <cuda_runtime.h>

namespace pg {
namespace {

template <typename T>
struct C2T;
template <>
struct C2T<float> {
  using type = float2;
};
template <>
struct C2T<double> {
  using type = double2;
};

template <typename C2>
__device__ __forceinline__ C2 cmul(C2 a, C2 b) {
  return C2{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename C2>
__device__ __forceinline__ C2 cmulc(C2 a, C2 b) {  // a * conj(b)
  return C2{a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}

// a * (h + l) and a * conj(h + l) for a twiddle carried as a rounded value h and its remainder
// l: the small product a * l is formed first and added inside the fused multiply-adds of a * h.
__device__ __forceinline__ float2 cmul2f(float2 a, float2 h, float2 l) {
  const float cr = fmaf(a.x, l.x, -a.y * l.y);
  const float ci = fmaf(a.x, l.y, a.y * l.x);
  return float2{fmaf(a.x, h.x, fmaf(-a.y, h.y, cr)), fmaf(a.x, h.y, fmaf(a.y, h.x, ci))};
}
__device__ __forceinline__ float2 cmulc2f(float2 a, float2 h, float2 l) {
  const float cr = fmaf(a.x, l.x, a.y * l.y);
  const float ci = fmaf(a.y, l.x, -a.x * l.y);
  return float2{fmaf(a.x, h.x, fmaf(a.y, h.y, cr)), fmaf(a.y, h.x, fmaf(-a.x, h.y, ci))};
}
template <bool INVERSE, typename C2>
__device__ __forceinline__ C2 twiddle_mul(C2 v, const C2* tw, int idx, int n, bool comp) {
  const C2 w = tw[idx];
  return INVERSE ? cmulc(v, w) : cmul(v, w);
}
template <bool INVERSE>
__device__ __forceinline__ float2 twiddle_mul(float2 v, const float2* tw, int idx, int n,
                                              bool comp) {
  const float2 w = tw[idx];
  if (comp) {
    const float2 l = tw[n + idx];
    return INVERSE ? cmulc2f(v, w, l) : cmul2f(v, w, l);
  }
  return INVERSE ? cmulc(v, w) : cmul(v, w);
}

// Complex values a thread stages per pass (keeps the 1024-thread blocks within 64 registers).
template <typename T>
struct MaxVals {
  static constexpr int value = sizeof(T) == 4 ? 16 : 8;
};

// One in-place radix-R Stockham pass over C sequences of length N (all powers of two).
// Element (i, c) of the shared buffer sits at buf[i * si + c * sc].  COLS selects which
// index varies fastest across threads (c for column panels, i within a row) so shared
// memory accesses stay contiguous.  s = stride (product of the radices already done),
// m = N / (R s).  Requires N * C <= MaxVals<T>::value * blockDim.x.  COMP (FP32 only):
// tw holds N rounded twiddles followed by their N remainders, and every twiddle product uses
// both.
template <typename T, bool INVERSE, bool COLS, int R, bool COMP = false>
__device__ __forceinline__ void stockham_pass(typename C2T<T>::type* buf,
                                              const typename C2T<T>::type* tw, int log2n,
                                              int log2c, int si, int sc, int log2s, int m) {
  using C2 = typename C2T<T>::type;
  constexpr int MAXB = MaxVals<T>::value / R;
  constexpr int LOG2R = R == 4 ? 2 : 1;
  const int log2per = log2n - LOG2R;  // butterflies per sequence = N / R
  const int nb = 1 << (log2per + log2c);
  const int s = 1 << log2s;
  C2 v[MAXB][R];
  int base_in[MAXB], cidx[MAXB];
#pragma unroll
  for (int kb = 0; kb < MAXB; ++kb) {
    const int b = threadIdx.x + kb * blockDim.x;
    if (b < nb) {
      int c, rest;
      if (COLS) {
        c = b & ((1 << log2c) - 1);
        rest = b >> log2c;
      } else {
        c = b >> log2per;
        rest = b & ((1 << log2per) - 1);
      }
      const int q = rest & (s - 1);
      const int p = rest >> log2s;
      base_in[kb] = q + s * p;
      cidx[kb] = c;
#pragma unroll
      for (int t = 0; t < R; ++t) v[kb][t] = buf[(base_in[kb] + s * m * t) * si + c * sc];
    }
  }
  __syncthreads();
#pragma unroll
  for (int kb = 0; kb < MAXB; ++kb) {
    const int b = threadIdx.x + kb * blockDim.x;
    if (b < nb) {
      const int c = cidx[kb];
      const int q = base_in[kb] & (s - 1);
      const int p = base_in[kb] >> log2s;
      C2 y[R];
      if (R == 2) {
        const C2 a = v[kb][0], bb = v[kb][1 % R];
        y[0] = C2{a.x + bb.x, a.y + bb.y};
        y[1 % R] = C2{a.x - bb.x, a.y - bb.y};
      } else {
        const C2 a0 = v[kb][0], a1 = v[kb][1 % R], a2 = v[kb][2 % R], a3 = v[kb][3 % R];
        const C2 t0{a0.x + a2.x, a0.y + a2.y}, t1{a0.x - a2.x, a0.y - a2.y};
        const C2 t2{a1.x + a3.x, a1.y + a3.y};
        const C2 d{a1.x - a3.x, a1.y - a3.y};
        // forward: t3 = -i d; inverse: t3 = +i d
        const C2 t3 = INVERSE ? C2{-d.y, d.x} : C2{d.y, -d.x};
        y[0] = C2{t0.x + t2.x, t0.y + t2.y};
        y[1 % R] = C2{t1.x + t3.x, t1.y + t3.y};
        y[2 % R] = C2{t0.x - t2.x, t0.y - t2.y};
        y[3 % R] = C2{t1.x - t3.x, t1.y - t3.y};
      }
      const int out = q + s * R * p;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        C2 val = y[r];
        if (r > 0) val = twiddle_mul<INVERSE>(val, tw, p * r * s, 1 << log2n, COMP);
        buf[(out + s * r) * si + c * sc] = val;
      }
    }
  }
  __syncthreads();
}

// In-place Stockham FFT (radix 4, with one radix-2 pass first when log2 N is odd).
template <typename T, bool INVERSE, bool COLS, bool COMP = false>
__device__ void smem_fft(typename C2T<T>::type* buf, const typename C2T<T>::type* tw, int log2n,
                         int log2c, int si, int sc) {
  int log2s = 0;
  int log2m = log2n;
  if (log2n & 1) {
    stockham_pass<T, INVERSE, COLS, 2, COMP>(buf, tw, log2n, log2c, si, sc, log2s, 1 << (log2m - 1));
    log2s += 1;
    log2m -= 1;
  }
  while (log2m > 0) {
    stockham_pass<T, INVERSE, COLS, 4, COMP>(buf, tw, log2n, log2c, si, sc, log2s, 1 << (log2m - 2));
    log2s += 2;
    log2m -= 2;
  }
}


}  // namespace
}  // namespace pg
