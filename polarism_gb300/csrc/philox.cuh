// Philox-4x32-10 counter RNG and the truncated-Wigner Box-Muller draw, held in registers.
//
// Counter stream and key layout follow polarism/noise/philox.py:7-38 (Random123
// Philox-4x32, counter = (cell, step_lo, step_hi, stream), key = 64-bit member
// seed).  Uniform construction follows polarism/noise/philox.py:41-56: 24-bit
// uniforms from words (a, b) in single precision, 53-bit uniforms from (a, b)
// and (c, d) in double precision.
#pragma once
#include <cstdint>

namespace pg {

struct Words4 {
  uint32_t a, b, c, d;
};

// Ten Philox rounds; the key schedule is bumped by the Weyl constants between rounds.
__host__ __device__ __forceinline__ Words4 philox4x32_10(Words4 x, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int round = 0; round < 10; ++round) {
    // One wide 32x32->64 multiply per word pair yields both halves.
    const uint64_t p0 = static_cast<uint64_t>(x.a) * 0xD2511F53ull;
    const uint64_t p1 = static_cast<uint64_t>(x.c) * 0xCD9E8D57ull;
    const uint32_t hi0 = static_cast<uint32_t>(p0 >> 32), lo0 = static_cast<uint32_t>(p0);
    const uint32_t hi1 = static_cast<uint32_t>(p1 >> 32), lo1 = static_cast<uint32_t>(p1);
    x = Words4{hi1 ^ x.b ^ k0, lo1, hi0 ^ x.d ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return x;
}

// Two counters under one key: the key schedule is shared between the two streams.
__host__ __device__ __forceinline__ void philox4x32_10_pair(Words4& x, Words4& y, uint32_t k0,
                                                           uint32_t k1) {
#pragma unroll
  for (int round = 0; round < 10; ++round) {
    const uint64_t px0 = static_cast<uint64_t>(x.a) * 0xD2511F53ull;
    const uint64_t px1 = static_cast<uint64_t>(x.c) * 0xCD9E8D57ull;
    const uint64_t py0 = static_cast<uint64_t>(y.a) * 0xD2511F53ull;
    const uint64_t py1 = static_cast<uint64_t>(y.c) * 0xCD9E8D57ull;
    x = Words4{static_cast<uint32_t>(px1 >> 32) ^ x.b ^ k0, static_cast<uint32_t>(px1),
               static_cast<uint32_t>(px0 >> 32) ^ x.d ^ k1, static_cast<uint32_t>(px0)};
    y = Words4{static_cast<uint32_t>(py1 >> 32) ^ y.b ^ k0, static_cast<uint32_t>(py1),
               static_cast<uint32_t>(py0 >> 32) ^ y.d ^ k1, static_cast<uint32_t>(py0)};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// Eight counters under one key (independent streams for instruction-level parallelism).
__device__ __forceinline__ void philox4x32_10_octet(Words4 (&x)[8], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int round = 0; round < 10; ++round) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const uint64_t p0 = static_cast<uint64_t>(x[q].a) * 0xD2511F53ull;
      const uint64_t p1 = static_cast<uint64_t>(x[q].c) * 0xCD9E8D57ull;
      x[q] = Words4{static_cast<uint32_t>(p1 >> 32) ^ x[q].b ^ k0, static_cast<uint32_t>(p1),
                    static_cast<uint32_t>(p0 >> 32) ^ x[q].d ^ k1, static_cast<uint32_t>(p0)};
    }
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// Philox of the Wigner counters (cell, step_lo, step_hi, stream) for eight cells.  In
// the first two rounds one of the two products depends only on (step, stream, key), so
// it is formed once per call instead of once per cell (the words are identical to
// philox4x32_10).
struct PhiloxCellPrefix {
  uint32_t a1, b1;     // words a, b after round 1 (cell independent)
  uint32_t hi0, lo0;   // product a1 * M0 of round 2 (cell independent)
  uint32_t stream_k1;  // stream ^ k1 (round 1)
  uint32_t k0r2, k1r2; // round-2 keys
  uint32_t k0, k1;     // round-3 keys
};

__device__ __forceinline__ PhiloxCellPrefix philox_cell_prefix(uint32_t step_lo, uint32_t step_hi,
                                                               uint32_t stream, uint32_t k0,
                                                               uint32_t k1) {
  PhiloxCellPrefix p;
  const uint64_t q1 = static_cast<uint64_t>(step_hi) * 0xCD9E8D57ull;
  p.a1 = static_cast<uint32_t>(q1 >> 32) ^ step_lo ^ k0;
  p.b1 = static_cast<uint32_t>(q1);
  p.stream_k1 = stream ^ k1;
  p.k0r2 = k0 + 0x9E3779B9u;
  p.k1r2 = k1 + 0xBB67AE85u;
  const uint64_t q0 = static_cast<uint64_t>(p.a1) * 0xD2511F53ull;
  p.hi0 = static_cast<uint32_t>(q0 >> 32);
  p.lo0 = static_cast<uint32_t>(q0);
  p.k0 = p.k0r2 + 0x9E3779B9u;
  p.k1 = p.k1r2 + 0xBB67AE85u;
  return p;
}

template <int N>
__device__ __forceinline__ void philox_cells(const uint32_t (&cell)[N], const PhiloxCellPrefix& p,
                                             Words4 (&x)[N]) {
#pragma unroll
  for (int q = 0; q < N; ++q) {
    // Round 1: a' = hi(c M1) ^ b ^ k0 and b' = lo(c M1) are cell independent.
    const uint64_t r0 = static_cast<uint64_t>(cell[q]) * 0xD2511F53ull;
    const uint32_t c1 = static_cast<uint32_t>(r0 >> 32) ^ p.stream_k1;
    const uint32_t d1 = static_cast<uint32_t>(r0);
    // Round 2: the product of a' is cell independent.
    const uint64_t r1 = static_cast<uint64_t>(c1) * 0xCD9E8D57ull;
    x[q] = Words4{static_cast<uint32_t>(r1 >> 32) ^ p.b1 ^ p.k0r2, static_cast<uint32_t>(r1),
                  p.hi0 ^ d1 ^ p.k1r2, p.lo0};
  }
  uint32_t k0 = p.k0, k1 = p.k1;
#pragma unroll
  for (int round = 2; round < 10; ++round) {
#pragma unroll
    for (int q = 0; q < N; ++q) {
      const uint64_t p0 = static_cast<uint64_t>(x[q].a) * 0xD2511F53ull;
      const uint64_t p1 = static_cast<uint64_t>(x[q].c) * 0xCD9E8D57ull;
      x[q] = Words4{static_cast<uint32_t>(p1 >> 32) ^ x[q].b ^ k0, static_cast<uint32_t>(p1),
                    static_cast<uint32_t>(p0 >> 32) ^ x[q].d ^ k1, static_cast<uint32_t>(p0)};
    }
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

__device__ __forceinline__ Words4 wigner_words(uint32_t cell, uint64_t step, uint32_t stream,
                                               uint64_t seed) {
  return philox4x32_10(Words4{cell, static_cast<uint32_t>(step),
                              static_cast<uint32_t>(step >> 32), stream},
                       static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
}

// Two standard normals scaled by sqrt(variance): returns (re, im) increments.
template <typename T>
struct WignerDraw;

// Single precision uses the SFU approximations.  With m1 = (a >> 8) + 1 and
// m2 = (b >> 8) + 1 (integers in [1, 2^24], so u = m 2^-24):
// * -2 ln u1 = -2 ln2 log2(u1) with the SFU log2 (absolute error below 2^-22 on [0.5, 2]; taken
//   of u1 itself, not of m1, so that radii near 0 keep the fine absolute resolution of values
//   near 1);
// * the angle 2 pi u2 is reduced to (-pi, pi] in integers: m2 - 2^24 when bit 23 of m2 is
//   set (u2 >= 1/2), which is the 24-bit sign extension of m2, then one multiply by
//   2 pi 2^-24 (u2 = 1/2 maps to -pi instead of pi: the same cosine, a sine of the same tiny
//   magnitude); SFU sine and cosine (absolute error about 2^-21 there);
// * sqrt(variance (-2 ln u1)) by the SFU square root (relative error about 2^-23; exact 0
//   at 0).
// The normals stay within a few 1e-6 of the correctly rounded Box-Muller transform except at
// radii below ~1e-3 (u1 within 2^-20 of 1), where the error is bounded in absolute terms by
// ~1e-4 * sqrt(variance).
__device__ __forceinline__ float sqrt_sfu(float x) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

template <>
struct WignerDraw<float> {
  static __device__ __forceinline__ float radius2(uint32_t a) {
    const float u1 = static_cast<float>((a >> 8) + 1u) * 5.9604644775390625e-08f;
    return -1.3862943611198906f * __log2f(u1);  // -2 ln(u1)
  }
  static __device__ __forceinline__ void angle(uint32_t b, float* s, float* c) {
    // ((b >> 8) + 1) << 8, reinterpreted as signed and shifted back: the 24-bit sign extension.
    const int32_t m2 = static_cast<int32_t>((b & 0xFFFFFF00u) + 256u) >> 8;
    __sincosf(static_cast<float>(m2) * 3.7450702829239286e-07f, s, c);  // 2 pi 2^-24
  }
  // Unit-variance normals (r cos theta, r sin theta) of one word quadruple.
  static __device__ __forceinline__ float2 unit(const Words4& w) {
    const float r = sqrt_sfu(radius2(w.a));
    float s, c;
    angle(w.b, &s, &c);
    return make_float2(r * c, r * s);
  }
  // The part of the draw that does not depend on the variance: -2 ln u1 and the angle.
  static __device__ __forceinline__ void prepare(const Words4& w, float& r2, float& s, float& c) {
    r2 = radius2(w.a);
    angle(w.b, &s, &c);
  }
  // Adds sqrt(variance * r2) (cos, sin) to (re, im).
  static __device__ __forceinline__ void add(float variance, float r2, float s, float c, float& re,
                                             float& im) {
    const float amp = sqrt_sfu(variance * r2);
    re = fmaf(amp, c, re);
    im = fmaf(amp, s, im);
  }
  static __device__ __forceinline__ void apply(const Words4& w, float variance, float& re,
                                               float& im) {
    float r2, s, c;
    prepare(w, r2, s, c);
    add(variance, r2, s, c, re, im);
  }
};

template <>
struct WignerDraw<double> {
  static __device__ __forceinline__ void apply(const Words4& w, double variance, double& re,
                                               double& im) {
    const double u1 = (static_cast<double>(w.a >> 5) * 67108864.0 +
                       static_cast<double>(w.b >> 6) + 1.0) * 1.1102230246251565404e-16;
    const double u2 = (static_cast<double>(w.c >> 5) * 67108864.0 +
                       static_cast<double>(w.d >> 6) + 1.0) * 1.1102230246251565404e-16;
    const double amp = sqrt(variance * (-2.0 * log(u1)));
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    re += amp * c;
    im += amp * s;
  }
};

}  // namespace pg
