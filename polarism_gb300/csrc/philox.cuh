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

__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t x, uint32_t y) {
#if defined(__CUDA_ARCH__)
  return __umulhi(x, y);
#else
  return static_cast<uint32_t>((static_cast<uint64_t>(x) * y) >> 32);
#endif
}

// Ten Philox rounds; the key schedule is bumped by the Weyl constants between rounds.
__host__ __device__ __forceinline__ Words4 philox4x32_10(Words4 x, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int round = 0; round < 10; ++round) {
    const uint32_t hi0 = mulhi32(0xD2511F53u, x.a);
    const uint32_t lo0 = 0xD2511F53u * x.a;
    const uint32_t hi1 = mulhi32(0xCD9E8D57u, x.c);
    const uint32_t lo1 = 0xCD9E8D57u * x.c;
    x = Words4{hi1 ^ x.b ^ k0, lo1, hi0 ^ x.d ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return x;
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

template <>
struct WignerDraw<float> {
  static __device__ __forceinline__ void apply(const Words4& w, float variance, float& re,
                                               float& im) {
    const float u1 = static_cast<float>((w.a >> 8) + 1u) * 5.9604644775390625e-08f;
    const float u2 = static_cast<float>((w.b >> 8) + 1u) * 5.9604644775390625e-08f;
    const float amp = sqrtf(variance * (-2.0f * logf(u1)));
    float s, c;
    sincosf(6.283185307179586f * u2, &s, &c);
    re += amp * c;
    im += amp * s;
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
    sincos(6.283185307179586476925286766559 * u2, &s, &c);
    re += amp * c;
    im += amp * s;
  }
};

}  // namespace pg
