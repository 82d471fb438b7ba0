// fp_convert.h — host-side IEEE-754 narrowing conversions (round to nearest,
// ties to even), written from the format definitions. Used to quantise
// matrix values on the host exactly as a C++ `half(double)` / `half(float)`
// conversion does (the reference reads MatrixMarket doubles straight into
// `half`, mmio_highlevel.h:608).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace smat {

inline uint32_t f32_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}
inline float bits_f32(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

inline uint16_t f64_to_f16_bits(double d) {
  uint64_t x;
  std::memcpy(&x, &d, 8);
  const uint16_t sign = (uint16_t)((x >> 48) & 0x8000);
  const uint64_t ax = x & 0x7fffffffffffffffull;
  if (ax >= 0x7ff0000000000000ull) return sign | (ax > 0x7ff0000000000000ull ? 0x7e00 : 0x7c00);
  if (std::fabs(d) >= 65520.0) return sign | 0x7c00;
  if (std::fabs(d) < 6.103515625e-05) {  // below 2^-14: subnormal half (or zero)
    double v = std::nearbyint(std::fabs(d) * 16777216.0);  // exact scaling, RNE
    return sign | (uint16_t)v;
  }
  const int e = (int)(ax >> 52) - 1023 + 15;
  const uint64_t mant = ax & 0xfffffffffffffull;
  uint32_t h = ((uint32_t)e << 10) | (uint32_t)(mant >> 42);
  const uint64_t rem = mant & ((1ull << 42) - 1), halfway = 1ull << 41;
  if (rem > halfway || (rem == halfway && (h & 1))) h++;
  return sign | (uint16_t)h;
}

inline uint16_t f32_to_f16_bits(float f) { return f64_to_f16_bits((double)f); }

inline float f16_bits_to_f32(uint16_t h) {
  const uint32_t sign = (uint32_t)(h & 0x8000) << 16;
  const uint32_t e = (h >> 10) & 0x1f, m = h & 0x3ff;
  if (e == 0) {
    float v = (float)m * 5.9604644775390625e-08f;  // m * 2^-24
    return sign ? -v : v;
  }
  if (e == 31) return bits_f32(sign | 0x7f800000u | (m << 13));
  return bits_f32(sign | ((e - 15 + 127) << 23) | (m << 13));
}

inline uint16_t f32_to_bf16_bits(float f) {
  uint32_t u = f32_bits(f);
  if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40);
  u += 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

inline float bf16_bits_to_f32(uint16_t b) { return bits_f32((uint32_t)b << 16); }

// OCP FP8 E4M3 ("e4m3fn": bias 7, no infinities, 0x7f = NaN, max 448),
// saturating to +-448.
inline uint8_t f32_to_e4m3_bits(float f) {
  const uint8_t sign = (f32_bits(f) >> 24) & 0x80;
  float a = std::fabs(f);
  if (std::isnan(f)) return 0x7f;
  if (a >= 464.0f) return sign | 0x7e;  // 448 + half an ulp rounds to NaN in RN; saturate
  if (a < 0.015625f) {                  // below 2^-6: subnormal, step 2^-9
    float v = std::nearbyint(a * 512.0f);
    return sign | (uint8_t)v;           // v == 8 lands on the smallest normal
  }
  int e;
  float m = std::frexp(a, &e);          // a = m * 2^e, m in [0.5, 1)
  // a = 1.f * 2^(e-1); 3 fraction bits
  float scaled = std::ldexp(a, 3 - (e - 1));  // in [8, 16)
  float r = std::nearbyint(scaled);
  int exp = e - 1;
  if (r >= 16.0f) {
    r = 8.0f;
    exp++;
  }
  uint32_t frac = (uint32_t)r - 8u;
  uint32_t be = (uint32_t)(exp + 7);
  uint8_t out = (uint8_t)((be << 3) | frac);
  if (out > 0x7e) out = 0x7e;
  return sign | out;
}

inline float e4m3_bits_to_f32(uint8_t b) {
  const float s = (b & 0x80) ? -1.0f : 1.0f;
  const int e = (b >> 3) & 0xf, m = b & 7;
  if (e == 0xf && m == 7) return NAN;
  if (e == 0) return s * std::ldexp((float)m, -9);
  return s * std::ldexp(1.0f + m / 8.0f, e - 7);
}

}  // namespace smat
