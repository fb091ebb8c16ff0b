// words.cuh -- pixels packed in 32-bit words (4 u8, 2 u16 or 1 i32/f32): SIMD-in-word
// min/max, splat, packing, sub-word shifts and E x E transposes.
#pragma once

#include "common.cuh"

namespace pg {

template <typename T, bool SUP> __device__ __forceinline__ uint32_t wop(uint32_t a, uint32_t b) {
  if constexpr (sizeof(T) == 1) return SUP ? __vmaxu4(a, b) : __vminu4(a, b);
  else if constexpr (sizeof(T) == 2) {
    uint32_t r;  // native 2 x 16-bit unsigned min/max
    if constexpr (SUP) asm("max.u16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    else asm("min.u16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
  }
  else if constexpr (std::is_same_v<T, int32_t>) {
    const int x = (int)a, y = (int)b;
    return (uint32_t)(SUP ? max(x, y) : min(x, y));
  } else {
    const float x = __uint_as_float(a), y = __uint_as_float(b);
    return __float_as_uint(SUP ? fmaxf(x, y) : fminf(x, y));
  }
}

template <typename T> __device__ __forceinline__ uint32_t splat(T v) {
  if constexpr (sizeof(T) == 1) return (uint32_t)v * 0x01010101u;
  else if constexpr (sizeof(T) == 2) return (uint32_t)v | ((uint32_t)v << 16);
  else if constexpr (std::is_same_v<T, float>) return __float_as_uint(v);
  else return (uint32_t)v;
}

template <typename T> __device__ __forceinline__ uint32_t pack(const T (&e)[4 / sizeof(T)]) {
  uint32_t w = 0;
  if constexpr (sizeof(T) == 4) {
    if constexpr (std::is_same_v<T, float>) w = __float_as_uint(e[0]);
    else w = (uint32_t)e[0];
  } else {
    for (int i = 0; i < 4 / (int)sizeof(T); ++i) w |= (uint32_t)e[i] << (8 * sizeof(T) * i);
  }
  return w;
}

// pixels s .. s+E-1 of the 2E-pixel run (lo, hi), s in [0, E)
template <typename T> __device__ __forceinline__ uint32_t shift_px(uint32_t lo, uint32_t hi, int s) {
  if constexpr (sizeof(T) == 4) return s ? hi : lo;
  else return __funnelshift_r(lo, hi, (unsigned)(s * 8 * (int)sizeof(T)));
}

// E x E transpose of pixels held as E words (an involution)
template <typename T> __device__ __forceinline__ void transpose_block(uint32_t (&w)[4 / sizeof(T)]) {
  if constexpr (sizeof(T) == 2) {
    const uint32_t a = w[0], b = w[1];
    w[0] = __byte_perm(a, b, 0x5410);
    w[1] = __byte_perm(a, b, 0x7632);
  } else if constexpr (sizeof(T) == 1) {
    const uint32_t t0 = __byte_perm(w[0], w[1], 0x5140), t1 = __byte_perm(w[2], w[3], 0x5140);
    const uint32_t t2 = __byte_perm(w[0], w[1], 0x7362), t3 = __byte_perm(w[2], w[3], 0x7362);
    w[0] = __byte_perm(t0, t1, 0x5410);
    w[1] = __byte_perm(t0, t1, 0x7632);
    w[2] = __byte_perm(t2, t3, 0x5410);
    w[3] = __byte_perm(t2, t3, 0x7632);
  }
}

}  // namespace pg
