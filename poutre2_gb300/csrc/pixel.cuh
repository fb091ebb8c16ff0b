// pixel.cuh -- shared pieces of the streaming pixel kernels (pixel.cu, compare.cu): 16-byte
// chunks of pixels moved with uint4 loads and stores that carry the streaming cache hint, the
// per-turn unroll, and the grid size (one full wave of resident CTAs, striding over the chunks).
#pragma once

#include "common.cuh"

namespace pg {
namespace pixel_detail {

constexpr int kPThreads = 256;

template <typename T, int N> struct alignas(16) Chunk { T v[N]; };

template <typename T, int N> __device__ __forceinline__ void chunk_load(Chunk<T, N> &d, const T *p) {
  if constexpr ((sizeof(T) * N) % 16 == 0) {
    const uint4 *q = reinterpret_cast<const uint4 *>(p);
    uint4 *r = reinterpret_cast<uint4 *>(d.v);
#pragma unroll
    for (int k = 0; k < (int)(sizeof(T) * N / 16); ++k) r[k] = __ldcs(q + k);
  } else {
#pragma unroll
    for (int k = 0; k < N; ++k) d.v[k] = p[k];
  }
}
template <typename T, int N> __device__ __forceinline__ void chunk_store(T *p, const Chunk<T, N> &d) {
  if constexpr ((sizeof(T) * N) % 16 == 0) {
    uint4 *q = reinterpret_cast<uint4 *>(p);
    const uint4 *r = reinterpret_cast<const uint4 *>(d.v);
#pragma unroll
    for (int k = 0; k < (int)(sizeof(T) * N / 16); ++k) __stcs(q + k, r[k]);
  } else {
#pragma unroll
    for (int k = 0; k < N; ++k) p[k] = d.v[k];
  }
}

// pixels per chunk: 16 bytes of the narrower of two pixel types
template <typename A, typename B> __host__ __device__ constexpr int chunk_pixels() {
  return 16 / (int)(sizeof(A) < sizeof(B) ? sizeof(A) : sizeof(B));
}

// Chunks in flight per thread and loop turn: all loads of a turn are issued before its first store,
// aiming at LOAD bytes of loads per chunk x U = 128 bytes in flight per thread (one 16-byte load per
// thread leaves HBM latency-bound), with at most HOLD bytes x U = 256 bytes of chunks held in
// registers; the U chunks of a turn are one grid stride apart, so each warp access stays contiguous.
template <int LOAD, int HOLD, int LOAD_BUDGET = 128, int HOLD_BUDGET = 256>
__host__ __device__ constexpr int unroll_for() {
  constexpr int a = LOAD_BUDGET / LOAD, b = HOLD_BUDGET / HOLD;
  constexpr int u = a < b ? a : b;
  return u < 1 ? 1 : (u > 8 ? 8 : u);
}

// 8- and 16-bit pixels of one type are processed four / two per 32-bit word with the CUDA SIMD
// intrinsics (__vminu4, __vcmpgtu2, ...), which give the per-pixel results bit for bit.
template <typename T> inline constexpr bool kPacked = std::is_same_v<T, uint8_t> || std::is_same_v<T, uint16_t>;

template <typename T, int N> __device__ __forceinline__ uint32_t *words(Chunk<T, N> &c) {
  return reinterpret_cast<uint32_t *>(c.v);
}
template <typename T, int N> __device__ __forceinline__ const uint32_t *words(const Chunk<T, N> &c) {
  return reinterpret_cast<const uint32_t *>(c.v);
}

inline unsigned grid_for_chunks(int64_t chunks) {
  int64_t b = ceil_div(chunks > 0 ? chunks : 1, kPThreads);
  // 8 CTAs of 256 threads per SM: one wave at the SM's 2048-thread limit (variants whose registers
  // allow fewer resident CTAs run it in several)
  const int64_t cap = (int64_t)num_sms() * (2048 / kPThreads);
  return (unsigned)(b < cap ? b : cap);
}

inline bool aligned16(const void *p) { return p == nullptr || ((uintptr_t)p & 15u) == 0; }

// PG_DISPATCH_PTYPE under a second name, for the output type inside a dispatch on the input type (a
// macro is not expanded again inside its own expansion)
#define PG_DISPATCH_PTYPE2(pt, T, ...)                                        \
  switch (pt) {                                                               \
    case PG_PTYPE_U8: { using T = uint8_t; __VA_ARGS__; } break;              \
    case PG_PTYPE_U16: { using T = uint16_t; __VA_ARGS__; } break;            \
    case PG_PTYPE_I32: { using T = int32_t; __VA_ARGS__; } break;             \
    case PG_PTYPE_I64: { using T = int64_t; __VA_ARGS__; } break;             \
    case PG_PTYPE_F32: { using T = float; __VA_ARGS__; } break;               \
    case PG_PTYPE_F64: { using T = double; __VA_ARGS__; } break;              \
    default: return ::pg::fail(PG_ERR_UNSUPPORTED_PTYPE, "unsupported PTYPE"); \
  }

}  // namespace pixel_detail
}  // namespace pg
