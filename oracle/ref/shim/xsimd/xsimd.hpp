// Project-written stand-in for the subset of xsimd 14.2.0 that poutre2 calls
// (batch/batch_bool, aligned and unaligned load/store, min, max, select, ssub, sadd,
// lane-wise arithmetic and comparisons, aligned_allocator, default_arch::alignment).
// xsimd itself is not vendored in the poutre2 tree and there is no network here.
//
// A batch is a fixed-width array of lanes: 32 bytes (the AVX2 width poutre2 targets on
// x86-64) or 16 bytes (NEON, what poutre2's build selects on aarch64).  Every operation
// is a plain lane loop that gcc -O3 turns into the host's vector instructions, so the
// reference's simd::transform bodies run vectorised.  Semantics follow the published
// xsimd ones: min/max lane-wise, saturating integer add/sub, select(mask, a, b).
#pragma once
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <new>
#include <type_traits>

namespace xsimd {

#if defined(__aarch64__) || defined(__ARM_NEON)
inline constexpr std::size_t kVectorBytes = 16;
#else
inline constexpr std::size_t kVectorBytes = 32;
#endif

struct default_arch {
  static constexpr std::size_t alignment() { return kVectorBytes; }
};

template <class T, class A = default_arch>
struct batch {
  static constexpr std::size_t size = kVectorBytes / sizeof(T);
  alignas(kVectorBytes) T lane[size];
  batch() = default;
  batch(T s) {
    for (std::size_t i = 0; i < size; ++i) lane[i] = s;
  }
};

template <class T, class A = default_arch>
struct batch_bool {
  static constexpr std::size_t size = kVectorBytes / sizeof(T);
  bool lane[size];
};

template <class T>
inline batch<T> load_unaligned(const T *p) {
  batch<T> r;
  for (std::size_t i = 0; i < batch<T>::size; ++i) r.lane[i] = p[i];
  return r;
}
template <class T>
inline batch<T> load_aligned(const T *p) {
  return load_unaligned(p);
}
template <class T>
inline void store_unaligned(T *p, const batch<T> &b) {
  for (std::size_t i = 0; i < batch<T>::size; ++i) p[i] = b.lane[i];
}
template <class T>
inline void store_aligned(T *p, const batch<T> &b) {
  store_unaligned(p, b);
}

#define XS_STANDIN_BINARY(NAME, EXPR)                                   \
  template <class T>                                                    \
  inline batch<T> NAME(const batch<T> &a, const batch<T> &b) {          \
    batch<T> r;                                                         \
    for (std::size_t i = 0; i < batch<T>::size; ++i) {                  \
      const T x = a.lane[i], y = b.lane[i];                             \
      r.lane[i] = (EXPR);                                               \
    }                                                                   \
    return r;                                                           \
  }
XS_STANDIN_BINARY(min, (y < x ? y : x))
XS_STANDIN_BINARY(max, (x < y ? y : x))
XS_STANDIN_BINARY(operator+, static_cast<T>(x + y))
XS_STANDIN_BINARY(operator-, static_cast<T>(x - y))
XS_STANDIN_BINARY(operator*, static_cast<T>(x * y))
XS_STANDIN_BINARY(operator/, static_cast<T>(x / y))
#undef XS_STANDIN_BINARY

template <class T>
inline T saturate_add_(T x, T y) {
  if constexpr (std::is_integral_v<T>) {
    using W = std::conditional_t<(sizeof(T) < 8), std::int64_t, __int128>;
    W r = static_cast<W>(x) + static_cast<W>(y);
    if (r < static_cast<W>(std::numeric_limits<T>::min())) return std::numeric_limits<T>::min();
    if (r > static_cast<W>(std::numeric_limits<T>::max())) return std::numeric_limits<T>::max();
    return static_cast<T>(r);
  } else {
    return x + y;
  }
}
template <class T>
inline T saturate_sub_(T x, T y) {
  if constexpr (std::is_integral_v<T>) {
    using W = std::conditional_t<(sizeof(T) < 8), std::int64_t, __int128>;
    W r = static_cast<W>(x) - static_cast<W>(y);
    if (r < static_cast<W>(std::numeric_limits<T>::min())) return std::numeric_limits<T>::min();
    if (r > static_cast<W>(std::numeric_limits<T>::max())) return std::numeric_limits<T>::max();
    return static_cast<T>(r);
  } else {
    return x - y;
  }
}
template <class T>
inline batch<T> sadd(const batch<T> &a, const batch<T> &b) {
  batch<T> r;
  for (std::size_t i = 0; i < batch<T>::size; ++i) r.lane[i] = saturate_add_(a.lane[i], b.lane[i]);
  return r;
}
template <class T>
inline batch<T> ssub(const batch<T> &a, const batch<T> &b) {
  batch<T> r;
  for (std::size_t i = 0; i < batch<T>::size; ++i) r.lane[i] = saturate_sub_(a.lane[i], b.lane[i]);
  return r;
}
template <class T>
inline batch<T> operator-(const batch<T> &a) {
  batch<T> r;
  for (std::size_t i = 0; i < batch<T>::size; ++i) r.lane[i] = static_cast<T>(-a.lane[i]);
  return r;
}

#define XS_STANDIN_COMPARE(OP)                                          \
  template <class T>                                                    \
  inline batch_bool<T> operator OP(const batch<T> &a, const batch<T> &b) { \
    batch_bool<T> r;                                                    \
    for (std::size_t i = 0; i < batch<T>::size; ++i) r.lane[i] = a.lane[i] OP b.lane[i]; \
    return r;                                                           \
  }
XS_STANDIN_COMPARE(==)
XS_STANDIN_COMPARE(!=)
XS_STANDIN_COMPARE(<)
XS_STANDIN_COMPARE(>)
XS_STANDIN_COMPARE(<=)
XS_STANDIN_COMPARE(>=)
#undef XS_STANDIN_COMPARE

template <class T>
inline batch_bool<T> operator&&(const batch_bool<T> &a, const batch_bool<T> &b) {
  batch_bool<T> r;
  for (std::size_t i = 0; i < batch_bool<T>::size; ++i) r.lane[i] = a.lane[i] && b.lane[i];
  return r;
}
template <class T>
inline batch_bool<T> operator&(const batch_bool<T> &a, const batch_bool<T> &b) {
  return a && b;
}
template <class T>
inline batch<T> select(const batch_bool<T> &m, const batch<T> &a, const batch<T> &b) {
  batch<T> r;
  for (std::size_t i = 0; i < batch<T>::size; ++i) r.lane[i] = m.lane[i] ? a.lane[i] : b.lane[i];
  return r;
}

template <class T>
struct simd_type {
  static constexpr std::size_t size = batch<T>::size;
};

template <class T, std::size_t Align>
struct aligned_allocator {
  using value_type = T;
  template <class U>
  struct rebind {
    using other = aligned_allocator<U, Align>;
  };
  aligned_allocator() = default;
  template <class U>
  aligned_allocator(const aligned_allocator<U, Align> &) {}
  T *allocate(std::size_t n) {
    return static_cast<T *>(::operator new(n * sizeof(T), std::align_val_t(Align)));
  }
  void deallocate(T *p, std::size_t) { ::operator delete(p, std::align_val_t(Align)); }
  template <class U>
  bool operator==(const aligned_allocator<U, Align> &) const { return true; }
  template <class U>
  bool operator!=(const aligned_allocator<U, Align> &) const { return false; }
};

}  // namespace xsimd
