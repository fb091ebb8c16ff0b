// pixel.cu -- poutre2's pixel_processing entry points on device images:
//   ArithInvertImage / ArithSupImage / ArithInfImage / ArithSaturatedAddImage / ArithSaturatedSubImage
//     (include/poutre/pixel_processing/arith.hpp:31-53; ops in details/arith_op_t.hpp:40-445),
//   CompareImage, all eight scalar / image overloads (compare.hpp:31-84; OpComp* compare_op_t.hpp:41-165),
//   ConvertInto (copy_convert.hpp; CopyOpDispatcher copy_convert_t.hpp:33-86: static_cast per pixel).
//
// One streaming kernel per operation and pixel type(s): every thread moves 16-byte chunks of the
// narrower operand type (uint4 loads and stores with the streaming cache hint, since each byte is
// touched once), the grid is sized to the SM count and strides over the chunks, and the last
// n mod chunk pixels are done one by one.  Operands that are not 16-byte aligned take the same
// kernel with one-pixel chunks.  Loads are coherent and no pointer is __restrict__, so an output
// may be one of the inputs (same buffer, same type): each pixel is read before it is written, by
// the same thread, as in the reference, which allows in-place arithmetic.
#include <cstring>

#include "common.cuh"

namespace pg {
namespace {

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

// -a in the pixel type, wrapping for unsigned pixels and for the most negative signed value
template <typename T> __device__ __forceinline__ T negate(T a) {
  if constexpr (std::is_integral_v<T>) {
    using U = std::make_unsigned_t<T>;
    return (T)(U)(U(0) - (U)a);
  } else {
    return -a;
  }
}

template <int OP, typename T> __device__ __forceinline__ T arith(T a, T b) {
  if constexpr (OP == PX_INF) return a < b ? a : b;      // op_Inf: a0 < a1 ? a0 : a1
  else if constexpr (OP == PX_SUP) return a > b ? a : b; // op_Sup: a0 > a1 ? a0 : a1
  else if constexpr (OP == PX_SADD) return sat_add_c(a, b);
  else if constexpr (OP == PX_SSUB) return sat_sub_c(a, b);
  else return negate(a);
}

template <typename T, int OP, bool VEC>
__global__ void __launch_bounds__(kPThreads) k_arith(const T *a, const T *b, T *o, int64_t n) {
  constexpr int N = VEC ? 16 / (int)sizeof(T) : 1;
  const int64_t chunks = n / N, stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t c = t0; c < chunks; c += stride) {
    Chunk<T, N> x, y, r;
    chunk_load(x, a + c * N);
    if constexpr (OP != PX_NEG) chunk_load(y, b + c * N);
#pragma unroll
    for (int k = 0; k < N; ++k) r.v[k] = arith<OP>(x.v[k], OP != PX_NEG ? y.v[k] : T(0));
    chunk_store(o + c * N, r);
  }
  const int64_t i = chunks * N + t0;  // the n mod N remainder
  if (i < n) o[i] = arith<OP>(a[i], OP != PX_NEG ? b[i] : T(0));
}

template <typename T> __device__ __forceinline__ bool comp_op(int op, T a, T b) {
  switch (op) {
    case PG_COMP_EQUAL: return a == b;
    case PG_COMP_DIFF: return a != b;
    case PG_COMP_SUP: return a > b;
    case PG_COMP_SUP_EQUAL: return a >= b;
    case PG_COMP_INF: return a < b;
    default: return a <= b;  // PG_COMP_INF_EQUAL
  }
}

// an operand of CompareImage on the device: an image, or (p == nullptr) a scalar of its type
template <typename T> struct Operand {
  const T *p;
  T v;
};

template <typename TI, typename TO, bool VEC>
__global__ void __launch_bounds__(kPThreads)
    k_compare(const TI *in, int op, Operand<TI> comp, Operand<TO> vt, Operand<TO> vf, TO *out, int64_t n) {
  constexpr int N = VEC ? chunk_pixels<TI, TO>() : 1;
  const int64_t chunks = n / N, stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t c = t0; c < chunks; c += stride) {
    const int64_t i = c * N;
    Chunk<TI, N> x, y;
    Chunk<TO, N> t, f, r;
    chunk_load(x, in + i);
    if (comp.p) chunk_load(y, comp.p + i);
    else
#pragma unroll
      for (int k = 0; k < N; ++k) y.v[k] = comp.v;
    if (vt.p) chunk_load(t, vt.p + i);
    else
#pragma unroll
      for (int k = 0; k < N; ++k) t.v[k] = vt.v;
    if (vf.p) chunk_load(f, vf.p + i);
    else
#pragma unroll
      for (int k = 0; k < N; ++k) f.v[k] = vf.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.v[k] = comp_op(op, x.v[k], y.v[k]) ? t.v[k] : f.v[k];
    chunk_store(out + i, r);
  }
  const int64_t i = chunks * N + t0;
  if (i < n) {
    const TI y = comp.p ? comp.p[i] : comp.v;
    out[i] = comp_op(op, in[i], y) ? (vt.p ? vt.p[i] : vt.v) : (vf.p ? vf.p[i] : vf.v);
  }
}

template <typename TI, typename TO, bool VEC>
__global__ void __launch_bounds__(kPThreads) k_convert(const TI *in, TO *out, int64_t n) {
  constexpr int N = VEC ? chunk_pixels<TI, TO>() : 1;
  const int64_t chunks = n / N, stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t c = t0; c < chunks; c += stride) {
    Chunk<TI, N> x;
    Chunk<TO, N> r;
    chunk_load(x, in + c * N);
#pragma unroll
    for (int k = 0; k < N; ++k) r.v[k] = static_cast<TO>(x.v[k]);
    chunk_store(out + c * N, r);
  }
  const int64_t i = chunks * N + t0;
  if (i < n) out[i] = static_cast<TO>(in[i]);
}

unsigned grid_for_chunks(int64_t chunks) {
  int64_t b = ceil_div(chunks > 0 ? chunks : 1, kPThreads);
  const int64_t cap = (int64_t)num_sms() * (2048 / kPThreads);  // one full wave of resident CTAs
  return (unsigned)(b < cap ? b : cap);
}

bool aligned16(const void *p) { return p == nullptr || ((uintptr_t)p & 15u) == 0; }

template <typename T> Operand<T> operand_of(const void *img, double v) {
  return Operand<T>{static_cast<const T *>(img), static_cast<T>(v)};
}

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

template <typename T, int OP>
void arith_launch(const void *a, const void *b, void *o, int64_t n, cudaStream_t s) {
  const T *pa = static_cast<const T *>(a), *pb = static_cast<const T *>(b);
  T *po = static_cast<T *>(o);
  if (aligned16(a) && aligned16(b) && aligned16(o))
    k_arith<T, OP, true><<<grid_for_chunks(n / (16 / (int)sizeof(T))), kPThreads, 0, s>>>(pa, pb, po, n);
  else
    k_arith<T, OP, false><<<grid_for_chunks(n), kPThreads, 0, s>>>(pa, pb, po, n);
}

}  // namespace

pg_status launch_pixel_arith(int op, const pg_image &a, const pg_image *b, const pg_image &out, cudaStream_t s) {
  const int64_t n = dims_of(a).count();
  if (n == 0) return PG_OK;
  const void *pb = b ? b->data : nullptr;
  PG_DISPATCH_PTYPE(a.ptype, T, {
    switch (op) {
      case PX_INF: arith_launch<T, PX_INF>(a.data, pb, out.data, n, s); break;
      case PX_SUP: arith_launch<T, PX_SUP>(a.data, pb, out.data, n, s); break;
      case PX_SADD: arith_launch<T, PX_SADD>(a.data, pb, out.data, n, s); break;
      case PX_SSUB: arith_launch<T, PX_SSUB>(a.data, pb, out.data, n, s); break;
      default: arith_launch<T, PX_NEG>(a.data, pb, out.data, n, s); break;
    }
  });
  return cuda_status(cudaGetLastError(), "pixel arithmetic kernel launch");
}

pg_status launch_compare(const pg_image &in, int op, const CompareOperand &comp, const CompareOperand &vt,
                         const CompareOperand &vf, const pg_image &out, cudaStream_t s) {
  const int64_t n = dims_of(in).count();
  if (n == 0) return PG_OK;
  const bool vec = aligned16(in.data) && aligned16(comp.data) && aligned16(vt.data) && aligned16(vf.data) &&
                   aligned16(out.data);
  PG_DISPATCH_PTYPE(in.ptype, TI, {
    PG_DISPATCH_PTYPE2(out.ptype, TO, {
      const TI *pi = static_cast<const TI *>(in.data);
      TO *po = static_cast<TO *>(out.data);
      const auto c = operand_of<TI>(comp.data, comp.value);
      const auto t = operand_of<TO>(vt.data, vt.value), f = operand_of<TO>(vf.data, vf.value);
      if (vec)
        k_compare<TI, TO, true><<<grid_for_chunks(n / chunk_pixels<TI, TO>()), kPThreads, 0, s>>>(pi, op, c, t, f,
                                                                                                  po, n);
      else
        k_compare<TI, TO, false><<<grid_for_chunks(n), kPThreads, 0, s>>>(pi, op, c, t, f, po, n);
    });
  });
  return cuda_status(cudaGetLastError(), "compare kernel launch");
}

pg_status launch_convert(const pg_image &in, const pg_image &out, cudaStream_t s) {
  const int64_t n = dims_of(in).count();
  if (n == 0) return PG_OK;
  const bool vec = aligned16(in.data) && aligned16(out.data);
  PG_DISPATCH_PTYPE(in.ptype, TI, {
    PG_DISPATCH_PTYPE2(out.ptype, TO, {
      const TI *pi = static_cast<const TI *>(in.data);
      TO *po = static_cast<TO *>(out.data);
      if (vec)
        k_convert<TI, TO, true><<<grid_for_chunks(n / chunk_pixels<TI, TO>()), kPThreads, 0, s>>>(pi, po, n);
      else
        k_convert<TI, TO, false><<<grid_for_chunks(n), kPThreads, 0, s>>>(pi, po, n);
    });
  });
  return cuda_status(cudaGetLastError(), "convert kernel launch");
}

}  // namespace pg
