// pixel.cu -- poutre2's pixel_processing entry points on device images:
//   ArithInvertImage / ArithSupImage / ArithInfImage / ArithSaturatedAddImage / ArithSaturatedSubImage
//     (include/poutre/pixel_processing/arith.hpp:31-53; ops in details/arith_op_t.hpp:40-445),
//   ConvertInto (copy_convert.hpp; CopyOpDispatcher copy_convert_t.hpp:33-86: static_cast per pixel).
//
// One streaming kernel per operation and pixel type(s): every thread moves 16-byte chunks of the
// narrower operand type (uint4 loads and stores with the streaming cache hint, since each byte is
// touched once), the grid is sized to the SM count and strides over the chunks, and the last
// n mod chunk pixels are done one by one.  Operands that are not 16-byte aligned take the same
// kernel with one-pixel chunks.  Loads are coherent and no pointer is __restrict__, so an output
// may be one of the inputs (same buffer, same type): each pixel is read before it is written, by
// the same thread, as in the reference, which allows in-place arithmetic.
#include "pixel.cuh"

namespace pg {
namespace {
using namespace pixel_detail;

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

// the same operation on the four bytes / two halfwords of a word
template <int OP, typename T> __device__ __forceinline__ uint32_t arith_word(uint32_t a, uint32_t b) {
  if constexpr (sizeof(T) == 1) {
    if constexpr (OP == PX_INF) return __vminu4(a, b);
    else if constexpr (OP == PX_SUP) return __vmaxu4(a, b);
    else if constexpr (OP == PX_SADD) return __vaddus4(a, b);
    else if constexpr (OP == PX_SSUB) return __vsubus4(a, b);
    else return __vneg4(a);
  } else {
    if constexpr (OP == PX_INF) return __vminu2(a, b);
    else if constexpr (OP == PX_SUP) return __vmaxu2(a, b);
    else if constexpr (OP == PX_SADD) return __vaddus2(a, b);
    else if constexpr (OP == PX_SSUB) return __vsubus2(a, b);
    else return __vneg2(a);
  }
}

template <typename T, int OP, bool VEC>
__global__ void __launch_bounds__(kPThreads) k_arith(const T *a, const T *b, T *o, int64_t n) {
  constexpr int N = VEC ? 16 / (int)sizeof(T) : 1;
  constexpr int U = VEC ? unroll_for<OP == PX_NEG ? 16 : 32, OP == PX_NEG ? 16 : 32>() : 1;
  const int64_t chunks = n / N, stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t c0 = t0; c0 < chunks; c0 += U * stride) {
    Chunk<T, N> x[U], y[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t c = c0 + u * stride;
      if (c < chunks) {
        chunk_load(x[u], a + c * N);
        if constexpr (OP != PX_NEG) chunk_load(y[u], b + c * N);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t c = c0 + u * stride;
      if (c < chunks) {
        Chunk<T, N> r;
        if constexpr (VEC && kPacked<T>) {
#pragma unroll
          for (int k = 0; k < 4; ++k) words(r)[k] = arith_word<OP, T>(words(x[u])[k], words(y[u])[k]);
        } else {
#pragma unroll
          for (int k = 0; k < N; ++k) r.v[k] = arith<OP>(x[u].v[k], OP != PX_NEG ? y[u].v[k] : T(0));
        }
        chunk_store(o + c * N, r);
      }
    }
  }
  const int64_t i = chunks * N + t0;  // the n mod N remainder
  if (i < n) o[i] = arith<OP>(a[i], OP != PX_NEG ? b[i] : T(0));
}

template <typename TI, typename TO, bool VEC>
__global__ void __launch_bounds__(kPThreads) k_convert(const TI *in, TO *out, int64_t n) {
  constexpr int N = VEC ? chunk_pixels<TI, TO>() : 1;
  constexpr int U = VEC ? unroll_for<N * (int)sizeof(TI), N * (int)sizeof(TI), 64>() : 1;
  const int64_t chunks = n / N, stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t c0 = t0; c0 < chunks; c0 += U * stride) {
    Chunk<TI, N> x[U];
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (c0 + u * stride < chunks) chunk_load(x[u], in + (c0 + u * stride) * N);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t c = c0 + u * stride;
      if (c < chunks) {
        Chunk<TO, N> r;
#pragma unroll
        for (int k = 0; k < N; ++k) r.v[k] = static_cast<TO>(x[u].v[k]);
        chunk_store(out + c * N, r);
      }
    }
  }
  const int64_t i = chunks * N + t0;
  if (i < n) out[i] = static_cast<TO>(in[i]);
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
