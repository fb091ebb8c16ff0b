// compare.cu -- poutre2's CompareImage on device images, all eight scalar / image overloads
// (include/poutre/pixel_processing/compare.hpp:31-84; OpComp* compare_op_t.hpp:41-165):
// out = op(in, comp) ? valtrue : valfalse, comp of the input's pixel type, valtrue / valfalse and
// out of the output's.  Streaming chunks as in pixel.cu; the operation is a template parameter of
// the aligned loop (one specialised loop per CompOpType, chosen once per launch).
#include "pixel.cuh"

namespace pg {
namespace {
using namespace pixel_detail;

// OP = 0: the operation `op` chosen at run time
template <int OP, typename T> __device__ __forceinline__ bool comp_op(int op, T a, T b) {
  if constexpr (OP == 0) {
    switch (op) {
      case PG_COMP_EQUAL: return a == b;
      case PG_COMP_DIFF: return a != b;
      case PG_COMP_SUP: return a > b;
      case PG_COMP_SUP_EQUAL: return a >= b;
      case PG_COMP_INF: return a < b;
      default: return a <= b;
    }
  } else if constexpr (OP == PG_COMP_EQUAL) return a == b;
  else if constexpr (OP == PG_COMP_DIFF) return a != b;
  else if constexpr (OP == PG_COMP_SUP) return a > b;
  else if constexpr (OP == PG_COMP_SUP_EQUAL) return a >= b;
  else if constexpr (OP == PG_COMP_INF) return a < b;
  else return a <= b;  // PG_COMP_INF_EQUAL
}

// per-byte / per-halfword compare masks (0xff / 0xffff where true) for 8- / 16-bit unsigned pixels
template <int OP, typename T> __device__ __forceinline__ uint32_t comp_mask(int op, uint32_t a, uint32_t b) {
  const int o = OP == 0 ? op : OP;
  if constexpr (sizeof(T) == 1) {
    switch (o) {
      case PG_COMP_EQUAL: return __vcmpeq4(a, b);
      case PG_COMP_DIFF: return __vcmpne4(a, b);
      case PG_COMP_SUP: return __vcmpgtu4(a, b);
      case PG_COMP_SUP_EQUAL: return __vcmpgeu4(a, b);
      case PG_COMP_INF: return __vcmpltu4(a, b);
      default: return __vcmpleu4(a, b);
    }
  } else {
    switch (o) {
      case PG_COMP_EQUAL: return __vcmpeq2(a, b);
      case PG_COMP_DIFF: return __vcmpne2(a, b);
      case PG_COMP_SUP: return __vcmpgtu2(a, b);
      case PG_COMP_SUP_EQUAL: return __vcmpgeu2(a, b);
      case PG_COMP_INF: return __vcmpltu2(a, b);
      default: return __vcmpleu2(a, b);
    }
  }
}

// an operand of CompareImage on the device: an image, or (p == nullptr) a scalar of its type
template <typename T> struct Operand {
  const T *p;
  T v;
};

template <typename T, int N> __device__ __forceinline__ void operand_load(Chunk<T, N> &d, const Operand<T> &o,
                                                                          int64_t i) {
  if (o.p) {
    chunk_load(d, o.p + i);
  } else {
#pragma unroll
    for (int k = 0; k < N; ++k) d.v[k] = o.v;
  }
}

template <int OP, typename TI, typename TO, bool VEC>
__device__ __forceinline__ void compare_body(const TI *in, int op, const Operand<TI> &comp, const Operand<TO> &vt,
                                             const Operand<TO> &vf, TO *out, int64_t n) {
  constexpr int N = VEC ? chunk_pixels<TI, TO>() : 1;
  // sized for an image comparand and scalar true / false values (the binary-output form); image
  // true / false values add to the chunks held
  constexpr int U = VEC ? unroll_for<2 * N * (int)sizeof(TI), 2 * N * (int)(sizeof(TI) + sizeof(TO)), 128, 128>() : 1;
  const int64_t chunks = n / N, stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t c0 = t0; c0 < chunks; c0 += U * stride) {
    Chunk<TI, N> x[U], y[U];
    Chunk<TO, N> t[U], f[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t c = c0 + u * stride;
      if (c < chunks) {
        chunk_load(x[u], in + c * N);
        operand_load(y[u], comp, c * N);
        operand_load(t[u], vt, c * N);
        operand_load(f[u], vf, c * N);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t c = c0 + u * stride;
      if (c < chunks) {
        Chunk<TO, N> r;
        if constexpr (VEC && kPacked<TI> && std::is_same_v<TI, TO>) {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const uint32_t m = comp_mask<OP, TI>(op, words(x[u])[k], words(y[u])[k]);
            words(r)[k] = (words(t[u])[k] & m) | (words(f[u])[k] & ~m);
          }
        } else {
#pragma unroll
          for (int k = 0; k < N; ++k) r.v[k] = comp_op<OP>(op, x[u].v[k], y[u].v[k]) ? t[u].v[k] : f[u].v[k];
        }
        chunk_store(out + c * N, r);
      }
    }
  }
  const int64_t i = chunks * N + t0;
  if (i < n) {
    const TI y = comp.p ? comp.p[i] : comp.v;
    out[i] = comp_op<OP>(op, in[i], y) ? (vt.p ? vt.p[i] : vt.v) : (vf.p ? vf.p[i] : vf.v);
  }
}

template <typename TI, typename TO, bool VEC>
__global__ void __launch_bounds__(kPThreads)
    k_compare(const TI *in, int op, Operand<TI> comp, Operand<TO> vt, Operand<TO> vf, TO *out, int64_t n) {
  if constexpr (!VEC) {  // the unaligned fallback: one loop, the operation chosen per pixel
    compare_body<0, TI, TO, VEC>(in, op, comp, vt, vf, out, n);
    return;
  }
  switch (op) {  // one specialised loop per CompOpType (the operation is uniform over the launch)
    case PG_COMP_EQUAL: compare_body<PG_COMP_EQUAL, TI, TO, VEC>(in, op, comp, vt, vf, out, n); break;
    case PG_COMP_DIFF: compare_body<PG_COMP_DIFF, TI, TO, VEC>(in, op, comp, vt, vf, out, n); break;
    case PG_COMP_SUP: compare_body<PG_COMP_SUP, TI, TO, VEC>(in, op, comp, vt, vf, out, n); break;
    case PG_COMP_SUP_EQUAL: compare_body<PG_COMP_SUP_EQUAL, TI, TO, VEC>(in, op, comp, vt, vf, out, n); break;
    case PG_COMP_INF: compare_body<PG_COMP_INF, TI, TO, VEC>(in, op, comp, vt, vf, out, n); break;
    default: compare_body<PG_COMP_INF_EQUAL, TI, TO, VEC>(in, op, comp, vt, vf, out, n); break;
  }
}

template <typename T> Operand<T> operand_of(const void *img, const pg_scalar &v) {
  return Operand<T>{static_cast<const T *>(img), img ? T(0) : scalar_as<T>(v)};
}

}  // namespace

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

}  // namespace pg
