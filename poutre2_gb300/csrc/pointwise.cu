// pointwise.cu -- the pixel_processing subset the geodesy chains need, plus copy and the
// plain difference of the morphological gradient.
//
// Reference: op_Saturated_Sub_Constant / op_Saturated_Add_Constant / op_Saturated_Sub
// (pixel_processing/details/arith_op_t.hpp:84-345) and the CompareImage marker steps of
// dynamic_pseudo_opening/closing (src/geodesy/extrema.cpp:75-114).  Grid-stride
// elementwise kernels: HBM-bound, one read (or two) and one write per pixel.
#include <cmath>

#include "common.cuh"

namespace pg {

static unsigned grid_for(int64_t n, int threads = 256) {
  int64_t b = ceil_div(n, threads);
  const int64_t cap = (int64_t)num_sms() * 32;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

template <typename T>
__global__ void k_sat_const(const T *__restrict__ in, T *__restrict__ out, int64_t n, T v, bool add) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T a = ldg(in + i);
    out[i] = add ? sat_add_c(a, v) : sat_sub_c(a, v);
  }
}

template <typename T>
__global__ void k_sat_sub_image(const T *__restrict__ a, const T *__restrict__ b, T *__restrict__ out, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = sat_sub_c(ldg(a + i), ldg(b + i));
}

template <typename T>
__global__ void k_sub(const T *__restrict__ a, const T *__restrict__ b, T *__restrict__ out, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (T)(ldg(a + i) - ldg(b + i));
}

// Marker of the second reconstruction of dynamic_pseudo_opening (closing: dual), fused from
// the two CompareImage calls of src/geodesy/extrema.cpp:86-90 (:106-110):
//   tmp  = sat_sub(f, h)                               (sat_add for closing)
//   mask = (ext == tmp) ? f : lowest                   (highest)
//   out  = (ext != lowest) ? mask : lowest             (highest)
template <typename T>
__global__ void k_dyn_marker(const T *__restrict__ f, const T *__restrict__ ext, T *__restrict__ out, int64_t n, T h,
                             bool opening) {
  const T ext_v = opening ? Lim<T>::lo() : Lim<T>::hi();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T fv = ldg(f + i), e = ldg(ext + i);
    const T tmp = opening ? sat_sub_c(fv, h) : sat_add_c(fv, h);
    const T m = (e == tmp) ? fv : ext_v;
    out[i] = (e != ext_v) ? m : ext_v;
  }
}

pg_status launch_copy(const pg_image &in, const pg_image &out, cudaStream_t s) {
  const size_t bytes = (size_t)dims_of(in).count() * elem_size(in.ptype);
  if (bytes == 0) return PG_OK;
  PG_CUDA_TRY(cudaMemcpyAsync(out.data, in.data, bytes, cudaMemcpyDeviceToDevice, s), "device copy");
  return PG_OK;
}

pg_status launch_sub(const pg_image &a, const pg_image &b, const pg_image &out, cudaStream_t s) {
  const int64_t n = dims_of(a).count();
  if (n == 0) return PG_OK;
  PG_DISPATCH_PTYPE(a.ptype, T, {
    k_sub<T><<<grid_for(n), 256, 0, s>>>(static_cast<const T *>(a.data), static_cast<const T *>(b.data),
                                        static_cast<T *>(out.data), n);
  });
  return cuda_status(cudaGetLastError(), "difference kernel launch");
}

pg_status launch_sat_const(const pg_image &in, const pg_scalar &v, bool add, const pg_image &out, cudaStream_t s) {
  const int64_t n = dims_of(in).count();
  if (n == 0) return PG_OK;
  PG_DISPATCH_PTYPE(in.ptype, T, {
    k_sat_const<T><<<grid_for(n), 256, 0, s>>>(static_cast<const T *>(in.data), static_cast<T *>(out.data), n,
                                              scalar_as<T>(v), add);
  });
  return cuda_status(cudaGetLastError(), "saturated constant kernel launch");
}

pg_status launch_sat_sub_image(const pg_image &a, const pg_image &b, const pg_image &out, cudaStream_t s) {
  const int64_t n = dims_of(a).count();
  if (n == 0) return PG_OK;
  PG_DISPATCH_PTYPE(a.ptype, T, {
    k_sat_sub_image<T><<<grid_for(n), 256, 0, s>>>(static_cast<const T *>(a.data), static_cast<const T *>(b.data),
                                                  static_cast<T *>(out.data), n);
  });
  return cuda_status(cudaGetLastError(), "saturated difference kernel launch");
}

pg_status launch_dyn_pseudo_marker(const pg_image &f, const pg_image &ext, const pg_scalar &h, bool opening,
                                   const pg_image &out, cudaStream_t s) {
  const int64_t n = dims_of(f).count();
  if (n == 0) return PG_OK;
  PG_DISPATCH_PTYPE(f.ptype, T, {
    k_dyn_marker<T><<<grid_for(n), 256, 0, s>>>(static_cast<const T *>(f.data), static_cast<const T *>(ext.data),
                                               static_cast<T *>(out.data), n, scalar_as<T>(h), opening);
  });
  return cuda_status(cudaGetLastError(), "pseudo-dynamic marker kernel launch");
}

}  // namespace pg
