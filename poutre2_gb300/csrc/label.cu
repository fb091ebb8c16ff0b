// label.cu -- connected-component labelling: poutre::label::label_binary and label_flat_zones
// (src/label/label_binary.cpp, src/label/label_flat_zones.cpp; algorithm in
// include/poutre/label/details/label_t.hpp:132-247).
//
// The reference scans in raster order: an accepted pixel joins the provisional labels of its
// related upper-half neighbours (disjoint sets, the smaller root wins) or opens a new one; the
// roots are then numbered 1.. in creation order and every accepted pixel takes its root's number.
// A component's root is the provisional label of its first pixel in raster order (that pixel has no
// related earlier neighbour), so the result is: components numbered by the raster position of their
// first pixel.  The GPU builds the same components with a concurrent union-find over pixel indices
// (parent[] only ever points to a smaller index; a root hangs under the smaller root by
// compare-and-swap), so each component's root is its first pixel; a block-wise count and an
// exclusive scan of the roots number them in raster order.
//
// Edges are the reference's: pixel p and its upper-half neighbour q (earlier in raster order) of the
// SE are joined when p is accepted and q is related -- binary: p != 0 and q > 0 (a negative pixel is
// accepted but joins no later pixel), flat zones: p == q.  Binary labelling of float images is not
// on this path (the reference's background test |v| > 1e-10 and its neighbour test v > 0 disagree on
// (0, 1e-10], where it reads an unset label), nor is SESquare3D (its upper half in the reference is
// not the raster-earlier half).
//
// Every find / union loop is bounded (kLabelIters); exceeding it records PG_ERR_CUDA in
// g_label_status, read by pg_check_device.
#include <algorithm>
#include <array>
#include <initializer_list>

#include "common.cuh"

namespace pg {

__device__ int g_label_status = 0;

namespace {

constexpr int kLabelIters = 1 << 24;
constexpr int kLThreads = 256, kLItems = 4;  // pixels per block in the numbering passes: 1024

struct UpperOffsets {
  int n;
  int dz[4], dy[4], dx[4];
};

__device__ __forceinline__ int32_t find_root(int32_t *par, int32_t x) {
  for (int it = 0; it < kLabelIters; ++it) {
    const int32_t p = __ldcg(par + x);
    if (p == x) return x;
    if (p < 0) break;  // a background pixel: never reached (only foreground pixels are joined)
    x = p;
  }
  atomicCAS(&g_label_status, 0, (int)PG_ERR_CUDA);
  return x;
}

__device__ __forceinline__ void unite(int32_t *par, int32_t a, int32_t b) {
  for (int it = 0; it < kLabelIters; ++it) {
    a = find_root(par, a);
    b = find_root(par, b);
    if (a == b) return;
    if (a < b) { const int32_t t = a; a = b; b = t; }  // hang the larger root under the smaller
    const int32_t old = atomicCAS(par + a, a, b);
    if (old == a) return;
    a = old;
  }
  atomicCAS(&g_label_status, 0, (int)PG_ERR_CUDA);
}

template <typename T, bool FLAT> __device__ __forceinline__ bool accepted(T v) { return FLAT || v != T(0); }

template <typename T, bool FLAT>
__global__ void k_label_init(const T *__restrict__ in, int32_t *__restrict__ par, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    par[i] = accepted<T, FLAT>(in[i]) ? (int32_t)i : -1;
}

template <typename T, bool FLAT>
__global__ void k_label_merge(const T *__restrict__ in, int32_t *par, int64_t nz, int64_t ny, int64_t nx,
                              UpperOffsets up) {
  const int64_t n = nz * ny * nx;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T v = in[i];
    if (!accepted<T, FLAT>(v)) continue;
    const int64_t x = i % nx, y = (i / nx) % ny, z = i / (nx * ny);
    for (int k = 0; k < up.n; ++k) {
      const int64_t zz = z + up.dz[k], yy = y + up.dy[k], xx = x + up.dx[k];
      if (zz < 0 || yy < 0 || xx < 0 || zz >= nz || yy >= ny || xx >= nx) continue;
      const int64_t j = (zz * ny + yy) * nx + xx;
      const T w = in[j];
      if (FLAT ? (w == v) : (w > T(0))) unite(par, (int32_t)i, (int32_t)j);
    }
  }
}

__global__ void k_label_compress(int32_t *par, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (par[i] >= 0) par[i] = find_root(par, (int32_t)i);
}

// roots of each 1024-pixel block
__global__ void k_label_count(const int32_t *__restrict__ par, int64_t n, int32_t *__restrict__ bsum) {
  __shared__ int32_t s_w[kLThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kLThreads * kLItems;
  int c = 0;
#pragma unroll
  for (int k = 0; k < kLItems; ++k) {
    const int64_t i = base + (int64_t)k * kLThreads + threadIdx.x;
    if (i < n && par[i] == (int32_t)i) ++c;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < kLThreads / 32; ++w) t += s_w[w];
    bsum[blockIdx.x] = t;
  }
}

// exclusive scan of the block counts in place (one CTA), total into *total
__global__ void k_label_scan(int32_t *bsum, int64_t nb, int64_t *total) {
  __shared__ int32_t s_w[32];
  __shared__ int64_t s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t c0 = 0; c0 < nb; c0 += blockDim.x) {
    const int64_t i = c0 + threadIdx.x;
    const int32_t v = i < nb ? bsum[i] : 0;
    int32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      const int nw = blockDim.x / 32;
      int32_t w = lane < nw ? s_w[lane] : 0, wi = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int32_t t = __shfl_up_sync(0xffffffffu, wi, o);
        if (lane >= o) wi += t;
      }
      if (lane < nw) s_w[lane] = wi - w;  // exclusive prefix of the warps
    }
    __syncthreads();
    const int64_t carry = s_carry;
    if (i < nb) bsum[i] = (int32_t)(carry + s_w[warp] + incl - v);
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) s_carry = carry + s_w[warp] + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = s_carry;
}

// number the roots: label = roots before it + 1, written at the root's own pixel
__global__ void k_label_roots(const int32_t *__restrict__ par, int64_t n, const int32_t *__restrict__ boff,
                              int64_t *__restrict__ out) {
  __shared__ int32_t s_w[kLThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kLThreads * kLItems;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t run = boff[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kLItems; ++k) {
    const int64_t i = base + (int64_t)k * kLThreads + threadIdx.x;
    const int f = (i < n && par[i] == (int32_t)i) ? 1 : 0;
    int32_t incl = f;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    int32_t before = 0, all = 0;
    for (int w = 0; w < kLThreads / 32; ++w) {
      if (w < warp) before += s_w[w];
      all += s_w[w];
    }
    if (f) out[i] = (int64_t)run + before + incl;  // 1-based
    run += all;
    __syncthreads();
  }
}

__global__ void k_label_final(const int32_t *__restrict__ par, int64_t n, int64_t *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t r = par[i];
    if (r < 0) out[i] = 0;
    else if (r != (int32_t)i) out[i] = out[r];
  }
}

// upper raster half of the SE, (dz, dy, dx) over (nz, ny, nx)
bool upper_offsets(int se, UpperOffsets *u) {
  auto set = [&](std::initializer_list<std::array<int, 3>> l) {
    u->n = 0;
    for (const auto &o : l) {
      u->dz[u->n] = o[0]; u->dy[u->n] = o[1]; u->dx[u->n] = o[2];
      ++u->n;
    }
    return true;
  };
  switch (se) {
    case PG_SE_SEGMENT_X_1D: case PG_SE_SEGMENT_X_2D: case PG_SE_SEGMENT_X_3D: return set({{0, 0, -1}});
    case PG_SE_SEGMENT_Y_2D: case PG_SE_SEGMENT_Y_3D: return set({{0, -1, 0}});
    case PG_SE_SEGMENT_Z_3D: return set({{-1, 0, 0}});
    case PG_SE_SQUARE_2D: return set({{0, -1, -1}, {0, -1, 0}, {0, -1, 1}, {0, 0, -1}});
    case PG_SE_CROSS_2D: return set({{0, -1, 0}, {0, 0, -1}});
    case PG_SE_CROSS_3D: return set({{0, 0, -1}, {0, -1, 0}, {-1, 0, 0}});
    default: return false;
  }
}

template <typename T, bool FLAT>
pg_status label_t(const pg_image &in, const pg_image &out, const UpperOffsets &up, int64_t *count, cudaStream_t s) {
  const Dims d = dims_of(in);
  const int64_t n = d.count();
  const int64_t nb = ceil_div(n, (int64_t)kLThreads * kLItems);
  Scratch par, bs, tot;
  PG_TRY(par.alloc(sizeof(int32_t) * (size_t)n, s));
  PG_TRY(bs.alloc(sizeof(int32_t) * (size_t)nb, s));
  PG_TRY(tot.alloc(sizeof(int64_t), s));
  const int64_t cap = (int64_t)num_sms() * 8;
  const unsigned g = (unsigned)std::min<int64_t>(ceil_div(n, kLThreads), cap);
  int32_t *p = par.as<int32_t>();
  int64_t *o = static_cast<int64_t *>(out.data);
  k_label_init<T, FLAT><<<g, kLThreads, 0, s>>>(static_cast<const T *>(in.data), p, n);
  k_label_merge<T, FLAT><<<g, kLThreads, 0, s>>>(static_cast<const T *>(in.data), p, d.nz, d.ny, d.nx, up);
  k_label_compress<<<g, kLThreads, 0, s>>>(p, n);
  k_label_count<<<(unsigned)nb, kLThreads, 0, s>>>(p, n, bs.as<int32_t>());
  k_label_scan<<<1, 1024, 0, s>>>(bs.as<int32_t>(), nb, tot.as<int64_t>());
  k_label_roots<<<(unsigned)nb, kLThreads, 0, s>>>(p, n, bs.as<int32_t>(), o);
  k_label_final<<<g, kLThreads, 0, s>>>(p, n, o);
  PG_TRY(cuda_status(cudaGetLastError(), "labelling kernels launch"));
  if (count) {
    PG_CUDA_TRY(cudaMemcpyAsync(count, tot.ptr, sizeof(int64_t), cudaMemcpyDeviceToHost, s), "label count copy");
    PG_CUDA_TRY(cudaStreamSynchronize(s), "label count synchronisation");
  }
  return PG_OK;
}

}  // namespace

pg_status launch_label(const pg_image &in, int se, const pg_image &out, bool flat, int64_t *count, cudaStream_t s) {
  UpperOffsets up;
  if (!upper_offsets(se, &up))
    return fail(PG_ERR_UNSUPPORTED_SE, flat ? "t_label_flat_zonesDispatch unsupported nl_static on the GPU path"
                                            : "t_label_binaryDispatch unsupported nl_static on the GPU path");
  const Dims d = dims_of(in);
  const int64_t n = d.count();
  if (n > (int64_t)INT32_MAX) return fail(PG_ERR_INVALID_ARGUMENT, "labelling: image larger than 2^31 - 1 pixels");
  if (n == 0) {
    if (count) *count = 0;
    return PG_OK;
  }
  if (!flat && (in.ptype == PG_PTYPE_F32 || in.ptype == PG_PTYPE_F64))
    return fail(PG_ERR_UNSUPPORTED_PTYPE, "label_binary of a float image is not on the GPU path");
  PG_DISPATCH_PTYPE(in.ptype, T, {
    return flat ? label_t<T, true>(in, out, up, count, s) : label_t<T, false>(in, out, up, count, s);
  });
  return PG_OK;
}

int take_label_status() {
  int st = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&st, g_label_status, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  if (st != 0 && cudaMemcpyToSymbol(g_label_status, &zero, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  return st;
}

}  // namespace pg
