// recon3d.cu -- geodesic reconstruction of volumes (rank 3, SECross3D) and, through the same request,
// the 3D h-extrema, dynamic pseudo filters, leveling and binary h-maxima.
//
// Reference: t_ReconstructionViewDispatcher (geodesy/details/mreconstruct_t.hpp:84-195, 3D SEs at
// :469-474) and t_low/high_levelingHelper (geodesy/details/leveling_t.hpp:45-202, 3D at :260-340).
// The reconstruction is the least fixpoint of the geodesic dilation g -> min(dilate(g), mask) (the
// dual for erosion) from the clamped marker; for SECross3D poutre2's raster / anti-raster / FIFO
// schedule reaches it and so does iterating the geodesic dilation until nothing changes, which is
// what runs here (for SESquare3D poutre2 stops short of it, and that SE is refused):
//   prep     -- the initial value (marker clamped to the mask, or the mask shifted by h) and, for
//               leveling, the effective mask max(marker, ref) / min(marker, ref);
//   step     -- one voxel per thread: the extremum over the SE's voxels inside the volume, clamped to
//               the mask, into the other buffer; a warp vote sets a change flag;
//   epilogue -- the reconstruction itself, its clip to the leveling reference, or the binary
//               h-maxima output ref > rec.
// The host runs the steps in batches of kStepBatch between two reads of the flag; a step that
// changes nothing is a fixpoint, and after at most (voxels + 1) steps one always is.
#include "common.cuh"

namespace pg {
namespace {

constexpr int kStepBatch = 8;

template <typename T, bool SUP> __device__ __forceinline__ T shift_h(T m, T h) {
  return SUP ? sat_sub_c(m, h) : sat_add_c(m, h);  // h-maxima marker f - h, h-minima marker f + h
}

template <typename T, bool SUP>
__global__ void k_r3_prep(const T *__restrict__ ref, const T *__restrict__ marker, T *__restrict__ eff_mask,
                          T *__restrict__ cur, int64_t n, int init, int mask_mode, T h) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T a = ref[i];
    if (init == INIT_SAT_CONST) {
      cur[i] = shift_h<T, SUP>(a, h);
      continue;
    }
    const T mk = marker[i];
    T m = a;
    if (mask_mode == MASK_MAX_MARKER) m = Op<T, true>::apply(mk, a);
    else if (mask_mode == MASK_MIN_MARKER) m = Op<T, false>::apply(mk, a);
    if (eff_mask) eff_mask[i] = m;
    cur[i] = Op<T, !SUP>::apply(mk, m);  // marker clamped to the mask
  }
}

template <typename T, bool SUP>
__global__ void __launch_bounds__(256) k_r3_step(const T *__restrict__ cur, const T *__restrict__ mask,
                                                 T *__restrict__ next, int D, int H, int W, int *__restrict__ changed) {
  const int x = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int y = (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int z = (int)blockIdx.z;
  bool diff = false;
  if (x < W && y < H) {
    const int64_t c = ((int64_t)z * H + y) * W + x;
    const T v0 = cur[c];
    T v = v0;  // the SECross3D voxels inside the volume
    if (x > 0) v = Op<T, SUP>::apply(v, cur[c - 1]);
    if (x + 1 < W) v = Op<T, SUP>::apply(v, cur[c + 1]);
    if (y > 0) v = Op<T, SUP>::apply(v, cur[c - W]);
    if (y + 1 < H) v = Op<T, SUP>::apply(v, cur[c + W]);
    if (z > 0) v = Op<T, SUP>::apply(v, cur[c - (int64_t)H * W]);
    if (z + 1 < D) v = Op<T, SUP>::apply(v, cur[c + (int64_t)H * W]);
    v = Op<T, !SUP>::apply(v, mask[c]);
    next[c] = v;
    diff = !(v == v0);
  }
  if (__any_sync(0xffffffffu, diff) && (threadIdx.x & 31) == 0) atomicOr(changed, 1);
}

template <typename T, bool SUP>
__global__ void k_r3_epilogue(const T *__restrict__ rec, const T *__restrict__ ref, void *__restrict__ out, int64_t n,
                              int epi) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T r = rec[i];
    if (epi == EPI_BINARY_SUP) static_cast<uint8_t *>(out)[i] = ref[i] > r ? 255 : 0;
    else if (epi == EPI_CLIP_REF) static_cast<T *>(out)[i] = Op<T, !SUP>::apply(r, ref[i]);
    else static_cast<T *>(out)[i] = r;
  }
}

unsigned flat_grid(int64_t n) {
  int64_t b = ceil_div(n > 0 ? n : 1, 256);
  const int64_t cap = (int64_t)num_sms() * 8;
  return (unsigned)(b < cap ? b : cap);
}

template <typename T, bool SUP>
pg_status recon3d_t(const pg_image *marker, const pg_image &mask, const pg_image &out, const ReconRequest &rq,
                    cudaStream_t s) {
  const Dims d = dims_of(mask);
  const int64_t n = d.count();
  if (n == 0) return PG_OK;
  if (d.nz > 65535) return fail(PG_ERR_INVALID_ARGUMENT, "3D reconstruction: more than 65535 slices");
  if (rq.init != INIT_SAT_CONST && !marker) return fail(PG_ERR_INVALID_ARGUMENT, "3D reconstruction: null marker");
  const size_t bytes = (size_t)n * sizeof(T);
  const bool own_mask = rq.init != INIT_SAT_CONST && rq.mask_mode != MASK_PLAIN;
  Scratch bufs, emask, flag;
  PG_TRY(bufs.alloc(2 * bytes, s));
  if (own_mask) PG_TRY(emask.alloc(bytes, s));
  PG_TRY(flag.alloc(sizeof(int), s));
  T *a = static_cast<T *>(bufs.ptr), *b = a + n;
  const T *ref = static_cast<const T *>(mask.data);
  const T *eff = own_mask ? static_cast<const T *>(emask.ptr) : ref;
  int *d_flag = static_cast<int *>(flag.ptr);
  k_r3_prep<T, SUP><<<flat_grid(n), 256, 0, s>>>(ref, marker ? static_cast<const T *>(marker->data) : nullptr,
                                                 own_mask ? static_cast<T *>(emask.ptr) : nullptr, a, n, rq.init,
                                                 rq.mask_mode, scalar_as<T>(rq.h));
  PG_CUDA_TRY(cudaGetLastError(), "3D reconstruction prep launch");
  const dim3 block(32, 8), grid((unsigned)ceil_div(d.nx, 32), (unsigned)ceil_div(d.ny, 8), (unsigned)d.nz);
  const int64_t max_steps = n + kStepBatch + 1;
  int64_t steps = 0;
  for (;;) {
    PG_CUDA_TRY(cudaMemsetAsync(d_flag, 0, sizeof(int), s), "3D reconstruction flag reset");
    for (int k = 0; k < kStepBatch; ++k) {
      k_r3_step<T, SUP><<<grid, block, 0, s>>>(a, eff, b, (int)d.nz, (int)d.ny, (int)d.nx, d_flag);
      T *t = a;
      a = b;
      b = t;
    }
    PG_CUDA_TRY(cudaGetLastError(), "3D reconstruction step launch");
    steps += kStepBatch;
    int h_flag = 0;
    PG_CUDA_TRY(cudaMemcpyAsync(&h_flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, s), "3D reconstruction flag read");
    PG_CUDA_TRY(cudaStreamSynchronize(s), "3D reconstruction synchronisation");
    if (!h_flag) break;
    if (steps > max_steps) return fail(PG_ERR_NOT_CONVERGED, "3D reconstruction did not reach its fixpoint");
  }
  k_r3_epilogue<T, SUP><<<flat_grid(n), 256, 0, s>>>(a, ref, out.data, n, rq.epi);
  return cuda_status(cudaGetLastError(), "3D reconstruction epilogue launch");
}

}  // namespace

pg_status launch_reconstruction3d(const pg_image *marker, const pg_image &mask, const pg_image &out,
                                  const ReconRequest &rq, cudaStream_t s) {
  if (mask.rank != 3) return fail(PG_ERR_INVALID_ARGUMENT, "3D reconstruction of a non-3D image");
  PG_DISPATCH_PTYPE(mask.ptype, T, {
    return rq.dilate ? recon3d_t<T, true>(marker, mask, out, rq, s) : recon3d_t<T, false>(marker, mask, out, rq, s);
  });
  return PG_OK;
}

}  // namespace pg
