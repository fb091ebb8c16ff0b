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
//   brick    -- a CTA loads a brick of 32 x 8 x 8 voxels of the current value (plus a one-voxel halo)
//               and of the mask into shared memory and repeats the geodesic step on the brick, the
//               halo held fixed, until the brick stops changing (or an iteration cap); it writes the
//               brick to the other buffer and sets a change flag when any voxel differs from its
//               input.  Every update is a geodesic step from a lower bound of the fixpoint (monotone
//               and below it), so the order is immaterial; a launch that changes nothing is the
//               fixpoint.  One launch carries values across a whole brick, where a plain step moves
//               them one voxel;
//   epilogue -- the reconstruction itself, its clip to the leveling reference, or the binary
//               h-maxima output ref > rec.
// The host runs the launches in batches of kStepBatch between two reads of the flag; a launch that
// changes nothing is a fixpoint, and after at most (voxels + 1) launches one always is (each launch
// does at least one geodesic step everywhere).
#include "common.cuh"

namespace pg {
namespace {

constexpr int kStepBatch = 2;
constexpr int kBX = 32, kBY = 8, kBZ = 8;  // brick
constexpr int kBrickIters = 2 * (kBX + kBY + kBZ);  // local iteration cap per launch

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
__global__ void __launch_bounds__(kBX * kBY) k_r3_brick(const T *__restrict__ cur, const T *__restrict__ mask,
                                                        T *__restrict__ next, int D, int H, int W,
                                                        int *__restrict__ changed) {
  constexpr int HX = kBX + 2, HY = kBY + 2, HZ = kBZ + 2;
  __shared__ T sr[HZ][HY][HX];      // current value with a one-voxel halo
  __shared__ T sk[kBZ][kBY][kBX];   // mask of the brick
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kBX + tx;
  const int x0 = blockIdx.x * kBX, y0 = blockIdx.y * kBY, z0 = blockIdx.z * kBZ;
  const int64_t plane = (int64_t)H * W;
  const T NEU = Op<T, SUP>::neutral();  // never wins the extremum: voxels outside the volume
  for (int i = tid; i < HX * HY * HZ; i += kBX * kBY) {
    const int hx = i % HX, hy = (i / HX) % HY, hz = i / (HX * HY);
    const int x = x0 - 1 + hx, y = y0 - 1 + hy, z = z0 - 1 + hz;
    sr[hz][hy][hx] = (x >= 0 && x < W && y >= 0 && y < H && z >= 0 && z < D) ? cur[z * plane + (int64_t)y * W + x] : NEU;
  }
  const int x = x0 + tx, y = y0 + ty;
  const bool xy_in = x < W && y < H;
#pragma unroll
  for (int k = 0; k < kBZ; ++k) {
    const int z = z0 + k;
    sk[k][ty][tx] = (xy_in && z < D) ? mask[z * plane + (int64_t)y * W + x] : NEU;
  }
  __syncthreads();
  T start[kBZ];
#pragma unroll
  for (int k = 0; k < kBZ; ++k) start[k] = sr[k + 1][ty + 1][tx + 1];
  // this thread's z column, updated in place (values only move towards the fixpoint, so reading a
  // neighbour's old or new value are both valid steps)
  for (int it = 0; it < kBrickIters; ++it) {
    bool ch = false;
    if (xy_in) {
#pragma unroll
      for (int k = 0; k < kBZ; ++k) {
        if (z0 + k >= D) break;
        volatile T *c = &sr[k + 1][ty + 1][tx + 1];
        const T v = *c;
        T n = Op<T, SUP>::apply(v, sr[k + 1][ty + 1][tx]);
        n = Op<T, SUP>::apply(n, sr[k + 1][ty + 1][tx + 2]);
        n = Op<T, SUP>::apply(n, sr[k + 1][ty][tx + 1]);
        n = Op<T, SUP>::apply(n, sr[k + 1][ty + 2][tx + 1]);
        n = Op<T, SUP>::apply(n, sr[k][ty + 1][tx + 1]);
        n = Op<T, SUP>::apply(n, sr[k + 2][ty + 1][tx + 1]);
        n = Op<T, !SUP>::apply(n, sk[k][ty][tx]);
        if (!(n == v)) {
          *c = n;
          ch = true;
        }
      }
    }
    if (!__syncthreads_or(ch)) break;
  }
  bool diff = false;
  if (xy_in) {
#pragma unroll
    for (int k = 0; k < kBZ; ++k) {
      const int z = z0 + k;
      if (z >= D) break;
      const T v = sr[k + 1][ty + 1][tx + 1];
      next[z * plane + (int64_t)y * W + x] = v;
      diff |= !(v == start[k]);
    }
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
  if (d.nx > INT32_MAX || d.ny > INT32_MAX || d.nz > INT32_MAX || ceil_div(d.ny, kBY) > 65535 || ceil_div(d.nz, kBZ) > 65535)
    return fail(PG_ERR_INVALID_ARGUMENT, "3D reconstruction: volume too large (ny <= 524280, nz <= 524280)");
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
  const dim3 block(kBX, kBY), grid((unsigned)ceil_div(d.nx, kBX), (unsigned)ceil_div(d.ny, kBY), (unsigned)ceil_div(d.nz, kBZ));
  const int64_t max_steps = n + kStepBatch + 1;
  int64_t steps = 0;
  for (;;) {
    PG_CUDA_TRY(cudaMemsetAsync(d_flag, 0, sizeof(int), s), "3D reconstruction flag reset");
    for (int k = 0; k < kStepBatch; ++k) {
      k_r3_brick<T, SUP><<<grid, block, 0, s>>>(a, eff, b, (int)d.nz, (int)d.ny, (int)d.nx, d_flag);
      T *t = a;
      a = b;
      b = t;
    }
    PG_CUDA_TRY(cudaGetLastError(), "3D reconstruction brick launch");
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
