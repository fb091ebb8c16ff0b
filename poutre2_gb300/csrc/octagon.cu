// octagon.cu -- the octagon compound SE in one pass over HBM.
//
// Reference: t_DilateOctagon / t_ErodeOctagon (low_level_morpho/details/ero_dil_compound_static_se_t.hpp:34-64,
// :97-127): `size` successive clipped-border passes, the first size - nb_square by the 3x3 cross, the last
// nb_square by the 3x3 square.  Every pass takes the extremum over the neighbours inside the image, so the
// run equals the same passes over a tile with a halo of `size` pixels in which the pixels outside the
// image hold the neutral value (lowest for a dilation, highest for an erosion) and keep it: the centre
// pixel is always inside, so the neutral value never wins.
//
// One CTA per 64 x 64 output tile: the tile and its halo are read once into shared memory, the passes
// ping-pong between two shared buffers (pass k updates rows / columns [k, RW - k) of the RW x RW
// region, exactly the positions whose 3x3 neighbourhood the previous pass left valid), and the centre
// is written once.  HBM traffic: the tile plus halo read ((64 + 2 size)^2 / 64^2 of the image) and the
// image written; shared-memory work: about size x 5 (cross) or 9 (square) reads per pixel.
#include "common.cuh"

namespace pg {
namespace {

constexpr int kOT = 64;                 // output tile edge
constexpr int kOTx = 64, kOTy = 4;      // threads: 64 along x, 4 along y
constexpr int kOctMaxSize = 16;         // halo limit of the fused kernel (larger sizes take the passes)

template <bool DIL, typename T> __device__ __forceinline__ T ext(T a, T b) {
  if constexpr (DIL) return a > b ? a : b;
  else return a < b ? a : b;
}

template <typename T, bool DIL>
__global__ void __launch_bounds__(kOTx * kOTy) k_octagon(const T *__restrict__ in, T *__restrict__ out, int H, int W,
                                                         int n_cross, int n_square) {
  extern __shared__ __align__(16) unsigned char oct_smem[];
  const int M = n_cross + n_square;
  const int RW = kOT + 2 * M;  // region edge
  T *A = reinterpret_cast<T *>(oct_smem);
  T *B = A + RW * RW;
  const int y0 = (int)blockIdx.y * kOT - M, x0 = (int)blockIdx.x * kOT - M;  // region origin in the image
  const T neutral = DIL ? Lim<T>::lo() : Lim<T>::hi();

  for (int r = threadIdx.y; r < RW; r += kOTy) {
    const int gy = y0 + r;
    const bool row_in = gy >= 0 && gy < H;
    for (int c = threadIdx.x; c < RW; c += kOTx) {
      const int gx = x0 + c;
      A[r * RW + c] = (row_in && gx >= 0 && gx < W) ? in[(size_t)gy * W + gx] : neutral;
    }
  }
  __syncthreads();

  for (int k = 1; k <= M; ++k) {
    const bool cross = k <= n_cross;
    for (int r = k + threadIdx.y; r < RW - k; r += kOTy) {
      const int gy = y0 + r;
      const bool row_in = gy >= 0 && gy < H;
      for (int c = k + threadIdx.x; c < RW - k; c += kOTx) {
        const int gx = x0 + c;
        const T *p = A + r * RW + c;
        T v = neutral;
        if (row_in && gx >= 0 && gx < W) {
          v = ext<DIL>(ext<DIL>(p[0], ext<DIL>(p[-1], p[1])), ext<DIL>(p[-RW], p[RW]));
          if (!cross) v = ext<DIL>(v, ext<DIL>(ext<DIL>(p[-RW - 1], p[-RW + 1]), ext<DIL>(p[RW - 1], p[RW + 1])));
        }
        B[r * RW + c] = v;
      }
    }
    __syncthreads();
    T *t = A;
    A = B;
    B = t;
  }

  for (int r = threadIdx.y; r < kOT; r += kOTy) {
    const int gy = (int)blockIdx.y * kOT + r;
    if (gy >= H) break;
    for (int c = threadIdx.x; c < kOT; c += kOTx) {
      const int gx = (int)blockIdx.x * kOT + c;
      if (gx < W) out[(size_t)gy * W + gx] = A[(r + M) * RW + (c + M)];
    }
  }
}

template <typename T> size_t octagon_smem(int size) {
  const size_t rw = (size_t)(kOT + 2 * size);
  return 2 * rw * rw * sizeof(T);
}

template <typename T, bool DIL>
pg_status octagon_t(const pg_image &in, const pg_image &out, int n_cross, int n_square, cudaStream_t s) {
  const int H = (int)in.shape[0], W = (int)in.shape[1];
  const size_t smem = octagon_smem<T>(n_cross + n_square);
  static int configured_dev = -1;  // the attribute is per device
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev), "octagon: device");
  if (configured_dev != dev) {
    PG_CUDA_TRY(cudaFuncSetAttribute(k_octagon<T, DIL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)octagon_smem<T>(kOctMaxSize)),
                "octagon: shared memory attribute");
    configured_dev = dev;
  }
  const dim3 grid((unsigned)ceil_div(W, kOT), (unsigned)ceil_div(H, kOT));
  k_octagon<T, DIL><<<grid, dim3(kOTx, kOTy), smem, s>>>(static_cast<const T *>(in.data), static_cast<T *>(out.data),
                                                         H, W, n_cross, n_square);
  return cuda_status(cudaGetLastError(), "octagon kernel launch");
}

}  // namespace

bool octagon_fused_ok(const pg_image &in, int size) {
  return in.rank == 2 && size >= 2 && size <= kOctMaxSize && in.shape[0] > 0 && in.shape[1] > 0 &&
         in.shape[0] < (1 << 30) && in.shape[1] < (1 << 30) &&
         (size_t)elem_size(in.ptype) * 2 * (kOT + 2 * kOctMaxSize) * (kOT + 2 * kOctMaxSize) <= 227 * 1024;
}

pg_status launch_octagon_fused(const pg_image &in, const pg_image &out, int n_cross, int n_square, bool dilate,
                               cudaStream_t s) {
  PG_DISPATCH_PTYPE(in.ptype, T, {
    return dilate ? octagon_t<T, true>(in, out, n_cross, n_square, s) : octagon_t<T, false>(in, out, n_cross, n_square, s);
  });
  return PG_OK;
}

}  // namespace pg
