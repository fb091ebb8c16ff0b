// adjoint.cu -- flat dilation / erosion of float32 planes by a (2ry+1) x (2rx+1) rectangle and
// its adjoint, for the differentiable morphology (no counterpart in the reference; the
// forward equals poutre::Dilate/Erode by that rectangle, e.g. SESquare2D iterated twice for
// 5x5).
//
// Adjoint: each output p routes its upstream gradient to the FIRST position, in scan order
// of the window (dy-major, then dx, clipped to the image), holding the window's max (min).
// The backward pass recomputes that arg index instead of storing it, and is a gather:
// grad_in[q] = sum over the outputs p of q's window, in raster order of p, of grad_out[p]
// when arg(p) == q -- no atomics, so the result is deterministic and equals a sequential
// accumulation in raster order.
//
// GPU design: a CTA owns a 32x64 tile of one plane.  It stages x over the tile plus a 2r
// halo, computes per row of the halo region the first-best value and column (separable
// arg-extremum: the first row, in dy order, whose row-best is strictly best, then that
// row's first column), stores the arg of every output that can reach the tile as one byte,
// stages grad_out, and gathers.  Forward uses the same separable scheme without args.
#include <cmath>
#include <atomic>

#include "common.cuh"

namespace pg {

static constexpr int AT_H = 32, AT_W = 64, AT_THREADS = 256, AR_MAX = 7;

template <bool SUP> __device__ __forceinline__ bool better(float v, float best) { return SUP ? (v > best) : (v < best); }
template <bool SUP> __device__ __forceinline__ float outside() { return SUP ? -INFINITY : INFINITY; }

template <bool SUP>
__global__ void __launch_bounds__(AT_THREADS) k_flat_fwd(const float *__restrict__ x, float *__restrict__ y,
                                                         int64_t planes, int H, int W, int ry, int rx) {
  extern __shared__ __align__(16) float smf[];
  const int XH = AT_H + 2 * ry, XW = AT_W + 2 * rx;
  float *X = smf;              // XH x XW
  float *RV = X + XH * XW;     // XH x AT_W row-best values
  const int ty0 = blockIdx.y * AT_H, tx0 = blockIdx.x * AT_W;
  for (int64_t pl = blockIdx.z; pl < planes; pl += gridDim.z) {
    const float *xp = x + pl * (int64_t)H * W;
    for (int i = threadIdx.x; i < XH * XW; i += AT_THREADS) {
      const int r = i / XW, c = i - r * XW;
      const int gy = ty0 - ry + r, gx = tx0 - rx + c;
      X[i] = (gy >= 0 && gy < H && gx >= 0 && gx < W) ? __ldg(xp + (int64_t)gy * W + gx) : outside<SUP>();
    }
    __syncthreads();
    for (int i = threadIdx.x; i < XH * AT_W; i += AT_THREADS) {
      const int r = i / AT_W, c = i - r * AT_W;
      const float *row = X + r * XW + c;
      float b = row[0];
      for (int d = 1; d <= 2 * rx; ++d) if (better<SUP>(row[d], b)) b = row[d];
      RV[i] = b;
    }
    __syncthreads();
    float *yp = y + pl * (int64_t)H * W;
    for (int i = threadIdx.x; i < AT_H * AT_W; i += AT_THREADS) {
      const int r = i / AT_W, c = i - r * AT_W;
      const int gy = ty0 + r, gx = tx0 + c;
      if (gy >= H || gx >= W) continue;
      float b = RV[r * AT_W + c];
      for (int d = 1; d <= 2 * ry; ++d) {
        const float v = RV[(r + d) * AT_W + c];
        if (better<SUP>(v, b)) b = v;
      }
      yp[(int64_t)gy * W + gx] = b;
    }
    __syncthreads();
  }
}

template <bool SUP>
__global__ void __launch_bounds__(AT_THREADS) k_flat_bwd(const float *__restrict__ x, const float *__restrict__ gy,
                                                         float *__restrict__ gx, int64_t planes, int H, int W, int ry,
                                                         int rx) {
  extern __shared__ __align__(16) float smf[];
  const int XH = AT_H + 4 * ry, XW = AT_W + 4 * rx;  // x staged over the tile + 2r
  const int PH = AT_H + 2 * ry, PW = AT_W + 2 * rx;  // outputs that can route into the tile
  float *X = smf;                                     // XH x XW
  float *RV = X + XH * XW;                            // XH x PW row-best values
  float *G = RV + XH * PW;                            // PH x PW upstream gradient
  unsigned char *RA = reinterpret_cast<unsigned char *>(G + PH * PW);  // XH x PW row-best column
  unsigned char *CODE = RA + XH * PW;                                  // PH x PW arg code
  const int ty0 = blockIdx.y * AT_H, tx0 = blockIdx.x * AT_W;
  const int wx = 2 * rx + 1;
  for (int64_t pl = blockIdx.z; pl < planes; pl += gridDim.z) {
    const float *xp = x + pl * (int64_t)H * W;
    const float *gp = gy + pl * (int64_t)H * W;
    for (int i = threadIdx.x; i < XH * XW; i += AT_THREADS) {
      const int r = i / XW, c = i - r * XW;
      const int yy = ty0 - 2 * ry + r, xx = tx0 - 2 * rx + c;
      X[i] = (yy >= 0 && yy < H && xx >= 0 && xx < W) ? __ldg(xp + (int64_t)yy * W + xx) : outside<SUP>();
    }
    for (int i = threadIdx.x; i < PH * PW; i += AT_THREADS) {
      const int r = i / PW, c = i - r * PW;
      const int yy = ty0 - ry + r, xx = tx0 - rx + c;
      G[i] = (yy >= 0 && yy < H && xx >= 0 && xx < W) ? __ldg(gp + (int64_t)yy * W + xx) : 0.f;
    }
    __syncthreads();
    // row pass: first strictly-best column of each row segment
    for (int i = threadIdx.x; i < XH * PW; i += AT_THREADS) {
      const int r = i / PW, c = i - r * PW;
      const float *row = X + r * XW + c;
      float b = row[0];
      int a = 0;
      for (int d = 1; d <= 2 * rx; ++d)
        if (better<SUP>(row[d], b)) { b = row[d]; a = d; }
      RV[i] = b;
      RA[i] = (unsigned char)a;
    }
    __syncthreads();
    // column pass: first strictly-best row, then that row's column -> window code
    for (int i = threadIdx.x; i < PH * PW; i += AT_THREADS) {
      const int r = i / PW, c = i - r * PW;
      const int yy = ty0 - ry + r, xx = tx0 - rx + c;
      unsigned char code = 255;
      if (yy >= 0 && yy < H && xx >= 0 && xx < W) {
        float b = RV[r * PW + c];
        int a = 0;
        for (int d = 1; d <= 2 * ry; ++d) {
          const float v = RV[(r + d) * PW + c];
          if (better<SUP>(v, b)) { b = v; a = d; }
        }
        code = (unsigned char)(a * wx + RA[(r + a) * PW + c]);
      }
      CODE[i] = code;
    }
    __syncthreads();
    // gather in raster order of the routing outputs
    float *op = gx + pl * (int64_t)H * W;
    for (int i = threadIdx.x; i < AT_H * AT_W; i += AT_THREADS) {
      const int r = i / AT_W, c = i - r * AT_W;
      const int yy = ty0 + r, xx = tx0 + c;
      if (yy >= H || xx >= W) continue;
      float sum = 0.f;
      for (int a = -ry; a <= ry; ++a) {
        const int pr = r + ry + a;  // routing output row in the P region
        for (int b = -rx; b <= rx; ++b) {
          const int pc = c + rx + b;
          // arg(p) == q  <=>  the window offset of q seen from p is (-a, -b)
          const unsigned char want = (unsigned char)((ry - a) * wx + (rx - b));
          if (CODE[pr * PW + pc] == want) sum += G[pr * PW + pc];
        }
      }
      op[(int64_t)yy * W + xx] = sum;
    }
    __syncthreads();
  }
}

static size_t fwd_smem(int ry, int rx) {
  const int XH = AT_H + 2 * ry, XW = AT_W + 2 * rx;
  return sizeof(float) * ((size_t)XH * XW + (size_t)XH * AT_W);
}
static size_t bwd_smem(int ry, int rx) {
  const int XH = AT_H + 4 * ry, XW = AT_W + 4 * rx, PH = AT_H + 2 * ry, PW = AT_W + 2 * rx;
  return sizeof(float) * ((size_t)XH * XW + (size_t)XH * PW + (size_t)PH * PW) + (size_t)XH * PW + (size_t)PH * PW;
}

template <typename K>
static pg_status ensure_smem(K kern, std::atomic<uint64_t> &flag) {
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  const uint64_t bit = 1ull << (dev & 63);
  if (!(flag.load() & bit)) {
    PG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024), "smem attribute");
    flag.fetch_or(bit);
  }
  return PG_OK;
}

static dim3 flat_grid(int64_t planes, int64_t H, int64_t W) {
  int64_t z = planes < 65535 ? planes : 65535;
  return dim3((unsigned)ceil_div(W, AT_W), (unsigned)ceil_div(H, AT_H), (unsigned)(z > 0 ? z : 1));
}

pg_status launch_flat2d(const float *x, float *y, int64_t planes, int64_t h, int64_t w, int ry, int rx, bool dilate,
                        cudaStream_t s) {
  if (ry < 0 || rx < 0 || ry > AR_MAX || rx > AR_MAX) return fail(PG_ERR_INVALID_ARGUMENT, "half sizes must be in [0, 7]");
  if (planes * h * w == 0) return PG_OK;
  if (h > (1 << 30) || w > (1 << 30) || ceil_div(h, AT_H) > 65535) return fail(PG_ERR_INVALID_ARGUMENT, "plane too large");
  static std::atomic<uint64_t> fs{0}, fe{0};
  const size_t sm = fwd_smem(ry, rx);
  if (dilate) {
    PG_TRY(ensure_smem(k_flat_fwd<true>, fs));
    k_flat_fwd<true><<<flat_grid(planes, h, w), AT_THREADS, sm, s>>>(x, y, planes, (int)h, (int)w, ry, rx);
  } else {
    PG_TRY(ensure_smem(k_flat_fwd<false>, fe));
    k_flat_fwd<false><<<flat_grid(planes, h, w), AT_THREADS, sm, s>>>(x, y, planes, (int)h, (int)w, ry, rx);
  }
  return cuda_status(cudaGetLastError(), "flat morphology forward launch");
}

pg_status launch_flat2d_backward(const float *x, const float *gy, float *gx, int64_t planes, int64_t h, int64_t w,
                                 int ry, int rx, bool dilate, cudaStream_t s) {
  if (ry < 0 || rx < 0 || ry > AR_MAX || rx > AR_MAX) return fail(PG_ERR_INVALID_ARGUMENT, "half sizes must be in [0, 7]");
  if (planes * h * w == 0) return PG_OK;
  if (h > (1 << 30) || w > (1 << 30) || ceil_div(h, AT_H) > 65535) return fail(PG_ERR_INVALID_ARGUMENT, "plane too large");
  static std::atomic<uint64_t> fs{0}, fe{0};
  const size_t sm = bwd_smem(ry, rx);
  if (dilate) {
    PG_TRY(ensure_smem(k_flat_bwd<true>, fs));
    k_flat_bwd<true><<<flat_grid(planes, h, w), AT_THREADS, sm, s>>>(x, gy, gx, planes, (int)h, (int)w, ry, rx);
  } else {
    PG_TRY(ensure_smem(k_flat_bwd<false>, fe));
    k_flat_bwd<false><<<flat_grid(planes, h, w), AT_THREADS, sm, s>>>(x, gy, gx, planes, (int)h, (int)w, ry, rx);
  }
  return cuda_status(cudaGetLastError(), "flat morphology backward launch");
}

}  // namespace pg
