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

// ------------------------------------------------------------------ fixed window sizes
// The same two kernels for a square (2R+1)^2 window known at compile time (R = 1, 2, 3): 2D thread
// indexing (no integer division per element), unrolled window loops, staging loads issued before
// the shared-memory stores, and a backward that does not test every window offset of every
// output.  Backward: each routing output p sets bit `code` (its arg's position in its window) in
// a 32-bit mask of the tile pixel q it routes to (shared atomicOr: order-free); then q adds the
// upstream gradient of each contributor from the highest set bit to the lowest.  A higher code
// means a contributor earlier in raster order, so the sum runs in the same order as the generic
// kernel's gather and the result is bit-identical.  Needs (2R+1)^2 <= 32.
static constexpr int AF_TX = 64, AF_TY = 4;  // 256 threads as 64 columns x 4 row groups

template <bool SUP> __device__ __forceinline__ float best_of(float a, float b) { return SUP ? fmaxf(a, b) : fminf(a, b); }

template <bool SUP, int R>
__global__ void __launch_bounds__(AT_THREADS) k_flat_fwd_r(const float *__restrict__ x, float *__restrict__ y, int H, int W) {
  constexpr int XH = AT_H + 2 * R, XW = AT_W + 2 * R;
  __shared__ float X[XH][XW + 1];
  __shared__ float RV[XH][AT_W + 1];
  const int tx = threadIdx.x % AF_TX, tq = threadIdx.x / AF_TX;
  const int ty0 = blockIdx.y * AT_H, tx0 = blockIdx.x * AT_W;
  const int64_t plane = (int64_t)blockIdx.z * H * W;
  const float *xp = x + plane;
  constexpr int RI = (XH + AF_TY - 1) / AF_TY;  // staged rows per thread
#pragma unroll
  for (int cc = 0; cc < XW; cc += AF_TX) {
    const int c = cc + tx;
    const int gx = tx0 - R + c;
    float v[RI];
#pragma unroll
    for (int k = 0; k < RI; ++k) {
      const int r = tq + k * AF_TY, gy = ty0 - R + r;
      const bool in = c < XW && r < XH && gy >= 0 && gy < H && gx >= 0 && gx < W;
      v[k] = in ? __ldg(xp + (int64_t)gy * W + gx) : outside<SUP>();
    }
#pragma unroll
    for (int k = 0; k < RI; ++k) {
      const int r = tq + k * AF_TY;
      if (c < XW && r < XH) X[r][c] = v[k];
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < RI; ++k) {
    const int r = tq + k * AF_TY;
    if (r < XH) {
      float b = X[r][tx];
#pragma unroll
      for (int d = 1; d <= 2 * R; ++d) b = best_of<SUP>(b, X[r][tx + d]);
      RV[r][tx] = b;
    }
  }
  __syncthreads();
  float *yp = y + plane;
  constexpr int OR = AT_H / AF_TY;  // output rows per thread, consecutive
  const int r0 = tq * OR, gx = tx0 + tx;
  float col[OR + 2 * R];
#pragma unroll
  for (int i = 0; i < OR + 2 * R; ++i) col[i] = RV[r0 + i][tx];
#pragma unroll
  for (int i = 0; i < OR; ++i) {
    float b = col[i];
#pragma unroll
    for (int d = 1; d <= 2 * R; ++d) b = best_of<SUP>(b, col[i + d]);
    const int gy = ty0 + r0 + i;
    if (gy < H && gx < W) yp[(int64_t)gy * W + gx] = b;
  }
}

template <bool SUP, int R>
__global__ void __launch_bounds__(AT_THREADS) k_flat_bwd_r(const float *__restrict__ x, const float *__restrict__ gy,
                                                           float *__restrict__ gx, int H, int W) {
  constexpr int WX = 2 * R + 1;
  static_assert(WX * WX <= 32, "codes must fit a 32-bit mask");
  constexpr int XH = AT_H + 4 * R, XW = AT_W + 4 * R;  // x over the tile + 2R
  constexpr int PH = AT_H + 2 * R, PW = AT_W + 2 * R;  // outputs that can route into the tile
  __shared__ float X[XH][XW + 1];
  __shared__ float RV[XH][PW + 1];
  __shared__ unsigned char RA[XH][PW + 1];
  __shared__ float G[PH][PW + 1];
  __shared__ unsigned M[AT_H][AT_W];
  const int tx = threadIdx.x % AF_TX, tq = threadIdx.x / AF_TX;
  const int ty0 = blockIdx.y * AT_H, tx0 = blockIdx.x * AT_W;
  const int64_t plane = (int64_t)blockIdx.z * H * W;
  const float *xp = x + plane;
  const float *gp = gy + plane;
  // stage x (tile + 2R) and the upstream gradient (tile + R); clear the masks
  {
    constexpr int RI = (XH + AF_TY - 1) / AF_TY;
#pragma unroll
    for (int cc = 0; cc < XW; cc += AF_TX) {
      const int c = cc + tx, xx = tx0 - 2 * R + c;
      float v[RI];
#pragma unroll
      for (int k = 0; k < RI; ++k) {
        const int r = tq + k * AF_TY, yy = ty0 - 2 * R + r;
        const bool in = c < XW && r < XH && yy >= 0 && yy < H && xx >= 0 && xx < W;
        v[k] = in ? __ldg(xp + (int64_t)yy * W + xx) : outside<SUP>();
      }
#pragma unroll
      for (int k = 0; k < RI; ++k) {
        const int r = tq + k * AF_TY;
        if (c < XW && r < XH) X[r][c] = v[k];
      }
    }
    constexpr int RG = (PH + AF_TY - 1) / AF_TY;
#pragma unroll
    for (int cc = 0; cc < PW; cc += AF_TX) {
      const int c = cc + tx, xx = tx0 - R + c;
      float v[RG];
#pragma unroll
      for (int k = 0; k < RG; ++k) {
        const int r = tq + k * AF_TY, yy = ty0 - R + r;
        const bool in = c < PW && r < PH && yy >= 0 && yy < H && xx >= 0 && xx < W;
        v[k] = in ? __ldg(gp + (int64_t)yy * W + xx) : 0.f;
      }
#pragma unroll
      for (int k = 0; k < RG; ++k) {
        const int r = tq + k * AF_TY;
        if (c < PW && r < PH) G[r][c] = v[k];
      }
    }
#pragma unroll
    for (int r = tq; r < AT_H; r += AF_TY) M[r][tx] = 0u;
  }
  __syncthreads();
  // row pass over the P columns: first strictly-best column of each row segment
  for (int cc = 0; cc < PW; cc += AF_TX) {
    const int c = cc + tx;
    if (c < PW) {
#pragma unroll 4
      for (int r = tq; r < XH; r += AF_TY) {
        float b = X[r][c];
        int a = 0;
#pragma unroll
        for (int d = 1; d <= 2 * R; ++d)
          if (better<SUP>(X[r][c + d], b)) { b = X[r][c + d]; a = d; }
        RV[r][c] = b;
        RA[r][c] = (unsigned char)a;
      }
    }
  }
  __syncthreads();
  // column pass: each routing output's arg code, posted as a bit to the tile pixel it routes to
  for (int cc = 0; cc < PW; cc += AF_TX) {
    const int c = cc + tx;
    if (c >= PW) continue;
    const int xx = tx0 - R + c;
#pragma unroll 2
    for (int r = tq; r < PH; r += AF_TY) {
      const int yy = ty0 - R + r;
      if (yy < 0 || yy >= H || xx < 0 || xx >= W) continue;  // not an output
      float b = RV[r][c];
      int a = 0;
#pragma unroll
      for (int d = 1; d <= 2 * R; ++d)
        if (better<SUP>(RV[r + d][c], b)) { b = RV[r + d][c]; a = d; }
      const int ac = RA[r + a][c];
      // the arg, in tile coordinates: output (r - R, c - R) + window (a - R, ac - R)
      const int qr = r - 2 * R + a, qc = c - 2 * R + ac;
      if (qr >= 0 && qr < AT_H && qc >= 0 && qc < AT_W) atomicOr(&M[qr][qc], 1u << (a * WX + ac));
    }
  }
  __syncthreads();
  // gather: contributors in raster order = codes from high to low
  float *op = gx + plane;
  const int xx = tx0 + tx;
#pragma unroll 2
  for (int r = tq; r < AT_H; r += AF_TY) {
    const int yy = ty0 + r;
    if (yy >= H || xx >= W) continue;
    unsigned m = M[r][tx];
    float sum = 0.f;
    while (m) {
      const int code = 31 - __clz(m);
      m &= ~(1u << code);
      const int a = code / WX, ac = code - a * WX;
      // contributor p = q - (window offset) in P coordinates: (r + R) + R - a, (tx + R) + R - ac
      sum += G[r + 2 * R - a][tx + 2 * R - ac];
    }
    op[(int64_t)yy * W + xx] = sum;
  }
}

template <bool SUP>
static bool flat_fwd_fixed(const float *x, float *y, int64_t planes, int64_t h, int64_t w, int ry, int rx, cudaStream_t s) {
  if (ry != rx || ry < 1 || ry > 3 || planes > 65535) return false;
  const dim3 grid((unsigned)ceil_div(w, AT_W), (unsigned)ceil_div(h, AT_H), (unsigned)planes);
  if (ry == 1) k_flat_fwd_r<SUP, 1><<<grid, AT_THREADS, 0, s>>>(x, y, (int)h, (int)w);
  else if (ry == 2) k_flat_fwd_r<SUP, 2><<<grid, AT_THREADS, 0, s>>>(x, y, (int)h, (int)w);
  else k_flat_fwd_r<SUP, 3><<<grid, AT_THREADS, 0, s>>>(x, y, (int)h, (int)w);
  return true;
}

template <bool SUP>
static bool flat_bwd_fixed(const float *x, const float *g, float *o, int64_t planes, int64_t h, int64_t w, int ry, int rx,
                           cudaStream_t s) {
  if (ry != rx || ry < 1 || ry > 2 || planes > 65535) return false;  // (2R+1)^2 <= 32
  const dim3 grid((unsigned)ceil_div(w, AT_W), (unsigned)ceil_div(h, AT_H), (unsigned)planes);
  if (ry == 1) k_flat_bwd_r<SUP, 1><<<grid, AT_THREADS, 0, s>>>(x, g, o, (int)h, (int)w);
  else k_flat_bwd_r<SUP, 2><<<grid, AT_THREADS, 0, s>>>(x, g, o, (int)h, (int)w);
  return true;
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
  if (dilate ? flat_fwd_fixed<true>(x, y, planes, h, w, ry, rx, s) : flat_fwd_fixed<false>(x, y, planes, h, w, ry, rx, s))
    return cuda_status(cudaGetLastError(), "flat morphology forward launch");
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
  if (dilate ? flat_bwd_fixed<true>(x, gy, gx, planes, h, w, ry, rx, s)
             : flat_bwd_fixed<false>(x, gy, gx, planes, h, w, ry, rx, s))
    return cuda_status(cudaGetLastError(), "flat morphology backward launch");
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
