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
// GPU design: a CTA owns a tile of one plane.  It stages x over the tile plus a halo, computes per
// row of the halo region the first-best value and column (separable arg-extremum: the first row, in
// dy order, whose row-best is strictly best, then that row's first column), and for the backward
// stages grad_out and gathers each input pixel's contributors.  Square windows of half size 1-3
// have fixed-size kernels (k_flat_fwd_r, and k_flat_bwd_g for half sizes 1 and 2); other windows the
// generic ones.
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
// Kernels for a square (2R+1)^2 window known at compile time: 2D thread indexing (no integer
// division per element), unrolled window loops, staging loads issued before the shared-memory
// stores.
static constexpr int AF_TX = 64, AF_TY = 4;  // 256 threads as 64 columns x 4 row groups

template <bool SUP> __device__ __forceinline__ float best_of(float a, float b) { return SUP ? fmaxf(a, b) : fminf(a, b); }

template <bool SUP, int R>
__global__ void __launch_bounds__(AT_THREADS) k_flat_fwd_r(const float *__restrict__ x, float *__restrict__ y, int H, int W) {
  // Tile: AT_H x FW outputs, FW = 64 - 2R, so that the staged band (FW + 2R) is exactly one
  // column per thread of a 64-wide row and every phase is a single pass.
  constexpr int FW = AF_TX - 2 * R;
  constexpr int XH = AT_H + 2 * R, XW = AF_TX;
  __shared__ float X[XH][XW + 1];
  __shared__ float RV[XH][FW + 1];
  const int tx = threadIdx.x % AF_TX, tq = threadIdx.x / AF_TX;
  const int ty0 = blockIdx.y * AT_H, tx0 = blockIdx.x * FW;
  const int64_t plane = (int64_t)blockIdx.z * H * W;
  const float *xp = x + plane;
  constexpr int RI = (XH + AF_TY - 1) / AF_TY;  // staged rows per thread
  {
    const int gx = tx0 - R + tx;
    const bool colin = gx >= 0 && gx < W;
    float v[RI];
#pragma unroll
    for (int k = 0; k < RI; ++k) {
      const int r = tq + k * AF_TY, gy = ty0 - R + r;
      v[k] = (r < XH && colin && gy >= 0 && gy < H) ? __ldg(xp + (int64_t)gy * W + gx) : outside<SUP>();
    }
#pragma unroll
    for (int k = 0; k < RI; ++k) {
      const int r = tq + k * AF_TY;
      if (r < XH) X[r][tx] = v[k];
    }
  }
  __syncthreads();
  if (tx < FW) {
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
  }
  __syncthreads();
  if (tx < FW) {
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
}

// Forward that also saves each output's arg code for the backward: code(p) = a * (2R+1) + b, (a, b)
// the window row and column of p's first-in-scan-order arg-extremum.  The values are the best_of
// chains of k_flat_fwd_r (y is bit-identical to the plain forward); the arg is the first position
// equal to that value -- in the row pass the first column of each row window equal to its best, in the
// column pass the first window row whose row-best equals the output.  Without NaN in x that is the
// position the strictly-better chains of k_flat_bwd find (equal values, -0 and +0 included, compare
// equal), so the backward from these codes is bit-identical to the recomputing one.
template <bool SUP, int R>
__global__ void __launch_bounds__(AT_THREADS) k_flat_fwd_arg(const float *__restrict__ x, float *__restrict__ y,
                                                             unsigned char *__restrict__ code, int H, int W) {
  constexpr int FW = AF_TX - 2 * R, WX = 2 * R + 1;
  constexpr int XH = AT_H + 2 * R, XW = AF_TX;
  __shared__ float X[XH][XW + 1];
  __shared__ float RV[XH][FW + 1];   // row-best values
  __shared__ unsigned char RA[XH][FW + 1];
  const int tx = threadIdx.x % AF_TX, tq = threadIdx.x / AF_TX;
  const int ty0 = blockIdx.y * AT_H, tx0 = blockIdx.x * FW;
  const int64_t plane = (int64_t)blockIdx.z * H * W;
  const float *xp = x + plane;
  constexpr int RI = (XH + AF_TY - 1) / AF_TY;
  {
    const int gx = tx0 - R + tx;
    const bool colin = gx >= 0 && gx < W;
    float v[RI];
#pragma unroll
    for (int k = 0; k < RI; ++k) {
      const int r = tq + k * AF_TY, gy = ty0 - R + r;
      v[k] = (r < XH && colin && gy >= 0 && gy < H) ? __ldg(xp + (int64_t)gy * W + gx) : outside<SUP>();
    }
#pragma unroll
    for (int k = 0; k < RI; ++k) {
      const int r = tq + k * AF_TY;
      if (r < XH) X[r][tx] = v[k];
    }
  }
  __syncthreads();
  if (tx < FW) {
#pragma unroll
    for (int k = 0; k < RI; ++k) {
      const int r = tq + k * AF_TY;
      if (r < XH) {
        float e[2 * R + 1];
#pragma unroll
        for (int d = 0; d <= 2 * R; ++d) e[d] = X[r][tx + d];
        float b = e[0];
#pragma unroll
        for (int d = 1; d <= 2 * R; ++d) b = best_of<SUP>(b, e[d]);
        int a = 2 * R;
#pragma unroll
        for (int d = 2 * R - 1; d >= 0; --d) a = (e[d] == b) ? d : a;
        RV[r][tx] = b;
        RA[r][tx] = (unsigned char)a;
      }
    }
  }
  __syncthreads();
  if (tx < FW) {
    float *yp = y + plane;
    unsigned char *cp = code + plane;
    constexpr int OR = AT_H / AF_TY;
    const int r0 = tq * OR, gx = tx0 + tx;
    float col[OR + 2 * R];
#pragma unroll
    for (int i = 0; i < OR + 2 * R; ++i) col[i] = RV[r0 + i][tx];
#pragma unroll
    for (int i = 0; i < OR; ++i) {
      float b = col[i];
#pragma unroll
      for (int d = 1; d <= 2 * R; ++d) b = best_of<SUP>(b, col[i + d]);
      int a = 2 * R;
#pragma unroll
      for (int d = 2 * R - 1; d >= 0; --d) a = (col[i + d] == b) ? d : a;
      const int gy = ty0 + r0 + i;
      if (gy < H && gx < W) {
        yp[(int64_t)gy * W + gx] = b;
        cp[(int64_t)gy * W + gx] = (unsigned char)(a * WX + RA[r0 + i + a][tx]);
      }
    }
  }
}

// Backward from the saved codes: grad_in[q] = sum over the outputs p of q's window, in raster order
// of p, of grad_out[p] when code(p) names q -- the gather of k_flat_bwd without recomputing the
// codes.  A thread owns four consecutive outputs q of a row (a quad at columns 4t .. 4t + 3 of the
// tile); for window row a the codes of all 4 x (2R+1) candidates p sit in the 4 + 2R bytes at staged
// column 4t, read as whole 32-bit words.  For each candidate column b one funnel shift lines up the
// four codes (one per q of the quad) and one exact zero-byte test of (codes ^ splat(want)) tells
// which q of the quad p routes to -- usually none; grad_out of the window row comes in as whole
// 16-byte vectors and is added only where the code matched.  (a, b)
// run in raster order, so each q adds its contributions in the order of a sequential accumulation
// in raster order of the outputs.  Codes outside the image are 255 and never match.
static constexpr int AQ_QUADS = 64, AQ_ROWS = 4;  // 256 threads: 64 quads x 4 row groups
// The staged band starts 4 columns left of the tile (a 16-byte boundary when rows are whole 16-byte
// vectors), so logical column c -- tile column c - R -- sits at staged column c + 4 - R.
template <int R>
__global__ void __launch_bounds__(AT_THREADS) k_flat_bwd_arg(const unsigned char *__restrict__ code,
                                                             const float *__restrict__ gy, float *__restrict__ gx,
                                                             int H, int W, int vec) {
  constexpr int WX = 2 * R + 1, TW = 4 * AQ_QUADS, SH = AT_H + 2 * R, OFF = 4 - R;
  constexpr int GV = (OFF + 2 * R + 3) / 4 + 1;  // words / float4s per window row and quad
  constexpr int SWW = AQ_QUADS + GV;             // staged words (4 codes, or 4 floats) per row
  constexpr int SW = 4 * SWW;
  __shared__ uint32_t C[SH][SWW];
  __shared__ __align__(16) float G[SH][SW];
  const int ty0 = blockIdx.y * AT_H, tx0 = blockIdx.x * TW;
  const int64_t plane = (int64_t)blockIdx.z * H * W;
  const float *gp = gy + plane;
  const unsigned char *cp = code + plane;
  if (vec) {
    // whole 16-byte groups of 4 columns, each wholly inside or outside the image
    for (int i = threadIdx.x; i < SH * SWW; i += AT_THREADS) {
      const int r = i / SWW, m = i - r * SWW;
      const int yy = ty0 - R + r, xx = tx0 - 4 + 4 * m;
      const bool in = yy >= 0 && yy < H && xx >= 0 && xx < W;
      const int64_t o = in ? (int64_t)yy * W + xx : 0;
      const float4 g = __ldg(reinterpret_cast<const float4 *>(gp + o));
      const uint32_t k = __ldg(reinterpret_cast<const unsigned int *>(cp + o));
      *reinterpret_cast<float4 *>(&G[r][4 * m]) = in ? g : make_float4(0.f, 0.f, 0.f, 0.f);
      C[r][m] = in ? k : 0xffffffffu;
    }
  } else {
    unsigned char *Cb = reinterpret_cast<unsigned char *>(&C[0][0]);
    for (int i = threadIdx.x; i < SH * SW; i += AT_THREADS) {
      const int r = i / SW, c = i - r * SW;
      const int yy = ty0 - R + r, xx = tx0 - 4 + c;
      const bool in = yy >= 0 && yy < H && xx >= 0 && xx < W;
      const int64_t o = in ? (int64_t)yy * W + xx : 0;
      const float g = __ldg(gp + o);
      const unsigned char k = __ldg(cp + o);
      G[r][c] = in ? g : 0.f;
      Cb[r * SW + c] = in ? k : (unsigned char)255;
    }
  }
  __syncthreads();
  const int t = threadIdx.x % AQ_QUADS, tq = threadIdx.x / AQ_QUADS;
  const int xq = tx0 + 4 * t;  // the quad's first column
  if (xq >= W) return;
  float *op = gx + plane;
  for (int r = tq; r < AT_H; r += AQ_ROWS) {
    const int yy = ty0 + r;
    if (yy >= H) break;
    float sum[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int a = 0; a < WX; ++a) {
      uint32_t w[GV];
      float g[4 * GV];  // grad_out of staged columns 4t .. 4t + 4GV - 1 of window row a
#pragma unroll
      for (int k = 0; k < GV; ++k) {
        w[k] = C[r + a][t + k];
        const float4 v = *reinterpret_cast<const float4 *>(&G[r + a][4 * (t + k)]);
        g[4 * k] = v.x; g[4 * k + 1] = v.y; g[4 * k + 2] = v.z; g[4 * k + 3] = v.w;
      }
#pragma unroll
      for (int b = 0; b < WX; ++b) {
        // codes of the candidates at column b of window row a (staged column 4t + OFF + b + j), for
        // q = quad + j, j = 0..3
        const int sb = OFF + b;
        const uint32_t cw = (sb % 4 == 0) ? w[sb / 4] : __funnelshift_r(w[sb / 4], w[sb / 4 + 1], 8 * (sb % 4));
        const uint32_t want = 0x01010101u * (uint32_t)((2 * R - a) * WX + (2 * R - b));
        const uint32_t x = cw ^ want;
        const uint32_t z = ~((((x & 0x7f7f7f7fu) + 0x7f7f7f7fu) | x) | 0x7f7f7f7fu);  // 0x80 in each zero byte
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (z & (0x80u << (8 * j))) sum[j] += g[sb + j];
      }
    }
    float *o = op + (int64_t)yy * W + xq;
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (xq + j < W) o[j] = sum[j];
  }
}

template <bool SUP>
static bool flat_fwd_fixed(const float *x, float *y, int64_t planes, int64_t h, int64_t w, int ry, int rx, cudaStream_t s) {
  if (ry != rx || ry < 1 || ry > 3 || planes > 65535) return false;
  const dim3 grid((unsigned)ceil_div(w, AF_TX - 2 * ry), (unsigned)ceil_div(h, AT_H), (unsigned)planes);
  if (ry == 1) k_flat_fwd_r<SUP, 1><<<grid, AT_THREADS, 0, s>>>(x, y, (int)h, (int)w);
  else if (ry == 2) k_flat_fwd_r<SUP, 2><<<grid, AT_THREADS, 0, s>>>(x, y, (int)h, (int)w);
  else k_flat_fwd_r<SUP, 3><<<grid, AT_THREADS, 0, s>>>(x, y, (int)h, (int)w);
  return true;
}

// Backward for R = 1, 2 (the 3x3 and 5x5 squares), atomic-free.  With va(p) the window row of output
// p's first-in-scan-order arg-extremum and ra(y, x) the column of the first-best pixel of row y's
// window centred at x, output p routes to q iff  va(p) = 2R - a  for p = (q.y - R + a, .)  and
// ra(q.y, p.x) = 2R - b  for p = (., q.x - R + b).  So:
//   row pass    -- ra and the row-best value of every (x row, node column) of the tile's halo;
//   column pass -- for every node (q row y, column x): the bits a of the outputs p = (y - R + a, x)
//                  whose va is 2R - a (their row arg lands on row y), packed with ra(y, x) in one
//                  word (bits a * (2R+1), ra at bit 28) -- a gather down the column, in registers;
//   gather      -- q reads the words of nodes (q.y, q.x - R + b), keeps those whose ra points at q
//                  (ra = 2R - b), shifts each by b, and so gets the mask of its contributors, bit
//                  a * (2R+1) + b: raster order of the outputs.  It sums grad_out over the set bits
//                  from the lowest, the order of a sequential accumulation in raster order of the
//                  outputs, so the result is bit-identical to it.
// No atomics.  Tile: AT_H x QW outputs, QW = 64 - 4R (the staged x band is one 64-thread row).
// Shared-memory layout of k_flat_bwd_g for a tile of TH rows (bytes, each part 16-byte aligned).  The
// node words reuse the staged x once the row pass has read it.
template <int R, int TH> struct BwdG {
  static constexpr int WX = 2 * R + 1, QW = AF_TX - 4 * R, XH = TH + 4 * R, XW = AF_TX + 1;
  static constexpr int PH = TH + 2 * R, PW = QW + 2 * R + 1;  // padded pitches (+1)
  static constexpr int WARP_PIX = TH / AF_TY * 32;           // tile pixels a warp handles
  static constexpr size_t al(size_t b) { return (b + 15) / 16 * 16; }
  static constexpr size_t X_OFF = 0, X_BYTES = al((size_t)XH * XW * 4);  // x, later the node words
  static constexpr size_t RV_OFF = X_OFF + X_BYTES, RV_BYTES = al((size_t)XH * PW * 4);
  static constexpr size_t G_OFF = RV_OFF + RV_BYTES, G_BYTES = al((size_t)PH * PW * 4);
  static constexpr size_t RA_OFF = G_OFF + G_BYTES, RA_BYTES = al((size_t)XH * PW);
  static constexpr size_t H_OFF = RA_OFF + RA_BYTES, H_BYTES = al((size_t)(AT_THREADS / 32) * WARP_PIX * 2);
  static constexpr size_t smem = H_OFF + H_BYTES;
  static_assert((size_t)TH * PW * 4 <= X_BYTES, "node words must fit in the x buffer");
};

template <bool SUP, int R, int TH>
__global__ void __launch_bounds__(AT_THREADS) k_flat_bwd_g(const float *__restrict__ x, const float *__restrict__ gy,
                                                           float *__restrict__ gx, int H, int W) {
  using L = BwdG<R, TH>;
  constexpr int WX = L::WX;
  static_assert(WX * WX <= 28, "contributor mask and row arg must share one word");
  constexpr unsigned MASK = (1u << (WX * WX)) - 1u;
  constexpr int QW = L::QW;
  constexpr int XH = L::XH, XW = L::XW;               // x rows: tile rows -2R .. TH + 2R - 1
  constexpr int PH = L::PH, PW = QW + 2 * R, PP = L::PW;  // outputs: tile rows / cols -R .. +R beyond the tile
  constexpr int XR = (XH + AF_TY - 1) / AF_TY;       // staged x rows per thread
  constexpr int GR = (PH + AF_TY - 1) / AF_TY;       // staged gradient rows per thread
  constexpr int NR = TH / AF_TY;                     // node rows per thread (consecutive)
  extern __shared__ __align__(16) unsigned char smb[];
  float(*X)[XW] = reinterpret_cast<float(*)[XW]>(smb + L::X_OFF);
  unsigned(*NODE)[PP] = reinterpret_cast<unsigned(*)[PP]>(smb + L::X_OFF);  // after the row pass
  float(*RV)[PP] = reinterpret_cast<float(*)[PP]>(smb + L::RV_OFF);
  float(*G)[PP] = reinterpret_cast<float(*)[PP]>(smb + L::G_OFF);
  unsigned char(*RA)[PP] = reinterpret_cast<unsigned char(*)[PP]>(smb + L::RA_OFF);
  unsigned short *HEAVY = reinterpret_cast<unsigned short *>(smb + L::H_OFF);
  const int tx = threadIdx.x % AF_TX, tq = threadIdx.x / AF_TX;
  const int ty0 = blockIdx.y * TH, tx0 = blockIdx.x * QW;
  const int64_t plane = (int64_t)blockIdx.z * H * W;
  const float *xp = x + plane;
  const float *gp = gy + plane;
  {  // stage x and the upstream gradient, loads first
    const int xx = tx0 - 2 * R + tx;
    const bool xin = xx >= 0 && xx < W;
    float v[XR];
#pragma unroll
    for (int k = 0; k < XR; ++k) {
      const int r = tq + k * AF_TY, yy = ty0 - 2 * R + r;
      v[k] = (r < XH && xin && yy >= 0 && yy < H) ? __ldg(xp + (int64_t)yy * W + xx) : outside<SUP>();
    }
    const int gxx = tx0 - R + tx;
    const bool gin = tx < PW && gxx >= 0 && gxx < W;
    float g[GR];
#pragma unroll
    for (int k = 0; k < GR; ++k) {
      const int r = tq + k * AF_TY, yy = ty0 - R + r;
      g[k] = (r < PH && gin && yy >= 0 && yy < H) ? __ldg(gp + (int64_t)yy * W + gxx) : 0.f;
    }
#pragma unroll
    for (int k = 0; k < XR; ++k) {
      const int r = tq + k * AF_TY;
      if (r < XH) X[r][tx] = v[k];
    }
#pragma unroll
    for (int k = 0; k < GR; ++k) {
      const int r = tq + k * AF_TY;
      if (r < PH && tx < PW) G[r][tx] = g[k];
    }
  }
  __syncthreads();
  // row pass over the node columns: first strictly-best column of each row segment
  if (tx < PW) {
#pragma unroll
    for (int k = 0; k < XR; ++k) {
      const int r = tq + k * AF_TY;
      if (r < XH) {
        float b = X[r][tx];
        int a = 0;
#pragma unroll
        for (int d = 1; d <= 2 * R; ++d) {
          const float v = X[r][tx + d];
          if (better<SUP>(v, b)) { b = v; a = d; }
        }
        RV[r][tx] = b;
        RA[r][tx] = (unsigned char)a;
      }
    }
  }
  __syncthreads();  // x is dead from here on: its buffer takes the node words
  // column pass: thread (tx, tq) owns node rows [tq * NR, tq * NR + NR) of node column tx.  Node row
  // y needs va of the outputs in P rows y .. y + 2R (output row y - R + a is P row y + a), and the
  // output in P row pr takes its window rows from RV rows pr .. pr + 2R.  The node's word holds those
  // bits already shifted by its own b = 2R - ra (its column offset seen from the pixel it routes to),
  // with that b at bit 28.
  if (tx < PW) {
    const int xx = tx0 - R + tx;
    const bool colin = xx >= 0 && xx < W;
    const int y0 = tq * NR;
    float col[NR + 4 * R];
#pragma unroll
    for (int i = 0; i < NR + 4 * R; ++i) col[i] = RV[y0 + i][tx];
    unsigned va[NR + 2 * R];  // 0xff for outputs outside the image: never a route
#pragma unroll
    for (int i = 0; i < NR + 2 * R; ++i) {
      float b = col[i];
      unsigned a = 0;
#pragma unroll
      for (int d = 1; d <= 2 * R; ++d)
        if (better<SUP>(col[i + d], b)) { b = col[i + d]; a = d; }
      const int oy = ty0 - R + y0 + i;  // image row of the output in P row y0 + i
      va[i] = (colin && oy >= 0 && oy < H) ? a : 0xffu;
    }
#pragma unroll
    for (int j = 0; j < NR; ++j) {
      unsigned vm = 0u;
#pragma unroll
      for (int a = 0; a <= 2 * R; ++a) vm |= (va[j + a] == (unsigned)(2 * R - a) ? 1u : 0u) << (a * WX);
      const unsigned bsh = (unsigned)(2 * R) - RA[y0 + j + 2 * R][tx];
      NODE[y0 + j][tx] = (vm << bsh) | (bsh << 28);
    }
  }
  __syncthreads();
  // gather in raster order of the contributors; a pixel with more than two of them (a local extremum
  // collects up to (2R+1)^2) goes to its warp's list, handled in a second pass, so that one lane's long
  // chain does not hold up its warp (each warp keeps its own list, filled by ballot: no shared counter)
  auto mask_of = [&](int r, int c) -> unsigned {
    unsigned m = 0u;
#pragma unroll
    for (int b = 0; b <= 2 * R; ++b) {
      const unsigned w = NODE[r][c + b];
      if ((w >> 28) == (unsigned)b) m |= w & MASK;
    }
    return m;
  };
  auto gather = [&](int r, int c, unsigned m) -> float {
    float sum = 0.f;
    while (m) {
      const int bit = __ffs(m) - 1;
      m &= m - 1u;
      const int a = bit / WX, b = bit - a * WX;
      sum += G[r + a][c + b];
    }
    return sum;
  };
  float *op = gx + plane;
  const int lane = threadIdx.x & 31;
  unsigned short *heavy = HEAVY + (threadIdx.x / 32) * L::WARP_PIX;
  int n_heavy = 0;  // warp-uniform
  {
    const int xx = tx0 + tx;
#pragma unroll 4
    for (int r = tq; r < TH; r += AF_TY) {
      const int yy = ty0 + r;
      const bool mine = tx < QW && yy < H && xx < W;
      const unsigned m = mine ? mask_of(r, tx) : 0u;
      const bool defer = __popc(m) > 2;
      const unsigned db = __ballot_sync(0xffffffffu, defer);
      if (defer) heavy[n_heavy + __popc(db & ((1u << lane) - 1u))] = (unsigned short)(r * QW + tx);
      else if (mine) op[(int64_t)yy * W + xx] = gather(r, tx, m);
      n_heavy += __popc(db);
    }
  }
  __syncwarp();
  for (int i = lane; i < n_heavy; i += 32) {
    const int q = heavy[i], r = q / QW, c = q - r * QW;
    op[(int64_t)(ty0 + r) * W + tx0 + c] = gather(r, c, mask_of(r, c));
  }
}

template <bool SUP, int R, int TH>
static pg_status bwd_g_launch(const float *x, const float *g, float *o, int64_t planes, int64_t h, int64_t w,
                              cudaStream_t s) {
  using L = BwdG<R, TH>;
  static std::atomic<uint64_t> attr{0};
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  const uint64_t bit = 1ull << (dev & 63);
  if (!(attr.load() & bit)) {
    PG_CUDA_TRY(cudaFuncSetAttribute(k_flat_bwd_g<SUP, R, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::smem),
                "backward smem attribute");
    attr.fetch_or(bit);
  }
  const dim3 grid((unsigned)ceil_div(w, L::QW), (unsigned)ceil_div(h, TH), (unsigned)planes);
  k_flat_bwd_g<SUP, R, TH><<<grid, AT_THREADS, L::smem, s>>>(x, g, o, (int)h, (int)w);
  return cuda_status(cudaGetLastError(), "flat morphology backward launch");
}

// rows per backward tile: taller tiles stage less halo per pixel, at more shared memory per CTA
static constexpr int kBwdTileH = 32;

template <bool SUP>
static bool flat_bwd_fixed(const float *x, const float *g, float *o, int64_t planes, int64_t h, int64_t w, int ry, int rx,
                           cudaStream_t s, pg_status *st) {
  if (ry != rx || ry < 1 || ry > 2 || planes > 65535 || ceil_div(h, kBwdTileH) > 65535) return false;
  *st = ry == 1 ? bwd_g_launch<SUP, 1, kBwdTileH>(x, g, o, planes, h, w, s) : bwd_g_launch<SUP, 2, kBwdTileH>(x, g, o, planes, h, w, s);
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

pg_status launch_flat2d_arg(const float *x, float *y, unsigned char *code, int64_t planes, int64_t h, int64_t w, int r,
                            bool dilate, cudaStream_t s) {
  if (r < 1 || r > 3) return fail(PG_ERR_INVALID_ARGUMENT, "saved-arg forward: square windows of half size 1 to 3");
  if (planes * h * w == 0) return PG_OK;
  if (h > (1 << 30) || w > (1 << 30) || ceil_div(h, AT_H) > 65535 || planes > 65535)
    return fail(PG_ERR_INVALID_ARGUMENT, "plane too large");
  const dim3 grid((unsigned)ceil_div(w, AF_TX - 2 * r), (unsigned)ceil_div(h, AT_H), (unsigned)planes);
  const int ih = (int)h, iw = (int)w;
  if (dilate) {
    if (r == 1) k_flat_fwd_arg<true, 1><<<grid, AT_THREADS, 0, s>>>(x, y, code, ih, iw);
    else if (r == 2) k_flat_fwd_arg<true, 2><<<grid, AT_THREADS, 0, s>>>(x, y, code, ih, iw);
    else k_flat_fwd_arg<true, 3><<<grid, AT_THREADS, 0, s>>>(x, y, code, ih, iw);
  } else {
    if (r == 1) k_flat_fwd_arg<false, 1><<<grid, AT_THREADS, 0, s>>>(x, y, code, ih, iw);
    else if (r == 2) k_flat_fwd_arg<false, 2><<<grid, AT_THREADS, 0, s>>>(x, y, code, ih, iw);
    else k_flat_fwd_arg<false, 3><<<grid, AT_THREADS, 0, s>>>(x, y, code, ih, iw);
  }
  return cuda_status(cudaGetLastError(), "flat morphology forward (saved arg) launch");
}

pg_status launch_flat2d_backward_arg(const unsigned char *code, const float *gy, float *gx, int64_t planes, int64_t h,
                                     int64_t w, int r, cudaStream_t s) {
  if (r < 1 || r > 3) return fail(PG_ERR_INVALID_ARGUMENT, "saved-arg backward: square windows of half size 1 to 3");
  if (planes * h * w == 0) return PG_OK;
  if (h > (1 << 30) || w > (1 << 30) || ceil_div(h, AT_H) > 65535 || planes > 65535)
    return fail(PG_ERR_INVALID_ARGUMENT, "plane too large");
  const dim3 grid((unsigned)ceil_div(w, 4 * AQ_QUADS), (unsigned)ceil_div(h, AT_H), (unsigned)planes);
  // 16-byte staging: rows of whole vectors (4 floats, 4 codes) and aligned bases
  const int vec = (w % 4 == 0 && reinterpret_cast<uintptr_t>(gy) % 16 == 0 && reinterpret_cast<uintptr_t>(code) % 4 == 0)
                      ? 1 : 0;
  if (r == 1) k_flat_bwd_arg<1><<<grid, AT_THREADS, 0, s>>>(code, gy, gx, (int)h, (int)w, vec);
  else if (r == 2) k_flat_bwd_arg<2><<<grid, AT_THREADS, 0, s>>>(code, gy, gx, (int)h, (int)w, vec);
  else k_flat_bwd_arg<3><<<grid, AT_THREADS, 0, s>>>(code, gy, gx, (int)h, (int)w, vec);
  return cuda_status(cudaGetLastError(), "flat morphology backward (saved arg) launch");
}

pg_status launch_flat2d_backward(const float *x, const float *gy, float *gx, int64_t planes, int64_t h, int64_t w,
                                 int ry, int rx, bool dilate, cudaStream_t s) {
  if (ry < 0 || rx < 0 || ry > AR_MAX || rx > AR_MAX) return fail(PG_ERR_INVALID_ARGUMENT, "half sizes must be in [0, 7]");
  if (planes * h * w == 0) return PG_OK;
  if (h > (1 << 30) || w > (1 << 30) || ceil_div(h, AT_H) > 65535) return fail(PG_ERR_INVALID_ARGUMENT, "plane too large");
  pg_status st = PG_OK;
  if (dilate ? flat_bwd_fixed<true>(x, gy, gx, planes, h, w, ry, rx, s, &st)
             : flat_bwd_fixed<false>(x, gy, gx, planes, h, w, ry, rx, s, &st))
    return st;
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
