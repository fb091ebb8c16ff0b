// line_stream.cu -- register-streaming vertical and diagonal segments (van Herk / Gil-Werman in
// registers).
//
// Same result as line.cu / line_w.cu for the Y segment of 2K+1 pixels (DilateY/ErodeY,
// ero_dil_line_se_t.hpp:249-282; clipped window) and for the 45 / 135 degree segments (runtime
// neighbour lists).  Used for the half lengths instantiated below, 1/2/4-byte pixels, word-aligned
// rows (the 1-/2-byte diagonals through k_dline_words, which keeps whole words), where the TMA tiles of
// diag.cu do not apply (their half lengths 7, 15, 31 on rows of a multiple of 16 bytes take those).
//
// A thread owns one 32-bit word column (E = 4/sizeof(T) adjacent pixel columns) of a strip of
// rows and walks down it block by block (blocks of W = 2K+1 rows, anchored K rows above the
// strip).  A block's W words are loaded at once (W independent, coalesced loads in flight per
// warp); the running prefix of the block is formed while the outputs that need it are written
// -- out(y) = op(suffix of the previous block at y-K, prefix of this block at y+K) -- and the
// block's running suffix is then kept in registers for the next block.  No shared memory, no
// barriers: every warp streams independently, so DRAM stays busy.
#include "common.cuh"
#include "words.cuh"

namespace pg {

static constexpr int kLSThreads = 128;

template <typename T, bool SUP, int K>
__global__ void __launch_bounds__(kLSThreads) k_vline_stream(const uint32_t *__restrict__ in, uint32_t *__restrict__ out,
                                                            int H, int Wn, int strip) {
  constexpr int W = 2 * K + 1;
  const int col = blockIdx.x * kLSThreads + threadIdx.x;
  const int y0 = blockIdx.y * strip;
  if (col >= Wn) return;
  const int y1 = min(y0 + strip, H);
  const uint32_t NEUW = splat<T>(Op<T, SUP>::neutral());
  const uint32_t *src = in + col;
  uint32_t *dst = out + col;

  uint32_t suf[W];  // running suffix of the previous block
#pragma unroll
  for (int i = 0; i < W; ++i) suf[i] = NEUW;
  // blocks start at ys = y0 - K; block b covers rows [ys + b*W, ys + (b+1)*W); rows from y1 + K on
  // only feed outputs below the strip and are not read
  const int ys = y0 - K;
  const int ylim = min(y1 + K, H);
  for (int yb = ys; yb < y1 + K; yb += W) {
    uint32_t raw[W];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      const int y = yb + i;
      raw[i] = (y >= 0 && y < ylim) ? __ldg(src + (size_t)y * Wn) : NEUW;
    }
    // prefix of this block; the output row y = yb + i - K uses suf[i + 1] (previous block's
    // suffix at y - K) and the prefix at y + K; for i = W-1 the window is exactly this block
    uint32_t pre = raw[0];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      if (i > 0) pre = wop<T, SUP>(pre, raw[i]);
      const int y = yb + i - K;
      if (y >= y0 && y < y1) dst[(size_t)y * Wn] = (i < W - 1) ? wop<T, SUP>(suf[i + 1], pre) : pre;
    }
    // suffix of this block for the next one
    suf[W - 1] = raw[W - 1];
#pragma unroll
    for (int i = W - 2; i >= 0; --i) suf[i] = wop<T, SUP>(suf[i + 1], raw[i]);
  }
}

// Diagonal segments, same scheme along a diagonal, one pixel per thread: lane j of a warp follows
// the diagonal through pixel x0 + j of row y0, i.e. x(y) = x0 + j - d (45 degrees: x + y constant)
// or x0 + j + d (135 degrees: x - y constant), d = y - y0.  A warp's 32 pixels of a row are
// contiguous, so loads and stores stay coalesced (unaligned by the row's shift); pixels outside
// the image read as neutral and are not written.  Packing several pixels per word would make each
// lane's word unaligned by a row-dependent shift and need a shuffle per row; measured slower.
template <typename T, bool SUP, int K, int DIR>  // DIR = +1: 45 degrees (dx = -1), -1: 135 degrees (dx = +1)
__global__ void __launch_bounds__(kLSThreads) k_dline_stream(const T *__restrict__ in, T *__restrict__ out, int H,
                                                            int Wd, int strip, int x_first) {
  constexpr int W = 2 * K + 1;
  const int x0 = x_first + blockIdx.x * kLSThreads + threadIdx.x;  // this thread's pixel at row y0
  const int y0 = blockIdx.y * strip;
  const int y1 = min(y0 + strip, H);
  const T NEU = Op<T, SUP>::neutral();
  T suf[W];
#pragma unroll
  for (int i = 0; i < W; ++i) suf[i] = NEU;
  const int ys = y0 - K;
  for (int yb = ys; yb < y1 + K; yb += W) {
    T raw[W];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      const int y = yb + i;
      const int x = DIR > 0 ? x0 - (y - y0) : x0 + (y - y0);
      raw[i] = (y >= 0 && y < H && x >= 0 && x < Wd) ? ldg(in + (size_t)y * Wd + x) : NEU;
    }
    T pre = raw[0];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      if (i > 0) pre = Op<T, SUP>::apply(pre, raw[i]);
      const int y = yb + i - K;
      const int x = DIR > 0 ? x0 - (y - y0) : x0 + (y - y0);
      if (y >= y0 && y < y1 && x >= 0 && x < Wd)
        out[(size_t)y * Wd + x] = (i < W - 1) ? Op<T, SUP>::apply(suf[i + 1], pre) : pre;
    }
    suf[W - 1] = raw[W - 1];
#pragma unroll
    for (int i = W - 2; i >= 0; --i) suf[i] = Op<T, SUP>::apply(suf[i + 1], raw[i]);
  }
}

// Diagonal segments of 1- and 2-byte pixels, E = 4 / sizeof(T) adjacent diagonals per thread.  Lane j
// of a warp follows the E diagonals through word u = c + j of row y0 (pixels E*u .. E*u + E - 1).  At
// row y = y0 + d they sit at pixel E*u + s, s = -d (45 degrees) or +d (135 degrees): inside word
// u + q, q = floor(s / E), shifted by m = s - q*E pixels -- the same q and m for the whole warp.  Each
// lane loads word u + q and funnel-shifts it with the next lane's word by m pixels.  Results go back
// the same way: the aligned word u + q holds the last m pixels of lane j - 1 and the first E - m of
// lane j.  Lane 31 only lends its word to lane 30 and lane 0 only its results to lane 1, so a warp
// writes the 30 words c + q + 1 .. c + q + 30 of a row, and consecutive warps are 30 words apart.
// Loads and stores stay whole aligned words; no thread leaves early (the shuffles need every lane).
template <typename T, bool SUP, int K, int DIR>
__global__ void __launch_bounds__(kLSThreads) k_dline_words(const uint32_t *__restrict__ in, uint32_t *__restrict__ out,
                                                           int H, int Wn, int strip, int u_first) {
  constexpr int W = 2 * K + 1;
  constexpr int LOG2E = sizeof(T) == 1 ? 2 : 1;
  constexpr int E = 1 << LOG2E;
  constexpr int PB = 8 * (int)sizeof(T);
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * kLSThreads + threadIdx.x) >> 5);
  const int u = u_first + warp * 30 + lane - 1;
  const bool writer = lane >= 1 && lane <= 30;
  const int y0 = blockIdx.y * strip;
  const int y1 = min(y0 + strip, H);
  const uint32_t NEUW = splat<T>(Op<T, SUP>::neutral());
  uint32_t suf[W];
#pragma unroll
  for (int i = 0; i < W; ++i) suf[i] = NEUW;
  const int ys = y0 - K;
  const int ylim = min(y1 + K, H);  // rows below only feed outputs below the strip
  for (int yb = ys; yb < y1 + K; yb += W) {
    uint32_t raw[W];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      const int y = yb + i;
      const int wi = u + ((DIR > 0 ? y0 - y : y - y0) >> LOG2E);
      raw[i] = (y >= 0 && y < ylim && wi >= 0 && wi < Wn) ? __ldg(in + (size_t)y * Wn + wi) : NEUW;
    }
#pragma unroll
    for (int i = 0; i < W; ++i) {
      const int m = (DIR > 0 ? y0 - (yb + i) : (yb + i) - y0) & (E - 1);
      const uint32_t hi = __shfl_down_sync(FULL, raw[i], 1);
      raw[i] = __funnelshift_r(raw[i], hi, (unsigned)(m * PB));
    }
    uint32_t pre = raw[0];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      if (i > 0) pre = wop<T, SUP>(pre, raw[i]);
      const int y = yb + i - K;
      const uint32_t r = (i < W - 1) ? wop<T, SUP>(suf[i + 1], pre) : pre;
      const int s = DIR > 0 ? y0 - y : y - y0;
      const int m = s & (E - 1);
      const uint32_t prev = __shfl_up_sync(FULL, r, 1);
      const uint32_t w = m ? __funnelshift_r(prev, r, (unsigned)((E - m) * PB)) : r;
      const int wi = u + (s >> LOG2E);
      if (writer && y >= y0 && y < y1 && wi >= 0 && wi < Wn) out[(size_t)y * Wn + wi] = w;
    }
    suf[W - 1] = raw[W - 1];
#pragma unroll
    for (int i = W - 2; i >= 0; --i) suf[i] = wop<T, SUP>(suf[i + 1], raw[i]);
  }
}

template <typename T, bool SUP, int K, int DIR>
static void dw_launch(const T *in, T *out, int H, int W, cudaStream_t s) {
  constexpr int E = 4 / (int)sizeof(T);
  const int Wn = W / E;
  // rows of the strip shift the words by q in [qlo, qhi]; the warps' 30-word spans must cover
  // every word of every row.  Strips of about 8K rows keep the 2K-row halo small (measured on
  // 4096^2: 256 rows for K = 31, 128 for 15, 64 for 3), shorter ones only for small images.
  int strip = 64;
  while (strip < 512 && strip < 8 * K) strip *= 2;
  auto span = [&](int st) { return (int64_t)(st - 1 + E - 1) / E + 1; };  // qhi - qlo + 1 (upper bound)
  auto ctas_x = [&](int st) { return ceil_div(ceil_div((int64_t)Wn + span(st), 30) * 32, kLSThreads); };
  while (strip > 32 && ctas_x(strip) * ceil_div(H, strip) < 2LL * num_sms()) strip /= 2;
  const int qext = (strip - 1 + E - 1) / E;  // |q| over the strip's rows is at most this
  const int u_first = DIR > 0 ? 0 : -qext;
  dim3 grid((unsigned)ctas_x(strip), (unsigned)ceil_div(H, strip));
  k_dline_words<T, SUP, K, DIR><<<grid, kLSThreads, 0, s>>>(reinterpret_cast<const uint32_t *>(in),
                                                           reinterpret_cast<uint32_t *>(out), H, Wn, strip, u_first);
}

template <typename T, bool SUP, int K, int DIR>
static void ds_launch(const T *in, T *out, int H, int W, cudaStream_t s) {
  // threads cover W + strip pixels of row y0: the band drifts left (45) or right (135) by one pixel
  // per row over the strip
  int strip = 256;
  auto ctas_x = [&](int st) { return ceil_div((int64_t)W + st, kLSThreads); };
  while (strip > 32 && ctas_x(strip) * ceil_div(H, strip) < 4LL * num_sms()) strip /= 2;
  const int x_first = DIR > 0 ? 0 : -strip;
  dim3 grid((unsigned)ctas_x(strip), (unsigned)ceil_div(H, strip));
  k_dline_stream<T, SUP, K, DIR><<<grid, kLSThreads, 0, s>>>(in, out, H, W, strip, x_first);
}

template <typename T, bool SUP, int K>
static void vs_launch(const T *in, T *out, int H, int W, cudaStream_t s) {
  constexpr int E = 4 / (int)sizeof(T);
  const int Wn = W / E;
  // strips of rows: enough threads to fill the GPU, strips long relative to the 2K halo
  const int64_t cols_blocks = ceil_div(Wn, kLSThreads);
  int strip = 256;
  while (strip > 64 && cols_blocks * ceil_div(H, strip) < 4LL * num_sms()) strip /= 2;
  dim3 grid((unsigned)cols_blocks, (unsigned)ceil_div(H, strip));
  k_vline_stream<T, SUP, K><<<grid, kLSThreads, 0, s>>>(reinterpret_cast<const uint32_t *>(in),
                                                       reinterpret_cast<uint32_t *>(out), H, Wn, strip);
}

template <typename T, bool SUP, int K>
static void line_launch(const T *in, T *out, int H, int W, int dx, cudaStream_t s) {
  if (dx == 0) vs_launch<T, SUP, K>(in, out, H, W, s);
  else if constexpr (sizeof(T) < 4) {
    if (dx == -1) dw_launch<T, SUP, K, 1>(in, out, H, W, s);
    else dw_launch<T, SUP, K, -1>(in, out, H, W, s);
  } else if (dx == -1) ds_launch<T, SUP, K, 1>(in, out, H, W, s);
  else ds_launch<T, SUP, K, -1>(in, out, H, W, s);
}

template <typename T, bool SUP>
static bool vs_dispatch(const T *in, T *out, int H, int W, int dx, int k, cudaStream_t s) {
  switch (k) {
    case 1: line_launch<T, SUP, 1>(in, out, H, W, dx, s); return true;
    case 2: line_launch<T, SUP, 2>(in, out, H, W, dx, s); return true;
    case 3: line_launch<T, SUP, 3>(in, out, H, W, dx, s); return true;
    case 7: line_launch<T, SUP, 7>(in, out, H, W, dx, s); return true;
    case 15: line_launch<T, SUP, 15>(in, out, H, W, dx, s); return true;
    case 31: line_launch<T, SUP, 31>(in, out, H, W, dx, s); return true;
    default: return false;
  }
}

// Fast path of launch_line for Y and diagonal segments; false when the image or half length does
// not qualify.
bool try_line_stream(const pg_image &in, const pg_image &out, int dy, int dx, int k, bool dilate, cudaStream_t s,
                     pg_status *st) {
  const int es = elem_size(in.ptype);
  if (es > 4 || dy != 1 || dx < -1 || dx > 1) return false;
  const Dims d = dims_of(in);
  const int64_t H = d.ny, W = d.nx;
  if (H < 1 || H > (1 << 30) || W > (1 << 29) || ceil_div(H, 32) > 65535) return false;
  // the vertical kernel and the 1-/2-byte diagonal kernel move whole 32-bit words; the 4-byte
  // diagonal one single pixels
  // u8 diagonals of 63 pixels: the word kernel's register window (196 registers) leaves too few
  // warps; the staircase tiles of line_w.cu measured faster there (54 vs 68 us on 4096^2)
  if (dx != 0 && es == 1 && k > 15) return false;
  if ((W * es) % 4 != 0) return false;
  if ((reinterpret_cast<uintptr_t>(in.data) | reinterpret_cast<uintptr_t>(out.data)) % 4 != 0) return false;
  bool ok = false;
  switch (in.ptype) {
    case PG_PTYPE_U8: {
      using T = uint8_t;
      ok = dilate ? vs_dispatch<T, true>((const T *)in.data, (T *)out.data, (int)H, (int)W, dx, k, s)
                  : vs_dispatch<T, false>((const T *)in.data, (T *)out.data, (int)H, (int)W, dx, k, s);
      break;
    }
    case PG_PTYPE_U16: {
      using T = uint16_t;
      ok = dilate ? vs_dispatch<T, true>((const T *)in.data, (T *)out.data, (int)H, (int)W, dx, k, s)
                  : vs_dispatch<T, false>((const T *)in.data, (T *)out.data, (int)H, (int)W, dx, k, s);
      break;
    }
    case PG_PTYPE_I32: {
      using T = int32_t;
      ok = dilate ? vs_dispatch<T, true>((const T *)in.data, (T *)out.data, (int)H, (int)W, dx, k, s)
                  : vs_dispatch<T, false>((const T *)in.data, (T *)out.data, (int)H, (int)W, dx, k, s);
      break;
    }
    case PG_PTYPE_F32: {
      using T = float;
      ok = dilate ? vs_dispatch<T, true>((const T *)in.data, (T *)out.data, (int)H, (int)W, dx, k, s)
                  : vs_dispatch<T, false>((const T *)in.data, (T *)out.data, (int)H, (int)W, dx, k, s);
      break;
    }
    default: return false;
  }
  if (ok) *st = cuda_status(cudaGetLastError(), "streaming line kernel launch");
  return ok;
}

}  // namespace pg
