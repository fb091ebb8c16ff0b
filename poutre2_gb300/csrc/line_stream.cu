// line_stream.cu -- register-streaming vertical segments (van Herk / Gil-Werman in registers).
//
// Same result as line.cu / line_w.cu for the Y segment of 2K+1 pixels (DilateY/ErodeY,
// ero_dil_line_se_t.hpp:249-282; clipped window).  Used for the half lengths instantiated
// below, 1/2/4-byte pixels, word-aligned rows.
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
  // blocks start at ys = y0 - K; block b covers rows [ys + b*W, ys + (b+1)*W)
  const int ys = y0 - K;
  for (int yb = ys; yb < y1 + K; yb += W) {
    uint32_t raw[W];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      const int y = yb + i;
      raw[i] = (y >= 0 && y < H) ? __ldg(src + (size_t)y * Wn) : NEUW;
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

template <typename T, bool SUP>
static bool vs_dispatch(const T *in, T *out, int H, int W, int k, cudaStream_t s) {
  switch (k) {
    case 1: vs_launch<T, SUP, 1>(in, out, H, W, s); return true;
    case 2: vs_launch<T, SUP, 2>(in, out, H, W, s); return true;
    case 3: vs_launch<T, SUP, 3>(in, out, H, W, s); return true;
    case 7: vs_launch<T, SUP, 7>(in, out, H, W, s); return true;
    case 15: vs_launch<T, SUP, 15>(in, out, H, W, s); return true;
    case 31: vs_launch<T, SUP, 31>(in, out, H, W, s); return true;
    default: return false;
  }
}

// Fast path of launch_line for Y segments; false when the image or half length does not qualify.
bool try_line_stream(const pg_image &in, const pg_image &out, int dy, int dx, int k, bool dilate, cudaStream_t s,
                     pg_status *st) {
  const int es = elem_size(in.ptype);
  if (es > 4 || dx != 0 || dy != 1) return false;
  const Dims d = dims_of(in);
  const int64_t H = d.ny, W = d.nx;
  if (H < 1 || H > (1 << 30) || W > (1 << 30) || ceil_div(H, 64) > 65535) return false;
  if ((W * es) % 4 != 0) return false;
  if ((reinterpret_cast<uintptr_t>(in.data) | reinterpret_cast<uintptr_t>(out.data)) % 4 != 0) return false;
  bool ok = false;
  switch (in.ptype) {
    case PG_PTYPE_U8: {
      using T = uint8_t;
      ok = dilate ? vs_dispatch<T, true>((const T *)in.data, (T *)out.data, (int)H, (int)W, k, s)
                  : vs_dispatch<T, false>((const T *)in.data, (T *)out.data, (int)H, (int)W, k, s);
      break;
    }
    case PG_PTYPE_U16: {
      using T = uint16_t;
      ok = dilate ? vs_dispatch<T, true>((const T *)in.data, (T *)out.data, (int)H, (int)W, k, s)
                  : vs_dispatch<T, false>((const T *)in.data, (T *)out.data, (int)H, (int)W, k, s);
      break;
    }
    case PG_PTYPE_I32: {
      using T = int32_t;
      ok = dilate ? vs_dispatch<T, true>((const T *)in.data, (T *)out.data, (int)H, (int)W, k, s)
                  : vs_dispatch<T, false>((const T *)in.data, (T *)out.data, (int)H, (int)W, k, s);
      break;
    }
    case PG_PTYPE_F32: {
      using T = float;
      ok = dilate ? vs_dispatch<T, true>((const T *)in.data, (T *)out.data, (int)H, (int)W, k, s)
                  : vs_dispatch<T, false>((const T *)in.data, (T *)out.data, (int)H, (int)W, k, s);
      break;
    }
    default: return false;
  }
  if (ok) *st = cuda_status(cudaGetLastError(), "streaming line kernel launch");
  return ok;
}

}  // namespace pg
