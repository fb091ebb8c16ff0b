// octagon.cu -- the octagon's sequence of 3x3 passes (crosses, then squares) of size n <= 16 in one
// launch, through shared memory, on 1- and 2-byte pixels with rows of a multiple of 16 bytes.
//
// Same result as t_DilateOctagon / t_ErodeOctagon (ero_dil_compound_static_se_t.hpp:34-160): n passes,
// the first n - round(n / (1 + sqrt 2)) by the 3x3 cross and the rest by the 3x3 square, each clipped
// at the image border (pixels outside the image are the operator's neutral value).
//
// The passes run on 16-bit lanes, two pixels a word (u8 images are widened on the way in and narrowed
// on the way out).  A CTA (256 threads) owns an output tile of TWO = 64 - 2*HW lane words by 128 - 2n
// rows.  One TMA copy brings the 64-lane-word x 128-row box around it (HW words and n rows of halo)
// into shared memory; the n passes then ping-pong between two 32 KB buffers, every pass recomputing
// the whole box except its outermost words and rows.  Those keep stale values, and a wrong value moves
// one pixel per pass, so after n passes the centre -- 2*HW >= n pixels and n rows from the edges -- is
// exact.  A pass is word-parallel: lanes take consecutive words of a row (conflict-free shared-memory
// loads), the left / right neighbour of each packed pixel comes from one funnel shift with the
// neighbouring word, and min / max run on both pixels of a word at once (u16x2 SIMD).  Each
// thread slides down its column over a quarter of the rows, holding the rows above and below in registers.
// In tiles that touch the image border, every pass writes the neutral value at the pixels outside
// the image, as the clipped passes read them.  The TMA wait is bounded (tile::kWaitNs); on expiry the
// CTA records PG_ERR_CUDA in g_oct_status (read by pg_check_device) and leaves its tile unwritten.
#include <atomic>

#include "tile.cuh"

namespace pg {

__device__ int g_oct_status = 0;

namespace {

using namespace tile;
constexpr int kOThreads = 256;
constexpr int kOW = 64;    // box width, words (two warps of columns)
constexpr int kOR = 128;   // box rows
constexpr int kOBands = kOThreads / kOW;  // rows 1 .. kOR - 2 are recomputed, in four bands

// T: the image's pixels; the passes run on 16-bit lanes (u8 pixels are widened on the way in and
// narrowed on the way out: min / max of u8x4 words has no single instruction, of u16x2 words it has).
// HW: halo, in 16-bit-lane words (HW * 2 >= n pixels).
template <typename T, bool SUP, int HW>
__global__ void __launch_bounds__(kOThreads) k_octagon(const __grid_constant__ CUtensorMap tmap, uint32_t *__restrict__ out,
                                                       int H, int Wn, int n_cross, int n_square) {
  using L = uint16_t;
  constexpr int TWO = kOW - 2 * HW;                // output words (16-bit lanes) per row
  constexpr int EW = 4 / (int)sizeof(T) / 2;       // lane words per image word: u8 2, u16 1
  extern __shared__ __align__(128) uint32_t s_buf[];  // [2][kOR][kOW] words + the mbarrier
  __shared__ int s_ok;
  uint64_t *bar = reinterpret_cast<uint64_t *>(s_buf + 2 * kOR * kOW);
  const int n = n_cross + n_square;
  const int tho = kOR - 2 * n;                     // output rows
  const int tx = (int)blockIdx.x * TWO - HW;       // box origin, in lane words (image words: tx / EW)
  const int ty = (int)blockIdx.y * tho - n;
  const int Wl = Wn * EW;                          // image row, in lane words
  const uint32_t NEUW = splat<L>((L)Op<T, SUP>::neutral());

  // u16: the box lands in buffer 0; u8: in buffer 1 (as kOW / 2 words per row), widened below
  uint32_t *land = s_buf + (EW == 2 ? kOR * kOW : 0);
  if (!load_tile(&tmap, land, bar, (unsigned)(kOR * kOW / EW * 4), tx / EW, ty, &g_oct_status, &s_ok)) return;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int c = (warp & 1) * 32 + lane;            // this thread's word column
  const int band = warp >> 1;
  const int r0 = 1 + band * (kOR - 2) / kOBands, r1 = 1 + (band + 1) * (kOR - 2) / kOBands;  // rows of each pass
  const int cl = c > 0 ? c - 1 : c, cr = c < kOW - 1 ? c + 1 : c;
  // whether this column and the box meet the image (an image word is wholly inside or outside)
  const bool border = tx < 0 || tx + kOW > Wl || ty < 0 || ty + kOR > H;
  const uint32_t cmask = (tx + c >= 0 && tx + c < Wl) ? 0xffffffffu : 0u;
  auto masked = [&](uint32_t w, int r) {
    const int gy = ty + r;
    return (gy >= 0 && gy < H) ? ((w & cmask) | (NEUW & ~cmask)) : NEUW;
  };

  if constexpr (EW == 2) {
    // widen: lane word c holds image pixels 2c, 2c + 1 of the box row as u16
    for (int r = band; r < kOR; r += kOBands) {
      const uint32_t w8 = land[r * (kOW / 2) + c / 2];
      uint32_t w = __byte_perm(w8, 0u, (c & 1) ? 0x4342 : 0x4140);
      if (border) w = masked(w, r);
      s_buf[r * kOW + c] = w;
    }
    __syncthreads();
  } else if (border) {
    // TMA filled the outside of the image with zeros: the first pass reads the neutral value there
    for (int r = band; r < kOR; r += kOBands) s_buf[r * kOW + c] = masked(s_buf[r * kOW + c], r);
    __syncthreads();
  }

  for (int p = 0; p < n; ++p) {
    const uint32_t *src = s_buf + (p & 1) * (kOR * kOW);
    uint32_t *dst = s_buf + ((p + 1) & 1) * (kOR * kOW);
    auto hmax = [&](const uint32_t *row) {  // max / min of each pixel with its left and right neighbours
      const uint32_t w = row[c];
      const uint32_t l = __funnelshift_l(row[cl], w, 16), rr = __funnelshift_r(w, row[cr], 16);
      return wop<L, SUP>(w, wop<L, SUP>(l, rr));
    };
    if (p < n_cross) {
      // cross: centre, up, down, left, right
      uint32_t up = src[(r0 - 1) * kOW + c], cc = src[r0 * kOW + c];
      uint32_t hc = hmax(src + r0 * kOW);
#pragma unroll 4
      for (int r = r0; r < r1; ++r) {
        const uint32_t dn = src[(r + 1) * kOW + c];
        uint32_t v = wop<L, SUP>(hc, wop<L, SUP>(up, dn));
        if (border) v = masked(v, r);
        dst[r * kOW + c] = v;
        up = cc;
        cc = dn;
        hc = hmax(src + (r + 1) * kOW);
      }
    } else {
      // square: the horizontal 3-pixel extremum of three rows
      uint32_t ha = hmax(src + (r0 - 1) * kOW), hb = hmax(src + r0 * kOW);
#pragma unroll 4
      for (int r = r0; r < r1; ++r) {
        const uint32_t hn = hmax(src + (r + 1) * kOW);
        uint32_t v = wop<L, SUP>(hb, wop<L, SUP>(ha, hn));
        if (border) v = masked(v, r);
        dst[r * kOW + c] = v;
        ha = hb;
        hb = hn;
      }
    }
    __syncthreads();
  }

  // the exact centre: rows n .. n + tho - 1, lane words HW .. HW + TWO - 1 (u8: narrowed in pairs)
  const uint32_t *fin = s_buf + (n & 1) * (kOR * kOW);
  if (c % EW == 0 && c >= HW && c < HW + TWO && tx + c < Wl) {
    const int gx = (tx + c) / EW;
    for (int r = n + band; r < n + tho; r += kOBands) {
      const int gy = ty + r;
      if (gy >= H) break;
      uint32_t w = fin[r * kOW + c];
      if constexpr (EW == 2) w = __byte_perm(w, fin[r * kOW + c + 1], 0x6420);
      out[(size_t)gy * Wn + gx] = w;
    }
  }
}

template <typename T, bool SUP, int HW>
pg_status octagon_launch(const pg_image &in, const pg_image &out, int n_cross, int n_square, cudaStream_t s) {
  constexpr int EW = 4 / (int)sizeof(T) / 2;
  const Dims d = dims_of(in);
  const int64_t H = d.ny, Wn = d.nx * (int64_t)sizeof(T) / 4;
  CUtensorMap map;
  PG_TRY(word_map(&map, in.data, H, Wn, kOW / EW, kOR));
  constexpr size_t smem = (size_t)2 * kOR * kOW * 4 + 16;
  static std::atomic<uint64_t> attr_devices{0};
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  const uint64_t bit = 1ull << (dev & 63);
  if (!(attr_devices.load() & bit)) {
    PG_CUDA_TRY(cudaFuncSetAttribute(k_octagon<T, SUP, HW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                "octagon smem attribute");
    attr_devices.fetch_or(bit);
  }
  const int n = n_cross + n_square;
  const dim3 grid((unsigned)ceil_div(Wn * EW, kOW - 2 * HW), (unsigned)ceil_div(H, kOR - 2 * n));
  k_octagon<T, SUP, HW><<<grid, kOThreads, smem, s>>>(map, static_cast<uint32_t *>(out.data), (int)H, (int)Wn, n_cross,
                                                      n_square);
  return cuda_status(cudaGetLastError(), "octagon tile launch");
}

}  // namespace

bool try_octagon_tile(const pg_image &in, const pg_image &out, int n_cross, int n_square, bool dilate, cudaStream_t s,
                      pg_status *st) {
  const int n = n_cross + n_square;
  if (in.rank != 2 || n < 2 || n > 16 || n_cross < 1 || n_square < 0) return false;
  const int es = elem_size(in.ptype);
  if (!(in.ptype == PG_PTYPE_U8 || in.ptype == PG_PTYPE_U16)) return false;
  // fewer passes run faster one launch each (4096^2, dilation by the iterated cross: u8 2 passes 24.6
  // against 34.8 us in the tile, 5 passes 61.5 against 57.3; u16 2 passes 28.6 against 28.7)
  if (n < (es == 1 ? 5 : 3)) return false;
  const Dims d = dims_of(in);
  const int64_t H = d.ny, W = d.nx;
  if (H < 1 || W < 1 || (W * es) % 16 != 0) return false;
  if ((reinterpret_cast<uintptr_t>(in.data) | reinterpret_cast<uintptr_t>(out.data)) % 16 != 0) return false;
  if (H > (1 << 30) || W * es / 4 > (1 << 30) || ceil_div(H, kOR - 2 * n) > 65535) return false;
  // halo lane words: 2 * HW pixels >= n (u8: HW / 2 image words, a multiple of 4 for the tensor map)
  if (in.ptype == PG_PTYPE_U8) {
    *st = dilate ? octagon_launch<uint8_t, true, 8>(in, out, n_cross, n_square, s)
                 : octagon_launch<uint8_t, false, 8>(in, out, n_cross, n_square, s);
  } else if (n <= 8) {
    *st = dilate ? octagon_launch<uint16_t, true, 4>(in, out, n_cross, n_square, s)
                 : octagon_launch<uint16_t, false, 4>(in, out, n_cross, n_square, s);
  } else {
    *st = dilate ? octagon_launch<uint16_t, true, 8>(in, out, n_cross, n_square, s)
                 : octagon_launch<uint16_t, false, 8>(in, out, n_cross, n_square, s);
  }
  return true;
}

int take_oct_status() {
  int st = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&st, g_oct_status, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  if (st != 0 && cudaMemcpyToSymbol(g_oct_status, &zero, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  return st;
}

}  // namespace pg
