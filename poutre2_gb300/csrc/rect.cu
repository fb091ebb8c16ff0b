// rect.cu -- erosion / dilation by the (2KY+1) x (2KX+1) box in one pass through shared memory: the
// square (KY = KX), the X segment (KY = 0) and the Y segment (KX = 0), for K = 7, 15, 31; 2- and 4-byte
// pixels, and 1-byte pixels for the Y segment.
//
// Same result as the separable line passes of line.cu (DilateX then DilateY over a clipped window;
// the box is the Minkowski sum of an X and a Y segment, so the order is immaterial): one tile is read
// once and written once instead of the two round trips of the separable form, and one TMA copy per
// tile keeps a whole tile's loads in flight where the streaming kernels are limited by latency.
//
// A CTA (128 threads) owns an output tile of TH = 128 - 2KY rows by TW = 64 or 32 centre 32-bit words
// (E = 4 / sizeof(T) pixels per word).  One TMA copy (cp.async.bulk.tensor.2d, completion on an
// mbarrier) brings the 128 input rows of the tile plus HW halo words each side into shared memory;
// pixels outside the image are then set to the neutral value.  Row pass: thread r runs van Herk /
// Gil-Werman along input row r, in registers, reading the row in 16-byte chunks and writing the
// X-dilated centre words back in place in 16-byte chunks (the row pitch is an odd number of chunks,
// so the 8 threads of a shared-memory phase touch 8 distinct chunks).  Column pass: the 128 threads
// split into 128 / TW row groups of TW centre columns; each runs the same scan down its column over
// its group's rows (SIMD within the word: 2 x u16 or 4 x u8 min/max) and writes the output rows
// straight to global memory, a warp covering 32 consecutive words of a row (for KY = 0 the centre
// words are copied out; for KX = 0 there is no row pass).
//
// Gradient mode (GRAD): the same tile gives the dilation and the erosion at once -- the row pass keeps
// both running scans and writes the X-eroded centre words to a second shared array, the column pass
// scans both and stores dilation - erosion -- so the gradient costs one read and one write of the
// image.  Pixels outside the image then repeat the nearest image pixel instead of a neutral value (a
// clipped box window contains that pixel, so neither extremum changes).
//
// The wait on the mbarrier is bounded (tile::kWaitNs of %globaltimer); on expiry the CTA records
// PG_ERR_CUDA in g_rect_status (read by pg_check_device) and leaves its tile unwritten.
#include <atomic>

#include "tile.cuh"

namespace pg {

__device__ int g_rect_status = 0;

namespace {

using namespace tile;
constexpr int kRThreads = tile::kThreads;

template <typename T, int KY, int KX, bool GRAD> struct RectGeom {
  static constexpr int E = 4 / (int)sizeof(T);
  // centre words: 64, or 32 for KX = 31 (measured on 4096^2: the tile's shared memory sets the CTAs
  // per SM, and the row pass's share of halo work grows with KX)
  static constexpr int TW = KX >= 31 ? 32 : 64;
  static constexpr int HW = ((KX + E - 1) / E + 3) / 4 * 4;     // halo words per side, whole 16-byte chunks
  static constexpr int BW0 = TW + 2 * HW;
  static constexpr int BW = ((BW0 / 4) & 1) ? BW0 : BW0 + 4;    // row pitch: an odd number of 16-byte chunks
  static constexpr int TR = kRThreads;                          // input rows per tile
  static constexpr int TH = TR - 2 * KY;                        // output rows per tile
  static constexpr int NV = kRThreads / TW;                     // column-pass row groups
  static constexpr int THG = (TH + NV - 1) / NV;                // output rows per group
  // gradient with a row pass: the X-eroded centre words get their own rows (odd chunk count)
  static constexpr int MP = (GRAD && KX > 0) ? TW + 4 : 0;
  static constexpr size_t tile_bytes = (size_t)TR * BW * 4;
  static constexpr size_t smem = tile_bytes + (size_t)TR * MP * 4 + 16;  // + the mbarrier
  static_assert(BW <= 256 && TH > 0 && kRThreads % TW == 0, "tile geometry");
  static_assert(!GRAD || !(KY > 15 && KX > 0), "gradient: register window too large");
};

template <typename T, bool SUP, int KY, int KX, bool GRAD>
__global__ void __launch_bounds__(kRThreads, 1) k_rect_fused(const __grid_constant__ CUtensorMap tmap,
                                                          uint32_t *__restrict__ out, int H, int Wn) {
  using G = RectGeom<T, KY, KX, GRAD>;
  constexpr int E = G::E, HW = G::HW, BW = G::BW, TR = G::TR, TH = G::TH, TW = G::TW, THG = G::THG, MP = G::MP;
  using O = Op<T, SUP>;
  extern __shared__ __align__(128) uint32_t s_tile[];
  __shared__ int s_ok;
  uint32_t *s_min = s_tile + TR * BW;  // GRAD with a row pass: X-eroded centre words, [TR][MP]
  uint64_t *bar = reinterpret_cast<uint64_t *>(s_tile + TR * BW + TR * MP);
  const int t = threadIdx.x;
  const int wx0 = blockIdx.x * TW;         // first centre word
  const int y0 = blockIdx.y * TH;          // first output row
  const int tx = wx0 - HW, ty = y0 - KY;   // tile origin: word (a multiple of 4), row

  if (!load_tile(&tmap, s_tile, bar, (unsigned)G::tile_bytes, tx, ty, &g_rect_status, &s_ok)) return;

  // pixels outside the image (TMA fills them with zeros): the neutral value of the operator, or for
  // the gradient (two operators) the nearest image pixel -- a clipped box window always contains
  // that pixel, so repeating it changes neither the maximum nor the minimum
  if (tx < 0 || ty < 0 || tx + BW > Wn || ty + TR > H) {
    if constexpr (!GRAD) {
      const uint32_t NEUW = splat<T>(O::neutral());
      for (int r = 0; r < TR; ++r) {
        const bool row_out = ty + r < 0 || ty + r >= H;
        for (int c = t; c < BW; c += kRThreads)
          if (row_out || tx + c < 0 || tx + c >= Wn) s_tile[r * BW + c] = NEUW;
      }
    } else {
      for (int r = 0; r < TR; ++r) {
        if (ty + r < 0 || ty + r >= H) continue;
        const uint32_t lw = splat<T>(px_of<T>(s_tile[r * BW + max(-tx, 0)], 0));
        const uint32_t rw = splat<T>(px_of<T>(s_tile[r * BW + min(Wn - 1 - tx, BW - 1)], E - 1));
        for (int c = t; c < BW; c += kRThreads) {
          if (tx + c < 0) s_tile[r * BW + c] = lw;
          else if (tx + c >= Wn) s_tile[r * BW + c] = rw;
        }
      }
      __syncthreads();
      for (int r = 0; r < TR; ++r) {
        const int yr = ty + r;
        if (yr >= 0 && yr < H) continue;
        const int src = (yr < 0 ? 0 : H - 1) - ty;
        for (int c = t; c < BW; c += kRThreads) s_tile[r * BW + c] = s_tile[src * BW + c];
      }
    }
    __syncthreads();
  }

  // ---- row pass: thread t scans input row t
  if constexpr (KX > 0) {
    row_scan<T, SUP, KX, TW, HW, GRAD>(s_tile + t * BW, s_min + t * MP);
    __syncthreads();
  }

  // ---- column pass: thread t scans centre word column HW + t % TW over the rows of output group
  // t / TW (THG output rows, from tile row j0); output row j0 + j is formed at q = j + 2KY.  Without
  // a vertical extent the centre words are copied out.
  const int j0 = (t / TW) * THG;
  const uint32_t *col = s_tile + j0 * BW + HW + t % TW;
  constexpr int SB = KX > 0 ? MP : BW;
  const uint32_t *colb = (GRAD && KX > 0) ? s_min + j0 * MP + t % TW : col;
  const int gx = wx0 + t % TW;
  if constexpr (KY == 0) {
    if (gx < Wn)
#pragma unroll 4
      for (int j = 0; j < THG && j0 + j < TH && y0 + j0 + j < H; ++j) {
        uint32_t v = col[j * BW];
        if constexpr (GRAD) v = wdiff<T>(v, colb[j * SB]);
        out[(size_t)(y0 + j0 + j) * Wn + gx] = v;
      }
  } else {
    col_scan<T, SUP, KY, THG, TH, TR, BW, SB, GRAD>(col, colb, out, j0, y0, gx, H, Wn);
  }
}

template <typename T, bool SUP, int KY, int KX, bool GRAD>
pg_status rect_fused(const pg_image &in, const pg_image &out, cudaStream_t s) {
  using G = RectGeom<T, KY, KX, GRAD>;
  const Dims d = dims_of(in);
  const int64_t H = d.ny, Wn = d.nx / G::E;
  CUtensorMap map;
  PG_TRY(word_map(&map, in.data, H, Wn, G::BW, G::TR));
  // the opt-in shared-memory size is a per-device attribute of each instantiation
  static std::atomic<uint64_t> attr_devices{0};
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  const uint64_t bit = 1ull << (dev & 63);
  if (!(attr_devices.load() & bit)) {
    PG_CUDA_TRY(cudaFuncSetAttribute(k_rect_fused<T, SUP, KY, KX, GRAD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)G::smem),
                "tile kernel smem attribute");
    attr_devices.fetch_or(bit);
  }
  const dim3 grid((unsigned)ceil_div(Wn, G::TW), (unsigned)ceil_div(H, G::TH));
  k_rect_fused<T, SUP, KY, KX, GRAD><<<grid, kRThreads, G::smem, s>>>(map, static_cast<uint32_t *>(out.data), (int)H,
                                                                     (int)Wn);
  return cuda_status(cudaGetLastError(), "tile erosion / dilation launch");
}

// (hy, hx): (k, k) square, (0, k) X segment, (k, 0) Y segment, k in {7, 15, 31}
template <typename T, bool SUP>
pg_status rect_fused_k(const pg_image &in, const pg_image &out, int hy, int hx, cudaStream_t s) {
  if (hy == hx) {
    switch (hy) {
      case 7: return rect_fused<T, SUP, 7, 7, false>(in, out, s);
      case 15: return rect_fused<T, SUP, 15, 15, false>(in, out, s);
      default: return rect_fused<T, SUP, 31, 31, false>(in, out, s);
    }
  }
  if (hy == 0) {
    switch (hx) {
      case 7: return rect_fused<T, SUP, 0, 7, false>(in, out, s);
      case 15: return rect_fused<T, SUP, 0, 15, false>(in, out, s);
      default: return rect_fused<T, SUP, 0, 31, false>(in, out, s);
    }
  }
  switch (hy) {
    case 7: return rect_fused<T, SUP, 7, 0, false>(in, out, s);
    case 15: return rect_fused<T, SUP, 15, 0, false>(in, out, s);
    default: return rect_fused<T, SUP, 31, 0, false>(in, out, s);
  }
}

// the gradient (dilation - erosion) in one pass; not for the 63 x 63 square
template <typename T>
pg_status rect_grad_k(const pg_image &in, const pg_image &out, int hy, int hx, cudaStream_t s) {
  if (hy == hx) return hy == 7 ? rect_fused<T, true, 7, 7, true>(in, out, s) : rect_fused<T, true, 15, 15, true>(in, out, s);
  if (hy == 0) {
    switch (hx) {
      case 7: return rect_fused<T, true, 0, 7, true>(in, out, s);
      case 15: return rect_fused<T, true, 0, 15, true>(in, out, s);
      default: return rect_fused<T, true, 0, 31, true>(in, out, s);
    }
  }
  switch (hy) {
    case 7: return rect_fused<T, true, 7, 0, true>(in, out, s);
    case 15: return rect_fused<T, true, 15, 0, true>(in, out, s);
    default: return rect_fused<T, true, 31, 0, true>(in, out, s);
  }
}

}  // namespace

bool rect_fused_ok(const pg_image &in, const pg_image &out, int64_t hy, int64_t hx, bool grad) {
  auto ok_k = [](int64_t k) { return k == 7 || k == 15 || k == 31; };
  if (in.rank != 2 || !((hy == hx && ok_k(hy)) || (hy == 0 && ok_k(hx)) || (hx == 0 && ok_k(hy)))) return false;
  if (grad && hy == 31 && hx == 31) return false;
  const int es = elem_size(in.ptype);
  // 2- and 4-byte pixels; u8 only without a row pass (its register window of single pixels spills:
  // the line passes run instead)
  if (es != 2 && es != 4 && !(es == 1 && hx == 0)) return false;
  const Dims d = dims_of(in);
  const int64_t H = d.ny, Wd = d.nx;
  if (H < 1 || Wd < 1 || (Wd * es) % 16 != 0) return false;
  if ((reinterpret_cast<uintptr_t>(in.data) | reinterpret_cast<uintptr_t>(out.data)) % 16 != 0) return false;
  if (H > (1 << 30) || Wd * es / 4 > (1 << 30) || ceil_div(H, kRThreads - 2 * hy) > 65535) return false;
  return in.ptype == PG_PTYPE_U8 || in.ptype == PG_PTYPE_U16 || in.ptype == PG_PTYPE_I32 || in.ptype == PG_PTYPE_F32;
}

// u8: Y segments only (no row pass)
template <bool SUP, bool GRAD>
pg_status rect_fused_u8_y(const pg_image &in, const pg_image &out, int hy, cudaStream_t s) {
  switch (hy) {
    case 7: return rect_fused<uint8_t, SUP, 7, 0, GRAD>(in, out, s);
    case 15: return rect_fused<uint8_t, SUP, 15, 0, GRAD>(in, out, s);
    default: return rect_fused<uint8_t, SUP, 31, 0, GRAD>(in, out, s);
  }
}

bool try_rect_fused(const pg_image &in, const pg_image &out, int64_t hy, int64_t hx, bool dilate, cudaStream_t s,
                    pg_status *st) {
  if (!rect_fused_ok(in, out, hy, hx, false)) return false;
  const int y = (int)hy, x = (int)hx;
  switch (in.ptype) {
    case PG_PTYPE_U8:
      *st = dilate ? rect_fused_u8_y<true, false>(in, out, y, s) : rect_fused_u8_y<false, false>(in, out, y, s);
      return true;
    case PG_PTYPE_U16:
      *st = dilate ? rect_fused_k<uint16_t, true>(in, out, y, x, s) : rect_fused_k<uint16_t, false>(in, out, y, x, s);
      return true;
    case PG_PTYPE_I32:
      *st = dilate ? rect_fused_k<int32_t, true>(in, out, y, x, s) : rect_fused_k<int32_t, false>(in, out, y, x, s);
      return true;
    case PG_PTYPE_F32:
      *st = dilate ? rect_fused_k<float, true>(in, out, y, x, s) : rect_fused_k<float, false>(in, out, y, x, s);
      return true;
    default: return false;
  }
}

bool try_rect_gradient(const pg_image &in, const pg_image &out, int64_t hy, int64_t hx, cudaStream_t s, pg_status *st) {
  if (!rect_fused_ok(in, out, hy, hx, true)) return false;
  const int y = (int)hy, x = (int)hx;
  switch (in.ptype) {
    case PG_PTYPE_U8: *st = rect_fused_u8_y<true, true>(in, out, y, s); return true;
    case PG_PTYPE_U16: *st = rect_grad_k<uint16_t>(in, out, y, x, s); return true;
    case PG_PTYPE_I32: *st = rect_grad_k<int32_t>(in, out, y, x, s); return true;
    case PG_PTYPE_F32: *st = rect_grad_k<float>(in, out, y, x, s); return true;
    default: return false;
  }
}

int take_rect_status() {
  int st = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&st, g_rect_status, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  if (st != 0 && cudaMemcpyToSymbol(g_rect_status, &zero, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  return st;
}

}  // namespace pg
