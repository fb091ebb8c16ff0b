// rect_open.cu -- opening and closing by an X segment (KX = 7, 15, 31) in one pass through shared
// memory, where the tile keeps four CTAs per SM (2-byte pixels; 4-byte pixels at KX = 7).  The kernel
// is written for any box (KY > 0 adds the column passes); squares and Y segments measured slower
// than two single passes and are not instantiated.
//
// Same result as the two passes of the composite (Opening = Dilate(Erode(f)), Closing =
// Erode(Dilate(f)), each over the clipped window, src/low_level_morpho/ero_dil.cpp): the first
// operator's result is only defined inside the image, so it is formed for the tile and the second
// operator's halo, pixels outside the image are then reset to the second operator's neutral value, and
// the second operator runs on it.  One read and one write of the image instead of two of each.
//
// A CTA of 128 threads owns TH = 128 - 4KY output rows by TW = 64 (32 for KX = 31) centre words.  One
// TMA copy brings the 128 input rows with HW2 halo words each side (2KX pixels and more).  First
// operator: row pass over the centre plus HW1 words each side (the second operator's horizontal halo),
// in place; column pass over those columns, in place, giving rows [KY, 128 - KY).  Second operator: row
// pass over the centre, in place; column pass over rows [KY, 128 - KY) storing the output rows to
// global memory (tile::row_scan / tile::col_scan; the in-place column helper is below).
#include <atomic>

#include "tile.cuh"

namespace pg {

__device__ int g_open_status = 0;

namespace {

using namespace tile;

template <typename T, int KY, int KX> struct OpenGeom {
  static constexpr int E = 4 / (int)sizeof(T);
  static constexpr int TW = KX >= 31 ? 32 : 64;                 // centre words
  static constexpr int HW1 = ((KX + E - 1) / E + 3) / 4 * 4;     // second operator's halo words per side
  static constexpr int HW2 = ((2 * KX + E - 1) / E + 3) / 4 * 4; // tile halo words per side
  static constexpr int NC1 = TW + 2 * HW1;                       // columns of the first operator's result
  static constexpr int BW0 = TW + 2 * HW2;
  static constexpr int BW = ((BW0 / 4) & 1) ? BW0 : BW0 + 4;     // row pitch: an odd number of 16-byte chunks
  static constexpr int TR = kThreads;                            // input rows per tile
  static constexpr int TH = TR - 4 * KY;                         // output rows per tile
  static constexpr int NV = kThreads / TW;                       // final column-pass row groups
  static constexpr int THG = (TH + NV - 1) / NV;
  static constexpr size_t tile_bytes = (size_t)TR * BW * 4;
  static constexpr size_t smem = tile_bytes + 16;
  static_assert(BW <= 256 && TH > 0 && kThreads % TW == 0, "tile geometry");
  static_assert((HW2 - HW1) * E >= KX, "the first row pass needs KX pixels left of its outputs");
  static_assert(HW1 + (KX + E - 1) / E <= HW2, "and KX pixels right of them inside the tile");
  static_assert(NC1 <= kThreads || KY == 0, "one thread per first-operator column");
};

// Column of NR words (stride `stride`), in place: the result for window rows j .. j + 2K is stored
// at row j + K, for j in [0, NR - 2K).  Every row is read (into registers) before any row at or
// below it is written.
template <typename T, bool SUP, int K, int NR>
__device__ __forceinline__ void col_inplace(uint32_t *col, int stride) {
  constexpr int W = 2 * K + 1, NB = (NR + W - 1) / W;
  const uint32_t NEUW = splat<T>(Op<T, SUP>::neutral());
  uint32_t suf[W];
#pragma unroll
  for (int i = 0; i < W; ++i) suf[i] = NEUW;
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    uint32_t raw[W];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      const int q = b * W + i;
      raw[i] = q < NR ? col[q * stride] : NEUW;
    }
    uint32_t pre = raw[0];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      if (i > 0) pre = wop<T, SUP>(pre, raw[i]);
      const int j = b * W + i - 2 * K;
      if (j >= 0 && j < NR - 2 * K) col[(j + K) * stride] = (i < W - 1) ? wop<T, SUP>(suf[i + 1], pre) : pre;
    }
    suf[W - 1] = raw[W - 1];
#pragma unroll
    for (int i = W - 2; i >= 0; --i) suf[i] = wop<T, SUP>(suf[i + 1], raw[i]);
  }
}

// pixels of the tile outside the image := v
template <int TR, int BW>
__device__ __forceinline__ void fill_outside(uint32_t *s, int tx, int ty, int H, int Wn, uint32_t v) {
  for (int r = 0; r < TR; ++r) {
    const bool row_out = ty + r < 0 || ty + r >= H;
    for (int c = threadIdx.x; c < BW; c += kThreads)
      if (row_out || tx + c < 0 || tx + c >= Wn) s[r * BW + c] = v;
  }
}

template <typename T, bool OPEN, int KY, int KX>
__global__ void __launch_bounds__(kThreads, 1) k_rect_open(const __grid_constant__ CUtensorMap tmap,
                                                        uint32_t *__restrict__ out, int H, int Wn) {
  using G = OpenGeom<T, KY, KX>;
  constexpr int HW1 = G::HW1, HW2 = G::HW2, BW = G::BW, TR = G::TR, TH = G::TH, TW = G::TW, THG = G::THG;
  constexpr bool FSUP = !OPEN, SSUP = OPEN;  // opening: erosion then dilation
  extern __shared__ __align__(128) uint32_t s_tile[];
  __shared__ int s_ok;
  uint64_t *bar = reinterpret_cast<uint64_t *>(s_tile + TR * BW);
  const int t = threadIdx.x;
  const int wx0 = blockIdx.x * TW;         // first centre word
  const int y0 = blockIdx.y * TH;          // first output row
  const int tx = wx0 - HW2, ty = y0 - 2 * KY;
  if (!load_tile(&tmap, s_tile, bar, (unsigned)G::tile_bytes, tx, ty, &g_open_status, &s_ok)) return;
  const bool edge = tx < 0 || ty < 0 || tx + BW > Wn || ty + TR > H;
  if (edge) {
    fill_outside<TR, BW>(s_tile, tx, ty, H, Wn, splat<T>(Op<T, FSUP>::neutral()));
    __syncthreads();
  }
  // first operator over the centre and the second operator's halo
  if constexpr (KX > 0) {
    row_scan<T, FSUP, KX, G::NC1, HW2 - HW1, false>(s_tile + t * BW, nullptr);
    __syncthreads();
  }
  if constexpr (KY > 0) {
    if (t < G::NC1) col_inplace<T, FSUP, KY, TR>(s_tile + HW2 - HW1 + t, BW);
    __syncthreads();
  }
  // the first result exists only inside the image
  if (edge) {
    fill_outside<TR, BW>(s_tile, tx, ty, H, Wn, splat<T>(Op<T, SSUP>::neutral()));
    __syncthreads();
  }
  // second operator: rows [KY, TR - KY) hold the first result
  if constexpr (KX > 0) {
    row_scan<T, SSUP, KX, TW, HW2, false>(s_tile + t * BW, nullptr);
    __syncthreads();
  }
  const int j0 = (t / TW) * THG;
  const int gx = wx0 + t % TW;
  const uint32_t *col = s_tile + (KY + j0) * BW + HW2 + t % TW;
  if constexpr (KY == 0) {
    if (gx < Wn)
#pragma unroll 4
      for (int j = 0; j < THG && j0 + j < TH && y0 + j0 + j < H; ++j) out[(size_t)(y0 + j0 + j) * Wn + gx] = col[j * BW];
  } else {
    col_scan<T, SSUP, KY, THG, TH, TR - 2 * KY, BW, BW, false>(col, col, out, j0, y0, gx, H, Wn);
  }
}

template <typename T, bool OPEN, int KY, int KX>
pg_status rect_open(const pg_image &in, const pg_image &out, cudaStream_t s) {
  using G = OpenGeom<T, KY, KX>;
  const Dims d = dims_of(in);
  const int64_t H = d.ny, Wn = d.nx / G::E;
  CUtensorMap map;
  PG_TRY(word_map(&map, in.data, H, Wn, G::BW, G::TR));
  static std::atomic<uint64_t> attr_devices{0};  // per-device attribute of each instantiation
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  const uint64_t bit = 1ull << (dev & 63);
  if (!(attr_devices.load() & bit)) {
    PG_CUDA_TRY(cudaFuncSetAttribute(k_rect_open<T, OPEN, KY, KX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)G::smem),
                "opening kernel smem attribute");
    attr_devices.fetch_or(bit);
  }
  const dim3 grid((unsigned)ceil_div(Wn, G::TW), (unsigned)ceil_div(H, G::TH));
  k_rect_open<T, OPEN, KY, KX><<<grid, kThreads, G::smem, s>>>(map, static_cast<uint32_t *>(out.data), (int)H, (int)Wn);
  return cuda_status(cudaGetLastError(), "opening / closing tile launch");
}

template <typename T, bool OPEN>
pg_status rect_open_k(const pg_image &in, const pg_image &out, int hx, cudaStream_t s) {
  switch (hx) {
    case 7: return rect_open<T, OPEN, 0, 7>(in, out, s);
    case 15: return rect_open<T, OPEN, 0, 15>(in, out, s);
    default: return rect_open<T, OPEN, 0, 31>(in, out, s);
  }
}

// Tile shared memory of the X segment of half size hx for pixels of es bytes; the one-pass form runs
// where it keeps four CTAs per SM, like the single passes it replaces (measured on 4096^2: X 63 px u16
// opening 36.5 -> 29.3 us; with larger tiles (f32 at 31 and 63 px), and for squares and Y segments,
// whose 4K-row halo leaves 128 - 4K output rows of 128, the two passes were faster).
template <typename T> size_t open_smem(int hx) {
  return hx == 7 ? OpenGeom<T, 0, 7>::smem : hx == 15 ? OpenGeom<T, 0, 15>::smem : OpenGeom<T, 0, 31>::smem;
}

}  // namespace

bool try_rect_open(const pg_image &in, const pg_image &out, int64_t hy, int64_t hx, bool opening, cudaStream_t s,
                   pg_status *st) {
  if (in.rank != 2 || hy != 0 || !(hx == 7 || hx == 15 || hx == 31)) return false;
  const int es = elem_size(in.ptype);
  if (es != 2 && es != 4) return false;
  if ((es == 2 ? open_smem<uint16_t>((int)hx) : open_smem<float>((int)hx)) > 56 * 1024) return false;
  const Dims d = dims_of(in);
  const int64_t H = d.ny, Wd = d.nx;
  if (H < 1 || Wd < 1 || (Wd * es) % 16 != 0) return false;
  if ((reinterpret_cast<uintptr_t>(in.data) | reinterpret_cast<uintptr_t>(out.data)) % 16 != 0) return false;
  if (H > (1 << 30) || Wd * es / 4 > (1 << 30) || ceil_div(H, kThreads) > 65535) return false;
  const int x = (int)hx;
  switch (in.ptype) {
    case PG_PTYPE_U16:
      *st = opening ? rect_open_k<uint16_t, true>(in, out, x, s) : rect_open_k<uint16_t, false>(in, out, x, s);
      return true;
    case PG_PTYPE_I32:
      *st = opening ? rect_open_k<int32_t, true>(in, out, x, s) : rect_open_k<int32_t, false>(in, out, x, s);
      return true;
    case PG_PTYPE_F32:
      *st = opening ? rect_open_k<float, true>(in, out, x, s) : rect_open_k<float, false>(in, out, x, s);
      return true;
    default: return false;
  }
}

int take_open_status() {
  int st = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&st, g_open_status, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  if (st != 0 && cudaMemcpyToSymbol(g_open_status, &zero, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  return st;
}

}  // namespace pg
