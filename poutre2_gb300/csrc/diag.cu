// diag.cu -- erosion / dilation by the vertical, 45- and 135-degree segments of 2K+1 pixels (K = 7, 15,
// 31), and the opening / closing by those segments in one pass, through shared-memory parallelogram
// tiles loaded by TMA; 1-, 2- and 4-byte pixels, rows of a multiple of 16 bytes.
//
// Same result as the streaming segment kernels of line_stream.cu, as DilateY / ErodeY
// (ero_dil_line_se_t.hpp:249-282) for the vertical segment and as the runtime neighbour list of the
// diagonal segments (ero_dil_runtime_nl_se_t.hpp:129-193): the window is clipped at the image border,
// i.e. pixels outside the image are the operator's neutral value.  The opening is the dilation of the
// erosion (ero_dil.hpp Opening), each clipped at the border in the same way.
//
// A CTA owns TW adjacent segment lines ("diagonals"; columns for the vertical segment) over TH output
// rows, so its output tile is a parallelogram leaning with the segment; the tiles of one tile row,
// shifted by TW pixels, cover every pixel of those rows once.  The tile's input rows come in as a
// staircase of TMA boxes: the rows are cut into groups of G = 16 / sizeof(T) rows, the drift of one
// 16-byte chunk, and group g is one 2D box of G rows x (TW + G) pixels that starts G pixels further
// left (45 degrees) or right (135 degrees) than group g - 1 -- for the vertical segment one box of TW
// pixels holds all rows, and a 45-degree tile whose columns all lie in the image takes the whole
// staircase as one box of a sheared 3D view of the image.  Every box starts on a 16-byte boundary, the
// tile rows start on a multiple of G, and in shared memory line t at row k of a group sits at column
// t + G - k (45 degrees), t + k (135) or t (vertical).  Pixels outside the image arrive as TMA's zero
// fill and are then set to the first operator's neutral value (nothing to do when that is 0: the
// dilation of unsigned pixels).
//
// Each thread runs van Herk / Gil-Werman down one line: the CH windows starting at tile rows R0 .. R0 +
// CH - 1 (CH the largest multiple of G <= 2K + 1, R0 a multiple of G) take the running suffix of block
// A = rows R0 .. R0 + 2K, kept in registers, and the running prefix of the rows after it.  With R0 a
// multiple of G the row's place in its group is known at compile time, so every shared-memory access is
// one load at a constant offset from the thread's column.  Single operator: the outputs go straight to
// global memory, the 32 lanes of a warp writing 32 consecutive pixels of a row; for 4-byte pixels two
// thread groups split the tile's rows.  Opening / closing: the tile holds 2K more input rows above and
// below; the first operator's result for the window starting at row r is written back over input row r
// of the thread's own line -- no later window of that line reads row r -- with the second operator's
// neutral value where the window's centre lies outside the image, and the second operator then runs
// over those values; a line belongs to one thread, so no barrier separates the two scans.
//
// The wait for the boxes is bounded (tile::kWaitNs of %globaltimer); on expiry the CTA records
// PG_ERR_CUDA in g_diag_status (read by pg_check_device) and leaves its tile unwritten.
#include <atomic>

#include "tile.cuh"

namespace pg {

__device__ int g_diag_status = 0;

namespace {

using namespace tile;

constexpr int ceil_to(int a, int m) { return (a + m - 1) / m * m; }

// output rows per tile for the opening / closing: the multiple of G (48 .. 192) with the least work
// per output row -- both scans' chunk rows, plus a share for each input row copied -- whose tile fits
// in 76 KB of shared memory (3 CTAs per SM for 2-byte pixels)
constexpr int fused_rows(int G, int CH, int K, int GP) {
  int best = G, best_cost = 1 << 30;
  for (int th = ceil_to(CH > 48 ? CH : 48, G); th <= 192; th += G) {
    const int nc1 = (th + 2 * K + CH - 1) / CH, nc2 = (th + CH - 1) / CH;
    const int rows = ceil_to(nc1 * CH + 2 * K, G);
    if (rows / G * GP > 76 * 1024) continue;
    const int cost = ((nc1 + nc2) * CH * 10 + rows * 3) * 64 / th;
    if (cost < best_cost) { best_cost = cost; best = th; }
  }
  return best;
}

template <typename T, int K, int DIR, bool FUSED> struct DiagGeom {
  static constexpr int S = (int)sizeof(T);
  static constexpr int G = 16 / S;                       // rows per box: one 16-byte chunk of drift
  static constexpr int W2 = 2 * K + 1;                   // segment length
  static constexpr int TW = S == 4 ? 64 : 128;           // lines per tile (256 or 128 bytes of a row)
  static constexpr int NT = FUSED ? TW : 128;            // threads
  static constexpr int NV = NT / TW;                     // thread groups stacked along the tile's rows
  static constexpr int CH = W2 / G * G;                  // windows per van Herk chunk
  static constexpr int KH = FUSED ? 2 * K : K;           // input rows above the first output row
  // box width, pixels: a whole number of 16-byte chunks with G rows of it a multiple of 128 bytes, so
  // that the groups lie back to back in shared memory (the 45-degree tile arrives as one 3D box)
  static constexpr int BWP = ceil_to(TW + (DIR != 0 ? G : 0), 8);
  static constexpr int RP = BWP * S;                     // bytes per box row
  static constexpr int GP = ceil_to(G * RP, 128);        // bytes per group in shared memory (TMA: 128-aligned)
  static constexpr int THG = FUSED ? fused_rows(G, CH, K, GP) : (120 / NV) / CH * CH;  // output rows per group
  static constexpr int TH = NV * THG;                    // output rows per tile
  static constexpr int NC1 = FUSED ? (TH + 2 * K + CH - 1) / CH : 0;  // chunks of the first scan (fused)
  static constexpr int NC2 = (THG + CH - 1) / CH;        // chunks of the (last) scan per thread
  // input rows: the last chunk of the first scan reads rows up to NC1*CH + 2K - 2 (fused), the last
  // chunk of a single scan rows up to TH + 2K - 2
  static constexpr int BR = ceil_to(FUSED ? NC1 * CH + 2 * K : TH + 2 * K, G);
  static constexpr int RB = (DIR == 0 && GP == G * RP && BR <= 256) ? BR : G;  // rows per TMA box
  static constexpr int NB = BR / RB;                     // boxes per tile
  static constexpr int D = (G - KH % G) % G;             // tile row b: output rows from b*TH - D
  static constexpr unsigned tile_bytes = (unsigned)(BR * RP);
  static constexpr size_t smem = (size_t)(BR / G) * GP + 16;  // + the mbarrier
  static_assert(CH >= G && THG >= CH && NT % TW == 0 && BWP <= 256 && TH % G == 0 && BR % RB == 0,
                "segment tile geometry");
  static_assert(GP == G * RP, "groups back to back in shared memory");
  static_assert(!FUSED || NC2 * CH + 2 * K <= NC1 * CH + 2 * K, "second scan inside the first scan's rows");
  static_assert(FUSED || THG % CH == 0, "single scan: whole chunks");
};

// tile columns: tile bx has line 0 at column x0 = cx + (bx - M0) * TW of its first output row y0 and
// covers [x0 - d, x0 - d + TW) (45 degrees), [x0 + d, ..) (135) or [x0, ..) (vertical) at row y0 + d
template <typename Gm, int DIR> struct DiagCols {
  static constexpr int M0 = DIR > 0 ? 1 : DIR < 0 ? (Gm::TH + Gm::G - 2 + Gm::TW - 1) / Gm::TW : 0;
  static int64_t count(int64_t W) {
    if (DIR == 0) return (W + Gm::TW - 1) / Gm::TW;
    return DIR > 0 ? (W + Gm::TH - 2) / Gm::TW + 2 : (W - 1) / Gm::TW + M0 + 1;
  }
};

__device__ __forceinline__ int pos_mod(int a, int m) { return ((a % m) + m) % m; }

// row i of a chunk that starts on a group boundary at p: group i / G, row i % G, column -/+ (i % G)
template <typename T, int DIR, int G, int GP, int RP> __device__ __forceinline__ constexpr int row_off(int i) {
  return (i / G) * GP + (i % G) * RP + (DIR > 0 ? -(i % G) : DIR < 0 ? (i % G) : 0) * (int)sizeof(T);
}

// One van Herk / Gil-Werman chunk on the line at p: emit(i, op over rows i .. i + 2K) for i < CH.
template <typename T, bool SUP, int DIR, int W2, int CH, int G, int GP, int RP, typename F>
__device__ __forceinline__ void vh_chunk(const unsigned char *p, F &&emit) {
  using O = Op<T, SUP>;
#define PG_LD(i) (*reinterpret_cast<const T *>(p + row_off<T, DIR, G, GP, RP>(i)))
  T suf[W2];
  suf[W2 - 1] = PG_LD(W2 - 1);
#pragma unroll
  for (int i = W2 - 2; i >= 0; --i) suf[i] = O::apply(suf[i + 1], PG_LD(i));
  T pre = O::neutral();
#pragma unroll
  for (int i = 0; i < CH; ++i) {
    if (i > 0) pre = O::apply(pre, PG_LD(W2 + i - 1));
    emit(i, i > 0 ? O::apply(suf[i], pre) : suf[0]);
  }
#undef PG_LD
}

// The same chunk for the dilation and the erosion at once (one load feeds both): emit(i, dil, ero).
template <typename T, int DIR, int W2, int CH, int G, int GP, int RP, typename F>
__device__ __forceinline__ void vh_chunk2(const unsigned char *p, F &&emit) {
  using D = Op<T, true>;
  using E = Op<T, false>;
#define PG_LD(i) (*reinterpret_cast<const T *>(p + row_off<T, DIR, G, GP, RP>(i)))
  T sd[W2], se[W2];
  sd[W2 - 1] = se[W2 - 1] = PG_LD(W2 - 1);
#pragma unroll
  for (int i = W2 - 2; i >= 0; --i) {
    const T v = PG_LD(i);
    sd[i] = D::apply(sd[i + 1], v);
    se[i] = E::apply(se[i + 1], v);
  }
  T pd = D::neutral(), pe = E::neutral();
#pragma unroll
  for (int i = 0; i < CH; ++i) {
    if (i > 0) {
      const T v = PG_LD(W2 + i - 1);
      pd = D::apply(pd, v);
      pe = E::apply(pe, v);
    }
    emit(i, i > 0 ? D::apply(sd[i], pd) : sd[0], i > 0 ? E::apply(se[i], pe) : se[0]);
  }
#undef PG_LD
}

// dilation - erosion: exact for unsigned pixels (never negative), i32 wraps like the difference
// kernel's int arithmetic, f32 is one rounded subtraction
template <typename T> __device__ __forceinline__ T grad_of(T d, T e) {
  if constexpr (std::is_same_v<T, int32_t>) return (int32_t)((uint32_t)d - (uint32_t)e);
  else return (T)(d - e);
}

// MODE: 0 erosion, 1 dilation, 2 opening (erosion, then dilation), 3 closing, 4 gradient (dilation - erosion)
template <typename T, int K, int DIR, int MODE>
__global__ void __launch_bounds__(DiagGeom<T, K, DIR, (MODE == 2 || MODE == 3)>::NT, (MODE == 4 ? 3 : 0))
    k_segment_tile(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap smap,
                   T *__restrict__ out, int H, int W, int shear_rows) {
  constexpr bool FUSED = MODE == 2 || MODE == 3;
  constexpr bool GRAD = MODE == 4;
  using Gm = DiagGeom<T, K, DIR, FUSED>;
  constexpr int S = Gm::S, G = Gm::G, W2 = Gm::W2, TW = Gm::TW, CH = Gm::CH, THG = Gm::THG, TH = Gm::TH;
  constexpr int BR = Gm::BR, BWP = Gm::BWP, RP = Gm::RP, GP = Gm::GP, RB = Gm::RB, NB = Gm::NB;
  constexpr bool SUP_A = MODE == 1 || MODE == 3;  // the first (or only) operator is a dilation
  using OA = Op<T, SUP_A>;
  using OB = Op<T, !SUP_A>;
  extern __shared__ __align__(128) unsigned char s_box[];
  __shared__ int s_ok;
  uint64_t *bar = reinterpret_cast<uint64_t *>(s_box + (BR / G) * GP);
  const unsigned bar_a = smem_u32(bar);
  const int tid = threadIdx.x;
  const int y0 = (int)blockIdx.y * TH - Gm::D;  // first output row
  const int ty = y0 - Gm::KH;                   // first input row, a multiple of G
  const int cx = DIR > 0 ? pos_mod(-y0, G) : DIR < 0 ? pos_mod(y0, G) : 0;
  const int x0 = cx + ((int)blockIdx.x - DiagCols<Gm, DIR>::M0) * TW;  // line 0 at row y0
  // first column of group g (input rows ty + gG ..): x0 - DIR * (ty + gG - y0), less G for 45 degrees
  auto box_x = [&](int g) { return DIR > 0 ? x0 + Gm::KH - g * G - G : DIR < 0 ? x0 - Gm::KH + g * G : x0; };

  if (tid == 0) {
    if (smem_u32(s_box) & 127u) {  // a TMA destination starts on a 128-byte boundary
      atomicCAS(&g_diag_status, 0, (int)PG_ERR_CUDA);
      s_ok = 0;
    } else {
      s_ok = 1;
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a), "r"(Gm::tile_bytes)
                   : "memory");
    }
  }
  __syncthreads();
  if (!s_ok) return;
  // 45 degrees: the whole staircase is one box of the sheared view `smap` (group j of the view starts
  // 16 bytes left of row G*j, so view column X of group j is image column X - G*j), unless the tile
  // reaches the last H mod G rows, which the view leaves out (shear_rows = G * floor(H / G)), or a
  // side of the image, where the view would bring pixels of the neighbouring rows instead of the 2D
  // boxes' zero fill
  const bool sheared = DIR > 0 && shear_rows > 0 && (shear_rows == H || ty + BR <= shear_rows) &&
                       box_x(BR / G - 1) >= 0 && box_x(0) + BWP <= W;
  if (sheared) {
    if (tid == 0)
      asm volatile(
          "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
              smem_u32(s_box)),
          "l"(&smap), "r"(box_x(0) + ty), "r"(0), "r"(ty / G), "r"(bar_a)
          : "memory");
  } else if (tid < 32) {
    for (int b = tid; b < NB; b += 32) {
      const int g = b * (RB / G);
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
              smem_u32(s_box + g * GP)),
          "l"(&tmap), "r"(box_x(g)), "r"(ty + g * G), "r"(bar_a)
          : "memory");
    }
  }
  if (tid == 0) {
    bool done = mbar_try(bar_a, 0);
    const unsigned long long t0 = now_ns();
    while (!done && now_ns() - t0 < kWaitNs) done = mbar_try(bar_a, 0);
    if (!done) atomicCAS(&g_diag_status, 0, (int)PG_ERR_CUDA);
    s_ok = done;
  }
  __syncthreads();
  if (!s_ok) return;
  (void)mbar_try(bar_a, 0);  // the phase is complete: each thread observes it (acquire)

  // pixels outside the image: TMA's zero fill (the sheared view is used only where no column is outside
  // the image); the first operator needs its neutral value there -- zero already is it for the dilation
  // of unsigned pixels
  if constexpr (!GRAD && !(std::is_unsigned_v<T> && SUP_A)) {
    const int xa = box_x(0), xb = box_x(BR / G - 1);
    const int xlo = DIR > 0 ? xb : xa, xhi = (DIR > 0 ? xa : xb) + BWP;
    if (ty < 0 || ty + BR > H || xlo < 0 || xhi > W) {
      const T NEU = OA::neutral();
      for (int r = tid; r < BR; r += Gm::NT) {
        const int g = r / G;
        T *row = reinterpret_cast<T *>(s_box + g * GP + (r % G) * RP);
        const int bx = box_x(g), yr = ty + r;
        const int lo = (yr < 0 || yr >= H) ? BWP : min(max(-bx, 0), BWP);  // columns [0, lo) are outside
        const int hi = (yr < 0 || yr >= H) ? BWP : max(min(W - bx, BWP), lo);  // and [hi, BWP)
        for (int c = 0; c < lo; ++c) row[c] = NEU;
        for (int c = hi; c < BWP; ++c) row[c] = NEU;
      }
      __syncthreads();
    }
  }

  const int t = tid % TW, v = tid / TW;
  unsigned char *colp = s_box + (DIR > 0 ? t + G : t) * S;
  // line t is at column x0 + t - DIR * (y - y0) of row y; all of rows y_a .. y_b inside the image?
  auto inside = [&](int ya, int yb) {
    const int xmin = x0 - (DIR > 0 ? DIR * (yb - y0) : DIR * (ya - y0));
    const int xmax = x0 + TW - 1 - (DIR > 0 ? DIR * (ya - y0) : DIR * (yb - y0));
    return ya >= 0 && yb < H && xmin >= 0 && xmax < W;
  };
  const int step = W - DIR;  // one row down the line

  if constexpr (GRAD) {
    // two operators, two neutral values: instead, the pixels of a line outside the image repeat the
    // line's nearest pixel inside it.  A clipped window holds its centre, so a window that reaches
    // past the image along the line also holds that nearest pixel: neither extremum changes.
    const int xr = x0 + t + DIR * (y0 - ty);  // column of line t at tile row 0 is xr - DIR * r
    int ra = max(0, -ty), rb = min(BR - 1, H - 1 - ty);
    if (DIR > 0) { ra = max(ra, xr - W + 1); rb = min(rb, xr); }
    else if (DIR < 0) { ra = max(ra, -xr); rb = min(rb, W - 1 - xr); }
    else if (xr < 0 || xr >= W) rb = -1;
    if (ty < 0 || ty + BR > H || !inside(ty, ty + BR - 1)) {
      auto px = [&](int r) {
        return reinterpret_cast<T *>(colp + (r / G) * GP + (r % G) * RP +
                                     (DIR > 0 ? -(r % G) : DIR < 0 ? (r % G) : 0) * S);
      };
      if (v == 0 && ra <= rb) {
        const T top = *px(ra), bot = *px(rb);
        for (int r = 0; r < ra; ++r) *px(r) = top;
        for (int r = rb + 1; r < BR; ++r) *px(r) = bot;
      }
      __syncthreads();
    }
    const bool in = inside(y0, y0 + TH - 1);
#pragma unroll 1
    for (int c = 0; c < Gm::NC2; ++c) {
      const int R0 = v * THG + c * CH;
      const unsigned char *p = colp + (R0 / G) * GP;
      const int y = y0 + R0, x = x0 + t - DIR * R0;
      T *o = out + ((size_t)(int64_t)y * W + x);
      if (in) {
        vh_chunk2<T, DIR, W2, CH, G, GP, RP>(p, [&](int, T d, T e) {
          *o = grad_of<T>(d, e);
          o += step;
        });
      } else {
        vh_chunk2<T, DIR, W2, CH, G, GP, RP>(p, [&](int i, T d, T e) {
          const int yy = y + i, xx = x - DIR * i;
          if ((unsigned)yy < (unsigned)H && (unsigned)xx < (unsigned)W) *o = grad_of<T>(d, e);
          o += step;
        });
      }
    }
    return;
  }

  if constexpr (FUSED) {
    // first operator: the window starting at tile row R0 + i is centred on image row y0 - K + R0 + i;
    // its value replaces input row R0 + i of this line (the second operator's neutral value outside
    // the image).  The border tests sit outside the unrolled chunks: tiles inside the image skip them.
    const bool in1 = inside(y0 - K, y0 + TH + K - 1);
#pragma unroll 1
    for (int c = 0; c < Gm::NC1; ++c) {
      const int R0 = c * CH;
      unsigned char *p = colp + (R0 / G) * GP;
      if (in1) {
        vh_chunk<T, SUP_A, DIR, W2, CH, G, GP, RP>(
            p, [&](int i, T val) { *reinterpret_cast<T *>(p + row_off<T, DIR, G, GP, RP>(i)) = val; });
      } else {
        const int yc = y0 - K + R0, xc = x0 + t - DIR * (R0 - K);
        vh_chunk<T, SUP_A, DIR, W2, CH, G, GP, RP>(p, [&](int i, T val) {
          const int yy = yc + i, xx = xc - DIR * i;
          *reinterpret_cast<T *>(p + row_off<T, DIR, G, GP, RP>(i)) =
              ((unsigned)yy < (unsigned)H && (unsigned)xx < (unsigned)W) ? val : OB::neutral();
        });
      }
    }
    // second operator over those values: window R0 + i is centred on output row y0 + R0 + i
    const bool in2 = inside(y0, y0 + TH - 1);
#pragma unroll 1
    for (int c = 0; c < Gm::NC2; ++c) {
      const int R0 = c * CH;
      const unsigned char *p = colp + (R0 / G) * GP;
      const int y = y0 + R0, x = x0 + t - DIR * R0;
      T *o = out + ((size_t)(int64_t)y * W + x);
      if (in2 && R0 + CH <= TH) {
        vh_chunk<T, !SUP_A, DIR, W2, CH, G, GP, RP>(p, [&](int, T val) {
          *o = val;
          o += step;
        });
      } else {
        vh_chunk<T, !SUP_A, DIR, W2, CH, G, GP, RP>(p, [&](int i, T val) {
          const int yy = y + i, xx = x - DIR * i;
          if (R0 + i < TH && (unsigned)yy < (unsigned)H && (unsigned)xx < (unsigned)W) *o = val;
          o += step;
        });
      }
    }
  } else {
    const bool in = inside(y0, y0 + TH - 1);
#pragma unroll 1
    for (int c = 0; c < Gm::NC2; ++c) {
      const int R0 = v * THG + c * CH;  // tile row of the chunk's first window (a multiple of G)
      const unsigned char *p = colp + (R0 / G) * GP;
      const int y = y0 + R0, x = x0 + t - DIR * R0;  // window R0 + i: output row y + i, column x - DIR * i
      T *o = out + ((size_t)(int64_t)y * W + x);
      if (in) {  // the whole tile lies in the image: one pointer step per output
        vh_chunk<T, SUP_A, DIR, W2, CH, G, GP, RP>(p, [&](int, T val) {
          *o = val;
          o += step;
        });
      } else {
        vh_chunk<T, SUP_A, DIR, W2, CH, G, GP, RP>(p, [&](int i, T val) {
          const int yy = y + i, xx = x - DIR * i;
          if ((unsigned)yy < (unsigned)H && (unsigned)xx < (unsigned)W) *o = val;
          o += step;
        });
      }
    }
  }
}

// Tensor map of an image of H rows x W pixels of S bytes, box of bw pixels x rows rows.
pg_status pixel_map(CUtensorMap *map, const void *data, int64_t H, int64_t W, int S, int bw, int rows) {
  auto fn = encode_tiled();
  if (!fn) return fail(PG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  cuuint64_t dims[2] = {(cuuint64_t)W, (cuuint64_t)H};
  cuuint64_t strides[1] = {(cuuint64_t)W * S};
  cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)rows};
  cuuint32_t estr[2] = {1, 1};
  const CUtensorMapDataType dt = S == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                 : S == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16
                                          : CU_TENSOR_MAP_DATA_TYPE_UINT32;
  const CUresult r = fn(map, dt, 2, const_cast<void *>(data), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(PG_ERR_CUDA, "cuTensorMapEncodeTiled failed for the segment tile");
  return PG_OK;
}

// Sheared view of the same image for 45-degree tiles: dims (X, k, j) -> image row G*j + k, column
// X - G*j, with j < floor(H / G) and X < W + G*(floor(H / G) - 1).  Every coordinate inside those
// bounds addresses a pixel of the image buffer: the largest is row G*floor(H/G) - 1 <= H - 1 at a
// column <= W - 1, the smallest the first pixel, so the view reads nothing outside the buffer; left and
// right of the image it would read pixels of the neighbouring rows, so tiles reaching a side use the 2D
// boxes.  Box:
// bw pixels x G rows x groups.  False if the driver refuses the view (the kernel then uses 2D boxes).
bool sheared_map(CUtensorMap *map, const void *data, int64_t H, int64_t W, int S, int bw, int G, int groups) {
  auto fn = encode_tiled();
  if (!fn) return false;
  const int64_t Jn = H / G;
  cuuint64_t dims[3] = {(cuuint64_t)(W + G * (Jn - 1)), (cuuint64_t)G, (cuuint64_t)Jn};
  cuuint64_t strides[2] = {(cuuint64_t)W * S, (cuuint64_t)(G * W * S - 16)};
  cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)G, (cuuint32_t)groups};
  cuuint32_t estr[3] = {1, 1, 1};
  const CUtensorMapDataType dt = S == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                 : S == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16
                                          : CU_TENSOR_MAP_DATA_TYPE_UINT32;
  return fn(map, dt, 3, const_cast<void *>(data), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

template <typename T, int K, int DIR, int MODE>
pg_status segment_tile(const pg_image &in, const pg_image &out, cudaStream_t s) {
  using Gm = DiagGeom<T, K, DIR, (MODE == 2 || MODE == 3)>;
  const Dims d = dims_of(in);
  const int64_t H = d.ny, W = d.nx;
  CUtensorMap map, smap;
  PG_TRY(pixel_map(&map, in.data, H, W, Gm::S, Gm::BWP, Gm::RB));
  int shear_rows = 0;
  smap = map;
  if (DIR > 0 && H >= Gm::G && sheared_map(&smap, in.data, H, W, Gm::S, Gm::BWP, Gm::G, Gm::BR / Gm::G))
    shear_rows = (int)(H / Gm::G * Gm::G);
  static std::atomic<uint64_t> attr_devices{0};
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  const uint64_t bit = 1ull << (dev & 63);
  if (!(attr_devices.load() & bit)) {
    PG_CUDA_TRY(cudaFuncSetAttribute(k_segment_tile<T, K, DIR, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)Gm::smem),
                "segment tile smem attribute");
    attr_devices.fetch_or(bit);
  }
  const int64_t gy = ceil_div(H + Gm::D, Gm::TH);
  if (gy > 65535) return fail(PG_ERR_INVALID_ARGUMENT, "image too tall for the segment tile kernel");
  const dim3 grid((unsigned)DiagCols<Gm, DIR>::count(W), (unsigned)gy);
  k_segment_tile<T, K, DIR, MODE><<<grid, Gm::NT, Gm::smem, s>>>(map, smap, static_cast<T *>(out.data), (int)H, (int)W,
                                                                  shear_rows);
  return cuda_status(cudaGetLastError(), "segment tile launch");
}

template <typename T, int DIR, int MODE>
pg_status segment_k(const pg_image &in, const pg_image &out, int k, cudaStream_t s) {
  switch (k) {
    case 15: return segment_tile<T, 15, DIR, MODE>(in, out, s);
    case 31: return segment_tile<T, 31, DIR, MODE>(in, out, s);
    default:
      if constexpr (sizeof(T) == 1) return fail(PG_ERR_INVALID_ARGUMENT, "segment tile: half length");  // not reached
      else return segment_tile<T, 7, DIR, MODE>(in, out, s);
  }
}

template <typename T, int MODE>
pg_status segment_dir(const pg_image &in, const pg_image &out, int dx, int k, cudaStream_t s) {
  // (dy, dx) = (1, -1): x + y constant, 45 degrees; (1, 1): x - y constant, 135 degrees; (1, 0): vertical
  if (dx < 0) return segment_k<T, 1, MODE>(in, out, k, s);
  if (dx > 0) return segment_k<T, -1, MODE>(in, out, k, s);
  return segment_k<T, 0, MODE>(in, out, k, s);
}

template <int MODE>
bool segment_try(const pg_image &in, const pg_image &out, int dy, int dx, int k, cudaStream_t s, pg_status *st) {
  if (in.rank != 2 || dy != 1 || dx < -1 || dx > 1) return false;
  const int es = elem_size(in.ptype);
  if (!(in.ptype == PG_PTYPE_U8 || in.ptype == PG_PTYPE_U16 || in.ptype == PG_PTYPE_I32 || in.ptype == PG_PTYPE_F32))
    return false;
  // u8: a group is 16 rows, so the chunk needs 2K + 1 >= 16
  if (!(k == 15 || k == 31 || (k == 7 && es > 1))) return false;
  const Dims d = dims_of(in);
  const int64_t H = d.ny, W = d.nx;
  // the tensor map wants a 16-byte aligned base and rows of a multiple of 16 bytes
  if (H < 1 || W < 1 || (W * es) % 16 != 0 || reinterpret_cast<uintptr_t>(in.data) % 16 != 0) return false;
  if (reinterpret_cast<uintptr_t>(out.data) % es != 0) return false;
  if (H > (1 << 30) || W > (1 << 30) || ceil_div(H + 16, 48) > 65535) return false;
  switch (in.ptype) {
    case PG_PTYPE_U8: *st = segment_dir<uint8_t, MODE>(in, out, dx, k, s); return true;
    case PG_PTYPE_U16: *st = segment_dir<uint16_t, MODE>(in, out, dx, k, s); return true;
    case PG_PTYPE_I32: *st = segment_dir<int32_t, MODE>(in, out, dx, k, s); return true;
    default: *st = segment_dir<float, MODE>(in, out, dx, k, s); return true;
  }
}

}  // namespace

bool try_segment_tile(const pg_image &in, const pg_image &out, int dy, int dx, int k, bool dilate, cudaStream_t s,
                      pg_status *st) {
  return dilate ? segment_try<1>(in, out, dy, dx, k, s, st) : segment_try<0>(in, out, dy, dx, k, s, st);
}

bool try_segment_open(const pg_image &in, const pg_image &out, int dy, int dx, int k, bool opening, cudaStream_t s,
                      pg_status *st) {
  return opening ? segment_try<2>(in, out, dy, dx, k, s, st) : segment_try<3>(in, out, dy, dx, k, s, st);
}

bool try_segment_gradient(const pg_image &in, const pg_image &out, int dy, int dx, int k, cudaStream_t s,
                          pg_status *st) {
  return segment_try<4>(in, out, dy, dx, k, s, st);
}

int take_diag_status() {
  int st = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&st, g_diag_status, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  if (st != 0 && cudaMemcpyToSymbol(g_diag_status, &zero, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  return st;
}

}  // namespace pg
