// line_w.cu -- word-packed van Herk / Gil-Werman segments for 1-, 2- and 4-byte pixels.
//
// Same result as k_line (line.cu): out(p) = min/max of the input over p + t*d, t in [-k, k],
// clipped to the image (ero_dil_line_se_t.hpp:50-89 for X and Y; the diagonals are the
// runtime neighbour-list segments).  This kernel is the fast path when the image rows are
// whole 32-bit words (width * pixel size a multiple of 4, 4-byte aligned buffers).
//
// Every direction is reduced to scans DOWN THE COLUMNS of a shared-memory array of 32-bit
// words, each word packing E = 4 / sizeof(T) pixels that belong to E different lines, so one
// SIMD-in-word min/max (__vmaxu4 / __vmaxu2 / max) advances E lines at once:
//   * Y:  rows of the staged tile are the scan positions, words hold E adjacent columns;
//   * X:  E x E blocks are transposed while staging (__byte_perm), so columns become the scan
//         positions and a word holds E adjacent rows; transposed back on output;
//   * 45 / 135 degrees: staged row r is sheared by r pixels (funnel shifts), so the diagonal
//         lines become columns.  The output tiles are staircases that lean along the diagonal
//         (a tile row's word range moves by one word every E rows), so the sheared band a tile
//         stages is only TX + 2E pixels wide, not TX + TY.
// Per (word column, block of 2k+1 positions) one thread runs the running prefix into G and the
// running suffix in place; out = op(suffix(p - k), prefix(p + k)).  Staging and output are
// coalesced 32-bit accesses; shared rows have an odd word pitch (conflict-free scans).
#include <algorithm>
#include <atomic>

#include "common.cuh"
#include "words.cuh"

namespace pg {

enum { LW_V = 0, LW_H = 1, LW_D45 = 2, LW_D135 = 3 };
static constexpr int kLWThreads = 512;
static constexpr int kLWBatch = 8;  // staged loads kept in flight per thread

struct LWGeom {
  int k, KA;    // half length; for X, k rounded up to a multiple of E
  int TY, TX;   // output tile (pixels)
  int L;        // scan positions staged
  int NW, NWP;  // word lines and row pitch (odd)
  int nblk;     // blocks of 2k+1 positions per line
  int txl;      // diagonals: staircase tiles left of tile 0 (blockIdx.x - txl is the tile column)
};

template <typename T, bool SUP, int MODE>
__global__ void __launch_bounds__(kLWThreads) k_line_w(const T *__restrict__ in, T *__restrict__ out, int H, int W,
                                                       LWGeom g) {
  constexpr int E = 4 / (int)sizeof(T);
  extern __shared__ __align__(16) uint32_t smw[];
  uint32_t *F = smw;
  uint32_t *G = smw + (size_t)g.L * g.NWP;
  const int Wn = W / E;
  const uint32_t *inw = reinterpret_cast<const uint32_t *>(in);
  uint32_t *outw = reinterpret_cast<uint32_t *>(out);
  const T NEU = Op<T, SUP>::neutral();
  const uint32_t NEUW = splat<T>(NEU);
  const int ty0 = blockIdx.y * g.TY;
  const int tx0 = (MODE == LW_D45 || MODE == LW_D135) ? ((int)blockIdx.x - g.txl) * g.TX : (int)blockIdx.x * g.TX;
  const int k = g.k;

  // ------------------------------------------------------------------ stage
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NWARPS = kLWThreads / 32;
  if constexpr (MODE == LW_V) {
    for (int j = lane; j < g.NW; j += 32) {
      const int gw = tx0 / E + j;
      const bool col_ok = gw < Wn;
      for (int r0 = warp; r0 < g.L; r0 += NWARPS * kLWBatch) {
        uint32_t v[kLWBatch];
#pragma unroll
        for (int u = 0; u < kLWBatch; ++u) {  // all loads first: kLWBatch in flight
          const int r = r0 + u * NWARPS, gy = ty0 - k + r;
          v[u] = (r < g.L && col_ok && gy >= 0 && gy < H) ? __ldg(inw + (size_t)gy * Wn + gw) : NEUW;
        }
#pragma unroll
        for (int u = 0; u < kLWBatch; ++u) {
          const int r = r0 + u * NWARPS;
          if (r < g.L) F[r * g.NWP + j] = v[u];
        }
      }
    }
  } else if constexpr (MODE == LW_H) {
    const int CW = g.L / E;              // column words of the staged region
    const int gw0 = (tx0 - g.KA) / E;    // exact: both terms are multiples of E
    for (int jw = warp; jw < g.NW; jw += NWARPS)
    for (int cw = lane; cw < CW; cw += 32) {
      const int gw = gw0 + cw;
      uint32_t w[E];
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int gy = ty0 + jw * E + e;
        w[e] = (gy < H && gw >= 0 && gw < Wn) ? __ldg(inw + (size_t)gy * Wn + gw) : NEUW;
      }
      transpose_block<T>(w);
#pragma unroll
      for (int e = 0; e < E; ++e) F[(cw * E + e) * g.NWP + jw] = w[e];
    }
  } else {
#pragma unroll 4
    for (int r = warp; r < g.L; r += NWARPS)
    for (int uw = lane; uw < g.NW; uw += 32) {
      const int gy = ty0 - k + r;
      // staged pixel u of row r lies on diagonal u of the tile's band (x + y, resp. x - y, constant)
      const int c0 = (MODE == LW_D45) ? tx0 + (g.TY - E) + uw * E + k - r : tx0 - (E - 1) + uw * E - k + r;
      uint32_t v = NEUW;
      if (gy >= 0 && gy < H && c0 + E > 0 && c0 < W) {
        if (c0 >= 0 && c0 + E <= W) {
          const int a = c0 / E, s = c0 - a * E;
          const uint32_t *row = inw + (size_t)gy * Wn;
          const uint32_t lo = __ldg(row + a);
          const uint32_t hi = s ? __ldg(row + a + 1) : 0u;
          v = shift_px<T>(lo, hi, s);
        } else {
          T px[E];
#pragma unroll
          for (int e = 0; e < E; ++e) {
            const int c = c0 + e;
            px[e] = (c >= 0 && c < W) ? ldg(in + (size_t)gy * W + c) : NEU;
          }
          v = pack<T>(px);
        }
      }
      F[r * g.NWP + uw] = v;
    }
  }
  __syncthreads();

  // ------------------------------------------------------------------ prefix / suffix per block
  const int w = 2 * k + 1;
  for (int item = threadIdx.x; item < g.NW * g.nblk; item += kLWThreads) {
    const int l = item % g.NW, b = item / g.NW;
    const int j0 = b * w;
    if (j0 >= g.L) continue;
    const int j1 = min(j0 + w, g.L);
    const int n = j1 - j0;
    const int NWP = g.NWP;
    uint32_t *f = F + j0 * NWP + l;
    uint32_t *gg = G + j0 * NWP + l;
    uint32_t acc = f[0];
    gg[0] = acc;
#pragma unroll 8
    for (int j = 1; j < n; ++j) {
      acc = wop<T, SUP>(acc, f[j * NWP]);
      gg[j * NWP] = acc;
    }
    acc = f[(n - 1) * NWP];
#pragma unroll 8
    for (int j = n - 2; j >= 0; --j) {
      acc = wop<T, SUP>(acc, f[j * NWP]);
      f[j * NWP] = acc;
    }
  }
  __syncthreads();

  // ------------------------------------------------------------------ combine and store
  if constexpr (MODE == LW_V) {
    for (int j = lane; j < g.NW; j += 32) {
      const int gw = tx0 / E + j;
      if (gw >= Wn) continue;
      for (int y = warp; y < g.TY; y += NWARPS) {
        const int gy = ty0 + y;
        if (gy < H) outw[(size_t)gy * Wn + gw] = wop<T, SUP>(F[y * g.NWP + j], G[(y + 2 * k) * g.NWP + j]);
      }
    }
  } else if constexpr (MODE == LW_H) {
    const int XW = g.TX / E;
    for (int jw = warp; jw < g.NW; jw += NWARPS)
    for (int xw = lane; xw < XW; xw += 32) {
      const int gw = tx0 / E + xw;
      if (gw >= Wn) continue;
      uint32_t r[E];
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int x = xw * E + e;
        r[e] = wop<T, SUP>(F[(x + g.KA - k) * g.NWP + jw], G[(x + g.KA + k) * g.NWP + jw]);
      }
      transpose_block<T>(r);
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int gy = ty0 + jw * E + e;
        if (gy < H) outw[(size_t)gy * Wn + gw] = r[e];
      }
    }
  } else {
    // staircase row y: words [tx0 / E + sh, + XW) with sh = floor((TY - 1 - y) / E) (45 degrees) or
    // floor(y / E) (135 degrees); its pixel e of word xw is diagonal E * xw + e + s of the band
    const int XW = g.TX / E;
    for (int y = warp; y < g.TY; y += NWARPS)
    for (int xw = lane; xw < XW; xw += 32) {
      const int m = (MODE == LW_D45) ? g.TY - 1 - y : y;
      const int sh = m / E, s = E - 1 - (m - sh * E);
      const int gy = ty0 + y, gw = tx0 / E + sh + xw;
      if (gy >= H || gw < 0 || gw >= Wn) continue;
      const int uw = xw;
      const uint32_t *f = F + y * g.NWP;
      const uint32_t *gg = G + (y + 2 * k) * g.NWP;
      const uint32_t a = shift_px<T>(f[uw], s ? f[uw + 1] : 0u, s);
      const uint32_t b = shift_px<T>(gg[uw], s ? gg[uw + 1] : 0u, s);
      outw[(size_t)gy * Wn + gw] = wop<T, SUP>(a, b);
    }
  }
}

static size_t lw_smem(const LWGeom &g) { return 2ull * (size_t)g.L * (size_t)g.NWP * 4u; }

template <typename T>
static LWGeom lw_geom(int mode, int k, int TY, int TX) {
  constexpr int E = 4 / (int)sizeof(T);
  LWGeom g{};
  g.k = k;
  g.KA = (k + E - 1) / E * E;
  g.TY = TY;
  g.TX = TX;
  if (mode == LW_V) { g.L = TY + 2 * k; g.NW = TX / E; }
  else if (mode == LW_H) { g.L = TX + 2 * g.KA; g.NW = TY / E; }
  else { g.L = TY + 2 * k; g.NW = (TX + E - 1) / E + 1; }
  g.NWP = g.NW | 1;
  g.nblk = (g.L + 2 * k) / (2 * k + 1);  // ceil(L / (2k+1))
  g.txl = 0;
  return g;
}

template <typename T, bool SUP, int MODE>
static pg_status lw_launch(const T *in, T *out, int H, int W, int k, cudaStream_t s) {
  constexpr int E = 4 / (int)sizeof(T);
  const size_t budget = 100 * 1024, hard = 227 * 1024;
  LWGeom g{};
  bool ok = false;
  if (MODE == LW_V) {
    for (int nw : {64, 32, 16}) {
      for (int ty : {128, 64, 32, 16, 8}) {
        g = lw_geom<T>(MODE, k, ty, nw * E);
        if (lw_smem(g) <= budget) { ok = true; break; }
      }
      if (ok) break;
    }
  } else if (MODE == LW_H) {
    // wide, short tiles: measured best (4096^2, k = 15 and 31, u8/u16/f32) at 256 x 16 words
    for (int tx : {256, 128, 64, 32}) {
      for (int nw : {16, 32, 8, 64}) {
        g = lw_geom<T>(MODE, k, nw * E, tx);
        if (lw_smem(g) <= budget) { ok = true; break; }
      }
      if (ok) break;
    }
  } else {
    // tall staircase tiles: the band staged per tile is (TY + 2k) x (TX + 2E) pixels
    for (int ty : {128, 64, 32, 16}) {
      for (int nw : {64, 32, 16}) {
        g = lw_geom<T>(MODE, k, ty, nw * E);
        if (lw_smem(g) <= budget) { ok = true; break; }
      }
      if (ok) break;
    }
    const int shmax = (g.TY - 1) / E;  // largest staircase shift, in words
    g.txl = (int)ceil_div(shmax, g.TX / E);
  }
  if (!ok && lw_smem(g) <= hard) ok = true;
  if (!ok) return fail(PG_ERR_INVALID_ARGUMENT, "segment too long for the word-packed line kernel");
  static std::atomic<uint64_t> attr_devices{0};
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  const uint64_t bit = 1ull << (dev & 63);
  if (!(attr_devices.load() & bit)) {
    PG_CUDA_TRY(cudaFuncSetAttribute(k_line_w<T, SUP, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hard),
                "line kernel smem attribute");
    attr_devices.fetch_or(bit);
  }
  dim3 grid((unsigned)(ceil_div(W, g.TX) + g.txl), (unsigned)ceil_div(H, g.TY));
  if (grid.y > 65535) return fail(PG_ERR_INVALID_ARGUMENT, "image too tall for the line kernel");
  k_line_w<T, SUP, MODE><<<grid, kLWThreads, lw_smem(g), s>>>(in, out, H, W, g);
  return cuda_status(cudaGetLastError(), "word-packed line kernel launch");
}

template <typename T, bool SUP>
static pg_status lw_dispatch(const T *in, T *out, int64_t H, int64_t W, int dy, int dx, int k, cudaStream_t s) {
  if (dy == 0) return lw_launch<T, SUP, LW_H>(in, out, (int)H, (int)W, k, s);
  if (dx == 0) return lw_launch<T, SUP, LW_V>(in, out, (int)H, (int)W, k, s);
  if (dx == -1) return lw_launch<T, SUP, LW_D45>(in, out, (int)H, (int)W, k, s);
  return lw_launch<T, SUP, LW_D135>(in, out, (int)H, (int)W, k, s);
}

// Fast path of launch_line for 1/2/4-byte pixels in word-aligned rows.  Returns false (and does
// nothing) when the image does not qualify; k >= 1 is the already clipped half length.
bool try_line_words(const pg_image &in, const pg_image &out, int dy, int dx, int k, bool dilate, cudaStream_t s,
                    pg_status *st) {
  const int es = elem_size(in.ptype);
  if (es > 4 || k < 1) return false;
  const Dims d = dims_of(in);
  const int64_t H = d.ny, W = d.nx;
  if (H > (1 << 30) || W > (1 << 30)) return false;
  if ((W * es) % 4 != 0) return false;
  if ((reinterpret_cast<uintptr_t>(in.data) | reinterpret_cast<uintptr_t>(out.data)) % 4 != 0) return false;
  switch (in.ptype) {
    case PG_PTYPE_U8: {
      using T = uint8_t;
      *st = dilate ? lw_dispatch<T, true>((const T *)in.data, (T *)out.data, H, W, dy, dx, k, s)
                   : lw_dispatch<T, false>((const T *)in.data, (T *)out.data, H, W, dy, dx, k, s);
      return true;
    }
    case PG_PTYPE_U16: {
      using T = uint16_t;
      *st = dilate ? lw_dispatch<T, true>((const T *)in.data, (T *)out.data, H, W, dy, dx, k, s)
                   : lw_dispatch<T, false>((const T *)in.data, (T *)out.data, H, W, dy, dx, k, s);
      return true;
    }
    case PG_PTYPE_I32: {
      using T = int32_t;
      *st = dilate ? lw_dispatch<T, true>((const T *)in.data, (T *)out.data, H, W, dy, dx, k, s)
                   : lw_dispatch<T, false>((const T *)in.data, (T *)out.data, H, W, dy, dx, k, s);
      return true;
    }
    case PG_PTYPE_F32: {
      using T = float;
      *st = dilate ? lw_dispatch<T, true>((const T *)in.data, (T *)out.data, H, W, dy, dx, k, s)
                   : lw_dispatch<T, false>((const T *)in.data, (T *)out.data, H, W, dy, dx, k, s);
      return true;
    }
    default: return false;
  }
}

}  // namespace pg
