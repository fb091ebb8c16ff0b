// diag.cu -- erosion / dilation by the 45- and 135-degree segments of 2K+1 pixels (K = 7, 15, 31) on
// 2- and 4-byte pixels, through shared-memory parallelogram tiles loaded by TMA.
//
// Same result as the streaming diagonal kernels of line_stream.cu and as the runtime neighbour list of
// the segment (ero_dil_runtime_nl_se_t.hpp:129-193: the window is clipped at the image border, i.e.
// pixels outside the image are the operator's neutral value).
//
// A CTA (128 threads) owns TW = 256 / sizeof(T) adjacent diagonals over TH output rows, so its output
// tile is a parallelogram leaning with the segment; the tiles of one tile row, shifted by TW pixels,
// cover every pixel of those rows once.  The tile's input, TH + 2K rows, comes in as a staircase of TMA
// boxes: the rows are cut into groups of G = 16 / sizeof(T) rows, the drift of one 16-byte chunk, and
// group g is one 2D box of G rows x (TW + G) pixels that starts G pixels further left (45 degrees) or
// right (135 degrees) than group g - 1.  Every box therefore starts on a 16-byte boundary, the tile
// rows start on a multiple of G, and the boxes together hold the parallelogram plus G pixels a row.  In
// shared memory, diagonal t at row k of a group sits at column t + G - k (45 degrees) or t + k (135).
// Pixels outside the image arrive as TMA's zero fill and are then set to the neutral value (nothing to
// do for the dilation of unsigned pixels, whose neutral value is 0).
//
// Thread t (with, for 4-byte pixels, two thread groups stacked along the tile's rows) then runs van
// Herk / Gil-Werman down diagonal t: the CH windows starting at tile rows R0 .. R0 + CH - 1 (CH the
// largest multiple of G <= 2K + 1, R0 a multiple of G) take the running suffix of block A = rows R0 ..
// R0 + 2K, kept in registers, and the running prefix of the rows after it.  With R0 a multiple of G
// the row's place in its group is known at compile time, so every shared-memory read is one load at a
// constant offset from the thread's column.  Outputs go straight to global memory: the 32 lanes of a
// warp write 32 consecutive pixels of a row.
//
// The wait for the boxes is bounded (tile::kWaitNs of %globaltimer); on expiry the CTA records
// PG_ERR_CUDA in g_diag_status (read by pg_check_device) and leaves its tile unwritten.
#include <atomic>

#include "tile.cuh"

namespace pg {

__device__ int g_diag_status = 0;

namespace {

using namespace tile;
constexpr int kDThreads = 128;

template <typename T, int K> struct DiagGeom {
  static constexpr int S = (int)sizeof(T);
  static constexpr int G = 16 / S;                   // rows per box: one 16-byte chunk of drift
  static constexpr int W2 = 2 * K + 1;               // segment length
  static constexpr int TW = 256 / S;                 // diagonals per tile
  static constexpr int NV = kDThreads / TW;          // thread groups stacked along the tile's rows
  static constexpr int CH = W2 / G * G;              // windows per van Herk chunk
  static constexpr int THG = (120 / NV) / CH * CH;   // output rows per thread group
  static constexpr int TH = NV * THG;                // output rows per tile
  static constexpr int BR = (TH + 2 * K + G - 1) / G * G;  // input rows per tile
  static constexpr int NG = BR / G;                  // boxes per tile
  static constexpr int BWP = TW + G;                 // box width, pixels
  static constexpr int RP = BWP * S;                 // bytes per box row
  static constexpr int GP = (G * RP + 127) / 128 * 128;  // bytes per box in shared memory (TMA: 128-aligned)
  static constexpr int D = (G - K % G) % G;          // tile row b starts at output row b*TH - D, input row - K
  static constexpr unsigned box_bytes = (unsigned)(G * RP);
  static constexpr size_t smem = (size_t)NG * GP + 16;  // + the mbarrier
  static_assert(CH >= G && THG >= CH && kDThreads % TW == 0 && BWP <= 256 && TH % G == 0, "diagonal tile geometry");
  // every shared-memory row a thread reads lies in the tile: the last chunk's prefix ends at row
  // TH - CH + W2 + CH - 2 = TH + 2K - 1
  static_assert(TH + 2 * K <= BR, "diagonal tile rows");
};

// first tile column (in tiles) left of x0 = cx, and the tile columns of the grid
template <typename T, int K, int DIR> struct DiagCols {
  using Gm = DiagGeom<T, K>;
  // 45 degrees: tile bx covers [x0 - d, x0 - d + TW) at output row y0 + d; 135: [x0 + d, x0 + d + TW)
  static constexpr int M0 = DIR > 0 ? 1 : (Gm::TH + Gm::G - 2 + Gm::TW - 1) / Gm::TW;
  static int64_t count(int64_t W) {
    return DIR > 0 ? (W + Gm::TH - 2) / Gm::TW + 2 : (W - 1) / Gm::TW + M0 + 1;
  }
};

__device__ __forceinline__ int pos_mod(int a, int m) { return ((a % m) + m) % m; }

template <typename T, bool SUP, int K, int DIR>
__global__ void __launch_bounds__(kDThreads) k_diag_tile(const __grid_constant__ CUtensorMap tmap, T *__restrict__ out,
                                                         int H, int W) {
  using Gm = DiagGeom<T, K>;
  constexpr int S = Gm::S, G = Gm::G, W2 = Gm::W2, TW = Gm::TW, CH = Gm::CH, THG = Gm::THG, TH = Gm::TH;
  constexpr int BR = Gm::BR, NG = Gm::NG, BWP = Gm::BWP, RP = Gm::RP, GP = Gm::GP;
  using O = Op<T, SUP>;
  extern __shared__ __align__(128) unsigned char s_box[];
  __shared__ int s_ok;
  uint64_t *bar = reinterpret_cast<uint64_t *>(s_box + NG * GP);
  const unsigned bar_a = smem_u32(bar);
  const int tid = threadIdx.x;
  const int y0 = (int)blockIdx.y * TH - Gm::D;  // first output row
  const int ty = y0 - K;                        // first input row, a multiple of G
  const int cx = DIR > 0 ? pos_mod(-y0, G) : pos_mod(y0, G);
  const int x0 = cx + ((int)blockIdx.x - DiagCols<T, K, DIR>::M0) * TW;  // diagonal 0 at row y0
  // box of group g (input rows ty + gG ..): first column, a multiple of G
  auto box_x = [&](int g) { return DIR > 0 ? x0 + K - g * G - G : x0 - K + g * G; };

  if (tid == 0) {
    if (smem_u32(s_box) & 127u) {  // a TMA destination starts on a 128-byte boundary
      atomicCAS(&g_diag_status, 0, (int)PG_ERR_CUDA);
      s_ok = 0;
    } else {
      s_ok = 1;
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a), "r"(NG * Gm::box_bytes)
                   : "memory");
    }
  }
  __syncthreads();
  if (!s_ok) return;
  if (tid < 32) {
    for (int g = tid; g < NG; g += 32)
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
              smem_u32(s_box + g * GP)),
          "l"(&tmap), "r"(box_x(g)), "r"(ty + g * G), "r"(bar_a)
          : "memory");
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

  // pixels outside the image: TMA wrote zeros; the operator needs its neutral value there
  constexpr bool kZeroIsNeutral = std::is_unsigned_v<T> && SUP;
  if constexpr (!kZeroIsNeutral) {
    const int xa = box_x(0), xb = box_x(NG - 1);
    const int xlo = DIR > 0 ? xb : xa, xhi = (DIR > 0 ? xa : xb) + BWP;
    if (ty < 0 || ty + BR > H || xlo < 0 || xhi > W) {
      const T NEU = O::neutral();
      for (int r = tid; r < BR; r += kDThreads) {
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

  // every output pixel of the tile in the image: rows y0 .. y0 + TH - 1, and at row y0 + d columns
  // x0 - d .. x0 - d + TW - 1 (45 degrees) or x0 + d .. x0 + d + TW - 1 (135 degrees)
  const bool inside = y0 >= 0 && y0 + TH <= H &&
                      (DIR > 0 ? x0 - (TH - 1) >= 0 && x0 + TW <= W : x0 >= 0 && x0 + TH - 1 + TW <= W);
  const int t = tid % TW, v = tid / TW;
  const unsigned char *colp = s_box + (DIR > 0 ? t + G : t) * S;
  // row i of a chunk (starting on a group boundary): group i / G, row i % G, column shift -/+ (i % G)
#define PG_DIAG_LD(i) \
  (*reinterpret_cast<const T *>(p + ((i) / G) * GP + ((i) % G) * RP + (DIR > 0 ? -((i) % G) : ((i) % G)) * S))
#pragma unroll 1
  for (int c = 0; c < THG / CH; ++c) {
    const int R0 = v * THG + c * CH;  // tile row of the chunk's first window (a multiple of G)
    const unsigned char *p = colp + (R0 / G) * GP;
    T suf[W2];
    suf[W2 - 1] = PG_DIAG_LD(W2 - 1);
#pragma unroll
    for (int i = W2 - 2; i >= 0; --i) suf[i] = O::apply(suf[i + 1], PG_DIAG_LD(i));
    // window R0 + i is centred on output row y0 + R0 + i, where diagonal t is at column x - i (45) or
    // x + i (135)
    const int y = y0 + R0;
    const int x = DIR > 0 ? x0 + t - R0 : x0 + t + R0;
    T pre = O::neutral();
    if (inside) {  // the whole tile lies in the image: one pointer step per output
      T *o = out + (size_t)y * W + x;
      const int step = DIR > 0 ? W - 1 : W + 1;
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        if (i > 0) pre = O::apply(pre, PG_DIAG_LD(W2 + i - 1));
        *o = i > 0 ? O::apply(suf[i], pre) : suf[0];
        o += step;
      }
    } else {
#pragma unroll
      for (int i = 0; i < CH; ++i) {
        if (i > 0) pre = O::apply(pre, PG_DIAG_LD(W2 + i - 1));
        const T val = i > 0 ? O::apply(suf[i], pre) : suf[0];
        const int yy = y + i, xx = DIR > 0 ? x - i : x + i;
        if ((unsigned)yy < (unsigned)H && (unsigned)xx < (unsigned)W) out[(size_t)yy * W + xx] = val;
      }
    }
  }
#undef PG_DIAG_LD
}

// Tensor map of an image of H rows x W pixels of S bytes, box of bw pixels x rows rows.
pg_status pixel_map(CUtensorMap *map, const void *data, int64_t H, int64_t W, int S, int bw, int rows) {
  auto fn = encode_tiled();
  if (!fn) return fail(PG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  cuuint64_t dims[2] = {(cuuint64_t)W, (cuuint64_t)H};
  cuuint64_t strides[1] = {(cuuint64_t)W * S};
  cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)rows};
  cuuint32_t estr[2] = {1, 1};
  const CUtensorMapDataType dt = S == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16 : CU_TENSOR_MAP_DATA_TYPE_UINT32;
  const CUresult r = fn(map, dt, 2, const_cast<void *>(data), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(PG_ERR_CUDA, "cuTensorMapEncodeTiled failed for the diagonal tile");
  return PG_OK;
}

template <typename T, bool SUP, int K, int DIR>
pg_status diag_tile(const pg_image &in, const pg_image &out, cudaStream_t s) {
  using Gm = DiagGeom<T, K>;
  const Dims d = dims_of(in);
  const int64_t H = d.ny, W = d.nx;
  CUtensorMap map;
  PG_TRY(pixel_map(&map, in.data, H, W, Gm::S, Gm::BWP, Gm::G));
  static std::atomic<uint64_t> attr_devices{0};
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  const uint64_t bit = 1ull << (dev & 63);
  if (!(attr_devices.load() & bit)) {
    PG_CUDA_TRY(cudaFuncSetAttribute(k_diag_tile<T, SUP, K, DIR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)Gm::smem),
                "diagonal tile smem attribute");
    attr_devices.fetch_or(bit);
  }
  const dim3 grid((unsigned)DiagCols<T, K, DIR>::count(W), (unsigned)ceil_div(H + Gm::D, Gm::TH));
  k_diag_tile<T, SUP, K, DIR><<<grid, kDThreads, Gm::smem, s>>>(map, static_cast<T *>(out.data), (int)H, (int)W);
  return cuda_status(cudaGetLastError(), "diagonal tile launch");
}

template <typename T, bool SUP, int DIR>
pg_status diag_k(const pg_image &in, const pg_image &out, int k, cudaStream_t s) {
  switch (k) {
    case 7: return diag_tile<T, SUP, 7, DIR>(in, out, s);
    case 15: return diag_tile<T, SUP, 15, DIR>(in, out, s);
    default: return diag_tile<T, SUP, 31, DIR>(in, out, s);
  }
}

template <typename T, bool SUP>
pg_status diag_dir(const pg_image &in, const pg_image &out, int dx, int k, cudaStream_t s) {
  // dx = -1 (with dy = 1): x + y constant, 45 degrees; dx = +1: x - y constant, 135 degrees
  return dx < 0 ? diag_k<T, SUP, 1>(in, out, k, s) : diag_k<T, SUP, -1>(in, out, k, s);
}

}  // namespace

bool try_diag_tile(const pg_image &in, const pg_image &out, int dy, int dx, int k, bool dilate, cudaStream_t s,
                   pg_status *st) {
  if (in.rank != 2 || dy != 1 || (dx != 1 && dx != -1) || !(k == 7 || k == 15 || k == 31)) return false;
  const int es = elem_size(in.ptype);
  if (!(in.ptype == PG_PTYPE_U16 || in.ptype == PG_PTYPE_I32 || in.ptype == PG_PTYPE_F32)) return false;
  const Dims d = dims_of(in);
  const int64_t H = d.ny, W = d.nx;
  // the tensor map wants a 16-byte aligned base and rows of a multiple of 16 bytes
  if (H < 1 || W < 1 || (W * es) % 16 != 0 || reinterpret_cast<uintptr_t>(in.data) % 16 != 0) return false;
  if (reinterpret_cast<uintptr_t>(out.data) % es != 0) return false;
  if (H > (1 << 30) || W > (1 << 30) || ceil_div(H + 16, 56) > 65535) return false;
  switch (in.ptype) {
    case PG_PTYPE_U16:
      *st = dilate ? diag_dir<uint16_t, true>(in, out, dx, k, s) : diag_dir<uint16_t, false>(in, out, dx, k, s);
      return true;
    case PG_PTYPE_I32:
      *st = dilate ? diag_dir<int32_t, true>(in, out, dx, k, s) : diag_dir<int32_t, false>(in, out, dx, k, s);
      return true;
    default:
      *st = dilate ? diag_dir<float, true>(in, out, dx, k, s) : diag_dir<float, false>(in, out, dx, k, s);
      return true;
  }
}

int take_diag_status() {
  int st = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&st, g_diag_status, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  if (st != 0 && cudaMemcpyToSymbol(g_diag_status, &zero, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  return st;
}

}  // namespace pg
