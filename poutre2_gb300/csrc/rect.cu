// rect.cu -- erosion / dilation by the (2KY+1) x (2KX+1) box in one pass through shared memory: the
// square (KY = KX), the X segment (KY = 0) and the Y segment (KX = 0), for K = 7, 15, 31.
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
// The wait on the mbarrier is bounded (kRectWaitNs of %globaltimer); on expiry the CTA records
// PG_ERR_CUDA in g_rect_status (read by pg_check_device) and leaves its tile unwritten.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <mutex>

#include "common.cuh"
#include "words.cuh"

namespace pg {

__device__ int g_rect_status = 0;

namespace {

constexpr int kRThreads = 128;                             // = input rows per tile
constexpr unsigned long long kRectWaitNs = 1000000000ull;  // 1 s

template <typename T, int KY, int KX> struct RectGeom {
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
  static constexpr size_t tile_bytes = (size_t)TR * BW * 4;
  static constexpr size_t smem = tile_bytes + 16;               // + the mbarrier
  static_assert(BW <= 256 && TH > 0 && kRThreads % TW == 0, "tile geometry");
};

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool mbar_try(unsigned bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

template <typename T> __device__ __forceinline__ T px_of(uint32_t w, int k) {
  if constexpr (std::is_same_v<T, float>) return __uint_as_float(w);
  else if constexpr (sizeof(T) == 4) return (T)w;
  else return (T)(w >> (8 * (int)sizeof(T) * k));
}
template <typename T> __device__ __forceinline__ uint32_t bits_of(T v) {
  if constexpr (std::is_same_v<T, float>) return __float_as_uint(v);
  else return (uint32_t)v;
}

template <typename T, bool SUP, int KY, int KX>
__global__ void __launch_bounds__(kRThreads, 1) k_rect_fused(const __grid_constant__ CUtensorMap tmap,
                                                          uint32_t *__restrict__ out, int H, int Wn) {
  using G = RectGeom<T, KY, KX>;
  constexpr int E = G::E, HW = G::HW, BW = G::BW, TR = G::TR, TH = G::TH, TW = G::TW, THG = G::THG;
  using O = Op<T, SUP>;
  extern __shared__ __align__(128) uint32_t s_tile[];
  __shared__ int s_ok;
  uint64_t *bar = reinterpret_cast<uint64_t *>(s_tile + TR * BW);
  const unsigned bar_a = smem_u32(bar);
  const int t = threadIdx.x;
  const int wx0 = blockIdx.x * TW;         // first centre word
  const int y0 = blockIdx.y * TH;          // first output row
  const int tx = wx0 - HW, ty = y0 - KY;   // tile origin: word (a multiple of 4), row

  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a), "r"((unsigned)G::tile_bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(s_tile)),
        "l"(&tmap), "r"(tx), "r"(ty), "r"(bar_a)
        : "memory");
    bool done = mbar_try(bar_a, 0);
    const unsigned long long t0 = now_ns();
    while (!done && now_ns() - t0 < kRectWaitNs) done = mbar_try(bar_a, 0);
    if (!done) atomicCAS(&g_rect_status, 0, (int)PG_ERR_CUDA);
    s_ok = done;
  }
  __syncthreads();
  if (!s_ok) return;
  (void)mbar_try(bar_a, 0);  // the phase is complete: each thread observes it (acquire)

  // pixels outside the image (TMA fills them with zeros) become neutral
  if (tx < 0 || ty < 0 || tx + BW > Wn || ty + TR > H) {
    const uint32_t NEUW = splat<T>(O::neutral());
    for (int r = 0; r < TR; ++r) {
      const bool row_out = ty + r < 0 || ty + r >= H;
      for (int c = t; c < BW; c += kRThreads)
        if (row_out || tx + c < 0 || tx + c >= Wn) s_tile[r * BW + c] = NEUW;
    }
    __syncthreads();
  }

  // ---- row pass: thread t scans input row t; stream pixel q is tile pixel P0 + q, output pixel j
  // (tile pixel HW*E + j) is formed at q = j + 2KX
  if constexpr (KX > 0) {
    constexpr int K = KX, W = 2 * K + 1;
    uint32_t *row = s_tile + t * BW;
    constexpr int NQ = TW * E + 2 * K;
    constexpr int NB = (NQ + W - 1) / W;
    constexpr int P0 = HW * E - K;
    constexpr int CH = 4 * E;  // pixels per 16-byte chunk
    T suf[W];
#pragma unroll
    for (int i = 0; i < W; ++i) suf[i] = O::neutral();
    uint32_t cw[4] = {0, 0, 0, 0}, acc[4] = {0, 0, 0, 0};
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      T raw[W];
#pragma unroll
      for (int i = 0; i < W; ++i) {
        const int q = b * W + i;
        if (q < NQ) {
          const int p = P0 + q;
          if (q == 0 || p % CH == 0) {
            const uint4 v = *reinterpret_cast<const uint4 *>(row + (p / CH) * 4);
            cw[0] = v.x; cw[1] = v.y; cw[2] = v.z; cw[3] = v.w;
          }
          raw[i] = px_of<T>(cw[(p / E) % 4], p % E);
        } else {
          raw[i] = O::neutral();
        }
      }
      T pre = raw[0];
#pragma unroll
      for (int i = 0; i < W; ++i) {
        if (i > 0) pre = O::apply(pre, raw[i]);
        const int j = b * W + i - 2 * K;
        if (j >= 0 && j < TW * E) {
          const T r = (i < W - 1) ? O::apply(suf[i + 1], pre) : pre;
          const uint32_t v = bits_of<T>(r);
          if (j % E == 0) acc[(j / E) % 4] = v;
          else acc[(j / E) % 4] |= v << (8 * (int)sizeof(T) * (j % E));
          if (j % CH == CH - 1)
            *reinterpret_cast<uint4 *>(row + HW + (j / CH) * 4) = make_uint4(acc[0], acc[1], acc[2], acc[3]);
        }
      }
      suf[W - 1] = raw[W - 1];
#pragma unroll
      for (int i = W - 2; i >= 0; --i) suf[i] = O::apply(suf[i + 1], raw[i]);
    }
    __syncthreads();
  }

  // ---- column pass: thread t scans centre word column HW + t % TW over the rows of output group
  // t / TW (THG output rows, from tile row j0); output row j0 + j is formed at q = j + 2KY.  Without
  // a vertical extent the centre words are copied out.
  const int j0 = (t / TW) * THG;
  const uint32_t *col = s_tile + j0 * BW + HW + t % TW;
  const int gx = wx0 + t % TW;
  if constexpr (KY == 0) {
    if (gx < Wn)
#pragma unroll 4
      for (int j = 0; j < THG && j0 + j < TH && y0 + j0 + j < H; ++j) out[(size_t)(y0 + j0 + j) * Wn + gx] = col[j * BW];
  } else {
    constexpr int K = KY, W = 2 * K + 1;
    const uint32_t NEUW = splat<T>(O::neutral());
    constexpr int NB = (THG + 2 * K + W - 1) / W;
    uint32_t suf[W];
#pragma unroll
    for (int i = 0; i < W; ++i) suf[i] = NEUW;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      uint32_t raw[W];
#pragma unroll
      for (int i = 0; i < W; ++i) {
        const int q = b * W + i;
        raw[i] = (q < THG + 2 * K && j0 + q < TR) ? col[q * BW] : NEUW;
      }
      uint32_t pre = raw[0];
#pragma unroll
      for (int i = 0; i < W; ++i) {
        if (i > 0) pre = wop<T, SUP>(pre, raw[i]);
        const int j = b * W + i - 2 * K;
        if (j >= 0 && j < THG && j0 + j < TH) {
          const int gy = y0 + j0 + j;
          if (gy < H && gx < Wn) out[(size_t)gy * Wn + gx] = (i < W - 1) ? wop<T, SUP>(suf[i + 1], pre) : pre;
        }
      }
      suf[W - 1] = raw[W - 1];
#pragma unroll
      for (int i = W - 2; i >= 0; --i) suf[i] = wop<T, SUP>(suf[i + 1], raw[i]);
    }
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      (void)cudaGetLastError();
  });
  return fn;
}

template <typename T, bool SUP, int KY, int KX>
pg_status rect_fused(const pg_image &in, const pg_image &out, cudaStream_t s) {
  using G = RectGeom<T, KY, KX>;
  const Dims d = dims_of(in);
  const int64_t H = d.ny, Wn = d.nx / G::E;
  auto fn = encode_tiled();
  if (!fn) return fail(PG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  CUtensorMap map;
  cuuint64_t dims[2] = {(cuuint64_t)Wn, (cuuint64_t)H};
  cuuint64_t strides[1] = {(cuuint64_t)Wn * 4};
  cuuint32_t box[2] = {(cuuint32_t)G::BW, (cuuint32_t)G::TR};
  cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(&map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, in.data, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(PG_ERR_CUDA, "cuTensorMapEncodeTiled failed for the rectangle tile");
  // the opt-in shared-memory size is a per-device attribute of each instantiation
  static std::atomic<uint64_t> attr_devices{0};
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  const uint64_t bit = 1ull << (dev & 63);
  if (!(attr_devices.load() & bit)) {
    PG_CUDA_TRY(cudaFuncSetAttribute(k_rect_fused<T, SUP, KY, KX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)G::smem),
                "tile kernel smem attribute");
    attr_devices.fetch_or(bit);
  }
  const dim3 grid((unsigned)ceil_div(Wn, G::TW), (unsigned)ceil_div(H, G::TH));
  k_rect_fused<T, SUP, KY, KX><<<grid, kRThreads, G::smem, s>>>(map, static_cast<uint32_t *>(out.data), (int)H, (int)Wn);
  return cuda_status(cudaGetLastError(), "tile erosion / dilation launch");
}

// (hy, hx): (k, k) square, (0, k) X segment, (k, 0) Y segment, k in {7, 15, 31}
template <typename T, bool SUP>
pg_status rect_fused_k(const pg_image &in, const pg_image &out, int hy, int hx, cudaStream_t s) {
  if (hy == hx) {
    switch (hy) {
      case 7: return rect_fused<T, SUP, 7, 7>(in, out, s);
      case 15: return rect_fused<T, SUP, 15, 15>(in, out, s);
      default: return rect_fused<T, SUP, 31, 31>(in, out, s);
    }
  }
  if (hy == 0) {
    switch (hx) {
      case 7: return rect_fused<T, SUP, 0, 7>(in, out, s);
      case 15: return rect_fused<T, SUP, 0, 15>(in, out, s);
      default: return rect_fused<T, SUP, 0, 31>(in, out, s);
    }
  }
  switch (hy) {
    case 7: return rect_fused<T, SUP, 7, 0>(in, out, s);
    case 15: return rect_fused<T, SUP, 15, 0>(in, out, s);
    default: return rect_fused<T, SUP, 31, 0>(in, out, s);
  }
}

}  // namespace

bool try_rect_fused(const pg_image &in, const pg_image &out, int64_t hy, int64_t hx, bool dilate, cudaStream_t s,
                    pg_status *st) {
  auto ok_k = [](int64_t k) { return k == 7 || k == 15 || k == 31; };
  if (in.rank != 2 || !((hy == hx && ok_k(hy)) || (hy == 0 && ok_k(hx)) || (hx == 0 && ok_k(hy)))) return false;
  const int es = elem_size(in.ptype);
  // 2- and 4-byte pixels (for u8 the row pass's register window spills; the two line passes run)
  if (es != 2 && es != 4) return false;
  const Dims d = dims_of(in);
  const int64_t H = d.ny, Wd = d.nx;
  if (H < 1 || Wd < 1 || (Wd * es) % 16 != 0) return false;
  if ((reinterpret_cast<uintptr_t>(in.data) | reinterpret_cast<uintptr_t>(out.data)) % 16 != 0) return false;
  if (H > (1 << 30) || Wd * es / 4 > (1 << 30) || ceil_div(H, kRThreads - 2 * hy) > 65535) return false;
  const int y = (int)hy, x = (int)hx;
  switch (in.ptype) {
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

int take_rect_status() {
  int st = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&st, g_rect_status, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  if (st != 0 && cudaMemcpyToSymbol(g_rect_status, &zero, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  return st;
}

}  // namespace pg
