// tile.cuh -- pieces shared by the shared-memory tile kernels (rect.cu, rect_open.cu): the TMA tile
// copy with its bounded mbarrier wait, word / pixel helpers, and the register van Herk / Gil-Werman
// scans of a tile row and of a tile column.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "common.cuh"
#include "words.cuh"

namespace pg {
namespace tile {

constexpr int kThreads = 128;                          // threads = input rows of a tile
constexpr unsigned long long kWaitNs = 1000000000ull;  // bound of the tile-copy wait: 1 s

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
// a - b per pixel of a word, where a >= b in every pixel (a dilation minus an erosion): packed
// unsigned pixels never borrow from the next lane, so one 32-bit subtraction is exact; i32 wraps like
// the difference kernel's int arithmetic; f32 is one rounded subtraction, as there
template <typename T> __device__ __forceinline__ uint32_t wdiff(uint32_t a, uint32_t b) {
  if constexpr (std::is_same_v<T, float>) return __float_as_uint(__uint_as_float(a) - __uint_as_float(b));
  else return a - b;
}
template <typename T> __device__ __forceinline__ uint32_t bits_of(T v) {
  if constexpr (std::is_same_v<T, float>) return __float_as_uint(v);
  else return (uint32_t)v;
}

// Row scan of one tile row (registers), in place: stream pixel q is tile pixel P0 + q, output
// pixel j (tile pixel HW*E + j) is formed at q = j + 2K.  With GRAD both the dilation (in place) and
// the erosion (into `mrow`) are formed from the same pixels.
// Row scan of 2-byte pixels kept in pairs (word m = pixels 2m, 2m + 1), K = 2k + 1 odd, NOUT output
// words from word OUT0, in place.  With A(m) = op over words [m - k, m + k] and B(m) = op(A(m), word
// m - k - 1), pixel 2m's window [2m - K, 2m + K] holds the even pixels of A(m) and the odd pixels of
// B(m), and pixel 2m + 1's window the odd pixels of A(m) and the even pixels of B(m + 1), so
//   out word m = op(A(m), (odd half of B(m), even half of B(m + 1))).
// One van Herk / Gil-Werman scan over words (window 2k + 1) gives A; the word k + 1 left of A(m)'s
// window is the same register of the previous block.  Output word m - 1 is formed with A(m).
template <bool SUP, int K, int NOUT, int OUT0, bool GRAD>
__device__ __forceinline__ void row_scan_pairs(uint32_t *row, uint32_t *mrow) {
  using T = uint16_t;
  constexpr bool SA = GRAD ? true : SUP;    // GRAD: dilation in place, erosion into mrow
  constexpr int k = (K - 1) / 2, W = 2 * k + 1;
  constexpr int Q0 = OUT0 - k - 1;          // stream word 0 (a multiple of 4)
  constexpr int NQ = NOUT + 2 * k + 2;      // words Q0 .. OUT0 + NOUT + k
  constexpr int NB = (NQ + W - 1) / W;
  static_assert(K % 2 == 1 && Q0 >= 0 && Q0 % 4 == 0 && OUT0 % 4 == 0 && NOUT % 4 == 0, "pair scan geometry");
  const uint32_t NA = splat<T>(Op<T, SA>::neutral()), NBW = splat<T>(Op<T, false>::neutral());
  uint32_t sa[W], sb[GRAD ? W : 1], prev[W];
#pragma unroll
  for (int i = 0; i < W; ++i) {
    sa[i] = NA;
    prev[i] = NA;
    if constexpr (GRAD) sb[i] = NBW;
  }
  uint32_t cw[4] = {0, 0, 0, 0}, acca[4] = {0, 0, 0, 0}, accb[4] = {0, 0, 0, 0};
  uint32_t a_last = NA, b_last = NA, c_last = NBW, d_last = NBW;  // A(m - 1), B(m - 1) per operator
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    uint32_t raw[W];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      const int s = b * W + i;
      if (s < NQ) {
        const int q = Q0 + s;
        if (q % 4 == 0) {
          const uint4 v = *reinterpret_cast<const uint4 *>(row + q);
          cw[0] = v.x; cw[1] = v.y; cw[2] = v.z; cw[3] = v.w;
        }
        raw[i] = cw[q % 4];
      } else {
        raw[i] = NA;  // beyond the stream: feeds no output
      }
    }
    uint32_t pa = raw[0], pb = raw[0];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      if (i > 0) {
        pa = wop<T, SA>(pa, raw[i]);
        if constexpr (GRAD) pb = wop<T, false>(pb, raw[i]);
      }
      const int j = b * W + i - 2 * k;  // window start in the stream: A(m), m = Q0 + j + k
      if (j >= 0) {
        const int mo = Q0 + j + k - 1 - OUT0;  // output word (from OUT0) formed now
        const uint32_t A = (i < W - 1) ? wop<T, SA>(sa[i + 1], pa) : pa;
        const uint32_t B = wop<T, SA>(A, b > 0 ? prev[i] : NA);  // stream word j - 1 = one block back
        if (mo >= 0 && mo < NOUT) acca[mo % 4] = wop<T, SA>(a_last, __byte_perm(b_last, B, 0x5432));
        a_last = A;
        b_last = B;
        if constexpr (GRAD) {
          const uint32_t C = (i < W - 1) ? wop<T, false>(sb[i + 1], pb) : pb;
          const uint32_t D = wop<T, false>(C, b > 0 ? prev[i] : NBW);
          if (mo >= 0 && mo < NOUT) accb[mo % 4] = wop<T, false>(c_last, __byte_perm(d_last, D, 0x5432));
          c_last = C;
          d_last = D;
        }
        if (mo >= 0 && mo < NOUT && mo % 4 == 3) {
          *reinterpret_cast<uint4 *>(row + OUT0 + mo - 3) = make_uint4(acca[0], acca[1], acca[2], acca[3]);
          if constexpr (GRAD)
            *reinterpret_cast<uint4 *>(mrow + mo - 3) = make_uint4(accb[0], accb[1], accb[2], accb[3]);
        }
      }
    }
    sa[W - 1] = raw[W - 1];
    if constexpr (GRAD) sb[W - 1] = raw[W - 1];
#pragma unroll
    for (int i = W - 2; i >= 0; --i) {
      sa[i] = wop<T, SA>(sa[i + 1], raw[i]);
      if constexpr (GRAD) sb[i] = wop<T, false>(sb[i + 1], raw[i]);
    }
#pragma unroll
    for (int i = 0; i < W; ++i) prev[i] = raw[i];
  }
}

template <typename T, bool SUP, int K, int TW, int HW, bool GRAD>
__device__ __forceinline__ void row_scan(uint32_t *row, uint32_t *mrow) {
  if constexpr (sizeof(T) == 2 && K % 2 == 1 && HW - (K + 1) / 2 >= 0 && (HW - (K + 1) / 2) % 4 == 0) {
    row_scan_pairs<SUP, K, TW, HW, GRAD>(row, mrow);  // whole words, about half the operations per pixel
    return;
  }
  constexpr int E = 4 / (int)sizeof(T), W = 2 * K + 1;
  constexpr int NQ = TW * E + 2 * K, NB = (NQ + W - 1) / W, P0 = HW * E - K;
  constexpr int CH = 4 * E;  // pixels per 16-byte chunk
  using A = Op<T, GRAD ? true : SUP>;
  using B = Op<T, false>;
  T sa[W], sb[GRAD ? W : 1];
#pragma unroll
  for (int i = 0; i < W; ++i) {
    sa[i] = A::neutral();
    if constexpr (GRAD) sb[i] = B::neutral();
  }
  uint32_t cw[4] = {0, 0, 0, 0}, acca[4] = {0, 0, 0, 0}, accb[4] = {0, 0, 0, 0};
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
        raw[i] = A::neutral();  // beyond the stream: feeds no output
      }
    }
    T pa = raw[0], pb = raw[0];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      if (i > 0) {
        pa = A::apply(pa, raw[i]);
        if constexpr (GRAD) pb = B::apply(pb, raw[i]);
      }
      const int j = b * W + i - 2 * K;
      if (j >= 0 && j < TW * E) {
        const int sh = 8 * (int)sizeof(T) * (j % E), wi = (j / E) % 4;
        const uint32_t va = bits_of<T>((i < W - 1) ? A::apply(sa[i + 1], pa) : pa);
        acca[wi] = (j % E == 0) ? va : (acca[wi] | (va << sh));
        if constexpr (GRAD) {
          const uint32_t vb = bits_of<T>((i < W - 1) ? B::apply(sb[i + 1], pb) : pb);
          accb[wi] = (j % E == 0) ? vb : (accb[wi] | (vb << sh));
        }
        if (j % CH == CH - 1) {
          *reinterpret_cast<uint4 *>(row + HW + (j / CH) * 4) = make_uint4(acca[0], acca[1], acca[2], acca[3]);
          if constexpr (GRAD)
            *reinterpret_cast<uint4 *>(mrow + (j / CH) * 4) = make_uint4(accb[0], accb[1], accb[2], accb[3]);
        }
      }
    }
    sa[W - 1] = raw[W - 1];
    if constexpr (GRAD) sb[W - 1] = raw[W - 1];
#pragma unroll
    for (int i = W - 2; i >= 0; --i) {
      sa[i] = A::apply(sa[i + 1], raw[i]);
      if constexpr (GRAD) sb[i] = B::apply(sb[i + 1], raw[i]);
    }
  }
}

// Column scan of THG output rows (registers) from words `ca` (stride SA) -- and, with GRAD, the
// erosion from `cb` (stride SB) -- written to out[row y0 + j0 + j][gx] (GRAD: dilation - erosion).
template <typename T, bool SUP, int K, int THG, int TH, int TR, int SA, int SB, bool GRAD>
__device__ __forceinline__ void col_scan(const uint32_t *ca, const uint32_t *cb, uint32_t *__restrict__ out,
                                         int j0, int y0, int gx, int H, int Wn) {
  constexpr int W = 2 * K + 1, NB = (THG + 2 * K + W - 1) / W;
  constexpr bool SUPA = GRAD ? true : SUP;
  const uint32_t NA = splat<T>(Op<T, SUPA>::neutral()), NBW = splat<T>(Op<T, false>::neutral());
  uint32_t sa[W], sb[GRAD ? W : 1];
#pragma unroll
  for (int i = 0; i < W; ++i) {
    sa[i] = NA;
    if constexpr (GRAD) sb[i] = NBW;
  }
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    uint32_t ra[W], rb[GRAD ? W : 1];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      const int q = b * W + i;
      const bool in = q < THG + 2 * K && j0 + q < TR;
      ra[i] = in ? ca[q * SA] : NA;
      if constexpr (GRAD) rb[i] = in ? cb[q * SB] : NBW;
    }
    uint32_t pa = ra[0], pb = 0u;
    if constexpr (GRAD) pb = rb[0];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      if (i > 0) {
        pa = wop<T, SUPA>(pa, ra[i]);
        if constexpr (GRAD) pb = wop<T, false>(pb, rb[i]);
      }
      const int j = b * W + i - 2 * K;
      if (j >= 0 && j < THG && j0 + j < TH) {
        const int gy = y0 + j0 + j;
        if (gy < H && gx < Wn) {
          uint32_t v = (i < W - 1) ? wop<T, SUPA>(sa[i + 1], pa) : pa;
          if constexpr (GRAD) v = wdiff<T>(v, (i < W - 1) ? wop<T, false>(sb[i + 1], pb) : pb);
          out[(size_t)gy * Wn + gx] = v;
        }
      }
    }
    sa[W - 1] = ra[W - 1];
    if constexpr (GRAD) sb[W - 1] = rb[W - 1];
#pragma unroll
    for (int i = W - 2; i >= 0; --i) {
      sa[i] = wop<T, SUPA>(sa[i + 1], ra[i]);
      if constexpr (GRAD) sb[i] = wop<T, false>(sb[i + 1], rb[i]);
    }
  }
}


// TMA copy of the box at word tx, row ty (slice tz for a 3D map) into s (bytes long), completing on
// the mbarrier `bar`; thread 0 waits at most kWaitNs and records PG_ERR_CUDA in *status on expiry (and
// refuses to copy into an s that is not 128-byte aligned).  Returns, for every thread of the CTA,
// whether the tile arrived (one __syncthreads inside).
template <int NDIM = 2>
__device__ __forceinline__ bool load_box(const CUtensorMap *map, uint32_t *s, uint64_t *bar, unsigned bytes, int tx,
                                         int ty, int tz, int *status, int *s_ok) {
  const unsigned bar_a = smem_u32(bar);
  if (threadIdx.x == 0 && (smem_u32(s) & 127u)) {  // a TMA destination starts on a 128-byte boundary
    atomicCAS(status, 0, (int)PG_ERR_CUDA);
    *s_ok = 0;
  } else if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a), "r"(bytes) : "memory");
    if constexpr (NDIM == 2)
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
              smem_u32(s)),
          "l"(map), "r"(tx), "r"(ty), "r"(bar_a)
          : "memory");
    else
      asm volatile(
          "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
              smem_u32(s)),
          "l"(map), "r"(tx), "r"(ty), "r"(tz), "r"(bar_a)
          : "memory");
    bool done = mbar_try(bar_a, 0);
    const unsigned long long t0 = now_ns();
    while (!done && now_ns() - t0 < kWaitNs) done = mbar_try(bar_a, 0);
    if (!done) atomicCAS(status, 0, (int)PG_ERR_CUDA);
    *s_ok = done;
  }
  __syncthreads();
  if (!*s_ok) return false;
  (void)mbar_try(bar_a, 0);  // the phase is complete: each thread observes it (acquire)
  return true;
}

__device__ __forceinline__ bool load_tile(const CUtensorMap *map, uint32_t *s, uint64_t *bar, unsigned bytes, int tx,
                                          int ty, int *status, int *s_ok) {
  return load_box<2>(map, s, bar, bytes, tx, ty, 0, status, s_ok);
}

inline PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
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

// Tensor map of an image of H rows x Wn 32-bit words, box of bw words x rows rows.
inline pg_status word_map(CUtensorMap *map, const void *data, int64_t H, int64_t Wn, int bw, int rows) {
  auto fn = encode_tiled();
  if (!fn) return fail(PG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  cuuint64_t dims[2] = {(cuuint64_t)Wn, (cuuint64_t)H};
  cuuint64_t strides[1] = {(cuuint64_t)Wn * 4};
  cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)rows};
  cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<void *>(data), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(PG_ERR_CUDA, "cuTensorMapEncodeTiled failed for the image tile");
  return PG_OK;
}

// Tensor map of a volume of D slices x H rows x Wn 32-bit words, box of bw words x rows x slices.
inline pg_status word_map3(CUtensorMap *map, const void *data, int64_t D, int64_t H, int64_t Wn, int bw, int rows,
                           int slices) {
  auto fn = encode_tiled();
  if (!fn) return fail(PG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  cuuint64_t dims[3] = {(cuuint64_t)Wn, (cuuint64_t)H, (cuuint64_t)D};
  cuuint64_t strides[2] = {(cuuint64_t)Wn * 4, (cuuint64_t)(Wn * H) * 4};
  cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)rows, (cuuint32_t)slices};
  cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, const_cast<void *>(data), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(PG_ERR_CUDA, "cuTensorMapEncodeTiled failed for the volume tile");
  return PG_OK;
}

}  // namespace tile
}  // namespace pg
