// recon.cu -- geodesic reconstruction (by dilation / erosion) as one persistent kernel, and
// the filters built on it: h-extrema (marker made on the fly), low/high leveling (mask and
// final clip made on the fly), binary h-maxima (comparison fused), ragged batches.
//
// Reference: t_ReconstructionViewDispatcher (geodesy/details/mreconstruct_t.hpp:84-195), a
// sequential Vincent hybrid (raster scan, anti-raster scan, FIFO).  Its result is the
// least fixpoint rec = min(mask, dilate(rec)) above min(marker, mask) (dual for erosion),
// which is unique, so any order of monotone updates reaches the same image: the parallel
// scheme below is bit-exact with it.  Leveling (leveling_t.hpp:45-202) is the same fixpoint
// with mask max(marker, ref) (low) / min(marker, ref) (high) followed by a clip by ref.
//
// GPU design
//  * The image is cut into 64x64 tiles.  A CTA (64 threads) stages a tile of the current
//    reconstruction plus a one-pixel halo, and the tile's mask, in shared memory and iterates
//    directional sweeps there -- down, up (thread per column), right, left (thread per row),
//    each propagating along its whole direction in one pass -- until a full sweep set
//    changes nothing: a tile-local fixpoint.  It writes the tile back and flags the
//    neighbouring tiles whose shared border changed.
//  * A persistent cooperative grid (all CTAs resident) runs rounds over the flagged tiles
//    (round 0: all tiles, marker computed from the inputs), separated by a grid barrier,
//    until a round flags nothing.  Flags live in a double-buffered device worklist; the
//    "any flag" word is triple-buffered so no CTA resets a word another may still read.
//  * Reads of other tiles' pixels bypass L1 (ld.global.cg): values only grow (shrink for
//    erosion), so a concurrently updated halo value is either the old or the new one, both
//    below the fixpoint; a tile that saw an old value is re-flagged by its writer.
//  * Every wait is bounded: the grid barrier gives up after kBarrierTimeoutNs and the round
//    loop after max_rounds, recording PG_ERR_NOT_CONVERGED in a device status word.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>

#include "common.cuh"

namespace pg {

// tile side = threads per CTA: 64 (32 for 8-byte pixels, to keep the staged tile within the
// 48 KB static shared-memory limit)
template <typename T> __host__ __device__ constexpr int tile_side() { return sizeof(T) == 8 ? 32 : 64; }
static constexpr int kMaxSweeps = 512;
static constexpr unsigned long long kBarrierTimeoutNs = 4000000000ull;  // 4 s

// Device-wide sticky status of the reconstruction kernels (0 = ok) and the round count of
// the last completed launch.
__device__ int g_recon_status = 0;
__device__ int g_recon_rounds = 0;

struct RImg {
  const void *marker;  // marker (INIT_MARKER and the leveling masks)
  const void *mask;    // mask, or the leveling reference
  void *rec;           // reconstruction buffer
  void *out;           // epilogue output (binary u8 image, or == rec)
  int64_t H, W;
  int tiles_x, tiles_y;
  int tile_begin;
  int pad;
};

struct RCtl {
  unsigned any[3];
  unsigned bar_count;
  unsigned bar_gen;
  int status;
  int rounds;
  int pad;
};

template <typename T> struct RParams {
  RImg single;        // used when nimg == 1
  const RImg *imgs;   // device table when nimg > 1
  int nimg;
  int ntiles;
  RCtl *ctl;
  unsigned *flags;    // 2 * ntiles
  int max_rounds;
  int max_sweeps = kMaxSweeps;  // sweep sets per tile visit before the tile yields (and re-flags itself)
  int init, mask_mode, epi;
  T h;
};

// row pitch (in pixels) of a shared tile: a row spans an odd number of 32-bit words so that
// thread-per-row sweeps touch 32 distinct banks
template <typename T> __host__ __device__ constexpr int tile_pitch(int cols) {
  if constexpr (sizeof(T) <= 4) {
    int words = (cols * (int)sizeof(T) + 3) / 4;
    if (words % 2 == 0) ++words;
    return words * 4 / (int)sizeof(T);
  } else {
    return cols | 1;
  }
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void set_status(RCtl *ctl, int code) {
  atomicCAS(&ctl->status, 0, code);
  atomicCAS(&g_recon_status, 0, code);
}

// Grid barrier with a bounded wait.  Returns false once any CTA recorded an error; thread 0
// reads the status for its whole CTA so that every thread takes the same branch afterwards.
__device__ bool grid_barrier(RCtl *ctl) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *genp = &ctl->bar_gen;
    const unsigned gen = *genp;
    __threadfence();
    const unsigned arrived = atomicAdd(&ctl->bar_count, 1u) + 1u;
    if (arrived == gridDim.x) {
      atomicExch(&ctl->bar_count, 0u);
      __threadfence();
      atomicAdd(&ctl->bar_gen, 1u);
    } else {
      const unsigned long long t0 = global_ns();
      unsigned ns = 32;
      while (*genp == gen) {
        __nanosleep(ns);
        if (ns < 1024) ns <<= 1;
        if (global_ns() - t0 > kBarrierTimeoutNs) {
          set_status(ctl, PG_ERR_NOT_CONVERGED);
          break;
        }
      }
    }
    __threadfence();
    s_ok = *((volatile int *)&ctl->status) == 0;
  }
  __syncthreads();
  return s_ok != 0;
}

template <typename T, bool SUP>
__device__ __forceinline__ T sat_shift(T m, T h) {
  // marker of h-maxima (sat_sub) / h-minima (sat_add), op_Saturated_{Sub,Add}_Constant
  // (pixel_processing/details/arith_op_t.hpp:218-345), clamped to the pixel type's range
  if constexpr (std::is_integral_v<T>) {
    using Wide = std::conditional_t<(sizeof(T) < 4), int, std::conditional_t<(sizeof(T) < 8), long long, __int128>>;
    const Wide r = SUP ? (Wide)m - (Wide)h : (Wide)m + (Wide)h;
    if (r < (Wide)Lim<T>::lo()) return Lim<T>::lo();
    if (r > (Wide)Lim<T>::hi()) return Lim<T>::hi();
    return (T)r;
  } else {
    return SUP ? m - h : m + h;
  }
}

// Effective mask and initial value of a pixel from its loaded inputs -- `a` the mask (the
// leveling reference), `mk` the marker, loaded only when needs_marker() says so -- kept apart
// from the loads so that a caller can issue the loads of many pixels before it waits for the
// first.  Round 0 starts from select_marker: min(marker, mask) (max for erosion).
template <typename T>
__device__ __forceinline__ bool needs_marker(const RParams<T> &P, int round) {
  return P.init != INIT_SAT_CONST && (round == 0 || P.mask_mode != MASK_PLAIN);
}
template <typename T, bool SUP>
__device__ __forceinline__ void combine_init(const RParams<T> &P, T a, T mk, T &mask, T &init) {
  if (P.init == INIT_SAT_CONST) {
    mask = a;
    init = sat_shift<T, SUP>(a, P.h);
    return;
  }
  if (P.mask_mode == MASK_MAX_MARKER) mask = Op<T, true>::apply(mk, a);
  else if (P.mask_mode == MASK_MIN_MARKER) mask = Op<T, false>::apply(mk, a);
  else mask = a;
  init = Op<T, !SUP>::apply(mk, mask);
}
template <typename T>
__device__ __forceinline__ T combine_mask(const RParams<T> &P, T a, T mk) {
  if (P.init == INIT_SAT_CONST || P.mask_mode == MASK_PLAIN) return a;
  return P.mask_mode == MASK_MAX_MARKER ? Op<T, true>::apply(mk, a) : Op<T, false>::apply(mk, a);
}

template <typename T> __device__ __forceinline__ T ld_cg(const T *p) {
  if constexpr (sizeof(T) == 1) return (T)__ldcg(reinterpret_cast<const unsigned char *>(p));
  else if constexpr (sizeof(T) == 2) return (T)__ldcg(reinterpret_cast<const unsigned short *>(p));
  else if constexpr (std::is_same_v<T, int64_t>) return (T)__ldcg(reinterpret_cast<const long long *>(p));
  else return __ldcg(p);
}
template <typename T> __device__ __forceinline__ void st_cg(T *p, T v) {
  if constexpr (sizeof(T) == 1) __stcg(reinterpret_cast<unsigned char *>(p), (unsigned char)v);
  else if constexpr (sizeof(T) == 2) __stcg(reinterpret_cast<unsigned short *>(p), (unsigned short)v);
  else if constexpr (std::is_same_v<T, int64_t>) __stcg(reinterpret_cast<long long *>(p), (long long)v);
  else __stcg(p, v);
}

enum : int { B_N = 1, B_S = 2, B_W = 4, B_E = 8, B_NW = 16, B_NE = 32, B_SW = 64, B_SE = 128, B_SELF = 256 };

// Puts the tiles next to tile (tx, ty) whose shared border changed (f: B_* bits) on the next
// round's worklist, and the tile itself when it yielded before its local fixpoint.
template <bool CONN8>
__device__ void flag_neighbours(const RImg &im, unsigned *flags, int ntiles, RCtl *ctl, int round, int tx, int ty,
                                int f) {
  unsigned *fnext = flags + (size_t)((round + 1) & 1) * ntiles;
  auto flag = [&](int dx, int dy) {
    const int nx = tx + dx, ny = ty + dy;
    if (nx < 0 || ny < 0 || nx >= im.tiles_x || ny >= im.tiles_y) return;
    fnext[im.tile_begin + ny * im.tiles_x + nx] = 1u;
  };
  if (f & B_N) flag(0, -1);
  if (f & B_S) flag(0, 1);
  if (f & B_W) flag(-1, 0);
  if (f & B_E) flag(1, 0);
  if (CONN8) {
    if (f & B_NW) flag(-1, -1);
    if (f & B_NE) flag(1, -1);
    if (f & B_SW) flag(-1, 1);
    if (f & B_SE) flag(1, 1);
  }
  if (f & B_SELF) flag(0, 0);
  // a changed corner pixel is also on a changed edge, so the edge bits cover every flag.  The
  // word is read before it is written: thousands of tiles set it in a busy round, and the
  // same-address writes would queue at one L2 slice.
  if (f & (B_N | B_S | B_W | B_E | B_SELF)) {
    volatile unsigned *any = &ctl->any[(round + 1) % 3];
    if (*any == 0u) *any = 1u;
  }
}

template <typename T, bool SUP, bool CONN8, int RT>
__device__ void process_tile(const RImg &im, const RParams<T> &P, int t_local, int round, T *s_out, T *s_mask,
                             int *s_flag) {
  constexpr int RTHREADS = RT;
  constexpr int PO = tile_pitch<T>(RT + 2);
  constexpr int PM = tile_pitch<T>(RT);
  const T NEU = Op<T, SUP>::neutral();
  const int tx = t_local % im.tiles_x, ty = t_local / im.tiles_x;
  const int64_t y0 = (int64_t)ty * RT, x0 = (int64_t)tx * RT;
  const T *rec_in = static_cast<const T *>(im.rec);

  // stage: current reconstruction (round 0: marker) with halo, effective mask.  Eight pixels
  // per thread at a time: their loads (at clamped, always valid addresses) are all issued
  // before the first shared-memory store.
  constexpr int NEL = (RT + 2) * (RT + 2);
  constexpr int ITER = (NEL + RTHREADS - 1) / RTHREADS;
  constexpr int CH = 8;
  const bool need_mk = needs_marker(P, round);
  const T *ms_in = static_cast<const T *>(im.mask);
  const T *mk_in = static_cast<const T *>(im.marker);
  for (int k0 = 0; k0 < ITER; k0 += CH) {
    T a[CH], b[CH], c[CH];
#pragma unroll
    for (int k = 0; k < CH; ++k) {
      const int i = (k0 + k) * RTHREADS + threadIdx.x;
      const int r = i / (RT + 2) - 1, cc = i % (RT + 2) - 1;
      const int64_t gy = y0 + r, gx = x0 + cc;
      const bool inside = i < NEL && gy >= 0 && gy < im.H && gx >= 0 && gx < im.W;
      const int64_t gi = inside ? gy * im.W + gx : 0;
      a[k] = ldg(ms_in + gi);
      b[k] = need_mk ? ldg(mk_in + gi) : a[k];
      c[k] = round > 0 ? ld_cg(rec_in + gi) : a[k];
    }
#pragma unroll
    for (int k = 0; k < CH; ++k) {
      const int i = (k0 + k) * RTHREADS + threadIdx.x;
      if (i >= NEL) break;
      const int r = i / (RT + 2) - 1, cc = i % (RT + 2) - 1;
      const int64_t gy = y0 + r, gx = x0 + cc;
      const bool inside = gy >= 0 && gy < im.H && gx >= 0 && gx < im.W;
      const bool interior = r >= 0 && r < RT && cc >= 0 && cc < RT;
      T v = NEU, m = NEU;
      if (inside) {
        if (round == 0) combine_init<T, SUP>(P, a[k], b[k], m, v);
        else {
          v = c[k];
          m = combine_mask(P, a[k], b[k]);
        }
      }
      s_out[(r + 1) * PO + (cc + 1)] = v;
      if (interior) s_mask[r * PM + cc] = m;
    }
  }
  if (threadIdx.x == 0) *s_flag = 0;
  __syncthreads();

  int bflags = 0;
  bool converged = false;
  // one update: v = sel(op(cur, nb), mask); values are monotone, so "changed" means "grew"
  auto upd = [&](int r, int c, T nb) -> bool {
    T *cell = s_out + (r + 1) * PO + (c + 1);
    const T cur = *cell;
    const T v = Op<T, !SUP>::apply(Op<T, SUP>::apply(cur, nb), s_mask[r * PM + c]);
    if (v != cur) {
      *cell = v;
      if (r == 0) bflags |= B_N;
      if (r == RT - 1) bflags |= B_S;
      if (c == 0) bflags |= B_W;
      if (c == RT - 1) bflags |= B_E;
      if (r == 0 && c == 0) bflags |= B_NW;
      if (r == 0 && c == RT - 1) bflags |= B_NE;
      if (r == RT - 1 && c == 0) bflags |= B_SW;
      if (r == RT - 1 && c == RT - 1) bflags |= B_SE;
      return true;
    }
    return false;
  };
  const int lane = threadIdx.x;  // column for vertical sweeps, row for horizontal ones
  bool changed = false;          // any pixel of the tile changed during this visit
  for (int sweep = 0; sweep < P.max_sweeps; ++sweep) {
    bool ch = false;
    // down: neighbours in the row above
    for (int r = 0; r < RT; ++r) {
      const T *up = s_out + r * PO + lane;  // (r-1, lane-1 .. lane+1) in interior coords
      T nb = up[1];
      if (CONN8) nb = Op<T, SUP>::apply(nb, Op<T, SUP>::apply(up[0], up[2]));
      ch |= upd(r, lane, nb);
      __syncwarp();
    }
    __syncthreads();
    // up: neighbours in the row below
    for (int r = RT - 1; r >= 0; --r) {
      const T *dn = s_out + (r + 2) * PO + lane;
      T nb = dn[1];
      if (CONN8) nb = Op<T, SUP>::apply(nb, Op<T, SUP>::apply(dn[0], dn[2]));
      ch |= upd(r, lane, nb);
      __syncwarp();
    }
    __syncthreads();
    // right: neighbours in the column to the left
    for (int c = 0; c < RT; ++c) {
      const T *lf = s_out + lane * PO + c;  // (lane-1 .. lane+1, c-1)
      T nb = lf[PO];
      if (CONN8) nb = Op<T, SUP>::apply(nb, Op<T, SUP>::apply(lf[0], lf[2 * PO]));
      ch |= upd(lane, c, nb);
      __syncwarp();
    }
    __syncthreads();
    // left: neighbours in the column to the right
    for (int c = RT - 1; c >= 0; --c) {
      const T *rt = s_out + lane * PO + c + 2;
      T nb = rt[PO];
      if (CONN8) nb = Op<T, SUP>::apply(nb, Op<T, SUP>::apply(rt[0], rt[2 * PO]));
      ch |= upd(lane, c, nb);
      __syncwarp();
    }
    if (!__syncthreads_or(ch)) {
      converged = true;
      break;
    }
    changed = true;
  }
  if (!converged) bflags |= B_SELF;
  if (bflags) atomicOr(s_flag, bflags);
  __syncthreads();
  const int f = *s_flag;

  // write back (round 0 always: the marker itself is new; later rounds whenever a pixel
  // changed -- an interior-only change happens when the previous visit yielded) and flag the
  // neighbours
  T *rec = static_cast<T *>(im.rec);
  if (round == 0 || changed) {
    for (int i = threadIdx.x; i < RT * RT; i += RTHREADS) {
      const int r = i / RT, c = i % RT;
      const int64_t gy = y0 + r, gx = x0 + c;
      if (gy < im.H && gx < im.W) st_cg(rec + gy * im.W + gx, s_out[(r + 1) * PO + (c + 1)]);
    }
  }
  if (threadIdx.x == 0 && f != 0) flag_neighbours<CONN8>(im, P.flags, P.ntiles, P.ctl, round, tx, ty, f);
  __syncthreads();
}

template <typename T>
__device__ __forceinline__ const RImg &image_of(const RParams<T> &P, int tile, int &t_local) {
  if (P.nimg == 1) { t_local = tile; return P.single; }
  int lo = 0, hi = P.nimg - 1;
  while (lo < hi) {  // last image whose tile_begin <= tile
    const int mid = (lo + hi + 1) >> 1;
    if (P.imgs[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
  }
  t_local = tile - P.imgs[lo].tile_begin;
  return P.imgs[lo];
}

// Epilogue over every pixel of every image, after the last round: the binary h-maxima
// comparison or the leveling clip by the reference.
template <typename T, bool SUP>
__device__ void recon_epilogue(const RParams<T> &P) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int k = 0; k < P.nimg; ++k) {
    const RImg &im = (P.nimg == 1) ? P.single : P.imgs[k];
    const int64_t n = im.H * im.W;
    const T *rec = static_cast<const T *>(im.rec);
    const T *ref = static_cast<const T *>(im.mask);
    if (P.epi == EPI_BINARY_SUP) {
      uint8_t *o = static_cast<uint8_t *>(im.out);
      for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        o[i] = (ldg(ref + i) > ld_cg(rec + i)) ? 255 : 0;
    } else {  // EPI_CLIP_REF: low leveling min(rec, ref), high leveling max(rec, ref)
      T *o = static_cast<T *>(im.out);
      for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        o[i] = Op<T, !SUP>::apply(ld_cg(rec + i), ldg(ref + i));
    }
  }
}

template <typename T, bool SUP, bool CONN8, int RT = tile_side<T>()>
__global__ void __launch_bounds__(RT) k_reconstruct(RParams<T> P) {
  constexpr int RTHREADS = RT;
  constexpr int PO = tile_pitch<T>(RT + 2);
  constexpr int PM = tile_pitch<T>(RT);
  __shared__ __align__(16) T s_out[(RT + 2) * PO];
  __shared__ __align__(16) T s_mask[RT * PM];
  __shared__ int s_flag;
  __shared__ int s_active;
  RCtl *ctl = P.ctl;

  int round = 0;
  bool ok = true;
  for (;;) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->any[(round + 2) % 3] = 0u;
    unsigned *fcur = P.flags + (size_t)(round & 1) * P.ntiles;
    for (int t = blockIdx.x; t < P.ntiles; t += gridDim.x) {
      if (threadIdx.x == 0) {
        int a = 1;
        if (round > 0) {
          a = *((volatile unsigned *)(fcur + t)) != 0u;
          if (a) fcur[t] = 0u;
        }
        s_active = a;
      }
      __syncthreads();
      const bool active = s_active != 0;
      __syncthreads();
      if (active) {
        int tl = 0;
        const RImg &im = image_of(P, t, tl);
        process_tile<T, SUP, CONN8, RT>(im, P, tl, round, s_out, s_mask, &s_flag);
      }
    }
    if (!grid_barrier(ctl)) { ok = false; break; }
    const unsigned any = *((volatile unsigned *)&ctl->any[(round + 1) % 3]);
    ++round;
    if (!any) break;
    if (round >= P.max_rounds) {
      if (threadIdx.x == 0) set_status(ctl, PG_ERR_NOT_CONVERGED);
      ok = false;
      break;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->rounds = round;
    g_recon_rounds = round;
  }
  if (!ok || P.epi == EPI_NONE) return;
  recon_epilogue<T, SUP>(P);
}

// ------------------------------------------------------------------ register tiles
// For pixels of at most 4 bytes the tiles are 32x32 and one warp owns a tile with its values in
// registers: for the vertical sweeps lane c holds column c (v[r] = row r), for the horizontal
// ones the tile goes through shared memory once each way and lane r holds row r.
//  * down / up sweeps take the three pixels of the previous row (8-connected; the same column
//    4-connected), the neighbours' columns by warp shuffles;
//  * right / left sweeps take only the pixel before in the row, a chain inside each lane's
//    registers.  The diagonal relations inside the tile are all covered by the vertical sweeps,
//    and every halo pixel's relations by the one-off halo values below, so a sweep set that
//    changes nothing still means a local fixpoint of the full neighbourhood;
//  * the mask is read from shared memory in either layout (pitch 33 words: conflict-free).
// About one instruction per pixel and sweep set, against some seventy for the shared-memory
// tile above; a CTA holds kRegWarps independent warps.
static constexpr int kRegWarps = 4;
static constexpr int kRP = 33;  // pitch in words of the per-warp shared arrays

template <typename T> using RegS = std::conditional_t<(sizeof(T) < 4), uint32_t, T>;

// Mask reads inside the sweeps: a volatile shared load is performed where it is written, so the
// compiler does not keep the whole 32x32 mask in registers across sweeps (which would cost 64
// registers per thread and most of the occupancy).
template <typename T> __device__ __forceinline__ T lds_mask(const RegS<T> *p) {
  const unsigned addr = (unsigned)__cvta_generic_to_shared(p);
  uint32_t r;
  asm volatile("ld.volatile.shared.b32 %0, [%1];" : "=r"(r) : "r"(addr));
  if constexpr (std::is_same_v<T, float>) return __uint_as_float(r);
  else return (T)r;
}

template <typename T> __device__ __forceinline__ T shfl_up1(T v) {
  if constexpr (sizeof(T) < 4) return (T)__shfl_up_sync(0xffffffffu, (unsigned)v, 1);
  else return __shfl_up_sync(0xffffffffu, v, 1);
}
template <typename T> __device__ __forceinline__ T shfl_dn1(T v) {
  if constexpr (sizeof(T) < 4) return (T)__shfl_down_sync(0xffffffffu, (unsigned)v, 1);
  else return __shfl_down_sync(0xffffffffu, v, 1);
}

// Pixel (gy, gx) seen from a neighbouring tile: neutral outside the image, the marker in round
// 0, the current reconstruction later.  halo_load issues the loads (at a clamped, always valid
// address), halo_finish combines them, so that all halo loads of a visit are in flight at once.
template <typename T> struct HaloPx {
  T a, mk;
  bool in;
};
template <typename T>
__device__ __forceinline__ HaloPx<T> halo_load(const RImg &im, const RParams<T> &P, int round, bool need_mk,
                                               int64_t gy, int64_t gx) {
  HaloPx<T> h;
  h.in = gy >= 0 && gy < im.H && gx >= 0 && gx < im.W;
  const int64_t gi = h.in ? gy * im.W + gx : 0;
  if (round == 0) {
    h.a = ldg(static_cast<const T *>(im.mask) + gi);
    h.mk = need_mk ? ldg(static_cast<const T *>(im.marker) + gi) : h.a;
  } else {
    h.a = ld_cg(static_cast<const T *>(im.rec) + gi);
    h.mk = h.a;
  }
  return h;
}
template <typename T, bool SUP>
__device__ __forceinline__ T halo_finish(const RParams<T> &P, int round, const HaloPx<T> &h) {
  if (!h.in) return Op<T, SUP>::neutral();
  if (round > 0) return h.a;
  T m, v;
  combine_init<T, SUP>(P, h.a, h.mk, m, v);
  return v;
}

template <typename T, bool SUP, bool CONN8>
__device__ void process_tile_reg(const RImg &im, const RParams<T> &P, int t_local, int round, RegS<T> *s_m,
                                 RegS<T> *s_t) {
  using OS = Op<T, SUP>;   // propagation
  using OC = Op<T, !SUP>;  // clip by the mask
  const int lane = threadIdx.x & 31;
  const T NEU = OS::neutral();
  const int tx = t_local % im.tiles_x, ty = t_local / im.tiles_x;
  const int64_t y0 = (int64_t)ty * 32, x0 = (int64_t)tx * 32;
  const T *rec_in = static_cast<const T *>(im.rec);
  const int64_t gx = x0 + lane;
  const bool colin = gx < im.W;

  // stage, lane = column: tile values and mask (pixels outside the image: neutral, fixed).
  // Loads come first, 16 rows at a time, so that they are all in flight together; the
  // addresses of pixels outside the image are clamped to pixel 0 and the values discarded.
  const T *mk_in = static_cast<const T *>(im.marker);
  const T *ms_in = static_cast<const T *>(im.mask);
  const bool need_mk = needs_marker(P, round);
  T v[32];
#pragma unroll
  for (int h = 0; h < 32; h += 16) {
    T a[16], b[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int64_t gy = y0 + h + r;
      const int64_t gi = (colin && gy < im.H) ? gy * im.W + gx : 0;
      a[r] = ldg(ms_in + gi);
      b[r] = need_mk ? ldg(mk_in + gi) : a[r];
      if (round > 0) v[h + r] = ld_cg(rec_in + gi);
    }
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const bool ok = colin && y0 + h + r < im.H;
      T m;
      if (round == 0) combine_init<T, SUP>(P, a[r], b[r], m, v[h + r]);
      else m = combine_mask(P, a[r], b[r]);
      if (!ok) {
        m = NEU;
        v[h + r] = NEU;
      }
      s_m[(h + r) * kRP + lane] = m;
    }
  }
  // Halo.  Its values stay fixed during the visit, so each halo pixel's contribution is
  // folded into one value per border pixel: `top`/`bot` per column (lane = column: the three
  // pixels above / below), `hl`/`hr` per row (lane = row: the three pixels left / right; one
  // in 4-connectivity).  The sweeps apply them at the tile's first/last row and column.
  T top, bot, hl, hr;
  {
    HaloPx<T> q[12];
    q[0] = halo_load(im, P, round, need_mk, y0 - 1, gx);
    q[1] = halo_load(im, P, round, need_mk, y0 + 32, gx);
    q[2] = halo_load(im, P, round, need_mk, y0 + lane, x0 - 1);
    q[3] = halo_load(im, P, round, need_mk, y0 + lane, x0 + 32);
    if (CONN8) {
      q[4] = halo_load(im, P, round, need_mk, y0 - 1, gx - 1);
      q[5] = halo_load(im, P, round, need_mk, y0 - 1, gx + 1);
      q[6] = halo_load(im, P, round, need_mk, y0 + 32, gx - 1);
      q[7] = halo_load(im, P, round, need_mk, y0 + 32, gx + 1);
      q[8] = halo_load(im, P, round, need_mk, y0 + lane - 1, x0 - 1);
      q[9] = halo_load(im, P, round, need_mk, y0 + lane + 1, x0 - 1);
      q[10] = halo_load(im, P, round, need_mk, y0 + lane - 1, x0 + 32);
      q[11] = halo_load(im, P, round, need_mk, y0 + lane + 1, x0 + 32);
    }
    top = halo_finish<T, SUP>(P, round, q[0]);
    bot = halo_finish<T, SUP>(P, round, q[1]);
    hl = halo_finish<T, SUP>(P, round, q[2]);
    hr = halo_finish<T, SUP>(P, round, q[3]);
    if (CONN8) {
      top = OS::apply(top, OS::apply(halo_finish<T, SUP>(P, round, q[4]), halo_finish<T, SUP>(P, round, q[5])));
      bot = OS::apply(bot, OS::apply(halo_finish<T, SUP>(P, round, q[6]), halo_finish<T, SUP>(P, round, q[7])));
      hl = OS::apply(hl, OS::apply(halo_finish<T, SUP>(P, round, q[8]), halo_finish<T, SUP>(P, round, q[9])));
      hr = OS::apply(hr, OS::apply(halo_finish<T, SUP>(P, round, q[10]), halo_finish<T, SUP>(P, round, q[11])));
    }
  }
  // staged borders, to tell afterwards which neighbours must be revisited
#pragma unroll
  for (int r = 0; r < 32; ++r) s_t[r * kRP + lane] = v[r];
  __syncwarp();
  const T initL = (T)s_t[lane * kRP], initR = (T)s_t[lane * kRP + 31];
  const T initT = v[0], initB = v[31];
  __syncwarp();

  bool converged = false, changed = false, wch = false, ech = false;
  for (int sweep = 0; sweep < P.max_sweeps; ++sweep) {
    bool ch = false;
    // down: the row above (lane 0 / 31 get their own value back from the shuffle: the pixels
    // beyond the tile's side columns are halo, applied by the horizontal sweeps)
#pragma unroll
    for (int r = 0; r < 32; ++r) {
      T nb;
      if (r == 0) nb = top;
      else {
        nb = v[r - 1];
        if (CONN8) nb = OS::apply(nb, OS::apply(shfl_up1(nb), shfl_dn1(nb)));
      }
      const T nv = OC::apply(OS::apply(v[r], nb), lds_mask<T>(s_m + r * kRP + lane));
      ch |= nv != v[r];
      v[r] = nv;
    }
    // up: the row below
#pragma unroll
    for (int r = 31; r >= 0; --r) {
      T nb;
      if (r == 31) nb = bot;
      else {
        nb = v[r + 1];
        if (CONN8) nb = OS::apply(nb, OS::apply(shfl_up1(nb), shfl_dn1(nb)));
      }
      const T nv = OC::apply(OS::apply(v[r], nb), lds_mask<T>(s_m + r * kRP + lane));
      ch |= nv != v[r];
      v[r] = nv;
    }
    // to lane = row
#pragma unroll
    for (int r = 0; r < 32; ++r) s_t[r * kRP + lane] = v[r];
    __syncwarp();
#pragma unroll
    for (int c = 0; c < 32; ++c) v[c] = (T)s_t[lane * kRP + c];
    __syncwarp();
    // right: the pixel on the left; left: the pixel on the right
    T prev = hl;
#pragma unroll
    for (int c = 0; c < 32; ++c) {
      const T nv = OC::apply(OS::apply(v[c], prev), lds_mask<T>(s_m + lane * kRP + c));
      ch |= nv != v[c];
      v[c] = nv;
      prev = nv;
    }
    prev = hr;
#pragma unroll
    for (int c = 31; c >= 0; --c) {
      const T nv = OC::apply(OS::apply(v[c], prev), lds_mask<T>(s_m + lane * kRP + c));
      ch |= nv != v[c];
      v[c] = nv;
      prev = nv;
    }
    wch = v[0] != initL;
    ech = v[31] != initR;
    // back to lane = column
#pragma unroll
    for (int c = 0; c < 32; ++c) s_t[lane * kRP + c] = v[c];
    __syncwarp();
#pragma unroll
    for (int r = 0; r < 32; ++r) v[r] = (T)s_t[r * kRP + lane];
    __syncwarp();
    if (!__any_sync(0xffffffffu, ch)) {
      converged = true;
      break;
    }
    changed = true;
  }

  const unsigned bN = __ballot_sync(0xffffffffu, v[0] != initT);
  const unsigned bS = __ballot_sync(0xffffffffu, v[31] != initB);
  const unsigned bW = __ballot_sync(0xffffffffu, wch);
  const unsigned bE = __ballot_sync(0xffffffffu, ech);
  int f = converged ? 0 : B_SELF;
  if (bN) f |= B_N;
  if (bS) f |= B_S;
  if (bW) f |= B_W;
  if (bE) f |= B_E;
  if (bN & 1u) f |= B_NW;
  if (bN >> 31) f |= B_NE;
  if (bS & 1u) f |= B_SW;
  if (bS >> 31) f |= B_SE;

  if (round == 0 || changed) {
    // the row stride goes through a shuffle so that the compiler recomputes these addresses
    // here instead of keeping the stage's 32 row addresses alive across the sweeps
    const long long Wd = __shfl_sync(0xffffffffu, (long long)im.W, 0);
    T *p = static_cast<T *>(im.rec) + (y0 * Wd + gx);
#pragma unroll
    for (int r = 0; r < 32; ++r) {
      if (colin && y0 + r < im.H) st_cg(p, v[r]);
      p += Wd;
    }
  }
  if (lane == 0 && f != 0) flag_neighbours<CONN8>(im, P.flags, P.ntiles, P.ctl, round, tx, ty, f);
  __syncwarp();
}

template <typename T, bool SUP, bool CONN8>
__global__ void __launch_bounds__(kRegWarps * 32, 4) k_reconstruct_reg(RParams<T> P) {
  static_assert(sizeof(T) <= 4, "register tiles hold pixels of at most 4 bytes");
  __shared__ RegS<T> s_m[kRegWarps][32 * kRP];
  __shared__ RegS<T> s_t[kRegWarps][32 * kRP];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  RCtl *ctl = P.ctl;
  const int wstride = gridDim.x * kRegWarps;

  int round = 0;
  bool ok = true;
  for (;;) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->any[(round + 2) % 3] = 0u;
    unsigned *fcur = P.flags + (size_t)(round & 1) * P.ntiles;
    for (int t = blockIdx.x * kRegWarps + warp; t < P.ntiles; t += wstride) {
      int a = 1;
      if (round > 0) {
        if (lane == 0) {
          a = *((volatile unsigned *)(fcur + t)) != 0u;
          if (a) fcur[t] = 0u;
        }
        a = __shfl_sync(0xffffffffu, a, 0);
      }
      if (a) {
        int tl = 0;
        const RImg &im = image_of(P, t, tl);
        process_tile_reg<T, SUP, CONN8>(im, P, tl, round, s_m[warp], s_t[warp]);
      }
    }
    if (!grid_barrier(ctl)) { ok = false; break; }
    const unsigned any = *((volatile unsigned *)&ctl->any[(round + 1) % 3]);
    ++round;
    if (!any) break;
    if (round >= P.max_rounds) {
      if (threadIdx.x == 0) set_status(ctl, PG_ERR_NOT_CONVERGED);
      ok = false;
      break;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->rounds = round;
    g_recon_rounds = round;
  }
  if (!ok || P.epi == EPI_NONE) return;
  recon_epilogue<T, SUP>(P);
}

// ------------------------------------------------------------------ host side
template <typename T, bool SUP, bool CONN8>
static pg_status run_t(std::vector<RImg> &imgs, const ReconRequest &rq, bool binary, cudaStream_t s) {
  // register tiles (32x32, a warp each) up to 4-byte pixels, shared-memory tiles for 8-byte ones
  constexpr bool REG = sizeof(T) <= 4;
  constexpr int RT = REG ? 32 : tile_side<T>();
  constexpr int RTHREADS = REG ? kRegWarps * 32 : RT;
  constexpr int TILES_PER_CTA = REG ? kRegWarps : 1;
  int ntiles = 0;
  size_t rec_bytes = 0;
  for (auto &im : imgs) {
    im.tiles_x = (int)ceil_div(im.W, RT);
    im.tiles_y = (int)ceil_div(im.H, RT);
    im.tile_begin = ntiles;
    ntiles += im.tiles_x * im.tiles_y;
    if (binary) rec_bytes += (sizeof(T) * (size_t)(im.H * im.W) + 15) / 16 * 16;  // 16-byte aligned slots
  }
  if (ntiles == 0) return PG_OK;
  const int nimg = (int)imgs.size();
  // scratch: control block | flags | image table | reconstruction buffers (binary mode)
  const size_t off_flags = 256;
  const size_t off_tab = off_flags + ((sizeof(unsigned) * 2 * (size_t)ntiles + 255) / 256) * 256;
  const size_t off_rec = off_tab + ((sizeof(RImg) * (size_t)(nimg > 1 ? nimg : 0) + 255) / 256) * 256;
  const size_t total = off_rec + rec_bytes + 256;
  Scratch scr;
  PG_TRY(scr.alloc(total, s));
  char *base = scr.as<char>();
  if (binary) {
    size_t off = off_rec;
    for (auto &im : imgs) {
      im.rec = base + off;
      off += sizeof(T) * (size_t)(im.H * im.W);
      off = (off + 15) / 16 * 16;
    }
  }
  PG_CUDA_TRY(cudaMemsetAsync(base, 0, off_tab, s), "clear reconstruction control block");
  std::vector<RImg> table;
  if (nimg > 1) {
    table = imgs;
    PG_CUDA_TRY(cudaMemcpyAsync(base + off_tab, table.data(), sizeof(RImg) * (size_t)nimg, cudaMemcpyHostToDevice, s),
                "upload image table");
  }
  RParams<T> P{};
  P.single = imgs[0];
  P.imgs = reinterpret_cast<const RImg *>(base + off_tab);
  P.nimg = nimg;
  P.ntiles = ntiles;
  P.ctl = reinterpret_cast<RCtl *>(base);
  P.flags = reinterpret_cast<unsigned *>(base + off_flags);
  // A round moves information across at least one tile border, so the rounds needed are
  // bounded by the tile crossings of the longest geodesic path; the cap only guards against
  // a runaway (termination is guaranteed: every round raises some pixel to another input value).
  P.max_rounds = (int)std::min<int64_t>(INT32_MAX / 2, 1024 + 64 * (int64_t)ntiles);
  P.init = rq.init;
  P.mask_mode = rq.mask_mode;
  P.epi = rq.epi;
  P.h = static_cast<T>(rq.h);

  void (*kern)(RParams<T>) = nullptr;
  if constexpr (REG) kern = k_reconstruct_reg<T, SUP, CONN8>;
  else kern = k_reconstruct<T, SUP, CONN8>;
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  static std::mutex mu;
  static int cached_dev = -1, cached_blocks = 0;
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (cached_dev != dev) {
      PG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cached_blocks, kern, RTHREADS, 0), "occupancy");
      cached_dev = dev;
    }
    per_sm = cached_blocks;
  }
  if (per_sm < 1) return fail(PG_ERR_CUDA, "reconstruction kernel cannot be resident");
  int grid = per_sm * num_sms();
  if (grid > ceil_div(ntiles, TILES_PER_CTA)) grid = (int)ceil_div(ntiles, TILES_PER_CTA);

  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(RTHREADS);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  PG_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, P), "cooperative reconstruction launch");
  return PG_OK;
}

template <typename T>
static pg_status run_dispatch(std::vector<RImg> &imgs, const ReconRequest &rq, cudaStream_t s) {
  const bool binary = rq.epi == EPI_BINARY_SUP;
  if (rq.dilate) return rq.conn8 ? run_t<T, true, true>(imgs, rq, binary, s) : run_t<T, true, false>(imgs, rq, binary, s);
  return rq.conn8 ? run_t<T, false, true>(imgs, rq, binary, s) : run_t<T, false, false>(imgs, rq, binary, s);
}

pg_status launch_reconstruction(const pg_image *markers, const pg_image *masks, const pg_image *outs, int n_images,
                                const ReconRequest &rq, cudaStream_t s) {
  if (n_images < 1) return PG_OK;
  std::vector<RImg> imgs((size_t)n_images);
  for (int i = 0; i < n_images; ++i) {
    const Dims d = dims_of(masks[i]);
    RImg &im = imgs[(size_t)i];
    im = RImg{};
    im.marker = markers ? markers[i].data : nullptr;
    im.mask = masks[i].data;
    im.rec = outs[i].data;
    im.out = outs[i].data;
    im.H = d.nz * d.ny;  // rank 1: one row
    im.W = d.nx;
  }
  PG_DISPATCH_PTYPE(masks[0].ptype, T, { return run_dispatch<T>(imgs, rq, s); });
  return PG_OK;
}

// ------------------------------------------------------------------ batch plans + autotuner
// A plan keeps a ragged batch's image tables, worklist and reconstruction buffers on the device
// so that each run is one memset and one cooperative launch (both capturable in a CUDA graph).
// The autotuner times the candidate configurations -- tile side (32: register tiles, 64: shared-
// memory tiles) x sweep sets per tile visit before the tile yields to the next global round
// (4, 16, unbounded) -- on the plan's own batch and keeps the fastest; the choice is cached per
// (pixel type, connectivity, batch size class).
struct PlanCfg {
  int rt = 64;
  int sweeps = kMaxSweeps;
};

struct PlanTable {  // one tile decomposition of the batch
  int ntiles = 0;
  RImg *d_imgs = nullptr;  // device table
  std::vector<RImg> imgs;  // host copy
};

}  // namespace pg

struct pg_batch_plan {
  int device = 0;
  int ptype = 0;
  bool conn8 = true;
  double h = 0;
  void *scratch = nullptr;  // control block | flags (sized for the finest tiling) | recon buffers
  size_t clear_bytes = 0;
  pg::PlanTable t64, t32;
  pg::PlanCfg cfg;
  int grid = 0;
};

namespace pg {

template <int RT> static PlanTable &plan_table(pg_batch_plan &p) { return RT == 64 ? p.t64 : p.t32; }

template <typename T, bool CONN8, int RT>
static pg_status plan_launch_t(pg_batch_plan &p, int sweeps, cudaStream_t s, int *grid_out) {
  PlanTable &tb = plan_table<RT>(p);
  RParams<T> P{};
  P.single = tb.imgs[0];
  P.imgs = tb.d_imgs;
  P.nimg = (int)tb.imgs.size();
  P.ntiles = tb.ntiles;
  P.ctl = static_cast<RCtl *>(p.scratch);
  P.flags = reinterpret_cast<unsigned *>(static_cast<char *>(p.scratch) + 256);
  P.max_rounds = (int)std::min<int64_t>(INT32_MAX / 2, 1024 + 64 * (int64_t)tb.ntiles);
  P.max_sweeps = sweeps;
  P.init = INIT_SAT_CONST;
  P.mask_mode = MASK_PLAIN;
  P.epi = EPI_BINARY_SUP;
  P.h = static_cast<T>(p.h);
  // 32-pixel tiles of pixels up to 4 bytes run as register tiles (a warp per tile)
  constexpr bool REG = RT == 32 && sizeof(T) <= 4;
  constexpr int THREADS = REG ? kRegWarps * 32 : RT;
  constexpr int TILES_PER_CTA = REG ? kRegWarps : 1;
  void (*kern)(RParams<T>) = nullptr;
  if constexpr (REG) kern = k_reconstruct_reg<T, true, CONN8>;
  else kern = k_reconstruct<T, true, CONN8, RT>;
  int per_sm = 0;
  PG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, THREADS, 0), "occupancy");
  if (per_sm < 1) return fail(PG_ERR_CUDA, "reconstruction kernel cannot be resident");
  int grid = per_sm * num_sms();
  if (grid > ceil_div(tb.ntiles, TILES_PER_CTA)) grid = (int)ceil_div(tb.ntiles, TILES_PER_CTA);
  if (grid_out) *grid_out = grid;
  PG_CUDA_TRY(cudaMemsetAsync(p.scratch, 0, p.clear_bytes, s), "clear batch worklist");
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(THREADS);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  PG_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, P), "cooperative batch launch");
  return PG_OK;
}

template <typename T>
static pg_status plan_launch(pg_batch_plan &p, const PlanCfg &c, cudaStream_t s, int *grid_out) {
  if constexpr (sizeof(T) == 8) {
    return p.conn8 ? plan_launch_t<T, true, 32>(p, c.sweeps, s, grid_out) : plan_launch_t<T, false, 32>(p, c.sweeps, s, grid_out);
  } else {
    if (c.rt == 64)
      return p.conn8 ? plan_launch_t<T, true, 64>(p, c.sweeps, s, grid_out) : plan_launch_t<T, false, 64>(p, c.sweeps, s, grid_out);
    return p.conn8 ? plan_launch_t<T, true, 32>(p, c.sweeps, s, grid_out) : plan_launch_t<T, false, 32>(p, c.sweeps, s, grid_out);
  }
}

static pg_status plan_run(pg_batch_plan &p, const PlanCfg &c, cudaStream_t s, int *grid_out) {
  PG_DISPATCH_PTYPE(p.ptype, T, { return plan_launch<T>(p, c, s, grid_out); });
  return PG_OK;
}

static void plan_tables(pg_batch_plan &p, const std::vector<RImg> &base, int rt, PlanTable &tb) {
  tb.imgs = base;
  int ntiles = 0;
  for (auto &im : tb.imgs) {
    im.tiles_x = (int)ceil_div(im.W, rt);
    im.tiles_y = (int)ceil_div(im.H, rt);
    im.tile_begin = ntiles;
    ntiles += im.tiles_x * im.tiles_y;
  }
  tb.ntiles = ntiles;
}

struct TuneKey {
  int ptype, conn8, size_class, count_class;
  bool operator<(const TuneKey &o) const {
    return std::tie(ptype, conn8, size_class, count_class) < std::tie(o.ptype, o.conn8, o.size_class, o.count_class);
  }
};

pg_status create_batch_plan(const pg_image *ins, const pg_image *outs, int n, double h, bool conn8, bool autotune,
                            cudaStream_t s, pg_batch_plan **out_plan) {
  auto plan = std::make_unique<pg_batch_plan>();
  PG_CUDA_TRY(cudaGetDevice(&plan->device), "cudaGetDevice");
  plan->ptype = ins[0].ptype;
  plan->conn8 = conn8;
  plan->h = h;
  const size_t es = (size_t)elem_size(plan->ptype);
  std::vector<RImg> base((size_t)n);
  int64_t pixels = 0;
  for (int i = 0; i < n; ++i) {
    const Dims d = dims_of(ins[i]);
    RImg &im = base[(size_t)i];
    im = RImg{};
    im.mask = ins[i].data;
    im.out = outs[i].data;
    im.H = d.nz * d.ny;
    im.W = d.nx;
    pixels += im.H * im.W;
  }
  plan_tables(*plan, base, 64, plan->t64);
  plan_tables(*plan, base, 32, plan->t32);
  const int max_tiles = std::max(plan->t64.ntiles, plan->t32.ntiles);
  const size_t off_flags = 256;
  const size_t flags_bytes = ((sizeof(unsigned) * 2 * (size_t)max_tiles + 255) / 256) * 256;
  const size_t off_tab64 = off_flags + flags_bytes;
  const size_t tab_bytes = ((sizeof(RImg) * (size_t)n + 255) / 256) * 256;
  const size_t off_tab32 = off_tab64 + tab_bytes;
  size_t off_rec = off_tab32 + tab_bytes;
  size_t rec_bytes = 0;
  for (auto &im : base) rec_bytes += (es * (size_t)(im.H * im.W) + 255) / 256 * 256;
  PG_CUDA_TRY(cudaMalloc(&plan->scratch, off_rec + rec_bytes + 256), "batch plan allocation");
  plan->clear_bytes = off_tab64;
  // reconstruction buffers, then device copies of both tile tables
  char *b = static_cast<char *>(plan->scratch);
  size_t off = off_rec;
  for (size_t i = 0; i < base.size(); ++i) {
    plan->t64.imgs[i].rec = b + off;
    plan->t32.imgs[i].rec = b + off;
    off += (es * (size_t)(base[i].H * base[i].W) + 255) / 256 * 256;
  }
  plan->t64.d_imgs = reinterpret_cast<RImg *>(b + off_tab64);
  plan->t32.d_imgs = reinterpret_cast<RImg *>(b + off_tab32);
  cudaError_t e = cudaMemcpy(plan->t64.d_imgs, plan->t64.imgs.data(), sizeof(RImg) * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(plan->t32.d_imgs, plan->t32.imgs.data(), sizeof(RImg) * (size_t)n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(plan->scratch);
    return cuda_status(e, "upload batch tile tables");
  }

  static std::mutex mu;
  static std::map<TuneKey, PlanCfg> cache;
  const TuneKey key{plan->ptype, conn8 ? 1 : 0, (int)std::log2((double)std::max<int64_t>(pixels, 1)),
                    (int)std::log2((double)std::max(n, 1))};
  bool cached = false;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) { plan->cfg = it->second; cached = true; }
  }
  if (autotune && !cached) {
    std::vector<PlanCfg> cands;
    for (int rt : {64, 32}) {
      if (es == 8 && rt == 64) continue;
      for (int sw : {4, 16, kMaxSweeps}) cands.push_back(PlanCfg{rt, sw});
    }
    cudaEvent_t a, z;
    PG_CUDA_TRY(cudaEventCreate(&a), "event");
    PG_CUDA_TRY(cudaEventCreate(&z), "event");
    float best = 1e30f;
    for (const PlanCfg &c : cands) {
      pg_status st = plan_run(*plan, c, s, nullptr);  // warm
      if (st != PG_OK) { cudaEventDestroy(a); cudaEventDestroy(z); cudaFree(plan->scratch); return st; }
      float tot = 0.f;
      for (int r = 0; r < 2; ++r) {
        cudaEventRecord(a, s);
        plan_run(*plan, c, s, nullptr);
        cudaEventRecord(z, s);
        cudaEventSynchronize(z);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, z);
        tot += ms;
      }
      if (tot < best) { best = tot; plan->cfg = c; }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(z);
    std::lock_guard<std::mutex> lk(mu);
    cache[key] = plan->cfg;
  } else if (!cached) {
    plan->cfg = PlanCfg{32, kMaxSweeps};
  }
  *out_plan = plan.release();
  return PG_OK;
}

pg_status run_batch_plan(pg_batch_plan *p, cudaStream_t s) {
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev != p->device) return fail(PG_ERR_INVALID_ARGUMENT, "batch plan used on another device");
  return plan_run(*p, p->cfg, s, &p->grid);
}

void destroy_batch_plan(pg_batch_plan *p) {
  if (!p) return;
  if (p->scratch) cudaFree(p->scratch);
  delete p;
}

// ------------------------------------------------------------------ allocation-free variant
// For callers that must not touch the device allocator (see pg_reconstruction_noalloc in
// include/poutre_gb300.h).  Its only scratch -- the control block and the tile worklist --
// lives in this file-scope array, which every GPU that loads the library holds until exit.
static constexpr size_t kNoAllocScratchBytes = PG_NOALLOC_SCRATCH_BYTES;
static constexpr size_t kNoAllocFlagsOffset = 256;  // RCtl fits below
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static_assert(sizeof(RCtl) <= kNoAllocFlagsOffset, "control block must fit below the flags");

// Device address of g_noalloc_scratch, looked up once per device with that device current.
// In host code the symbol name is only a host-side stand-in, so the kernel is given this
// address instead.
static pg_status noalloc_scratch(void **out) {
  static std::mutex mu;
  static std::vector<void *> addr;  // indexed by device ordinal
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lk(mu);
  if ((size_t)dev >= addr.size()) addr.resize((size_t)dev + 1, nullptr);
  if (!addr[(size_t)dev]) {
    void *p = nullptr;
    PG_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(no-alloc scratch)");
    addr[(size_t)dev] = p;
  }
  *out = addr[(size_t)dev];
  return PG_OK;
}

template <typename T, bool SUP, bool CONN8>
static pg_status run_noalloc_t(RImg im, cudaStream_t s) {
  constexpr int RT = tile_side<T>(), RTHREADS = RT;
  im.tiles_x = (int)ceil_div(im.W, RT);
  im.tiles_y = (int)ceil_div(im.H, RT);
  im.tile_begin = 0;
  const int64_t ntiles = (int64_t)im.tiles_x * im.tiles_y;
  if (ntiles == 0) return PG_OK;
  const int64_t max_tiles = (int64_t)((kNoAllocScratchBytes - kNoAllocFlagsOffset) / (2 * sizeof(unsigned)));
  if (ntiles > max_tiles)
    return fail(PG_ERR_INVALID_ARGUMENT, "pg_reconstruction_noalloc: the image needs " + std::to_string(ntiles) +
                                             " tiles of " + std::to_string(RT) + "x" + std::to_string(RT) +
                                             " pixels; the fixed scratch holds at most " + std::to_string(max_tiles));
  void *base = nullptr;
  PG_TRY(noalloc_scratch(&base));
  // the control block and both flag buffers must start at zero; the array keeps the
  // previous call's contents
  const size_t used = kNoAllocFlagsOffset + 2 * sizeof(unsigned) * (size_t)ntiles;
  PG_CUDA_TRY(cudaMemsetAsync(base, 0, used, s), "clear no-alloc scratch");
  RParams<T> P{};
  P.single = im;
  P.imgs = nullptr;
  P.nimg = 1;
  P.ntiles = (int)ntiles;
  P.ctl = static_cast<RCtl *>(base);
  P.flags = reinterpret_cast<unsigned *>(static_cast<char *>(base) + kNoAllocFlagsOffset);
  P.max_rounds = (int)std::min<int64_t>(INT32_MAX / 2, 1024 + 64 * ntiles);
  P.init = INIT_MARKER;
  P.mask_mode = MASK_PLAIN;
  P.epi = EPI_NONE;
  P.h = static_cast<T>(0);
  auto kern = k_reconstruct<T, SUP, CONN8>;
  int per_sm = 0;
  PG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, RTHREADS, 0), "occupancy");
  if (per_sm < 1) return fail(PG_ERR_CUDA, "reconstruction kernel cannot be resident");
  int64_t grid = (int64_t)per_sm * num_sms();
  if (grid > ntiles) grid = ntiles;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(RTHREADS);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  PG_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, P), "cooperative reconstruction launch (no-alloc)");
  return PG_OK;
}

static pg_status reconstruction_noalloc(bool dilate, bool conn8, const pg_image &marker, const pg_image &mask,
                                        const pg_image &out, cudaStream_t s) {
  const Dims d = dims_of(mask);
  RImg im{};
  im.marker = marker.data;
  im.mask = mask.data;
  im.rec = out.data;
  im.out = out.data;
  im.H = d.nz * d.ny;
  im.W = d.nx;
  PG_DISPATCH_PTYPE(mask.ptype, T, {
    if (dilate) return conn8 ? run_noalloc_t<T, true, true>(im, s) : run_noalloc_t<T, true, false>(im, s);
    return conn8 ? run_noalloc_t<T, false, true>(im, s) : run_noalloc_t<T, false, false>(im, s);
  });
  return PG_OK;
}

}  // namespace pg

extern "C" {

// Synchronises `stream`, then reads and clears the device status of the reconstruction
// kernels (PG_ERR_NOT_CONVERGED if one gave up since the last check).
pg_status pg_check_device(pg_stream_t stream) {
  PG_CUDA_TRY(cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream)), "stream synchronisation");
  int st = 0, zero = 0;
  PG_CUDA_TRY(cudaMemcpyFromSymbol(&st, pg::g_recon_status, sizeof(int)), "read device status");
  if (st != 0) {
    PG_CUDA_TRY(cudaMemcpyToSymbol(pg::g_recon_status, &zero, sizeof(int)), "clear device status");
    return pg::fail(static_cast<pg_status>(st), "reconstruction did not converge within its round cap or wait limit");
  }
  return PG_OK;
}

int32_t pg_last_reconstruction_rounds(void) {
  int r = -1;
  if (cudaDeviceSynchronize() != cudaSuccess) return -1;
  if (cudaMemcpyFromSymbol(&r, pg::g_recon_rounds, sizeof(int)) != cudaSuccess) return -1;
  return r;
}

// Reconstruction that allocates nothing: same checks and result as pg_reconstruction, scratch
// taken from g_noalloc_scratch.  The first call on a device looks up that array's device
// address; make it before any stream capture.
pg_status pg_reconstruction_noalloc(int32_t type, const pg_image *marker, const pg_image *mask, int32_t se,
                                    const pg_image *out, pg_stream_t stream) {
  auto chk = [](const pg_image *a, const pg_image *b) -> pg_status {
    if (!a || !b) return pg::fail(PG_ERR_INVALID_ARGUMENT, "t_Reconstruct: null image descriptor");
    if (a->rank < 1 || a->rank > 3 || b->rank != a->rank)
      return pg::fail(PG_ERR_INCOMPATIBLE, "t_Reconstruct incompatible size");
    for (int i = 0; i < a->rank; ++i)
      if (a->shape[i] != b->shape[i] || a->shape[i] < 0) return pg::fail(PG_ERR_INCOMPATIBLE, "t_Reconstruct incompatible size");
    if (!pg::elem_size(a->ptype)) return pg::fail(PG_ERR_UNSUPPORTED_PTYPE, "unsupported PTYPE");
    if (a->ptype != b->ptype) return pg::fail(PG_ERR_INCOMPATIBLE, "t_Reconstruct incompatible types");
    const int64_t n = pg::dims_of(*a).count();
    if (n > 0 && (!a->data || !b->data)) return pg::fail(PG_ERR_INVALID_ARGUMENT, "t_Reconstruct: null data pointer");
    return PG_OK;
  };
  auto distinct = [](const pg_image *a, const pg_image *b) -> pg_status {
    const int64_t n = pg::dims_of(*a).count();
    const size_t bytes = (size_t)n * pg::elem_size(a->ptype);
    const char *pa = static_cast<const char *>(a->data), *pb = static_cast<const char *>(b->data);
    if (n > 0 && pa < pb + bytes && pb < pa + bytes)
      return pg::fail(PG_ERR_ALIASING, "t_Reconstruct output must be != than input images");
    return PG_OK;
  };
  PG_TRY(chk(marker, out));
  PG_TRY(chk(mask, out));
  {
    // size limit of the fixed scratch, checked on the shape alone
    const pg::Dims d = pg::dims_of(*mask);
    const int rt = pg::elem_size(mask->ptype) == 8 ? 32 : 64;
    const int64_t ntiles = pg::ceil_div(d.nz * d.ny, rt) * pg::ceil_div(d.nx, rt);
    const int64_t max_tiles = (int64_t)((pg::kNoAllocScratchBytes - pg::kNoAllocFlagsOffset) / (2 * sizeof(unsigned)));
    if (ntiles > max_tiles)
      return pg::fail(PG_ERR_INVALID_ARGUMENT, "pg_reconstruction_noalloc: the image needs " + std::to_string(ntiles) +
                                                   " tiles; the fixed scratch holds at most " +
                                                   std::to_string(max_tiles));
  }
  PG_TRY(distinct(marker, out));
  PG_TRY(distinct(mask, out));
  if (type != PG_RECONSTRUCT_ERODE && type != PG_RECONSTRUCT_DILATE)
    return pg::fail(PG_ERR_INVALID_ARGUMENT, "t_ReconstructionDispatchRectType unsupported reconstruction_type");
  bool conn8 = true;
  const int rank = mask->rank;
  if (rank == 1 && se == PG_SE_SEGMENT_X_1D) conn8 = true;
  else if (rank == 2 && se == PG_SE_SQUARE_2D) conn8 = true;
  else if (rank == 2 && se == PG_SE_CROSS_2D) conn8 = false;
  else return pg::fail(PG_ERR_UNSUPPORTED_SE, "t_ReconstructionDispatchNl unsupported nl_static");
  return pg::reconstruction_noalloc(type == PG_RECONSTRUCT_DILATE, conn8, *marker, *mask, *out,
                                    reinterpret_cast<cudaStream_t>(stream));
}

pg_status pg_batch_plan_set_config(pg_batch_plan *plan, int32_t tile, int32_t sweeps) {
  if (!plan) return pg::fail(PG_ERR_INVALID_ARGUMENT, "null plan");
  if (tile != 32 && tile != 64) return pg::fail(PG_ERR_INVALID_ARGUMENT, "batch plan tile side must be 32 or 64");
  if (tile == 64 && pg::elem_size(plan->ptype) == 8)
    return pg::fail(PG_ERR_INVALID_ARGUMENT, "batch plan tile side 64 needs pixels of at most 4 bytes");
  if (sweeps < 1) return pg::fail(PG_ERR_INVALID_ARGUMENT, "batch plan sweeps per visit must be >= 1");
  plan->cfg = pg::PlanCfg{tile, sweeps};
  return PG_OK;
}

pg_status pg_batch_plan_config(const pg_batch_plan *plan, int32_t *tile, int32_t *sweeps, int32_t *grid) {
  if (!plan) return pg::fail(PG_ERR_INVALID_ARGUMENT, "null plan");
  if (tile) *tile = plan->cfg.rt;
  if (sweeps) *sweeps = plan->cfg.sweeps;
  if (grid) *grid = plan->grid;
  return PG_OK;
}

}  // extern "C"
