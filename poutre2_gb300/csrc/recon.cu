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
// GPU design: tiles iterated to a tile-local fixpoint, scheduled until no tile changes.
//  * Pixels of at most 4 bytes (k_reconstruct_wl): 32x32 tiles, one warp per tile, the tile
//    in registers; directional sweep sets (down/up by warp shuffles, right/left after a
//    shared-memory transpose; two rows per register for 1- and 2-byte pixels) until a set
//    changes nothing.  The tiles are driven by a device worklist (a ticket ring and a state
//    per tile, below): a warp pops a tile, visits it, and queues the neighbours whose shared
//    border changed, until no tile is queued or running.
//  * 8-byte pixels, the allocation-free entry and one batch-plan configuration
//    (k_reconstruct): 64x64 (32x32) tiles staged in shared memory with a one-pixel halo and
//    swept by a CTA; rounds over the flagged tiles (round 0: all tiles, marker computed from
//    the inputs) separated by a grid barrier, until a round flags nothing.  Flags live in a
//    double-buffered device worklist; the "any flag" word is triple-buffered so no CTA resets
//    a word another may still read.
//  * Reads of other tiles' pixels bypass L1 (ld.global.cg): values only grow (shrink for
//    erosion), so a concurrently updated halo value is either the old or the new one, both
//    below the fixpoint; a tile that saw an old value is queued (flagged) again by its writer.
//  * Every wait is bounded (kBarrierTimeoutNs of %globaltimer on the grid barrier and on the
//    worklist; visit and round caps), recording PG_ERR_NOT_CONVERGED in a device status word.
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
__host__ __device__ constexpr int tile_side_for(int elem_bytes) { return elem_bytes == 8 ? 32 : 64; }
template <typename T> __host__ __device__ constexpr int tile_side() { return tile_side_for((int)sizeof(T)); }
static constexpr int kMaxSweeps = 512;
static constexpr int kVisitSweeps = 2;  // sweep sets per visit of a register tile (single calls)
static constexpr unsigned long long kBarrierTimeoutNs = 4000000000ull;  // 4 s

// Limits that a test may lower (pg_debug_set_limits): the device wait limit, passed to every launch
// and used by every bounded wait below, and a cap on the rounds (round kernel) / visits per tile
// (worklist kernel) that replaces the host's default when positive.
static std::atomic<unsigned long long> g_dbg_wait_ns{kBarrierTimeoutNs};
static std::atomic<int> g_dbg_max_rounds{0};

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
  unsigned long long wait_ns = kBarrierTimeoutNs;  // limit of every bounded device wait
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
__device__ bool grid_barrier(RCtl *ctl, unsigned long long wait_ns) {
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
        if (global_ns() - t0 > wait_ns) {
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

enum : int { B_N = 1, B_S = 2, B_W = 4, B_E = 8, B_NW = 16, B_NE = 32, B_SW = 64, B_SE = 128, B_SELF = 256 };  // B_x = 1 << direction

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
  // a changed corner pixel is also on a changed edge, so the edge bits cover every flag.  A
  // plain store: the writer does not wait for it (an atomic exchange would return a value).
  if (f & (B_N | B_S | B_W | B_E | B_SELF)) *((volatile unsigned *)&ctl->any[(round + 1) % 3]) = 1u;
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
// comparison or the leveling clip by the reference.  Pure streaming: 16-byte vectors when the
// image's buffers allow it, otherwise EPI_UNROLL independent elements per thread per step, so
// that many loads are in flight (a plain grid-stride loop over single pixels would wait for
// each load in turn).
static constexpr int EPI_UNROLL = 8;

template <typename T, bool SUP>
__device__ __forceinline__ uint8_t epi_binary(T ref, T rec) { return ref > rec ? 255 : 0; }

template <typename T, bool SUP>
__device__ void epilogue_image(const RImg &im, int epi, int64_t tid, int64_t nth) {
  const int64_t n = im.H * im.W;
  const T *rec = static_cast<const T *>(im.rec);
  const T *ref = static_cast<const T *>(im.mask);
  constexpr int VE = 16 / (int)sizeof(T);  // pixels per 16-byte vector
  const bool vec = ((reinterpret_cast<uintptr_t>(rec) | reinterpret_cast<uintptr_t>(ref) |
                     reinterpret_cast<uintptr_t>(im.out)) % 16 == 0);
  int64_t done = 0;
  if (epi == EPI_BINARY_SUP) {
    uint8_t *o = static_cast<uint8_t *>(im.out);
    if (vec && sizeof(T) == 1) {
      // 16 u8 pixels per thread and step: byte-wise unsigned compare gives 0xff / 0x00 directly
      const int64_t nv = n / 16;
      for (int64_t j = tid; j < nv; j += nth) {
        const uint4 a = __ldg(reinterpret_cast<const uint4 *>(ref) + j);
        const uint4 b = __ldcg(reinterpret_cast<const uint4 *>(rec) + j);
        reinterpret_cast<uint4 *>(o)[j] =
            make_uint4(__vcmpgtu4(a.x, b.x), __vcmpgtu4(a.y, b.y), __vcmpgtu4(a.z, b.z), __vcmpgtu4(a.w, b.w));
      }
      done = nv * 16;
    }
    for (int64_t i0 = done + tid; i0 < n; i0 += nth * EPI_UNROLL) {
      T a[EPI_UNROLL], b[EPI_UNROLL];
#pragma unroll
      for (int u = 0; u < EPI_UNROLL; ++u) {
        const int64_t i = i0 + u * nth;
        a[u] = i < n ? ldg(ref + i) : T(0);
        b[u] = i < n ? ld_cg(rec + i) : T(0);
      }
#pragma unroll
      for (int u = 0; u < EPI_UNROLL; ++u) {
        const int64_t i = i0 + u * nth;
        if (i < n) o[i] = epi_binary<T, SUP>(a[u], b[u]);
      }
    }
  } else {  // EPI_CLIP_REF: low leveling min(rec, ref), high leveling max(rec, ref)
    T *o = static_cast<T *>(im.out);
    if (vec) {
      const int64_t nv = n / VE;
      for (int64_t j = tid; j < nv; j += nth) {
        const Pack<T> a = Pack<T>::load_cg(rec + j * VE);
        const Pack<T> b = Pack<T>::load(ref + j * VE);
        Pack<T>::template op<!SUP>(a, b).store(o + j * VE);
      }
      done = nv * VE;
    }
    for (int64_t i0 = done + tid; i0 < n; i0 += nth * EPI_UNROLL) {
      T a[EPI_UNROLL], b[EPI_UNROLL];
#pragma unroll
      for (int u = 0; u < EPI_UNROLL; ++u) {
        const int64_t i = i0 + u * nth;
        a[u] = i < n ? ld_cg(rec + i) : T(0);
        b[u] = i < n ? ldg(ref + i) : T(0);
      }
#pragma unroll
      for (int u = 0; u < EPI_UNROLL; ++u) {
        const int64_t i = i0 + u * nth;
        if (i < n) o[i] = Op<T, !SUP>::apply(a[u], b[u]);
      }
    }
  }
}

template <typename T, bool SUP>
__device__ void recon_epilogue(const RParams<T> &P) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  for (int k = 0; k < P.nimg; ++k) epilogue_image<T, SUP>((P.nimg == 1) ? P.single : P.imgs[k], P.epi, tid, nth);
}

template <typename T, bool SUP, bool CONN8, int RT = tile_side<T>()>
__global__ void __launch_bounds__(RT) k_reconstruct(RParams<T> P) {
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
    if (!grid_barrier(ctl, P.wait_ns)) { ok = false; break; }
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

// element e (a compile-time constant after unrolling) of a 16-byte vector of 1- or 2-byte pixels
template <typename T> __device__ __forceinline__ T vec_elem(const uint4 &v, int e) {
  constexpr int PW = 4 / (int)sizeof(T);  // pixels per 32-bit word
  const int w = e / PW, sh = (e % PW) * 8 * (int)sizeof(T);
  const uint32_t word = w == 0 ? v.x : w == 1 ? v.y : w == 2 ? v.z : v.w;
  return (T)(word >> sh);
}

// Sweep sets of a 32x32 tile of 1- or 2-byte pixels with two rows per 32-bit register: pair p
// holds row p (low half) and row 31 - p (high half) of the lane's column, so the two chains that
// the vertical sweeps run at once (down over the top half with up over the bottom half, then the
// reverse) advance together in one 2x16-bit min/max per step; after the transpose, pair c holds
// columns c and 31 - c of the lane's row and the horizontal chains pair up the same way.  The
// masks are packed the same way.  Same updates, in the same order, as the
// unpacked sweeps.  Returns through v (unpacked) and the flags; s_m is overwritten.
__device__ __forceinline__ uint32_t u16x2_max(uint32_t a, uint32_t b) {
  uint32_t r;
  asm("max.u16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t u16x2_min(uint32_t a, uint32_t b) {
  uint32_t r;
  asm("min.u16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t pk2(uint32_t lo, uint32_t hi) { return (lo & 0xffffu) | (hi << 16); }
__device__ __forceinline__ uint32_t swap2(uint32_t x) { return __byte_perm(x, 0, 0x1032); }

__device__ __forceinline__ uint32_t lds_u32(const uint32_t *p) {  // see lds_mask
  const unsigned addr = (unsigned)__cvta_generic_to_shared(p);
  uint32_t r;
  asm volatile("ld.volatile.shared.b32 %0, [%1];" : "=r"(r) : "r"(addr));
  return r;
}

template <typename T, bool SUP, bool CONN8>
__device__ void sweeps_packed(T (&v)[32], RegS<T> *s_m, RegS<T> *s_t, int max_sweeps, T top, T bot, T hl, T hr,
                              T initL, T initR, bool &converged, bool &changed, bool &wch, bool &ech) {
  static_assert(sizeof(T) <= 2, "two pixels per register");
  const int lane = threadIdx.x & 31;
  auto OS = [](uint32_t a, uint32_t b) { return SUP ? u16x2_max(a, b) : u16x2_min(a, b); };  // propagation
  auto OC = [](uint32_t a, uint32_t b) { return SUP ? u16x2_min(a, b) : u16x2_max(a, b); };  // clip by the mask
  // packed masks, rewritten over the unpacked ones: rows 0-15 of s_m hold the column pairs
  // (lane = column), rows 16-31 the row pairs (lane = row)
  uint32_t P[16];
  {
    uint32_t MA[16], MB[16];
#pragma unroll
    for (int p = 0; p < 16; ++p) {
      MA[p] = pk2((uint32_t)s_m[p * kRP + lane], (uint32_t)s_m[(31 - p) * kRP + lane]);
      MB[p] = pk2((uint32_t)s_m[lane * kRP + p], (uint32_t)s_m[lane * kRP + 31 - p]);
    }
    __syncwarp();
#pragma unroll
    for (int p = 0; p < 16; ++p) {
      s_m[p * kRP + lane] = MA[p];
      s_m[(16 + p) * kRP + lane] = MB[p];
    }
    __syncwarp();
  }
  const uint32_t *MAs = reinterpret_cast<const uint32_t *>(s_m) + lane;
  const uint32_t *MBs = reinterpret_cast<const uint32_t *>(s_m) + 16 * kRP + lane;
#pragma unroll
  for (int p = 0; p < 16; ++p) P[p] = pk2(v[p], v[31 - p]);
  const uint32_t tb = pk2(top, bot), lr = pk2(hl, hr);
  auto nbrow = [&](uint32_t x) -> uint32_t {
    if (CONN8) {
      const uint32_t a = __shfl_up_sync(0xffffffffu, x, 1), b = __shfl_down_sync(0xffffffffu, x, 1);
      return OS(x, OS(a, b));
    }
    return x;
  };
  converged = false;
  changed = false;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    uint32_t ch = 0;
    // vertical: pair k from pair k - 1 (k = 0: the halo rows), then pair 15 from itself swapped
    // and pair q from pair q + 1
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const uint32_t nb = k == 0 ? tb : nbrow(P[k - 1]);  // the halo rows are already 3-wide
      const uint32_t nv = OC(OS(P[k], nb), lds_u32(MAs + k * kRP));
      ch |= nv ^ P[k];
      P[k] = nv;
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const int q = 15 - k;
      const uint32_t nb = nbrow(k == 0 ? swap2(P[15]) : P[q + 1]);
      const uint32_t nv = OC(OS(P[q], nb), lds_u32(MAs + q * kRP));
      ch |= nv ^ P[q];
      P[q] = nv;
    }
    // to lane = row
#pragma unroll
    for (int p = 0; p < 16; ++p) {
      s_t[p * kRP + lane] = P[p] & 0xffffu;
      s_t[(31 - p) * kRP + lane] = P[p] >> 16;
    }
    __syncwarp();
    uint32_t Q[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) Q[c] = pk2((uint32_t)s_t[lane * kRP + c], (uint32_t)s_t[lane * kRP + 31 - c]);
    __syncwarp();
    // horizontal, the same pairing
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const uint32_t nb = k == 0 ? lr : Q[k - 1];
      const uint32_t nv = OC(OS(Q[k], nb), lds_u32(MBs + k * kRP));
      ch |= nv ^ Q[k];
      Q[k] = nv;
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const int q = 15 - k;
      const uint32_t nb = k == 0 ? swap2(Q[15]) : Q[q + 1];
      const uint32_t nv = OC(OS(Q[q], nb), lds_u32(MBs + q * kRP));
      ch |= nv ^ Q[q];
      Q[q] = nv;
    }
    wch = (T)(Q[0] & 0xffffu) != initL;
    ech = (T)(Q[0] >> 16) != initR;
    // back to lane = column
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      s_t[lane * kRP + c] = Q[c] & 0xffffu;
      s_t[lane * kRP + 31 - c] = Q[c] >> 16;
    }
    __syncwarp();
#pragma unroll
    for (int p = 0; p < 16; ++p) P[p] = pk2((uint32_t)s_t[p * kRP + lane], (uint32_t)s_t[(31 - p) * kRP + lane]);
    __syncwarp();
    if (!__any_sync(0xffffffffu, ch != 0)) {
      converged = true;
      break;
    }
    changed = true;
  }
#pragma unroll
  for (int p = 0; p < 16; ++p) {
    v[p] = (T)(P[p] & 0xffffu);
    v[31 - p] = (T)(P[p] >> 16);
  }
}

// One visit of a register tile: stage it from the reconstruction buffer (which the worklist
// kernel's first phase set to the marker), iterate sweep sets to the tile-local fixpoint (or
// P.max_sweeps), write it back if anything changed.  Returns the B_* bits of the borders that
// changed (the neighbours to revisit) and B_SELF when the tile yielded.  Warp-uniform.
template <typename T, bool SUP, bool CONN8>
__device__ int process_tile_reg(const RImg &im, const RParams<T> &P, int t_local, RegS<T> *s_m, RegS<T> *s_t) {
  using OS = Op<T, SUP>;   // propagation
  using OC = Op<T, !SUP>;  // clip by the mask
  const int lane = threadIdx.x & 31;
  const T NEU = OS::neutral();
  const int tx = t_local % im.tiles_x, ty = t_local / im.tiles_x;
  const int64_t y0 = (int64_t)ty * 32, x0 = (int64_t)tx * 32;
  const T *rec_in = static_cast<const T *>(im.rec);
  const int64_t gx = x0 + lane;
  const bool colin = gx < im.W;

  // Halo loads first (they stay in flight during the stage).  Its values stay fixed during the
  // visit, so each halo pixel's contribution is folded into one value per border pixel:
  // `top`/`bot` per column (lane = column: the three pixels above / below), `hl`/`hr` per row
  // (lane = row: the three pixels left / right; one in 4-connectivity).  The sweeps apply them
  // at the tile's first/last row and column.  Addresses outside the image are clamped to pixel
  // 0 and the values replaced by the neutral element.
  constexpr int NH = CONN8 ? 12 : 4;
  const int64_t hy[12] = {y0 - 1, y0 + 32, y0 + lane, y0 + lane, y0 - 1, y0 - 1, y0 + 32, y0 + 32,
                          y0 + lane - 1, y0 + lane + 1, y0 + lane - 1, y0 + lane + 1};
  const int64_t hx[12] = {gx, gx, x0 - 1, x0 + 32, gx - 1, gx + 1, gx - 1, gx + 1, x0 - 1, x0 - 1, x0 + 32, x0 + 32};
  T hv[NH];
#pragma unroll
  for (int k = 0; k < NH; ++k) {
    const bool in = hy[k] >= 0 && hy[k] < im.H && hx[k] >= 0 && hx[k] < im.W;
    hv[k] = ld_cg(rec_in + (in ? hy[k] * im.W + hx[k] : 0));
    if (!in) hv[k] = NEU;  // applied after the load returns; the load itself is unconditional
  }

  // stage, lane = column: tile values and mask (pixels outside the image: neutral, fixed).
  const T *mk_in = static_cast<const T *>(im.marker);
  const T *ms_in = static_cast<const T *>(im.mask);
  const bool need_mk = needs_marker(P, 1);
  T v[32];
  bool vec = false;
  if constexpr (sizeof(T) <= 2) {
    // rows of whole 16-byte vectors: the tile (32 rows x 32 or 64 bytes) comes in 2 * sizeof(T)
    // vector loads per lane and array, unpacked into shared memory; v is then read per column
    vec = (im.W * (int64_t)sizeof(T)) % 16 == 0 &&
          ((reinterpret_cast<uintptr_t>(ms_in) | reinterpret_cast<uintptr_t>(rec_in) |
            (need_mk ? reinterpret_cast<uintptr_t>(mk_in) : (uintptr_t)0)) % 16) == 0;
  }
  if (vec) {
    constexpr int VPR = 2 * (int)sizeof(T);   // 16-byte vectors per tile row
    constexpr int VPX = 16 / (int)sizeof(T);  // pixels per vector
    uint4 ma[VPR], ka[VPR], ra[VPR];
#pragma unroll
    for (int k = 0; k < VPR; ++k) {
      const int q = k * 32 + lane, row = q / VPR, vc = q % VPR;
      const int64_t gy = y0 + row, gx0 = x0 + vc * VPX;
      const int64_t gi = (gy < im.H && gx0 < im.W) ? gy * im.W + gx0 : 0;
      ma[k] = __ldg(reinterpret_cast<const uint4 *>(ms_in + gi));
      ka[k] = need_mk ? __ldg(reinterpret_cast<const uint4 *>(mk_in + gi)) : ma[k];
      ra[k] = __ldcg(reinterpret_cast<const uint4 *>(rec_in + gi));
    }
#pragma unroll
    for (int k = 0; k < VPR; ++k) {
      const int q = k * 32 + lane, row = q / VPR, vc = q % VPR;
      const bool ok = y0 + row < im.H && x0 + vc * VPX < im.W;
#pragma unroll
      for (int e = 0; e < VPX; ++e) {
        const T a = vec_elem<T>(ma[k], e), b = vec_elem<T>(ka[k], e), c = vec_elem<T>(ra[k], e);
        s_m[row * kRP + vc * VPX + e] = ok ? combine_mask(P, a, b) : NEU;
        s_t[row * kRP + vc * VPX + e] = ok ? c : NEU;
      }
    }
    __syncwarp();
#pragma unroll
    for (int r = 0; r < 32; ++r) v[r] = (T)s_t[r * kRP + lane];
    __syncwarp();
  } else {
  // scalar stage: loads come first, 16 rows at a time, so that they are all in flight together
#pragma unroll
  for (int h = 0; h < 32; h += 16) {
    T a[16], b[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int64_t gy = y0 + h + r;
      const int64_t gi = (colin && gy < im.H) ? gy * im.W + gx : 0;
      a[r] = ldg(ms_in + gi);
      b[r] = need_mk ? ldg(mk_in + gi) : a[r];
      v[h + r] = ld_cg(rec_in + gi);
    }
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const bool ok = colin && y0 + h + r < im.H;
      T m = combine_mask(P, a[r], b[r]);
      if (!ok) {
        m = NEU;
        v[h + r] = NEU;
      }
      s_m[(h + r) * kRP + lane] = m;
    }
  }
  }
  T top = hv[0], bot = hv[1], hl = hv[2], hr = hv[3];
  if (CONN8) {
    top = OS::apply(top, OS::apply(hv[4], hv[5]));
    bot = OS::apply(bot, OS::apply(hv[6], hv[7]));
    hl = OS::apply(hl, OS::apply(hv[8], hv[9]));
    hr = OS::apply(hr, OS::apply(hv[10], hv[11]));
  }
  // staged borders, to tell afterwards which neighbours must be revisited
#pragma unroll
  for (int r = 0; r < 32; ++r) s_t[r * kRP + lane] = v[r];
  __syncwarp();
  const T initL = (T)s_t[lane * kRP], initR = (T)s_t[lane * kRP + 31];
  const T initT = v[0], initB = v[31];
  __syncwarp();

  bool converged = false, changed = false, wch = false, ech = false;
  if constexpr (sizeof(T) <= 2) {
    sweeps_packed<T, SUP, CONN8>(v, s_m, s_t, P.max_sweeps, top, bot, hl, hr, initL, initR, converged, changed, wch, ech);
  } else {
  for (int sweep = 0; sweep < P.max_sweeps; ++sweep) {
    bool ch = false;
    auto vstep = [&](int r, T nb) {
      const T nv = OC::apply(OS::apply(v[r], nb), lds_mask<T>(s_m + r * kRP + lane));
      ch |= nv != v[r];
      v[r] = nv;
    };
    // the three pixels of a row seen from the row below / above (lanes 0 and 31 get their own
    // value back from the shuffle: the pixels beyond the tile's sides are halo, applied by the
    // horizontal sweeps)
    auto nbrow = [&](T p) -> T {
      if (CONN8) return OS::apply(p, OS::apply(shfl_up1(p), shfl_dn1(p)));
      return p;
    };
    // vertical, two independent chains at once: down over the top half with up over the
    // bottom half, then down over the bottom half with up over the top half.  A value still
    // travels the whole column in one direction per sweep set.
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const T nd = (k == 0) ? top : nbrow(v[k - 1]);
      const T nu = (k == 0) ? bot : nbrow(v[32 - k]);
      vstep(k, nd);
      vstep(31 - k, nu);
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const T nd = nbrow(v[15 + k]);
      const T nu = nbrow(v[16 - k]);
      vstep(16 + k, nd);
      vstep(15 - k, nu);
    }
    // to lane = row
#pragma unroll
    for (int r = 0; r < 32; ++r) s_t[r * kRP + lane] = v[r];
    __syncwarp();
#pragma unroll
    for (int c = 0; c < 32; ++c) v[c] = (T)s_t[lane * kRP + c];
    __syncwarp();
    // horizontal (the pixel on the left / on the right), two chains at once in the same way
    auto hstep = [&](int c, T nb) {
      const T nv = OC::apply(OS::apply(v[c], nb), lds_mask<T>(s_m + lane * kRP + c));
      ch |= nv != v[c];
      v[c] = nv;
    };
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      hstep(k, k == 0 ? hl : v[k - 1]);
      hstep(31 - k, k == 0 ? hr : v[32 - k]);
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      hstep(16 + k, v[15 + k]);
      hstep(15 - k, v[16 - k]);
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

  if (changed && vec) {
    // the stage's vector layout in reverse: columns to shared memory, rows out as 16-byte stores
    if constexpr (sizeof(T) <= 2) {
      constexpr int VPR = 2 * (int)sizeof(T), VPX = 16 / (int)sizeof(T), PW = 4 / (int)sizeof(T);
#pragma unroll
      for (int r = 0; r < 32; ++r) s_t[r * kRP + lane] = v[r];
      __syncwarp();
      T *rec = static_cast<T *>(im.rec);
#pragma unroll
      for (int k = 0; k < VPR; ++k) {
        const int q = k * 32 + lane, row = q / VPR, vc = q % VPR;
        const int64_t gy = y0 + row, gx0 = x0 + vc * VPX;
        uint32_t w[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          w[j] = 0u;
#pragma unroll
          for (int e = 0; e < PW; ++e)
            w[j] |= ((uint32_t)s_t[row * kRP + vc * VPX + j * PW + e] & Lim<T>::hi()) << (8 * (int)sizeof(T) * e);
        }
        if (gy < im.H && gx0 < im.W) __stcg(reinterpret_cast<uint4 *>(rec + gy * im.W + gx0), make_uint4(w[0], w[1], w[2], w[3]));
      }
      __syncwarp();
    }
  } else if (changed) {
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
  return f;
}

// ------------------------------------------------------------------ tile worklist
// The register-tile kernel has no rounds.  Every tile is queued once at the start; a warp pops
// a tile, visits it, and queues the neighbours whose shared border changed.  The kernel ends
// when no tile is queued or being visited (`pending` == 0).  A tile is visited by one warp at a
// time, through its state:
//   IDLE --queue--> QUEUED --pop--> RUNNING --done--> IDLE (or QUEUED again if it yielded)
//   RUNNING --a neighbour changed its border meanwhile--> DIRTY --done--> QUEUED
// The queue is a ring of 64-bit slots (position tag << 32 | tile + 1), a multi-producer multi-
// consumer ring with sequence numbers: a popper takes a ticket with one atomicAdd on `head`
// and waits for its slot to carry its position; a pusher takes positions with one atomicAdd
// on `tail` and waits until the slot's previous lap was consumed (tag = position - cap, tile
// field 0).  No compare-and-swap retries on the shared counters.
enum : unsigned { TS_IDLE = 0, TS_QUEUED = 1, TS_RUNNING = 2, TS_DIRTY = 3 };

// `tail` (next position to push, low 32 bits) and `pending` (tiles queued or being visited, high
// 32 bits) share one 64-bit word, so that a warp counts the tiles it pushes and reserves their
// positions in one atomic: a tile cannot be popped and finished (pending - 1) before its own
// pending + 1 is performed.
struct RQueue {                // each counter on its own 128-byte line
  unsigned head, pad0[31];     // next ticket to pop
  unsigned long long tp;       // pending << 32 | tail
  unsigned pad1[30];
  unsigned pad2[64];
};
__device__ __forceinline__ unsigned tp_tail(unsigned long long tp) { return (unsigned)tp; }
__device__ __forceinline__ int tp_pending(unsigned long long tp) { return (int)(tp >> 32); }
static_assert(sizeof(RQueue) == 512, "RQueue layout");

template <typename T> struct WorkList {
  RQueue *q;
  unsigned *state;             // ntiles
  unsigned long long *ring;    // cap slots
  unsigned cap;
  unsigned long long wait_ns;  // limit of every bounded wait
};

__device__ __forceinline__ bool wait_expired(RCtl *ctl, unsigned long long t0, unsigned long long wait_ns) {
  if (global_ns() - t0 > wait_ns) {
    set_status(ctl, PG_ERR_NOT_CONVERGED);
    return true;
  }
  return false;
}

__device__ __forceinline__ unsigned long long slot_val(unsigned pos, unsigned tile1) {
  return ((unsigned long long)pos << 32) | tile1;
}

// Lane 0 pops: the tile to visit, or -1 when the work is done or an error was recorded.
template <typename T>
__device__ int wl_pop(const WorkList<T> &wl, RCtl *ctl, long long max_tickets) {
  const unsigned pos = atomicAdd(&wl.q->head, 1u);
  if ((long long)pos >= max_tickets) {  // runaway guard: far more visits than any input needs
    set_status(ctl, PG_ERR_NOT_CONVERGED);
    return -1;
  }
  volatile unsigned long long *slot = wl.ring + pos % wl.cap;
  const unsigned long long t0 = global_ns();
  unsigned ns = 32;
  unsigned long long v;
  for (;;) {
    // the three words are read together (one memory round trip per poll, not three in a row)
    v = *slot;
    const unsigned long long tp = *((volatile unsigned long long *)&wl.q->tp);
    const int st = *((volatile int *)&ctl->status);
    if ((unsigned)(v >> 32) == pos && (unsigned)v != 0u) break;
    if (tp_pending(tp) == 0) return -1;
    if (st != 0) return -1;
    __nanosleep(ns);
    if (ns < 1024) ns <<= 1;  // longest back-off 1 us: measured 6 % faster than 4 us on the h-maxima input
    if (wait_expired(ctl, t0, wl.wait_ns)) return -1;
  }
  *slot = slot_val(pos, 0u);  // consumed: the next lap's pusher may write
  const unsigned tile = (unsigned)v - 1u;
  *((volatile unsigned *)(wl.state + tile)) = TS_RUNNING;  // QUEUED until now: nobody else moves it
  __threadfence();  // the neighbours' pixels written before they queued this tile
  return (int)tile;
}

// Retry limit of the state-change loops below: a retry means another warp changed the same
// word in between, which happens a bounded number of times; the limit only guards the kernel.
static constexpr int kCasRetries = 1 << 20;

// Warp-wide end of a visit: lanes 0..7 queue the neighbours whose shared border changed (one
// lane each, in parallel), lane 8 releases the tile (or queues it again), and the queued tiles
// are pushed with one position reservation for the warp.  Called by the whole warp.
// (Keeping one queued neighbour as the warp's next visit, past the ring, was measured: it
// shortens long propagations but makes tiles of short ones -- the h-extrema -- be revisited
// more often, so every queued tile goes through the ring.)
template <typename T, bool CONN8>
__device__ void wl_finish(const WorkList<T> &wl, RCtl *ctl, const RImg &im, int tile, int t_local, int f) {
  const int lane = threadIdx.x & 31;
  const int tx = t_local % im.tiles_x, ty = t_local / im.tiles_x;
  // lane d < 8 handles direction d = N S W E NW NE SW SE, whose B_* bit is 1 << d
  int cand = -1;
  bool push = false;
  if (lane < (CONN8 ? 8 : 4) && (f & (1 << lane))) {
    const int dx = lane < 2 ? 0 : ((lane & 1) ? 1 : -1);
    const int dy = lane < 2 ? (lane ? 1 : -1) : lane < 4 ? 0 : (lane < 6 ? -1 : 1);
    const int nx = tx + dx, ny = ty + dy;
    if (nx >= 0 && ny >= 0 && nx < im.tiles_x && ny < im.tiles_y) cand = im.tile_begin + ny * im.tiles_x + nx;
  }
  if (cand >= 0) {
    bool done = false;
    for (int it = 0; it < kCasRetries && !done; ++it) {
      const unsigned s = atomicCAS(wl.state + cand, TS_IDLE, TS_QUEUED);
      if (s == TS_IDLE) push = done = true;
      else if (s != TS_RUNNING) done = true;  // already queued, or already marked for another visit
      else if (atomicCAS(wl.state + cand, TS_RUNNING, TS_DIRTY) == TS_RUNNING) done = true;
    }
    if (!done) set_status(ctl, PG_ERR_NOT_CONVERGED);
  }
  if (lane == 8) {
    // release: back to IDLE, or queued again if it yielded or a neighbour changed meanwhile
    const bool yielded = (f & B_SELF) != 0;
    bool done = false;
    for (int it = 0; it < kCasRetries && !done; ++it) {
      const unsigned s = *((volatile unsigned *)(wl.state + tile));  // RUNNING or DIRTY: only we move it out
      if (s == TS_DIRTY || yielded) {
        if (atomicCAS(wl.state + tile, s, TS_QUEUED) == s) push = done = true;
      } else if (atomicCAS(wl.state + tile, TS_RUNNING, TS_IDLE) == TS_RUNNING) {
        done = true;
      }
    }
    if (!done) set_status(ctl, PG_ERR_NOT_CONVERGED);
    cand = tile;
  }
  const unsigned pm = __ballot_sync(0xffffffffu, push);
  const int n = __popc(pm);
  unsigned base = 0;
  if (lane == 0 && n > 0) {
    base = tp_tail(atomicAdd(&wl.q->tp, ((unsigned long long)n << 32) | (unsigned long long)n));
  }
  base = __shfl_sync(0xffffffffu, base, 0);
  if (push) {
    const unsigned pos = base + __popc(pm & ((1u << lane) - 1u));
    volatile unsigned long long *slot = wl.ring + pos % wl.cap;
    const unsigned long long want = slot_val(pos - wl.cap, 0u);  // previous lap consumed
    // the first lap's slots were set to `want` before the grid barrier of phase 0: no need to look
    if (pos >= wl.cap) {
      const unsigned long long t0 = global_ns();
      while (*slot != want) {
        __nanosleep(64);
        if (wait_expired(ctl, t0, wl.wait_ns)) break;
      }
    }
    *slot = slot_val(pos, (unsigned)cand + 1u);
  }
  // pending - 1, after this warp's pushes were counted (same word, same thread): never 0 early
  if (lane == 0) atomicAdd(&wl.q->tp, ~0ull << 32);
}

// first phase: every reconstruction buffer starts at the marker (select_marker, or the
// saturated shift of the h-extrema), EPI_UNROLL pixels per thread and step
template <typename T, bool SUP>
__device__ void init_rec(const RParams<T> &P, int64_t tid, int64_t nth) {
  const bool need_mk = needs_marker(P, 0);
  for (int k = 0; k < P.nimg; ++k) {
    const RImg &im = (P.nimg == 1) ? P.single : P.imgs[k];
    const int64_t n = im.H * im.W;
    const T *ms = static_cast<const T *>(im.mask);
    const T *mk = static_cast<const T *>(im.marker);
    T *rec = static_cast<T *>(im.rec);
    for (int64_t i0 = tid; i0 < n; i0 += nth * EPI_UNROLL) {
      T a[EPI_UNROLL], b[EPI_UNROLL];
#pragma unroll
      for (int u = 0; u < EPI_UNROLL; ++u) {
        const int64_t i = i0 + u * nth;
        a[u] = i < n ? ldg(ms + i) : T(0);
        b[u] = (need_mk && i < n) ? ldg(mk + i) : a[u];
      }
#pragma unroll
      for (int u = 0; u < EPI_UNROLL; ++u) {
        const int64_t i = i0 + u * nth;
        T m, v;
        combine_init<T, SUP>(P, a[u], b[u], m, v);
        if (i < n) st_cg(rec + i, v);
      }
    }
  }
}

__device__ long long g_recon_visits = 0;

template <typename T, bool SUP, bool CONN8>
__global__ void __launch_bounds__(kRegWarps * 32, 4) k_reconstruct_wl(RParams<T> P, WorkList<T> wl) {
  static_assert(sizeof(T) <= 4, "register tiles hold pixels of at most 4 bytes");
  __shared__ RegS<T> s_m[kRegWarps][32 * kRP];
  __shared__ RegS<T> s_t[kRegWarps][32 * kRP];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  RCtl *ctl = P.ctl;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;

  // phase 0: marker into the reconstruction buffers, every tile queued once
  init_rec<T, SUP>(P, tid, nth);
  for (int64_t i = tid; i < (int64_t)wl.cap; i += nth) {
    // positions 0..ntiles-1 hold the tiles; the others wait for their first lap
    wl.ring[i] = i < P.ntiles ? slot_val((unsigned)i, (unsigned)i + 1u) : slot_val((unsigned)i - wl.cap, 0u);
    if (i < P.ntiles) wl.state[i] = TS_QUEUED;
  }
  if (tid == 0) {
    wl.q->tp = ((unsigned long long)P.ntiles << 32) | (unsigned long long)P.ntiles;
  }
  if (!grid_barrier(ctl, P.wait_ns)) return;

  // phase 1: visits until no tile is queued or running
  // runaway guard on the tickets (visits plus idle pops), also below the wrap of the 32-bit ring
  // positions
  const long long max_tickets = std::min<long long>((long long)P.ntiles * P.max_rounds, (1ll << 31) - 2ll * P.ntiles);
  for (;;) {
    int t = -1;
    if (lane == 0) t = wl_pop(wl, ctl, max_tickets);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t < 0) break;
    int tl = 0;
    const RImg &im = image_of(P, t, tl);
    const int f = process_tile_reg<T, SUP, CONN8>(im, P, tl, s_m[warp], s_t[warp]);
    __threadfence();  // this tile's pixels, before any neighbour is queued
    __syncwarp();
    wl_finish<T, CONN8>(wl, ctl, im, t, tl, f);
    __syncwarp();
  }
  if (!grid_barrier(ctl, P.wait_ns)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const long long visits = (long long)tp_tail(*((volatile unsigned long long *)&wl.q->tp));  // every pushed tile was visited
    g_recon_visits = visits;
    g_recon_rounds = (int)((visits + P.ntiles - 1) / P.ntiles);
    ctl->rounds = g_recon_rounds;
  }
  if (P.epi == EPI_NONE) return;
  recon_epilogue<T, SUP>(P);
}

// ------------------------------------------------------------------ host side
// Scratch work area of one launch: control block (256 B) | worklist counters (512 B) | per-tile
// words: the double-buffered flags of the round kernel, or the tile states and the ring of the
// worklist.  The work area is cleared before the launch.
static constexpr size_t kWorkHead = 256 + sizeof(RQueue);

// Rounds (round kernel) or visits per tile (worklist kernel) before a launch gives up: far more than
// any input needs (a tile is revisited only when a neighbour changed its border), unless a test set
// a cap through pg_debug_set_limits.
static int max_rounds_for(int64_t ntiles) {
  const int cap = g_dbg_max_rounds.load();
  if (cap > 0) return cap;
  return (int)std::min<int64_t>(INT32_MAX / 2, 1024 + 64 * ntiles);
}
static unsigned ring_cap(int64_t ntiles) { return (unsigned)(2 * ntiles + 4096); }
static size_t ring_offset(int64_t ntiles) { return ((4 * (size_t)ntiles + 255) / 256) * 256; }
static size_t work_bytes(int64_t ntiles) {
  return kWorkHead + ring_offset(ntiles) + ((8 * (size_t)ring_cap(ntiles) + 255) / 256) * 256;
}

// Launches the reconstruction kernel for tile side RT: the worklist kernel on register tiles
// for 32-pixel tiles of pixels up to 4 bytes, the round kernel on shared-memory tiles otherwise.
// P's images, tiles and modes are set by the caller; `work` is a cleared work area.
template <typename T, bool SUP, bool CONN8, int RT>
static pg_status launch_recon(RParams<T> &P, char *work, cudaStream_t s, int *grid_out) {
  constexpr bool REG = RT == 32 && sizeof(T) <= 4;
  constexpr int THREADS = REG ? kRegWarps * 32 : RT;
  constexpr int TILES_PER_CTA = REG ? kRegWarps : 1;
  P.ctl = reinterpret_cast<RCtl *>(work);
  P.flags = reinterpret_cast<unsigned *>(work + kWorkHead);
  P.max_rounds = max_rounds_for(P.ntiles);
  P.wait_ns = g_dbg_wait_ns.load();
  WorkList<T> wl{};
  wl.wait_ns = P.wait_ns;
  wl.q = reinterpret_cast<RQueue *>(work + 256);
  wl.state = P.flags;
  wl.ring = reinterpret_cast<unsigned long long *>(work + kWorkHead + ring_offset(P.ntiles));
  wl.cap = ring_cap(P.ntiles);
  void *kern = nullptr;
  if constexpr (REG) kern = reinterpret_cast<void *>(k_reconstruct_wl<T, SUP, CONN8>);
  else kern = reinterpret_cast<void *>(k_reconstruct<T, SUP, CONN8, RT>);
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  static std::mutex mu;
  static std::vector<int> cached;  // blocks per SM, per device
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    if ((size_t)dev >= cached.size()) cached.resize((size_t)dev + 1, 0);
    if (cached[(size_t)dev] == 0)
      PG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cached[(size_t)dev], kern, THREADS, 0), "occupancy");
    per_sm = cached[(size_t)dev];
  }
  if (per_sm < 1) return fail(PG_ERR_CUDA, "reconstruction kernel cannot be resident");
  int grid = per_sm * num_sms();
  if (grid > ceil_div(P.ntiles, TILES_PER_CTA)) grid = (int)ceil_div(P.ntiles, TILES_PER_CTA);
  if (grid_out) *grid_out = grid;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(THREADS);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if constexpr (REG) PG_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_reconstruct_wl<T, SUP, CONN8>, P, wl), "cooperative reconstruction launch");
  else PG_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_reconstruct<T, SUP, CONN8, RT>, P), "cooperative reconstruction launch");
  return PG_OK;
}

template <typename T, bool SUP, bool CONN8>
static pg_status run_t(std::vector<RImg> &imgs, const ReconRequest &rq, bool binary, cudaStream_t s) {
  // register tiles (32x32, a warp each) up to 4-byte pixels, shared-memory tiles for 8-byte ones
  constexpr int RT = sizeof(T) <= 4 ? 32 : tile_side<T>();
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
  // scratch: work area | image table | reconstruction buffers (binary mode)
  const size_t off_tab = work_bytes(ntiles);
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
  PG_CUDA_TRY(cudaMemsetAsync(base, 0, off_tab, s), "clear reconstruction work area");
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
  P.init = rq.init;
  P.mask_mode = rq.mask_mode;
  P.epi = rq.epi;
  P.h = scalar_as<T>(rq.h);
  // register tiles yield after kVisitSweeps sweep sets and are revisited: measured as fast or faster
  // than sweeping each visit to its local fixpoint (h-maxima 4096^2 -2 %, a long propagation -6 %)
  if constexpr (RT == 32 && sizeof(T) <= 4) P.max_sweeps = kVisitSweeps;
  return launch_recon<T, SUP, CONN8, RT>(P, base, s, nullptr);
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
  if (masks[0].rank == 3) {  // volumes: the iterated geodesic step of recon3d.cu, one volume at a time
    for (int i = 0; i < n_images; ++i)
      PG_TRY(launch_reconstruction3d(markers ? &markers[i] : nullptr, masks[i], outs[i], rq, s));
    return PG_OK;
  }
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
  pg_scalar h{};
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
  P.max_sweeps = sweeps;
  P.init = INIT_SAT_CONST;
  P.mask_mode = MASK_PLAIN;
  P.epi = EPI_BINARY_SUP;
  P.h = scalar_as<T>(p.h);
  PG_CUDA_TRY(cudaMemsetAsync(p.scratch, 0, p.clear_bytes, s), "clear batch work area");
  return launch_recon<T, true, CONN8, RT>(P, static_cast<char *>(p.scratch), s, grid_out);
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

pg_status create_batch_plan(const pg_image *ins, const pg_image *outs, int n, const pg_scalar &h, bool conn8, bool autotune,
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
  const size_t off_tab64 = work_bytes(max_tiles);
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
      for (int sw : {kVisitSweeps, 4, 16, kMaxSweeps}) cands.push_back(PlanCfg{rt, sw});
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

// Tiles of an H x W image in the no-alloc kernel (tile_side<T>() squares: 64, or 32 for 8-byte
// pixels) and the most the fixed scratch holds (two flag words per tile above the control block).
// The one place both numbers are computed: the entry point's shape check and the launch use it.
static void noalloc_tiles(int elem_bytes, int64_t H, int64_t W, int64_t &ntiles, int64_t &max_tiles) {
  const int64_t rt = tile_side_for(elem_bytes);
  ntiles = ceil_div(H, rt) * ceil_div(W, rt);
  max_tiles = (int64_t)((kNoAllocScratchBytes - kNoAllocFlagsOffset) / (2 * sizeof(unsigned)));
}

// Device address of g_noalloc_scratch, looked up once per device with that device current.
// In host code the symbol name is only a host-side stand-in, so the kernel is given this
// address instead.  The address is kept for the life of the process: after cudaDeviceReset
// (which destroys the context holding the array) this entry point must not be called again.
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
  int64_t ntiles = 0, max_tiles = 0;
  noalloc_tiles((int)sizeof(T), im.H, im.W, ntiles, max_tiles);
  if (ntiles == 0) return PG_OK;
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
  P.max_rounds = max_rounds_for(ntiles);
  P.wait_ns = g_dbg_wait_ns.load();
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
  if (const int rs = pg::take_rect_status())
    return pg::fail(static_cast<pg_status>(rs), "a box tile load did not complete within its wait limit");
  if (const int ds = pg::take_diag_status())
    return pg::fail(static_cast<pg_status>(ds), "a segment tile load did not complete within its wait limit");
  if (const int os8 = pg::take_oct_status())
    return pg::fail(static_cast<pg_status>(os8), "an octagon tile load did not complete within its wait limit");
  if (const int ss = pg::take_small_tile_status())
    return pg::fail(static_cast<pg_status>(ss), "a small-SE tile load did not complete within its wait limit");
  if (const int os = pg::take_open_status())
    return pg::fail(static_cast<pg_status>(os), "an opening tile load did not complete within its wait limit");
  if (const int ls = pg::take_label_status())
    return pg::fail(static_cast<pg_status>(ls), "a labelling union-find loop exceeded its iteration limit");
  return PG_OK;
}

// Test hooks: lower the reconstruction's round / visit cap and its device wait limit so that a test
// can make a bounded wait run out and read PG_ERR_NOT_CONVERGED back; 0 restores the defaults.
pg_status pg_debug_set_limits(int32_t max_rounds, int64_t wait_ns) {
  if (max_rounds < 0 || wait_ns < 0) return pg::fail(PG_ERR_INVALID_ARGUMENT, "pg_debug_set_limits: negative limit");
  pg::g_dbg_max_rounds.store(max_rounds);
  pg::g_dbg_wait_ns.store(wait_ns > 0 ? (unsigned long long)wait_ns : pg::kBarrierTimeoutNs);
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
  // the checks of pg_reconstruction, in its order
  PG_TRY(pg::check_in_out(marker, out, "t_Reconstruct"));
  PG_TRY(pg::check_in_out(mask, out, "t_Reconstruct"));
  if (type != PG_RECONSTRUCT_ERODE && type != PG_RECONSTRUCT_DILATE)
    return pg::fail(PG_ERR_INVALID_ARGUMENT, "t_ReconstructionDispatchRectType unsupported reconstruction_type");
  bool conn8 = true;
  PG_TRY(pg::recon_se(se, mask->rank, conn8));
  // then the limits of this entry point
  if (mask->rank == 3)
    return pg::fail(PG_ERR_UNSUPPORTED_SE, "pg_reconstruction_noalloc: 1D and 2D images only (volumes need "
                                           "pg_reconstruction)");
  const pg::Dims d = pg::dims_of(*mask);
  int64_t ntiles = 0, max_tiles = 0;
  pg::noalloc_tiles(pg::elem_size(mask->ptype), d.nz * d.ny, d.nx, ntiles, max_tiles);
  if (ntiles > max_tiles)
    return pg::fail(PG_ERR_INVALID_ARGUMENT, "pg_reconstruction_noalloc: the image needs " + std::to_string(ntiles) +
                                                 " tiles; the fixed scratch holds at most " + std::to_string(max_tiles));
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
