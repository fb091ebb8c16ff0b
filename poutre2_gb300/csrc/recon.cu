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

// Grid barrier with a bounded wait.  Returns false once any CTA recorded an error.
__device__ bool grid_barrier(RCtl *ctl) {
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
  }
  __syncthreads();
  return *((volatile int *)&ctl->status) == 0;
}

template <typename T, bool SUP>
__device__ __forceinline__ T sat_shift(T m, T h) {
  // marker of h-maxima (sat_sub) / h-minima (sat_add), op_Saturated_{Sub,Add}_Constant
  // (pixel_processing/details/arith_op_t.hpp:218-345), clamped to the pixel type's range
  if constexpr (std::is_integral_v<T>) {
    using Wide = std::conditional_t<(sizeof(T) < 8), long long, __int128>;
    const Wide r = SUP ? (Wide)m - (Wide)h : (Wide)m + (Wide)h;
    if (r < (Wide)Lim<T>::lo()) return Lim<T>::lo();
    if (r > (Wide)Lim<T>::hi()) return Lim<T>::hi();
    return (T)r;
  } else {
    return SUP ? m - h : m + h;
  }
}

// effective mask and initial value of pixel i
template <typename T, bool SUP>
__device__ __forceinline__ void pixel_init(const RImg &im, const RParams<T> &P, int64_t i, T &mask, T &init) {
  const T a = ldg(static_cast<const T *>(im.mask) + i);
  if (P.init == INIT_SAT_CONST) {
    mask = a;
    init = sat_shift<T, SUP>(a, P.h);
    return;
  }
  const T mk = ldg(static_cast<const T *>(im.marker) + i);
  if (P.mask_mode == MASK_MAX_MARKER) mask = Op<T, true>::apply(mk, a);
  else if (P.mask_mode == MASK_MIN_MARKER) mask = Op<T, false>::apply(mk, a);
  else mask = a;
  init = Op<T, !SUP>::apply(mk, mask);  // select_marker: min(marker, mask) / max for erosion
}

template <typename T, bool SUP>
__device__ __forceinline__ T pixel_mask(const RImg &im, const RParams<T> &P, int64_t i) {
  const T a = ldg(static_cast<const T *>(im.mask) + i);
  if (P.init == INIT_SAT_CONST || P.mask_mode == MASK_PLAIN) return a;
  const T mk = ldg(static_cast<const T *>(im.marker) + i);
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

  // stage: current reconstruction (round 0: marker) with halo, effective mask
  for (int i = threadIdx.x; i < (RT + 2) * (RT + 2); i += RTHREADS) {
    const int r = i / (RT + 2) - 1, c = i % (RT + 2) - 1;
    const int64_t gy = y0 + r, gx = x0 + c;
    const bool inside = gy >= 0 && gy < im.H && gx >= 0 && gx < im.W;
    const bool interior = r >= 0 && r < RT && c >= 0 && c < RT;
    T v = NEU, m = NEU;
    if (inside) {
      const int64_t gi = gy * im.W + gx;
      if (round == 0) pixel_init<T, SUP>(im, P, gi, m, v);
      else {
        v = ld_cg(rec_in + gi);
        if (interior) m = pixel_mask<T, SUP>(im, P, gi);
      }
    }
    s_out[(r + 1) * PO + (c + 1)] = v;
    if (interior) s_mask[r * PM + c] = m;
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
  }
  if (!converged) bflags |= B_SELF;
  if (bflags) atomicOr(s_flag, bflags);
  __syncthreads();
  const int f = *s_flag;

  // write back (round 0 always: the marker itself is new) and flag the neighbours
  T *rec = static_cast<T *>(im.rec);
  if (round == 0 || f != 0) {
    for (int i = threadIdx.x; i < RT * RT; i += RTHREADS) {
      const int r = i / RT, c = i % RT;
      const int64_t gy = y0 + r, gx = x0 + c;
      if (gy < im.H && gx < im.W) st_cg(rec + gy * im.W + gx, s_out[(r + 1) * PO + (c + 1)]);
    }
  }
  if (threadIdx.x == 0 && f != 0) {
    unsigned *fnext = P.flags + (size_t)((round + 1) & 1) * P.ntiles;
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
    if (f & (B_N | B_S | B_W | B_E | B_SELF)) atomicExch(&P.ctl->any[(round + 1) % 3], 1u);
  }
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

  // epilogue over every pixel of every image
  const int64_t stride = (int64_t)gridDim.x * RTHREADS;
  for (int k = 0; k < P.nimg; ++k) {
    const RImg &im = (P.nimg == 1) ? P.single : P.imgs[k];
    const int64_t n = im.H * im.W;
    const T *rec = static_cast<const T *>(im.rec);
    const T *ref = static_cast<const T *>(im.mask);
    if (P.epi == EPI_BINARY_SUP) {
      uint8_t *o = static_cast<uint8_t *>(im.out);
      for (int64_t i = (int64_t)blockIdx.x * RTHREADS + threadIdx.x; i < n; i += stride)
        o[i] = (ldg(ref + i) > ld_cg(rec + i)) ? 255 : 0;
    } else {  // EPI_CLIP_REF: low leveling min(rec, ref), high leveling max(rec, ref)
      T *o = static_cast<T *>(im.out);
      for (int64_t i = (int64_t)blockIdx.x * RTHREADS + threadIdx.x; i < n; i += stride)
        o[i] = Op<T, !SUP>::apply(ld_cg(rec + i), ldg(ref + i));
    }
  }
}

// ------------------------------------------------------------------ host side
template <typename T, bool SUP, bool CONN8>
static pg_status run_t(std::vector<RImg> &imgs, const ReconRequest &rq, bool binary, cudaStream_t s) {
  constexpr int RT = tile_side<T>(), RTHREADS = RT;
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

  auto kern = k_reconstruct<T, SUP, CONN8>;
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
// The autotuner times the candidate configurations -- tile side (64 or 32 pixels, i.e. 64 or
// 32 threads per tile) x sweep sets per tile visit before the tile yields to the next global
// round (4, 16, unbounded) -- on the plan's own batch and keeps the fastest; the choice is
// cached per (pixel type, connectivity, batch size class).
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
  auto kern = k_reconstruct<T, true, CONN8, RT>;
  int per_sm = 0;
  PG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, RT, 0), "occupancy");
  if (per_sm < 1) return fail(PG_ERR_CUDA, "reconstruction kernel cannot be resident");
  int grid = per_sm * num_sms();
  if (grid > tb.ntiles) grid = tb.ntiles;
  if (grid_out) *grid_out = grid;
  PG_CUDA_TRY(cudaMemsetAsync(p.scratch, 0, p.clear_bytes, s), "clear batch worklist");
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(RT);
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
    plan->cfg = PlanCfg{es == 8 ? 32 : 64, kMaxSweeps};
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

pg_status pg_batch_plan_config(const pg_batch_plan *plan, int32_t *tile, int32_t *sweeps, int32_t *grid) {
  if (!plan) return pg::fail(PG_ERR_INVALID_ARGUMENT, "null plan");
  if (tile) *tile = plan->cfg.rt;
  if (sweeps) *sweeps = plan->cfg.sweeps;
  if (grid) *grid = plan->grid;
  return PG_OK;
}

}  // extern "C"
