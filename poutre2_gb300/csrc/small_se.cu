// small_se.cu -- flat erosion/dilation by the predefined 3-tap / 3x3 / 3x3x3 structuring
// elements, and by an arbitrary neighbour list.
//
// Reference: llm::details::t_ErodeDilateDispatcher specialisations
// (low_level_morpho/details/ero_dil_static_se_t.hpp:298-915) and the runtime neighbour-list
// dispatcher (ero_dil_runtime_nl_se_t.hpp:54-193).  All compute, per output pixel, the
// min/max of the input over the SE's offsets that fall inside the image.
//
// GPU design: HBM-bound streaming.  A thread owns 16 contiguous bytes of a row (a Pack:
// 16 u8, 8 u16, 4 i32/f32, 2 i64/f64) and a strip of rows (2D) or slices (3D); it slides a
// three-row (three-slice) window down the strip, so every input byte is read from DRAM
// once and every output byte written once.  The horizontal 3-neighbourhood of a pack comes
// from its two edge neighbours (one scalar load each, L1 hits) and a funnel shift;
// u8/u16 use the SIMD-in-word min/max.
#include <algorithm>
#include <atomic>
#include <vector>

#include "common.cuh"
#include "words.cuh"

namespace pg {

enum { SH_SQUARE = 0, SH_CROSS = 1, SH_SEGX = 2, SH_SEGY = 3, SH_SEGZ = 4 };

template <typename T> struct Scalar {
  static constexpr int N = 1;
  T e0;
  __device__ __forceinline__ static Scalar load(const T *p) { Scalar r; r.e0 = ldg(p); return r; }
  __device__ __forceinline__ void store(T *p) const { *p = e0; }
  __device__ __forceinline__ static Scalar fill(T x) { Scalar r; r.e0 = x; return r; }
  template <bool SUP> __device__ __forceinline__ static Scalar op(const Scalar &a, const Scalar &b) {
    Scalar r; r.e0 = Op<T, SUP>::apply(a.e0, b.e0); return r;
  }
  __device__ __forceinline__ Scalar shl(T left) const { Scalar r; r.e0 = left; return r; }
  __device__ __forceinline__ Scalar shr(T right) const { Scalar r; r.e0 = right; return r; }
};

// 16 u8 pixels held as eight words: for each 32-bit word of the pack its even bytes (bits 0-7,
// 16-23) and its odd bytes (bits 8-15, 24-31) with the other bytes zeroed.  max/min of u8 pairs
// is then the native 2x16-bit max/min (the odd bytes compare as x << 8), two instructions per
// word, where a packed 4x8-bit max/min is emulated by a much longer sequence.
struct PackU8S {
  static constexpr int N = 16;
  static constexpr uint32_t ME = 0x00ff00ffu, MO = 0xff00ff00u;
  uint32_t e[4], o[4];
  __device__ __forceinline__ void split(const uint32_t (&w)[4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) { e[i] = w[i] & ME; o[i] = w[i] & MO; }
  }
  __device__ __forceinline__ static PackU8S load(const uint8_t *p) {
    const uint4 v = __ldg(reinterpret_cast<const uint4 *>(p));
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
    PackU8S r;
    r.split(w);
    return r;
  }
  __device__ __forceinline__ void store(uint8_t *p) const {
    *reinterpret_cast<uint4 *>(p) = make_uint4(e[0] | o[0], e[1] | o[1], e[2] | o[2], e[3] | o[3]);
  }
  __device__ __forceinline__ static PackU8S fill(uint8_t x) {
    const uint32_t s = (uint32_t)x * 0x01010101u;
    PackU8S r;
#pragma unroll
    for (int i = 0; i < 4; ++i) { r.e[i] = s & ME; r.o[i] = s & MO; }
    return r;
  }
  template <bool SUP> __device__ __forceinline__ static PackU8S op(const PackU8S &a, const PackU8S &b) {
    PackU8S r;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      r.e[i] = wop<uint16_t, SUP>(a.e[i], b.e[i]);
      r.o[i] = wop<uint16_t, SUP>(a.o[i], b.o[i]);
    }
    return r;
  }
  __device__ __forceinline__ PackU8S shl(uint8_t left) const {
    uint32_t w[4];
    uint32_t prev = (uint32_t)left << 24;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const uint32_t x = e[i] | o[i];
      w[i] = __funnelshift_l(prev, x, 8);
      prev = x;
    }
    PackU8S r;
    r.split(w);
    return r;
  }
  __device__ __forceinline__ PackU8S shr(uint8_t right) const {
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const uint32_t x = e[i] | o[i];
      const uint32_t next = (i < 3) ? (e[i + 1] | o[i + 1]) : (uint32_t)right;
      w[i] = __funnelshift_r(x, next, 8);
    }
    PackU8S r;
    r.split(w);
    return r;
  }
};

// the pack type of a pixel type: split words for u8, plain 16-byte packs otherwise
template <typename T> struct PackOf { using type = Pack<T>; };
template <> struct PackOf<uint8_t> { using type = PackU8S; };

// centre pack and its horizontal 3-neighbourhood of one row (neutral outside the image)
template <typename T, bool SUP, typename P>
__device__ __forceinline__ void load_row(const T *__restrict__ row, bool valid, int64_t x0, int64_t W, bool need_h,
                                         P &c, P &h) {
  const T NEU = Op<T, SUP>::neutral();
  if (!valid) { c = P::fill(NEU); h = c; return; }
  c = P::load(row + x0);
  if (!need_h) { h = c; return; }
  const T left = (x0 > 0) ? ldg(row + x0 - 1) : NEU;
  const T right = (x0 + P::N < W) ? ldg(row + x0 + P::N) : NEU;
  h = P::template op<SUP>(P::template op<SUP>(c, c.shl(left)), c.shr(right));
}

// 2D: SESquare2D / SECross2D / SESegmentX2D / SESegmentY2D (and SESegmentX1D as H == 1).
template <typename T, bool SUP, int SHAPE, typename P>
__global__ void __launch_bounds__(256) k_small2d(const T *__restrict__ in, T *__restrict__ out, int64_t H, int64_t W,
                                                 int64_t npack, int R) {
  const int64_t xp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t y0 = ((int64_t)blockIdx.y * blockDim.y + threadIdx.y) * R;
  if (xp >= npack || y0 >= H) return;
  const int64_t x0 = xp * P::N;
  const int64_t y1 = (y0 + R < H) ? y0 + R : H;
  constexpr bool NEED_H = (SHAPE != SH_SEGY);
  P cp, hp, cc, hc, cn, hn;
  load_row<T, SUP>(in + (y0 - 1) * W, y0 >= 1, x0, W, NEED_H, cp, hp);
  load_row<T, SUP>(in + y0 * W, true, x0, W, NEED_H, cc, hc);
  for (int64_t y = y0; y < y1; ++y) {
    load_row<T, SUP>(in + (y + 1) * W, y + 1 < H, x0, W, NEED_H, cn, hn);
    P r;
    if constexpr (SHAPE == SH_SQUARE) r = P::template op<SUP>(P::template op<SUP>(hp, hc), hn);
    else if constexpr (SHAPE == SH_CROSS) r = P::template op<SUP>(P::template op<SUP>(cp, hc), cn);
    else if constexpr (SHAPE == SH_SEGX) r = hc;
    else r = P::template op<SUP>(P::template op<SUP>(cp, cc), cn);
    r.store(out + y * W + x0);
    cp = cc; hp = hc; cc = cn; hc = hn;
  }
}

// 3D: SESquare3D (26-conn.), SECross3D (6), SESegmentX3D/Y3D/Z3D.  out(z) = op(B(z-1), A(z), B(z+1))
// with A the in-slice part and B the part taken from the adjacent slices.
template <typename T, bool SUP, int SHAPE, typename P>
__global__ void __launch_bounds__(256) k_small3d(const T *__restrict__ in, T *__restrict__ out, int64_t D, int64_t H,
                                                 int64_t W, int64_t npack, int R) {
  const int64_t xp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t y = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  const int64_t z0 = (int64_t)blockIdx.z * R;
  if (xp >= npack || y >= H || z0 >= D) return;
  const int64_t x0 = xp * P::N;
  const int64_t z1 = (z0 + R < D) ? z0 + R : D;
  const T NEU = Op<T, SUP>::neutral();
  const int64_t plane = H * W;
  const bool has_up = y >= 1, has_dn = y + 1 < H;
  // row pointers of this thread's (y-1, y, y+1) rows in slice z, advanced by one plane per slice
  const T *row_m = in + y * W;
  auto slice = [&](int64_t z, P &A, P &B) {
    if (z < 0 || z >= D) { A = P::fill(NEU); B = A; return; }
    const T *rm = row_m + z * plane;
    if constexpr (SHAPE == SH_SQUARE) {
      // separable: the column max of the three rows first (and of their edge neighbours), then
      // one horizontal 3-neighbourhood instead of three
      const T *ru = rm - W, *rd = rm + W;
      const P cu = has_up ? P::load(ru + x0) : P::fill(NEU);
      const P cm = P::load(rm + x0);
      const P cd = has_dn ? P::load(rd + x0) : P::fill(NEU);
      T left = NEU, right = NEU;
      if (x0 > 0) {
        left = ldg(rm + x0 - 1);
        if (has_up) left = Op<T, SUP>::apply(left, ldg(ru + x0 - 1));
        if (has_dn) left = Op<T, SUP>::apply(left, ldg(rd + x0 - 1));
      }
      if (x0 + P::N < W) {
        right = ldg(rm + x0 + P::N);
        if (has_up) right = Op<T, SUP>::apply(right, ldg(ru + x0 + P::N));
        if (has_dn) right = Op<T, SUP>::apply(right, ldg(rd + x0 + P::N));
      }
      const P v = P::template op<SUP>(P::template op<SUP>(cu, cm), cd);
      A = P::template op<SUP>(P::template op<SUP>(v, v.shl(left)), v.shr(right));
      B = A;
      return;
    }
    P cu, hu, cm, hm, cd, hd;
    const bool need_rows = (SHAPE == SH_CROSS || SHAPE == SH_SEGY);
    const bool need_h = (SHAPE != SH_SEGY && SHAPE != SH_SEGZ);
    load_row<T, SUP>(rm, true, x0, W, need_h, cm, hm);
    if (need_rows) {
      load_row<T, SUP>(rm - W, has_up, x0, W, false, cu, hu);
      load_row<T, SUP>(rm + W, has_dn, x0, W, false, cd, hd);
    }
    if constexpr (SHAPE == SH_SQUARE) { A = P::fill(NEU); B = A; }
    else if constexpr (SHAPE == SH_CROSS) { A = P::template op<SUP>(P::template op<SUP>(cu, hm), cd); B = cm; }
    else if constexpr (SHAPE == SH_SEGX) { A = hm; B = P::fill(NEU); }
    else if constexpr (SHAPE == SH_SEGY) { A = P::template op<SUP>(P::template op<SUP>(cu, cm), cd); B = P::fill(NEU); }
    else { A = cm; B = cm; }
  };
  P Ap, Bp, Ac, Bc, An, Bn;
  slice(z0 - 1, Ap, Bp);
  slice(z0, Ac, Bc);
  for (int64_t z = z0; z < z1; ++z) {
    slice(z + 1, An, Bn);
    P r = P::template op<SUP>(P::template op<SUP>(Bp, Ac), Bn);
    r.store(out + (z * H + y) * W + x0);
    Ap = Ac; Bp = Bc; Ac = An; Bc = Bn;
  }
}

// Arbitrary neighbour list, gather form with border clipping.
template <typename T, bool SUP>
__global__ void __launch_bounds__(256) k_nl(const T *__restrict__ in, T *__restrict__ out, int64_t D, int64_t H,
                                            int64_t W, const int4 *__restrict__ offs, int n) {
  const int64_t total = D * H * W;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = i % W, y = (i / W) % H, z = i / (W * H);
    T v = Op<T, SUP>::neutral();
    for (int k = 0; k < n; ++k) {
      const int4 o = __ldg(offs + k);
      const int64_t zz = z + o.x, yy = y + o.y, xx = x + o.z;
      if (zz < 0 || yy < 0 || xx < 0 || zz >= D || yy >= H || xx >= W) continue;
      v = Op<T, SUP>::apply(v, ldg(in + (zz * H + yy) * W + xx));
    }
    out[i] = v;
  }
}

// ------------------------------------------------------------------ launchers
static int rows_per_thread(int64_t threads_without_strips, int64_t length, int cap) {
  const int64_t target = (int64_t)num_sms() * 1024;
  int64_t r = threads_without_strips * length / (target > 0 ? target : 1);
  if (r < 1) r = 1;
  if (r > cap) r = cap;
  if (r > length) r = length;
  return (int)r;
}

// CTAs of 256 threads of kernel KERN that fit on the GPU at once (cached per kernel)
template <auto KERN> static int64_t resident_ctas() {
  static std::atomic<int> cached{0};
  int v = cached.load();
  if (v == 0) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, KERN, 256, 0) != cudaSuccess || per_sm < 1) {
      (void)cudaGetLastError();
      per_sm = 1;
    }
    v = per_sm * num_sms();
    cached.store(v);
  }
  return v;
}

// Rows (slices) per thread: the fewest that keep the grid within one wave of resident CTAs, so that
// no short second wave runs alone (4096^2 u8: 688 CTAs on 608 slots before, 1.13 waves); images too
// large for that at `cap` rows per thread run several full waves at the heuristic's length.
template <typename F> static int strip_rows(int64_t length, int cap, int64_t slots, int heuristic, F ctas_for) {
  int lo = 1, hi = (int)std::min<int64_t>(cap, std::max<int64_t>(length, 1));
  if (ctas_for(hi) > slots) return heuristic;
  while (lo < hi) {
    const int mid = (lo + hi) / 2;
    if (ctas_for(mid) <= slots) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

template <typename T, bool SUP, int SHAPE>
static pg_status small2d_t(const T *in, T *out, int64_t H, int64_t W, cudaStream_t s) {
  const bool aligned = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) % 16 == 0);
  const bool vec = aligned && (W % Pack<T>::N == 0);
  const int64_t npack = vec ? W / Pack<T>::N : W;
  const int bx = npack >= 32 ? 32 : npack >= 16 ? 16 : npack >= 8 ? 8 : npack >= 4 ? 4 : npack >= 2 ? 2 : 1;
  const int64_t gx = ceil_div(npack, bx);
  const int64_t slots = vec ? resident_ctas<k_small2d<T, SUP, SHAPE, typename PackOf<T>::type>>()
                            : resident_ctas<k_small2d<T, SUP, SHAPE, Scalar<T>>>();
  const int R = strip_rows(H, 32, slots, rows_per_thread(npack, H, 32),
                           [&](int r) { return gx * ceil_div(ceil_div(H, r), 256 / bx); });
  dim3 block(bx, 256 / bx);
  dim3 grid((unsigned)gx, (unsigned)ceil_div(ceil_div(H, R), 256 / bx));
  if (grid.y > 65535) return fail(PG_ERR_INVALID_ARGUMENT, "image too tall for the small-SE kernel");
  if (vec) k_small2d<T, SUP, SHAPE, typename PackOf<T>::type><<<grid, block, 0, s>>>(in, out, H, W, npack, R);
  else k_small2d<T, SUP, SHAPE, Scalar<T>><<<grid, block, 0, s>>>(in, out, H, W, npack, R);
  return cuda_status(cudaGetLastError(), "small-SE 2D kernel launch");
}

template <typename T, bool SUP, int SHAPE>
static pg_status small3d_t(const T *in, T *out, int64_t D, int64_t H, int64_t W, cudaStream_t s) {
  const bool aligned = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) % 16 == 0);
  const bool vec = aligned && (W % Pack<T>::N == 0);
  const int64_t npack = vec ? W / Pack<T>::N : W;
  // no idle lanes when a row holds fewer than 32 packs
  const int bx = npack >= 32 ? 32 : npack >= 16 ? 16 : npack >= 8 ? 8 : npack >= 4 ? 4 : npack >= 2 ? 2 : 1;
  const int64_t gxy = ceil_div(npack, bx) * ceil_div(H, 256 / bx);
  const int64_t slots = vec ? resident_ctas<k_small3d<T, SUP, SHAPE, typename PackOf<T>::type>>()
                            : resident_ctas<k_small3d<T, SUP, SHAPE, Scalar<T>>>();
  const int R = strip_rows(D, 16, slots, rows_per_thread(npack * H, D, 16), [&](int r) { return gxy * ceil_div(D, r); });
  dim3 block(bx, 256 / bx);
  dim3 grid((unsigned)ceil_div(npack, bx), (unsigned)ceil_div(H, 256 / bx), (unsigned)ceil_div(D, R));
  if (grid.y > 65535 || grid.z > 65535) return fail(PG_ERR_INVALID_ARGUMENT, "volume too large for the small-SE kernel");
  if (vec) k_small3d<T, SUP, SHAPE, typename PackOf<T>::type><<<grid, block, 0, s>>>(in, out, D, H, W, npack, R);
  else k_small3d<T, SUP, SHAPE, Scalar<T>><<<grid, block, 0, s>>>(in, out, D, H, W, npack, R);
  return cuda_status(cudaGetLastError(), "small-SE 3D kernel launch");
}

template <typename T, bool SUP>
static pg_status small_dispatch(const pg_image &in, const pg_image &out, int se, cudaStream_t s) {
  const Dims d = dims_of(in);
  const T *src = static_cast<const T *>(in.data);
  T *dst = static_cast<T *>(out.data);
  if (d.count() == 0) return PG_OK;
  switch (se) {
    case PG_SE_SEGMENT_X_1D: return small2d_t<T, SUP, SH_SEGX>(src, dst, 1, d.nx, s);
    case PG_SE_SQUARE_2D: return small2d_t<T, SUP, SH_SQUARE>(src, dst, d.ny, d.nx, s);
    case PG_SE_CROSS_2D: return small2d_t<T, SUP, SH_CROSS>(src, dst, d.ny, d.nx, s);
    case PG_SE_SEGMENT_X_2D: return small2d_t<T, SUP, SH_SEGX>(src, dst, d.ny, d.nx, s);
    case PG_SE_SEGMENT_Y_2D: return small2d_t<T, SUP, SH_SEGY>(src, dst, d.ny, d.nx, s);
    case PG_SE_SQUARE_3D: return small3d_t<T, SUP, SH_SQUARE>(src, dst, d.nz, d.ny, d.nx, s);
    case PG_SE_CROSS_3D: return small3d_t<T, SUP, SH_CROSS>(src, dst, d.nz, d.ny, d.nx, s);
    case PG_SE_SEGMENT_X_3D: return small3d_t<T, SUP, SH_SEGX>(src, dst, d.nz, d.ny, d.nx, s);
    case PG_SE_SEGMENT_Y_3D: return small3d_t<T, SUP, SH_SEGY>(src, dst, d.nz, d.ny, d.nx, s);
    case PG_SE_SEGMENT_Z_3D: return small3d_t<T, SUP, SH_SEGZ>(src, dst, d.nz, d.ny, d.nx, s);
    default: return fail(PG_ERR_UNSUPPORTED_SE, "unsupported nl_static");
  }
}

pg_status launch_small_se(const pg_image &in, const pg_image &out, int se, bool dilate, cudaStream_t s) {
  if (dims_of(in).count() == 0) return PG_OK;  // nothing to compute (and no empty grid to launch)
  pg_status st;
  if (try_small_tile(in, out, se, dilate, s, &st)) return st;
  PG_DISPATCH_PTYPE(in.ptype, T, {
    return dilate ? small_dispatch<T, true>(in, out, se, s) : small_dispatch<T, false>(in, out, se, s);
  });
  return PG_OK;
}

pg_status launch_nl(const pg_image &in, const pg_image &out, const int32_t *offsets, int n, bool dilate,
                    cudaStream_t s) {
  const Dims d = dims_of(in);
  if (d.count() == 0) return PG_OK;
  // offsets -> (dz, dy, dx, 0) int4 in device memory.  The host copy is pageable: the
  // runtime stages it before cudaMemcpyAsync returns, so it may be released right away.
  Scratch dev;
  PG_TRY(dev.alloc(sizeof(int4) * (size_t)n, s));
  std::vector<int4> host((size_t)n);
  for (int k = 0; k < n; ++k) {
    int o[3] = {0, 0, 0};
    for (int r = 0; r < in.rank; ++r) o[3 - in.rank + r] = offsets[k * in.rank + r];
    host[(size_t)k] = make_int4(o[0], o[1], o[2], 0);
  }
  PG_CUDA_TRY(cudaMemcpyAsync(dev.ptr, host.data(), sizeof(int4) * (size_t)n, cudaMemcpyHostToDevice, s),
              "copy of the offsets");
  const int threads = 256;
  int64_t blocks = ceil_div(d.count(), threads);
  const int64_t cap = (int64_t)num_sms() * 16;
  if (blocks > cap) blocks = cap;
  PG_DISPATCH_PTYPE(in.ptype, T, {
    if (dilate) k_nl<T, true><<<(unsigned)blocks, threads, 0, s>>>(static_cast<const T *>(in.data), static_cast<T *>(out.data), d.nz, d.ny, d.nx, dev.as<int4>(), n);
    else k_nl<T, false><<<(unsigned)blocks, threads, 0, s>>>(static_cast<const T *>(in.data), static_cast<T *>(out.data), d.nz, d.ny, d.nx, dev.as<int4>(), n);
  });
  return cuda_status(cudaGetLastError(), "neighbour-list kernel launch");
}

}  // namespace pg
