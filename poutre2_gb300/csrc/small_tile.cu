// small_tile.cu -- erosion / dilation of u8 / u16 / i32 / f32 images and volumes by the 3x3 square,
// the 3x3 cross, the 3x3x3 cube, the 3D cross and the 3-pixel X / Y segments through shared-memory
// tiles loaded by TMA (rows of a multiple of 16 bytes).
//
// Same result as k_small2d / k_small3d (small_se.cu) and the reference's static-SE dispatchers
// (ero_dil_static_se_t.hpp:298-915): per pixel the min / max over the SE's offsets inside the image.
//
// A CTA owns an output tile of 64 32-bit words (4 / sizeof(T) pixels each) by 64 rows (a volume's: by
// 8 rows by 8 slices).  One TMA copy brings the box around it -- a 16-byte chunk of halo left
// and right, a row above and below, a slice before and after -- into shared memory, so all of the
// tile's loads are in flight at once; the grids of the usual image sizes fit in one wave of resident
// CTAs.  A thread owns one word column (or, for u8 images, a 16-byte quad of words) over a run of the
// tile's rows (of every slice of the tile): the left and right neighbours of each pixel come from
// funnel shifts with the neighbouring words, the rows above and below are the next shared-memory
// rows, and a volume's slices slide through registers.  u16 words are min / max'ed as u16x2; u8 words
// are split once into their even and odd pixels on 16-bit lanes (the native u16x2 min / max; the
// packed 8-bit form is emulated), combined there and merged once; i32 / f32 words hold one pixel.
// Pixels outside the image arrive as TMA's zero fill, the neutral value of the unsigned dilations;
// for the other operators, tiles at the border set them to the neutral value first.  The TMA wait is
// bounded (tile::kWaitNs); on expiry the CTA records PG_ERR_CUDA in g_small_tile_status (read by
// pg_check_device) and leaves its tile unwritten.
#include "tile.cuh"

namespace pg {

__device__ int g_small_tile_status = 0;

namespace {

using namespace tile;
constexpr int kSTThreads = 256;
constexpr int kSTW = 64;         // output words per tile row
constexpr int kSTBW = kSTW + 8;  // box words: one 16-byte chunk of halo each side
constexpr int kST2Rows = 64;     // output rows of a 2D tile (a thread per word)
constexpr int kST2QRows = 64;    // output rows of a 2D tile (a thread per quad of words)
// u8 images take the quad kernel (4096^2 square 12.3 -> 10.2 us); for u16 / i32 / f32 the thread per
// word measured 1-2 % faster on 8192^2 / 16384^2 images and the same on 4096^2
template <typename T> constexpr bool kQuad2D = sizeof(T) == 1;
constexpr int kST2QThreads = 128;  // threads of a quad tile
constexpr int kST3Rows = 8;        // output rows of a 3D tile
constexpr int kST3Slices = 8;      // output slices of a 3D tile
constexpr int kST3Threads = 128;   // threads of a 3D tile
enum { ST_SQUARE = 0, ST_CROSS = 1, ST_SEGX = 2, ST_SEGY = 3 };

template <bool SUP> __device__ __forceinline__ uint32_t m16(uint32_t a, uint32_t b) { return wop<uint16_t, SUP>(a, b); }

// the pixels of one word on 16-bit lanes: u16 as is; u8 as its even (p0, p2) and odd (p1, p3) pixels
template <typename T, bool SUP> struct Lanes;
template <bool SUP> struct Lanes<uint16_t, SUP> {
  uint32_t w;
  static __device__ __forceinline__ Lanes at(const uint32_t *p) { return {p[0]}; }
  // op over each pixel and its left and right neighbours
  static __device__ __forceinline__ Lanes hor(const uint32_t *p) {
    const uint32_t w = p[0];
    return {m16<SUP>(w, m16<SUP>(__funnelshift_l(p[-1], w, 16), __funnelshift_r(w, p[1], 16)))};
  }
  // the four words from p (16-byte aligned): plain, and op with the left and right neighbours
  static __device__ __forceinline__ void at4(const uint32_t *p, Lanes (&v)[4]) {
    const uint4 q = *reinterpret_cast<const uint4 *>(p);
    v[0] = {q.x}; v[1] = {q.y}; v[2] = {q.z}; v[3] = {q.w};
  }
  static __device__ __forceinline__ void hor4(const uint32_t *p, Lanes (&h)[4]) {
    const uint4 q = *reinterpret_cast<const uint4 *>(p);
    const uint32_t w[6] = {p[-1], q.x, q.y, q.z, q.w, p[4]};
#pragma unroll
    for (int k = 0; k < 4; ++k)
      h[k] = {m16<SUP>(w[k + 1],
                       m16<SUP>(__funnelshift_l(w[k], w[k + 1], 16), __funnelshift_r(w[k + 1], w[k + 2], 16)))};
  }
  __device__ __forceinline__ Lanes op(Lanes b) const { return {m16<SUP>(w, b.w)}; }
  __device__ __forceinline__ uint32_t word() const { return w; }
};
template <bool SUP> struct Lanes<uint8_t, SUP> {
  uint32_t e, o;
  static __device__ __forceinline__ Lanes at(const uint32_t *p) {
    const uint32_t w = p[0];
    return {__byte_perm(w, 0, 0x4240), __byte_perm(w, 0, 0x4341)};
  }
  // even pixel 2j: window (odd 2j - 1, 2j, odd 2j + 1); odd pixel 2j + 1: (even 2j, 2j + 1, even 2j + 2)
  static __device__ __forceinline__ Lanes hor(const uint32_t *p) {
    const uint32_t w = p[0];
    const uint32_t E = __byte_perm(w, 0, 0x4240), O = __byte_perm(w, 0, 0x4341);
    const uint32_t Op = __byte_perm(p[-1], 0, 0x4341), En = __byte_perm(p[1], 0, 0x4240);
    const uint32_t M = m16<SUP>(E, O);
    return {m16<SUP>(M, __funnelshift_l(Op, O, 16)), m16<SUP>(M, __funnelshift_r(E, En, 16))};
  }
  static __device__ __forceinline__ void at4(const uint32_t *p, Lanes (&v)[4]) {
    const uint4 q = *reinterpret_cast<const uint4 *>(p);
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = {__byte_perm(w[k], 0, 0x4240), __byte_perm(w[k], 0, 0x4341)};
  }
  // each word split once; the left word's odd and the right word's even pixels from the neighbours
  static __device__ __forceinline__ void hor4(const uint32_t *p, Lanes (&h)[4]) {
    const uint4 q = *reinterpret_cast<const uint4 *>(p);
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
    uint32_t E[6], O[6];  // index k + 1 = word k; O[0] of the left word, E[5] of the right one
    O[0] = __byte_perm(p[-1], 0, 0x4341);
    E[5] = __byte_perm(p[4], 0, 0x4240);
#pragma unroll
    for (int k = 0; k < 4; ++k) { E[k + 1] = __byte_perm(w[k], 0, 0x4240); O[k + 1] = __byte_perm(w[k], 0, 0x4341); }
#pragma unroll
    for (int k = 1; k <= 4; ++k) {
      const uint32_t M = m16<SUP>(E[k], O[k]);
      h[k - 1] = {m16<SUP>(M, __funnelshift_l(O[k - 1], O[k], 16)), m16<SUP>(M, __funnelshift_r(E[k], E[k + 1], 16))};
    }
  }
  __device__ __forceinline__ Lanes op(Lanes b) const { return {m16<SUP>(e, b.e), m16<SUP>(o, b.o)}; }
  __device__ __forceinline__ uint32_t word() const { return __byte_perm(e, o, 0x6240); }
};
// i32 / f32: one pixel per word, min / max as everywhere else (wop: signed compare, fminf / fmaxf)
template <typename T, bool SUP> struct Lanes {
  uint32_t w;
  static __device__ __forceinline__ Lanes at(const uint32_t *p) { return {p[0]}; }
  static __device__ __forceinline__ Lanes hor(const uint32_t *p) {
    return {wop<T, SUP>(p[0], wop<T, SUP>(p[-1], p[1]))};
  }
  static __device__ __forceinline__ void at4(const uint32_t *p, Lanes (&v)[4]) {
    const uint4 q = *reinterpret_cast<const uint4 *>(p);
    v[0] = {q.x}; v[1] = {q.y}; v[2] = {q.z}; v[3] = {q.w};
  }
  static __device__ __forceinline__ void hor4(const uint32_t *p, Lanes (&h)[4]) {
    const uint4 q = *reinterpret_cast<const uint4 *>(p);
    const uint32_t w[6] = {p[-1], q.x, q.y, q.z, q.w, p[4]};
#pragma unroll
    for (int k = 0; k < 4; ++k) h[k] = {wop<T, SUP>(w[k + 1], wop<T, SUP>(w[k], w[k + 2]))};
  }
  __device__ __forceinline__ Lanes op(Lanes b) const { return {wop<T, SUP>(w, b.w)}; }
  __device__ __forceinline__ uint32_t word() const { return w; }
};

// The operator's neutral value in place of TMA's zero fill (which is the neutral value only of the
// unsigned dilations): box rows wholly outside the image (row_in(r) false), and the words left of box
// word c_lo / from box word c_hi of the others (c_lo, c_hi multiples of 4; box rows of 72 words start
// on 16-byte boundaries).
template <int NT, typename F>
__device__ __forceinline__ void fill_outside(uint32_t *box, int nrows, int c_lo, int c_hi, uint32_t neu, F row_in) {
  const uint4 ones = make_uint4(neu, neu, neu, neu);
  for (int r = threadIdx.x; r < nrows; r += NT) {
    uint4 *row = reinterpret_cast<uint4 *>(box + r * kSTBW);
    if (!row_in(r)) {
#pragma unroll
      for (int k = 0; k < kSTBW / 4; ++k) row[k] = ones;
    } else {
      for (int k = 0; k < c_lo / 4; ++k) row[k] = ones;
      for (int k = c_hi / 4; k < kSTBW / 4; ++k) row[k] = ones;
    }
  }
  __syncthreads();
}

template <typename T, bool SUP, int SHAPE>
__global__ void __launch_bounds__(kSTThreads) k_small2d_tile(const __grid_constant__ CUtensorMap tmap,
                                                            uint32_t *__restrict__ out, int H, int Wn) {
  using L = Lanes<T, SUP>;
  constexpr int TH = kST2Rows, BH = TH + 2, RPT = TH / (kSTThreads / kSTW);
  extern __shared__ __align__(128) uint32_t s_box[];  // [BH][kSTBW] + the mbarrier
  __shared__ int s_ok;
  uint64_t *bar = reinterpret_cast<uint64_t *>(s_box + BH * kSTBW);
  const int wx0 = (int)blockIdx.x * kSTW, y0 = (int)blockIdx.y * TH;
  const int tx = wx0 - 4, ty = y0 - 1;  // box origin: word (a multiple of 4: 16 bytes), row
  if (!load_tile(&tmap, s_box, bar, (unsigned)(BH * kSTBW * 4), tx, ty, &g_small_tile_status, &s_ok)) return;
  if constexpr (!(SUP && std::is_unsigned_v<T>)) {
    if (tx < 0 || tx + kSTBW > Wn || ty < 0 || ty + BH > H)
      fill_outside<kSTThreads>(s_box, BH, max(0, -tx), min(kSTBW, Wn - tx), splat<T>(Op<T, SUP>::neutral()),
                               [&](int r) { return ty + r >= 0 && ty + r < H; });
  }

  const int c = threadIdx.x % kSTW, g = threadIdx.x / kSTW;
  const int gw = wx0 + c;
  if (gw >= Wn) return;
  const int r0 = g * RPT;  // output rows r0 .. r0 + RPT - 1 of the tile = box rows r0 + 1 .. r0 + RPT
  const int nrows = min(RPT, H - (y0 + r0));
  if (nrows <= 0) return;
  const uint32_t *col = s_box + 4 + c + r0 * kSTBW;  // box row r0, the word of output column c
  uint32_t *dst = out + (size_t)(y0 + r0) * Wn + gw;
  L a, b;  // the two rows above the current output row (horizontal results, or plain words)
  if constexpr (SHAPE == ST_SQUARE) { a = L::hor(col); b = L::hor(col + kSTBW); }
  else if constexpr (SHAPE == ST_CROSS || SHAPE == ST_SEGY) { a = L::at(col); b = L::at(col + kSTBW); }
#pragma unroll 4
  for (int i = 0; i < RPT; ++i) {
    const uint32_t *p = col + (i + 2) * kSTBW;  // the row below output row i
    L res;
    if constexpr (SHAPE == ST_SQUARE) {
      const L n = L::hor(p);
      res = b.op(a).op(n);
      a = b; b = n;
    } else if constexpr (SHAPE == ST_CROSS) {
      const L n = L::at(p);
      res = L::hor(p - kSTBW).op(a).op(n);
      a = b; b = n;
    } else if constexpr (SHAPE == ST_SEGY) {
      const L n = L::at(p);
      res = b.op(a).op(n);
      a = b; b = n;
    } else {
      res = L::hor(p - kSTBW);
    }
    if (i < nrows) dst[(size_t)i * Wn] = res.word();
  }
}

// The same tile of 64 words by kST2QRows rows with a thread per 16-byte quad of words and
// kST2QRows / 8 rows: each box row is read as one 16-byte load plus the two neighbouring words, each
// u8 word split once (not three times, as the centre and as each neighbour's neighbour), and the
// results stored 16 bytes at a time.
template <typename T, bool SUP, int SHAPE>
__global__ void __launch_bounds__(kST2QThreads) k_small2d_quad(const __grid_constant__ CUtensorMap tmap,
                                                            uint32_t *__restrict__ out, int H, int Wn) {
  using L = Lanes<T, SUP>;
  constexpr int TH = kST2QRows, BH = TH + 2, QC = kSTW / 4, RPT = TH / (kST2QThreads / QC);
  extern __shared__ __align__(128) uint32_t s_box[];  // [BH][kSTBW] + the mbarrier
  __shared__ int s_ok;
  uint64_t *bar = reinterpret_cast<uint64_t *>(s_box + BH * kSTBW);
  const int wx0 = (int)blockIdx.x * kSTW, y0 = (int)blockIdx.y * TH;
  const int tx = wx0 - 4, ty = y0 - 1;
  if (!load_tile(&tmap, s_box, bar, (unsigned)(BH * kSTBW * 4), tx, ty, &g_small_tile_status, &s_ok)) return;
  if constexpr (!(SUP && std::is_unsigned_v<T>)) {
    if (tx < 0 || tx + kSTBW > Wn || ty < 0 || ty + BH > H)
      fill_outside<kST2QThreads>(s_box, BH, max(0, -tx), min(kSTBW, Wn - tx), splat<T>(Op<T, SUP>::neutral()),
                                 [&](int r) { return ty + r >= 0 && ty + r < H; });
  }

  const int q = threadIdx.x % QC, g = threadIdx.x / QC;
  const int gw = wx0 + 4 * q;  // first word of the quad (Wn is a multiple of 4: quads are whole)
  if (gw >= Wn) return;
  const int r0 = g * RPT;
  const int nrows = min(RPT, H - (y0 + r0));
  if (nrows <= 0) return;
  const uint32_t *col = s_box + 4 + 4 * q + r0 * kSTBW;  // box row r0, the quad's first word
  uint4 *dst = reinterpret_cast<uint4 *>(out + (size_t)(y0 + r0) * Wn + gw);
  const size_t pitch = (size_t)Wn / 4;
  L a[4], b[4];
  if constexpr (SHAPE == ST_SQUARE) { L::hor4(col, a); L::hor4(col + kSTBW, b); }
  else if constexpr (SHAPE == ST_CROSS || SHAPE == ST_SEGY) { L::at4(col, a); L::at4(col + kSTBW, b); }
#pragma unroll
  for (int i = 0; i < RPT; ++i) {
    const uint32_t *p = col + (i + 2) * kSTBW;
    L res[4], n[4];
    if constexpr (SHAPE == ST_SQUARE) {
      L::hor4(p, n);
#pragma unroll
      for (int k = 0; k < 4; ++k) res[k] = b[k].op(a[k]).op(n[k]);
    } else if constexpr (SHAPE == ST_CROSS) {
      L::at4(p, n);
      L h[4];
      L::hor4(p - kSTBW, h);
#pragma unroll
      for (int k = 0; k < 4; ++k) res[k] = h[k].op(a[k]).op(n[k]);
    } else if constexpr (SHAPE == ST_SEGY) {
      L::at4(p, n);
#pragma unroll
      for (int k = 0; k < 4; ++k) res[k] = b[k].op(a[k]).op(n[k]);
    } else {
      L::hor4(p - kSTBW, res);
    }
    if constexpr (SHAPE != ST_SEGX) {
#pragma unroll
      for (int k = 0; k < 4; ++k) { a[k] = b[k]; b[k] = n[k]; }
    }
    if (i < nrows) dst[i * pitch] = make_uint4(res[0].word(), res[1].word(), res[2].word(), res[3].word());
  }
}

// Volumes: per box slice s and output row j of the thread, A(s) = the slice's own part of the SE and
// B(s) = what the slices before and after contribute; out(z) = op(B(z - 1), A(z), B(z + 1)) (B is
// unused for the X and Y segments).
template <typename T, bool SUP, int SHAPE>
__global__ void __launch_bounds__(kST3Threads) k_small3d_tile(const __grid_constant__ CUtensorMap tmap,
                                                            uint32_t *__restrict__ out, int D, int H, int Wn) {
  using L = Lanes<T, SUP>;
  constexpr int BY = kST3Rows, BZ = kST3Slices, RY = BY + 2, RZ = BZ + 2, PL = RY * kSTBW;
  constexpr int NR = BY / (kST3Threads / kSTW);  // output rows per thread
  constexpr bool USE_B = SHAPE == ST_SQUARE || SHAPE == ST_CROSS;
  extern __shared__ __align__(128) uint32_t s_box[];  // [RZ][RY][kSTBW] + the mbarrier
  __shared__ int s_ok;
  uint64_t *bar = reinterpret_cast<uint64_t *>(s_box + RZ * PL);
  const int wx0 = (int)blockIdx.x * kSTW, y0 = (int)blockIdx.y * BY, z0 = (int)blockIdx.z * BZ;
  const int tx = wx0 - 4, ty = y0 - 1, tz = z0 - 1;
  if (!load_box<3>(&tmap, s_box, bar, (unsigned)(RZ * PL * 4), tx, ty, tz, &g_small_tile_status, &s_ok)) return;
  if constexpr (!(SUP && std::is_unsigned_v<T>)) {
    if (tx < 0 || tx + kSTBW > Wn || ty < 0 || ty + RY > H || tz < 0 || tz + RZ > D)
      fill_outside<kST3Threads>(s_box, RZ * RY, max(0, -tx), min(kSTBW, Wn - tx), splat<T>(Op<T, SUP>::neutral()),
                                [&](int r) {
                                  const int s = r / RY, gz = tz + s, gy = ty + (r - s * RY);
                                  return gz >= 0 && gz < D && gy >= 0 && gy < H;
                                });
  }

  const int c = threadIdx.x % kSTW, g = threadIdx.x / kSTW;
  const int gw = wx0 + c;
  if (gw >= Wn) return;
  const int yr0 = g * NR;  // output rows yr0 .. yr0 + NR - 1 of the tile = box rows yr0 + 1 .. yr0 + NR
  const int ny = min(NR, H - (y0 + yr0)), nz = min(BZ, D - z0);
  if (ny <= 0) return;
  const uint32_t *col = s_box + 4 + c + yr0 * kSTBW;  // box slice 0, box row yr0, word of column c
  auto slice = [&](int s, L (&A)[NR], L (&B)[NR]) {
    const uint32_t *p = col + s * PL;
    if constexpr (SHAPE == ST_SQUARE) {
      L h[NR + 2];
#pragma unroll
      for (int i = 0; i < NR + 2; ++i) h[i] = L::hor(p + i * kSTBW);
#pragma unroll
      for (int j = 0; j < NR; ++j) { A[j] = h[j + 1].op(h[j]).op(h[j + 2]); B[j] = A[j]; }
    } else if constexpr (SHAPE == ST_CROSS) {
      L v[NR + 2];
#pragma unroll
      for (int i = 0; i < NR + 2; ++i) v[i] = L::at(p + i * kSTBW);
#pragma unroll
      for (int j = 0; j < NR; ++j) { A[j] = L::hor(p + (j + 1) * kSTBW).op(v[j]).op(v[j + 2]); B[j] = v[j + 1]; }
    } else if constexpr (SHAPE == ST_SEGX) {
#pragma unroll
      for (int j = 0; j < NR; ++j) A[j] = L::hor(p + (j + 1) * kSTBW);
    } else {
      L v[NR + 2];
#pragma unroll
      for (int i = 0; i < NR + 2; ++i) v[i] = L::at(p + i * kSTBW);
#pragma unroll
      for (int j = 0; j < NR; ++j) A[j] = v[j + 1].op(v[j]).op(v[j + 2]);
    }
  };
  L Ap[NR], Bp[NR], Ac[NR], Bc[NR];
  if constexpr (USE_B) slice(0, Ap, Bp);
  slice(1, Ac, Bc);
  uint32_t *dst = out + ((size_t)z0 * H + (y0 + yr0)) * Wn + gw;
#pragma unroll
  for (int z = 0; z < BZ; ++z) {
    L An[NR], Bn[NR];
    if (USE_B || z + 1 < BZ) slice(z + 2, An, Bn);
    if (z < nz) {
#pragma unroll
      for (int j = 0; j < NR; ++j) {
        L r = Ac[j];
        if constexpr (USE_B) r = r.op(Bp[j]).op(Bn[j]);
        if (j < ny) dst[((size_t)z * H + j) * Wn] = r.word();
      }
    }
#pragma unroll
    for (int j = 0; j < NR; ++j) { Bp[j] = Bc[j]; Ac[j] = An[j]; Bc[j] = Bn[j]; }
  }
}

template <typename T, bool SUP, int SHAPE>
pg_status small2d_tile_t(const pg_image &in, const pg_image &out, cudaStream_t s) {
  const Dims d = dims_of(in);
  const int64_t H = d.ny, Wn = d.nx * (int64_t)sizeof(T) / 4;
  CUtensorMap map;
  constexpr int TH = kQuad2D<T> ? kST2QRows : kST2Rows;
  PG_TRY(word_map(&map, in.data, H, Wn, kSTBW, TH + 2));
  constexpr size_t smem = (size_t)(TH + 2) * kSTBW * 4 + 16;
  static_assert(smem <= 48 * 1024, "above 48 KB the kernel needs the dynamic shared memory attribute");
  const dim3 grid((unsigned)ceil_div(Wn, kSTW), (unsigned)ceil_div(H, TH));
  uint32_t *dst = static_cast<uint32_t *>(out.data);
  if constexpr (kQuad2D<T>) k_small2d_quad<T, SUP, SHAPE><<<grid, kST2QThreads, smem, s>>>(map, dst, (int)H, (int)Wn);
  else k_small2d_tile<T, SUP, SHAPE><<<grid, kSTThreads, smem, s>>>(map, dst, (int)H, (int)Wn);
  return cuda_status(cudaGetLastError(), "small-SE tile launch");
}

template <typename T, bool SUP, int SHAPE>
pg_status small3d_tile_t(const pg_image &in, const pg_image &out, cudaStream_t s) {
  const Dims d = dims_of(in);
  const int64_t D = d.nz, H = d.ny, Wn = d.nx * (int64_t)sizeof(T) / 4;
  CUtensorMap map;
  PG_TRY(word_map3(&map, in.data, D, H, Wn, kSTBW, kST3Rows + 2, kST3Slices + 2));
  constexpr size_t smem = (size_t)(kST3Slices + 2) * (kST3Rows + 2) * kSTBW * 4 + 16;
  static_assert(smem <= 48 * 1024, "above 48 KB the kernel needs the dynamic shared memory attribute");
  const dim3 grid((unsigned)ceil_div(Wn, kSTW), (unsigned)ceil_div(H, kST3Rows), (unsigned)ceil_div(D, kST3Slices));
  k_small3d_tile<T, SUP, SHAPE><<<grid, kST3Threads, smem, s>>>(map, static_cast<uint32_t *>(out.data), (int)D, (int)H,
                                                              (int)Wn);
  return cuda_status(cudaGetLastError(), "small-SE volume tile launch");
}

template <typename T, bool SUP>
pg_status small_tile_se(const pg_image &in, const pg_image &out, int se, cudaStream_t s) {
  switch (se) {
    case PG_SE_SQUARE_2D: return small2d_tile_t<T, SUP, ST_SQUARE>(in, out, s);
    case PG_SE_CROSS_2D: return small2d_tile_t<T, SUP, ST_CROSS>(in, out, s);
    case PG_SE_SEGMENT_X_2D: return small2d_tile_t<T, SUP, ST_SEGX>(in, out, s);
    case PG_SE_SEGMENT_Y_2D: return small2d_tile_t<T, SUP, ST_SEGY>(in, out, s);
    case PG_SE_SQUARE_3D: return small3d_tile_t<T, SUP, ST_SQUARE>(in, out, s);
    case PG_SE_CROSS_3D: return small3d_tile_t<T, SUP, ST_CROSS>(in, out, s);
    case PG_SE_SEGMENT_X_3D: return small3d_tile_t<T, SUP, ST_SEGX>(in, out, s);
    default: return small3d_tile_t<T, SUP, ST_SEGY>(in, out, s);  // PG_SE_SEGMENT_Y_3D
  }
}

}  // namespace

bool try_small_tile(const pg_image &in, const pg_image &out, int se, bool dilate, cudaStream_t s, pg_status *st) {
  const bool two = se == PG_SE_SQUARE_2D || se == PG_SE_CROSS_2D || se == PG_SE_SEGMENT_X_2D ||
                   se == PG_SE_SEGMENT_Y_2D;
  // the Z segment stays on k_small3d (one slice window per word, no row or column halo): faster there
  const bool three = se == PG_SE_SQUARE_3D || se == PG_SE_CROSS_3D || se == PG_SE_SEGMENT_X_3D ||
                     se == PG_SE_SEGMENT_Y_3D;
  if (!((two && in.rank == 2) || (three && in.rank == 3))) return false;
  if (!(in.ptype == PG_PTYPE_U8 || in.ptype == PG_PTYPE_U16 || in.ptype == PG_PTYPE_I32 ||
        in.ptype == PG_PTYPE_F32))
    return false;
  const int es = elem_size(in.ptype);
  const Dims d = dims_of(in);
  if (d.count() == 0 || (d.nx * es) % 16 != 0) return false;
  if ((reinterpret_cast<uintptr_t>(in.data) | reinterpret_cast<uintptr_t>(out.data)) % 16 != 0) return false;
  // int indices inside the kernels; grid y / z within 65535
  if (d.nx * es / 4 > (1 << 30) || d.ny > (1 << 30) || d.nz > (1 << 30)) return false;
  if (two && ceil_div(d.ny, kST2Rows) > 65535) return false;
  if (three && (ceil_div(d.ny, kST3Rows) > 65535 || ceil_div(d.nz, kST3Slices) > 65535)) return false;
  auto run = [&](auto tag) {
    using T = decltype(tag);
    *st = dilate ? small_tile_se<T, true>(in, out, se, s) : small_tile_se<T, false>(in, out, se, s);
  };
  switch (in.ptype) {
    case PG_PTYPE_U8: run(uint8_t{}); break;
    case PG_PTYPE_U16: run(uint16_t{}); break;
    case PG_PTYPE_I32: run(int32_t{}); break;
    default: run(float{}); break;
  }
  return true;
}

int take_small_tile_status() {
  int st = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&st, g_small_tile_status, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  if (st != 0 && cudaMemcpyToSymbol(g_small_tile_status, &zero, sizeof(int)) != cudaSuccess) return (int)PG_ERR_CUDA;
  return st;
}

}  // namespace pg
