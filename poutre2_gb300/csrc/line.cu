// line.cu -- flat erosion/dilation by a line segment of 2k+1 pixels along X, Y or a diagonal,
// and by a rectangle as the composition Y o X.
//
// Reference: llm::details::van_herck_1d (low_level_morpho/details/ero_dil_line_se_t.hpp:50-89)
// applied per row for X (t_ErodeDilateXOpLineDispatcher :143-190) and through a transpose
// for Y (t_DilateY/t_ErodeY :249-282).  The diagonal segment has no reference entry point
// (the reference expresses it as a runtime neighbour list, ero_dil_runtime_nl_se_t.hpp);
// its result is the same clipped window min/max.
//
// GPU design: one CTA owns a tile of outputs and stages the tile plus a k-pixel halo along
// the line direction in shared memory (neutral outside the image).  The van Herk/Gil-Werman
// recurrence runs there: every line of the staged region is cut into blocks of w = 2k+1
// positions; one thread per (line, block) computes the running prefix G and, in place, the
// running suffix of its block; then out(p) = op(suffix(p - k d), prefix(p + k d)).
// Three min/max per pixel whatever k, each input byte read once from DRAM (the halo is
// re-read from L2 by the neighbouring tile).  Y needs no transpose.
#include <algorithm>
#include <atomic>

#include "common.cuh"

namespace pg {

static constexpr int kLineThreads = 256;

struct LineGeom {
  int dy, dx;       // direction, dy in {0,1}; dx in {-1,0,1}; (0,1) for X
  int k;            // half length (>= 1)
  int TY, TX;       // output tile
  int hy, hx;       // halo rows / cols
  int RH, RW, RWP;  // staged region and its padded row pitch
};

template <typename T, bool SUP>
__global__ void __launch_bounds__(kLineThreads) k_line(const T *__restrict__ in, T *__restrict__ out, int64_t H,
                                                       int64_t W, LineGeom g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *F = reinterpret_cast<T *>(smem_raw);
  T *G = F + (size_t)g.RH * g.RWP;
  const T NEU = Op<T, SUP>::neutral();
  const int64_t ty0 = (int64_t)blockIdx.y * g.TY, tx0 = (int64_t)blockIdx.x * g.TX;
  const int64_t ry0 = ty0 - g.hy, rx0 = tx0 - g.hx;

  // 1. stage the region
  const int area = g.RH * g.RW;
  for (int i = threadIdx.x; i < area; i += blockDim.x) {
    const int r = i / g.RW, c = i - r * g.RW;
    const int64_t gy = ry0 + r, gx = rx0 + c;
    T v = NEU;
    if (gy >= 0 && gy < H && gx >= 0 && gx < W) v = ldg(in + gy * W + gx);
    F[r * g.RWP + c] = v;
  }
  __syncthreads();

  // 2. per (line, block): forward prefix into G, backward suffix in place into F
  const int w = 2 * g.k + 1;
  int nlines, maxlen;
  if (g.dy == 0) { nlines = g.RH; maxlen = g.RW; }
  else if (g.dx == 0) { nlines = g.RW; maxlen = g.RH; }
  else { nlines = g.RH + g.RW - 1; maxlen = min(g.RH, g.RW); }
  const int nblk = (maxlen + w - 1) / w;
  const int step = g.dy * g.RWP + g.dx;
  for (int item = threadIdx.x; item < nlines * nblk; item += blockDim.x) {
    const int l = item % nlines, b = item / nlines;
    int r0, c0, len;
    if (g.dy == 0) { r0 = l; c0 = 0; len = g.RW; }
    else if (g.dx == 0) { r0 = 0; c0 = l; len = g.RH; }
    else if (g.dx == 1) {
      if (l < g.RW) { r0 = 0; c0 = l; len = min(g.RH, g.RW - l); }
      else { r0 = l - g.RW + 1; c0 = 0; len = min(g.RH - r0, g.RW); }
    } else {
      if (l < g.RW) { r0 = 0; c0 = l; len = min(g.RH, l + 1); }
      else { r0 = l - g.RW + 1; c0 = g.RW - 1; len = min(g.RH - r0, g.RW); }
    }
    const int j0 = b * w;
    if (j0 >= len) continue;
    const int j1 = min(j0 + w, len);
    const int base = r0 * g.RWP + c0;
    int p = base + j0 * step;
    T acc = F[p];
    G[p] = acc;
    for (int j = j0 + 1; j < j1; ++j) {
      p += step;
      acc = Op<T, SUP>::apply(acc, F[p]);
      G[p] = acc;
    }
    // p is at j1-1: suffix maxima back to j0, written over F
    acc = F[p];
    for (int j = j1 - 2; j >= j0; --j) {
      p -= step;
      acc = Op<T, SUP>::apply(acc, F[p]);
      F[p] = acc;
    }
  }
  __syncthreads();

  // 3. combine
  const int kd = g.k * step;
  for (int i = threadIdx.x; i < g.TY * g.TX; i += blockDim.x) {
    const int y = i / g.TX, x = i - y * g.TX;
    const int64_t gy = ty0 + y, gx = tx0 + x;
    if (gy >= H || gx >= W) continue;
    const int p = (y + g.hy) * g.RWP + (x + g.hx);
    out[gy * W + gx] = Op<T, SUP>::apply(F[p - kd], G[p + kd]);
  }
}

static size_t line_smem(const LineGeom &g, int es) { return 2ull * (size_t)g.RH * (size_t)g.RWP * (size_t)es; }

static LineGeom make_geom(int dy, int dx, int k, int TY, int TX) {
  LineGeom g;
  g.dy = dy; g.dx = dx; g.k = k; g.TY = TY; g.TX = TX;
  g.hy = k * dy; g.hx = k * (dx < 0 ? -dx : dx);
  g.RH = TY + 2 * g.hy; g.RW = TX + 2 * g.hx;
  g.RWP = g.RW | 1;  // odd pitch: row-wise scans of 4-byte pixels hit distinct banks
  return g;
}

template <typename T, bool SUP>
static pg_status line_t(const T *in, T *out, int64_t H, int64_t W, int dy, int dx, int64_t half, cudaStream_t s) {
  // window reach beyond which every position is outside the image: clipping makes larger
  // halves equivalent
  int64_t kmax;
  if (dy == 0) kmax = W - 1;
  else if (dx == 0) kmax = H - 1;
  else kmax = std::min(H, W) - 1;
  const int64_t k64 = std::min<int64_t>(half, std::max<int64_t>(kmax, 0));
  if (k64 <= 0) {
    PG_CUDA_TRY(cudaMemcpyAsync(out, in, sizeof(T) * (size_t)(H * W), cudaMemcpyDeviceToDevice, s), "copy");
    return PG_OK;
  }
  if (k64 > (1 << 20)) return fail(PG_ERR_INVALID_ARGUMENT, "segment too long");
  const int k = (int)k64;
  const size_t budget = 96 * 1024, hard = 227 * 1024;
  LineGeom g{};
  bool ok = false;
  // largest tile whose staged region fits the budget; narrower tiles for very long segments
  if (dy == 0) {
    for (int tx : {256, 128, 64, 32}) {
      for (int ty : {16, 8, 4, 2, 1}) {
        g = make_geom(0, 1, k, ty, tx);
        if (line_smem(g, sizeof(T)) <= budget) { ok = true; break; }
      }
      if (ok) break;
    }
  } else if (dx == 0) {
    for (int tx : {64, 32, 16, 8}) {
      for (int ty : {256, 128, 64, 32, 16, 8, 4, 2, 1}) {
        g = make_geom(1, 0, k, ty, tx);
        if (line_smem(g, sizeof(T)) <= budget) { ok = true; break; }
      }
      if (ok) break;
    }
  } else {
    for (int t : {128, 64, 32, 16, 8, 4, 2, 1}) {
      g = make_geom(1, dx, k, t, t);
      if (line_smem(g, sizeof(T)) <= budget) { ok = true; break; }
    }
  }
  if (!ok && line_smem(g, sizeof(T)) <= hard) ok = true;
  if (!ok) return fail(PG_ERR_INVALID_ARGUMENT, "segment too long for the shared-memory line kernel");
  const size_t smem = line_smem(g, sizeof(T));
  // the opt-in shared-memory size is a per-device attribute of each instantiation
  static std::atomic<uint64_t> attr_devices{0};
  int dev = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  const uint64_t bit = 1ull << (dev & 63);
  if (!(attr_devices.load() & bit)) {
    PG_CUDA_TRY(cudaFuncSetAttribute(k_line<T, SUP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hard),
                "line kernel smem attribute");
    attr_devices.fetch_or(bit);
  }
  dim3 grid((unsigned)ceil_div(W, g.TX), (unsigned)ceil_div(H, g.TY));
  if (grid.y > 65535) return fail(PG_ERR_INVALID_ARGUMENT, "image too tall for the line kernel");
  k_line<T, SUP><<<grid, kLineThreads, smem, s>>>(in, out, H, W, g);
  return cuda_status(cudaGetLastError(), "line kernel launch");
}

pg_status launch_line(const pg_image &in, const pg_image &out, int dy, int dx, int64_t half, bool dilate,
                      cudaStream_t s) {
  const Dims d = dims_of(in);
  if (d.count() == 0) return PG_OK;
  if (in.rank == 3) return fail(PG_ERR_UNSUPPORTED_SE, "line segments are 1D/2D only");
  // normalise the direction: dy >= 0, and (0, 1) for X
  if (dy < 0 || (dy == 0 && dx < 0)) { dy = -dy; dx = -dx; }
  if (!((dy == 0 && dx == 1) || (dy == 1 && (dx == 0 || dx == 1 || dx == -1))))
    return fail(PG_ERR_UNSUPPORTED_SE, "line direction must be X, Y or a 45-degree diagonal");
  if (half < 0) return fail(PG_ERR_INVALID_ARGUMENT, "negative half segment");
  // clipping makes any half length beyond the image's reach equivalent to that reach
  int64_t kmax;
  if (dy == 0) kmax = d.nx - 1;
  else if (dx == 0) kmax = d.ny - 1;
  else kmax = std::min(d.ny, d.nx) - 1;
  const int64_t k = std::min<int64_t>(half, std::max<int64_t>(kmax, 0));
  if (k >= 1 && k <= (1 << 20)) {
    pg_status st = PG_OK;
    if (dx != 0 && try_segment_tile(in, out, dy, dx, (int)k, dilate, s, &st)) return st;
    if (try_line_stream(in, out, dy, dx, (int)k, dilate, s, &st)) return st;
    if (try_line_words(in, out, dy, dx, (int)k, dilate, s, &st)) return st;
  }
  PG_DISPATCH_PTYPE(in.ptype, T, {
    const T *src = static_cast<const T *>(in.data);
    T *dst = static_cast<T *>(out.data);
    return dilate ? line_t<T, true>(src, dst, d.ny, d.nx, dy, dx, half, s)
                  : line_t<T, false>(src, dst, d.ny, d.nx, dy, dx, half, s);
  });
  return PG_OK;
}

pg_status launch_rect(const pg_image &in, const pg_image &out, int64_t hy, int64_t hx, bool dilate, cudaStream_t s) {
  if (hy < 0 || hx < 0) return fail(PG_ERR_INVALID_ARGUMENT, "negative rectangle half size");
  if (hy == 0) return launch_line(in, out, 0, 1, hx, dilate, s);
  if (hx == 0) return launch_line(in, out, 1, 0, hy, dilate, s);
  const Dims d = dims_of(in);
  Scratch tmp;
  PG_TRY(tmp.alloc((size_t)d.count() * elem_size(in.ptype), s));
  pg_image t = in;
  t.data = tmp.ptr;
  PG_TRY(launch_line(in, t, 0, 1, hx, dilate, s));
  return launch_line(t, out, 1, 0, hy, dilate, s);
}

}  // namespace pg
