// capi.cu -- the extern "C" boundary: argument checks that mirror the reference's
// (AssertSizesCompatible / AssertAsTypesCompatible / AssertImagesAreDifferent, the
// rank x PType x SE switches of src/low_level_morpho/*.cpp and src/geodesy/*.cpp), then
// dispatch to the kernels.  No exception crosses the boundary.
#include <atomic>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace pg {

static thread_local std::string t_err;

void set_error(const std::string &msg) { t_err = msg; }

pg_status fail(pg_status st, const std::string &msg) {
  t_err = msg;
  return st;
}

pg_status cuda_status(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return PG_OK;
  t_err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? PG_ERR_OUT_OF_MEMORY : PG_ERR_CUDA;
}

static std::atomic<int> g_alloc_failures{0};

bool take_injected_alloc_failure() {
  int n = g_alloc_failures.load();
  while (n > 0)
    if (g_alloc_failures.compare_exchange_weak(n, n - 1)) return true;
  return false;
}

void retain_pool_memory() {
  static std::mutex mu;
  static std::vector<bool> done;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  std::lock_guard<std::mutex> lk(mu);
  if ((size_t)dev >= done.size()) done.resize((size_t)dev + 1, false);
  if (done[(size_t)dev]) return;
  done[(size_t)dev] = true;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return;
  }
  uint64_t keep = kPoolRetainBytes;
  if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) (void)cudaGetLastError();
}

int num_sms() {
  static std::mutex mu;
  static int cached_dev = -1, cached = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  std::lock_guard<std::mutex> lk(mu);
  if (dev != cached_dev) {
    if (cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) cached = 1;
    cached_dev = dev;
  }
  return cached;
}

// ------------------------------------------------------------------ checks
static pg_status check_image(const pg_image *im, const char *what) {
  if (!im) return fail(PG_ERR_INVALID_ARGUMENT, std::string(what) + ": null image descriptor");
  if (im->rank < 1 || im->rank > 3) return fail(PG_ERR_INVALID_ARGUMENT, std::string(what) + ": unsupported number of dims");
  if (!elem_size(im->ptype)) return fail(PG_ERR_UNSUPPORTED_PTYPE, std::string(what) + ": unsupported PTYPE");
  int64_t n = 1;
  for (int i = 0; i < im->rank; ++i) {
    if (im->shape[i] < 0) return fail(PG_ERR_INVALID_ARGUMENT, std::string(what) + ": negative dimension");
    n *= im->shape[i];
  }
  if (n > 0 && !im->data) return fail(PG_ERR_INVALID_ARGUMENT, std::string(what) + ": null data pointer");
  return PG_OK;
}

static bool same_geometry(const pg_image &a, const pg_image &b) {
  if (a.rank != b.rank) return false;
  for (int i = 0; i < a.rank; ++i) if (a.shape[i] != b.shape[i]) return false;
  return true;
}

static bool overlaps(const pg_image &a, const pg_image &b) {
  const size_t na = (size_t)dims_of(a).count() * elem_size(a.ptype), nb = (size_t)dims_of(b).count() * elem_size(b.ptype);
  if (na == 0 || nb == 0) return false;
  const char *pa = static_cast<const char *>(a.data), *pb = static_cast<const char *>(b.data);
  return pa < pb + nb && pb < pa + na;
}

// in -> out of the same geometry and type, distinct buffers
pg_status check_in_out(const pg_image *in, const pg_image *out, const char *what) {
  PG_TRY(check_image(in, what));
  PG_TRY(check_image(out, what));
  if (!same_geometry(*in, *out)) return fail(PG_ERR_INCOMPATIBLE, std::string(what) + " images have not compatible sizes");
  if (in->ptype != out->ptype) return fail(PG_ERR_INCOMPATIBLE, std::string(what) + " images must have compatible types");
  if (overlaps(*in, *out)) return fail(PG_ERR_ALIASING, std::string(what) + " input output images must be different");
  return PG_OK;
}

static int se_rank(int se) {
  switch (se) {
    case PG_SE_SEGMENT_X_1D: return 1;
    case PG_SE_SQUARE_2D: case PG_SE_CROSS_2D: case PG_SE_SEGMENT_X_2D: case PG_SE_SEGMENT_Y_2D: return 2;
    case PG_SE_SEGMENT_X_3D: case PG_SE_SEGMENT_Y_3D: case PG_SE_SEGMENT_Z_3D: case PG_SE_CROSS_3D: case PG_SE_SQUARE_3D: return 3;
    default: return 0;
  }
}

// A ScalarTypeVariant must hold exactly the pixel type the reference's std::get<T> asks for
// (src/pixel_processing/arith.cpp:55, compare.cpp:51-61); where it does not, poutre2 catches
// std::bad_variant_access and throws "unable to extract suitable type".  Floating-point values must
// also be finite.
static const char *ptype_name(int pt) {
  switch (pt) {
    case PG_PTYPE_U8: return "UINT8";
    case PG_PTYPE_U16: return "UINT16";
    case PG_PTYPE_I32: return "INT32";
    case PG_PTYPE_I64: return "INT64";
    case PG_PTYPE_F32: return "FLOAT";
    case PG_PTYPE_F64: return "DOUBLE";
    default: return "undefined";
  }
}

static pg_status check_scalar(int ptype, const pg_scalar *v, const char *what) {
  if (!v) return fail(PG_ERR_INVALID_ARGUMENT, std::string(what) + ": null scalar");
  if (v->ptype != ptype)
    return fail(PG_ERR_SCALAR_TYPE, std::string(what) + " unable to extract suitable type from the scalar (it holds " +
                                        ptype_name(v->ptype) + ", the pixel type is " + ptype_name(ptype) + ")");
  if ((ptype == PG_PTYPE_F32 && !std::isfinite(v->v.f32)) || (ptype == PG_PTYPE_F64 && !std::isfinite(v->v.f64)))
    return fail(PG_ERR_INVALID_ARGUMENT, std::string(what) + ": non-finite scalar");
  return PG_OK;
}

// ------------------------------------------------------------------ erosion / dilation
// `iter` passes of a small static SE, alternating between `out` and a temporary
static pg_status repeat_small(const pg_image &in, int se, int iter, const pg_image &out, bool dilate, cudaStream_t s) {
  if (iter == 1) return launch_small_se(in, out, se, dilate, s);
  if (se == PG_SE_CROSS_2D && in.rank == 2) {  // the iterated cross: all passes in one tile kernel (octagon.cu)
    pg_status st = PG_OK;
    if (try_octagon_tile(in, out, iter, 0, dilate, s, &st)) return st;
  }
  Scratch tmp;
  PG_TRY(tmp.alloc((size_t)dims_of(in).count() * elem_size(in.ptype), s));
  pg_image t = in;
  t.data = tmp.ptr;
  // pass k writes `out` when (iter - k) is even, so the last pass lands in `out`
  const pg_image *src = &in;
  for (int k = 1; k <= iter; ++k) {
    const pg_image *dst = ((iter - k) % 2 == 0) ? &out : &t;
    PG_TRY(launch_small_se(*src, *dst, se, dilate, s));
    src = dst;
  }
  return PG_OK;
}

// Erosion / dilation of a 1D or 2D image by the (2hy+1) x (2hx+1) box (hy = 0: X segment, hx = 0:
// Y segment).  Iterating the 3x3 square, or a 3-pixel X or Y segment, k times under the clipped
// border equals one pass of the box k times as wide: along each axis every pixel between two
// in-image pixels is in the image, so both reach the same pixels.  Whichever form is faster runs.
// On 4096^2 images a 3-pixel pass costs 10-15 us (1-, 2-byte pixels), a line pass of any length
// 20-30 us: the square runs as repeated 3x3 passes up to 4 (1-, 2-byte pixels) or 2 (wider),
// a 3-pixel segment as one 3-pixel pass, anything else as line passes.
static pg_status box(const pg_image &in, const pg_image &out, int64_t hy, int64_t hx, bool dilate, cudaStream_t s) {
  const int64_t square_passes_max = elem_size(in.ptype) <= 2 ? 4 : 2;
  if (hy == 0 && hx == 1)
    return launch_small_se(in, out, in.rank == 1 ? PG_SE_SEGMENT_X_1D : PG_SE_SEGMENT_X_2D, dilate, s);
  if (in.rank == 2 && hy == 1 && hx == 0) return launch_small_se(in, out, PG_SE_SEGMENT_Y_2D, dilate, s);
  if (in.rank == 2 && hy == hx && hy >= 1 && hy <= square_passes_max)
    return repeat_small(in, PG_SE_SQUARE_2D, (int)hy, out, dilate, s);
  pg_status st = PG_OK;
  // Y segment: the segment tile kernel (diag.cu), measured faster than the box tile for every type
  if (hx == 0 && hy <= 31 && try_segment_tile(in, out, 1, 0, (int)hy, dilate, s, &st)) return st;
  if (try_rect_fused(in, out, hy, hx, dilate, s, &st)) return st;  // shared-memory tile pass (rect.cu)
  if (hy == 0) return launch_line(in, out, 0, 1, hx, dilate, s);
  return launch_rect(in, out, hy, hx, dilate, s);
}

static pg_status static_iter(const pg_image &in, int se, int iter, const pg_image &out, bool dilate, cudaStream_t s) {
  if (se_rank(se) == 0 || se_rank(se) != in.rank) return fail(PG_ERR_UNSUPPORTED_SE, "unsupported nl_static");
  if (iter < 0) return fail(PG_ERR_INVALID_ARGUMENT, "iter must be >= 0");
  if (iter == 0) return launch_copy(in, out, s);
  switch (se) {  // the boxes: one pass of the box `iter` times as wide (see box())
    case PG_SE_SEGMENT_X_1D:
    case PG_SE_SEGMENT_X_2D: return box(in, out, 0, iter, dilate, s);
    case PG_SE_SEGMENT_Y_2D: return box(in, out, iter, 0, dilate, s);
    case PG_SE_SQUARE_2D: return box(in, out, iter, iter, dilate, s);
    default: return repeat_small(in, se, iter, out, dilate, s);
  }
}

// sequence of static passes (compound SEs): passes[i] applied in order
static pg_status static_sequence(const pg_image &in, const std::vector<int> &passes, const pg_image &out, bool dilate,
                                 cudaStream_t s) {
  const int n = (int)passes.size();
  if (n == 0) return launch_copy(in, out, s);
  if (n == 1) return launch_small_se(in, out, passes[0], dilate, s);
  Scratch tmp;
  PG_TRY(tmp.alloc((size_t)dims_of(in).count() * elem_size(in.ptype), s));
  pg_image t = in;
  t.data = tmp.ptr;
  const pg_image *src = &in;
  for (int k = 1; k <= n; ++k) {
    const pg_image *dst = ((n - k) % 2 == 0) ? &out : &t;
    PG_TRY(launch_small_se(*src, *dst, passes[k - 1], dilate, s));
    src = dst;
  }
  return PG_OK;
}

// t_DilateOctagon / t_DilateRhombicuboctahedron (ero_dil_compound_static_se_t.hpp:34-160):
// `size` passes, the last round(size / (1 + sqrt 2)) of them by the square, the others by
// the cross.
static pg_status compound(const pg_image &in, int compound_se, int size, const pg_image &out, bool dilate, cudaStream_t s) {
  int cross, square;
  if (compound_se == PG_COMPOUND_OCTAGON) {
    if (in.rank != 2) return fail(PG_ERR_INVALID_ARGUMENT, "Octagon: unsupported number of dims");
    cross = PG_SE_CROSS_2D; square = PG_SE_SQUARE_2D;
  } else if (compound_se == PG_COMPOUND_RHOMBICUBOCTAHEDRON) {
    if (in.rank != 3) return fail(PG_ERR_INVALID_ARGUMENT, "Rhombicuboctahedron: unsupported number of dims");
    // size 1 applies the 2D cross to the volume in the reference, which t_Dilate rejects
    if (size == 1) return fail(PG_ERR_UNSUPPORTED_SE, "unsupported nl_static");
    cross = PG_SE_CROSS_3D; square = PG_SE_SQUARE_3D;
  } else {
    return fail(PG_ERR_UNSUPPORTED_SE, "unsupported Compound_NL_SE");
  }
  if (size < 0) return fail(PG_ERR_INVALID_ARGUMENT, "size must be >= 0");
  if (size == 0) return launch_copy(in, out, s);
  if (size == 1) return launch_small_se(in, out, cross, dilate, s);
  const double nb = (double)size / (1.0 + std::sqrt(2.0));
  const double fl = std::floor(nb);
  const int nb_square = (int)((nb - fl) < 0.5 ? fl : fl + 1);
  if (in.rank == 2) {  // all passes in one shared-memory tile kernel (octagon.cu)
    pg_status st = PG_OK;
    if (try_octagon_tile(in, out, size - nb_square, nb_square, dilate, s, &st)) return st;
  }
  std::vector<int> passes;
  passes.push_back(cross);
  for (int i = 1; i < size - nb_square; ++i) passes.push_back(cross);
  if (in.rank == 2 && nb_square >= 2) {
    // the trailing run of squares is one box (see box())
    Scratch tmp;
    PG_TRY(tmp.alloc((size_t)dims_of(in).count() * elem_size(in.ptype), s));
    pg_image t = in;
    t.data = tmp.ptr;
    PG_TRY(static_sequence(in, passes, t, dilate, s));
    return box(t, out, nb_square, nb_square, dilate, s);
  }
  for (int i = 0; i < nb_square; ++i) passes.push_back(square);
  return static_sequence(in, passes, out, dilate, s);
}

static pg_status by_se(const pg_image &in, const pg_se &se, const pg_image &out, bool dilate, cudaStream_t s) {
  switch (se.kind) {
    case PG_SE_KIND_STATIC: return static_iter(in, se.common_se, se.iter, out, dilate, s);
    case PG_SE_KIND_RECT:
      if (in.rank != 2) return fail(PG_ERR_UNSUPPORTED_SE, "rectangle SE needs a 2D image");
      if (se.hy < 0 || se.hx < 0) return fail(PG_ERR_INVALID_ARGUMENT, "negative rectangle half size");
      return box(in, out, se.hy, se.hx, dilate, s);
    case PG_SE_KIND_LINE:
      if (in.rank != 2) return fail(PG_ERR_UNSUPPORTED_SE, "line SE needs a 2D image");
      if (se.half < 0) return fail(PG_ERR_INVALID_ARGUMENT, "negative half segment");
      if (se.dy == 0 && (se.dx == 1 || se.dx == -1)) return box(in, out, 0, se.half, dilate, s);
      if (se.dx == 0 && (se.dy == 1 || se.dy == -1)) return box(in, out, se.half, 0, dilate, s);
      return launch_line(in, out, se.dy, se.dx, se.half, dilate, s);
    case PG_SE_KIND_NL:
      if (!se.offsets || se.n < 1 || se.n > 4096) return fail(PG_ERR_INVALID_ARGUMENT, "neighbour list must hold 1..4096 offsets");
      return launch_nl(in, out, se.offsets, se.n, dilate, s);
    default: return fail(PG_ERR_UNSUPPORTED_SE, "unknown pg_se kind");
  }
}

enum Composite { C_OPEN, C_CLOSE, C_GRAD };
// the box (hy, hx) an SE stands for (see box()), if it is one
static bool se_box(const pg_se &se, int rank, int64_t &hy, int64_t &hx) {
  if (rank != 2) return false;
  switch (se.kind) {
    case PG_SE_KIND_RECT: hy = se.hy; hx = se.hx; return hy >= 0 && hx >= 0;
    case PG_SE_KIND_LINE:
      if (se.half < 0) return false;
      if (se.dy == 0 && (se.dx == 1 || se.dx == -1)) { hy = 0; hx = se.half; return true; }
      if (se.dx == 0 && (se.dy == 1 || se.dy == -1)) { hy = se.half; hx = 0; return true; }
      return false;
    case PG_SE_KIND_STATIC:
      if (se.iter < 1) return false;
      if (se.common_se == PG_SE_SQUARE_2D) { hy = hx = se.iter; return true; }
      if (se.common_se == PG_SE_SEGMENT_X_2D) { hy = 0; hx = se.iter; return true; }
      if (se.common_se == PG_SE_SEGMENT_Y_2D) { hy = se.iter; hx = 0; return true; }
      return false;
    default: return false;
  }
}

// the segment (dy = 1, dx in {-1, 0, 1}: 45 degrees, vertical, 135 degrees) of half length k an SE
// stands for, if it is one; horizontal segments are boxes (se_box)
static bool se_segment(const pg_se &se, int rank, int &dx, int64_t &k) {
  if (rank != 2) return false;
  switch (se.kind) {
    case PG_SE_KIND_LINE: {
      int dy = se.dy;
      dx = se.dx;
      if (dy < 0 || (dy == 0 && dx < 0)) { dy = -dy; dx = -dx; }
      k = se.half;
      return dy == 1 && dx >= -1 && dx <= 1 && k >= 0;
    }
    case PG_SE_KIND_RECT: dx = 0; k = se.hy; return se.hx == 0 && k >= 0;
    case PG_SE_KIND_STATIC: dx = 0; k = se.iter; return se.common_se == PG_SE_SEGMENT_Y_2D && k >= 1;
    default: return false;
  }
}

static pg_status composite(const pg_image &in, const pg_se &se, const pg_image &out, Composite c, cudaStream_t s) {
  int64_t hy = 0, hx = 0;
  pg_status st = PG_OK;
  int sdx = 0;
  int64_t sk = 0;
  // the gradient by a vertical or diagonal segment: both operators from one scan of one tile (diag.cu)
  if (c == C_GRAD && se_segment(se, in.rank, sdx, sk) && sk <= 31 && try_segment_gradient(in, out, 1, sdx, (int)sk, s, &st))
    return st;
  // the gradient of a box: dilation and erosion of one tile in one pass (rect.cu)
  if (c == C_GRAD && se_box(se, in.rank, hy, hx) && try_rect_gradient(in, out, hy, hx, s, &st)) return st;
  // opening / closing of a box: both operators on one tile (rect_open.cu)
  if (c != C_GRAD && se_box(se, in.rank, hy, hx) && try_rect_open(in, out, hy, hx, c == C_OPEN, s, &st)) return st;
  // opening / closing by a vertical or diagonal segment: both operators on one tile (diag.cu)
  if (c != C_GRAD && se_segment(se, in.rank, sdx, sk) && sk <= 31 &&
      try_segment_open(in, out, 1, sdx, (int)sk, c == C_OPEN, s, &st))
    return st;
  Scratch tmp;
  PG_TRY(tmp.alloc((size_t)dims_of(in).count() * elem_size(in.ptype), s));
  pg_image t = in;
  t.data = tmp.ptr;
  if (c == C_OPEN) {
    PG_TRY(by_se(in, se, t, false, s));
    return by_se(t, se, out, true, s);
  }
  if (c == C_CLOSE) {
    PG_TRY(by_se(in, se, t, true, s));
    return by_se(t, se, out, false, s);
  }
  Scratch tmp2;
  PG_TRY(tmp2.alloc((size_t)dims_of(in).count() * elem_size(in.ptype), s));
  pg_image e = in;
  e.data = tmp2.ptr;
  PG_TRY(by_se(in, se, t, true, s));
  PG_TRY(by_se(in, se, e, false, s));
  return launch_sub(t, e, out, s);
}

// ------------------------------------------------------------------ geodesy helpers
pg_status recon_se(int se, int rank, bool &conn8) {
  if (rank == 1 && se == PG_SE_SEGMENT_X_1D) { conn8 = true; return PG_OK; }
  if (rank == 2 && se == PG_SE_SQUARE_2D) { conn8 = true; return PG_OK; }
  if (rank == 2 && se == PG_SE_CROSS_2D) { conn8 = false; return PG_OK; }
  if (rank == 3 && se == PG_SE_CROSS_3D) { conn8 = false; return PG_OK; }
  // poutre2's raster / anti-raster schedule stops short of the fixpoint for SESquare3D (it differs
  // from the iterated geodesic dilation on thin volumes), so no GPU result could match it
  if (rank == 3 && se == PG_SE_SQUARE_3D)
    return fail(PG_ERR_UNSUPPORTED_SE, "SESquare3D reconstruction is not on the GPU path");
  return fail(PG_ERR_UNSUPPORTED_SE, "t_ReconstructionDispatchNl unsupported nl_static");
}

static pg_status h_recon(const pg_image *in, const pg_scalar &h, int se, const pg_image *out, bool maxima, cudaStream_t s) {
  ReconRequest rq;
  PG_TRY(recon_se(se, in->rank, rq.conn8));
  rq.dilate = maxima;
  rq.init = INIT_SAT_CONST;
  rq.h = h;
  return launch_reconstruction(nullptr, in, out, 1, rq, s);
}

// poutre::label::label_minima / label_maxima (src/label/label_extrema.cpp): label_binary of
// h_concave(f, 1) / h_convex(f, 1) -- the regional minima / maxima, numbered in raster order.
static pg_status label_extrema(const pg_image *in, int32_t se, const pg_image *out, int64_t *nb_labels, bool maxima,
                               cudaStream_t s) {
  const char *what = maxima ? "label_maxima" : "label_minima";
  PG_TRY(check_image(in, what));
  PG_TRY(check_image(out, what));
  if (!same_geometry(*in, *out)) return fail(PG_ERR_INCOMPATIBLE, std::string(what) + " incompatible size");
  if (overlaps(*in, *out)) return fail(PG_ERR_ALIASING, std::string(what) + " output must be != than input images");
  if (out->ptype != PG_PTYPE_I64)
    return fail(PG_ERR_INCOMPATIBLE, "label_binaryImageDispatch o_img downcast fail (output must be INT64)");
  if (in->ptype == PG_PTYPE_F32 || in->ptype == PG_PTYPE_F64)
    return fail(PG_ERR_UNSUPPORTED_PTYPE, "label_binary of a float image is not on the GPU path");
  if (se_rank(se) == 0 || se_rank(se) != in->rank) return fail(PG_ERR_UNSUPPORTED_SE, "t_label_binaryDispatch unsupported nl_static");
  bool conn8;
  PG_TRY(recon_se(se, in->rank, conn8));  // the h-extrema reconstruction's own SE rule
  const size_t bytes = (size_t)dims_of(*in).count() * elem_size(in->ptype);
  Scratch rec, ext;
  PG_TRY(rec.alloc(bytes, s));
  PG_TRY(ext.alloc(bytes, s));
  pg_image r = *in, e = *in;
  r.data = rec.ptr;
  e.data = ext.ptr;
  PG_TRY(h_recon(in, scalar_of(in->ptype, 1), se, &r, maxima, s));  // h_maxima / h_minima with h = 1
  // h_convex = sat_sub(f, h_maxima(f)), h_concave = sat_sub(h_minima(f), f) (extrema.cpp:51-73)
  PG_TRY(maxima ? launch_sat_sub_image(*in, r, e, s) : launch_sat_sub_image(r, *in, e, s));
  return launch_label(e, se, *out, false, nb_labels, s);
}

// ---------------------------------------------------------------- labelling
// poutre::label::label_binary / label_flat_zones (src/label/label_binary.cpp, label_flat_zones.cpp):
// the output is an INT64 image of the input's shape (the reference's dispatch downcasts it to
// image_t<int64>), distinct from the input; the SE's rank must be the image's.
static pg_status label_call(const pg_image *in, int32_t se, const pg_image *out, int64_t *nb_labels, bool flat,
                            cudaStream_t s) {
  const char *what = flat ? "label_flat_zones" : "label_binary";
  PG_TRY(check_image(in, what));
  PG_TRY(check_image(out, what));
  if (!same_geometry(*in, *out)) return fail(PG_ERR_INCOMPATIBLE, std::string(what) + " incompatible size");
  if (out->ptype != PG_PTYPE_I64)
    return fail(PG_ERR_INCOMPATIBLE, std::string(what) + "ImageDispatch o_img downcast fail (output must be INT64)");
  if (overlaps(*in, *out)) return fail(PG_ERR_ALIASING, std::string(what) + " input output images must be different");
  if (se_rank(se) == 0 || se_rank(se) != in->rank)
    return fail(PG_ERR_UNSUPPORTED_SE, flat ? "t_label_flat_zonesDispatch unsupported nl_static"
                                            : "t_label_binaryDispatch unsupported nl_static");
  return launch_label(*in, se, *out, flat, nb_labels, s);
}

}  // namespace pg

using namespace pg;

#define STREAM(s) reinterpret_cast<cudaStream_t>(s)

extern "C" {

const char *pg_last_error(void) { return t_err.c_str(); }
const char *pg_version(void) { return "poutre2_gb300 0.1 (sm_103a)"; }

// Test hook: the next n temporary allocations fail as if the device were out of memory.
pg_status pg_debug_fail_allocations(int32_t n) {
  if (n < 0) return pg::fail(PG_ERR_INVALID_ARGUMENT, "pg_debug_fail_allocations: negative count");
  pg::g_alloc_failures.store(n);
  return PG_OK;
}

// ---------------------------------------------------------------- low_level_morpho
pg_status pg_erode(const pg_image *in, int32_t se, int32_t iter, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "Erode iter"));
  return static_iter(*in, se, iter, *out, false, STREAM(s));
}
pg_status pg_dilate(const pg_image *in, int32_t se, int32_t iter, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "Dilate iter"));
  return static_iter(*in, se, iter, *out, true, STREAM(s));
}
pg_status pg_erode_compound(const pg_image *in, int32_t cse, int32_t size, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "Erode compound"));
  return compound(*in, cse, size, *out, false, STREAM(s));
}
pg_status pg_dilate_compound(const pg_image *in, int32_t cse, int32_t size, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "Dilate compound"));
  return compound(*in, cse, size, *out, true, STREAM(s));
}
pg_status pg_erode_nl(const pg_image *in, const int32_t *offsets, int32_t n, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "Erode IStructuringElement"));
  if (!offsets || n < 1 || n > 4096) return fail(PG_ERR_INVALID_ARGUMENT, "neighbour list must hold 1..4096 offsets");
  return launch_nl(*in, *out, offsets, n, false, STREAM(s));
}
pg_status pg_dilate_nl(const pg_image *in, const int32_t *offsets, int32_t n, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "Dilate IStructuringElement"));
  if (!offsets || n < 1 || n > 4096) return fail(PG_ERR_INVALID_ARGUMENT, "neighbour list must hold 1..4096 offsets");
  return launch_nl(*in, *out, offsets, n, true, STREAM(s));
}

static pg_status line_x(const pg_image *in, int64_t half, const pg_image *out, bool dilate, cudaStream_t s,
                        const char *what) {
  PG_TRY(check_in_out(in, out, what));
  if (in->rank > 2) return fail(PG_ERR_INVALID_ARGUMENT, std::string(what) + " Unsupported number of dims");
  if (half <= 0) return launch_copy(*in, *out, s);  // size_line_segment <= 0 copies (ero_dil_line_se_t.hpp:161-164)
  return box(*in, *out, 0, half, dilate, s);
}
static pg_status line_y(const pg_image *in, int64_t half, const pg_image *out, bool dilate, cudaStream_t s,
                        const char *what) {
  PG_TRY(check_in_out(in, out, what));
  if (in->rank != 2) return fail(PG_ERR_INVALID_ARGUMENT, std::string(what) + " Unsupported number of dims");
  // t_DilateY transposes into a temporary of the input's shape (ero_dil_line_se_t.hpp:258)
  if (in->shape[0] != in->shape[1]) return fail(PG_ERR_NOT_SQUARE, std::string(what) + " needs a square image (t_transpose)");
  if (half <= 0) return launch_copy(*in, *out, s);
  return box(*in, *out, half, 0, dilate, s);
}
pg_status pg_erode_x(const pg_image *in, int64_t half, const pg_image *out, pg_stream_t s) { return line_x(in, half, out, false, STREAM(s), "ErodeX"); }
pg_status pg_dilate_x(const pg_image *in, int64_t half, const pg_image *out, pg_stream_t s) { return line_x(in, half, out, true, STREAM(s), "DilateX"); }
pg_status pg_erode_y(const pg_image *in, int64_t half, const pg_image *out, pg_stream_t s) { return line_y(in, half, out, false, STREAM(s), "ErodeY"); }
pg_status pg_dilate_y(const pg_image *in, int64_t half, const pg_image *out, pg_stream_t s) { return line_y(in, half, out, true, STREAM(s), "DilateY"); }

pg_status pg_erode_se(const pg_image *in, const pg_se *se, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "Erode"));
  if (!se) return fail(PG_ERR_INVALID_ARGUMENT, "null SE");
  return by_se(*in, *se, *out, false, STREAM(s));
}
pg_status pg_dilate_se(const pg_image *in, const pg_se *se, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "Dilate"));
  if (!se) return fail(PG_ERR_INVALID_ARGUMENT, "null SE");
  return by_se(*in, *se, *out, true, STREAM(s));
}
pg_status pg_opening(const pg_image *in, const pg_se *se, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "Opening"));
  if (!se) return fail(PG_ERR_INVALID_ARGUMENT, "null SE");
  return composite(*in, *se, *out, C_OPEN, STREAM(s));
}
pg_status pg_closing(const pg_image *in, const pg_se *se, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "Closing"));
  if (!se) return fail(PG_ERR_INVALID_ARGUMENT, "null SE");
  return composite(*in, *se, *out, C_CLOSE, STREAM(s));
}
pg_status pg_gradient(const pg_image *in, const pg_se *se, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "Gradient"));
  if (!se) return fail(PG_ERR_INVALID_ARGUMENT, "null SE");
  return composite(*in, *se, *out, C_GRAD, STREAM(s));
}

pg_status pg_label_binary(const pg_image *in, int32_t common_se, const pg_image *out, int64_t *nb_labels,
                          pg_stream_t s) {
  return label_call(in, common_se, out, nb_labels, false, STREAM(s));
}
pg_status pg_label_flat_zones(const pg_image *in, int32_t common_se, const pg_image *out, int64_t *nb_labels,
                              pg_stream_t s) {
  return label_call(in, common_se, out, nb_labels, true, STREAM(s));
}
pg_status pg_label_minima(const pg_image *in, int32_t common_se, const pg_image *out, int64_t *nb_labels,
                          pg_stream_t s) {
  return label_extrema(in, common_se, out, nb_labels, false, STREAM(s));
}
pg_status pg_label_maxima(const pg_image *in, int32_t common_se, const pg_image *out, int64_t *nb_labels,
                          pg_stream_t s) {
  return label_extrema(in, common_se, out, nb_labels, true, STREAM(s));
}

// ---------------------------------------------------------------- geodesy
pg_status pg_reconstruction(int32_t type, const pg_image *marker, const pg_image *mask, int32_t se, const pg_image *out,
                            pg_stream_t s) {
  PG_TRY(check_in_out(marker, out, "t_Reconstruct"));
  PG_TRY(check_in_out(mask, out, "t_Reconstruct"));
  if (type != PG_RECONSTRUCT_ERODE && type != PG_RECONSTRUCT_DILATE)
    return fail(PG_ERR_INVALID_ARGUMENT, "t_ReconstructionDispatchRectType unsupported reconstruction_type");
  ReconRequest rq;
  PG_TRY(recon_se(se, mask->rank, rq.conn8));
  rq.dilate = type == PG_RECONSTRUCT_DILATE;
  return launch_reconstruction(marker, mask, out, 1, rq, STREAM(s));
}

pg_status pg_h_maxima(const pg_image *in, const pg_scalar *h, int32_t se, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "h_maxima"));
  PG_TRY(check_scalar(in->ptype, h, "h_maxima"));
  return h_recon(in, *h, se, out, true, STREAM(s));
}
pg_status pg_h_minima(const pg_image *in, const pg_scalar *h, int32_t se, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "h_minima"));
  PG_TRY(check_scalar(in->ptype, h, "h_minima"));
  return h_recon(in, *h, se, out, false, STREAM(s));
}
pg_status pg_h_convex(const pg_image *in, const pg_scalar *h, int32_t se, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "h_convex"));
  PG_TRY(check_scalar(in->ptype, h, "h_convex"));
  Scratch tmp;
  PG_TRY(tmp.alloc((size_t)dims_of(*in).count() * elem_size(in->ptype), STREAM(s)));
  pg_image t = *in;
  t.data = tmp.ptr;
  PG_TRY(h_recon(in, *h, se, &t, true, STREAM(s)));
  return launch_sat_sub_image(*in, t, *out, STREAM(s));  // sat_sub(f, h_maxima(f)) (extrema.cpp:63-73)
}
pg_status pg_h_concave(const pg_image *in, const pg_scalar *h, int32_t se, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "h_concave"));
  PG_TRY(check_scalar(in->ptype, h, "h_concave"));
  Scratch tmp;
  PG_TRY(tmp.alloc((size_t)dims_of(*in).count() * elem_size(in->ptype), STREAM(s)));
  pg_image t = *in;
  t.data = tmp.ptr;
  PG_TRY(h_recon(in, *h, se, &t, false, STREAM(s)));
  return launch_sat_sub_image(t, *in, *out, STREAM(s));  // sat_sub(h_minima(f), f) (extrema.cpp:51-61)
}

static pg_status dyn_pseudo(const pg_image *in, const pg_scalar &h, int se, const pg_image *out, bool opening, cudaStream_t s) {
  Scratch a, b;
  const size_t bytes = (size_t)dims_of(*in).count() * elem_size(in->ptype);
  PG_TRY(a.alloc(bytes, s));
  PG_TRY(b.alloc(bytes, s));
  pg_image ext = *in, mk = *in;
  ext.data = a.ptr;
  mk.data = b.ptr;
  PG_TRY(h_recon(in, h, se, &ext, opening, s));
  PG_TRY(launch_dyn_pseudo_marker(*in, ext, h, opening, mk, s));
  ReconRequest rq;
  PG_TRY(recon_se(se, in->rank, rq.conn8));
  rq.dilate = opening;
  return launch_reconstruction(&mk, in, out, 1, rq, s);
}
pg_status pg_dynamic_pseudo_opening(const pg_image *in, const pg_scalar *h, int32_t se, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "dynamic_pseudo_opening"));
  PG_TRY(check_scalar(in->ptype, h, "dynamic_pseudo_opening"));
  return dyn_pseudo(in, *h, se, out, true, STREAM(s));
}
pg_status pg_dynamic_pseudo_closing(const pg_image *in, const pg_scalar *h, int32_t se, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "dynamic_pseudo_closing"));
  PG_TRY(check_scalar(in->ptype, h, "dynamic_pseudo_closing"));
  return dyn_pseudo(in, *h, se, out, false, STREAM(s));
}

static pg_status check_binary_out(const pg_image *in, const pg_image *out, const char *what) {
  PG_TRY(check_image(in, what));
  PG_TRY(check_image(out, what));
  if (!same_geometry(*in, *out)) return fail(PG_ERR_INCOMPATIBLE, std::string(what) + " images have not compatible sizes");
  if (out->ptype != PG_PTYPE_U8) return fail(PG_ERR_INCOMPATIBLE, std::string(what) + " output must be uint8");
  if (overlaps(*in, *out)) return fail(PG_ERR_ALIASING, std::string(what) + " input output images must be different");
  return PG_OK;
}

pg_status pg_h_maxima_binary(const pg_image *in, const pg_scalar *h, int32_t se, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_binary_out(in, out, "h_maxima_binary"));
  PG_TRY(check_scalar(in->ptype, h, "h_maxima_binary"));
  ReconRequest rq;
  PG_TRY(recon_se(se, in->rank, rq.conn8));
  rq.dilate = true;
  rq.init = INIT_SAT_CONST;
  rq.epi = EPI_BINARY_SUP;
  rq.h = *h;
  return launch_reconstruction(nullptr, in, out, 1, rq, STREAM(s));
}

pg_status pg_h_maxima_binary_batch(const pg_image *ins, const pg_image *outs, int32_t n, const pg_scalar *h, int32_t se,
                                   pg_stream_t s) {
  if (n < 0 || (n > 0 && (!ins || !outs))) return fail(PG_ERR_INVALID_ARGUMENT, "h_maxima_binary_batch: bad image arrays");
  if (n == 0) return PG_OK;
  for (int i = 0; i < n; ++i) {
    PG_TRY(check_binary_out(&ins[i], &outs[i], "h_maxima_binary_batch"));
    if (ins[i].ptype != ins[0].ptype || ins[i].rank != ins[0].rank)
      return fail(PG_ERR_INCOMPATIBLE, "h_maxima_binary_batch: all images must share pixel type and rank");
  }
  PG_TRY(check_scalar(ins[0].ptype, h, "h_maxima_binary_batch"));
  ReconRequest rq;
  PG_TRY(recon_se(se, ins[0].rank, rq.conn8));
  rq.dilate = true;
  rq.init = INIT_SAT_CONST;
  rq.epi = EPI_BINARY_SUP;
  rq.h = *h;
  return launch_reconstruction(nullptr, ins, outs, n, rq, STREAM(s));
}

pg_status pg_h_maxima_binary_batch_plan(const pg_image *ins, const pg_image *outs, int32_t n, const pg_scalar *h, int32_t se,
                                        int32_t autotune, pg_batch_plan **plan, pg_stream_t s) {
  if (!plan) return fail(PG_ERR_INVALID_ARGUMENT, "null plan pointer");
  *plan = nullptr;
  if (n < 1 || !ins || !outs) return fail(PG_ERR_INVALID_ARGUMENT, "h_maxima_binary_batch_plan: bad image arrays");
  for (int i = 0; i < n; ++i) {
    PG_TRY(check_binary_out(&ins[i], &outs[i], "h_maxima_binary_batch_plan"));
    if (ins[i].ptype != ins[0].ptype || ins[i].rank != ins[0].rank)
      return fail(PG_ERR_INCOMPATIBLE, "h_maxima_binary_batch_plan: all images must share pixel type and rank");
    if (dims_of(ins[i]).count() == 0) return fail(PG_ERR_INVALID_ARGUMENT, "h_maxima_binary_batch_plan: empty image");
  }
  PG_TRY(check_scalar(ins[0].ptype, h, "h_maxima_binary_batch_plan"));
  if (ins[0].rank == 3) return fail(PG_ERR_INVALID_ARGUMENT, "h_maxima_binary_batch_plan: images of rank 1 or 2");
  bool conn8 = true;
  PG_TRY(recon_se(se, ins[0].rank, conn8));
  return create_batch_plan(ins, outs, n, *h, conn8, autotune != 0, STREAM(s), plan);
}
pg_status pg_batch_plan_run(pg_batch_plan *plan, pg_stream_t s) {
  if (!plan) return fail(PG_ERR_INVALID_ARGUMENT, "null plan");
  return run_batch_plan(plan, STREAM(s));
}
pg_status pg_batch_plan_destroy(pg_batch_plan *plan) {
  destroy_batch_plan(plan);
  return PG_OK;
}

static pg_status leveling_half(const pg_image *ref, const pg_image *marker, int se, const pg_image *out, bool low,
                               cudaStream_t s) {
  ReconRequest rq;
  PG_TRY(recon_se(se, ref->rank, rq.conn8));
  rq.dilate = low;
  rq.init = INIT_MARKER;
  rq.mask_mode = low ? MASK_MAX_MARKER : MASK_MIN_MARKER;
  rq.epi = EPI_CLIP_REF;
  return launch_reconstruction(marker, ref, out, 1, rq, s);
}
static pg_status check_leveling(const pg_image *ref, const pg_image *marker, const pg_image *out, const char *what) {
  PG_TRY(check_in_out(ref, out, what));
  PG_TRY(check_in_out(marker, out, what));
  return PG_OK;
}
pg_status pg_low_leveling(const pg_image *ref, const pg_image *marker, int32_t se, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_leveling(ref, marker, out, "low_leveling"));
  return leveling_half(ref, marker, se, out, true, STREAM(s));
}
pg_status pg_high_leveling(const pg_image *ref, const pg_image *marker, int32_t se, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_leveling(ref, marker, out, "high_leveling"));
  return leveling_half(ref, marker, se, out, false, STREAM(s));
}
pg_status pg_leveling(const pg_image *ref, const pg_image *marker, int32_t se, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_leveling(ref, marker, out, "leveling"));
  Scratch tmp;
  PG_TRY(tmp.alloc((size_t)dims_of(*ref).count() * elem_size(ref->ptype), STREAM(s)));
  pg_image t = *ref;
  t.data = tmp.ptr;
  PG_TRY(leveling_half(ref, marker, se, &t, false, STREAM(s)));  // high_leveling(ref, marker)
  return leveling_half(&t, marker, se, out, true, STREAM(s));     // low_leveling(that, marker)
}

// ---------------------------------------------------------------- pixel processing
pg_status pg_sat_sub_constant(const pg_image *in, const pg_scalar *v, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "ArithSaturatedSubConstant"));
  PG_TRY(check_scalar(in->ptype, v, "ArithSaturatedSubConstant"));
  return launch_sat_const(*in, *v, false, *out, STREAM(s));
}
pg_status pg_sat_add_constant(const pg_image *in, const pg_scalar *v, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_in_out(in, out, "ArithSaturatedAddConstant"));
  PG_TRY(check_scalar(in->ptype, v, "ArithSaturatedAddConstant"));
  return launch_sat_const(*in, *v, true, *out, STREAM(s));
}

// ---------------------------------------------------------------- pixel processing
// An output may be exactly one of the inputs (same buffer, same pixel size: every pixel is read
// before it is written, by one thread) but may not overlap one partially.
static bool partial_overlap(const pg_image &a, const pg_image &b) {
  return overlaps(a, b) && !(a.data == b.data && elem_size(a.ptype) == elem_size(b.ptype));
}

// src/pixel_processing/arith.cpp:125-300: AssertSizesCompatible / AssertAsTypesCompatible on every pair
static pg_status pixel_arith(const pg_image *a, const pg_image *b, const pg_image *out, int op, const char *what,
                             cudaStream_t s) {
  PG_TRY(check_image(a, what));
  if (b) PG_TRY(check_image(b, what));
  PG_TRY(check_image(out, what));
  if (!same_geometry(*a, *out) || (b && !same_geometry(*b, *out)))
    return fail(PG_ERR_INCOMPATIBLE, std::string(what) + " images have not compatible sizes");
  if (a->ptype != out->ptype || (b && b->ptype != out->ptype))
    return fail(PG_ERR_INCOMPATIBLE, std::string(what) + " images must have compatible types");
  if (partial_overlap(*a, *out) || (b && partial_overlap(*b, *out)))
    return fail(PG_ERR_ALIASING, std::string(what) + " output overlaps an input partially");
  return launch_pixel_arith(op, *a, b, *out, s);
}

pg_status pg_arith_invert_image(const pg_image *in, const pg_image *out, pg_stream_t s) {
  return pixel_arith(in, nullptr, out, PX_NEG, "ArithInvertImage", STREAM(s));
}
pg_status pg_arith_sup_image(const pg_image *a, const pg_image *b, const pg_image *out, pg_stream_t s) {
  return pixel_arith(a, b, out, PX_SUP, "ArithSupImage", STREAM(s));
}
pg_status pg_arith_inf_image(const pg_image *a, const pg_image *b, const pg_image *out, pg_stream_t s) {
  return pixel_arith(a, b, out, PX_INF, "ArithInfImage", STREAM(s));
}
pg_status pg_sat_add_image(const pg_image *a, const pg_image *b, const pg_image *out, pg_stream_t s) {
  return pixel_arith(a, b, out, PX_SADD, "ArithSaturatedAddImage", STREAM(s));
}
pg_status pg_sat_sub_image(const pg_image *a, const pg_image *b, const pg_image *out, pg_stream_t s) {
  return pixel_arith(a, b, out, PX_SSUB, "ArithSaturatedSubImage", STREAM(s));
}

// src/pixel_processing/compare.cpp:601-1000: sizes of every image compatible with the output; the
// comparand has the input's type, the true / false values the output's (std::get<pType> on a
// scalar, a downcast on an image, both throwing otherwise)
pg_status pg_compare_image(const pg_image *in, int32_t op, const pg_operand *comp, const pg_operand *valtrue,
                           const pg_operand *valfalse, const pg_image *out, pg_stream_t s) {
  const char *what = "CompareImage";
  PG_TRY(check_image(in, what));
  PG_TRY(check_image(out, what));
  if (!same_geometry(*in, *out)) return fail(PG_ERR_INCOMPATIBLE, "CompareImage images have not compatible sizes");
  switch (op) {
    case PG_COMP_EQUAL: case PG_COMP_DIFF: case PG_COMP_SUP: case PG_COMP_SUP_EQUAL: case PG_COMP_INF:
    case PG_COMP_INF_EQUAL: break;
    default: return fail(PG_ERR_INVALID_ARGUMENT, "CompareImage unsupported CompOpType");
  }
  if (!comp || !valtrue || !valfalse) return fail(PG_ERR_INVALID_ARGUMENT, "CompareImage: null operand");
  if (partial_overlap(*in, *out)) return fail(PG_ERR_ALIASING, "CompareImage output overlaps an input partially");
  const pg_operand *src[3] = {comp, valtrue, valfalse};
  static const char *names[3] = {"i_comp", "i_valtrue", "i_valfalse"};
  CompareOperand ops[3];
  for (int k = 0; k < 3; ++k) {
    const int pt = k == 0 ? in->ptype : out->ptype;
    const pg_image *im = src[k]->image;
    if (im) {
      PG_TRY(check_image(im, what));
      if (!same_geometry(*im, *out)) return fail(PG_ERR_INCOMPATIBLE, "CompareImage images have not compatible sizes");
      if (im->ptype != pt) return fail(PG_ERR_INCOMPATIBLE, std::string("CompareImage ") + names[k] + " downcast fail");
      if (partial_overlap(*im, *out)) return fail(PG_ERR_ALIASING, "CompareImage output overlaps an input partially");
      ops[k] = CompareOperand{im->data, pg_scalar{}};
    } else {
      PG_TRY(check_scalar(pt, &src[k]->value,
                          (std::string("CompareImage unable to extract suitable type from ") + names[k]).c_str()));
      ops[k] = CompareOperand{nullptr, src[k]->value};
    }
  }
  return launch_compare(*in, op, ops[0], ops[1], ops[2], *out, STREAM(s));
}

// src/pixel_processing/copy_convert.cpp:59-67, :301-306
pg_status pg_copy_into(const pg_image *in, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_image(in, "CopyInto"));
  PG_TRY(check_image(out, "CopyInto"));
  if (!same_geometry(*in, *out)) return fail(PG_ERR_INCOMPATIBLE, "Copy images have not compatible sizes");
  if (in->ptype != out->ptype) return fail(PG_ERR_INCOMPATIBLE, "Copy images have not compatible types");
  if (in->data == out->data) return PG_OK;
  if (overlaps(*in, *out)) return fail(PG_ERR_ALIASING, "Copy images overlap partially");
  return launch_copy(*in, *out, STREAM(s));
}
pg_status pg_convert_into(const pg_image *in, const pg_image *out, pg_stream_t s) {
  PG_TRY(check_image(in, "ConvertInto"));
  PG_TRY(check_image(out, "ConvertInto"));
  if (!same_geometry(*in, *out)) return fail(PG_ERR_INCOMPATIBLE, "ConvertInto images have not compatible sizes");
  if (overlaps(*in, *out)) return fail(PG_ERR_ALIASING, "ConvertInto images must be differents");
  return launch_convert(*in, *out, STREAM(s));
}

// ---------------------------------------------------------------- adjoint
pg_status pg_flat_morph2d_forward(const float *x, float *y, int64_t planes, int64_t h, int64_t w, int32_t ry,
                                  int32_t rx, int32_t dilate, pg_stream_t s) {
  if (planes < 0 || h < 0 || w < 0) return fail(PG_ERR_INVALID_ARGUMENT, "negative dimension");
  if (planes * h * w > 0 && (!x || !y)) return fail(PG_ERR_INVALID_ARGUMENT, "null tensor");
  if (x == y && x) return fail(PG_ERR_ALIASING, "input output tensors must be different");
  return launch_flat2d(x, y, planes, h, w, ry, rx, dilate != 0, STREAM(s));
}
pg_status pg_flat_morph2d_backward(const float *x, const float *gy, float *gx, int64_t planes, int64_t h, int64_t w,
                                   int32_t ry, int32_t rx, int32_t dilate, pg_stream_t s) {
  if (planes < 0 || h < 0 || w < 0) return fail(PG_ERR_INVALID_ARGUMENT, "negative dimension");
  if (planes * h * w > 0 && (!x || !gy || !gx)) return fail(PG_ERR_INVALID_ARGUMENT, "null tensor");
  if (gx && (gx == x || gx == gy)) return fail(PG_ERR_ALIASING, "grad_in must be a distinct tensor");
  return launch_flat2d_backward(x, gy, gx, planes, h, w, ry, rx, dilate != 0, STREAM(s));
}

pg_status pg_flat_morph2d_forward_arg(const float *x, float *y, uint8_t *code, int64_t planes, int64_t h, int64_t w,
                                      int32_t r, int32_t dilate, pg_stream_t s) {
  if (planes < 0 || h < 0 || w < 0) return fail(PG_ERR_INVALID_ARGUMENT, "negative dimension");
  if (planes * h * w > 0 && (!x || !y || !code)) return fail(PG_ERR_INVALID_ARGUMENT, "null tensor");
  if (x == y && x) return fail(PG_ERR_ALIASING, "input output tensors must be different");
  return launch_flat2d_arg(x, y, code, planes, h, w, r, dilate != 0, STREAM(s));
}
pg_status pg_flat_morph2d_backward_arg(const uint8_t *code, const float *gy, float *gx, int64_t planes, int64_t h,
                                       int64_t w, int32_t r, pg_stream_t s) {
  if (planes < 0 || h < 0 || w < 0) return fail(PG_ERR_INVALID_ARGUMENT, "negative dimension");
  if (planes * h * w > 0 && (!code || !gy || !gx)) return fail(PG_ERR_INVALID_ARGUMENT, "null tensor");
  if (gx && gx == gy) return fail(PG_ERR_ALIASING, "grad_in must be a distinct tensor");
  return launch_flat2d_backward_arg(code, gy, gx, planes, h, w, r, STREAM(s));
}

}  // extern "C"
