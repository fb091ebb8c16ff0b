// common.cuh -- shared device/host helpers of the GB300 morphology library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cfloat>
#include <climits>
#include <string>
#include <type_traits>

#include "../../include/poutre_gb300.h"

namespace pg {

// ------------------------------------------------------------------ pixel value traits
// Neutral elements: numeric_limits<T>::lowest() for dilation, ::max() for erosion
// (BinOpSup/BinOpInf, low_level_morpho/details/ero_dil_static_se_t.hpp:45-57).
template <typename T> struct Lim;
template <> struct Lim<uint8_t>  { __host__ __device__ static constexpr uint8_t lo() { return 0; }          __host__ __device__ static constexpr uint8_t hi() { return 255; } };
template <> struct Lim<uint16_t> { __host__ __device__ static constexpr uint16_t lo() { return 0; }         __host__ __device__ static constexpr uint16_t hi() { return 65535; } };
template <> struct Lim<int32_t>  { __host__ __device__ static constexpr int32_t lo() { return INT_MIN; }    __host__ __device__ static constexpr int32_t hi() { return INT_MAX; } };
template <> struct Lim<int64_t>  { __host__ __device__ static constexpr int64_t lo() { return LLONG_MIN; }  __host__ __device__ static constexpr int64_t hi() { return LLONG_MAX; } };
template <> struct Lim<float>    { __host__ __device__ static constexpr float lo() { return -FLT_MAX; }     __host__ __device__ static constexpr float hi() { return FLT_MAX; } };
template <> struct Lim<double>   { __host__ __device__ static constexpr double lo() { return -DBL_MAX; }    __host__ __device__ static constexpr double hi() { return DBL_MAX; } };

// read-only cached load for every pixel type (8-byte integers through long long)
// saturating a - v and a + v: integers clamped to the pixel type's range (TypeTraits<T>::min/max,
// xsimd's ssub / sadd), floating point the plain IEEE result
template <typename T>
__host__ __device__ __forceinline__ T sat_sub_c(T a, T v) {
  if constexpr (std::is_integral_v<T>) {
    using Wide = std::conditional_t<(sizeof(T) < 8), long long, __int128>;
    const Wide r = (Wide)a - (Wide)v;
    if (r > (Wide)Lim<T>::hi()) return Lim<T>::hi();
    if (r < (Wide)Lim<T>::lo()) return Lim<T>::lo();
    return (T)r;
  } else {
    return a - v;
  }
}
template <typename T>
__host__ __device__ __forceinline__ T sat_add_c(T a, T v) {
  if constexpr (std::is_integral_v<T>) {
    using Wide = std::conditional_t<(sizeof(T) < 8), long long, __int128>;
    const Wide r = (Wide)a + (Wide)v;
    if (r > (Wide)Lim<T>::hi()) return Lim<T>::hi();
    if (r < (Wide)Lim<T>::lo()) return Lim<T>::lo();
    return (T)r;
  } else {
    return a + v;
  }
}

template <typename T> __device__ __forceinline__ T ldg(const T *p) {
  if constexpr (std::is_same_v<T, int64_t>) return (T)__ldg(reinterpret_cast<const long long *>(p));
  else return __ldg(p);
}

// Supremum (dilation) / infimum (erosion) operator.  On float data min/max use the
// hardware min/max; the reference's own scalar (std::max) and SIMD (xsimd max) paths
// already disagree on which zero they return for (-0, +0), and no NaN is involved.
template <typename T, bool SUP> struct Op {
  __device__ __forceinline__ static T apply(T a, T b) {
    if constexpr (std::is_same_v<T, float>) return SUP ? fmaxf(a, b) : fminf(a, b);
    else if constexpr (std::is_same_v<T, double>) return SUP ? fmax(a, b) : fmin(a, b);
    else return SUP ? (a < b ? b : a) : (b < a ? b : a);
  }
  __host__ __device__ static constexpr T neutral() { return SUP ? Lim<T>::lo() : Lim<T>::hi(); }
};

// ------------------------------------------------------------------ 16-byte packs
// A Pack holds 16 contiguous bytes of pixels in four 32-bit words.  u8 and u16 pixels are
// combined four / two at a time with the SIMD-in-word min/max instructions; wider types
// element by element.  shl(left) = pixels shifted one position right in memory order,
// i.e. element i takes element i-1 and element 0 takes `left`; shr(right) the converse.
template <typename T> struct Pack {
  static constexpr int N = 16 / sizeof(T);
  union { uint4 v; uint32_t w[4]; T e[N]; };
  __device__ __forceinline__ Pack() {}
  __device__ __forceinline__ static Pack load(const T *p) { Pack r; r.v = __ldg(reinterpret_cast<const uint4 *>(p)); return r; }
  __device__ __forceinline__ static Pack load_cg(const T *p) { Pack r; r.v = __ldcg(reinterpret_cast<const uint4 *>(p)); return r; }
  __device__ __forceinline__ void store(T *p) const { *reinterpret_cast<uint4 *>(p) = v; }
  __device__ __forceinline__ static Pack fill(T x) { Pack r; for (int i = 0; i < N; ++i) r.e[i] = x; return r; }
  __device__ __forceinline__ T first() const { return e[0]; }
  __device__ __forceinline__ T last() const { return e[N - 1]; }

  template <bool SUP> __device__ __forceinline__ static Pack op(const Pack &a, const Pack &b) {
    Pack r;
    if constexpr (std::is_same_v<T, uint8_t>) {
      for (int i = 0; i < 4; ++i) r.w[i] = SUP ? __vmaxu4(a.w[i], b.w[i]) : __vminu4(a.w[i], b.w[i]);
    } else if constexpr (std::is_same_v<T, uint16_t>) {
      for (int i = 0; i < 4; ++i) r.w[i] = SUP ? __vmaxu2(a.w[i], b.w[i]) : __vminu2(a.w[i], b.w[i]);
    } else {
      for (int i = 0; i < N; ++i) r.e[i] = Op<T, SUP>::apply(a.e[i], b.e[i]);
    }
    return r;
  }
  __device__ __forceinline__ Pack shl(T left) const {
    Pack r;
    if constexpr (sizeof(T) == 1 || sizeof(T) == 2) {
      constexpr int S = 8 * sizeof(T);
      uint32_t prev = static_cast<uint32_t>(left) << (32 - S);
      for (int i = 0; i < 4; ++i) { r.w[i] = __funnelshift_l(prev, w[i], S); prev = w[i]; }
    } else {
      r.e[0] = left;
      for (int i = 1; i < N; ++i) r.e[i] = e[i - 1];
    }
    return r;
  }
  __device__ __forceinline__ Pack shr(T right) const {
    Pack r;
    if constexpr (sizeof(T) == 1 || sizeof(T) == 2) {
      constexpr int S = 8 * sizeof(T);
      for (int i = 0; i < 4; ++i) {
        uint32_t next = (i < 3) ? w[i + 1] : static_cast<uint32_t>(right);
        r.w[i] = __funnelshift_r(w[i], next, S);
      }
    } else {
      for (int i = 0; i < N - 1; ++i) r.e[i] = e[i + 1];
      r.e[N - 1] = right;
    }
    return r;
  }
};

// ------------------------------------------------------------------ host-side plumbing
void set_error(const std::string &msg);
pg_status fail(pg_status st, const std::string &msg);
pg_status cuda_status(cudaError_t e, const char *what);
int num_sms();
// Argument checks shared by the entry points (capi.cu): `in` -> `out` of one geometry and pixel
// type in distinct buffers; the reconstruction's SE rule (sets conn8: 8-connected / 26 vs 4 / 6).
pg_status check_in_out(const pg_image *in, const pg_image *out, const char *what);
pg_status recon_se(int se, int rank, bool &conn8);

#define PG_CUDA_TRY(expr, what)                                    \
  do {                                                             \
    cudaError_t e_ = (expr);                                       \
    if (e_ != cudaSuccess) return ::pg::cuda_status(e_, what);     \
  } while (0)

#define PG_TRY(expr)                 \
  do {                               \
    pg_status s_ = (expr);           \
    if (s_ != PG_OK) return s_;      \
  } while (0)

// Stream-ordered temporary (cudaMallocAsync / cudaFreeAsync on the call's stream).
// Stream-ordered temporaries come from the device's default memory pool.  By default that pool
// hands its memory back to the driver at every synchronisation, so the next call would map
// fresh pages again; the pool keeps up to kPoolRetainBytes instead (set once per device).
static constexpr uint64_t kPoolRetainBytes = 1ull << 30;
void retain_pool_memory();
// Test hook (pg_debug_fail_allocations): true while injected allocation failures remain; each call
// that returns true uses one up.
bool take_injected_alloc_failure();

struct Scratch {
  void *ptr = nullptr;
  cudaStream_t stream = nullptr;
  Scratch() = default;
  Scratch(const Scratch &) = delete;
  Scratch &operator=(const Scratch &) = delete;
  pg_status alloc(size_t bytes, cudaStream_t s) {
    retain_pool_memory();
    stream = s;
    if (take_injected_alloc_failure())
      return fail(PG_ERR_OUT_OF_MEMORY, "temporary allocation of " + std::to_string(bytes) + " bytes failed (injected)");
    cudaError_t e = cudaMallocAsync(&ptr, bytes ? bytes : 16, s);
    if (e != cudaSuccess) {
      ptr = nullptr;
      (void)cudaGetLastError();
      return fail(PG_ERR_OUT_OF_MEMORY, "temporary allocation of " + std::to_string(bytes) + " bytes failed");
    }
    return PG_OK;
  }
  ~Scratch() {
    if (ptr) cudaFreeAsync(ptr, stream);
  }
  template <typename U> U *as() const { return static_cast<U *>(ptr); }
};

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// The value of a pg_scalar as pixel type T.  The entry points check that the scalar holds T's own
// pg_ptype (check_scalar), so this reads the member that holds the value and converts nothing.
template <typename T> inline T scalar_as(const pg_scalar &s) {
  switch (s.ptype) {
    case PG_PTYPE_U8: return static_cast<T>(s.v.u8);
    case PG_PTYPE_U16: return static_cast<T>(s.v.u16);
    case PG_PTYPE_I32: return static_cast<T>(s.v.i32);
    case PG_PTYPE_I64: return static_cast<T>(s.v.i64);
    case PG_PTYPE_F32: return static_cast<T>(s.v.f32);
    case PG_PTYPE_F64: return static_cast<T>(s.v.f64);
    default: return T(0);
  }
}

// A pg_scalar holding `v` as pixel type `ptype` (for constants the library itself passes, e.g. h = 1).
inline pg_scalar scalar_of(int ptype, int64_t v) {
  pg_scalar s{};
  s.ptype = ptype;
  switch (ptype) {
    case PG_PTYPE_U8: s.v.u8 = (uint8_t)v; break;
    case PG_PTYPE_U16: s.v.u16 = (uint16_t)v; break;
    case PG_PTYPE_I32: s.v.i32 = (int32_t)v; break;
    case PG_PTYPE_I64: s.v.i64 = v; break;
    case PG_PTYPE_F32: s.v.f32 = (float)v; break;
    case PG_PTYPE_F64: s.v.f64 = (double)v; break;
    default: break;
  }
  return s;
}

// Dispatch over pixel types.
#define PG_DISPATCH_PTYPE(pt, T, ...)                                        \
  switch (pt) {                                                              \
    case PG_PTYPE_U8: { using T = uint8_t; __VA_ARGS__; } break;             \
    case PG_PTYPE_U16: { using T = uint16_t; __VA_ARGS__; } break;           \
    case PG_PTYPE_I32: { using T = int32_t; __VA_ARGS__; } break;            \
    case PG_PTYPE_I64: { using T = int64_t; __VA_ARGS__; } break;            \
    case PG_PTYPE_F32: { using T = float; __VA_ARGS__; } break;              \
    case PG_PTYPE_F64: { using T = double; __VA_ARGS__; } break;             \
    default: return ::pg::fail(PG_ERR_UNSUPPORTED_PTYPE, "unsupported PTYPE"); \
  }

inline int elem_size(int pt) {
  switch (pt) {
    case PG_PTYPE_U8: return 1;
    case PG_PTYPE_U16: return 2;
    case PG_PTYPE_I32: case PG_PTYPE_F32: return 4;
    case PG_PTYPE_I64: case PG_PTYPE_F64: return 8;
    default: return 0;
  }
}

// Volume view (nz, ny, nx) of a rank-1..3 image, reference order d0 slowest.
struct Dims {
  int64_t nz = 1, ny = 1, nx = 1;
  int64_t count() const { return nz * ny * nx; }
};
inline Dims dims_of(const pg_image &im) {
  Dims d;
  if (im.rank == 1) { d.nx = im.shape[0]; }
  else if (im.rank == 2) { d.ny = im.shape[0]; d.nx = im.shape[1]; }
  else { d.nz = im.shape[0]; d.ny = im.shape[1]; d.nx = im.shape[2]; }
  return d;
}

// ------------------------------------------------------------------ kernel entry points
// (host launchers, implemented in the .cu files)
pg_status launch_small_se(const pg_image &in, const pg_image &out, int se, bool dilate, cudaStream_t s);
pg_status launch_nl(const pg_image &in, const pg_image &out, const int32_t *offsets, int n, bool dilate, cudaStream_t s);
pg_status launch_line(const pg_image &in, const pg_image &out, int dy, int dx, int64_t half, bool dilate, cudaStream_t s);
bool try_line_stream(const pg_image &in, const pg_image &out, int dy, int dx, int k, bool dilate, cudaStream_t s,
                     pg_status *st);
bool try_line_words(const pg_image &in, const pg_image &out, int dy, int dx, int k, bool dilate, cudaStream_t s,
                    pg_status *st);
// Vertical, 45- and 135-degree segments (dy = 1, dx = 0 / -1 / +1) of 2k+1 pixels through TMA
// parallelogram tiles (diag.cu): k = 7 (not u8), 15, 31; u8, u16, i32 and f32 images with rows of a
// multiple of 16 bytes.  try_segment_open: the opening (closing) by that segment in one pass.
bool try_segment_tile(const pg_image &in, const pg_image &out, int dy, int dx, int k, bool dilate, cudaStream_t s,
                      pg_status *st);
bool try_segment_open(const pg_image &in, const pg_image &out, int dy, int dx, int k, bool opening, cudaStream_t s,
                      pg_status *st);
bool try_segment_gradient(const pg_image &in, const pg_image &out, int dy, int dx, int k, cudaStream_t s,
                          pg_status *st);  // dilation - erosion by that segment in one pass
int take_diag_status();  // device status of the diagonal tile kernel since the last call (0: none)
// The octagon's n = n_cross + n_square passes in one shared-memory tile kernel (octagon.cu): u8 images
// for 5 <= n <= 16, u16 for 3 <= n <= 16, rows of a multiple of 16 bytes.  n_square = 0: the cross
// iterated n times (SECross2D, iter = n).
bool try_octagon_tile(const pg_image &in, const pg_image &out, int n_cross, int n_square, bool dilate, cudaStream_t s,
                      pg_status *st);
int take_oct_status();  // device status of the octagon tile kernel since the last call (0: none)
// 3x3 square / cross and 3-pixel X / Y segments on TMA tiles (small_tile.cu): 2D u8 / u16 images with
// rows of a multiple of 16 bytes.
bool try_small_tile(const pg_image &in, const pg_image &out, int se, bool dilate, cudaStream_t s, pg_status *st);
int take_small_tile_status();  // device status of the small-SE tile kernel since the last call (0: none)
pg_status launch_rect(const pg_image &in, const pg_image &out, int64_t hy, int64_t hx, bool dilate, cudaStream_t s);
// One-pass box (rect.cu): (hy, hx) = (k, k), (0, k) or (k, 0), k in {7, 15, 31}; 2-/4-byte pixels,
// rows of a multiple of 16 bytes.  try_rect_gradient: dilation - erosion in the same pass.
bool rect_fused_ok(const pg_image &in, const pg_image &out, int64_t hy, int64_t hx, bool grad);
bool try_rect_fused(const pg_image &in, const pg_image &out, int64_t hy, int64_t hx, bool dilate, cudaStream_t s,
                    pg_status *st);
bool try_rect_gradient(const pg_image &in, const pg_image &out, int64_t hy, int64_t hx, cudaStream_t s, pg_status *st);
// One-pass opening / closing by an X segment (rect_open.cu): hy = 0, hx = 7, 15, 31.
bool try_rect_open(const pg_image &in, const pg_image &out, int64_t hy, int64_t hx, bool opening, cudaStream_t s,
                   pg_status *st);
int take_open_status();  // device status of the one-pass opening kernel since the last call (0: none)
// connected-component labelling into an int64 image (label.cu); count may be null
pg_status launch_label(const pg_image &in, int se, const pg_image &out, bool flat, int64_t *count, cudaStream_t s);
int take_label_status();
int take_rect_status();  // device status of the fused square kernel since the last call (0: none)
pg_status launch_copy(const pg_image &in, const pg_image &out, cudaStream_t s);
pg_status launch_sub(const pg_image &a, const pg_image &b, const pg_image &out, cudaStream_t s);
pg_status launch_sat_const(const pg_image &in, const pg_scalar &v, bool add, const pg_image &out, cudaStream_t s);
pg_status launch_sat_sub_image(const pg_image &a, const pg_image &b, const pg_image &out, cudaStream_t s);

// pixel.cu: ArithInf/Sup/SaturatedAdd/SaturatedSub/Invert image, CompareImage, ConvertInto
enum PixelOp { PX_INF = 0, PX_SUP = 1, PX_SADD = 2, PX_SSUB = 3, PX_NEG = 4 };
pg_status launch_pixel_arith(int op, const pg_image &a, const pg_image *b, const pg_image &out, cudaStream_t s);
struct CompareOperand {
  const void *data;  // image pixels, or nullptr for the scalar `value`
  pg_scalar value;
};
pg_status launch_compare(const pg_image &in, int op, const CompareOperand &comp, const CompareOperand &vt,
                         const CompareOperand &vf, const pg_image &out, cudaStream_t s);
pg_status launch_convert(const pg_image &in, const pg_image &out, cudaStream_t s);
pg_status launch_dyn_pseudo_marker(const pg_image &f, const pg_image &ext, const pg_scalar &h, bool opening, const pg_image &out,
                                   cudaStream_t s);

// Reconstruction family (recon.cu)
enum ReconInit { INIT_MARKER = 0, INIT_SAT_CONST = 1 };
enum ReconMask { MASK_PLAIN = 0, MASK_MAX_MARKER = 1, MASK_MIN_MARKER = 2 };
enum ReconEpi { EPI_NONE = 0, EPI_CLIP_REF = 1, EPI_BINARY_SUP = 2 };
struct ReconRequest {
  bool dilate = true;     // reconstruction by dilation (else by erosion)
  bool conn8 = true;      // SESquare2D (else SECross2D / SESegmentX1D)
  int init = INIT_MARKER;
  int mask_mode = MASK_PLAIN;
  int epi = EPI_NONE;
  pg_scalar h{};          // INIT_SAT_CONST constant (holds the image's pixel type)
};
pg_status launch_reconstruction(const pg_image *markers, const pg_image *masks, const pg_image *outs, int n_images,
                                const ReconRequest &rq, cudaStream_t s);

// recon3d.cu: the same request for one volume (rank 3, SECross3D)
pg_status launch_reconstruction3d(const pg_image *marker, const pg_image &mask, const pg_image &out,
                                  const ReconRequest &rq, cudaStream_t s);

pg_status create_batch_plan(const pg_image *ins, const pg_image *outs, int n, const pg_scalar &h, bool conn8, bool autotune,
                            cudaStream_t s, pg_batch_plan **out_plan);
pg_status run_batch_plan(pg_batch_plan *p, cudaStream_t s);
void destroy_batch_plan(pg_batch_plan *p);

pg_status launch_flat2d(const float *x, float *y, int64_t planes, int64_t h, int64_t w, int ry, int rx, bool dilate,
                        cudaStream_t s);
pg_status launch_flat2d_backward(const float *x, const float *gy, float *gx, int64_t planes, int64_t h, int64_t w,
                                 int ry, int rx, bool dilate, cudaStream_t s);
pg_status launch_flat2d_arg(const float *x, float *y, unsigned char *code, int64_t planes, int64_t h, int64_t w, int r,
                            bool dilate, cudaStream_t s);
pg_status launch_flat2d_backward_arg(const unsigned char *code, const float *gy, float *gx, int64_t planes, int64_t h,
                                     int64_t w, int r, cudaStream_t s);

}  // namespace pg
