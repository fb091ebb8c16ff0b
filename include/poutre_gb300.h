/*
 * poutre_gb300.h -- C ABI of the GB300 (sm_103a) morphology + geodesy library.
 *
 * This is the drop-in boundary for poutre2's low_level_morpho and geodesy entry points:
 * each function below replaces one reference entry point (cited beside it, paths relative
 * to the poutre2 source tree) with the same argument meaning, on device images.
 *
 * Conventions
 *   - Images are dense, row-major, last dimension fastest, in device memory owned by the
 *     caller (poutre::details::image_t layout, array_view.hpp:908-912).  shape[] holds the
 *     reference's dimensions {d0, .., d_{rank-1}}, d0 slowest.
 *   - ptype values are poutre::PType's (include/poutre/base/types.hpp:517-526); uint16 is
 *     an addition (PG_PTYPE_U16).
 *   - Every call is asynchronous on `stream` (a cudaStream_t; NULL = legacy default
 *     stream) and returns a status; no exception crosses the ABI.  Where the reference
 *     throws std::runtime_error, the call returns the matching status and
 *     pg_last_error() (thread-local) holds the message.
 *   - Outputs must be distinct from inputs (AssertImagesAreDifferent,
 *     src/base/image_interface.cpp:52-56,74-80); sizes and types must match
 *     (AssertSizesCompatible / AssertAsTypesCompatible).
 *   - Temporaries are taken from the device's stream-ordered pool (cudaMallocAsync)
 *     on `stream`, as the reference allocates its own temporaries.
 */
#ifndef POUTRE_GB300_H
#define POUTRE_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(_WIN32)
#define PG_API __declspec(dllexport)
#else
#define PG_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *pg_stream_t; /* == cudaStream_t */

typedef enum pg_status {
  PG_OK = 0,
  PG_ERR_INVALID_ARGUMENT = 1,  /* null pointer, bad rank/shape, negative iter, bad scalar  */
  PG_ERR_UNSUPPORTED_PTYPE = 2, /* "unsupported PTYPE"                                      */
  PG_ERR_UNSUPPORTED_SE = 3,    /* "unsupported nl_static" / SE rank differs from image rank */
  PG_ERR_INCOMPATIBLE = 4,      /* sizes or types of the images differ                      */
  PG_ERR_ALIASING = 5,          /* output is one of the inputs                              */
  PG_ERR_NOT_SQUARE = 6,        /* DilateY/ErodeY on a non-square image (the reference throws) */
  PG_ERR_CUDA = 7,              /* a CUDA runtime error (message in pg_last_error)          */
  PG_ERR_OUT_OF_MEMORY = 8,     /* a temporary could not be allocated                       */
  PG_ERR_NOT_CONVERGED = 9,     /* reconstruction hit its round cap or a device wait limit  */
  PG_ERR_SCALAR_TYPE = 10       /* a pg_scalar does not hold the pixel type the call needs   */
                                /* ("unable to extract suitable type" in the reference)      */
} pg_status;

typedef enum pg_ptype {
  PG_PTYPE_U8 = 4,
  PG_PTYPE_I32 = 8,
  PG_PTYPE_F32 = 16,
  PG_PTYPE_I64 = 32,
  PG_PTYPE_F64 = 64,
  PG_PTYPE_U16 = 128
} pg_ptype;

/* poutre::se::Common_NL_SE, include/poutre/structuring_element/se_types_and_tags.hpp:45-57 */
typedef enum pg_common_se {
  PG_SE_UNDEF = 0,
  PG_SE_SEGMENT_X_1D = 1,
  PG_SE_SQUARE_2D = 2,
  PG_SE_CROSS_2D = 3,
  PG_SE_SEGMENT_X_2D = 4,
  PG_SE_SEGMENT_Y_2D = 5,
  PG_SE_SEGMENT_X_3D = 6,
  PG_SE_SEGMENT_Y_3D = 7,
  PG_SE_SEGMENT_Z_3D = 8,
  PG_SE_CROSS_3D = 9,
  PG_SE_SQUARE_3D = 10
} pg_common_se;

/* poutre::se::Compound_NL_SE, se_types_and_tags.hpp:59-63 */
typedef enum pg_compound_se { PG_COMPOUND_UNDEF = 0, PG_COMPOUND_OCTAGON = 1, PG_COMPOUND_RHOMBICUBOCTAHEDRON = 2 } pg_compound_se;

/* poutre::geo::reconstruction_type, include/poutre/geodesy/mreconstruct.hpp:28-31 */
typedef enum pg_reconstruction_type { PG_RECONSTRUCT_ERODE = 0, PG_RECONSTRUCT_DILATE = 1 } pg_reconstruction_type;

/* A device image (the role of poutre::IInterface / image_t<T,Rank> at the boundary). */
typedef struct pg_image {
  void *data;       /* device pointer, dense row-major                   */
  int32_t ptype;    /* pg_ptype                                          */
  int32_t rank;     /* 1, 2 or 3                                         */
  int64_t shape[3]; /* d0 .. d_{rank-1}; unused entries ignored          */
} pg_image;

/* One pixel value, held exactly: the role of poutre::ScalarTypeVariant
 * (std::variant<pUINT8, pINT32, pINT64, pFLOAT, pDOUBLE>, include/poutre/base/types.hpp:529), plus
 * uint16.  `ptype` names the member that is set.  A call taking a pg_scalar requires it to hold
 * exactly the pixel type the reference's std::get<T> asks for (the image's, src/pixel_processing/
 * arith.cpp:55; the output's for CompareImage's true / false values, compare.cpp:51-61), else it
 * returns PG_ERR_SCALAR_TYPE where the reference's std::get throws std::bad_variant_access, which
 * poutre2 rethrows as std::runtime_error "unable to extract suitable type" (arith.cpp:55-59,
 * compare.cpp:50-62).  Every int64 value
 * crosses the boundary exactly.  Floating-point values must be finite. */
typedef struct pg_scalar {
  int32_t ptype; /* pg_ptype of the member that holds the value */
  int32_t reserved_;
  union {
    uint8_t u8;
    uint16_t u16;
    int32_t i32;
    int64_t i64;
    float f32;
    double f64;
  } v;
} pg_scalar;

/* Structuring element for the composite filters (opening/closing/gradient), which the
 * reference does not have: one of its SE vocabularies, selected by `kind`. */
typedef enum pg_se_kind {
  PG_SE_KIND_STATIC = 0,   /* common_se iterated `iter` times (Erode/Dilate(.., Common_NL_SE, iter, ..)) */
  PG_SE_KIND_RECT = 1,     /* flat (2*hy+1) x (2*hx+1) rectangle = line Y(hy) o line X(hx)              */
  PG_SE_KIND_LINE = 2,     /* segment t*(dy,dx), t in [-half, half]; (0,1) X, (1,0) Y, (-1,1) 45 degrees */
  PG_SE_KIND_NL = 3        /* explicit offset list (neighbor_list_t), host array n x rank               */
} pg_se_kind;

typedef struct pg_se {
  int32_t kind;
  int32_t common_se, iter;           /* PG_SE_KIND_STATIC */
  int32_t hy, hx;                    /* PG_SE_KIND_RECT   */
  int32_t dy, dx, half;              /* PG_SE_KIND_LINE   */
  const int32_t *offsets; int32_t n; /* PG_SE_KIND_NL     */
} pg_se;

PG_API const char *pg_last_error(void);
PG_API const char *pg_version(void);

/* ---------------------------------------------------------------- low_level_morpho */

/* poutre::Erode / poutre::Dilate(const IInterface&, se::Common_NL_SE, int iter, IInterface&)
 * include/poutre/low_level_morpho/ero_dil.hpp:32-35 (src/low_level_morpho/ero_dil_static.cpp:229-306) */
PG_API pg_status pg_erode(const pg_image *in, int32_t common_se, int32_t iter, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_dilate(const pg_image *in, int32_t common_se, int32_t iter, const pg_image *out, pg_stream_t stream);

/* poutre::Erode / Dilate(const IInterface&, se::Compound_NL_SE, int size, IInterface&), ero_dil.hpp:38-41
 * (ero_dil_compound_static_se_t.hpp:34-160) */
PG_API pg_status pg_erode_compound(const pg_image *in, int32_t compound_se, int32_t size, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_dilate_compound(const pg_image *in, int32_t compound_se, int32_t size, const pg_image *out, pg_stream_t stream);

/* poutre::Erode / Dilate(const IInterface&, const se::IStructuringElement&, IInterface&), ero_dil.hpp:44-47
 * with a neighbour list: `offsets` is a HOST array of n offsets of `in->rank` ints each, reference
 * coordinate order (neighbor_list_t<Rank>, neighbor_list_se_t.hpp:36-228). n <= 4096. */
PG_API pg_status pg_erode_nl(const pg_image *in, const int32_t *offsets, int32_t n, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_dilate_nl(const pg_image *in, const int32_t *offsets, int32_t n, const pg_image *out, pg_stream_t stream);

/* poutre::ErodeX / DilateX / ErodeY / DilateY(const IInterface&, ptrdiff_t size_half_segment, IInterface&)
 * include/poutre/low_level_morpho/ero_dil_line.hpp:32-47.  Y requires a square 2D image, as in the reference. */
PG_API pg_status pg_erode_x(const pg_image *in, int64_t half, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_dilate_x(const pg_image *in, int64_t half, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_erode_y(const pg_image *in, int64_t half, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_dilate_y(const pg_image *in, int64_t half, const pg_image *out, pg_stream_t stream);

/* Erosion / dilation / opening / closing / morphological gradient by any pg_se.  No reference
 * counterpart (low_level_morpho.hpp:15 announces them); opening = dilate(erode(.)), closing =
 * erode(dilate(.)), gradient = dilate(.) - erode(.) (plain subtraction). */
PG_API pg_status pg_erode_se(const pg_image *in, const pg_se *se, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_dilate_se(const pg_image *in, const pg_se *se, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_opening(const pg_image *in, const pg_se *se, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_closing(const pg_image *in, const pg_se *se, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_gradient(const pg_image *in, const pg_se *se, const pg_image *out, pg_stream_t stream);

/* ---------------------------------------------------------------- labelling */

/* poutre::label::label_binary(const IInterface&, se::Common_NL_SE, IInterface&) -> size_t,
 * include/poutre/label/label_binary.hpp (src/label/label_binary.cpp); and label_flat_zones,
 * include/poutre/label/label_flat_zones.hpp (src/label/label_flat_zones.cpp).  Connected components
 * numbered 1.. by the raster position of their first pixel, 0 for the background, into `out`, an
 * PG_PTYPE_I64 image of the input's shape.  label_binary: foreground = pixel != 0, and a pixel joins
 * its earlier neighbours that are > 0; label_flat_zones: every pixel, joined to equal neighbours.
 * Neighbourhood: the SE's earlier half (1D/2D SEs, SECross3D and the 3D segments; SESquare3D
 * returns PG_ERR_UNSUPPORTED_SE).  label_binary takes u8, u16, i32, i64 images; label_flat_zones
 * all six types.  When nb_labels is not null the call waits for the stream and writes the label
 * count there (the reference's return value); otherwise it is asynchronous. */
PG_API pg_status pg_label_binary(const pg_image *in, int32_t common_se, const pg_image *out, int64_t *nb_labels,
                                 pg_stream_t stream);
PG_API pg_status pg_label_flat_zones(const pg_image *in, int32_t common_se, const pg_image *out,
                                     int64_t *nb_labels, pg_stream_t stream);

/* poutre::label::label_minima / label_maxima(const IInterface&, se::Common_NL_SE, IInterface&),
 * include/poutre/label/label_extrema.hpp (src/label/label_extrema.cpp): the regional minima /
 * maxima, labelled: label_binary of h_concave(f, 1) / h_convex(f, 1).  Integer images; SESegmentX1D,
 * SESquare2D, SECross2D, SECross3D; output and nb_labels as label_binary. */
PG_API pg_status pg_label_minima(const pg_image *in, int32_t common_se, const pg_image *out, int64_t *nb_labels,
                                 pg_stream_t stream);
PG_API pg_status pg_label_maxima(const pg_image *in, int32_t common_se, const pg_image *out, int64_t *nb_labels,
                                 pg_stream_t stream);

/* ---------------------------------------------------------------- geodesy */

/* poutre::geo::Reconstruction(reconstruction_type, const IInterface& marker, const IInterface& mask,
 * se::Common_NL_SE, IInterface&), include/poutre/geodesy/mreconstruct.hpp:37-41.
 * 1D (SESegmentX1D), 2D (SESquare2D, SECross2D) and 3D (SECross3D) SEs; pixel types u8,
 * u16, i32, i64, f32, f64.  Volumes iterate the geodesic step (extremum over the SE clamped to the
 * mask) to its fixpoint, one launch per step, the host reading a change flag every 8 steps; the
 * h-extrema, dynamic pseudo filters, leveling and binary h-maxima of volumes take the same route.
 * SESquare3D is refused (PG_ERR_UNSUPPORTED_SE): poutre2's schedule stops short of the fixpoint for
 * it on thin volumes, so no GPU result could match it. */
PG_API pg_status pg_reconstruction(int32_t type, const pg_image *marker, const pg_image *mask, int32_t common_se,
                            const pg_image *out, pg_stream_t stream);

/* poutre::geo::h_minima / h_maxima / h_concave / h_convex / dynamic_pseudo_opening /
 * dynamic_pseudo_closing(const IInterface&, const ScalarTypeVariant& h, se::Common_NL_SE, IInterface&),
 * include/poutre/geodesy/extrema.hpp:33-64.  `h` must hold the image's pixel type, as the reference's
 * ScalarTypeVariant must (src/pixel_processing/arith.cpp:55); else PG_ERR_SCALAR_TYPE. */
PG_API pg_status pg_h_minima(const pg_image *in, const pg_scalar *h, int32_t common_se, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_h_maxima(const pg_image *in, const pg_scalar *h, int32_t common_se, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_h_concave(const pg_image *in, const pg_scalar *h, int32_t common_se, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_h_convex(const pg_image *in, const pg_scalar *h, int32_t common_se, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_dynamic_pseudo_opening(const pg_image *in, const pg_scalar *h, int32_t common_se, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_dynamic_pseudo_closing(const pg_image *in, const pg_scalar *h, int32_t common_se, const pg_image *out, pg_stream_t stream);

/* Binary regional maxima of the h-maxima transform, one fused launch: out(u8) = 255 where
 * in > h_maxima(in) else 0, i.e. h_maxima followed by CompareImage(in, CompOpSup, rec, 255, 0)
 * (include/poutre/pixel_processing/compare.hpp:69). `out` is a u8 image of in's shape. */
PG_API pg_status pg_h_maxima_binary(const pg_image *in, const pg_scalar *h, int32_t common_se, const pg_image *out, pg_stream_t stream);

/* Ragged batch of the binary h-maxima: n independent 2D images of any sizes in ONE persistent
 * launch (tile table over all images).  ins[i]/outs[i] are device images (outs u8); volumes are
 * taken one after the other by the 3D route of pg_reconstruction. */
PG_API pg_status pg_h_maxima_binary_batch(const pg_image *ins, const pg_image *outs, int32_t n, const pg_scalar *h,
                                          int32_t common_se,
                                   pg_stream_t stream);

/* A prepared ragged batch of the binary h-maxima (no reference counterpart): the image and tile
 * tables, the worklist and the reconstruction buffers stay on the device, so a run is one
 * memset plus one persistent cooperative launch, both of which can be captured in a CUDA graph.
 * With autotune != 0 the plan times tile side (32: register tiles, a warp per tile; 64: shared-
 * memory tiles, a 64-thread CTA per tile) x sweep sets per tile visit (2, 4, 16, unbounded) on this
 * batch and keeps the fastest; the choice is cached per (pixel type, connectivity, batch size
 * class).  Without autotune the configuration is 32 / unbounded.  Images of rank 1 or 2.  Inputs/outputs must stay valid
 * while the plan is used.  Plan creation synchronises the device.
 * pg_batch_plan_set_config pins the configuration: tile 32 or 64 (64 only for pixels of at most
 * 4 bytes), sweeps >= 1 (a tile that reaches the cap yields and is revisited next round). */
typedef struct pg_batch_plan pg_batch_plan;
PG_API pg_status pg_h_maxima_binary_batch_plan(const pg_image *ins, const pg_image *outs, int32_t n, const pg_scalar *h,
                                               int32_t common_se, int32_t autotune, pg_batch_plan **plan,
                                               pg_stream_t stream);
PG_API pg_status pg_batch_plan_run(pg_batch_plan *plan, pg_stream_t stream);
PG_API pg_status pg_batch_plan_config(const pg_batch_plan *plan, int32_t *tile, int32_t *sweeps, int32_t *grid);
PG_API pg_status pg_batch_plan_set_config(pg_batch_plan *plan, int32_t tile, int32_t sweeps);
PG_API pg_status pg_batch_plan_destroy(pg_batch_plan *plan);

/* poutre::geo::low_leveling / high_leveling / leveling(const IInterface& ref, const IInterface& marker,
 * se::Common_NL_SE, IInterface&), include/poutre/geodesy/leveling.hpp:37-52. */
PG_API pg_status pg_low_leveling(const pg_image *ref, const pg_image *marker, int32_t common_se, const pg_image *out,
                          pg_stream_t stream);
PG_API pg_status pg_high_leveling(const pg_image *ref, const pg_image *marker, int32_t common_se, const pg_image *out,
                           pg_stream_t stream);
PG_API pg_status pg_leveling(const pg_image *ref, const pg_image *marker, int32_t common_se, const pg_image *out,
                      pg_stream_t stream);

/* ---------------------------------------------------------------- pixel_processing subset */

/* poutre::ArithSaturatedSubConstant / ArithSaturatedAddConstant (src/pixel_processing/arith.cpp:471):
 * integers clamp to the pixel type's range, floating point is the plain IEEE result (as for the
 * saturated image arithmetic below); `v` must hold the image's pixel type (PG_ERR_SCALAR_TYPE). */
PG_API pg_status pg_sat_sub_constant(const pg_image *in, const pg_scalar *v, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_sat_add_constant(const pg_image *in, const pg_scalar *v, const pg_image *out, pg_stream_t stream);

/* ---------------------------------------------------------------- pixel processing */
/* poutre::CompOpType (include/poutre/base/types.hpp:443-452), same values. */
typedef enum {
  PG_COMP_EQUAL = 1,     /* p1 == p2 */
  PG_COMP_DIFF = 2,      /* p1 != p2 */
  PG_COMP_SUP = 4,       /* p1 >  p2 */
  PG_COMP_SUP_EQUAL = 8, /* p1 >= p2 */
  PG_COMP_INF = 16,      /* p1 <  p2 */
  PG_COMP_INF_EQUAL = 32 /* p1 <= p2 */
} pg_comp_op;

/* One operand of CompareImage: an image of the input's geometry (image != NULL) or the scalar
 * `value` (the reference's ScalarTypeVariant): the comparand holds the input's pixel type, the
 * true / false values the output's (compare.cpp:51-61), else PG_ERR_SCALAR_TYPE. */
typedef struct {
  const pg_image *image;
  pg_scalar value;
} pg_operand;

/* poutre::ArithInvertImage / ArithSupImage / ArithInfImage / ArithSaturatedAddImage /
 * ArithSaturatedSubImage (include/poutre/pixel_processing/arith.hpp:31-53): images of one type
 * and geometry; the output may be one of the inputs (in place), not a partial overlap.  Invert is
 * -v in the pixel type (wrapping for unsigned pixels); inf / sup are v1 < v2 ? v1 : v2 and
 * v1 > v2 ? v1 : v2; the saturated sum / difference clamps integers to the type's range and is the
 * plain IEEE result for floating point, as the reference's vector body computes it (its scalar
 * remainder loop raises differences below TypeTraits<float>::min() = FLT_MIN, the smallest positive
 * normal, to FLT_MIN and lowers sums above FLT_MAX to FLT_MAX, so on float images the reference's
 * last n mod SIMD-width pixels can differ from its others). */
PG_API pg_status pg_arith_invert_image(const pg_image *in, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_arith_sup_image(const pg_image *in1, const pg_image *in2, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_arith_inf_image(const pg_image *in1, const pg_image *in2, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_sat_add_image(const pg_image *in1, const pg_image *in2, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_sat_sub_image(const pg_image *in1, const pg_image *in2, const pg_image *out, pg_stream_t stream);

/* poutre::CompareImage(i_img, CompOpType, comp, valtrue, valfalse, o_img), all eight overloads
 * (include/poutre/pixel_processing/compare.hpp:31-84): out = op(in, comp) ? valtrue : valfalse per
 * pixel.  comp has the input's pixel type, valtrue / valfalse and out the output's (which may
 * differ from the input's); every image operand has the input's geometry. */
PG_API pg_status pg_compare_image(const pg_image *in, int32_t op, const pg_operand *comp, const pg_operand *valtrue,
                                  const pg_operand *valfalse, const pg_image *out, pg_stream_t stream);

/* poutre::CopyInto (same type and geometry) and poutre::ConvertInto (any two pixel types:
 * static_cast per pixel, defined for values the output type holds; distinct images)
 * (include/poutre/pixel_processing/copy_convert.hpp, src/pixel_processing/copy_convert.cpp:59,301). */
PG_API pg_status pg_copy_into(const pg_image *in, const pg_image *out, pg_stream_t stream);
PG_API pg_status pg_convert_into(const pg_image *in, const pg_image *out, pg_stream_t stream);

/* ---------------------------------------------------------------- flat morphology adjoint (float32) */

/* Flat dilation (dilate != 0) or erosion by a (2*ry+1) x (2*rx+1) rectangle of `planes` stacked
 * h x w float32 planes (an NCHW tensor with planes = N*C), and its adjoint: grad_in[q] is the sum,
 * in raster order of the outputs, of grad_out[p] over every output p whose first-in-scan-order
 * (dy-major, then dx) arg-extremum within its clipped window is q.  Deterministic (gather, no
 * atomics).  No reference counterpart.  ry, rx <= 7. */
PG_API pg_status pg_flat_morph2d_forward(const float *x, float *y, int64_t planes, int64_t h, int64_t w, int32_t ry,
                                  int32_t rx, int32_t dilate, pg_stream_t stream);
PG_API pg_status pg_flat_morph2d_backward(const float *x, const float *grad_out, float *grad_in, int64_t planes, int64_t h,
                                   int64_t w, int32_t ry, int32_t rx, int32_t dilate, pg_stream_t stream);

/* The same forward and adjoint for a square (2r+1) x (2r+1) window, r = 1..3, with the arg saved
 * instead of recomputed: the forward also writes code[p] = a*(2r+1) + b (one byte per pixel), the
 * window row a and column b of p's first-in-scan-order arg-extremum; the backward gathers from the
 * codes and grad_out alone.  y is bit-identical to pg_flat_morph2d_forward; grad_in to
 * pg_flat_morph2d_backward for every x without NaN. */
PG_API pg_status pg_flat_morph2d_forward_arg(const float *x, float *y, uint8_t *code, int64_t planes, int64_t h,
                                             int64_t w, int32_t r, int32_t dilate, pg_stream_t stream);
PG_API pg_status pg_flat_morph2d_backward_arg(const uint8_t *code, const float *grad_out, float *grad_in, int64_t planes,
                                              int64_t h, int64_t w, int32_t r, pg_stream_t stream);

/* Size of the fixed device scratch of pg_reconstruction_noalloc (1 MiB). */
#define PG_NOALLOC_SCRATCH_BYTES (1u << 20)

/* Geodesic reconstruction that allocates no device memory.  No counterpart in the reference:
 * it exists for callers that cannot allocate -- e.g. a real-time imaging pipeline that
 * reserves all of its device memory up front and forbids cudaMalloc in steady state (an
 * allocation may synchronise the device or fail under memory pressure), or a host that gives
 * this library a fixed memory budget.  Same arguments, checks (in the same order) and result
 * as pg_reconstruction, for 1D and 2D images; a volume is refused with PG_ERR_UNSUPPORTED_SE.
 * The caller still provides marker, mask and output.
 * Its scratch (control block + tile worklist) is a 1 MiB file-scope device array that every
 * GPU loading the library holds until exit, so the image may span at most 131040 tiles
 * (64x64 pixels; 32x32 for 8-byte pixels) -- about 536 Mpixel for 1..4-byte pixels, 134 Mpixel
 * for 8-byte pixels -- and larger images are rejected with PG_ERR_INVALID_ARGUMENT.  All calls
 * share that array: calls that overlap on the GPU (other streams, other threads) race and must
 * be serialised by the caller.  The first call on a device looks the array's address up and
 * keeps it; make that call before any stream capture, and do not call this entry point again
 * on a device after cudaDeviceReset.  Device-side failure is reported by pg_check_device, as
 * for the others. */
PG_API pg_status pg_reconstruction_noalloc(int32_t type, const pg_image *marker, const pg_image *mask,
                                           int32_t common_se, const pg_image *out, pg_stream_t stream);

/* Synchronises `stream`, then returns (and clears) the device-side status of the kernels:
 * PG_ERR_NOT_CONVERGED when a reconstruction gave up (round cap or a bounded device wait), or
 * PG_ERR_CUDA when a shared-memory tile kernel (box erosion / dilation, gradient, opening) found a
 * tile load unfinished after its bounded wait or a labelling union-find loop hit its iteration
 * bound, since the last check; else PG_OK.  The calls are asynchronous; call this to
 * observe the failure the reference would have thrown. */
PG_API pg_status pg_check_device(pg_stream_t stream);

/* Test hooks (no counterpart in the reference), for tests of the failure paths without a GPU fault.
 * pg_debug_set_limits: max_rounds > 0 caps the reconstruction's rounds (round kernel) or visits per
 * tile (worklist kernel), wait_ns > 0 sets the limit of every bounded device wait of the
 * reconstruction kernels launched afterwards (default 4 s); a run that reaches either gives up and
 * pg_check_device returns PG_ERR_NOT_CONVERGED.  0 restores the default.  Process-wide.
 * pg_debug_fail_allocations: the next n temporary allocations fail (PG_ERR_OUT_OF_MEMORY). */
PG_API pg_status pg_debug_set_limits(int32_t max_rounds, int64_t wait_ns);
PG_API pg_status pg_debug_fail_allocations(int32_t n);

/* Passes of the last completed reconstruction on the current device (diagnostics; synchronises
 * the device): for the shared-memory tile kernel the rounds of tile visits, for the worklist kernel
 * (pixels of at most 4 bytes) the tile visits divided by the number of tiles, rounded up. */
PG_API int32_t pg_last_reconstruction_rounds(void);

#ifdef __cplusplus
}
#endif

#endif /* POUTRE_GB300_H */
