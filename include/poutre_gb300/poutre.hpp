// poutre.hpp -- header-only C++ facade with poutre2's signatures over the GB300 C ABI.
//
// Mirrors the reference's public API (include/poutre/low_level_morpho/ero_dil.hpp,
// ero_dil_line.hpp, include/poutre/geodesy/{mreconstruct,extrema,leveling}.hpp): the same
// function names, argument order and meaning, on device images.  A non-OK status from the
// C ABI is thrown as std::runtime_error carrying pg_last_error(), where poutre throws (a scalar of
// the wrong pixel type included: poutre rethrows std::get's bad_variant_access as runtime_error).
// Device-side give-ups of the geodesy kernels are checked after each geodesy call
// (pg_check_device), so those calls are synchronous like the reference's.
//
// Two ways to build it:
//  * Inside poutre2 (define POUTRE_GB300_WITH_POUTRE2, poutre2's include directory on the path):
//    DeviceImage derives from poutre::IInterface (include/poutre/base/image_interface.hpp:39-56),
//    and the facade takes poutre's own types -- poutre::IInterface, se::Common_NL_SE,
//    se::Compound_NL_SE, geo::reconstruction_type, ScalarTypeVariant -- so a poutre2 dispatcher
//    that holds an IInterface& can test is_device_image() and forward it unchanged.
//  * Standalone (default): the same names with local stand-ins for those types (an IInterface
//    with the same virtual functions, the same enum values, a ScalarTypeVariant with the same
//    alternatives plus uint16).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <variant>
#include <vector>

#include "../poutre_gb300.h"

#if defined(POUTRE_GB300_WITH_POUTRE2)
#include <poutre/base/image_interface.hpp>
#include <poutre/base/types.hpp>
#include <poutre/geodesy/mreconstruct.hpp>
#include <poutre/structuring_element/se_types_and_tags.hpp>
#endif

namespace poutre::gb300 {

// Pixel types of device images: poutre::PType's values (include/poutre/base/types.hpp:517-526),
// plus uint16
enum class PType : int32_t {
  PType_Undef = 0,
  PType_GrayUINT8 = PG_PTYPE_U8,
  PType_GrayINT32 = PG_PTYPE_I32,
  PType_F32 = PG_PTYPE_F32,
  PType_GrayINT64 = PG_PTYPE_I64,
  PType_D64 = PG_PTYPE_F64,
  PType_GrayUINT16 = PG_PTYPE_U16
};

#if defined(POUTRE_GB300_WITH_POUTRE2)
using IInterface = ::poutre::IInterface;
using CompoundType = ::poutre::CompoundType;
using ScalarTypeVariant = ::poutre::ScalarTypeVariant;
namespace se {
using ::poutre::se::Common_NL_SE;
using ::poutre::se::Compound_NL_SE;
}  // namespace se
namespace geo {
using ::poutre::geo::reconstruction_type;
}  // namespace geo
// the interface's own pixel-type enum (poutre::PType has no uint16: such images report PType_Undef)
using InterfacePType = ::poutre::PType;
inline InterfacePType interface_ptype(PType p) {
  return p == PType::PType_GrayUINT16 ? ::poutre::PType::PType_Undef : static_cast<::poutre::PType>(p);
}
#else
// poutre::CompoundType (include/poutre/base/types.hpp:503-509)
enum class CompoundType { CompoundType_Undef = 0, CompoundType_Scalar = 1, CompoundType_3Planes = 2, CompoundType_4Planes = 4 };
// poutre::ScalarTypeVariant (types.hpp:529), plus uint16
using ScalarTypeVariant = std::variant<uint8_t, int32_t, int64_t, float, double, uint16_t>;
namespace se {
// poutre::se::Common_NL_SE / Compound_NL_SE (se_types_and_tags.hpp:45-63)
enum class Common_NL_SE : uint8_t {
  Undef, SESegmentX1D, SESquare2D, SECross2D, SESegmentX2D, SESegmentY2D, SESegmentX3D, SESegmentY3D, SESegmentZ3D,
  SECross3D, SESquare3D
};
enum class Compound_NL_SE : uint8_t { Undef, Octagon, Rhombicuboctahedron };
}  // namespace se
namespace geo {
// poutre::geo::reconstruction_type (include/poutre/geodesy/mreconstruct.hpp:28-31)
enum class reconstruction_type : uint8_t { erode, dilate };
}  // namespace geo
using InterfacePType = PType;
inline InterfacePType interface_ptype(PType p) { return p; }
// The role of poutre::IInterface (include/poutre/base/image_interface.hpp:39-56): the same virtual
// functions.
class IInterface {
 public:
  virtual ~IInterface() = default;
  virtual PType GetPType() const = 0;
  virtual CompoundType GetCType() const = 0;
  virtual std::vector<std::size_t> GetShape() const = 0;
  virtual std::size_t GetRank() const = 0;
  virtual std::string str() const = 0;
};
#endif

namespace se {
// runtime neighbour list (neighbor_list_t<Rank>): offsets in reference order, rank ints each
struct NeighborList {
  int rank = 2;
  std::vector<int32_t> offsets;
  int32_t size() const { return (int32_t)(offsets.size() / (size_t)rank); }
};
}  // namespace se

inline void check(pg_status st) {
  if (st != PG_OK) throw std::runtime_error(pg_last_error());
}

inline std::size_t pixel_size(PType p) {
  switch (p) {
    case PType::PType_GrayUINT8: return 1;
    case PType::PType_GrayUINT16: return 2;
    case PType::PType_GrayINT32: case PType::PType_F32: return 4;
    case PType::PType_GrayINT64: case PType::PType_D64: return 8;
    default: throw std::runtime_error("unsupported PTYPE");
  }
}

inline const char *ptype_token(PType p) {
  switch (p) {
    case PType::PType_GrayUINT8: return "GUINT8";
    case PType::PType_GrayUINT16: return "GUINT16";
    case PType::PType_GrayINT32: return "GINT32";
    case PType::PType_GrayINT64: return "GINT64";
    case PType::PType_F32: return "F32";
    case PType::PType_D64: return "D64";
    default: return "UNDEF";
  }
}

// Owning dense device image (image_t<T, Rank> on the GPU): row-major, last dimension fastest.
// It is an IInterface (poutre's own when built inside poutre2), so poutre's dispatchers can take it.
class DeviceImage : public IInterface {
 public:
  DeviceImage(std::vector<std::size_t> dims, PType ptype, cudaStream_t s = nullptr)
      : dims_(std::move(dims)), ptype_(ptype), stream_(s) {
    if (dims_.empty() || dims_.size() > 3) throw std::runtime_error("Unsupported number of dims");
    const std::size_t bytes = count() * pixel_size(ptype_);
    if (bytes && cudaMalloc(&data_, bytes) != cudaSuccess) throw std::runtime_error("device allocation failed");
  }
  DeviceImage(const DeviceImage &) = delete;
  DeviceImage &operator=(const DeviceImage &) = delete;
  DeviceImage(DeviceImage &&o) noexcept : dims_(std::move(o.dims_)), ptype_(o.ptype_), stream_(o.stream_), data_(o.data_) {
    o.data_ = nullptr;
  }
  ~DeviceImage() override {
    if (data_) cudaFree(data_);
  }
  // the IInterface functions
  InterfacePType GetPType() const override { return interface_ptype(ptype_); }
  CompoundType GetCType() const override { return CompoundType::CompoundType_Scalar; }
  std::vector<std::size_t> GetShape() const override { return dims_; }
  std::size_t GetRank() const override { return dims_.size(); }
  std::string str() const override {
    std::ostringstream os;
    os << "DeviceImage Scalar " << ptype_token(ptype_) << " rank " << dims_.size() << " shape";
    for (auto d : dims_) os << ' ' << d;
    return os.str();
  }
  // the device side
  PType GetDevicePType() const { return ptype_; }
  cudaStream_t stream() const { return stream_; }
  void *data() const { return data_; }
  std::size_t count() const {
    std::size_t n = 1;
    for (auto d : dims_) n *= d;
    return n;
  }
  pg_image descriptor() const {
    pg_image d{};
    d.data = data_;
    d.ptype = static_cast<int32_t>(ptype_);
    d.rank = (int32_t)dims_.size();
    for (std::size_t i = 0; i < dims_.size(); ++i) d.shape[i] = (int64_t)dims_[i];
    return d;
  }
  void upload(const void *host) {
    if (cudaMemcpy(data_, host, count() * pixel_size(ptype_), cudaMemcpyHostToDevice) != cudaSuccess)
      throw std::runtime_error("upload failed");
  }
  void download(void *host) const {
    if (cudaStreamSynchronize(stream_) != cudaSuccess ||
        cudaMemcpy(host, data_, count() * pixel_size(ptype_), cudaMemcpyDeviceToHost) != cudaSuccess)
      throw std::runtime_error("download failed");
  }

 private:
  std::vector<std::size_t> dims_;
  PType ptype_;
  cudaStream_t stream_;
  void *data_ = nullptr;
};

// True when an IInterface is a device image: the test a poutre2 dispatcher makes before forwarding.
inline bool is_device_image(const IInterface &img) { return dynamic_cast<const DeviceImage *>(&img) != nullptr; }

// The device image behind an IInterface; throws like poutre's failed downcasts when it is not one.
inline const DeviceImage &device_of(const IInterface &img) {
  if (auto *d = dynamic_cast<const DeviceImage *>(&img)) return *d;
  throw std::runtime_error("downcast fail: the image is not a device image (poutre::gb300::DeviceImage)");
}
inline pg_image desc(const IInterface &img) { return device_of(img).descriptor(); }
inline cudaStream_t stream_of(const IInterface &img) { return device_of(img).stream(); }

// A ScalarTypeVariant as the C ABI's exact tagged scalar (the alternative held decides the type).
inline pg_scalar to_scalar(const ScalarTypeVariant &v) {
  pg_scalar s{};
  std::visit(
      [&s](auto x) {
        using X = std::decay_t<decltype(x)>;
        if constexpr (std::is_same_v<X, uint8_t>) { s.ptype = PG_PTYPE_U8; s.v.u8 = x; }
        else if constexpr (std::is_same_v<X, uint16_t>) { s.ptype = PG_PTYPE_U16; s.v.u16 = x; }
        else if constexpr (std::is_same_v<X, int32_t>) { s.ptype = PG_PTYPE_I32; s.v.i32 = x; }
        else if constexpr (std::is_same_v<X, int64_t>) { s.ptype = PG_PTYPE_I64; s.v.i64 = x; }
        else if constexpr (std::is_same_v<X, float>) { s.ptype = PG_PTYPE_F32; s.v.f32 = x; }
        else { s.ptype = PG_PTYPE_F64; s.v.f64 = static_cast<double>(x); }
      },
      v);
  return s;
}

// The value `v` held as pixel type `p` (as a caller builds pUINT8{20} for a UINT8 image).
inline ScalarTypeVariant PixelValue(PType p, double v) {
  switch (p) {
    case PType::PType_GrayUINT8: return ScalarTypeVariant(static_cast<uint8_t>(v));
    case PType::PType_GrayINT32: return ScalarTypeVariant(static_cast<int32_t>(v));
    case PType::PType_GrayINT64: return ScalarTypeVariant(static_cast<int64_t>(v));
    case PType::PType_F32: return ScalarTypeVariant(static_cast<float>(v));
    case PType::PType_D64: return ScalarTypeVariant(static_cast<double>(v));
#if !defined(POUTRE_GB300_WITH_POUTRE2)
    case PType::PType_GrayUINT16: return ScalarTypeVariant(static_cast<uint16_t>(v));
#endif
    default: throw std::runtime_error("unsupported PTYPE");
  }
}

inline DeviceImage CloneGeometry(const IInterface &i) {
  const DeviceImage &d = device_of(i);
  return DeviceImage(d.GetShape(), d.GetDevicePType(), d.stream());
}

// ---------------------------------------------------------------- low_level_morpho
inline void Erode(const IInterface &i_img, se::Common_NL_SE nl, int iter, IInterface &o_img) {
  pg_image a = desc(i_img), b = desc(o_img);
  check(pg_erode(&a, (int32_t)nl, iter, &b, stream_of(o_img)));
}
inline void Dilate(const IInterface &i_img, se::Common_NL_SE nl, int iter, IInterface &o_img) {
  pg_image a = desc(i_img), b = desc(o_img);
  check(pg_dilate(&a, (int32_t)nl, iter, &b, stream_of(o_img)));
}
inline void Erode(const IInterface &i_img, se::Compound_NL_SE nl, int size, IInterface &o_img) {
  pg_image a = desc(i_img), b = desc(o_img);
  check(pg_erode_compound(&a, (int32_t)nl, size, &b, stream_of(o_img)));
}
inline void Dilate(const IInterface &i_img, se::Compound_NL_SE nl, int size, IInterface &o_img) {
  pg_image a = desc(i_img), b = desc(o_img);
  check(pg_dilate_compound(&a, (int32_t)nl, size, &b, stream_of(o_img)));
}
inline void Erode(const IInterface &i_img, const se::NeighborList &nl, IInterface &o_img) {
  pg_image a = desc(i_img), b = desc(o_img);
  if ((std::size_t)nl.rank != i_img.GetRank()) throw std::runtime_error("Erode Unsupported IStructuringElement type");
  check(pg_erode_nl(&a, nl.offsets.data(), nl.size(), &b, stream_of(o_img)));
}
inline void Dilate(const IInterface &i_img, const se::NeighborList &nl, IInterface &o_img) {
  pg_image a = desc(i_img), b = desc(o_img);
  if ((std::size_t)nl.rank != i_img.GetRank()) throw std::runtime_error("Dilate Unsupported IStructuringElement type");
  check(pg_dilate_nl(&a, nl.offsets.data(), nl.size(), &b, stream_of(o_img)));
}
inline void ErodeX(const IInterface &i, std::ptrdiff_t half, IInterface &o) {
  pg_image a = desc(i), b = desc(o);
  check(pg_erode_x(&a, half, &b, stream_of(o)));
}
inline void DilateX(const IInterface &i, std::ptrdiff_t half, IInterface &o) {
  pg_image a = desc(i), b = desc(o);
  check(pg_dilate_x(&a, half, &b, stream_of(o)));
}
inline void ErodeY(const IInterface &i, std::ptrdiff_t half, IInterface &o) {
  pg_image a = desc(i), b = desc(o);
  check(pg_erode_y(&a, half, &b, stream_of(o)));
}
inline void DilateY(const IInterface &i, std::ptrdiff_t half, IInterface &o) {
  pg_image a = desc(i), b = desc(o);
  check(pg_dilate_y(&a, half, &b, stream_of(o)));
}

// ---------------------------------------------------------------- geodesy
namespace geo {
inline void checked(pg_status st, cudaStream_t s) {
  check(st);
  check(pg_check_device(s));
}
inline void Reconstruction(reconstruction_type t, const IInterface &marker, const IInterface &mask, se::Common_NL_SE nl,
                           IInterface &o) {
  pg_image m = desc(marker), k = desc(mask), b = desc(o);
  checked(pg_reconstruction(t == reconstruction_type::dilate ? PG_RECONSTRUCT_DILATE : PG_RECONSTRUCT_ERODE, &m, &k,
                            (int32_t)nl, &b, stream_of(o)),
          stream_of(o));
}
#define PG_FACADE_EXTREMA(NAME)                                                                      \
  inline void NAME(const IInterface &i, const ScalarTypeVariant &h, se::Common_NL_SE nl, IInterface &o) { \
    pg_image a = desc(i), b = desc(o);                                                               \
    const pg_scalar hv = to_scalar(h);                                                               \
    checked(pg_##NAME(&a, &hv, (int32_t)nl, &b, stream_of(o)), stream_of(o));                        \
  }
PG_FACADE_EXTREMA(h_minima)
PG_FACADE_EXTREMA(h_maxima)
PG_FACADE_EXTREMA(h_concave)
PG_FACADE_EXTREMA(h_convex)
PG_FACADE_EXTREMA(dynamic_pseudo_opening)
PG_FACADE_EXTREMA(dynamic_pseudo_closing)
#undef PG_FACADE_EXTREMA
#define PG_FACADE_LEVELING(NAME)                                                                    \
  inline void NAME(const IInterface &ref, const IInterface &marker, se::Common_NL_SE nl, IInterface &o) { \
    pg_image r = desc(ref), m = desc(marker), b = desc(o);                    \
    checked(pg_##NAME(&r, &m, (int32_t)nl, &b, stream_of(o)), stream_of(o));                           \
  }
PG_FACADE_LEVELING(low_leveling)
PG_FACADE_LEVELING(high_leveling)
PG_FACADE_LEVELING(leveling)
#undef PG_FACADE_LEVELING
}  // namespace geo

// ---------------------------------------------------------------- labelling
namespace label {
// poutre::label::label_binary / label_flat_zones (include/poutre/label/label_binary.hpp,
// label_flat_zones.hpp): o_img is an INT64 image; returns the number of labels (synchronous).
inline std::size_t label_binary(const IInterface &i_img, se::Common_NL_SE nl, IInterface &o_img) {
  pg_image a = desc(i_img), b = desc(o_img);
  int64_t n = 0;
  check(pg_label_binary(&a, (int32_t)nl, &b, &n, stream_of(o_img)));
  check(pg_check_device(stream_of(o_img)));
  return (std::size_t)n;
}
inline std::size_t label_flat_zones(const IInterface &i_img, se::Common_NL_SE nl, IInterface &o_img) {
  pg_image a = desc(i_img), b = desc(o_img);
  int64_t n = 0;
  check(pg_label_flat_zones(&a, (int32_t)nl, &b, &n, stream_of(o_img)));
  check(pg_check_device(stream_of(o_img)));
  return (std::size_t)n;
}
// poutre::label::label_minima / label_maxima (include/poutre/label/label_extrema.hpp)
inline void label_minima(const IInterface &i_img, se::Common_NL_SE nl, IInterface &o_img) {
  pg_image a = desc(i_img), b = desc(o_img);
  check(pg_label_minima(&a, (int32_t)nl, &b, nullptr, stream_of(o_img)));
  check(pg_check_device(stream_of(o_img)));
}
inline void label_maxima(const IInterface &i_img, se::Common_NL_SE nl, IInterface &o_img) {
  pg_image a = desc(i_img), b = desc(o_img);
  check(pg_label_maxima(&a, (int32_t)nl, &b, nullptr, stream_of(o_img)));
  check(pg_check_device(stream_of(o_img)));
}
}  // namespace label

// ---------------------------------------------------------------- pixel processing
// poutre::ArithInvertImage / ArithSupImage / ArithInfImage / ArithSaturatedAddImage /
// ArithSaturatedSubImage / ArithSaturatedAddConstant / ArithSaturatedSubConstant
// (include/poutre/pixel_processing/arith.hpp:31-53)
inline void ArithInvertImage(const IInterface &i_img, IInterface &o_img) {
  pg_image a = desc(i_img), b = desc(o_img);
  check(pg_arith_invert_image(&a, &b, stream_of(o_img)));
}
#define PG_FACADE_ARITH2(NAME, FN)                                                 \
  inline void NAME(const IInterface &i_img1, const IInterface &i_img2, IInterface &o_img) { \
    pg_image a = desc(i_img1), b = desc(i_img2), c = desc(o_img);     \
    check(FN(&a, &b, &c, stream_of(o_img)));                                                  \
  }
PG_FACADE_ARITH2(ArithSupImage, pg_arith_sup_image)
PG_FACADE_ARITH2(ArithInfImage, pg_arith_inf_image)
PG_FACADE_ARITH2(ArithSaturatedAddImage, pg_sat_add_image)
PG_FACADE_ARITH2(ArithSaturatedSubImage, pg_sat_sub_image)
#undef PG_FACADE_ARITH2
inline void ArithSaturatedAddConstant(const IInterface &i_img, const ScalarTypeVariant &pvalue, IInterface &o_img) {
  pg_image a = desc(i_img), b = desc(o_img);
  const pg_scalar v = to_scalar(pvalue);
  check(pg_sat_add_constant(&a, &v, &b, stream_of(o_img)));
}
inline void ArithSaturatedSubConstant(const IInterface &i_img, const ScalarTypeVariant &pvalue, IInterface &o_img) {
  pg_image a = desc(i_img), b = desc(o_img);
  const pg_scalar v = to_scalar(pvalue);
  check(pg_sat_sub_constant(&a, &v, &b, stream_of(o_img)));
}

#if defined(POUTRE_GB300_WITH_POUTRE2)
using CompOpType = ::poutre::CompOpType;
#else
// poutre::CompOpType (include/poutre/base/types.hpp:443-452)
enum class CompOpType : int32_t {
  CompOpUndef = 0,
  CompOpEqual = PG_COMP_EQUAL,
  CompOpDiff = PG_COMP_DIFF,
  CompOpSup = PG_COMP_SUP,
  CompOpSupEqual = PG_COMP_SUP_EQUAL,
  CompOpInf = PG_COMP_INF,
  CompOpInfEqual = PG_COMP_INF_EQUAL
};
#endif

// An operand of CompareImage: an image, or a ScalarTypeVariant (holding the input's pixel type for
// the comparand, the output's for the true / false values).  Converts implicitly from either, so
// the one CompareImage below takes every one of the reference's eight overloads.
class CompareOperand {
 public:
  CompareOperand(const IInterface &img) : img_(&img) {}             // NOLINT(runtime/explicit)
  CompareOperand(const ScalarTypeVariant &v) : v_(to_scalar(v)) {}  // NOLINT(runtime/explicit)
  pg_operand operand(pg_image &storage) const {
    if (!img_) return pg_operand{nullptr, v_};
    storage = desc(*img_);
    return pg_operand{&storage, pg_scalar{}};
  }

 private:
  const IInterface *img_ = nullptr;
  pg_scalar v_{};
};

// poutre::CompareImage(i_img, compOpType, comp, valtrue, valfalse, o_img)
// (include/poutre/pixel_processing/compare.hpp:31-84)
inline void CompareImage(const IInterface &i_img, CompOpType op, const CompareOperand &i_comp,
                         const CompareOperand &i_valtrue, const CompareOperand &i_valfalse, IInterface &o_img) {
  pg_image a = desc(i_img), o = desc(o_img), sc, st, sf;
  const pg_operand c = i_comp.operand(sc), t = i_valtrue.operand(st), f = i_valfalse.operand(sf);
  check(pg_compare_image(&a, (int32_t)op, &c, &t, &f, &o, stream_of(o_img)));
}

// poutre::CopyInto / ConvertInto / Clone (include/poutre/pixel_processing/copy_convert.hpp)
inline void CopyInto(const IInterface &i_img, IInterface &o_img) {
  pg_image a = desc(i_img), b = desc(o_img);
  check(pg_copy_into(&a, &b, stream_of(o_img)));
}
inline void ConvertInto(const IInterface &i_img, IInterface &o_img) {
  pg_image a = desc(i_img), b = desc(o_img);
  check(pg_convert_into(&a, &b, stream_of(o_img)));
}
inline DeviceImage Clone(const IInterface &i_img) {
  DeviceImage o = ::poutre::gb300::CloneGeometry(i_img);
  ::poutre::gb300::CopyInto(i_img, o);  // qualified: poutre::CopyInto is found by argument lookup too
  return o;
}

// ---------------------------------------------------------------- image strings
// "Scalar <GUINT8|GUINT16|GINT32|GINT64|F32|D64> <rank> <d0..> <values..>", as poutre's
// ImageFromString / ImageToString (include/poutre/base/image_interface.hpp:114-122).
namespace detail {
template <typename T> inline void parse_values(std::istringstream &is, std::size_t n, std::vector<unsigned char> &buf) {
  buf.resize(n * sizeof(T));
  T *p = reinterpret_cast<T *>(buf.data());
  for (std::size_t i = 0; i < n; ++i) {
    double v;
    if (!(is >> v)) throw std::runtime_error("ImageFromString: unable to read current pixel");
    p[i] = static_cast<T>(v);
  }
}
template <typename T> inline void print_values(std::ostringstream &os, const std::vector<unsigned char> &buf) {
  const T *p = reinterpret_cast<const T *>(buf.data());
  for (std::size_t i = 0; i < buf.size() / sizeof(T); ++i) {
    if constexpr (sizeof(T) == 1) os << ' ' << static_cast<int>(p[i]);
    else os << ' ' << p[i];
  }
}
}  // namespace detail

inline DeviceImage ImageFromString(const std::string &s, cudaStream_t stream = nullptr) {
  std::istringstream is(s);
  std::string c, t;
  int rank = 0;
  is >> c >> t >> rank;
  if (c != "Scalar" || rank < 1 || rank > 3) throw std::runtime_error("ImageFromString: unsupported image string");
  PType p;
  if (t == "GUINT8") p = PType::PType_GrayUINT8;
  else if (t == "GUINT16") p = PType::PType_GrayUINT16;
  else if (t == "GINT32") p = PType::PType_GrayINT32;
  else if (t == "GINT64") p = PType::PType_GrayINT64;
  else if (t == "F32") p = PType::PType_F32;
  else if (t == "D64") p = PType::PType_D64;
  else throw std::runtime_error("ImageFromString: unsupported PTYPE");
  std::vector<std::size_t> dims((std::size_t)rank);
  std::size_t n = 1;
  for (auto &d : dims) {
    is >> d;
    n *= d;
  }
  std::vector<unsigned char> buf;
  switch (p) {
    case PType::PType_GrayUINT8: detail::parse_values<uint8_t>(is, n, buf); break;
    case PType::PType_GrayUINT16: detail::parse_values<uint16_t>(is, n, buf); break;
    case PType::PType_GrayINT32: detail::parse_values<int32_t>(is, n, buf); break;
    case PType::PType_GrayINT64: detail::parse_values<int64_t>(is, n, buf); break;
    case PType::PType_F32: detail::parse_values<float>(is, n, buf); break;
    default: detail::parse_values<double>(is, n, buf); break;
  }
  DeviceImage img(dims, p, stream);
  img.upload(buf.data());
  return img;
}

inline std::string ImageToString(const DeviceImage &img) {
  std::vector<unsigned char> buf(img.count() * pixel_size(img.GetDevicePType()));
  img.download(buf.data());
  std::ostringstream os;
  os << "Scalar " << ptype_token(img.GetDevicePType()) << ' ' << img.GetRank();
  for (auto d : img.GetShape()) os << ' ' << d;
  switch (img.GetDevicePType()) {
    case PType::PType_GrayUINT8: detail::print_values<uint8_t>(os, buf); break;
    case PType::PType_GrayUINT16: detail::print_values<uint16_t>(os, buf); break;
    case PType::PType_GrayINT32: detail::print_values<int32_t>(os, buf); break;
    case PType::PType_GrayINT64: detail::print_values<int64_t>(os, buf); break;
    case PType::PType_F32: detail::print_values<float>(os, buf); break;
    default: detail::print_values<double>(os, buf); break;
  }
  return os.str();
}

}  // namespace poutre::gb300
