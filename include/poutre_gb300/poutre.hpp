// poutre.hpp -- header-only C++ facade with poutre2's signatures over the GB300 C ABI.
//
// Mirrors the reference's public API (include/poutre/low_level_morpho/ero_dil.hpp,
// ero_dil_line.hpp, include/poutre/geodesy/{mreconstruct,extrema,leveling}.hpp): the same
// function names, argument order and meaning, on device images.  A non-OK status from the
// C ABI is thrown as std::runtime_error carrying pg_last_error(), where poutre throws.
// Device-side give-ups of the geodesy kernels are checked after each geodesy call
// (pg_check_device), so those calls are synchronous like the reference's.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../poutre_gb300.h"

namespace poutre::gb300 {

// poutre::PType (include/poutre/base/types.hpp:517-526), plus uint16
enum class PType : int32_t {
  PType_Undef = 0,
  PType_GrayUINT8 = PG_PTYPE_U8,
  PType_GrayINT32 = PG_PTYPE_I32,
  PType_F32 = PG_PTYPE_F32,
  PType_GrayINT64 = PG_PTYPE_I64,
  PType_D64 = PG_PTYPE_F64,
  PType_GrayUINT16 = PG_PTYPE_U16
};

namespace se {
// poutre::se::Common_NL_SE / Compound_NL_SE (se_types_and_tags.hpp:45-63)
enum class Common_NL_SE : uint8_t {
  Undef, SESegmentX1D, SESquare2D, SECross2D, SESegmentX2D, SESegmentY2D, SESegmentX3D, SESegmentY3D, SESegmentZ3D,
  SECross3D, SESquare3D
};
enum class Compound_NL_SE : uint8_t { Undef, Octagon, Rhombicuboctahedron };
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

// The role of poutre::IInterface for device images.
class IInterface {
 public:
  virtual ~IInterface() = default;
  virtual PType GetPType() const = 0;
  virtual std::vector<std::size_t> GetShape() const = 0;
  virtual std::size_t GetRank() const = 0;
  virtual pg_image descriptor() const = 0;
  virtual cudaStream_t stream() const = 0;
};

// Owning dense device image (image_t<T, Rank> on the GPU): row-major, last dimension fastest.
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
  PType GetPType() const override { return ptype_; }
  std::vector<std::size_t> GetShape() const override { return dims_; }
  std::size_t GetRank() const override { return dims_.size(); }
  cudaStream_t stream() const override { return stream_; }
  void *data() const { return data_; }
  std::size_t count() const {
    std::size_t n = 1;
    for (auto d : dims_) n *= d;
    return n;
  }
  pg_image descriptor() const override {
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

inline DeviceImage CloneGeometry(const IInterface &i) { return DeviceImage(i.GetShape(), i.GetPType(), i.stream()); }

// ---------------------------------------------------------------- low_level_morpho
inline void Erode(const IInterface &i_img, se::Common_NL_SE nl, int iter, IInterface &o_img) {
  pg_image a = i_img.descriptor(), b = o_img.descriptor();
  check(pg_erode(&a, (int32_t)nl, iter, &b, o_img.stream()));
}
inline void Dilate(const IInterface &i_img, se::Common_NL_SE nl, int iter, IInterface &o_img) {
  pg_image a = i_img.descriptor(), b = o_img.descriptor();
  check(pg_dilate(&a, (int32_t)nl, iter, &b, o_img.stream()));
}
inline void Erode(const IInterface &i_img, se::Compound_NL_SE nl, int size, IInterface &o_img) {
  pg_image a = i_img.descriptor(), b = o_img.descriptor();
  check(pg_erode_compound(&a, (int32_t)nl, size, &b, o_img.stream()));
}
inline void Dilate(const IInterface &i_img, se::Compound_NL_SE nl, int size, IInterface &o_img) {
  pg_image a = i_img.descriptor(), b = o_img.descriptor();
  check(pg_dilate_compound(&a, (int32_t)nl, size, &b, o_img.stream()));
}
inline void Erode(const IInterface &i_img, const se::NeighborList &nl, IInterface &o_img) {
  pg_image a = i_img.descriptor(), b = o_img.descriptor();
  if ((std::size_t)nl.rank != i_img.GetRank()) throw std::runtime_error("Erode Unsupported IStructuringElement type");
  check(pg_erode_nl(&a, nl.offsets.data(), nl.size(), &b, o_img.stream()));
}
inline void Dilate(const IInterface &i_img, const se::NeighborList &nl, IInterface &o_img) {
  pg_image a = i_img.descriptor(), b = o_img.descriptor();
  if ((std::size_t)nl.rank != i_img.GetRank()) throw std::runtime_error("Dilate Unsupported IStructuringElement type");
  check(pg_dilate_nl(&a, nl.offsets.data(), nl.size(), &b, o_img.stream()));
}
inline void ErodeX(const IInterface &i, std::ptrdiff_t half, IInterface &o) {
  pg_image a = i.descriptor(), b = o.descriptor();
  check(pg_erode_x(&a, half, &b, o.stream()));
}
inline void DilateX(const IInterface &i, std::ptrdiff_t half, IInterface &o) {
  pg_image a = i.descriptor(), b = o.descriptor();
  check(pg_dilate_x(&a, half, &b, o.stream()));
}
inline void ErodeY(const IInterface &i, std::ptrdiff_t half, IInterface &o) {
  pg_image a = i.descriptor(), b = o.descriptor();
  check(pg_erode_y(&a, half, &b, o.stream()));
}
inline void DilateY(const IInterface &i, std::ptrdiff_t half, IInterface &o) {
  pg_image a = i.descriptor(), b = o.descriptor();
  check(pg_dilate_y(&a, half, &b, o.stream()));
}

// ---------------------------------------------------------------- geodesy
namespace geo {
enum class reconstruction_type : uint8_t { erode, dilate };

inline void checked(pg_status st, cudaStream_t s) {
  check(st);
  check(pg_check_device(s));
}
inline void Reconstruction(reconstruction_type t, const IInterface &marker, const IInterface &mask, se::Common_NL_SE nl,
                           IInterface &o) {
  pg_image m = marker.descriptor(), k = mask.descriptor(), b = o.descriptor();
  checked(pg_reconstruction(t == reconstruction_type::dilate ? PG_RECONSTRUCT_DILATE : PG_RECONSTRUCT_ERODE, &m, &k,
                            (int32_t)nl, &b, o.stream()),
          o.stream());
}
#define PG_FACADE_EXTREMA(NAME)                                                             \
  inline void NAME(const IInterface &i, double h, se::Common_NL_SE nl, IInterface &o) {     \
    pg_image a = i.descriptor(), b = o.descriptor();                                       \
    checked(pg_##NAME(&a, h, (int32_t)nl, &b, o.stream()), o.stream());                    \
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
    pg_image r = ref.descriptor(), m = marker.descriptor(), b = o.descriptor();                    \
    checked(pg_##NAME(&r, &m, (int32_t)nl, &b, o.stream()), o.stream());                           \
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
  pg_image a = i_img.descriptor(), b = o_img.descriptor();
  int64_t n = 0;
  check(pg_label_binary(&a, (int32_t)nl, &b, &n, o_img.stream()));
  check(pg_check_device(o_img.stream()));
  return (std::size_t)n;
}
inline std::size_t label_flat_zones(const IInterface &i_img, se::Common_NL_SE nl, IInterface &o_img) {
  pg_image a = i_img.descriptor(), b = o_img.descriptor();
  int64_t n = 0;
  check(pg_label_flat_zones(&a, (int32_t)nl, &b, &n, o_img.stream()));
  check(pg_check_device(o_img.stream()));
  return (std::size_t)n;
}
// poutre::label::label_minima / label_maxima (include/poutre/label/label_extrema.hpp)
inline void label_minima(const IInterface &i_img, se::Common_NL_SE nl, IInterface &o_img) {
  pg_image a = i_img.descriptor(), b = o_img.descriptor();
  check(pg_label_minima(&a, (int32_t)nl, &b, nullptr, o_img.stream()));
  check(pg_check_device(o_img.stream()));
}
inline void label_maxima(const IInterface &i_img, se::Common_NL_SE nl, IInterface &o_img) {
  pg_image a = i_img.descriptor(), b = o_img.descriptor();
  check(pg_label_maxima(&a, (int32_t)nl, &b, nullptr, o_img.stream()));
  check(pg_check_device(o_img.stream()));
}
}  // namespace label

// ---------------------------------------------------------------- pixel processing
// poutre::ArithInvertImage / ArithSupImage / ArithInfImage / ArithSaturatedAddImage /
// ArithSaturatedSubImage / ArithSaturatedAddConstant / ArithSaturatedSubConstant
// (include/poutre/pixel_processing/arith.hpp:31-53)
inline void ArithInvertImage(const IInterface &i_img, IInterface &o_img) {
  pg_image a = i_img.descriptor(), b = o_img.descriptor();
  check(pg_arith_invert_image(&a, &b, o_img.stream()));
}
#define PG_FACADE_ARITH2(NAME, FN)                                                 \
  inline void NAME(const IInterface &i_img1, const IInterface &i_img2, IInterface &o_img) { \
    pg_image a = i_img1.descriptor(), b = i_img2.descriptor(), c = o_img.descriptor();     \
    check(FN(&a, &b, &c, o_img.stream()));                                                  \
  }
PG_FACADE_ARITH2(ArithSupImage, pg_arith_sup_image)
PG_FACADE_ARITH2(ArithInfImage, pg_arith_inf_image)
PG_FACADE_ARITH2(ArithSaturatedAddImage, pg_sat_add_image)
PG_FACADE_ARITH2(ArithSaturatedSubImage, pg_sat_sub_image)
#undef PG_FACADE_ARITH2
inline void ArithSaturatedAddConstant(const IInterface &i_img, double pvalue, IInterface &o_img) {
  pg_image a = i_img.descriptor(), b = o_img.descriptor();
  check(pg_sat_add_constant(&a, pvalue, &b, o_img.stream()));
}
inline void ArithSaturatedSubConstant(const IInterface &i_img, double pvalue, IInterface &o_img) {
  pg_image a = i_img.descriptor(), b = o_img.descriptor();
  check(pg_sat_sub_constant(&a, pvalue, &b, o_img.stream()));
}

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

// An operand of CompareImage: an image, or a scalar (the role of ScalarTypeVariant; its value must
// be representable in the operand's pixel type).  Converts implicitly from either, so the one
// CompareImage below takes every one of the reference's eight overloads.
class CompareOperand {
 public:
  CompareOperand(const IInterface &img) : img_(&img) {}  // NOLINT(runtime/explicit)
  CompareOperand(double v) : v_(v) {}                    // NOLINT(runtime/explicit)
  pg_operand operand(pg_image &storage) const {
    if (!img_) return pg_operand{nullptr, v_};
    storage = img_->descriptor();
    return pg_operand{&storage, 0.0};
  }

 private:
  const IInterface *img_ = nullptr;
  double v_ = 0.0;
};

// poutre::CompareImage(i_img, compOpType, comp, valtrue, valfalse, o_img)
// (include/poutre/pixel_processing/compare.hpp:31-84)
inline void CompareImage(const IInterface &i_img, CompOpType op, const CompareOperand &i_comp,
                         const CompareOperand &i_valtrue, const CompareOperand &i_valfalse, IInterface &o_img) {
  pg_image a = i_img.descriptor(), o = o_img.descriptor(), sc, st, sf;
  const pg_operand c = i_comp.operand(sc), t = i_valtrue.operand(st), f = i_valfalse.operand(sf);
  check(pg_compare_image(&a, (int32_t)op, &c, &t, &f, &o, o_img.stream()));
}

// poutre::CopyInto / ConvertInto / Clone (include/poutre/pixel_processing/copy_convert.hpp)
inline void CopyInto(const IInterface &i_img, IInterface &o_img) {
  pg_image a = i_img.descriptor(), b = o_img.descriptor();
  check(pg_copy_into(&a, &b, o_img.stream()));
}
inline void ConvertInto(const IInterface &i_img, IInterface &o_img) {
  pg_image a = i_img.descriptor(), b = o_img.descriptor();
  check(pg_convert_into(&a, &b, o_img.stream()));
}
inline DeviceImage Clone(const IInterface &i_img) {
  DeviceImage o = CloneGeometry(i_img);
  CopyInto(i_img, o);
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
  std::vector<unsigned char> buf(img.count() * pixel_size(img.GetPType()));
  img.download(buf.data());
  std::ostringstream os;
  const char *tok = "";
  switch (img.GetPType()) {
    case PType::PType_GrayUINT8: tok = "GUINT8"; break;
    case PType::PType_GrayUINT16: tok = "GUINT16"; break;
    case PType::PType_GrayINT32: tok = "GINT32"; break;
    case PType::PType_GrayINT64: tok = "GINT64"; break;
    case PType::PType_F32: tok = "F32"; break;
    default: tok = "D64"; break;
  }
  os << "Scalar " << tok << ' ' << img.GetRank();
  for (auto d : img.GetShape()) os << ' ' << d;
  switch (img.GetPType()) {
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
