// ref_harness.cpp -- extern "C" shims over poutre2's OWN public API, compiled together
// with poutre2's sources into oracle/_ref/libpoutre_ref.so by oracle/ref/build_ref.py.
//
// TEST INFRASTRUCTURE ONLY (the checker and the CPU baseline).  Each shim copies plain
// buffers into poutre::details::image_t objects, calls the reference entry point named in
// its comment through the IInterface API, and copies the result back.  Exceptions thrown
// by the reference become a negative return code; the message is kept for ref_last_error().
#include <poutre/base/details/data_structures/image_t.hpp>
#include <poutre/base/image_interface.hpp>
#include <poutre/base/types.hpp>
#include <poutre/geodesy/extrema.hpp>
#include <poutre/geodesy/leveling.hpp>
#include <poutre/geodesy/mreconstruct.hpp>
#include <poutre/label/label_binary.hpp>
#include <poutre/label/label_extrema.hpp>
#include <poutre/label/label_flat_zones.hpp>
#include <poutre/low_level_morpho/ero_dil.hpp>
#include <poutre/low_level_morpho/ero_dil_line.hpp>
#include <poutre/pixel_processing/arith.hpp>
#include <poutre/pixel_processing/compare.hpp>
#include <poutre/pixel_processing/copy_convert.hpp>
#include <poutre/structuring_element/details/neighbor_list_se_t.hpp>

#include <cstdint>
#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <vector>

namespace {
thread_local std::string g_err;

std::vector<std::size_t> dims_of(int rank, const int64_t *shape) {
  std::vector<std::size_t> d;
  for (int i = 0; i < rank; ++i) d.push_back(static_cast<std::size_t>(shape[i]));
  return d;
}

std::size_t count_of(int rank, const int64_t *shape) {
  std::size_t n = 1;
  for (int i = 0; i < rank; ++i) n *= static_cast<std::size_t>(shape[i]);
  return n;
}

std::size_t elem_size(int pt) {
  switch (pt) {
    case 4: return 1;
    case 8: return 4;
    case 16: return 4;
    case 32: return 8;
    case 64: return 8;
    default: return 0;
  }
}

// raw pointer of an image created by poutre::Create
template <class T, std::ptrdiff_t R>
void *raw_t(poutre::IInterface &img) {
  auto *p = dynamic_cast<poutre::details::image_t<T, R> *>(&img);
  if (!p) throw std::runtime_error("harness: downcast failed");
  return p->data();
}

template <std::ptrdiff_t R>
void *raw_r(poutre::IInterface &img) {
  switch (img.GetPType()) {
    case poutre::PType::PType_GrayUINT8: return raw_t<poutre::pUINT8, R>(img);
    case poutre::PType::PType_GrayINT32: return raw_t<poutre::pINT32, R>(img);
    case poutre::PType::PType_GrayINT64: return raw_t<poutre::pINT64, R>(img);
    case poutre::PType::PType_F32: return raw_t<poutre::pFLOAT, R>(img);
    case poutre::PType::PType_D64: return raw_t<poutre::pDOUBLE, R>(img);
    default: throw std::runtime_error("harness: ptype");
  }
}

void *raw(poutre::IInterface &img) {
  switch (img.GetRank()) {
    case 1: return raw_r<1>(img);
    case 2: return raw_r<2>(img);
    case 3: return raw_r<3>(img);
    default: throw std::runtime_error("harness: rank");
  }
}

std::unique_ptr<poutre::IInterface> make(int pt, int rank, const int64_t *shape, const void *src) {
  auto img = poutre::Create(dims_of(rank, shape), poutre::CompoundType::CompoundType_Scalar,
                            static_cast<poutre::PType>(pt));
  if (src) std::memcpy(raw(*img), src, count_of(rank, shape) * elem_size(pt));
  return img;
}

void take(poutre::IInterface &img, int pt, int rank, const int64_t *shape, void *dst) {
  std::memcpy(dst, raw(img), count_of(rank, shape) * elem_size(pt));
}

poutre::ScalarTypeVariant scalar_of(int pt, double v) {
  switch (pt) {
    case 4: return static_cast<poutre::pUINT8>(v);
    case 8: return static_cast<poutre::pINT32>(v);
    case 32: return static_cast<poutre::pINT64>(v);
    case 16: return static_cast<poutre::pFLOAT>(v);
    case 64: return static_cast<poutre::pDOUBLE>(v);
    default: throw std::runtime_error("harness: ptype");
  }
}

template <class F>
int guarded(F &&f) {
  try {
    f();
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return -1;
  } catch (...) {
    g_err = "unknown exception";
    return -1;
  }
}
}  // namespace

extern "C" {

const char *ref_last_error() { return g_err.c_str(); }

// poutre::Erode / poutre::Dilate (const IInterface&, Common_NL_SE, int iter, IInterface&)
// include/poutre/low_level_morpho/ero_dil.hpp:32-35
int ref_erode_dilate_static(int pt, int rank, const int64_t *shape, const void *in, void *out, int se,
                            int iter, int dilate) {
  return guarded([&] {
    auto a = make(pt, rank, shape, in);
    auto b = make(pt, rank, shape, nullptr);
    auto nl = static_cast<poutre::se::Common_NL_SE>(se);
    if (dilate) poutre::Dilate(*a, nl, iter, *b);
    else poutre::Erode(*a, nl, iter, *b);
    take(*b, pt, rank, shape, out);
  });
}

// poutre::Erode / poutre::Dilate (const IInterface&, Compound_NL_SE, int size, IInterface&)
// include/poutre/low_level_morpho/ero_dil.hpp:38-41
int ref_erode_dilate_compound(int pt, int rank, const int64_t *shape, const void *in, void *out, int cse,
                              int size, int dilate) {
  return guarded([&] {
    auto a = make(pt, rank, shape, in);
    auto b = make(pt, rank, shape, nullptr);
    auto c = static_cast<poutre::se::Compound_NL_SE>(cse);
    if (dilate) poutre::Dilate(*a, c, size, *b);
    else poutre::Erode(*a, c, size, *b);
    take(*b, pt, rank, shape, out);
  });
}

// poutre::Erode / Dilate (const IInterface&, const IStructuringElement&, IInterface&)
// include/poutre/low_level_morpho/ero_dil.hpp:44-47; offs = n x rank ints, reference order.
int ref_erode_dilate_nl(int pt, int rank, const int64_t *shape, const void *in, void *out,
                        const int32_t *offs, int n, int dilate) {
  return guarded([&] {
    auto a = make(pt, rank, shape, in);
    auto b = make(pt, rank, shape, nullptr);
    auto run = [&](const poutre::se::IStructuringElement &s) {
      if (dilate) poutre::Dilate(*a, s, *b);
      else poutre::Erode(*a, s, *b);
    };
    if (rank == 1) {
      std::vector<poutre::details::av::index<1>> v;
      for (int k = 0; k < n; ++k) v.push_back(poutre::details::av::index<1>{offs[k]});
      run(poutre::se::details::neighbor_list_t<1>(v));
    } else if (rank == 2) {
      std::vector<poutre::details::av::index<2>> v;
      for (int k = 0; k < n; ++k) v.push_back(poutre::details::av::index<2>{offs[2 * k], offs[2 * k + 1]});
      run(poutre::se::details::neighbor_list_t<2>(v));
    } else {
      std::vector<poutre::details::av::index<3>> v;
      for (int k = 0; k < n; ++k)
        v.push_back(poutre::details::av::index<3>{offs[3 * k], offs[3 * k + 1], offs[3 * k + 2]});
      run(poutre::se::details::neighbor_list_t<3>(v));
    }
    take(*b, pt, rank, shape, out);
  });
}

// poutre::ErodeX/DilateX/ErodeY/DilateY, include/poutre/low_level_morpho/ero_dil_line.hpp:32-47
int ref_line(int pt, int rank, const int64_t *shape, const void *in, void *out, int64_t half, int axis,
             int dilate) {
  return guarded([&] {
    auto a = make(pt, rank, shape, in);
    auto b = make(pt, rank, shape, nullptr);
    if (axis == 0) {
      if (dilate) poutre::DilateX(*a, half, *b);
      else poutre::ErodeX(*a, half, *b);
    } else {
      if (dilate) poutre::DilateY(*a, half, *b);
      else poutre::ErodeY(*a, half, *b);
    }
    take(*b, pt, rank, shape, out);
  });
}

// poutre::geo::Reconstruction, include/poutre/geodesy/mreconstruct.hpp:37-41
int ref_reconstruct(int pt, int rank, const int64_t *shape, const void *marker, const void *mask, void *out,
                    int se, int dilate) {
  return guarded([&] {
    auto m = make(pt, rank, shape, marker);
    auto k = make(pt, rank, shape, mask);
    auto o = make(pt, rank, shape, nullptr);
    poutre::geo::Reconstruction(dilate ? poutre::geo::reconstruction_type::dilate
                                       : poutre::geo::reconstruction_type::erode,
                                *m, *k, static_cast<poutre::se::Common_NL_SE>(se), *o);
    take(*o, pt, rank, shape, out);
  });
}

// poutre::label::label_binary (flat = 0) / label_flat_zones (flat = 1),
// include/poutre/label/label_binary.hpp, label_flat_zones.hpp: int64 labels into out, count into *n.
int ref_label(int flat, int pt, int rank, const int64_t *shape, const void *in, int64_t *out, int se, int64_t *n) {
  return guarded([&] {
    auto a = make(pt, rank, shape, in);
    auto o = make(32, rank, shape, nullptr);
    auto s = static_cast<poutre::se::Common_NL_SE>(se);
    const std::size_t c = flat ? poutre::label::label_flat_zones(*a, s, *o) : poutre::label::label_binary(*a, s, *o);
    take(*o, 32, rank, shape, out);
    *n = static_cast<int64_t>(c);
  });
}

// poutre::ArithInvertImage (kind 0), ArithSupImage (1), ArithInfImage (2), ArithSaturatedAddImage (3),
// ArithSaturatedSubImage (4), include/poutre/pixel_processing/arith.hpp:31-53
int ref_arith(int kind, int pt, int rank, const int64_t *shape, const void *a, const void *b, void *out) {
  return guarded([&] {
    auto x = make(pt, rank, shape, a);
    auto y = make(pt, rank, shape, b);
    auto o = make(pt, rank, shape, nullptr);
    switch (kind) {
      case 0: poutre::ArithInvertImage(*x, *o); break;
      case 1: poutre::ArithSupImage(*x, *y, *o); break;
      case 2: poutre::ArithInfImage(*x, *y, *o); break;
      case 3: poutre::ArithSaturatedAddImage(*x, *y, *o); break;
      case 4: poutre::ArithSaturatedSubImage(*x, *y, *o); break;
      default: throw std::runtime_error("harness: arith kind");
    }
    take(*o, pt, rank, shape, out);
  });
}

// poutre::CompareImage, the overload chosen per operand: image k when imgs[k] != nullptr, else the
// scalar vals[k] (k = comparand, true value, false value), include/poutre/pixel_processing/compare.hpp:31-84
int ref_compare(int pt_in, int pt_out, int rank, const int64_t *shape, const void *in, int op,
                const void *const *imgs, const double *vals, void *out) {
  return guarded([&] {
    auto x = make(pt_in, rank, shape, in);
    auto o = make(pt_out, rank, shape, nullptr);
    std::unique_ptr<poutre::IInterface> im[3];
    poutre::ScalarTypeVariant sc[3];
    for (int k = 0; k < 3; ++k) {
      const int pt = k == 0 ? pt_in : pt_out;
      if (imgs[k]) im[k] = make(pt, rank, shape, imgs[k]);
      else sc[k] = scalar_of(pt, vals[k]);
    }
    const auto c = static_cast<poutre::CompOpType>(op);
    const int form = (im[0] ? 4 : 0) | (im[1] ? 2 : 0) | (im[2] ? 1 : 0);
    switch (form) {
      case 0: poutre::CompareImage(*x, c, sc[0], sc[1], sc[2], *o); break;
      case 1: poutre::CompareImage(*x, c, sc[0], sc[1], *im[2], *o); break;
      case 2: poutre::CompareImage(*x, c, sc[0], *im[1], sc[2], *o); break;
      case 3: poutre::CompareImage(*x, c, sc[0], *im[1], *im[2], *o); break;
      case 4: poutre::CompareImage(*x, c, *im[0], sc[1], sc[2], *o); break;
      case 5: poutre::CompareImage(*x, c, *im[0], sc[1], *im[2], *o); break;
      case 6: poutre::CompareImage(*x, c, *im[0], *im[1], sc[2], *o); break;
      default: poutre::CompareImage(*x, c, *im[0], *im[1], *im[2], *o); break;
    }
    take(*o, pt_out, rank, shape, out);
  });
}

// poutre::ConvertInto, src/pixel_processing/copy_convert.cpp:301
int ref_convert(int pt_in, int pt_out, int rank, const int64_t *shape, const void *in, void *out) {
  return guarded([&] {
    auto x = make(pt_in, rank, shape, in);
    auto o = make(pt_out, rank, shape, nullptr);
    poutre::ConvertInto(*x, *o);
    take(*o, pt_out, rank, shape, out);
  });
}

// poutre::label::label_minima (maxima = 0) / label_maxima (maxima = 1),
// include/poutre/label/label_extrema.hpp: int64 labels into out (the reference returns no count).
int ref_label_extrema(int maxima, int pt, int rank, const int64_t *shape, const void *in, int64_t *out, int se) {
  return guarded([&] {
    auto a = make(pt, rank, shape, in);
    auto o = make(32, rank, shape, nullptr);
    auto s = static_cast<poutre::se::Common_NL_SE>(se);
    if (maxima) poutre::label::label_maxima(*a, s, *o);
    else poutre::label::label_minima(*a, s, *o);
    take(*o, 32, rank, shape, out);
  });
}

// poutre::geo::h_minima/h_maxima/h_concave/h_convex/dynamic_pseudo_opening/closing
// include/poutre/geodesy/extrema.hpp:33-64; kind 0..5 in that order.
int ref_extrema(int kind, int pt, int rank, const int64_t *shape, const void *in, void *out, double h, int se) {
  return guarded([&] {
    auto a = make(pt, rank, shape, in);
    auto o = make(pt, rank, shape, nullptr);
    auto s = static_cast<poutre::se::Common_NL_SE>(se);
    auto hv = scalar_of(pt, h);
    switch (kind) {
      case 0: poutre::geo::h_minima(*a, hv, s, *o); break;
      case 1: poutre::geo::h_maxima(*a, hv, s, *o); break;
      case 2: poutre::geo::h_concave(*a, hv, s, *o); break;
      case 3: poutre::geo::h_convex(*a, hv, s, *o); break;
      case 4: poutre::geo::dynamic_pseudo_opening(*a, hv, s, *o); break;
      case 5: poutre::geo::dynamic_pseudo_closing(*a, hv, s, *o); break;
      default: throw std::runtime_error("harness: extrema kind");
    }
    take(*o, pt, rank, shape, out);
  });
}

// Binary h-maxima as the benchmark defines it: h_maxima, then
// CompareImage(f, CompOpSup, rec, 255, 0) (include/poutre/pixel_processing/compare.hpp:69).
// u8 only.
int ref_h_maxima_binary(int rank, const int64_t *shape, const void *in, void *out, double h, int se) {
  return guarded([&] {
    auto a = make(4, rank, shape, in);
    auto rec = make(4, rank, shape, nullptr);
    auto o = make(4, rank, shape, nullptr);
    poutre::geo::h_maxima(*a, scalar_of(4, h), static_cast<poutre::se::Common_NL_SE>(se), *rec);
    poutre::CompareImage(*a, poutre::CompOpType::CompOpSup, *rec, scalar_of(4, 255), scalar_of(4, 0), *o);
    take(*o, 4, rank, shape, out);
  });
}

// poutre::geo::low_leveling / high_leveling / leveling, include/poutre/geodesy/leveling.hpp:37-52
int ref_leveling(int kind, int pt, int rank, const int64_t *shape, const void *ref, const void *marker,
                 void *out, int se) {
  return guarded([&] {
    auto r = make(pt, rank, shape, ref);
    auto m = make(pt, rank, shape, marker);
    auto o = make(pt, rank, shape, nullptr);
    auto s = static_cast<poutre::se::Common_NL_SE>(se);
    if (kind == 0) poutre::geo::low_leveling(*r, *m, s, *o);
    else if (kind == 1) poutre::geo::high_leveling(*r, *m, s, *o);
    else poutre::geo::leveling(*r, *m, s, *o);
    take(*o, pt, rank, shape, out);
  });
}

}  // extern "C"
