// dispatch_test.cpp -- the branch a poutre2 maintainer adds to poutre2's dispatchers, compiled against
// poutre2's OWN headers and linked with poutre2 itself (oracle/_ref/libpoutre_ref.so) and the GB300
// library.
//
// Every function in `integration` has the signature of a poutre2 entry point, on poutre2's own types
// (poutre::IInterface, se::Common_NL_SE, se::IStructuringElement, geo::reconstruction_type,
// ScalarTypeVariant, CompOpType).  It asks whether the images are device images
// (poutre::gb300::DeviceImage derives from poutre::IInterface in this build) and forwards them to the
// C ABI through the facade; any other image goes on to poutre2's own implementation.  The test replays
// the reference's known answers through the SAME integration functions twice: on host images made by
// poutre::ImageFromString (poutre2's CPU path) and, unless --host-only, on device images (the GPU path).
//
// Usage: dispatch_test [--host-only] <cases file> (the facade test's format).  Exit status: failures.
#ifndef POUTRE_GB300_WITH_POUTRE2
#define POUTRE_GB300_WITH_POUTRE2
#endif
#include <poutre/base/image_interface.hpp>
#include <poutre/geodesy/extrema.hpp>
#include <poutre/geodesy/leveling.hpp>
#include <poutre/geodesy/mreconstruct.hpp>
#include <poutre/label/label_binary.hpp>
#include <poutre/label/label_extrema.hpp>
#include <poutre/label/label_flat_zones.hpp>
#include <poutre/low_level_morpho/ero_dil.hpp>
#include <poutre/low_level_morpho/ero_dil_line.hpp>
#include <poutre/pixel_processing/compare.hpp>
#include <poutre/pixel_processing/copy_convert.hpp>
#include <poutre/structuring_element/details/neighbor_list_se_t.hpp>
#include <poutre/structuring_element/predefined_nl_se.hpp>

#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <variant>
#include <vector>

#include "poutre_gb300/poutre.hpp"

namespace gb = poutre::gb300;
using poutre::IInterface;
using poutre::ScalarTypeVariant;
namespace pse = poutre::se;

// ----------------------------------------------------------------------------- the dispatcher branch
namespace integration {

// poutre::Dilate / Erode(const IInterface&, se::Common_NL_SE, int, IInterface&), ero_dil.hpp:32-35
void Dilate(const IInterface &i_img, pse::Common_NL_SE nl, int iter, IInterface &o_img) {
  if (gb::is_device_image(i_img)) return gb::Dilate(i_img, nl, iter, o_img);
  poutre::Dilate(i_img, nl, iter, o_img);
}
void Erode(const IInterface &i_img, pse::Common_NL_SE nl, int iter, IInterface &o_img) {
  if (gb::is_device_image(i_img)) return gb::Erode(i_img, nl, iter, o_img);
  poutre::Erode(i_img, nl, iter, o_img);
}

// poutre::Dilate / Erode(const IInterface&, const se::IStructuringElement&, IInterface&), ero_dil.hpp:44-47:
// a neighbour list becomes the C ABI's offset list
template <std::ptrdiff_t R> bool offsets_of(const pse::IStructuringElement &s, gb::se::NeighborList &nl) {
  auto *l = dynamic_cast<const pse::details::neighbor_list_t<R> *>(&s);
  if (!l) return false;
  nl.rank = (int)R;
  nl.offsets.clear();
  for (const auto &c : *l)
    for (std::ptrdiff_t k = 0; k < R; ++k) nl.offsets.push_back((int32_t)c[k]);
  return true;
}
gb::se::NeighborList to_offsets(const pse::IStructuringElement &s) {
  gb::se::NeighborList nl;
  if (offsets_of<1>(s, nl) || offsets_of<2>(s, nl) || offsets_of<3>(s, nl)) return nl;
  POUTRE_RUNTIME_ERROR("Unsupported IStructuringElement type on the device");
}
void Dilate(const IInterface &i_img, const pse::IStructuringElement &s, IInterface &o_img) {
  if (gb::is_device_image(i_img)) return gb::Dilate(i_img, to_offsets(s), o_img);
  poutre::Dilate(i_img, s, o_img);
}
void Erode(const IInterface &i_img, const pse::IStructuringElement &s, IInterface &o_img) {
  if (gb::is_device_image(i_img)) return gb::Erode(i_img, to_offsets(s), o_img);
  poutre::Erode(i_img, s, o_img);
}

// poutre::DilateX / ErodeX / DilateY / ErodeY, ero_dil_line.hpp:32-47
#define PG_DISPATCH_LINE(NAME)                                                  \
  void NAME(const IInterface &i_img, std::ptrdiff_t half, IInterface &o_img) { \
    if (gb::is_device_image(i_img)) return gb::NAME(i_img, half, o_img);      \
    poutre::NAME(i_img, half, o_img);                                           \
  }
PG_DISPATCH_LINE(DilateX)
PG_DISPATCH_LINE(ErodeX)
PG_DISPATCH_LINE(DilateY)
PG_DISPATCH_LINE(ErodeY)
#undef PG_DISPATCH_LINE

namespace geo {
// poutre::geo::Reconstruction, mreconstruct.hpp:37-41
void Reconstruction(poutre::geo::reconstruction_type t, const IInterface &marker, const IInterface &mask,
                    pse::Common_NL_SE nl, IInterface &o_img) {
  if (gb::is_device_image(mask)) return gb::geo::Reconstruction(t, marker, mask, nl, o_img);
  poutre::geo::Reconstruction(t, marker, mask, nl, o_img);
}
// poutre::geo::h_minima ... dynamic_pseudo_closing, extrema.hpp:33-64: the ScalarTypeVariant crosses as is
#define PG_DISPATCH_EXTREMA(NAME)                                                                    \
  void NAME(const IInterface &i_img, const ScalarTypeVariant &h, pse::Common_NL_SE nl, IInterface &o_img) { \
    if (gb::is_device_image(i_img)) return gb::geo::NAME(i_img, h, nl, o_img);                       \
    poutre::geo::NAME(i_img, h, nl, o_img);                                                           \
  }
PG_DISPATCH_EXTREMA(h_minima)
PG_DISPATCH_EXTREMA(h_maxima)
PG_DISPATCH_EXTREMA(h_concave)
PG_DISPATCH_EXTREMA(h_convex)
PG_DISPATCH_EXTREMA(dynamic_pseudo_opening)
PG_DISPATCH_EXTREMA(dynamic_pseudo_closing)
#undef PG_DISPATCH_EXTREMA
// poutre::geo::low_leveling / high_leveling / leveling, leveling.hpp:37-52
#define PG_DISPATCH_LEVELING(NAME)                                                                         \
  void NAME(const IInterface &ref, const IInterface &marker, pse::Common_NL_SE nl, IInterface &o_img) {    \
    if (gb::is_device_image(ref)) return gb::geo::NAME(ref, marker, nl, o_img);                            \
    poutre::geo::NAME(ref, marker, nl, o_img);                                                             \
  }
PG_DISPATCH_LEVELING(low_leveling)
PG_DISPATCH_LEVELING(high_leveling)
PG_DISPATCH_LEVELING(leveling)
#undef PG_DISPATCH_LEVELING
}  // namespace geo

namespace label {
// poutre::label::label_binary / label_flat_zones / label_minima / label_maxima (include/poutre/label)
std::size_t label_binary(const IInterface &i_img, pse::Common_NL_SE nl, IInterface &o_img) {
  if (gb::is_device_image(i_img)) return gb::label::label_binary(i_img, nl, o_img);
  return poutre::label::label_binary(i_img, nl, o_img);
}
std::size_t label_flat_zones(const IInterface &i_img, pse::Common_NL_SE nl, IInterface &o_img) {
  if (gb::is_device_image(i_img)) return gb::label::label_flat_zones(i_img, nl, o_img);
  return poutre::label::label_flat_zones(i_img, nl, o_img);
}
void label_minima(const IInterface &i_img, pse::Common_NL_SE nl, IInterface &o_img) {
  if (gb::is_device_image(i_img)) return gb::label::label_minima(i_img, nl, o_img);
  poutre::label::label_minima(i_img, nl, o_img);
}
void label_maxima(const IInterface &i_img, pse::Common_NL_SE nl, IInterface &o_img) {
  if (gb::is_device_image(i_img)) return gb::label::label_maxima(i_img, nl, o_img);
  poutre::label::label_maxima(i_img, nl, o_img);
}
}  // namespace label

// poutre::CompareImage, compare.hpp:31-84: one dispatcher per overload form
using Operand = std::variant<const IInterface *, ScalarTypeVariant>;
void CompareImage(const IInterface &i_img, poutre::CompOpType op, const Operand &c, const Operand &t, const Operand &f,
                  IInterface &o_img) {
  auto g = [](const Operand &x) -> gb::CompareOperand {
    if (auto *p = std::get_if<const IInterface *>(&x)) return gb::CompareOperand(**p);
    return gb::CompareOperand(std::get<ScalarTypeVariant>(x));
  };
  if (gb::is_device_image(i_img)) return gb::CompareImage(i_img, op, g(c), g(t), g(f), o_img);
  const IInterface *ic = c.index() == 0 ? std::get<0>(c) : nullptr, *it = t.index() == 0 ? std::get<0>(t) : nullptr,
                   *iff = f.index() == 0 ? std::get<0>(f) : nullptr;
  const ScalarTypeVariant sc = ic ? ScalarTypeVariant{} : std::get<1>(c), st = it ? ScalarTypeVariant{} : std::get<1>(t),
                          sf = iff ? ScalarTypeVariant{} : std::get<1>(f);
  switch ((ic ? 4 : 0) | (it ? 2 : 0) | (iff ? 1 : 0)) {
    case 0: poutre::CompareImage(i_img, op, sc, st, sf, o_img); break;
    case 1: poutre::CompareImage(i_img, op, sc, st, *iff, o_img); break;
    case 2: poutre::CompareImage(i_img, op, sc, *it, sf, o_img); break;
    case 3: poutre::CompareImage(i_img, op, sc, *it, *iff, o_img); break;
    case 4: poutre::CompareImage(i_img, op, *ic, st, sf, o_img); break;
    case 5: poutre::CompareImage(i_img, op, *ic, st, *iff, o_img); break;
    case 6: poutre::CompareImage(i_img, op, *ic, *it, sf, o_img); break;
    default: poutre::CompareImage(i_img, op, *ic, *it, *iff, o_img); break;
  }
}
}  // namespace integration

// ----------------------------------------------------------------------------- the known answers
static std::vector<std::string> split(const std::string &s, char c) {
  std::vector<std::string> out;
  std::string cur;
  std::istringstream is(s);
  while (std::getline(is, cur, c)) out.push_back(cur);
  if (!s.empty() && s.back() == c) out.push_back("");
  return out;
}

static pse::Common_NL_SE se_of(const std::string &n) {
  static const std::map<std::string, pse::Common_NL_SE> m = {
      {"SESegmentX1D", pse::Common_NL_SE::SESegmentX1D}, {"SESquare2D", pse::Common_NL_SE::SESquare2D},
      {"SECross2D", pse::Common_NL_SE::SECross2D},       {"SESegmentX2D", pse::Common_NL_SE::SESegmentX2D},
      {"SESegmentY2D", pse::Common_NL_SE::SESegmentY2D}, {"SESegmentX3D", pse::Common_NL_SE::SESegmentX3D},
      {"SESegmentY3D", pse::Common_NL_SE::SESegmentY3D}, {"SESegmentZ3D", pse::Common_NL_SE::SESegmentZ3D},
      {"SECross3D", pse::Common_NL_SE::SECross3D},       {"SESquare3D", pse::Common_NL_SE::SESquare3D}};
  return m.at(n);
}

// poutre2's predefined runtime neighbour lists (src/structuring_element/predefined_nl_se.cpp)
static const pse::IStructuringElement &nl_of(const std::string &n) {
  static const std::map<std::string, const pse::IStructuringElement *> m = {
      {"SESegmentX1D", &pse::SESegmentX1D}, {"SESquare2D", &pse::SESquare2D},   {"SECross2D", &pse::SECross2D},
      {"SESegmentX2D", &pse::SESegmentX2D}, {"SESegmentY2D", &pse::SESegmentY2D}, {"SESquare3D", &pse::SESquare3D},
      {"SECross3D", &pse::SECross3D},       {"SESegmentX3D", &pse::SESegmentX3D}, {"SESegmentY3D", &pse::SESegmentY3D},
      {"SESegmentZ3D", &pse::SESegmentZ3D}};
  return *m.at(n);
}

// One image in both worlds: a host poutre2 image or a device image, seen as a poutre::IInterface.
struct Img {
  std::unique_ptr<IInterface> host;
  std::unique_ptr<gb::DeviceImage> dev;
  IInterface &get() { return host ? *host : static_cast<IInterface &>(*dev); }
  std::string str() { return host ? poutre::ImageToString(*host) : gb::ImageToString(*dev); }
};

static Img make(bool device, const std::string &s) {
  Img i;
  if (device) i.dev = std::make_unique<gb::DeviceImage>(gb::ImageFromString(s));
  else i.host = poutre::ImageFromString(s);
  return i;
}

static Img like(bool device, const std::string &s) {  // an output with the geometry of image string s
  Img i;
  if (device) i.dev = std::make_unique<gb::DeviceImage>(gb::CloneGeometry(gb::ImageFromString(s)));
  else i.host = poutre::CloneGeometry(*poutre::ImageFromString(s));
  return i;
}

static int run_cases(const std::string &path, bool device, int &run) {
  std::ifstream f(path);
  std::string line;
  int failed = 0;
  while (std::getline(f, line)) {
    if (line.empty()) continue;
    auto v = split(line, ';');
    const std::string &op = v[0], &sen = v[1], &expected = v[3];
    const double param = v[2].empty() || op == "compare" ? 0.0 : std::stod(v[2]);
    try {
      Img a = make(device, v[4]);
      Img o = like(device, op == "compare" || op.rfind("label_", 0) == 0 ? expected : v[4]);
      IInterface &A = a.get(), &O = o.get();
      const ScalarTypeVariant h = poutre::CreatePixelValue(param, A.GetPType());
      if (op == "dilate_static") integration::Dilate(A, se_of(sen), 1, O);
      else if (op == "erode_static") integration::Erode(A, se_of(sen), 1, O);
      else if (op == "dilate_nl") integration::Dilate(A, nl_of(sen), O);
      else if (op == "erode_nl") integration::Erode(A, nl_of(sen), O);
      else if (op == "dilatex") integration::DilateX(A, (std::ptrdiff_t)param, O);
      else if (op == "erodex") integration::ErodeX(A, (std::ptrdiff_t)param, O);
      else if (op == "dilatey") integration::DilateY(A, (std::ptrdiff_t)param, O);
      else if (op == "erodey") integration::ErodeY(A, (std::ptrdiff_t)param, O);
      else if (op == "reconstruct_dilate" || op == "reconstruct_erode") {
        Img b = make(device, v[5]);
        integration::geo::Reconstruction(op == "reconstruct_dilate" ? poutre::geo::reconstruction_type::dilate
                                                                    : poutre::geo::reconstruction_type::erode,
                                         A, b.get(), se_of(sen), O);
      } else if (op == "low_leveling" || op == "high_leveling" || op == "leveling") {
        Img b = make(device, v[5]);
        if (op == "low_leveling") integration::geo::low_leveling(A, b.get(), se_of(sen), O);
        else if (op == "high_leveling") integration::geo::high_leveling(A, b.get(), se_of(sen), O);
        else integration::geo::leveling(A, b.get(), se_of(sen), O);
      } else if (op == "h_minima") integration::geo::h_minima(A, h, se_of(sen), O);
      else if (op == "h_maxima") integration::geo::h_maxima(A, h, se_of(sen), O);
      else if (op == "h_concave") integration::geo::h_concave(A, h, se_of(sen), O);
      else if (op == "h_convex") integration::geo::h_convex(A, h, se_of(sen), O);
      else if (op == "dynamic_pseudo_opening") integration::geo::dynamic_pseudo_opening(A, h, se_of(sen), O);
      else if (op == "dynamic_pseudo_closing") integration::geo::dynamic_pseudo_closing(A, h, se_of(sen), O);
      else if (op == "label_binary") integration::label::label_binary(A, se_of(sen), O);
      else if (op == "label_flat_zones") integration::label::label_flat_zones(A, se_of(sen), O);
      else if (op == "label_minima") integration::label::label_minima(A, se_of(sen), O);
      else if (op == "label_maxima") integration::label::label_maxima(A, se_of(sen), O);
      else if (op == "compare") {
        std::vector<Img> ins;
        for (std::size_t k = 5; k < v.size(); ++k) ins.push_back(make(device, v[k]));
        const auto tok = split(v[2], '|');
        auto opnd = [&](const std::string &t, poutre::PType pt) -> integration::Operand {
          if (t[0] == '#') {
            const int k = std::stoi(t.substr(1));
            return k == 0 ? &A : &ins.at(k - 1).get();
          }
          return poutre::CreatePixelValue(std::stod(t), pt);
        };
        static const std::map<std::string, poutre::CompOpType> ops = {
            {"equal", poutre::CompOpType::CompOpEqual}, {"diff", poutre::CompOpType::CompOpDiff},
            {"sup", poutre::CompOpType::CompOpSup},     {"sup_equal", poutre::CompOpType::CompOpSupEqual},
            {"inf", poutre::CompOpType::CompOpInf},     {"inf_equal", poutre::CompOpType::CompOpInfEqual}};
        integration::CompareImage(A, ops.at(sen), opnd(tok.at(0), A.GetPType()), opnd(tok.at(1), O.GetPType()),
                                  opnd(tok.at(2), O.GetPType()), O);
      } else {
        std::cerr << "unknown op " << op << "\n";
        return 1000;
      }
      ++run;
      const std::string got = o.str();
      if (got != expected) {
        ++failed;
        std::cerr << (device ? "DEVICE" : "HOST") << " FAIL " << op << " " << sen << "\n  got      " << got
                  << "\n  expected " << expected << "\n";
      }
    } catch (const std::exception &e) {
      ++failed;
      std::cerr << (device ? "DEVICE" : "HOST") << " EXCEPTION " << op << " " << sen << ": " << e.what() << "\n";
    }
  }
  return failed;
}

// The two paths throw std::runtime_error where poutre2 throws; each case is refused before any
// kernel runs.
static int error_behaviour(bool device) {
  int failed = 0;
  const char *where = device ? "DEVICE" : "HOST";
  Img a = make(device, "Scalar GUINT8 2 3 3 1 2 3 4 5 6 7 8 9");
  Img o = like(device, "Scalar GUINT8 2 3 3 1 2 3 4 5 6 7 8 9");
  auto expect_throw = [&](const char *what, auto &&fn, const char *text) {
    try {
      fn();
      std::cerr << where << " no exception: " << what << "\n";
      ++failed;
    } catch (const std::runtime_error &e) {
      if (text && std::string(e.what()).find(text) == std::string::npos) {
        std::cerr << where << " unexpected message for " << what << ": " << e.what() << "\n";
        ++failed;
      }
    }
  };
  expect_throw("INT32 h for a UINT8 image", [&] {
    integration::geo::h_maxima(a.get(), ScalarTypeVariant(poutre::pINT32{1}), pse::Common_NL_SE::SESquare2D, o.get());
  }, "unable to extract");
  expect_throw("output aliasing the input", [&] {
    integration::geo::Reconstruction(poutre::geo::reconstruction_type::dilate, a.get(), o.get(),
                                     pse::Common_NL_SE::SESquare2D, o.get());
  }, nullptr);
  expect_throw("3D SE on an image", [&] {
    integration::geo::Reconstruction(poutre::geo::reconstruction_type::dilate, a.get(), a.get(),
                                     pse::Common_NL_SE::SESquare3D, o.get());
  }, nullptr);
  return failed;
}

int main(int argc, char **argv) {
  bool host_only = false;
  std::string path;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "--host-only") host_only = true;
    else path = a;
  }
  if (path.empty()) {
    std::cerr << "usage: dispatch_test [--host-only] <cases>\n";
    return 100;
  }
  int failed = 0, run_host = 0, run_dev = 0;
  failed += run_cases(path, false, run_host) + error_behaviour(false);
  if (!host_only) {
    // a poutre::IInterface& that holds a device image reaches the C ABI
    gb::DeviceImage d = gb::ImageFromString("Scalar GUINT8 1 4 1 2 3 4");
    const IInterface &as_poutre = d;
    if (!gb::is_device_image(as_poutre) || as_poutre.GetPType() != poutre::PType::PType_GrayUINT8 ||
        as_poutre.GetRank() != 1) {
      std::cerr << "device image is not seen through poutre::IInterface\n";
      ++failed;
    }
    failed += run_cases(path, true, run_dev) + error_behaviour(true);
  }
  std::cout << "dispatch_test: host " << run_host << " cases, device " << run_dev << " cases, " << failed << " failed\n";
  return failed;
}
