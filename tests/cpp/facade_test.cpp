// facade_test.cpp -- the reference's known-answer tests replayed through the C++ facade
// (include/poutre_gb300/poutre.hpp), in the style of poutre2's Catch2 tests: parse images
// with ImageFromString, call the poutre-named entry point, compare ImageToString.
//
// Usage: facade_test <cases file>; one case per line, fields separated by ';':
//   op;se;param;expected;input1[;input2;...]
// For "compare" cases se is the CompOpType name and param lists the comparand, true and false
// operands as '|'-separated tokens: "#k" for input image k, a number for a scalar.
// Exit status: number of failed cases (0 = all pass).
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "poutre_gb300/poutre.hpp"

using namespace poutre::gb300;

static std::vector<std::string> split(const std::string &s, char c) {
  std::vector<std::string> out;
  std::string cur;
  std::istringstream is(s);
  while (std::getline(is, cur, c)) out.push_back(cur);
  if (!s.empty() && s.back() == c) out.push_back("");
  return out;
}

static se::Common_NL_SE se_of(const std::string &n) {
  static const std::map<std::string, se::Common_NL_SE> m = {
      {"SESegmentX1D", se::Common_NL_SE::SESegmentX1D}, {"SESquare2D", se::Common_NL_SE::SESquare2D},
      {"SECross2D", se::Common_NL_SE::SECross2D},       {"SESegmentX2D", se::Common_NL_SE::SESegmentX2D},
      {"SESegmentY2D", se::Common_NL_SE::SESegmentY2D}, {"SESegmentX3D", se::Common_NL_SE::SESegmentX3D},
      {"SESegmentY3D", se::Common_NL_SE::SESegmentY3D}, {"SESegmentZ3D", se::Common_NL_SE::SESegmentZ3D},
      {"SECross3D", se::Common_NL_SE::SECross3D},       {"SESquare3D", se::Common_NL_SE::SESquare3D}};
  return m.at(n);
}

// predefined runtime neighbour lists (src/structuring_element/predefined_nl_se.cpp:19-92)
static se::NeighborList nl_of(const std::string &n) {
  se::NeighborList nl;
  if (n == "SESegmentX1D") { nl.rank = 1; nl.offsets = {0, -1, 1}; }
  else if (n == "SESegmentX2D") nl.offsets = {0, 0, 0, -1, 0, 1};
  else if (n == "SESegmentY2D") nl.offsets = {0, 0, -1, 0, 1, 0};
  else if (n == "SESquare2D") nl.offsets = {0, 0, -1, -1, 0, -1, 1, -1, -1, 0, 1, 0, -1, 1, 0, 1, 1, 1};
  else if (n == "SECross2D") nl.offsets = {0, 0, 0, -1, -1, 0, 1, 0, 0, 1};
  else {
    nl.rank = 3;
    if (n == "SESegmentX3D") nl.offsets = {0, 0, 0, 0, 0, -1, 0, 0, 1};
    else if (n == "SESegmentY3D") nl.offsets = {0, 0, 0, 0, -1, 0, 0, 1, 0};
    else if (n == "SESegmentZ3D") nl.offsets = {0, 0, 0, -1, 0, 0, 1, 0, 0};
    else if (n == "SECross3D") nl.offsets = {0, 0, 0, 0, 0, -1, 0, -1, 0, -1, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1};
    else {  // SESquare3D
      nl.offsets = {0, 0, 0};
      for (int c = -1; c <= 1; ++c)
        for (int b = -1; b <= 1; ++b)
          for (int a = -1; a <= 1; ++a)
            if (a || b || c) nl.offsets.insert(nl.offsets.end(), {a, b, c});
    }
  }
  return nl;
}

int main(int argc, char **argv) {
  if (argc < 2) {
    std::cerr << "usage: facade_test <cases>\n";
    return 100;
  }
  std::ifstream f(argv[1]);
  std::string line;
  int failed = 0, run = 0;
  while (std::getline(f, line)) {
    if (line.empty()) continue;
    auto v = split(line, ';');
    if (v.size() < 5) { std::cerr << "bad case line\n"; return 101; }
    const std::string &op = v[0], &sen = v[1], &expected = v[3];
    const double param = v[2].empty() || op == "compare" ? 0.0 : std::stod(v[2]);
    try {
      DeviceImage a = ImageFromString(v[4]);
      DeviceImage o = op == "compare" ? CloneGeometry(ImageFromString(expected)) : CloneGeometry(a);
      if (op == "dilate_static") Dilate(a, se_of(sen), 1, o);
      else if (op == "erode_static") Erode(a, se_of(sen), 1, o);
      else if (op == "dilate_nl") Dilate(a, nl_of(sen), o);
      else if (op == "erode_nl") Erode(a, nl_of(sen), o);
      else if (op == "dilatex") DilateX(a, (std::ptrdiff_t)param, o);
      else if (op == "erodex") ErodeX(a, (std::ptrdiff_t)param, o);
      else if (op == "dilatey") DilateY(a, (std::ptrdiff_t)param, o);
      else if (op == "erodey") ErodeY(a, (std::ptrdiff_t)param, o);
      else if (op == "reconstruct_dilate" || op == "reconstruct_erode") {
        DeviceImage b = ImageFromString(v[5]);
        geo::Reconstruction(op == "reconstruct_dilate" ? geo::reconstruction_type::dilate : geo::reconstruction_type::erode,
                            a, b, se_of(sen), o);
      } else if (op == "low_leveling" || op == "high_leveling" || op == "leveling") {
        DeviceImage b = ImageFromString(v[5]);
        if (op == "low_leveling") geo::low_leveling(a, b, se_of(sen), o);
        else if (op == "high_leveling") geo::high_leveling(a, b, se_of(sen), o);
        else geo::leveling(a, b, se_of(sen), o);
      } else if (op == "h_minima") geo::h_minima(a, PixelValue(a.GetDevicePType(), param), se_of(sen), o);
      else if (op == "h_maxima") geo::h_maxima(a, PixelValue(a.GetDevicePType(), param), se_of(sen), o);
      else if (op == "h_concave") geo::h_concave(a, PixelValue(a.GetDevicePType(), param), se_of(sen), o);
      else if (op == "h_convex") geo::h_convex(a, PixelValue(a.GetDevicePType(), param), se_of(sen), o);
      else if (op == "dynamic_pseudo_opening") geo::dynamic_pseudo_opening(a, PixelValue(a.GetDevicePType(), param), se_of(sen), o);
      else if (op == "dynamic_pseudo_closing") geo::dynamic_pseudo_closing(a, PixelValue(a.GetDevicePType(), param), se_of(sen), o);
      else if (op == "label_binary") label::label_binary(a, se_of(sen), o);  // int64 in, int64 out
      else if (op == "label_flat_zones") label::label_flat_zones(a, se_of(sen), o);
      else if (op == "label_minima") label::label_minima(a, se_of(sen), o);
      else if (op == "label_maxima") label::label_maxima(a, se_of(sen), o);
      else if (op == "compare") {
        std::vector<DeviceImage> ins;
        for (std::size_t k = 5; k < v.size(); ++k) ins.push_back(ImageFromString(v[k]));
        const auto tok = split(v[2], '|');
        // a scalar holds the pixel type the reference's std::get<T> asks for: the input's for the
        // comparand, the output's for the true / false values (compare.cpp:51-61)
        auto opnd = [&](const std::string &t, PType pt) -> CompareOperand {
          if (t[0] == '#') return CompareOperand(std::stoi(t.substr(1)) == 0 ? (const IInterface &)a : ins.at(std::stoi(t.substr(1)) - 1));
          return CompareOperand(PixelValue(pt, std::stod(t)));
        };
        static const std::map<std::string, CompOpType> ops = {
            {"equal", CompOpType::CompOpEqual}, {"diff", CompOpType::CompOpDiff}, {"sup", CompOpType::CompOpSup},
            {"sup_equal", CompOpType::CompOpSupEqual}, {"inf", CompOpType::CompOpInf},
            {"inf_equal", CompOpType::CompOpInfEqual}};
        const PType pi = a.GetDevicePType(), po = o.GetDevicePType();
        CompareImage(a, ops.at(sen), opnd(tok.at(0), pi), opnd(tok.at(1), po), opnd(tok.at(2), po), o);
      }
      else { std::cerr << "unknown op " << op << "\n"; return 102; }
      ++run;
      const std::string got = ImageToString(o);
      if (got != expected) {
        ++failed;
        std::cerr << "FAIL " << op << " " << sen << "\n  got      " << got << "\n  expected " << expected << "\n";
      }
    } catch (const std::exception &e) {
      ++failed;
      std::cerr << "EXCEPTION " << op << " " << sen << ": " << e.what() << "\n";
    }
  }
  // error behaviour: the reference throws std::runtime_error for these (for a scalar that does not
  // hold the image's pixel type too: it rethrows std::get's bad_variant_access)
  int expected_throws = 0;
  try {
    DeviceImage a = ImageFromString("Scalar GUINT8 2 2 3 1 2 3 4 5 6");
    Dilate(a, se::Common_NL_SE::SESquare2D, 1, a);  // output aliases the input
  } catch (const std::runtime_error &) { ++expected_throws; }
  try {
    DeviceImage a = ImageFromString("Scalar GUINT8 2 2 3 1 2 3 4 5 6");
    DeviceImage o = CloneGeometry(a);
    DilateY(a, 1, o);  // non-square image
  } catch (const std::runtime_error &) { ++expected_throws; }
  try {
    DeviceImage a = ImageFromString("Scalar GUINT8 2 2 3 1 2 3 4 5 6");
    DeviceImage o = CloneGeometry(a);
    Dilate(a, se::Common_NL_SE::SESquare3D, 1, o);  // SE rank differs from the image's
  } catch (const std::runtime_error &) { ++expected_throws; }
  try {
    DeviceImage a = ImageFromString("Scalar GUINT8 2 2 3 1 2 3 4 5 6");
    DeviceImage o = CloneGeometry(a);
    geo::h_maxima(a, ScalarTypeVariant(int32_t{1}), se::Common_NL_SE::SESquare2D, o);  // INT32 h, UINT8 image
  } catch (const std::runtime_error &) { ++expected_throws; }
  if (expected_throws != 4) { std::cerr << "error behaviour differs\n"; ++failed; }
  std::cout << "facade_test: " << run << " cases, " << failed << " failed\n";
  return failed;
}
