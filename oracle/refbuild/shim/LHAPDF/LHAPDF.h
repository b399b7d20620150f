// Header-only stand-in for the two LHAPDF 6 entry points that the generator's
// library sources name (PDF set loading and evaluation). No parton densities are
// used on the central-exclusive weight path, so every call throws.
#ifndef GRN_LHAPDF_STANDIN_H
#define GRN_LHAPDF_STANDIN_H
#include <stdexcept>
#include <string>

namespace LHAPDF {
class PDF {
 public:
  virtual ~PDF() {}
  double xfxQ2(int, double, double) const { throw std::runtime_error("LHAPDF stand-in"); }
  double alphasQ2(double) const { throw std::runtime_error("LHAPDF stand-in"); }
};
inline PDF *mkPDF(const std::string &, int) {
  throw std::runtime_error("LHAPDF stand-in: no PDF sets in this build");
}
}  // namespace LHAPDF
#endif
