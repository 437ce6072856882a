// C entry points over the reference's own Lebedev source, compiled unmodified
// from the reference tree (src/numint/lebedev.cpp) into oracle/_ref.  Test
// infrastructure only: used to pin the product's angular grids.
#include <cstring>
#include <occ/numint/lebedev.h>
extern "C" int ref_lebedev(int n, double *out /* n x 4: x, y, z, w */) {
  auto m = occ::numint::grid::lebedev(n);
  std::memcpy(out, m.data(), sizeof(double) * 4 * n);
  return n;
}
