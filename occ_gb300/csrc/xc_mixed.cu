// Mixed-precision (tcgen05 3xTF32) XC build path.
#include "xc_engine.hpp"

namespace occx {

struct MixedState {};

void Molecule::prepare_mixed() {}

void Molecule::build_mixed(const double *, double *, double *, cudaStream_t) {
  throw ArgError("mixed-precision path is not available in this build");
}

} // namespace occx
