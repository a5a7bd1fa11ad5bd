// Kernel instantiations for an OTF size of 128.
#include "rdxg_inst.cuh"

namespace rdxg {
template struct Launcher<float, 128>;
template struct Launcher<double, 128>;
}  // namespace rdxg
