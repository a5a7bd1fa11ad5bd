// Kernel instantiations for an OTF size of 64.
#include "rdxg_inst.cuh"

namespace rdxg {
template struct Launcher<float, 64>;
template struct Launcher<double, 64>;
template struct EvalLauncher<float, 64>;
}  // namespace rdxg
