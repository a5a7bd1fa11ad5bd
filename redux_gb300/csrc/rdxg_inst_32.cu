// Kernel instantiations for an OTF size of 32.
#include "rdxg_inst.cuh"

namespace rdxg {
template struct Launcher<float, 32>;
template struct Launcher<double, 32>;
template struct EvalLauncher<float, 32>;
}  // namespace rdxg
