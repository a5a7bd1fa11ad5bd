// Kernel instantiations for an OTF size of 88.
#include "rdxg_inst.cuh"

namespace rdxg {
template struct Launcher<float, 88>;
template struct Launcher<double, 88>;
template struct EvalLauncher<float, 88>;
}  // namespace rdxg
