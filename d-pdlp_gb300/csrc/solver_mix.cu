// solver_mix.cu -- Solve<double, float>: FP32 matrix and SpMVs, FP64 iterates.
#include "solver_impl.cuh"

namespace pdlp {
template class Solve<double, float>;
}  // namespace pdlp
