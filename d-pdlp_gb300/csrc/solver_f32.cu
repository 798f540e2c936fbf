// solver_f32.cu -- Solve<float, float>: FP32 iterates and SpMVs.
#include "solver_impl.cuh"

namespace pdlp {
template class Solve<float, float>;
}  // namespace pdlp
