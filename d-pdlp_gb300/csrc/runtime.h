// runtime.h -- internal entry points shared by the C API (api.cpp) and the
// batch / serving runtime (serve.cpp).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "pdlp_gb300.h"

namespace pdlp {

struct DevProblem;

// One solve of an uploaded problem on the caller's stream: FP64, or FP32 with
// FP64 refinement, as `o` selects.  Throws on a CUDA error.
cupdlpx_result_t *solve_uploaded(const DevProblem &P, const pdhg_parameters_t &p,
                                 const pdlp_options_t &o, cudaStream_t st,
                                 pdlp_solve_info_t *info);

// Parameters of a solve (defaults for NULL), with the drop-in API's checks.
bool resolve_parameters(const pdhg_parameters_t *params, pdhg_parameters_t &p);

// Message for pdlp_last_error() of the calling thread.
void record_error(const std::string &msg);

}  // namespace pdlp
