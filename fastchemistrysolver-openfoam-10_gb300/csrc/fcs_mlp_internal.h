// fcs_mlp_internal.h -- what the surrogate gate (fcs_gate.cu) uses of the
// MLP ensemble (fcs_mlp.cu).  Internal: not part of the public headers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fcs_mlp.h"

namespace fcs {

// y[n][n_out] (de-normalised) = member's network at raw x[n][n_in]; device
// pointers, enqueued on `st`.
fcs_status mlp_forward_device(fcs_mlp* mlp, int member, int64_t n, const float* x, float* y, cudaStream_t st);
// FCS_OK, or FCS_ERR_CUDA if a tensor-core kernel reported a timed-out wait.
fcs_status mlp_check_errors(fcs_mlp* mlp);
int mlp_n_in(const fcs_mlp* mlp);
int mlp_n_out(const fcs_mlp* mlp);
int mlp_members(const fcs_mlp* mlp);
int mlp_device(const fcs_mlp* mlp);
const char* mlp_message(const fcs_mlp* mlp);

}  // namespace fcs
