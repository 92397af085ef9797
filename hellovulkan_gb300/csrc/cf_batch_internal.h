// cf_batch_internal.h — host-side hooks shared by the batch and server code.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cfcull.h"

namespace cfrt {

int context_device(const CfContext* ctx);
uint32_t* context_error_word(const CfContext* ctx);
// One culling pass of the batch on `st` (a CUDA-graph replay when enabled).
int batch_cull(CfBatch* b, cudaStream_t st);

}  // namespace cfrt
