// Device-driven FP32-refined solves captured into a caller's graph
// (solver.cu), for the batch's one-graph mode (batch.cpp).
#pragma once
#include <cuda_runtime.h>

#include "../../include/ocsl.h"

namespace ocsl {

// Factor, FP32 copies and stencil records of an OCSL_ILU_BICGSTAB_IR32 solve
// of A on the context's own stream, and `slots` control blocks; the
// context's error flag is cleared.  OCSL_ZERO_PIVOT when the factor has a
// zero or infinite pivot (no solve may then be captured for it).
int ir32_graph_prepare(ocsl_ctx* c, const double* A, const ocsl_opts* opts, int slots);
// Captures one solve of A x = b (x: the initial guess, overwritten) into
// `root` after node *last (none: at the root), with its result in control
// block `slot`; *last becomes the solve's last node.
int ir32_graph_capture(ocsl_ctx* c, cudaGraph_t root, cudaGraphNode_t* last, const double* A,
                       const double* b, double* x, const ocsl_opts* opts, int slot);
// The result in control block `slot` once the graph has run (synchronises
// the context's stream; a sweep wait that gave up is OCSL_TIMEOUT).
int ir32_graph_result(ocsl_ctx* c, int slot, ocsl_result* result);
// The context's own stream (the one the prepared work runs on).
cudaStream_t ir32_graph_stream(const ocsl_ctx* c);

}  // namespace ocsl
