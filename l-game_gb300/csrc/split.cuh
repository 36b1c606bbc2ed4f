// split.cuh -- FP32/FP64 split-precision HEVI step (interface used by lgame_gpu.cu).
#pragma once

#include "kernels.cuh"

namespace lg {

struct SplitCtx;

int split_create(const Dims& D, SplitCtx** out, long long* bytes);
void split_destroy(SplitCtx* s);
// converts the FP64 grid of the context into the FP32 metric copies the stencils read
int split_set_grid(SplitCtx* s, const Dims& D, const Grid<double>& G, cudaStream_t stream);
// refreshes FP32 copies of host-provided diagnostics (radiation tendency)
int split_sync_from_fp64(SplitCtx* s, const Dims& D, const double* rad, cudaStream_t stream);
int split_step(SplitCtx* s, const Dims& D, const Grid<double>& G, const State& So, const State& Sn, const Tend& T,
               double* temperature, const double* rad, double* csh, int step, cudaStream_t stream, int* nkernels);

}  // namespace lg
