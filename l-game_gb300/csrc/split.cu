// split.cu -- FP32/FP64 split-precision HEVI step.
#include "split.cuh"
#include "common.h"
#include "lgame_gpu.h"

namespace lg {

struct SplitCtx {
  int unused;
};

int split_create(const Dims&, SplitCtx** out, long long*) {
  *out = nullptr;
  lgame_set_error("the split-precision step is not available in this build");
  return LGAME_ERR_UNSUPPORTED;
}
void split_destroy(SplitCtx* s) { delete s; }
int split_set_grid(SplitCtx*, const Dims&, const Grid<double>&, cudaStream_t) { return LGAME_ERR_UNSUPPORTED; }
int split_sync_from_fp64(SplitCtx*, const Dims&, const double*, cudaStream_t) { return LGAME_ERR_UNSUPPORTED; }
int split_step(SplitCtx*, const Dims&, const Grid<double>&, const State&, const State&, const Tend&, double*,
               const double*, double*, int, cudaStream_t, int*) {
  return LGAME_ERR_UNSUPPORTED;
}

}  // namespace lg
