// emulator.cuh -- internal interface of the tensor-core MLP (emulator.cu) for the coupling code.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

struct lgame_emu;

namespace emu {

enum EpiKind { kEpiF32 = 0, kEpiBias = 1, kEpiBiasGelu = 2, kEpiGeluBwd = 3, kEpiBiasGeluH = 4 };

// epilogue of the tensor-core GEMM (fields used depend on kind):
//   kEpiF32      c[z*split_stride + m*ldc + n] = acc               (split-K partials)
//   kEpiBias     c[m*ldc + n] = acc + bias[n]
//   kEpiBiasGelu c[m*ldc + n] = z = acc + bias[n]; h[m*ldh + n] = ht[n*ldt + m] = bf16(gelu(z))
//   kEpiGeluBwd  c[m*ldc + n] = d = acc * gelu'(zprev[m*ldc + n]); h, ht = bf16(d)
//   kEpiBiasGeluH h[m*ldh + n] = bf16(gelu(acc + bias[n])) alone (inference)
struct Epi {
  int kind;
  const float* bias;
  const float* zprev;
  float* c;
  int ldc;
  long long split_stride;
  __nv_bfloat16* h;
  int ldh;
  __nv_bfloat16* ht;
  int ldt;
};

// heating rates (device, n x nout) of n rows of raw features (device, n x nin)
int infer_device(lgame_emu* e, const float* x_dev, long long n, float* y_dev, cudaStream_t st);
int nin_of(const lgame_emu* e);
int nout_of(const lgame_emu* e);
int nlev_of(const lgame_emu* e);

}  // namespace emu
