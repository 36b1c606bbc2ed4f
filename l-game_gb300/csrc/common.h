// common.h -- internal helpers shared by the host code and the CUDA library.
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

// Records the message returned by lgame_gpu_last_error() for the calling thread.
void lgame_set_error(const char* msg);

#ifdef __cplusplus
}
#endif
