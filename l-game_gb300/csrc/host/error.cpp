// error.cpp -- per-thread last-error message of the library (no exit() anywhere).
#include "common.h"
#include "lgame_gpu.h"

#include <cstdio>
#include <cstring>

namespace {
thread_local char g_last_error[1024] = "no error";
}

extern "C" void lgame_set_error(const char* msg) {
  std::snprintf(g_last_error, sizeof g_last_error, "%s", msg ? msg : "(null)");
}

extern "C" const char* lgame_gpu_last_error(void) { return g_last_error; }

extern "C" const char* lgame_gpu_version(void) { return "lgame-gb300 0.1.0 (sm_103a)"; }
