// Internal hooks of the tracing layer (profile.cu).
#pragma once
#include <cuda_runtime.h>

namespace gb {
void prof_before(int kind, cudaStream_t s);
void prof_after(int kind, cudaStream_t s);
}  // namespace gb

// Brackets one kernel launch statement with the tracing hooks.
#define GB_LAUNCH(kind, stream, ...)       \
  do {                                     \
    ::gb::prof_before((kind), (stream));   \
    __VA_ARGS__;                           \
    ::gb::prof_after((kind), (stream));    \
  } while (0)
