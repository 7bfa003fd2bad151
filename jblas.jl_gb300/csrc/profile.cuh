// Internal hooks of the tracing layer (profile.cu).
#pragma once
#include <cuda_runtime.h>

namespace gb {
void prof_before(int kind, cudaStream_t s);
void prof_after(int kind, cudaStream_t s);
// Counts one launch of `kind` without timing it (no CUDA events are created or recorded).
void prof_count(int kind);
}  // namespace gb

// Brackets one kernel launch statement with the tracing hooks.
#define GB_LAUNCH(kind, stream, ...)       \
  do {                                     \
    ::gb::prof_before((kind), (stream));   \
    __VA_ARGS__;                           \
    ::gb::prof_after((kind), (stream));    \
  } while (0)
