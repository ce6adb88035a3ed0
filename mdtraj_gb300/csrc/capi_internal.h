// Internal helpers shared by the C-ABI translation units: error strings,
// status codes and device-property caching.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/gbrmsd.h"

namespace gb {

// Records a formatted message for gbrmsd_last_error() and returns `code`.
int set_error(int code, const char* fmt, ...);
void clear_error();

// Converts a CUDA runtime error into a status code with context.
int cuda_status(cudaError_t e, const char* what);

// Number of SMs of the current device (cached per device).
int sm_count();

// Maximum opt-in dynamic shared memory per block of the current device.
int max_dyn_smem();

// Event timing of the dominant kernel of a call (gbrmsd_profile_enable).
void prof_begin(cudaStream_t st);
void prof_end(cudaStream_t st);

__host__ __device__ inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace gb

#define GB_CUDA_TRY(expr, what)                                   \
  do {                                                            \
    cudaError_t _e = (expr);                                      \
    if (_e != cudaSuccess) return ::gb::cuda_status(_e, (what));  \
  } while (0)
