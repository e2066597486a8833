// Shared helpers of libfdadi: error reporting and launch geometry.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/fdadi.h"

namespace fdadi {

// Thread-local message of the last failure (read by fdadi_last_error).
void set_error(const char *fmt, ...);

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Checks a CUDA runtime status; records the message and returns FDADI_E_CUDA.
#define FDADI_CUDA(call)                                                                  \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            ::fdadi::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #call,                \
                               cudaGetErrorString(e_));                                   \
            return FDADI_E_CUDA;                                                          \
        }                                                                                 \
    } while (0)

#define FDADI_CHECK_LAUNCH() FDADI_CUDA(cudaGetLastError())

#define FDADI_REQUIRE(cond, ...)                                                          \
    do {                                                                                  \
        if (!(cond)) {                                                                    \
            ::fdadi::set_error(__VA_ARGS__);                                              \
            return FDADI_E_ARG;                                                           \
        }                                                                                 \
    } while (0)

// Number of SMs of the current device (cached per device).
int sm_count();

inline unsigned grid_for(int64_t work, int threads, int per_sm = 8) {
    int64_t blocks = (work + threads - 1) / threads;
    int64_t cap = (int64_t)sm_count() * per_sm;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (unsigned)blocks;
}

}  // namespace fdadi
