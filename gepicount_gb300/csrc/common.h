// Shared host-side helpers: thread-local error message, status plumbing.
#pragma once

#include <string>

#include "../../include/gepi.h"

namespace gepi {

// Records `msg` as the calling thread's last error and returns `s`.
gepi_status set_error(gepi_status s, const std::string &msg);
void clear_error();

}  // namespace gepi

#ifdef __CUDACC__
#include <cuda_runtime.h>
// Evaluates a CUDA runtime call; on failure records the message and returns
// GEPI_ERR_CUDA from the enclosing function.
#define GEPI_CUDA(call)                                                                \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess)                                                         \
            return ::gepi::set_error(GEPI_ERR_CUDA, std::string(#call " failed: ") +   \
                                                        cudaGetErrorString(e_));       \
    } while (0)
#endif

#define GEPI_TRY(expr)                      \
    do {                                    \
        gepi_status s_ = (expr);            \
        if (s_ != GEPI_OK) return s_;       \
    } while (0)
