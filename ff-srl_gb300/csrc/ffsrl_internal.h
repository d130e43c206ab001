// ffsrl_internal.h -- error reporting and launch helpers shared by the library's units.
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include "../../include/ffsrl.h"

namespace ffsrl {

// Records `msg` as the calling thread's last error and returns `code`.
int32_t fail(int32_t code, const std::string& msg);
// Clears the calling thread's last error.
void clear_error();

}  // namespace ffsrl

#ifdef __CUDACC__
#include <cuda_runtime.h>

namespace ffsrl {
inline int32_t cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? FFSRL_ERR_OUT_OF_MEMORY : FFSRL_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}
inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }
}  // namespace ffsrl

#define FFSRL_CUDA_TRY(expr)                                              \
    do {                                                                  \
        cudaError_t _e = (expr);                                          \
        if (_e != cudaSuccess) return ::ffsrl::cuda_fail(_e, #expr);      \
    } while (0)

#define FFSRL_LAUNCH_CHECK(name)                                          \
    do {                                                                  \
        cudaError_t _e = cudaGetLastError();                              \
        if (_e != cudaSuccess) return ::ffsrl::cuda_fail(_e, name);       \
    } while (0)
#endif
