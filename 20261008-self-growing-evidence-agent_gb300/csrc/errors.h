// errors.h -- host-side error types shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>

#include <string>

#define SG_CUDA_TRY(expr)                                                       \
    do {                                                                        \
        cudaError_t e__ = (expr);                                               \
        if (e__ != cudaSuccess) {                                               \
            throw sg::CudaError(e__, #expr, __FILE__, __LINE__);               \
        }                                                                       \
    } while (0)

namespace sg {

struct CudaError {
    cudaError_t code;
    std::string what;
    CudaError(cudaError_t c, const char *expr, const char *file, int line) : code(c) {
        what = std::string(cudaGetErrorString(c)) + " at " + file + ":" + std::to_string(line) + " (" + expr + ")";
    }
};

struct EngineError {
    int code;
    std::string what;
    EngineError(int c, std::string w) : code(c), what(std::move(w)) {}
};

}  // namespace sg
