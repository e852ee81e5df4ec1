// TEST INFRASTRUCTURE — stands in for the header that the reference's CMake build
// generates from source/modules/cuda/cuda_helper.in (block size 1024 and the
// error-check macro, cuda_helper.in:8-21), for the host-only build of
// build_ref_cpu.py.
#ifndef CUDA_HELPER
#define CUDA_HELPER

#include "cuda.h"

#define CUDA_BLOCK_DIMENSON 1024

#define cudaCheckError(ans) \
    { ref_check((ans), __FILE__, __LINE__); }
inline void ref_check(cudaError_t code, const char* file, int line) {
    if (code != cudaSuccess) {
        fprintf(stderr, "host shim error %d at %s:%d\n", code, file, line);
        abort();
    }
}

#endif
