// TEST INFRASTRUCTURE — a host-only stand-in for the CUDA runtime, so that the
// reference's own kernel sources (plain SIMT templates with no shared memory, no
// synchronisation inside a kernel and no intrinsics beyond a few math functions)
// compile with g++ and run on the CPU.  A launch `k<<<g, b>>>(args)` is rewritten
// by build_ref_cpu.py into `ref_launch(g, b, [&]{ k(args); })`, which runs every
// (block, thread) pair in order.  Because no reference kernel on this path reads
// a location that another thread of the same launch writes, sequential execution
// gives the same results as the GPU's parallel execution.
#pragma once

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/types.h>

#include <cmath>
#include <cstddef>

#define __global__
#define __device__
#define __host__

struct dim3 {
    unsigned int x, y, z;
    dim3(unsigned int x_ = 1, unsigned int y_ = 1, unsigned int z_ = 1) : x(x_), y(y_), z(z_) {}
};

struct uint3_ {
    unsigned int x, y, z;
};

extern uint3_ blockIdx;
extern uint3_ threadIdx;
extern dim3 blockDim;
extern dim3 gridDim;

typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3
};

template <class T>
inline cudaError_t cudaMalloc(T** p, size_t size) {
    *p = (T*)malloc(size == 0 ? 1 : size);
    return *p ? cudaSuccess : 2;
}
inline cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, cudaMemcpyKind) {
    memcpy(dst, src, n);
    return cudaSuccess;
}
inline cudaError_t cudaFree(void* p) {
    free(p);
    return cudaSuccess;
}
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaGetDeviceCount(int* c) {
    *c = 1;
    return cudaSuccess;
}
struct cudaDeviceProp {
    int maxThreadsPerBlock;
};
inline cudaError_t cudaGetDeviceProperties(cudaDeviceProp* p, int) {
    p->maxThreadsPerBlock = 1024;
    return cudaSuccess;
}
inline const char* cudaGetErrorString(cudaError_t) { return "host shim error"; }

// cos(pi*a): the same definition as the oracle's cospi_d (oracle/tgv_oracle.hpp),
// so that the two CPU programs agree bit for bit where the algorithms agree.
inline double ref_cospi_d(double a) {
    double r = std::fmod(std::fabs(a), 2.0);
    if (r > 1.0) r = 2.0 - r;
    const double pi = 3.14159265358979323846;
    if (r <= 0.25) return std::cos(pi * r);
    if (r <= 0.75) return std::sin(pi * (0.5 - r));
    return -std::cos(pi * (1.0 - r));
}
inline double cospi(double a) { return ref_cospi_d(a); }
inline float cospi(float a) { return (float)ref_cospi_d((double)a); }
inline float norm3df(float a, float b, float c) {
    return (float)std::sqrt((double)a * a + (double)b * b + (double)c * c);
}

template <class F>
inline void ref_launch(dim3 grid, dim3 block, F&& body) {
    gridDim = grid;
    blockDim = block;
    for (unsigned int bz = 0; bz < grid.z; ++bz)
        for (unsigned int by = 0; by < grid.y; ++by)
            for (unsigned int bx = 0; bx < grid.x; ++bx)
                for (unsigned int tz = 0; tz < block.z; ++tz)
                    for (unsigned int ty = 0; ty < block.y; ++ty)
                        for (unsigned int tx = 0; tx < block.x; ++tx) {
                            blockIdx = uint3_{bx, by, bz};
                            threadIdx = uint3_{tx, ty, tz};
                            body();
                        }
}
