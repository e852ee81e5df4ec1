// Convergence metrics of the deshade (TGVDeshadeProcessor.cpp:168-220, :479-568) on
// the device: between two checks of the loop, the normalised cross-correlation of the
// shading field l with the previous one and their time total variation sum |l - l_b|.
// The sums are FP64 (block partials combined with double atomics); the host never
// waits for them inside the loop: every check appends one (ncc, tv) pair to a device
// history that is read once at the end.
#include "common.cuh"

namespace tgvdct {
namespace {

constexpr int MT_THREADS = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Adds the block's NV partial sums into out[0..NV).
template <int NV>
__device__ void block_add(double (&v)[NV], double* out) {
    __shared__ double part[MT_THREADS / 32][NV];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) part[warp][k] = v[k];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = lane < MT_THREADS / 32 ? part[lane][k] : 0.0;
            s = warp_sum(s);
            if (lane == 0) atomicAdd(out + k, s);
        }
    }
}

// sums[0] += sum l
__global__ void __launch_bounds__(MT_THREADS) sum_kernel(const float* l, size_t n, double* sums) {
    double v[1] = {0.0};
    for (size_t i = (size_t)blockIdx.x * MT_THREADS + threadIdx.x; i < n;
         i += (size_t)gridDim.x * MT_THREADS)
        v[0] += (double)l[i];
    block_add<1>(v, sums);
}

// With m = sums[0] / n (the mean of l, used for both images as the reference's
// normalized_cross_correlation does): sums[1] += (l - m)^2, sums[2] += (lb - m)^2,
// sums[3] += (l - m)(lb - m), sums[4] += |l - lb|.
__global__ void __launch_bounds__(MT_THREADS)
    moment_kernel(const float* l, const float* lb, size_t n, double* sums) {
    const double m = sums[0] / (double)n;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (size_t i = (size_t)blockIdx.x * MT_THREADS + threadIdx.x; i < n;
         i += (size_t)gridDim.x * MT_THREADS) {
        const double a = (double)l[i] - m, b = (double)lb[i] - m;
        v[0] += a * a;
        v[1] += b * b;
        v[2] += a * b;
        v[3] += fabs((double)l[i] - (double)lb[i]);
    }
    block_add<4>(v, sums + 1);
}

// ncc = sum (l-m)(lb-m) / (std(l) std(lb) n) with std = sqrt(sum / (n - 1))
// (TGVDeshadeProcessor.cpp:177-210); tv = sum |l - lb| (:212-220).  Clears the sums.
__global__ void finish_kernel(double* sums, size_t n, double* slot) {
    const double dn = (double)n;
    const double s1 = sqrt(sums[1] / (dn - 1.0)), s2 = sqrt(sums[2] / (dn - 1.0));
    slot[0] = sums[3] / (s1 * s2 * dn);
    slot[1] = sums[4];
    for (int k = 0; k < 8; ++k) sums[k] = 0.0;
}

int metric_grid(size_t n) {
    const size_t blocks = (n + MT_THREADS - 1) / MT_THREADS;
    return (int)(blocks < 152 * 8 ? blocks : 152 * 8);
}

}  // namespace

void convergence_metrics(const float* l, const float* l_before, size_t n, double* sums,
                         double* slot, cudaStream_t st) {
    const int g = metric_grid(n);
    sum_kernel<<<g, MT_THREADS, 0, st>>>(l, n, sums);
    TGV_CHECK_LAUNCH();
    moment_kernel<<<g, MT_THREADS, 0, st>>>(l, l_before, n, sums);
    TGV_CHECK_LAUNCH();
    finish_kernel<<<1, 1, 0, st>>>(sums, n, slot);
    TGV_CHECK_LAUNCH();
}

}  // namespace tgvdct
