// Reductions on the device, FP64 sums (block partials combined with double atomics):
// - convergence metrics of the deshade (TGVDeshadeProcessor.cpp:168-220, :479-568):
//   between two checks of the loop, the normalised cross-correlation of the shading
//   field l with the previous one and their time total variation sum |l - l_b|; the
//   host never waits for them inside the loop (every check appends one (ncc, tv) pair
//   to a device history read once at the end);
// - the TGV2 primal energy, which the loop can evaluate every k iterations to stop
//   once it no longer decreases.
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

// Primal energy terms of TGV2, the quantity the primal-dual iteration minimises, with
// the operators as the reference implements them (tgv2_common.cu:96-131, 174-276): F
// the forward differences with Neumann ends, E from the negated backward differences
// B with 1/2 on the mixed entries, and the Frobenius norm with weight 2 on the
// off-diagonal entries (the norm of the q projection).  FP32 per voxel, FP64 sums:
// sums[0] += |u - f| (L1) or (u - f)^2 / 2 (L2); sums[1] += |F u - v|; sums[2] += |E v|.
template <bool THREE>
__global__ void __launch_bounds__(MT_THREADS)
    energy_kernel(const float* f, const float* u, const float* vx, const float* vy,
                  const float* vz, int W, int H, int D, int data_term, double* sums) {
    double acc[3] = {0.0, 0.0, 0.0};
    const size_t WH = (size_t)W * H, n = WH * D;
    for (size_t i = (size_t)blockIdx.x * MT_THREADS + threadIdx.x; i < n;
         i += (size_t)gridDim.x * MT_THREADS) {
        const int x = (int)(i % W), y = (int)((i / W) % H), z = (int)(i / WH);
        const float ui = u[i], d = ui - f[i];
        const float dt = data_term == TGVDCT_DATA_L1 ? fabsf(d) : 0.5f * d * d;
        const float vxi = vx[i], vyi = vy[i];
        const float gx = (x + 1 < W ? u[i + 1] - ui : 0.f) - vxi;
        const float gy = (y + 1 < H ? u[i + W] - ui : 0.f) - vyi;
        float g2 = gx * gx + gy * gy;
        const float exx = (x > 0 ? vx[i - 1] : 0.f) - vxi;
        const float eyy = (y > 0 ? vy[i - W] : 0.f) - vyi;
        const float exy = (((x > 0 ? vy[i - 1] : 0.f) - vyi) + ((y > 0 ? vx[i - W] : 0.f) - vxi)) * 0.5f;
        float e2 = exx * exx + eyy * eyy + 2.f * exy * exy;
        if constexpr (THREE) {
            const float vzi = vz[i];
            const float gz = (z + 1 < D ? u[i + WH] - ui : 0.f) - vzi;
            g2 = g2 + gz * gz;
            const float ezz = (z > 0 ? vz[i - WH] : 0.f) - vzi;
            const float exz =
                (((x > 0 ? vz[i - 1] : 0.f) - vzi) + ((z > 0 ? vx[i - WH] : 0.f) - vxi)) * 0.5f;
            const float eyz =
                (((y > 0 ? vz[i - W] : 0.f) - vzi) + ((z > 0 ? vy[i - WH] : 0.f) - vyi)) * 0.5f;
            e2 = e2 + ezz * ezz + 2.f * exz * exz + 2.f * eyz * eyz;
        }
        acc[0] += (double)dt;
        acc[1] += (double)sqrtf(g2);
        acc[2] += (double)sqrtf(e2);
    }
    block_add<3>(acc, sums);
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

void tgv_energy_terms(const float* f, const float* u, const float* vx, const float* vy,
                      const float* vz, int W, int H, int D, bool three, int data_term,
                      double* sums, cudaStream_t st) {
    const size_t n = (size_t)W * H * D;
    TGV_CUDA(cudaMemsetAsync(sums, 0, 3 * sizeof(double), st));
    const int g = metric_grid(n);
    if (three) energy_kernel<true><<<g, MT_THREADS, 0, st>>>(f, u, vx, vy, vz, W, H, D, data_term, sums);
    else energy_kernel<false><<<g, MT_THREADS, 0, st>>>(f, u, vx, vy, vz, W, H, D, data_term, sums);
    TGV_CHECK_LAUNCH();
}

}  // namespace tgvdct
