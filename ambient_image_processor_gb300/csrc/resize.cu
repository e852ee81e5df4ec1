// Cubic B-spline resize: the reference's ResizeProcessor::process(image, width,
// height, depth, BSpline3) (resize/ResizeProcessor.cpp:49-143), which hands the work
// to ITK 4.8.1's ResampleImageFilter with an identity transform and a
// BSplineInterpolateImageFunction of order 3.  The down-sampled deshade
// (tgvk_deshade_downsampled/TGVKDeshadeDownsampledProcessor.cpp:63-111) resizes the
// image and the mask down, and the denoised image and the shading back up.
//
// The algorithm is ITK's, which is the published cubic B-spline interpolation
// (Unser, Aldroubi & Eden 1993; Thevenaz, Blu & Unser 2000):
//   1. coefficients: along x, then y, then z, every line is scaled by the gain
//      (1 - z)(1 - 1/z) and run through the causal and anti-causal first-order
//      recursions of the pole z = sqrt(3) - 2, with mirror boundaries; the causal
//      start value sums z^k c[k] over a horizon of ceil(log 1e-10 / log |z|) = 18
//      samples, or uses the closed mirror form on lines no longer than that;
//   2. evaluation: output index i sits at the continuous input index i * s, where
//      s = 1 / (float)(out_grid / n) is the spacing ratio ResizeProcessor sets
//      (:70-79); points outside [-0.5, n - 0.5) give 0; inside, the 4 x 4 x 4 taps
//      around floor(x) - 1 with mirrored indices are summed, x fastest, with weights
//      ((1 * wx) * wy) * wz, and the sum is cast to float.
// Upsampling (any axis grows) resamples onto a grid two samples longer per axis and
// keeps the first width x height x depth (:55-63 and :136-141), which fixes the
// sample positions.
//
// Everything is FP64, like ITK's coefficient type: the down-sampled mask is
// thresholded at 1 by the masked deshade, so values that should be exactly 1 must
// round to 1.0f.  This unit is compiled with -fmad=false and the per-axis positions,
// weights and mirrored indices are computed on the host in double, so the device
// sum is the same operation sequence as a double restatement on the CPU.
//
// Cost: the evaluation does 256 FP64 operations per output voxel (64 taps); the taps
// of neighbouring outputs overlap and come from L1/L2.  Resizes run a few times per
// deshade call, around a loop of hundreds of iterations.
#include <cmath>
#include <vector>

#include "common.cuh"

// first bad index of a bounds-checking build (see TGV_IN_BOUNDS)
static __device__ unsigned long long g_bounds_rs;
#define TGV_BOUNDS_WORD g_bounds_rs

namespace tgvdct {
namespace {

struct Axis {
    const int* idx;          // 4 per output index
    const double* wt;        // 4 per output index
    const uint8_t* inside;   // 1 per output index
};

struct Pole {
    double z, gain, z2n[3];
    long horizon;
};

__device__ void prefilter_line(double* c, long n, size_t s, const Pole& p, double z2n) {
    if (n == 1) return;
    const double z = p.z;
    for (long k = 0; k < n; ++k) c[k * s] = c[k * s] * p.gain;
    if (p.horizon < n) {
        double zn = z, sum = c[0];
        for (long k = 1; k < p.horizon; ++k) {
            sum = sum + zn * c[k * s];
            zn = zn * z;
        }
        c[0] = sum;
    } else {
        double zn = z;
        const double iz = 1.0 / z;
        double z2 = z2n;
        double sum = c[0] + z2 * c[(n - 1) * s];
        z2 = z2 * z2 * iz;
        for (long k = 1; k <= n - 2; ++k) {
            sum = sum + (zn + z2) * c[k * s];
            zn = zn * z;
            z2 = z2 * iz;
        }
        c[0] = sum / (1.0 - zn * zn);
    }
    for (long k = 1; k < n; ++k) c[k * s] = c[k * s] + z * c[(k - 1) * s];
    c[(n - 1) * s] = (z / (z * z - 1.0)) * (z * c[(n - 2) * s] + c[(n - 1) * s]);
    for (long k = n - 2; k >= 0; --k) c[k * s] = z * (c[(k + 1) * s] - c[k * s]);
}

__global__ void to_double_kernel(const float* __restrict__ in, double* __restrict__ c, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        c[i] = (double)in[i];
}

// One thread per line along AXIS.  Lines along y and z are coalesced across threads
// (neighbouring x); lines along x are walked by one thread each.
template <int AXIS>
__global__ void prefilter_kernel(double* c, int w, int h, int d, Pole p) {
    const size_t wh = (size_t)w * h;
    const size_t lines = AXIS == 0 ? (size_t)h * d : AXIS == 1 ? (size_t)w * d : wh;
    const size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (l >= lines) return;
    if constexpr (kCheckBounds) {  // the line's first and last element
        const size_t n = wh * d;
        const size_t first = AXIS == 0 ? l * w : AXIS == 1 ? (l / w) * wh + l % w : l;
        const size_t last = first + (AXIS == 0 ? (size_t)(w - 1) : AXIS == 1 ? (size_t)(h - 1) * w
                                                                              : (size_t)(d - 1) * wh);
        if (!TGV_IN_BOUNDS(first, n, 40) || !TGV_IN_BOUNDS(last, n, 41)) return;
    }
    if (AXIS == 0) {
        prefilter_line(c + l * w, w, 1, p, p.z2n[0]);
    } else if (AXIS == 1) {
        const size_t x = l % w, zz = l / w;
        prefilter_line(c + zz * wh + x, h, w, p, p.z2n[1]);
    } else {
        prefilter_line(c + l, d, wh, p, p.z2n[2]);
    }
}

__global__ void evaluate_kernel(const double* __restrict__ c, int w, int h, int d,
                                Axis ax, Axis ay, Axis az, float* __restrict__ out, int W, int H,
                                int D) {
    const size_t total = (size_t)W * H * D, wh = (size_t)w * h;
    for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < total;
         o += (size_t)gridDim.x * blockDim.x) {
        const int xo = (int)(o % W);
        const int yo = (int)((o / W) % H);
        const int zo = (int)(o / ((size_t)W * H));
        float v = 0.f;
        if (ax.inside[xo] && ay.inside[yo] && az.inside[zo]) {
            // The weight of tap (i, j, k) is ((1 * wx_i) * wy_j) * wz_k in ITK's order;
            // 1 * wx_i is wx_i exactly, so the 16 products wx_i * wy_j are formed once
            // (the same roundings) and each tap costs one product with wz_k, one with
            // the coefficient and the add: 208 FP64 operations per voxel instead of 256.
            int xi[4], yi[4];
            double wxy[4][4];
#pragma unroll
            for (int i = 0; i < 4; ++i) xi[i] = ax.idx[4 * xo + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                yi[j] = ay.idx[4 * yo + j];
                const double wy = ay.wt[4 * yo + j];
#pragma unroll
                for (int i = 0; i < 4; ++i) wxy[j][i] = ax.wt[4 * xo + i] * wy;
            }
            double acc = 0.0;
            for (int k = 0; k < 4; ++k) {
                const double wz = az.wt[4 * zo + k];
                const size_t bz = (size_t)az.idx[4 * zo + k] * wh;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const size_t by = bz + (size_t)yi[j] * w;
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const double wgt = wxy[j][i] * wz;
                        const size_t q = by + xi[i];
                        if (!TGV_IN_BOUNDS(q, wh * d, 42)) continue;
                        acc = acc + wgt * c[q];
                    }
                }
            }
            v = __double2float_rn(acc);
        }
        out[o] = v;
    }
}

int mirror_index(int k, int n) {
    if (n == 1) return 0;
    const int n2 = 2 * n - 2;
    if (k < 0) {
        k = -k;
        k -= n2 * (k / n2);
        if (k >= n) k = n2 - k;
    } else if (k >= n) {
        k -= n2 * (k / n2);
        if (k >= n) k = n2 - k;
    }
    return k;
}

// Host tables of one axis: out_keep samples of an out_grid-long grid over n inputs.
void axis_tables(int n, int out_grid, int out_keep, int* idx, double* wt, uint8_t* inside) {
    const float size_factor = (float)out_grid / (float)n;  // ResizeProcessor.cpp:70-72
    const double in_spacing = 1.0;
    const double out_spacing = in_spacing / (double)size_factor;
    for (int i = 0; i < out_keep; ++i) {
        const double x = ((double)i * out_spacing) * (1.0 / in_spacing);
        inside[i] = (x >= -0.5 && x < (double)n - 0.5) ? 1 : 0;
        const double fl = std::floor(x);
        const int base = (int)fl - 1;
        const double t = x - fl;
        double wv[4];
        wv[3] = (1.0 / 6.0) * t * t * t;
        wv[0] = (1.0 / 6.0) + 0.5 * t * (t - 1.0) - wv[3];
        wv[2] = t + wv[0] - 2.0 * wv[3];
        wv[1] = 1.0 - wv[0] - wv[2] - wv[3];
        for (int k = 0; k < 4; ++k) {
            idx[4 * i + k] = mirror_index(base + k, n);
            wt[4 * i + k] = wv[k];
        }
    }
}

size_t a256(size_t b) { return (b + 255) & ~size_t(255); }

size_t table_bytes(int W, int H, int D) {
    const size_t m = (size_t)W + H + D;
    return a256(m * 4 * sizeof(double)) + a256(m * 4 * sizeof(int)) + a256(m);
}

unsigned grid_for(size_t n, unsigned block) {
    size_t b = (n + block - 1) / block;
    if (b > 152 * 64) b = 152 * 64;
    return (unsigned)(b ? b : 1);
}

// The down-sampled deshade's full-resolution tail (TGVKDeshadeDownsampledProcessor.cpp:
// 114-125; NotMasked :100-114), one reference image operation per statement.
__global__ void downsampled_tail_kernel(const float* __restrict__ f, const float* __restrict__ mask,
                                        float* __restrict__ shading, float* __restrict__ r,
                                        size_t n, int not_masked, int clamp, int add_back) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float fi = f[i];
        float s = shading[i];
        float ri;
        if (!not_masked) {
            const float fin = mask ? fi * mask[i] : fi;  // the input times the mask (:59-60)
            ri = fin - s;                                // subtract (:114)
            if (mask) {
                s = s * mask[i];                         // :116
                ri = ri * mask[i];                       // :117
                shading[i] = s;
            }
        } else {
            ri = fi - s;
            if (mask) ri = ri * mask[i];
        }
        if (add_back && mask) ri = ri + fi * (1.f - mask[i]);  // background (:54-57, :120-121)
        if (clamp && ri < 0.f) ri = 0.f;                          // clamp_negative_values
        r[i] = ri;
    }
}

__global__ void multiply_kernel(const float* __restrict__ a, const float* __restrict__ b,
                                float* __restrict__ out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        out[i] = a[i] * b[i];
}

__global__ void fill_kernel(float* __restrict__ out, float v, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        out[i] = v;
}

}  // namespace

void downsampled_tail(const float* f, const float* mask, float* shading, float* r, size_t n,
                      bool not_masked, bool clamp, bool add_back, cudaStream_t st) {
    downsampled_tail_kernel<<<grid_for(n, 256), 256, 0, st>>>(f, mask, shading, r, n,
                                                               not_masked ? 1 : 0, clamp ? 1 : 0,
                                                               add_back ? 1 : 0);
    TGV_CHECK_LAUNCH();
}

void multiply_fields(const float* a, const float* b, float* out, size_t n, cudaStream_t st) {
    multiply_kernel<<<grid_for(n, 256), 256, 0, st>>>(a, b, out, n);
    TGV_CHECK_LAUNCH();
}

void fill_field(float* out, float v, size_t n, cudaStream_t st) {
    fill_kernel<<<grid_for(n, 256), 256, 0, st>>>(out, v, n);
    TGV_CHECK_LAUNCH();
}

uint64_t resize_bounds_take() {
    unsigned long long w = 0;
    TGV_CUDA(cudaMemcpyFromSymbol(&w, g_bounds_rs, sizeof(w)));
    if (w) {
        const unsigned long long zero = 0;
        TGV_CUDA(cudaMemcpyToSymbol(g_bounds_rs, &zero, sizeof(zero)));
    }
    return w;
}

unsigned resize_factor_extent(unsigned n, float factor) {
    const float e = std::ceil((float)n * factor);  // ResizeProcessor.cpp:38-45
    const unsigned u = (unsigned)e;
    return u < 1u ? 1u : u;
}

size_t resize_scratch_bytes(int w, int h, int d, int W, int H, int D) {
    return a256((size_t)w * h * d * sizeof(double)) + table_bytes(W, H, D);
}

void resize_bspline3(const float* in, int w, int h, int d, float* out, int W, int H, int D,
                     void* scratch, cudaStream_t st) {
    NvtxRange range("tgvdct resize");
    TGV_REQUIRE(w >= 1 && h >= 1 && d >= 1 && W >= 1 && H >= 1 && D >= 1,
                "resize extents must be >= 1");
    const bool up = W > w || H > h || D > d;
    const int gW = up ? W + 2 : W, gH = up ? H + 2 : H, gD = up ? D + 2 : D;
    const size_t n = (size_t)w * h * d;
    char* base = (char*)scratch;
    double* c = (double*)base;
    base += a256(n * sizeof(double));
    const size_t m = (size_t)W + H + D;
    double* wt_dev = (double*)base;
    int* idx_dev = (int*)(base + a256(m * 4 * sizeof(double)));
    uint8_t* in_dev = (uint8_t*)(base + a256(m * 4 * sizeof(double)) + a256(m * 4 * sizeof(int)));

    std::vector<double> wt(4 * m);
    std::vector<int> idx(4 * m);
    std::vector<uint8_t> inside(m);
    axis_tables(w, gW, W, idx.data(), wt.data(), inside.data());
    axis_tables(h, gH, H, idx.data() + 4 * W, wt.data() + 4 * W, inside.data() + W);
    axis_tables(d, gD, D, idx.data() + 4 * (W + H), wt.data() + 4 * (W + H),
                inside.data() + W + H);
    TGV_CUDA(cudaMemcpyAsync(wt_dev, wt.data(), wt.size() * sizeof(double),
                             cudaMemcpyHostToDevice, st));
    TGV_CUDA(cudaMemcpyAsync(idx_dev, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice,
                             st));
    TGV_CUDA(cudaMemcpyAsync(in_dev, inside.data(), m, cudaMemcpyHostToDevice, st));

    Pole p;
    p.z = std::sqrt(3.0) - 2.0;
    p.gain = (1.0 - p.z) * (1.0 - 1.0 / p.z);
    p.horizon = (long)std::ceil(std::log(1e-10) / std::log(std::fabs(p.z)));
    p.z2n[0] = std::pow(p.z, (double)(w - 1));
    p.z2n[1] = std::pow(p.z, (double)(h - 1));
    p.z2n[2] = std::pow(p.z, (double)(d - 1));

    to_double_kernel<<<grid_for(n, 256), 256, 0, st>>>(in, c, n);
    const unsigned B = 128;
    if (w > 1) prefilter_kernel<0><<<ceil_div((size_t)h * d, B), B, 0, st>>>(c, w, h, d, p);
    if (h > 1) prefilter_kernel<1><<<ceil_div((size_t)w * d, B), B, 0, st>>>(c, w, h, d, p);
    if (d > 1) prefilter_kernel<2><<<ceil_div((size_t)w * h, B), B, 0, st>>>(c, w, h, d, p);
    Axis ax{idx_dev, wt_dev, in_dev};
    Axis ay{idx_dev + 4 * W, wt_dev + 4 * W, in_dev + W};
    Axis az{idx_dev + 4 * (W + H), wt_dev + 4 * (W + H), in_dev + W + H};
    const size_t total = (size_t)W * H * D;
    evaluate_kernel<<<grid_for(total, 256), 256, 0, st>>>(c, w, h, d, ax, ay, az, out, W, H, D);
    TGV_CHECK_LAUNCH();
    // the tables were pageable host memory: each copy has staged them before returning
}

}  // namespace tgvdct
