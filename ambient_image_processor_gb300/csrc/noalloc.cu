// Allocation-free Poisson integration: tgvdct_integrate_poisson_noalloc_dev.
//
// Some callers of this library may not allocate device memory at all while they
// run the shading correction: a host application whose memory manager owns the
// whole GPU and forbids raw cudaMalloc, a pipeline with a fixed, pre-budgeted
// memory footprint, or a latency-critical loop where cudaMalloc / cudaFree would
// synchronise the device and stall other streams.  This entry point serves them.
// The caller still passes the input field v and the output l; the scratch the
// DCT passes need (two volumes and the per-axis cosine tables) lives in the
// file-scope device array below.  Every GPU that loads the library holds this
// array (about 18 MB) until the process exits.
//
// The array's host-side name is only a stand-in for the symbol, not a device
// address, so the host code below asks the runtime for the device address once
// per device (with that device current) and passes that pointer to the kernels.
#include <cmath>
#include <mutex>

#include "common.cuh"

namespace tgvdct {
namespace {

constexpr size_t kMaxVoxels = TGVDCT_NOALLOC_MAX_VOXELS;
constexpr size_t kMaxSide = TGVDCT_NOALLOC_MAX_SIDE;
// two scratch volumes, then per axis: forward matrix, inverse matrix, cospi(k/N),
// and the eigenvalue table
constexpr size_t kTableFloats = 2 * kMaxSide * kMaxSide + 2 * kMaxSide;
constexpr size_t kScratchFloats = 2 * kMaxVoxels + 3 * kTableFloats;

static __device__ __align__(256) float g_noalloc_scratch[kScratchFloats];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
float* g_scratch_addr[kMaxDevices] = {};

float* scratch_for_current_device() {
    int dev = 0;
    TGV_CUDA(cudaGetDevice(&dev));
    TGV_REQUIRE(dev >= 0 && dev < kMaxDevices, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        float* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            set_error(std::string("cudaGetSymbolAddress of the static scratch: ") +
                      cudaGetErrorString(e));
            throw Error{TGVDCT_ERR_CUDA};
        }
        g_scratch_addr[dev] = p;
    }
    return g_scratch_addr[dev];
}

// Fills one axis's tables: forward C[k][m] = cospi((m+1/2)k/N), inverse
// S[m][k] = w_k C[k][m], cospif(k/N) and 4 sin^2(pi k / 2N).  Every entry a call
// reads is rewritten here, so nothing left by an earlier call is used.
__global__ void fill_axis_tables(float* fwd, float* inv, float* cosk, float* eig, int N) {
    const int n2 = N * N;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n2; e += gridDim.x * blockDim.x) {
        const int k = e / N, m = e % N;
        const double c = cospi(((double)m + 0.5) * (double)k / (double)N);
        fwd[k * N + m] = (float)c;
        inv[m * N + k] = (float)(k == 0 ? c : 2.0 * c);
        if (m == 0) {
            cosk[k] = cospif((float)k / (float)N);
            const double s = sinpi((double)k / (2.0 * (double)N));
            eig[k] = (float)(4.0 * s * s);
        }
    }
}

}  // namespace
}  // namespace tgvdct

using namespace tgvdct;

extern "C" tgvdct_status tgvdct_integrate_poisson_noalloc_dev(
    const float* v_x_dev, const float* v_y_dev, const float* v_z_dev, uint32_t width,
    uint32_t height, uint32_t depth, int32_t dct_mode, int32_t poisson_eigen, float* l_dev,
    void* stream) {
    try {
        TGV_REQUIRE(v_x_dev && v_y_dev && l_dev && (v_z_dev || depth == 1), "null device buffer");
        TGV_REQUIRE(width >= 1 && height >= 1 && depth >= 1, "width, height, depth must be >= 1");
        TGV_REQUIRE(width <= kMaxSide && height <= kMaxSide && depth <= kMaxSide,
                    "tgvdct_integrate_poisson_noalloc_dev: every side must be <= "
                    "TGVDCT_NOALLOC_MAX_SIDE (256)");
        TGV_REQUIRE((size_t)width * height * depth <= kMaxVoxels,
                    "tgvdct_integrate_poisson_noalloc_dev: width*height*depth must be <= "
                    "TGVDCT_NOALLOC_MAX_VOXELS (2097152)");
        TGV_REQUIRE(poisson_eigen == TGVDCT_EIGEN_REFERENCE ||
                        poisson_eigen == TGVDCT_EIGEN_ACCURATE,
                    "unknown Poisson eigenvalue mode");
        // the tensor-core modes keep their matrices in allocations of a context's plan
        if (dct_mode != TGVDCT_DCT_FP32) {
            set_error("tgvdct_integrate_poisson_noalloc_dev: only TGVDCT_DCT_FP32 runs without "
                      "allocating (the tensor-core modes need a context's plan)");
            return TGVDCT_ERR_UNSUPPORTED;
        }
        float* base = scratch_for_current_device();
        cudaStream_t s = (cudaStream_t)stream;
        DctPlan view;
        view.W = (int)width;
        view.H = (int)height;
        view.D = (int)depth;
        view.tmp[0] = base;
        view.tmp[1] = base + kMaxVoxels;
        const int N[3] = {(int)width, (int)height, (int)depth};
        for (int a = 0; a < 3; ++a) {
            float* t = base + 2 * kMaxVoxels + a * kTableFloats;
            view.fwd[a] = t;
            view.inv[a] = t + kMaxSide * kMaxSide;
            view.cosk[a] = t + 2 * kMaxSide * kMaxSide;
            view.eig[a] = t + 2 * kMaxSide * kMaxSide + kMaxSide;
            const int n2 = N[a] * N[a];
            fill_axis_tables<<<ceil_div((size_t)n2, 256), 256, 0, s>>>(view.fwd[a], view.inv[a],
                                                                         view.cosk[a], view.eig[a],
                                                                         N[a]);
            TGV_CHECK_LAUNCH();
        }
        poisson_integrate(&view, v_x_dev, v_y_dev, v_z_dev, l_dev, dct_mode, poisson_eigen, s);
        return TGVDCT_OK;
    } catch (const Error& e) {
        return e.status;
    } catch (...) {
        set_error("unexpected exception");
        return TGVDCT_ERR_CUDA;
    }
}
