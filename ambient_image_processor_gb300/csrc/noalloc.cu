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
// array (about 19 MB) until the process exits.
//
// The array's host-side name is only a stand-in for the symbol, not a device
// address, so the host code below asks the runtime for the device address and
// passes that pointer to the kernels.  The look-up is set-up work done once per
// device context (with that device current): the address is kept together with
// the context's process-unique id, and looked up again whenever the current
// context has another id (after cudaDeviceReset, or a context the caller made
// current), so a kept address never outlives the module load it came from.
#include <cuda.h>
#include <cudaTypedefs.h>

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
// then, for every side N = 1 .. kMaxSide, the exact fixed-point form of 2 cospi(k/N)
// (kMaxSide 64-bit entries per side, two floats each), and one word for the set-up
// check of that form
constexpr size_t kFxOffset = 2 * kMaxVoxels + 3 * kTableFloats;
constexpr size_t kFlagOffset = kFxOffset + 2 * kMaxSide * kMaxSide;
constexpr size_t kScratchFloats = kFlagOffset + 64;
static_assert(kFxOffset % 2 == 0, "the fixed-point tables need 8-byte alignment");

static __device__ __align__(256) float g_noalloc_scratch[kScratchFloats];

// fx[(N - 1) * kMaxSide + k] = 2 cospif(k / N) * 2^32 as an integer, for every side
// N <= kMaxSide (block N - 1, thread k), exactly as the context plans build it;
// raises *inexact where the float is not an integer multiple of 2^-32.
__global__ void fill_fixed_point_cosines(long long* fx, int* inexact) {
    const int N = (int)blockIdx.x + 1;
    const int k = (int)threadIdx.x;
    if (k >= N) return;
    const float v = cospif((float)k / (float)N) * 8589934592.f;  // 2^33: exact scaling
    const long long t = __float2ll_rn(v);
    fx[(size_t)(N - 1) * kMaxSide + k] = t;
    if ((float)t != v) atomicExch(inexact, 1);
}

struct DeviceScratch {
    float* base = nullptr;
    unsigned long long ctx_id = 0;
    bool fx_exact = false;
};

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
DeviceScratch g_scratch[kMaxDevices];

// The process-unique id of the context current on this thread; false when no
// context is current yet (the runtime makes the device's primary context current
// on its first call, e.g. the symbol look-up below).
bool current_context_id(unsigned long long* id) {
    static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
    static PFN_cuCtxGetId_v12000 get_id = nullptr;
    if (!get_current || !get_id) {
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 4000, cudaEnableDefault,
                                             &qa) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) !=
                cudaSuccess ||
            qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || !a || !b)
            return false;
        get_current = (PFN_cuCtxGetCurrent_v4000)a;
        get_id = (PFN_cuCtxGetId_v12000)b;
    }
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return false;
    return get_id(ctx, id) == CUDA_SUCCESS;
}

// Set-up for the current device and context: the device address of the static
// array (checked), and the fixed-point cosine tables of every side with their
// exactness check (one synchronous read of one word).  Allocates nothing.
DeviceScratch& scratch_for_current_device() {
    int dev = 0;
    TGV_CUDA(cudaGetDevice(&dev));
    TGV_REQUIRE(dev >= 0 && dev < kMaxDevices, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceScratch& d = g_scratch[dev];
    unsigned long long id = 0;
    if (d.base && current_context_id(&id) && id == d.ctx_id) return d;
    float* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
        d.base = nullptr;
        set_error(std::string("cudaGetSymbolAddress of the static scratch: ") +
                  cudaGetErrorString(e));
        throw Error{TGVDCT_ERR_CUDA};
    }
    // the look-up made the primary context current if none was
    if (!current_context_id(&id)) {
        d.base = nullptr;
        set_error("no current CUDA context after the static scratch look-up");
        throw Error{TGVDCT_ERR_CUDA};
    }
    int* flag = (int*)(p + kFlagOffset);
    int inexact = 1;
    e = cudaMemset(flag, 0, sizeof(int));
    if (e == cudaSuccess) {
        fill_fixed_point_cosines<<<(unsigned)kMaxSide, (unsigned)kMaxSide>>>(
            (long long*)(p + kFxOffset), flag);
        e = cudaGetLastError();
    }
    // the synchronous copy waits for the set-up kernel (same legacy stream)
    if (e == cudaSuccess) e = cudaMemcpy(&inexact, flag, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        d.base = nullptr;
        set_error(std::string("static scratch set-up: ") + cudaGetErrorString(e));
        throw Error{TGVDCT_ERR_CUDA};
    }
    d.base = p;
    d.ctx_id = id;
    d.fx_exact = inexact == 0;
    return d;
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
        DeviceScratch& scratch = scratch_for_current_device();
        float* base = scratch.base;
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
            // the exact fixed-point form of the reference eigenvalues, as the context
            // plans use it (null: the FP64 form, only if the set-up check failed)
            view.cosk_fx[a] = scratch.fx_exact ? (long long*)(base + kFxOffset) +
                                                     (size_t)(N[a] - 1) * kMaxSide
                                               : nullptr;
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
