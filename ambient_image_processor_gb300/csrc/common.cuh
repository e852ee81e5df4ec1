// Internal declarations shared by the kernel files and the C ABI.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <memory>
#include <string>

#include <nvtx3/nvToolsExt.h>

#include "tgvdct.h"

namespace tgvdct {

// ---- error plumbing -------------------------------------------------------
void set_error(const std::string& msg);

struct Error {
    tgvdct_status status;
};

#define TGV_CUDA(call)                                                                   \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            ::tgvdct::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));     \
            throw ::tgvdct::Error{e_ == cudaErrorMemoryAllocation ? TGVDCT_ERR_OOM       \
                                                                  : TGVDCT_ERR_CUDA};    \
        }                                                                                \
    } while (0)

#define TGV_CHECK_LAUNCH() TGV_CUDA(cudaGetLastError())

#define TGV_REQUIRE(cond, msg)                                \
    do {                                                      \
        if (!(cond)) {                                        \
            ::tgvdct::set_error(msg);                         \
            throw ::tgvdct::Error{TGVDCT_ERR_BAD_ARG};        \
        }                                                     \
    } while (0)

// ---- TGV2 loop ---------------------------------------------------------------
// The fields an iteration reads with a stencil: ubar, vbar, p, q.  p (3 or 2
// components) and q (6 or 3) are stored in the state precision's element type.
struct TgvStencilFields {
    float* ubar = nullptr;
    float* vbar[3] = {nullptr, nullptr, nullptr};
    void* p[3] = {nullptr, nullptr, nullptr};
    void* q[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // xx yy zz xy xz yz
};

enum TgvKernel {
    TGV_KERNEL_TWO_PASS = 1,
    TGV_KERNEL_FUSED = 2,
    TGV_KERNEL_FUSED_REGISTER = 3,
    // runs of iterations as shifted passes (primal of n, dual of n + 1); single
    // iterations and the shapes it cannot take as TGV_KERNEL_FUSED
    TGV_KERNEL_SHIFTED = 4
};

// Bounds-checking builds (-DTGV_CHECK_BOUNDS, libtgvdct_checked.so): kernels check
// the indices they are about to use and record the first bad one instead of making
// the access.  Each translation unit keeps its own record word (a file-scope
// __device__ variable named by TGV_BOUNDS_WORD) and a host function that reads and
// clears it.  In normal builds the checks compile to nothing.
#ifdef TGV_CHECK_BOUNDS
constexpr bool kCheckBounds = true;
#else
constexpr bool kCheckBounds = false;
#endif
// True when 0 <= i < n; otherwise records (bit 63 set, site in bits 48..62, the
// index in bits 0..47) into *word unless something is recorded already.
__device__ __forceinline__ bool bounds_ok(long long i, long long n, int site,
                                          unsigned long long* word) {
    if (i >= 0 && i < n) return true;
    atomicCAS(word, 0ull,
              (1ull << 63) | ((unsigned long long)(site & 0x7fff) << 48) |
                  ((unsigned long long)i & 0xffffffffffffull));
    return false;
}
#define TGV_IN_BOUNDS(i, n, site) \
    (!kCheckBounds || bounds_ok((long long)(i), (long long)(n), (site), &TGV_BOUNDS_WORD))
// The record words of the units with checks (0 = nothing recorded); each call clears.
uint64_t tgv_kernels_bounds_take();
uint64_t adjoint_bounds_take();
uint64_t resize_bounds_take();

// An NVTX range over a host-side phase (deshade, loop, Poisson integration, resize,
// reverse sweep), for profilers that show ranges; free when none is attached.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// The first A-byte boundary at or after the shared-memory pointer p, as a pointer
// derived from p by pointer arithmetic.  The compiler then keeps the shared address
// space and accesses through the result are LDS / STS with 32-bit addresses; rounding
// through an integer (uintptr_t) loses it and turns every access into a generic load
// or store with 64-bit address arithmetic.
template <unsigned A, class T>
__device__ __forceinline__ T* align_shared(T* p) {
    static_assert((A & (A - 1)) == 0, "alignment must be a power of two");
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    return (T*)((uint8_t*)p + ((A - (a & (A - 1))) & (A - 1)));
}

// cudaFuncAttributeMaxDynamicSharedMemorySize is per device: raise it for `kern` once
// on every device that launches it (`done` holds one bit per device ordinal).
inline void smem_attr_once(const void* kern, size_t smem, std::atomic<uint64_t>& done) {
    int dev = 0;
    TGV_CUDA(cudaGetDevice(&dev));
    const uint64_t bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return;
    TGV_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    done.fetch_or(bit, std::memory_order_release);
}

// Device state of one volume.  Fields are planar (structure of arrays), x fastest.
// The two-pass kernels update set[0] in place.  The fused kernel reads set[cur]
// and writes set[cur ^ 1] (its halo recompute reads neighbours another block may
// already have advanced), so it needs the second set.
struct TgvState {
    int W = 0, H = 0, D = 0;
    bool three = true;       // 3-D operators (also for D == 1) vs the 2-D launcher
    int precision = TGVDCT_STATE_FP32;
    int kernel = TGV_KERNEL_FUSED;
    int zchunk = 32;         // planes per block of the fused kernel
    float* u = nullptr;
    float* f = nullptr;      // private copy of the input (log-domain runs rewrite it)
    float* v[3] = {nullptr, nullptr, nullptr};
    TgvStencilFields set[2];
    int cur = 0;
    // tensor maps of the TMA-pipelined fused kernel, one argument block per parity
    // (built on first use; the fused kernel falls back to register prefetch for
    // shapes the TMA stride rules exclude)
    std::shared_ptr<void> tma_cache;
    // tensor maps of the shifted passes (built on first use)
    std::shared_ptr<void> shifted_cache;
    int* err = nullptr;      // device flag raised by a pipeline wait that timed out
    // limit of the fused TMA kernel's pipeline waits (tgvdct_set_pipeline_wait_limit)
    uint64_t wait_ns = 200000000ull;
    // Optional domain of the masked deshade: voxels with domain[i] == 0 are never
    // updated and keep u = ubar = f, p = v = vbar = q = 0 (both sets of the fused
    // kernels hold those values).  Null: every voxel is updated.
    const uint8_t* domain = nullptr;
    // Per-block plane ranges of the fused TMA kernel's grid for that domain (built for
    // the z-chunk tile_zchunk): (first << 16) | end of the planes in which some of the
    // block's own voxels are in the domain, 0 when there are none.  The block works on
    // those planes only; the others are frozen.  Null: every block runs its chunk.
    const uint32_t* tile_active = nullptr;
    int tile_zchunk = 0;
    const TgvStencilFields& now() const { return set[cur]; }
};

struct TgvStep {
    float tau, sigma, theta, lambda, alpha0, alpha1;
    int data_term;
};

size_t tgv_state_bytes(int W, int H, int D, bool three, int precision, int kernel);
// Carves the state out of `base` (aligned to 256 bytes per field).
void tgv_state_bind(TgvState& s, char* base);
// u = ubar = f, p = q = v = vbar = 0 (in both sets of the fused kernels when a
// domain is set, so that skipped voxels read the same values from either set).
void tgv_state_init(TgvState& s, cudaStream_t st);
// domain[i] = mask[i] >= 1 (the masked processor's test, TGVDeshadeMaskedProcessor.cpp:347).
void build_domain(const float* mask, size_t n, uint8_t* domain, cudaStream_t st);
// Bytes of the fused kernel's per-block plane ranges (enough for any z-chunk).
size_t tgv_tile_flags_bytes(const TgvState& s);
// Fills `flags` from s.domain for the current z-chunk and points s.tile_active at it.
void tgv_build_tile_flags(TgvState& s, uint32_t* flags, cudaStream_t st);
// Snapshot of the whole loop state (f, u, v, and the current stencil set ubar, vbar,
// p, q) into or out of one contiguous device buffer of tgv_snapshot_bytes.
size_t tgv_snapshot_bytes(const TgvState& s);
void tgv_snapshot_save(const TgvState& s, void* dst, cudaStream_t st);
void tgv_snapshot_load(TgvState& s, const void* src, cudaStream_t st);
// One primal-dual iteration (advances s.cur for the fused kernel).
void tgv_iterate(TgvState& s, const TgvStep& k, cudaStream_t st);
// Number of kernels tgv_iterate launches.
int tgv_kernels_per_iteration(const TgvState& s);
// n iterations.  With TGV_KERNEL_SHIFTED (FP32, 3-D, depth >= 2, width a multiple of 4)
// and n >= 2 they run as a dual step, n - 1 shifted passes and a primal
// step; otherwise as n calls of tgv_iterate.  Either way the state ends in the
// standard form with the parity n single iterations give.  Returns the launches.
int tgv_iterate_n(TgvState& s, const TgvStep& k, uint32_t n, cudaStream_t st);
// Whether tgv_iterate_n runs shifted passes for this state.
bool tgv_uses_shifted(const TgvState& s);
// Sets the launch attributes of the kernels tgv_iterate_n may launch (before a
// stream capture).
void tgv_prepare_launches(const TgvState& s);
// Whether the fused kernel of this state runs the TMA pipeline.
bool tgv_uses_tma(const TgvState& s);

// ---- reverse mode (adjoint.cu) ---------------------------------------------------------
// One full FP32 state of the loop: 17 contiguous V-sized fields.
struct TgvFullDev {
    float* u = nullptr;
    float* ubar = nullptr;
    float* v[3] = {nullptr, nullptr, nullptr};
    float* vbar[3] = {nullptr, nullptr, nullptr};
    float* p[3] = {nullptr, nullptr, nullptr};
    float* q[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // xx yy zz xy xz yz
};
size_t tgv_full_state_bytes(size_t n);
void tgv_full_state_bind(TgvFullDev& s, char* base, size_t n);
void tgv_full_state_zero(const TgvFullDev& s, size_t n, cudaStream_t st);
// Copies the loop's current state (u, v and the current stencil set) into `out`.
void tgv_save_state(const TgvState& s, const TgvFullDev& out, cudaStream_t st);
// One FP32 iteration from `in` to `out` (distinct buffers), the same arithmetic as
// every forward kernel (they agree bit for bit). Where the shape allows TMA it runs
// the TMA kernel, whose tensor maps of each (in, out) pair are encoded once and kept
// in `cache`; otherwise the two-pass kernels.
void tgv_step_fp32(const TgvState& s, const TgvStep& k, const TgvFullDev& in,
                   const TgvFullDev& out, std::shared_ptr<void>& cache, cudaStream_t st);
// Adjoint of the `len` iterations states[0] -> ... -> states[len] (len + 1 states):
// How a segment's reverse passes run: R3.R1 and R2 as separate passes, or the fused pass
// (R3 of one iteration with R1 and R2 of the one before) between them -- always, or
// when its grid is at least three waves of two blocks per SM (below that the separate
// one-voxel passes fill the GPU better: 96^3 ran 14.1 ms fused against 13.6 ms).
enum AdjointPasses { ADJ_SEPARATE = 0, ADJ_FUSED_LARGE = 1, ADJ_FUSED = 2 };
// A holds the adjoint of states[len] on entry and of states[0] on return; accumulates
// d/df into grad_f and d/d(lambda, alpha0, alpha1) into gp[0..2]; uta and va are
// scratch (1 + 3 fields).  A2 is a second adjoint state of the same layout: the fused
// passes write from one into the other, and the two descriptors are swapped after
// each, so that on return A names the one holding the result.
void tgv_adjoint_segment(const TgvState& s, const TgvStep& k, const TgvFullDev* states,
                         int len, AdjointPasses passes, TgvFullDev& A, TgvFullDev& A2,
                         float* uta, float* const* va, float* grad_f, double* gp,
                         cudaStream_t st);
// grad_f += a(u_0) + a(ubar_0) (the loop starts from u = ubar = f).
void tgv_adjoint_finish(float* grad_f, const TgvFullDev& A, size_t n, cudaStream_t st);

// ---- TGV2 primal energy (metrics.cu) ------------------------------------------------
// sums[0..2] = sum |u - f| (L1) or (u - f)^2 / 2 (L2), sum |F u - v|, sum |E v|_F over
// every voxel (FP64 sums of FP32 terms); the energy is lambda sums[0] + alpha1 sums[1]
// + alpha0 sums[2].  vz is unused when !three.
void tgv_energy_terms(const float* f, const float* u, const float* vx, const float* vy,
                      const float* vz, int W, int H, int D, bool three, int data_term,
                      double* sums, cudaStream_t st);

// ---- cubic B-spline resize (resize.cu) -------------------------------------------
// ceil(n * factor) in float, at least 1: ResizeProcessor::process(image, factor).
unsigned resize_factor_extent(unsigned n, float factor);
// Device scratch of resize_bspline3 (FP64 coefficients of the input and the tables).
size_t resize_scratch_bytes(int w, int h, int d, int W, int H, int D);
// ResizeProcessor::process(image, W, H, D, BSpline3): in is w x h x d, out W x H x D.
void resize_bspline3(const float* in, int w, int h, int d, float* out, int W, int H, int D,
                     void* scratch, cudaStream_t st);
// The down-sampled deshade's tail at full resolution: r from the input f, the
// up-sampled shading (multiplied by the mask in place in the masked variant), the
// mask (may be null), the background add-back and the clamp.
void downsampled_tail(const float* f, const float* mask, float* shading, float* r, size_t n,
                      bool not_masked, bool clamp, bool add_back, cudaStream_t st);
void multiply_fields(const float* a, const float* b, float* out, size_t n, cudaStream_t st);
void fill_field(float* out, float v, size_t n, cudaStream_t st);

// ---- Poisson integration -------------------------------------------------------
// Per-shape cosine tables and scratch of the Poisson integration.
struct DctPlan {
    int W = 0, H = 0, D = 0;
    float* fwd[3] = {nullptr, nullptr, nullptr};   // C (N x N) per axis
    float* inv[3] = {nullptr, nullptr, nullptr};   // S (N x N) per axis
    float* cosk[3] = {nullptr, nullptr, nullptr};  // cospif(k / N), device-evaluated
    float* eig[3] = {nullptr, nullptr, nullptr};   // 4 sin^2(pi k / 2N)
    // 2 cosk * 2^32 as exact integers (sides <= 256; null otherwise): the FP64-free
    // form of the reference eigenvalues (poisson_den_ref)
    long long* cosk_fx[3] = {nullptr, nullptr, nullptr};
    float* tmp[2] = {nullptr, nullptr};            // two V-sized scratch volumes
    void* block = nullptr;                         // owning allocation (null for views)
    // tensor-core operands (sides <= 256): per axis, forward and inverse matrices
    // as BF16 hi/lo pairs and as TF32-rounded FP32, row-major N x N
    uint16_t* bf_hi[2][3] = {};                    // [fwd, inv][axis]
    uint16_t* bf_lo[2][3] = {};
    float* tf[2][3] = {};
    int* dev_err = nullptr;                        // set by a tensor-core pass whose wait timed out
    // limit of the pipelined tensor-core passes' waits (tgvdct_set_pipeline_wait_limit)
    uint64_t wait_ns = 200000000ull;
    void* tc_block = nullptr;
    // pipelined tensor-core passes (dct_tc2.cu): the matrices as shared-memory stage
    // images, [BF16X3, TF32][fwd, inv][axis], and their number of K stages
    void* pipe_img[2][2][3] = {};
    int pipe_chunks[2][2][3] = {};
    void* pipe_block = nullptr;
};
// Tensor-core passes need every side <= 256.
bool dct_tc_supported(const DctPlan* p);
// Prepares the tensor-core operands of a plan (allocates them once).
void dct_plan_prepare_tc(DctPlan* p);
// Reads (and clears) the device error flag of the tensor-core passes; synchronises.
bool dct_tc_check(DctPlan* p, cudaStream_t st);
// One separable pass on the tensor cores; epi: 0 none, 1 scale, 2/3 Poisson division
// (reference / accurate eigenvalues) on the last forward pass; div: the operand is
// the divergence of (vx, vy, vz) (x pass).
void pass_tc(DctPlan* p, int axis, bool inverse, const float* in, float* out, int epi, float scale,
             bool div, const float* vx, const float* vy, const float* vz, int dct_mode,
             cudaStream_t st);
// Pipelined tensor-core pass (TMA-fed, warp-specialised): returns false, doing
// nothing, where its rules exclude the plan or the buffers (then pass_tc applies).
bool dct_pipe_supported(const DctPlan* p);
bool pass_pipe(DctPlan* p, int axis, bool inverse, const float* in, float* out, int epi,
               float scale, int dct_mode, cudaStream_t st);
// tmp_voxels: size of each of the two scratch volumes (0: W * H * D)
DctPlan* dct_plan_create(int W, int H, int D, size_t tmp_voxels = 0);
void dct_plan_destroy(DctPlan* p);
size_t dct_plan_bytes(int W, int H, int D, size_t tmp_voxels = 0);
// z-slab decomposition of poisson_integrate (FP32): the divergence and the forward x, y
// passes over a slab's planes; the forward and inverse z passes (with the division) on
// a pencil of `columns` columns starting at column col_off of the W*H plane (a plan of
// the whole volume's shape whose scratch holds D * columns); the inverse y, x passes
// (x scaled) over `planes` planes.
void slab_poisson_xy(DctPlan* p, const float* vx, const float* vy, const float* vz, float* out,
                     cudaStream_t st);
void pencil_poisson_z(DctPlan* p, const float* in, float* out, long long columns,
                      long long col_off, int eigen_mode, cudaStream_t st);
void slab_poisson_inverse_yx(DctPlan* p, const float* in, float* out, int planes, float scale,
                             cudaStream_t st);

// l = DCT-III( DCT-II(div v) / eigenvalue ) with the reference's scale factors.
void poisson_integrate(DctPlan* plan, const float* vx, const float* vy, const float* vz,
                       float* l, int dct_mode, int eigen_mode, cudaStream_t st);
// l = DCT-III( DCT-II(rhs) / eigenvalue ): the Poisson solve of a given right-hand side.
void poisson_solve(DctPlan* plan, const float* rhs, float* l, int dct_mode, int eigen_mode,
                   cudaStream_t st);
// The separate steps of the reference's CudaImageOperationsProcessor.
void divergence(DctPlan* plan, const float* vx, const float* vy, const float* vz, float* out,
                cudaStream_t st);
void cosine_transform(DctPlan* plan, const float* in, float* out, int dct_mode, cudaStream_t st);
void inverse_cosine_transform(DctPlan* plan, const float* in, float* out, int dct_mode,
                              cudaStream_t st);
void solve_poisson(DctPlan* plan, const float* in, float* out, int eigen_mode, cudaStream_t st);

// ---- element-wise ------------------------------------------------------------
// The reference's Poisson denominator (float)(base - 2a - 2b - 2c), evaluated by
// solve_poisson_in_cosine_domain.cu:48-53 in FP64 from the float cosines a, b, c of
// the three frequencies (c = 0 in 2-D), without FP64 arithmetic (a small fraction of
// the FP32 rate on this GPU).  For sides <= 256 every float cospi(k / N) is 0 or at
// least sin(pi / 512) > 2^-8 in magnitude, so 2 cospi(k / N) is an integer multiple
// of 2^-32 and the FP64 sum is exact.  The plan keeps t[k] = 2 cospi(k / N) * 2^32 as
// 64-bit integers (DctPlan::cosk_fx, checked exact when built); the sum
// S = base * 2^32 - t0 - t1 - t2 is then exact, 0 <= S < 2^36, and
// fixed32_to_float rounds S * 2^-32 once to float: bit-identical to the FP64 form.
__device__ __forceinline__ float fixed32_to_float(long long S) {
    const unsigned long long u = (unsigned long long)S;
    const float hi = __uint2float_rn((unsigned)(u >> 12));                  // < 2^24: exact
    const float lo = __uint2float_rn((unsigned)(u & 4095u)) * 2.44140625e-4f;  // exact, < 1
    return (hi + lo) * 9.5367431640625e-07f;  // one rounding, then 2^-20 (exact)
}
__device__ __forceinline__ float poisson_den_ref(int three, const long long* t0,
                                                 const long long* t1, const long long* t2,
                                                 const float* c0, const float* c1,
                                                 const float* c2, int kx, int ky, int kz) {
    if (t0) {
        long long S = (three ? 6ll : 4ll) * 4294967296ll - t0[kx] - t1[ky];
        if (three) S -= t2[kz];
        return fixed32_to_float(S);
    }
    double den = (three ? 6.0 : 4.0) - 2.0 * (double)c0[kx] - 2.0 * (double)c1[ky];
    if (three) den -= 2.0 * (double)c2[kz];
    return (float)den;
}

// One check of the convergence test:// One check of the convergence test: appends (ncc(l, l_before), sum |l - l_before|)
// to slot[0..1] (FP64 device memory).  sums: 8 zeroed doubles of scratch, left zeroed.
void convergence_metrics(const float* l, const float* l_before, size_t n, double* sums,
                         double* slot, cudaStream_t st);
// Adjoint of poisson_integrate: (gvx, gvy, gvz) = B^T M gl, M the DCT Poisson solve
// (symmetric); scratch: V floats distinct from the plan's.  gvz unused when D == 1.
void poisson_integrate_adjoint(DctPlan* p, const float* gl, float* scratch, float* gvx,
                               float* gvy, float* gvz, int dct_mode, int eigen_mode,
                               cudaStream_t st);
void deshade_epilogue(const float* u, float* l, const float* mask, size_t n, bool mask_shading,
                      bool clamp, bool add_back, float* r, cudaStream_t st,
                      bool mask_again = false);
void log_inplace(float* x, size_t n, cudaStream_t st);
void exp_inplace(float* x, size_t n, cudaStream_t st);

inline unsigned ceil_div(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

}  // namespace tgvdct
