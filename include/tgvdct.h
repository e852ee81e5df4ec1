/*
 * tgvdct.h — C ABI of the GB300-native TGV-DCT shading-correction path.
 *
 * One data-parallel hot path of josefkoller/ambient_image_processor, rebuilt for
 * sm_103a: the TGV2 primal-dual loop (L1 or L2 data term, Neumann boundaries) that
 * produces the denoised image u and the bias gradient field v, followed by the
 * DCT-II Poisson solve that integrates v into the smooth shading field l, and the
 * deshade epilogue r = u - l.
 *
 * Conventions shared by every entry point:
 *   - Images are float32, x fastest: index = z*width*height + y*width + x
 *     (the reference's ITKImage layout, source/modules/itk/ITKImage.cpp:84).
 *   - Functions return a tgvdct_status; they never print-and-exit the way the
 *     reference's cudaCheckError does (source/modules/cuda/cuda_helper.in:11-21).
 *     tgvdct_last_error() describes the last failure on the calling thread.
 *   - "_launch" entry points take HOST buffers owned by the caller and do their
 *     own host<->device copies, like the reference launchers; the caller
 *     allocates the outputs (the reference returned new[] arrays instead).
 *   - "_dev" entry points take DEVICE buffers and a cudaStream_t (passed as
 *     void*, NULL = the legacy default stream) and are asynchronous unless a
 *     callback forces a synchronisation.
 *   - A context (tgvdct_context) owns the device workspace of one volume shape;
 *     one context must not be used by two threads at the same time.  Distinct
 *     contexts are independent.
 */
#ifndef TGVDCT_H
#define TGVDCT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TGVDCT_VERSION_MAJOR 0
#define TGVDCT_VERSION_MINOR 1

typedef enum tgvdct_status {
    TGVDCT_OK = 0,
    TGVDCT_ERR_BAD_ARG = 1,     /* invalid shape, parameter or null pointer */
    TGVDCT_ERR_OOM = 2,         /* device or host allocation failed */
    TGVDCT_ERR_CUDA = 3,        /* a CUDA runtime call or kernel launch failed */
    TGVDCT_ERR_NO_DEVICE = 4,   /* no CUDA device, or not an sm_103 device */
    TGVDCT_ERR_UNSUPPORTED = 5, /* a mode this library does not provide */
    TGVDCT_STOPPED = 6,         /* the loop ended early: the iteration callback or
                                   tgvdct_request_stop asked to stop, or the energy
                                   tolerance was met; outputs hold the state after
                                   the last iteration run (tgvdct_iterations_run) */
    TGVDCT_ERR_TIMEOUT = 7      /* a bounded wait inside a kernel ran out (a TMA
                                   pipeline stage that never landed); the kernel
                                   returned without finishing and the context is
                                   still usable */
} tgvdct_status;

typedef enum tgvdct_data_term {
    TGVDCT_DATA_L1 = 0, /* |u - f|: tgv_cuda/tgv2_l1.cu:27-60 */
    TGVDCT_DATA_L2 = 1  /* (u - f)^2 / 2: tgv_cuda/tgv2_l2.cu:27-56 */
} tgvdct_data_term;

typedef enum tgvdct_geometry {
    /* The 3-D launcher (tgv_deshade/tgv2_l1_deshade.cu), also for depth == 1 as
       the reference's terminal program runs 2-D images. */
    TGVDCT_GEOMETRY_3D = 0,
    /* The 2-D launcher (tgv_deshade/tgv2_l1_deshade_2d.cu): two gradient
       components, q = (xx, yy, xy).  Requires depth == 1. */
    TGVDCT_GEOMETRY_2D = 1
} tgvdct_geometry;

typedef enum tgvdct_state_precision {
    TGVDCT_STATE_FP32 = 0,      /* every field stored in FP32 (the plain drop-in) */
    TGVDCT_STATE_BF16_DUAL = 1, /* dual fields p, q stored in BF16, updates in FP32 */
    TGVDCT_STATE_FX16_DUAL = 2  /* p, q stored as 16-bit fixed point scaled by alpha1 /
                                   alpha0 (the projections bound every component by
                                   alpha), updates in FP32 */
} tgvdct_state_precision;

typedef enum tgvdct_dct_mode {
    TGVDCT_DCT_FP32 = 0,   /* FP32 FMA contractions on the CUDA cores */
    TGVDCT_DCT_TF32 = 1,   /* tensor cores (tcgen05), one TF32 product */
    TGVDCT_DCT_BF16X3 = 2  /* tensor cores (tcgen05), BF16 hi/lo split, three
                              products, FP32 accumulation */
} tgvdct_dct_mode;

typedef enum tgvdct_iteration_kernel {
    TGVDCT_KERNEL_AUTO = 0,     /* shifted passes for volumes, the two-pass kernels
                                   for a single plane (depth 1) */
    /* two coalesced passes per iteration (dual, then primal), every field updated
       in place: 176 bytes per voxel-iteration in FP32 */
    TGVDCT_KERNEL_TWO_PASS = 1,
    /* one pass per iteration: z-marching tiles that recompute the one-voxel halo
       of the dual fields on chip, input planes streamed in by TMA; the
       stencil-read fields are double-buffered: 140 bytes per voxel-iteration */
    TGVDCT_KERNEL_FUSED = 2,
    /* the fused pass with the input planes staged through registers instead of
       the TMA pipeline (the fused kernel uses it by itself when the width is not a
       multiple of 4, or of 8 with 16-bit dual fields) */
    TGVDCT_KERNEL_FUSED_REGISTER = 3,
    /* runs of iterations as shifted passes: each pass does the primal step of one
       iteration and the dual step of the next, so ubar and vbar stay on chip and a
       voxel-iteration moves 108 bytes (FP32 state, 3-D, depth >= 2, width a
       multiple of 4; masked runs too); one dual step before a run and one primal step
       after it (the two-pass kernels) convert the state.  Single iterations and the
       cases it does not take run as TGVDCT_KERNEL_FUSED.  Same bits as the others.
       The reverse sweep (tgvdct_tgv2_backward_dev) runs its fused adjoint pass (R3 of
       one iteration with R1 and R2 of the one before) with this kernel always, with
       TGVDCT_KERNEL_AUTO for volumes large enough to fill the GPU three times over,
       and separate adjoint passes otherwise; the gradients are the same bits. */
    TGVDCT_KERNEL_FUSED_SHIFTED = 4
} tgvdct_iteration_kernel;

typedef enum tgvdct_poisson_eigen {
    /* 6 - 2cospi(kx/W) - 2cospi(ky/H) - 2cospi(kz/D) with FP32 cosines summed in
       FP64, as solve_poisson_in_cosine_domain.cu:48-53 computes it. */
    TGVDCT_EIGEN_REFERENCE = 0,
    /* 4sin^2(pi kx/2W) + 4sin^2(pi ky/2H) + 4sin^2(pi kz/2D): the same value
       without the cancellation near the zero frequency. */
    TGVDCT_EIGEN_ACCURATE = 1
} tgvdct_poisson_eigen;

/* Parameters of one deshade.  tgvdct_params_init() fills the reference defaults. */
typedef struct tgvdct_params {
    uint32_t width, height, depth;
    float lambda;             /* data-term weight */
    float alpha0;             /* second-order weight: bounds q */
    float alpha1;             /* first-order weight: bounds p */
    uint32_t iteration_count;
    float tau, sigma, theta;  /* 1/sqrt(20), 1/sqrt(20), 1 in the reference
                                 (tgv_deshade/tgv2_l1_deshade.cu:148-150) */
    int32_t data_term;        /* tgvdct_data_term */
    int32_t geometry;         /* tgvdct_geometry */
    int32_t state_precision;  /* tgvdct_state_precision */
    int32_t dct_mode;         /* tgvdct_dct_mode */
    int32_t poisson_eigen;    /* tgvdct_poisson_eigen */
    uint32_t paint_iteration_interval; /* callback cadence; 0 = never */
    int32_t callback_on_device;        /* 0: callback gets host copies (reference
                                          behaviour); 1: device pointers */
    int32_t iteration_kernel;          /* tgvdct_iteration_kernel */
    int32_t z_chunk;                   /* planes per block of the fused kernel; 0 = auto */
    /* Stopping on the primal energy (no counterpart in the reference, which always
       runs iteration_count iterations): every energy_check_interval iterations
       (0 = never) the loop evaluates the TGV2 energy of (u, v) (tgvdct_tgv2_energy)
       and, when energy_tolerance > 0, stops after the first check whose energy
       differs from the previous check's by at most energy_tolerance x |energy|.  The
       call then returns TGVDCT_STOPPED; tgvdct_iterations_run gives the count and
       tgvdct_energy_history the energies. */
    uint32_t energy_check_interval;
    float energy_tolerance;
} tgvdct_params;

/* Called after iteration `iteration_index` when iteration_index > 0 and
   iteration_index % paint_iteration_interval == 0 (tgv_cuda/tgv2_common.cu:381-384).
   u, v_x, v_y, v_z are valid only during the call; v_z is NULL for 2-D geometry.
   Return nonzero to stop the loop (the reference's `return true`). */
typedef int (*tgvdct_iteration_callback)(uint32_t iteration_index, uint32_t iteration_count,
                                         const float* u, const float* v_x, const float* v_y,
                                         const float* v_z, void* user);

typedef struct tgvdct_context tgvdct_context;

/* ---- library ------------------------------------------------------------ */
const char* tgvdct_version(void);
const char* tgvdct_status_string(tgvdct_status s);
const char* tgvdct_last_error(void);
void tgvdct_params_init(tgvdct_params* p);
/* Bytes of device memory a context for these parameters allocates. */
size_t tgvdct_workspace_bytes(const tgvdct_params* p);

/* ---- device buffers for hosts without a CUDA runtime of their own ---------- */
/* cudaMalloc / cudaFree / blocking cudaMemcpy on the current device, for callers
   (FFI bindings, the reference-signature C++ layer) that hand device buffers to
   the _dev entry points without linking the CUDA runtime themselves. */
tgvdct_status tgvdct_device_alloc(size_t bytes, void** out);
tgvdct_status tgvdct_device_free(void* p);
tgvdct_status tgvdct_host_to_device(void* dst_dev, const void* src_host, size_t bytes);
tgvdct_status tgvdct_device_to_host(void* dst_host, const void* src_dev, size_t bytes);

/* ---- contexts (device workspace of one shape) --------------------------- */
tgvdct_status tgvdct_create(const tgvdct_params* p, tgvdct_context** out);
tgvdct_status tgvdct_destroy(tgvdct_context* ctx);
/* Change lambda, alpha, iterations, steps, data term, modes or callback cadence
   of a context; the shape, geometry and state precision must stay the same. */
tgvdct_status tgvdct_set_params(tgvdct_context* ctx, const tgvdct_params* p);
/* Number of iterations the last run completed (less than iteration_count when a
   callback stopped it). */
uint32_t tgvdct_iterations_run(const tgvdct_context* ctx);
/* Number of iteration kernels (fused or shifted passes and the two-pass kernels)
   the last loop of the context launched, graph replays included. */
uint64_t tgvdct_loop_launches(const tgvdct_context* ctx);

/* ---- the TGV2 loop ------------------------------------------------------ */
/* Replaces tgv2_l1_deshade_launch<float> (tgv_deshade/tgv2_l1_deshade.cu:33-41),
   the reference's TGV2-L1 deshade loop: host f in, host u and v out.  The 3-D
   operators run also when depth == 1, so v_z holds their z component then, as
   in the reference.  cuda_block_dimension is accepted for signature
   compatibility and ignored (launch shapes are chosen for sm_103a). */
tgvdct_status tgvdct_tgv2_l1_deshade_launch(const float* f_host, uint32_t width, uint32_t height,
                                            uint32_t depth, float lambda,
                                            uint32_t iteration_count,
                                            uint32_t paint_iteration_interval,
                                            int cuda_block_dimension,
                                            tgvdct_iteration_callback callback, void* user,
                                            float alpha0, float alpha1, float* u_host,
                                            float* v_x_host, float* v_y_host, float* v_z_host);

/* Replaces tgv2_l1_deshade_launch_2d<float> (tgv_deshade/tgv2_l1_deshade_2d.cu:29-36). */
tgvdct_status tgvdct_tgv2_l1_deshade_launch_2d(const float* f_host, uint32_t width,
                                               uint32_t height, float lambda,
                                               uint32_t iteration_count,
                                               uint32_t paint_iteration_interval,
                                               tgvdct_iteration_callback callback, void* user,
                                               float alpha0, float alpha1, float* u_host,
                                               float* v_x_host, float* v_y_host);

/* General host-buffer form of the loop: every parameter of tgvdct_params (data
   term, geometry, steps, precision), host f in, host u out; v_x/v_y/v_z_host may
   each be NULL (not copied out; v_z is zero for 2-D geometry).  With a callback,
   it is called as in tgvdct_tgv2_l1_deshade_launch (host copies).  Backs the
   reference-signature tgv2_l1_launch / tgv2_l2_launch (tgv_cuda/tgv2_l1.cu:64-72,
   tgv_cuda/tgv2_l2.cu:60-68), whose iteration callback sees u. */
tgvdct_status tgvdct_tgv2_run(const tgvdct_params* p, const float* f_host, float* u_host,
                             float* v_x_host, float* v_y_host, float* v_z_host,
                             tgvdct_iteration_callback callback, void* user);

/* Replaces tgv2_l1_launch / tgv2_l2_launch (tgv_cuda/tgv2_l1.cu:64-72,
   tgv_cuda/tgv2_l2.cu:60-68): the TGV filter's denoise loop, u only. */
tgvdct_status tgvdct_tgv2_denoise_launch(const float* f_host, uint32_t width, uint32_t height,
                                         uint32_t depth, int32_t data_term, float lambda,
                                         uint32_t iteration_count, float alpha0, float alpha1,
                                         float* u_host);

/* General form: every parameter of tgvdct_params, device buffers, stream.
   v_z_dev may be NULL for 2-D geometry.  f_dev is not modified. */
tgvdct_status tgvdct_tgv2_run_dev(tgvdct_context* ctx, const float* f_dev, float* u_dev,
                                  float* v_x_dev, float* v_y_dev, float* v_z_dev,
                                  tgvdct_iteration_callback callback, void* user, void* stream);

/* ---- reverse mode (no counterpart in the reference) ------------------------ */
/* The loop of tgvdct_tgv2_run_dev (iteration_count iterations from u = ubar = f),
   keeping a copy of the full state every `checkpoint_every` iterations on the
   context for tgvdct_tgv2_backward_dev.  Needs FP32 state and 3-D geometry.
   Device memory: ceil(K / checkpoint_every) states of 17 fields. */
tgvdct_status tgvdct_tgv2_forward_checkpointed_dev(tgvdct_context* ctx, const float* f_dev,
                                                   float* u_dev, float* v_x_dev,
                                                   float* v_y_dev, float* v_z_dev,
                                                   uint32_t checkpoint_every, void* stream);
/* Gradient of a loss through the last checkpointed forward run of this context:
   given dL/du_K (and dL/dv_K, each may be NULL for zero), writes dL/df to
   grad_f_dev and (dL/dlambda, dL/dalpha0, dL/dalpha1) as three doubles to
   grad_params_dev.  Recomputes each segment from its checkpoint (checkpoint_every
   + 1 further states of device memory) and runs the adjoint iteration backwards:
   the transposes of the difference operators and the Jacobians of the
   projections and of the prox (taken on the branch the forward run took).
   The context's f (from the forward call) and parameters must be unchanged. */
tgvdct_status tgvdct_tgv2_backward_dev(tgvdct_context* ctx, const float* grad_u_dev,
                                       const float* grad_v_x_dev, const float* grad_v_y_dev,
                                       const float* grad_v_z_dev, float* grad_f_dev,
                                       double* grad_params_dev, void* stream);

/* ---- Poisson integration of v (DCT-II / DCT-III) -------------------------- */
/* Each replaces the host-in/host-out launcher of the same name:
   divergence_kernel_launch (cuda_image_operations/divergence.cu:59-61; depth == 1
   uses the 2-D kernels as CudaImageOperationsProcessor.cpp:290-291 does),
   cosine_transform_kernel_launch (cosine_transform.cu:226-227),
   solve_poisson_in_cosine_domain_kernel_launch (solve_poisson_in_cosine_domain.cu:86-87),
   inverse_cosine_transform_kernel_launch (inverse_cosine_transform.cu:167-168). */
tgvdct_status tgvdct_divergence_launch(const float* dx, const float* dy, const float* dz,
                                       uint32_t width, uint32_t height, uint32_t depth,
                                       float* out);
/* Device form of divergence_kernel_launch with is_host_data == false
   (divergence.cu:59-61, whose inputs are device buffers): out_dev = B_x dx +
   B_y dy (+ B_z dz when depth > 1), the negated backward differences.
   Synchronises the stream before returning. */
tgvdct_status tgvdct_divergence_dev(const float* dx_dev, const float* dy_dev,
                                    const float* dz_dev, uint32_t width, uint32_t height,
                                    uint32_t depth, float* out_dev, void* stream);
tgvdct_status tgvdct_cosine_transform_launch(const float* in, uint32_t width, uint32_t height,
                                             uint32_t depth, int32_t dct_mode, float* out);
tgvdct_status tgvdct_inverse_cosine_transform_launch(const float* in, uint32_t width,
                                                     uint32_t height, uint32_t depth,
                                                     int32_t dct_mode, float* out);
tgvdct_status tgvdct_solve_poisson_in_cosine_domain_launch(const float* in, uint32_t width,
                                                           uint32_t height, uint32_t depth,
                                                           int32_t poisson_eigen, float* out);

/* Replaces TGVDeshadeProcessor::integrate_image_gradients_poisson_cosine_transform
   (tgv_deshade/TGVDeshadeProcessor.cpp:386-408, 2-D :410-431): l from v. */
tgvdct_status tgvdct_integrate_image_gradients_poisson_cosine_transform(
    const float* v_x, const float* v_y, const float* v_z, uint32_t width, uint32_t height,
    uint32_t depth, int32_t dct_mode, int32_t poisson_eigen, float* l_out);

/* Device form on a context: l_dev from v on the device (v_z_dev may be NULL when
   depth == 1).  Uses the context's dct_mode and poisson_eigen. */
tgvdct_status tgvdct_poisson_integrate_dev(tgvdct_context* ctx, const float* v_x_dev,
                                           const float* v_y_dev, const float* v_z_dev,
                                           float* l_dev, void* stream);

/* The DCT Poisson solve of a given right-hand side on a context's plan: l =
   iDCT(DCT(rhs) / eigenvalue), DC set to zero, i.e. the reference's
   cosineTransform -> solvePoissonInCosineDomain -> inverseCosineTransform chain
   (CudaImageOperationsProcessor.cpp:240-284, solve_poisson_in_cosine_domain.cu)
   without its three host round trips.  Uses the context's dct_mode and
   poisson_eigen; device buffers, stream-ordered. */
tgvdct_status tgvdct_poisson_solve_dev(tgvdct_context* ctx, const float* rhs_dev, float* l_dev,
                                       void* stream);
/* Adjoint of tgvdct_poisson_integrate_dev (no counterpart in the reference): given
   dL/dl, writes dL/dv = B^T M dL/dl, where l = M (B_x v_x + B_y v_y + B_z v_z), B the
   negated backward differences and M the DCT Poisson solve (a symmetric operator).
   Uses the context's dct_mode and poisson_eigen; grad_v_z_dev may be NULL when
   depth == 1 (the 2-D divergence has no z term; it is zeroed otherwise).  Synchronises
   the stream. */
tgvdct_status tgvdct_poisson_integrate_adjoint_dev(tgvdct_context* ctx, const float* grad_l_dev,
                                                   float* grad_v_x_dev, float* grad_v_y_dev,
                                                   float* grad_v_z_dev, void* stream);
/* Reads and clears the device error flags of a context: the TGV iteration kernels'
   and the tensor-core DCT passes' (raised when one of their bounded waits ran out);
   synchronises the stream.  Returns TGVDCT_ERR_TIMEOUT if a flag was set. */
tgvdct_status tgvdct_check_device_error(tgvdct_context* ctx, void* stream);
/* The limit, in nanoseconds, of the bounded waits with which the fused TMA iteration
   kernel and the pipelined tensor-core DCT passes of this context wait for their
   staged data: default 200 ms; 0 gives up at the first test that finds the data not
   yet there.  A wait that runs out raises the context's device error flag; the pass
   stops, each of its blocks first letting its own copies and tensor-core operations
   in flight finish (those waits always allow 200 ms), and later launches return at
   once.  tgvdct_check_device_error (or the next host-buffer call) then returns
   TGVDCT_ERR_TIMEOUT and clears the flag; the context stays usable.  No counterpart
   in the reference, whose cudaCheckError prints and exits (cuda_helper.in:11-21). */
tgvdct_status tgvdct_set_pipeline_wait_limit(tgvdct_context* ctx, uint64_t limit_ns);

/* Allocation-free form of tgvdct_poisson_integrate_dev.  It has no counterpart in
   the reference.  It is for callers that must not allocate device memory while
   they run (their memory manager owns the GPU, their footprint is fixed in
   advance, or a cudaMalloc/cudaFree would synchronise a latency-critical
   pipeline): it calls no cudaMalloc, cudaFree or other allocating routine.  Its
   scratch is one static device array of the library (about 19 MB, held by every
   GPU that loads the library until the process exits), which limits the volume
   to TGVDCT_NOALLOC_MAX_VOXELS voxels with every side <= TGVDCT_NOALLOC_MAX_SIDE;
   larger volumes are rejected with TGVDCT_ERR_BAD_ARG.  The first call in each
   device context does set-up: it looks up the array's device address and fills
   the array's exact fixed-point cosine tables, with one synchronous read on the
   legacy default stream (make that first call before any stream capture).  A
   context with a new id (after cudaDeviceReset, for one) gets the set-up again.
   All calls share the one array: calls that overlap on the
   GPU (different streams, no ordering between them) race and corrupt each
   other's results, so order them, e.g. on one stream.  The caller passes v on
   the device (v_z_dev may be NULL when depth == 1) and the output l_dev.  Only
   dct_mode TGVDCT_DCT_FP32 is available here (TGVDCT_ERR_UNSUPPORTED otherwise). */
#define TGVDCT_NOALLOC_MAX_VOXELS (1u << 21)
#define TGVDCT_NOALLOC_MAX_SIDE 256u
tgvdct_status tgvdct_integrate_poisson_noalloc_dev(const float* v_x_dev, const float* v_y_dev,
                                                   const float* v_z_dev, uint32_t width,
                                                   uint32_t height, uint32_t depth,
                                                   int32_t dct_mode, int32_t poisson_eigen,
                                                   float* l_dev, void* stream);

/* ---- deshade epilogue and the whole processor ----------------------------- */
/* Device form of TGVDeshadeProcessor::deshade_poisson_cosine_transform's tail
   (TGVDeshadeProcessor.cpp:83-92) plus the background add-back (:275-279):
   r = u - l; with a mask, l *= mask (when mask_shading) and r *= mask; clamp
   r < 0 to 0; add u*(1-mask) back.  mask_dev may be NULL. */
tgvdct_status tgvdct_deshade_epilogue_dev(const float* u_dev, float* l_dev, const float* mask_dev,
                                          uint64_t voxel_count, int32_t mask_shading,
                                          int32_t set_negative_values_to_zero,
                                          int32_t add_background_back, float* r_dev,
                                          void* stream);

/* Replaces TGVDeshadeProcessor::processTGV2L1GPUCuda (TGVDeshadeProcessor.cpp:122-166
   for the terminal program; :285-314 with a mask, callback and add-back for the
   GUI module): denoised u, shading l and deshaded r from f, host buffers.
   mask may be NULL.  With log_domain, f is replaced by log(f) before the loop and
   the three outputs are exponentiated (the multiplicative-bias use). */
tgvdct_status tgvdct_process_tgv2_l1(const tgvdct_params* p, const float* f_host,
                                     const float* mask_host, int32_t set_negative_values_to_zero,
                                     int32_t add_background_back, int32_t log_domain,
                                     tgvdct_iteration_callback callback, void* user,
                                     float* denoised_host, float* shading_host,
                                     float* deshaded_host);

/* The host-buffer one-shot calls (tgvdct_process_tgv2_l1, tgvdct_process_tgv2_l1_masked,
   tgvdct_tgv2_run, tgvdct_tgv2_l1_deshade_launch, tgvdct_tgv2_l1_deshade_launch_2d,
   tgvdct_tgv2_l1_deshade_masked_launch, tgvdct_tgv2_denoise_launch) keep their last
   context and its device buffers between calls, so that volumes of one shape streamed
   through them pay the state allocation, the DCT plan and the graph captures once.
   One entry, keyed by the parameters, the call and the current device; a concurrent
   or re-entrant call uses a private context; a failed call drops the entry.  This
   frees the entry: the TGV state and the call's device buffers.
   No replacement: the reference allocates and frees inside each call.  Returns
   TGVDCT_ERR_BAD_ARG while a call holds the entry. */
tgvdct_status tgvdct_release_cached(void);

/* Device form of the whole deshade on a context (no host copies): f_dev in; u,
   l, r out; mask_dev may be NULL.  Stream-ordered. */
tgvdct_status tgvdct_process_dev(tgvdct_context* ctx, const float* f_dev, const float* mask_dev,
                                 int32_t set_negative_values_to_zero, int32_t add_background_back,
                                 int32_t log_domain, float* u_dev, float* l_dev, float* r_dev,
                                 tgvdct_iteration_callback callback, void* user, void* stream);

/* ---- convergence metrics ------------------------------------------------------ */
/* Replaces TGVDeshadeProcessor::processTGV2L1DeshadeCuda_convergenceTest and
   ..._convergenceTestMetric (tgv_deshade/TGVDeshadeProcessor.cpp:479-568): runs the
   TGV loop of p (callback cadence check_iteration_interval) and at every check
   integrates l from v (times the mask when mask_host is given).  From the second
   check on it records the normalised cross-correlation of l with the previous
   check's l (normalised with the current l's mean for both images, as the reference
   does, :190-193) and their time total variation sum |l - l_before|.  The first
   `capacity` pairs go to ncc_history / time_tv_history, their number to
   *history_count (may be NULL).  metric_tv[0], [1]: the total variation of each
   series over the checks, sum |h[i+1] - h[i]| for i < count - 2 (the reference's
   bound).  Sums are FP64 on the device (the reference accumulates in float). */
tgvdct_status tgvdct_convergence_test(const tgvdct_params* p, const float* f_host,
                                      const float* mask_host, uint32_t check_iteration_interval,
                                      double* ncc_history, double* time_tv_history,
                                      uint32_t capacity, uint32_t* history_count,
                                      double* metric_tv);

/* Replaces TGVDeshadeProcessor::processTGV2L1DeshadeCuda_convergenceOptimization
   (TGVDeshadeProcessor.cpp:571-646): picks alpha1 = alpha0 = 10^-i by the first decade
   whose 10-iteration NCC-series TV drops, then alpha0 / alpha1 among {1, 1.5, 1.8, 2,
   2.2, 2.3, 2.35, 2.4, 2.45} by the largest time-TV-series TV, and runs the 500-iteration
   deshade with them (r weighted by the mask if given, then clamped if asked).  p gives
   lambda and the modes; its alphas and iteration count are not used. */
tgvdct_status tgvdct_convergence_optimization(const tgvdct_params* p, const float* f_host,
                                              const float* mask_host,
                                              int32_t set_negative_values_to_zero,
                                              float* alpha0_out, float* alpha1_out,
                                              float* denoised_host, float* shading_host,
                                              float* deshaded_host);

/* ---- masked deshade (tgv_deshade_masked/) ---------------------------------- */
/* Restricts the TGV loop of a context to the voxels whose mask value is >= 1
   (TGVDeshadeMaskedProcessor::buildMaskIndices, TGVDeshadeMaskedProcessor.cpp:337-385):
   the others are never updated and keep u = f and p = v = q = 0, and the
   difference operators at updated voxels read those values, as the reference's
   masked kernels do (tgv2_masked_common.cu, tgv_masked_common.cu).  The mask is
   copied; with a mask set, tgvdct_process_dev also applies the masked processor's
   epilogue (l and r weighted by the mask, then the background add-back or a second
   multiply of r by the mask; its mask_dev argument must be NULL).  NULL clears.
   The reverse mode refuses a context with a mask. */
tgvdct_status tgvdct_set_domain_mask_dev(tgvdct_context* ctx, const float* mask_dev, void* stream);

/* Replaces TGVDeshadeMaskedProcessor::processTGV2L1GPUCuda
   (TGVDeshadeMaskedProcessor.cpp:77-212, 2-D :214-330): the masked loop (2-D
   operators when depth == 1, whatever p->geometry says, as the reference chooses),
   the Poisson integration of v, and the masked epilogue.  Host buffers. */
tgvdct_status tgvdct_process_tgv2_l1_masked(const tgvdct_params* p, const float* f_host,
                                            const float* mask_host,
                                            int32_t set_negative_values_to_zero,
                                            int32_t add_background_back, int32_t log_domain,
                                            tgvdct_iteration_callback callback, void* user,
                                            float* denoised_host, float* shading_host,
                                            float* deshaded_host);

/* Replaces tgv2_l1_deshade_masked_launch<float> (tgv_deshade_masked/tgv2_l1_deshade_masked.cu)
   and tgv2_l1_deshade_masked_2d_launch (depth == 1): the masked loop alone.  The
   mask replaces the reference's index lists (voxels with mask >= 1; the face lists
   follow from the shape).  v_z_host may be NULL; it is zero when depth == 1. */
tgvdct_status tgvdct_tgv2_l1_deshade_masked_launch(
    const float* f_host, const float* mask_host, uint32_t width, uint32_t height, uint32_t depth,
    float lambda, uint32_t iteration_count, uint32_t paint_iteration_interval,
    int cuda_block_dimension, tgvdct_iteration_callback callback, void* user, float alpha0,
    float alpha1, float* u_host, float* v_x_host, float* v_y_host, float* v_z_host);

/* ---- energy, stopping ------------------------------------------------------------ */
/* TGV2 primal energy of (u, v) for f with p's shape, geometry, data term and weights,
   using the operators as the reference implements them: F forward differences with
   Neumann ends, E from the negated backward differences with 1/2 on the mixed
   entries, Frobenius norm with weight 2 off the diagonal (tgv2_common.cu:96-276).
   energy[0] = lambda sum |u - f| (L1) or lambda sum (u - f)^2 / 2 (L2),
   energy[1] = alpha1 sum |F u - v|, energy[2] = alpha0 sum |E v|, energy[3] = their
   sum.  FP32 per voxel, FP64 sums on the device.  No counterpart in the reference.
   v_z may be NULL for 2-D geometry.  Host buffers; energy is host memory. */
tgvdct_status tgvdct_tgv2_energy(const tgvdct_params* p, const float* f_host,
                                 const float* u_host, const float* v_x_host,
                                 const float* v_y_host, const float* v_z_host, double* energy);
/* Device form: f, u, v device buffers; energy_dev receives the 3 unweighted sums
   (sum |u - f| or sum (u - f)^2 / 2, sum |F u - v|, sum |E v|).  Stream-ordered. */
tgvdct_status tgvdct_tgv2_energy_dev(const tgvdct_params* p, const float* f_dev,
                                     const float* u_dev, const float* v_x_dev,
                                     const float* v_y_dev, const float* v_z_dev,
                                     double* energy_dev, void* stream);
/* The energies (weighted totals) of the energy checks of the context's last loop, in
   order; *count receives how many there were (at most capacity are copied). */
tgvdct_status tgvdct_energy_history(tgvdct_context* ctx, double* out, uint32_t capacity,
                                    uint32_t* count);
/* Asks the loop running on ctx (or the next one started on it) to stop: it is polled
   between host-side launch steps (every iteration, or every 32 iterations where the
   loop replays them as one CUDA graph) and at callback and energy checks.  Safe to
   call from another thread.  The call that stops returns TGVDCT_STOPPED and clears
   the request.  No counterpart in the reference (whose callback return is the only
   way to stop). */
tgvdct_status tgvdct_request_stop(tgvdct_context* ctx);

/* ---- checkpoint / resume (no counterpart in the reference, which cannot resume) - */
/* Bytes of one snapshot of a context's loop state: f, u, v and the current ubar,
   vbar, p, q (p, q in the context's dual storage precision). */
size_t tgvdct_state_bytes(const tgvdct_context* ctx);
/* Copies the loop state left by the last run (or load) into dst_dev, a device buffer
   of tgvdct_state_bytes.  Stream-ordered. */
tgvdct_status tgvdct_state_save_dev(tgvdct_context* ctx, void* dst_dev, void* stream);
/* Replaces the context's loop state by a snapshot saved from a context with the same
   shape, geometry and dual precision.  Stream-ordered. */
tgvdct_status tgvdct_state_load_dev(tgvdct_context* ctx, const void* src_dev, void* stream);
/* Runs the context's iteration_count more iterations from its current state (after
   a run, or a load) instead of from u = f, p = q = v = 0, and writes u and v as
   tgvdct_tgv2_run_dev does.  A run of K1 iterations, then a resume of K2, gives the
   bits of one run of K1 + K2.  Callback and energy-check indices count from the
   start of the resumed run. */
tgvdct_status tgvdct_tgv2_resume_dev(tgvdct_context* ctx, float* u_dev, float* v_x_dev,
                                     float* v_y_dev, float* v_z_dev,
                                     tgvdct_iteration_callback callback, void* user,
                                     void* stream);

/* ---- z-slab decomposition (building blocks; no counterpart in the reference) ----
   The reference runs one volume on one device (tgv_cuda/tgv_common.cu:249-253).  To
   spread a volume over several GPUs along z, each rank holds a context for its slab of
   planes plus one halo plane on each side that has a neighbour; the host moves halo
   planes and pencils between ranks with its own transport (NCCL, MPI, ...).  After
   every iteration a rank copies its first own plane's ubar and vbar into the rank
   below (that rank's top halo) and its last own plane's into the rank above (its
   bottom halo).  p and q at the halo planes need no exchange: p takes forward
   differences of ubar and q backward differences of vbar, so the bottom halo's p and
   the top halo's q are computed exactly from the halo and the own plane next to it.
   Every own plane then advances exactly as in the single volume.
   ambient_image_processor_gb300/slab.py is the host side over torch.distributed. */
/* Field-mask bits of the loop state (ubar, vbar, p, q: the current stencil set). */
#define TGVDCT_FIELD_F (1u << 0)
#define TGVDCT_FIELD_U (1u << 1)
#define TGVDCT_FIELD_V (7u << 2)     /* v_x, v_y, v_z */
#define TGVDCT_FIELD_UBAR (1u << 5)
#define TGVDCT_FIELD_VBAR (7u << 6)  /* vbar_x, vbar_y, vbar_z */
#define TGVDCT_FIELD_P (7u << 9)     /* p_x, p_y, p_z */
#define TGVDCT_FIELD_Q (63u << 12)   /* q_xx, q_yy, q_zz, q_xy, q_xz, q_yz */
#define TGVDCT_FIELD_ALL ((1u << 18) - 1u)
/* what a rank's halo planes receive from its neighbours after every iteration */
#define TGVDCT_HALO_FIELDS (TGVDCT_FIELD_UBAR | TGVDCT_FIELD_VBAR)
/* The loop's starting state from f (u = ubar = f, p = q = v = vbar = 0), no iteration. */
tgvdct_status tgvdct_state_init_dev(tgvdct_context* ctx, const float* f_dev, void* stream);
/* Advances the state by `iterations` iterations (no callbacks, no output copies). */
tgvdct_status tgvdct_tgv2_step_dev(tgvdct_context* ctx, uint32_t iterations, void* stream);
/* Bytes that tgvdct_state_read_dev / _write_dev move for these fields and planes
   (p, q in the context's dual element size); 0 for a bad mask. */
size_t tgvdct_state_planes_bytes(const tgvdct_context* ctx, uint32_t field_mask,
                                 uint32_t plane_count);
/* Copies planes [plane_begin, plane_begin + plane_count) of each field of the mask, in
   bit order, field after field, out of (read) or into (write) one device buffer.
   Stream-ordered. */
tgvdct_status tgvdct_state_read_dev(tgvdct_context* ctx, uint32_t field_mask,
                                    uint32_t plane_begin, uint32_t plane_count, void* dst_dev,
                                    void* stream);
tgvdct_status tgvdct_state_write_dev(tgvdct_context* ctx, uint32_t field_mask,
                                     uint32_t plane_begin, uint32_t plane_count,
                                     const void* src_dev, void* stream);
/* The Poisson integration of tgvdct_poisson_integrate_dev split for z-slabs (FP32
   contractions, dct_mode TGVDCT_DCT_FP32).  Its single-volume order is: divergence
   fused into the forward x pass, forward y, forward z with the eigenvalue division,
   inverse z, inverse y, inverse x (scaled).  A rank runs
     1. tgvdct_slab_poisson_xy_dev on its context's planes (v with the bottom halo
        plane's v_z from the rank below): divergence, forward x, forward y;
     2. sends each rank its columns of its own planes and receives its pencil: all D
        planes of the columns [column_begin, column_begin + columns) of the W*H plane;
     3. tgvdct_pencil_poisson_z_dev: forward z, division, inverse z on the pencil;
     4. sends the pencil back by planes and receives its own planes;
     5. tgvdct_slab_poisson_inverse_yx_dev over its own planes: inverse y, inverse x
        scaled by 1 / (8 W H total_depth).
   Every value is the same dot product, summed in the same order, as in the single
   volume: the slab result equals tgvdct_poisson_integrate_dev's bit for bit. */
tgvdct_status tgvdct_slab_poisson_xy_dev(tgvdct_context* ctx, const float* v_x_dev,
                                         const float* v_y_dev, const float* v_z_dev,
                                         float* out_dev, void* stream);
tgvdct_status tgvdct_slab_poisson_inverse_yx_dev(tgvdct_context* ctx, const float* in_dev,
                                                 float* out_dev, uint32_t plane_count,
                                                 uint32_t total_depth, void* stream);
typedef struct tgvdct_pencil tgvdct_pencil;
/* A pencil of the width x height x depth volume: `columns` columns, all depth planes
   (z-major, columns contiguous), with the z cosine tables and D * columns of scratch. */
tgvdct_status tgvdct_pencil_create(uint32_t width, uint32_t height, uint32_t depth,
                                   uint64_t columns, tgvdct_pencil** out);
tgvdct_status tgvdct_pencil_destroy(tgvdct_pencil* pencil);
tgvdct_status tgvdct_pencil_poisson_z_dev(tgvdct_pencil* pencil, const float* in_dev,
                                          float* out_dev, uint64_t column_begin,
                                          int32_t poisson_eigen, void* stream);

/* ---- bounds checking (a device-side stand-in for compute-sanitizer) -------------- */
/* In libtgvdct_checked.so (built with -DTGV_CHECK_BOUNDS) the iteration, adjoint and
   resize kernels check the indices they use and record the first bad one instead of
   making the access.  This call waits for the device, then returns that record
   (0: none; else bit 63 set, a site number in bits 48..62, the index in bits 0..47)
   and clears it.  The normal library returns TGVDCT_ERR_UNSUPPORTED.  No counterpart
   in the reference. */
tgvdct_status tgvdct_bounds_check(uint64_t* first_bad);

/* ---- down-sampled deshade (tgvk_deshade_downsampled/, resize/) ---------------- */
/* Replaces ResizeProcessor::process(image, width, height, depth, BSpline3)
   (resize/ResizeProcessor.cpp:49-143): ITK's cubic B-spline resample as that function
   sets it up (output spacing = input spacing / (float)(out / in) per axis, origin 0;
   when any axis grows, a grid two samples longer per axis of which the first
   out_width x out_height x out_depth are kept).  FP64 coefficients and sums, like
   ITK; float out.  Device form: stream-ordered, synchronises before returning. */
tgvdct_status tgvdct_resize_bspline3(const float* in_host, uint32_t width, uint32_t height,
                                     uint32_t depth, float* out_host, uint32_t out_width,
                                     uint32_t out_height, uint32_t out_depth);
tgvdct_status tgvdct_resize_bspline3_dev(const float* in_dev, uint32_t width, uint32_t height,
                                         uint32_t depth, float* out_dev, uint32_t out_width,
                                         uint32_t out_height, uint32_t out_depth, void* stream);
/* ceil(n * factor) in float, at least 1: the extent ResizeProcessor::process(image,
   size_factor, ...) gives (ResizeProcessor.cpp:35-47). */
uint32_t tgvdct_resize_factor_extent(uint32_t n, float factor);

/* Replaces TGVKDeshadeDownsampledProcessor::processTGVKL1Cuda
   (tgvk_deshade_downsampled/TGVKDeshadeDownsampledProcessor.cpp:30-129) and, with
   not_masked = 1, TGVKDeshadeDownsampledNotMaskedProcessor::processTGVKL1Cuda
   (TGVKDeshadeDownsampledNotMaskedProcessor.cpp:30-129): resize the image (the masked
   variant: the image times the mask) and the mask by downsampling_factor, deshade
   there, resize the denoised image and the shading back, and form the deshaded image
   at full resolution.  The inner deshade is the masked TGV2 processor (masked
   variant) or the plain one with the mask in its epilogue (not_masked), which is what
   the reference runs for order 2, with alpha0 = alpha[1] and alpha1 = alpha[0]
   (TGVKDeshadeMaskedProcessor.cpp:98-103, TGVKDeshadeProcessor.cpp:137-147).  Other
   orders return TGVDCT_ERR_UNSUPPORTED.  mask and div_v may be NULL; div_v is the
   up-sampled divergence of v (calculate_div_v).  The callback sees the down-sampled
   u, l, r.  A factor of 1 skips both resizes, as the reference does. */
tgvdct_status tgvdct_process_tgvk_l1_downsampled(
    const float* f_host, const float* mask_host, uint32_t width, uint32_t height, uint32_t depth,
    float downsampling_factor, float lambda, uint32_t order, const float* alpha,
    uint32_t iteration_count, int32_t set_negative_values_to_zero, int32_t add_background_back,
    int32_t not_masked, uint32_t paint_iteration_interval, tgvdct_iteration_callback callback,
    void* user, float* denoised_host, float* shading_host, float* deshaded_host,
    float* div_v_host);
tgvdct_status tgvdct_process_tgvk_l1_downsampled_dev(
    const float* f_dev, const float* mask_dev, uint32_t width, uint32_t height, uint32_t depth,
    float downsampling_factor, float lambda, uint32_t order, const float* alpha,
    uint32_t iteration_count, int32_t set_negative_values_to_zero, int32_t add_background_back,
    int32_t not_masked, uint32_t paint_iteration_interval, tgvdct_iteration_callback callback,
    void* user, float* denoised_dev, float* shading_dev, float* deshaded_dev, float* div_v_dev,
    void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TGVDCT_H */
