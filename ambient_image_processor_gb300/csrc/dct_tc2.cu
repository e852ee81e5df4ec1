// Tensor-core DCT passes, pipelined (sides <= 256, width a multiple of 4).
//
// A separable pass along one axis is D[m][k] = sum_n A[m][n] * M[k][n]: m runs over
// the 128 lines of a CTA, n over the axis, k over the N output frequencies (or
// samples), M is the N x N cosine matrix.  One CTA owns a 128 x N tile of D in TMEM
// (128 lanes x N FP32 columns).  The K dimension (the axis) streams through a
// shared-memory pipeline of 192 KB (3 stages for BF16x3, 6 for TF32); each stage
// holds a 64-byte slice of every row of both operands:
//
//   producer (warp 9, one lane)   TMA: the FP32 input slab, 128 lines x KE samples,
//                                 straight from the volume (2-D or 3-D tensor map);
//                                 bulk copy: the matching slice of M, which the plan
//                                 stores once in the shared-memory image the MMA
//                                 reads (BF16 hi and lo, or TF32).  Both complete on
//                                 the stage's `full` mbarrier.
//   converters (warps 0-7)        FP32 slab -> BF16 hi/lo (or TF32) in the canonical
//                                 K-major no-swizzle layout; arrive on `conv`.
//   MMA issuer (warp 8, one lane) tcgen05.mma kind::f16 (three products, hi*hi +
//                                 hi*lo + lo*hi) or kind::tf32, then tcgen05.commit
//                                 to the stage's `empty` mbarrier, which frees the
//                                 stage for the producer.
//   epilogue (warps 10-13)        tcgen05.ld of the accumulator, scale or Poisson
//                                 division, coalesced stores, while the next tile's
//                                 MMAs fill the other TMEM accumulator (persistent
//                                 CTAs, one per SM, two 128 x N accumulators).
//
// Canonical layout of a stage's operand tile (rows r, byte cb of the 64-byte slice):
// 8-row x 16-byte core matrices, K-adjacent ones 128 bytes apart (LBO) and 8-row groups
// 512 bytes apart (SBO).  One MMA consumes 32 bytes of K (16 BF16 or 8 TF32 values),
// two per stage.
//
// Every mbarrier wait is bounded; a timeout raises the plan's device error flag and a
// shared abort flag, every role leaves its loop, the copies and MMAs already issued
// are waited for (bounded), TMEM is freed and the CTA returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "common.cuh"

namespace tgvdct {
namespace {

constexpr int P_M = 128;          // lines per CTA (MMA M)
// 18 warps: 8 converters, MMA, producer, 8 epilogue.  Two epilogue warps share each
// TMEM lane quarter (warp % 4) and drain half of the columns each: with the Poisson
// division in the epilogue, four warps could not keep up with the tensor core (the z
// pass of a 256^3 solve took 158 us against 63 us with a plain scale).
constexpr int P_EPI_WARPS = 16;
constexpr int P_THREADS = 32 * (10 + P_EPI_WARPS);
constexpr int P_CONV = 256;       // converter threads (warps 0-7)
constexpr int P_MMA_WARP = 8, P_PROD_WARP = 9;  // epilogue: warps 10-17
constexpr int P_STAGES_MAX = 6;
constexpr int P_RB = 64;          // bytes per row per stage (K slice)
constexpr int P_NMAX = 256;
constexpr uint64_t P_WAIT_NS = 200000000ull;  // 200 ms: a stage normally lands in microseconds

enum PMode { PM_BF16X3 = 0, PM_TF32 = 1 };
enum PAxis { PA_X = 0, PA_Y = 1, PA_Z = 2 };
enum PEpi { PE_NONE = 0, PE_SCALE = 1, PE_POISSON_REF = 2, PE_POISSON_ACC = 3 };

template <int MODE>
struct PGeo {
    static constexpr int KE = MODE == PM_BF16X3 ? 32 : 16;   // axis samples per stage
    static constexpr int RAW = P_M * KE * 4;                 // FP32 slab bytes
    static constexpr int ATILE = P_M * P_RB;                 // 8 KB per operand tile
    static constexpr int BTILE = P_NMAX * P_RB;              // 16 KB (max N)
    static constexpr int NB = MODE == PM_BF16X3 ? 2 : 1;     // hi (+ lo)
    static constexpr int OFF_B = RAW;
    static constexpr int OFF_A = OFF_B + NB * BTILE;
    static constexpr int STAGE = OFF_A + NB * ATILE;         // 64 KB (BF16x3) / 32 KB (TF32)
    static constexpr int NS = MODE == PM_BF16X3 ? 3 : 6;     // stages in 192 KB
};

struct PArgs {
    CUtensorMap in_map;   // FP32 input: 2-D (x pass: {N, lines}; z pass: {lines, N}) or 3-D
    float* out;
    const uint8_t* bimg;  // the matrix in stage images: nchunks x NB x (NP rows x 64 B)
    int NA, NP, nchunks;
    long long L;          // lines per batch
    int batches;
    int W, H, D;
    // output addressing: out[batch * SB + line * SL + k * sn]
    long long SL, SB, sn;
    float scale;
    int pz_layout;        // Poisson epilogue: 1: (kx = line, ky = k); 2: (kx, ky) = line, kz = k
    const float* cosk0;
    const float* cosk1;
    const float* cosk2;
    const float* eig0;
    const float* eig1;
    const float* eig2;
    const long long* fx0;  // DctPlan::cosk_fx (null: the FP64 form)
    const long long* fx1;
    const long long* fx2;
    int* err;
    unsigned long long wait_ns;  // limit of the roles' pipeline waits (0: one test)
};

__device__ __forceinline__ uint32_t su32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t gtimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ bool mtest(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(su32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait.  With honour_abort (the roles' pipeline waits), returns false as soon
// as another role gave up, and gives up after limit_ns (limit_ns == 0: at the first
// test that finds the phase open).  Without it (the drain of an error exit), waits up
// to P_WAIT_NS whatever limit_ns says.
__device__ bool mwait(uint64_t* bar, uint32_t parity, int* err, volatile int* abort,
                      bool honour_abort, uint64_t limit_ns = P_WAIT_NS) {
    if (mtest(bar, parity)) return true;
    if (!honour_abort) limit_ns = P_WAIT_NS;
    if (limit_ns == 0) {
        atomicExch(err, 1);
        *abort = 1;
        return false;
    }
    const uint64_t t0 = gtimer();
    while (true) {
        if (mtest(bar, parity)) return true;
        if (honour_abort && *abort) return false;
        if (gtimer() - t0 > limit_ns) {
            atomicExch(err, 1);
            *abort = 1;
            return false;
        }
        __nanosleep(64);
    }
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void tma_2d(void* dst, const CUtensorMap* map, int c0, int c1,
                                       uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3}], [%4];" ::"r"(su32(dst)),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(su32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                       uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(su32(dst)),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(su32(bar))
        : "memory");
}
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes,
                                          uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(su32(dst)),
        "l"((uint64_t)src), "r"(bytes), "r"(su32(bar))
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
    // K-major, no swizzle: start, LBO = 128 B (K-adjacent core matrices), SBO = 512 B
    // (8-row groups), descriptor version 1 (bit 46)
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)((128u >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((512u >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}
template <int MODE>
__host__ __device__ constexpr uint32_t idesc(int n) {
    // D FP32 (bit 4), A and B BF16 (kind::f16: 1) or TF32 (2), both K-major, M = 128
    const uint32_t ab = MODE == PM_BF16X3 ? 1u : 2u;
    return (1u << 4) | (ab << 7) | (ab << 10) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(P_M >> 4) << 24);
}
template <int MODE>
__device__ __forceinline__ void mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t id,
                                    uint32_t acc) {
    if constexpr (MODE == PM_BF16X3) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(a), "l"(b), "r"(id), "r"(acc)
            : "memory");
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(a), "l"(b), "r"(id), "r"(acc)
            : "memory");
    }
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            su32(bar))
        : "memory");
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
// Byte offset, in the x pass's FP32 slab ([P_M rows][KE floats]), of the 16-byte chunk
// c of row r as the TMA swizzle placed it: the chunk index within a 128-byte (64-byte)
// span is XORed with address bits 7-9 (7-8), i.e. with r & 7 for 128-byte rows and
// (r >> 1) & 3 for 64-byte rows.
template <int MODE>
__device__ __forceinline__ int xslab_off(int r, int c) {
    if constexpr (MODE == PM_BF16X3) return r * 128 + ((c ^ (r & 7)) << 4);
    else return r * 64 + ((c ^ ((r >> 1) & 3)) << 4);
}
__device__ __forceinline__ uint32_t tile_off(int r, int cb) {
    return (uint32_t)((r >> 3) * 512 + (cb >> 4) * 128 + (r & 7) * 16 + (cb & 15));
}
__device__ __forceinline__ uint32_t bf16_pack(float a, float b) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(a)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(b)) << 16);
}
__device__ __forceinline__ float tf32r(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// Converts 8 (BF16: hi and lo) or 4 (TF32) consecutive axis samples of line r, group j.
template <int MODE>
__device__ __forceinline__ void convert_group(const float* v, uint8_t* ahi, uint8_t* alo, int r,
                                              int j) {
    const uint32_t off = tile_off(r, j * 16);
    if constexpr (MODE == PM_BF16X3) {
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const float a = v[2 * t], b = v[2 * t + 1];
            const float ah = __bfloat162float(__float2bfloat16_rn(a));
            const float bh = __bfloat162float(__float2bfloat16_rn(b));
            hi[t] = bf16_pack(ah, bh);
            lo[t] = bf16_pack(a - ah, b - bh);
        }
        *(uint4*)(ahi + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
        *(uint4*)(alo + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    } else {
        *(float4*)(ahi + off) = make_float4(tf32r(v[0]), tf32r(v[1]), tf32r(v[2]), tf32r(v[3]));
    }
}

// Persistent: every CTA loops over the (line tile, batch) tiles t = blockIdx.x,
// blockIdx.x + gridDim.x, ...; the accumulator alternates between two TMEM buffers so
// that the epilogue warps drain tile i while the MMAs of tile i + 1 run.
template <int MODE, int AXIS, int EPI>
__global__ void __launch_bounds__(P_THREADS, 1) dct_pipe_kernel(const __grid_constant__ PArgs g) {
    using G = PGeo<MODE>;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* base = align_shared<1024>(smem_raw);
    constexpr int P_STAGES = G::NS;
    __shared__ uint64_t full[P_STAGES_MAX], conv[P_STAGES_MAX], empty[P_STAGES_MAX];
    __shared__ uint64_t acc_full[2], acc_empty[2];
    __shared__ uint32_t tmem_s;
    __shared__ int abort_s;
    __shared__ int consumed_s, issued_s, mma_chunks_s;

    if (__syncthreads_or(threadIdx.x == 0 ? *(volatile int*)g.err : 0)) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nch = g.nchunks;
    const long long ntl = (g.L + P_M - 1) / P_M;            // line tiles per batch
    const long long ntiles = ntl * g.batches;
    const uint32_t bchunk = (uint32_t)(G::NB * g.NP * P_RB);  // matrix bytes per stage
    uint32_t acols = 32;                                       // accumulator columns
    while (acols < (uint32_t)g.NP) acols <<= 1;
    const uint32_t ncols = 2 * acols;
    volatile int* abort = &abort_s;

    if (tid == 0) {
        for (int s = 0; s < P_STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&conv[s], P_CONV);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], P_EPI_WARPS);  // one arrival per epilogue warp
        }
        abort_s = 0;
        consumed_s = issued_s = mma_chunks_s = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         su32(&tmem_s)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = tmem_s;

    if (warp == P_PROD_WARP) {
        // ---- producer
        if (lane == 0) {
            int gc = 0;
            bool go = true;
            for (long long t = blockIdx.x; t < ntiles && go; t += gridDim.x) {
                const long long line0 = (t % ntl) * P_M;
                const int batch = (int)(t / ntl);
                for (int c = 0; c < nch; ++c, ++gc) {
                    const int s = gc % P_STAGES;
                    if (gc >= P_STAGES &&
                        !mwait(&empty[s], (uint32_t)((gc / P_STAGES - 1) & 1), g.err, abort, true, g.wait_ns)) {
                        go = false;
                        break;
                    }
                    uint8_t* st = base + s * G::STAGE;
                    mbar_expect_tx(&full[s], (uint32_t)G::RAW + bchunk);
                    const int k0 = c * G::KE;
                    if constexpr (AXIS == PA_X) tma_2d(st, &g.in_map, k0, (int)line0, &full[s]);
                    else if constexpr (AXIS == PA_Y)
                        tma_3d(st, &g.in_map, (int)line0, k0, batch, &full[s]);
                    else tma_2d(st, &g.in_map, (int)line0, k0, &full[s]);
                    bulk_copy(st + G::OFF_B, g.bimg + (size_t)c * bchunk, bchunk, &full[s]);
                }
            }
            issued_s = gc;
        }
    } else if (warp < P_CONV / 32) {
        // ---- converters (256 threads)
        int gc = 0;
        bool go = true;
        for (long long t = blockIdx.x; t < ntiles && go; t += gridDim.x) {
            for (int c = 0; c < nch; ++c, ++gc) {
                const int s = gc % P_STAGES;
                if (!mwait(&full[s], (uint32_t)((gc / P_STAGES) & 1), g.err, abort, true, g.wait_ns)) {
                    go = false;
                    break;
                }
                const float* raw = (const float*)(base + s * G::STAGE);
                uint8_t* ahi = base + s * G::STAGE + G::OFF_A;
                uint8_t* alo = ahi + G::ATILE;
                constexpr int GS = MODE == PM_BF16X3 ? 8 : 4;   // samples per 16-byte group
                constexpr int NU = P_M * (G::KE / GS) / P_CONV;  // units per thread: 2
#pragma unroll
                for (int i = 0; i < NU; ++i) {
                    const int u = tid + P_CONV * i;             // 512 units: (line, group)
                    float v[8];
                    if constexpr (AXIS == PA_X) {
                        // slab [128 lines][KE], swizzled: lanes cover consecutive lines of
                        // one group, so that neither these reads nor the writes of
                        // convert_group meet bank conflicts
                        const int r = u & 127, j = u >> 7;
                        const uint8_t* rb = (const uint8_t*)raw;
                        constexpr int CPG = GS / 4;  // 16-byte chunks per group
                        const float4 a = *(const float4*)(rb + xslab_off<MODE>(r, j * CPG));
                        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
                        if constexpr (GS == 8) {
                            const float4 b = *(const float4*)(rb + xslab_off<MODE>(r, j * CPG + 1));
                            v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
                        }
                        convert_group<MODE>(v, ahi, alo, r, j);
                    } else {
                        // slab [KE][128 lines]: lanes cover consecutive lines
                        const int r = u & 127, j = u >> 7;
#pragma unroll
                        for (int q = 0; q < GS; ++q) v[q] = raw[(j * GS + q) * P_M + r];
                        convert_group<MODE>(v, ahi, alo, r, j);
                    }
                }
                fence_proxy_async();
                mbar_arrive(&conv[s]);
                if (tid == 0) consumed_s = gc + 1;
            }
        }
    } else if (warp == P_MMA_WARP) {
        // ---- MMA issuer
        if (lane == 0) {
            const uint32_t id = idesc<MODE>(g.NP);
            int gc = 0, ti = 0;
            bool go = true;
            for (long long t = blockIdx.x; t < ntiles && go; t += gridDim.x, ++ti) {
                const int b = ti & 1;
                // the epilogue of tile ti - 2 has read accumulator b
                if (ti >= 2 &&
                    !mwait(&acc_empty[b], (uint32_t)((ti / 2 - 1) & 1), g.err, abort, true, g.wait_ns))
                    break;
                tc_after();
                const uint32_t acc_t = tmem + (uint32_t)b * acols;
                for (int c = 0; c < nch; ++c, ++gc) {
                    const int s = gc % P_STAGES;
                    if (!mwait(&conv[s], (uint32_t)((gc / P_STAGES) & 1), g.err, abort, true, g.wait_ns)) {
                        go = false;
                        break;
                    }
                    tc_after();
                    const uint32_t st = su32(base + s * G::STAGE);
                    const uint32_t bhi = st + G::OFF_B, blo = bhi + (uint32_t)(g.NP * P_RB);
                    const uint32_t ahi = st + G::OFF_A, alo = ahi + G::ATILE;
#pragma unroll
                    for (int kk = 0; kk < 2; ++kk) {  // 32 bytes of K per MMA
                        const uint32_t ko = kk * 256;   // two core matrices along K
                        const uint32_t acc = (c > 0 || kk > 0) ? 1u : 0u;
                        mma<MODE>(acc_t, sdesc(ahi + ko), sdesc(bhi + ko), id, acc);
                        if constexpr (MODE == PM_BF16X3) {
                            mma<MODE>(acc_t, sdesc(ahi + ko), sdesc(blo + ko), id, 1u);
                            mma<MODE>(acc_t, sdesc(alo + ko), sdesc(bhi + ko), id, 1u);
                        }
                    }
                    mma_commit(&empty[s]);
                    mma_chunks_s = gc + 1;
                }
                if (go) mma_commit(&acc_full[b]);
            }
        }
    } else {
        // ---- epilogue (warps 10..: TMEM lane quarter q = warp % 4; each group of four
        // takes an equal share of the 8-column groups)
        const int q = warp & 3;
        constexpr int parts = P_EPI_WARPS / 4;
        const int ngroups = (g.NP + 7) / 8;
        const int part = (warp - 10) / 4;
        const int c_begin = 8 * (ngroups * part / parts);
        const int c_end = part + 1 == parts ? g.NP : 8 * (ngroups * (part + 1) / parts);
        int ti = 0;
        for (long long t = blockIdx.x; t < ntiles; t += gridDim.x, ++ti) {
            const int b = ti & 1;
            if (!mwait(&acc_full[b], (uint32_t)((ti / 2) & 1), g.err, abort, true, g.wait_ns)) break;
            tc_after();
            const long long line = (t % ntl) * P_M + q * 32 + lane;
            const int batch = (int)(t / ntl);
            float* out = g.out + (long long)batch * g.SB;
            // Poisson division: the line fixes kx (and ky on the z pass); the column k is
            // the remaining frequency.  Per line: the partial integer sum (reference
            // eigenvalues) or the partial float sum (accurate eigenvalues, same order).
            int kx = 0, ky = 0;
            long long pref = 0;
            float pacc = 0.f;
            const long long* tk = g.pz_layout == 1 ? g.fx1 : g.fx2;  // table of column k
            const float* ek = g.pz_layout == 1 ? g.eig1 : g.eig2;
            if constexpr (EPI == PE_POISSON_REF || EPI == PE_POISSON_ACC) {
                if (line < g.L) {
                    if (g.pz_layout == 1) kx = (int)line;
                    else { kx = (int)(line % g.W); ky = (int)(line / g.W); }
                    if (g.fx0) {
                        pref = (g.D > 1 ? 6ll : 4ll) * 4294967296ll - g.fx0[kx];
                        if (g.pz_layout == 2) pref -= g.fx1[ky];
                    }
                    pacc = g.pz_layout == 2 ? g.eig0[kx] + g.eig1[ky] : g.eig0[kx];
                }
            }
            for (int c0 = c_begin; c0 < c_end; c0 += 8) {
                float v[8];
                tmem_ld8(tmem + (uint32_t)b * acols + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
                if (line >= g.L) continue;
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int k = c0 + e;
                    float x = v[e];
                    if constexpr (EPI == PE_SCALE) {
                        x = x * g.scale;
                    } else if constexpr (EPI == PE_POISSON_REF || EPI == PE_POISSON_ACC) {
                        x = x * 8.f;
                        if (kx == 0 && ky == 0 && k == 0) {
                            x = 0.f;
                        } else if (k < g.NA) {
                            if constexpr (EPI == PE_POISSON_REF) {
                                if (g.fx0) {
                                    x = x / fixed32_to_float(pref - tk[k]);
                                } else {
                                    const int yy = g.pz_layout == 1 ? k : ky;
                                    x = x / poisson_den_ref(g.D > 1, nullptr, nullptr, nullptr,
                                                            g.cosk0, g.cosk1, g.cosk2, kx, yy, k);
                                }
                            } else {
                                x = x / (pacc + ek[k]);
                            }
                        }
                    }
                    v[e] = x;
                }
                if constexpr (AXIS == PA_X) {
                    // out[line][k]: 8 consecutive values of one line
                    float* dst = out + line * g.SL + c0;
                    if (c0 + 8 <= g.NA) {
                        *(float4*)dst = make_float4(v[0], v[1], v[2], v[3]);
                        *(float4*)(dst + 4) = make_float4(v[4], v[5], v[6], v[7]);
                    } else {
                        for (int e = 0; e < 8 && c0 + e < g.NA; ++e) dst[e] = v[e];
                    }
                } else {
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                        if (c0 + e < g.NA) out[line * g.SL + (long long)(c0 + e) * g.sn] = v[e];
                }
            }
            tc_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[b]);
        }
    }
    __syncthreads();
    // ---- error exit: let issued copies land and issued MMAs finish before TMEM and
    // shared memory go away (bounded waits; nothing is pending on the normal path)
    if (abort_s) {
        if (tid == 0 && mma_chunks_s > 0) {
            const int c = mma_chunks_s - 1;
            mwait(&empty[c % P_STAGES], (uint32_t)((c / P_STAGES) & 1), g.err, abort, false);
        }
        if (tid == 32) {
            for (int c = consumed_s; c < issued_s; ++c)
                mwait(&full[c % P_STAGES], (uint32_t)((c / P_STAGES) & 1), g.err, abort, false);
        }
    }
    tc_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(ncols)
                     : "memory");
}

// Both modes ask for the BF16x3 footprint (over half of an SM's shared memory), so
// that no SM holds two of these CTAs: each allocates all 512 TMEM columns.
template <int MODE>
constexpr size_t pipe_smem() {
    return (size_t)PGeo<PM_BF16X3>::NS * PGeo<PM_BF16X3>::STAGE + 1024;
}
// the TF32 ring must fit in the footprint both modes request
static_assert(PGeo<PM_TF32>::NS * PGeo<PM_TF32>::STAGE <=
                  PGeo<PM_BF16X3>::NS * PGeo<PM_BF16X3>::STAGE,
              "the TF32 stages overflow the shared memory both modes request");
static_assert(PGeo<PM_BF16X3>::NS <= P_STAGES_MAX && PGeo<PM_TF32>::NS <= P_STAGES_MAX,
              "more stages than mbarriers");

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        TGV_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000,
                                                  cudaEnableDefault, &q));
        TGV_REQUIRE(q == cudaDriverEntryPointSuccess && ptr, "cuTensorMapEncodeTiled unavailable");
        fn = (PFN_cuTensorMapEncodeTiled_v12000)ptr;
    }
    return fn;
}

void encode(CUtensorMap* m, const float* base, int rank, const cuuint64_t* dims,
            const cuuint64_t* strides, const cuuint32_t* box,
            CUtensorMapSwizzle swizzle = CU_TENSOR_MAP_SWIZZLE_NONE) {
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = encoder()(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, rank, const_cast<float*>(base),
                                 dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                 swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    TGV_REQUIRE(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled rejected a DCT operand");
}

template <int MODE, int AXIS>
void launch_axis(const PArgs& a, int batches, int epi, cudaStream_t st) {
    auto pick = [&]() {
        switch (epi) {
            case PE_SCALE: return dct_pipe_kernel<MODE, AXIS, PE_SCALE>;
            case PE_POISSON_REF: return dct_pipe_kernel<MODE, AXIS, PE_POISSON_REF>;
            case PE_POISSON_ACC: return dct_pipe_kernel<MODE, AXIS, PE_POISSON_ACC>;
            default: return dct_pipe_kernel<MODE, AXIS, PE_NONE>;
        }
    };
    auto k = pick();
    constexpr size_t smem = pipe_smem<MODE>();
    static std::atomic<uint64_t> configured[4] = {};
    smem_attr_once((const void*)k, smem, configured[epi & 3]);
    int dev = 0, sms = 0;
    TGV_CUDA(cudaGetDevice(&dev));
    TGV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PArgs b = a;
    b.batches = batches;
    const long long tiles = (long long)ceil_div((size_t)a.L, P_M) * batches;
    const unsigned grid = (unsigned)(tiles < sms ? tiles : sms);  // one persistent CTA per SM
    k<<<grid, P_THREADS, smem, st>>>(b);
    TGV_CHECK_LAUNCH();
}

template <int MODE>
void launch_mode(const PArgs& a, int axis, int batches, int epi, cudaStream_t st) {
    if (axis == 0) launch_axis<MODE, PA_X>(a, batches, epi, st);
    else if (axis == 1) launch_axis<MODE, PA_Y>(a, batches, epi, st);
    else launch_axis<MODE, PA_Z>(a, batches, epi, st);
}

uint16_t bf16_bits_h(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
float bf16_float_h(uint16_t h) { return __bfloat162float(__ushort_as_bfloat16(h)); }
float tf32_h(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;
    u += 0x1000u;
    u &= 0xffffe000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}
double cospi_hd(double a) {
    double r = std::fmod(std::fabs(a), 2.0);
    if (r > 1.0) r = 2.0 - r;
    const double pi = 3.14159265358979323846;
    if (r <= 0.25) return std::cos(pi * r);
    if (r <= 0.75) return std::sin(pi * (0.5 - r));
    return -std::cos(pi * (1.0 - r));
}

// The stage images of one matrix: chunk c holds, for every row k < NP, bytes
// [c*64, c*64+64) of the row's K-major values (BF16 hi then lo, or TF32) in the
// canonical layout, zero past N.
std::vector<uint8_t> stage_images(int n, bool inverse, int mode, int* nchunks_out) {
    const int NP = (n + 15) / 16 * 16;
    const int ke = mode == PM_BF16X3 ? 32 : 16;
    const int nch = (n + ke - 1) / ke;
    const int nb = mode == PM_BF16X3 ? 2 : 1;
    const size_t chunk = (size_t)nb * NP * P_RB;
    std::vector<uint8_t> img(chunk * nch, 0);
    for (int k = 0; k < NP; ++k)
        for (int m = 0; m < n && k < n; ++m) {
            const double cv = cospi_hd(((double)(inverse ? k : m) + 0.5) *
                                       (double)(inverse ? m : k) / (double)n);
            // forward: row = frequency k, column = sample m; inverse: row = sample k,
            // column = frequency m (weight 2 for m >= 1)
            const double val = inverse && m > 0 ? 2.0 * cv : cv;
            const int c = m / ke, e = m % ke;
            uint8_t* t = img.data() + (size_t)c * chunk;
            if (mode == PM_BF16X3) {
                const int cb = e * 2;
                const size_t off = (size_t)(k >> 3) * 512 + (cb >> 4) * 128 + (k & 7) * 16 + (cb & 15);
                const uint16_t h = bf16_bits_h((float)val);
                const uint16_t l = bf16_bits_h((float)(val - (double)bf16_float_h(h)));
                std::memcpy(t + off, &h, 2);
                std::memcpy(t + (size_t)NP * P_RB + off, &l, 2);
            } else {
                const int cb = e * 4;
                const size_t off = (size_t)(k >> 3) * 512 + (cb >> 4) * 128 + (k & 7) * 16 + (cb & 15);
                const float f = tf32_h((float)val);
                std::memcpy(t + off, &f, 4);
            }
        }
    *nchunks_out = nch;
    return img;
}

}  // namespace

bool dct_pipe_supported(const DctPlan* p) {
    return p->W % 4 == 0 && p->W <= 256 && p->H <= 256 && p->D <= 256;
}

void dct_plan_prepare_pipe(DctPlan* p) {
    if (p->pipe_block) return;
    TGV_REQUIRE(dct_pipe_supported(p), "pipelined tensor-core DCT needs sides <= 256, W % 4 == 0");
    const int N[3] = {p->W, p->H, p->D};
    std::vector<std::vector<uint8_t>> imgs;
    size_t bytes = 0;
    for (int mode = 0; mode < 2; ++mode)
        for (int dir = 0; dir < 2; ++dir)
            for (int a = 0; a < 3; ++a) {
                int nch = 0;
                imgs.push_back(stage_images(N[a], dir == 1, mode, &nch));
                p->pipe_chunks[mode][dir][a] = nch;
                bytes += (imgs.back().size() + 255) & ~size_t(255);
            }
    TGV_CUDA(cudaMalloc(&p->pipe_block, bytes));
    uint8_t* c = (uint8_t*)p->pipe_block;
    int i = 0;
    for (int mode = 0; mode < 2; ++mode)
        for (int dir = 0; dir < 2; ++dir)
            for (int a = 0; a < 3; ++a, ++i) {
                p->pipe_img[mode][dir][a] = c;
                TGV_CUDA(cudaMemcpy(c, imgs[i].data(), imgs[i].size(), cudaMemcpyHostToDevice));
                c += (imgs[i].size() + 255) & ~size_t(255);
            }
}

bool pass_pipe(DctPlan* p, int axis, bool inverse, const float* in, float* out, int epi,
               float scale, int dct_mode, cudaStream_t st) {
    if (!dct_pipe_supported(p) || ((uintptr_t)in & 15) != 0 || ((uintptr_t)out & 15) != 0)
        return false;
    dct_plan_prepare_pipe(p);
    if (!p->dev_err) dct_plan_prepare_tc(p);  // the device error flag lives there
    const int mode = dct_mode == TGVDCT_DCT_BF16X3 ? PM_BF16X3 : PM_TF32;
    const int ke = mode == PM_BF16X3 ? 32 : 16;
    const long long W = p->W, H = p->H, D = p->D, WH = W * H;
    PArgs a{};
    a.out = out;
    a.W = p->W;
    a.H = p->H;
    a.D = p->D;
    a.scale = scale;
    a.cosk0 = p->cosk[0];
    a.cosk1 = p->cosk[1];
    a.cosk2 = p->cosk[2];
    a.eig0 = p->eig[0];
    a.eig1 = p->eig[1];
    a.eig2 = p->eig[2];
    a.err = p->dev_err;
    a.wait_ns = p->wait_ns;
    a.fx0 = p->cosk_fx[0];
    a.fx1 = p->cosk_fx[1];
    a.fx2 = p->cosk_fx[2];
    const int dir = inverse ? 1 : 0;
    a.bimg = (const uint8_t*)p->pipe_img[mode][dir][axis];
    a.nchunks = p->pipe_chunks[mode][dir][axis];
    int batches = 1;
    if (axis == 0) {
        a.NA = (int)W;
        a.L = H * D;
        a.SL = W;
        a.SB = 0;
        a.sn = 1;
        const cuuint64_t dims[2] = {(cuuint64_t)W, (cuuint64_t)(H * D)};
        const cuuint64_t strides[1] = {(cuuint64_t)W * 4};
        const cuuint32_t box[2] = {(cuuint32_t)ke, (cuuint32_t)P_M};
        // rows of ke floats (128 or 64 bytes) land swizzled, so that the converters can
        // read eight consecutive lines at once without bank conflicts (xslab_off)
        encode(&a.in_map, in, 2, dims, strides, box,
               mode == PM_BF16X3 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B);
    } else if (axis == 1) {
        a.NA = (int)H;
        a.L = W;
        a.SL = 1;
        a.SB = WH;
        a.sn = W;
        a.pz_layout = 1;
        batches = (int)D;
        const cuuint64_t dims[3] = {(cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)D};
        const cuuint64_t strides[2] = {(cuuint64_t)W * 4, (cuuint64_t)WH * 4};
        const cuuint32_t box[3] = {(cuuint32_t)P_M, (cuuint32_t)ke, 1};
        encode(&a.in_map, in, 3, dims, strides, box);
    } else {
        a.NA = (int)D;
        a.L = WH;
        a.SL = 1;
        a.SB = 0;
        a.sn = WH;
        a.pz_layout = 2;
        const cuuint64_t dims[2] = {(cuuint64_t)WH, (cuuint64_t)D};
        const cuuint64_t strides[1] = {(cuuint64_t)WH * 4};
        const cuuint32_t box[2] = {(cuuint32_t)P_M, (cuuint32_t)ke};
        encode(&a.in_map, in, 2, dims, strides, box);
    }
    a.NP = (a.NA + 15) / 16 * 16;
    if (mode == PM_BF16X3) launch_mode<PM_BF16X3>(a, axis, batches, epi, st);
    else launch_mode<PM_TF32>(a, axis, batches, epi, st);
    return true;
}

}  // namespace tgvdct
