// Tensor-core (tcgen05) DCT passes for sides <= 256.
//
// A separable pass along one axis is D[m][k] = sum_n A[m][n] * M[k][n], where m
// runs over the 128 lines of a block (voxels of one axis position set: rows for
// the x pass, x positions for the y pass, (x, y) columns for the z pass), n over
// the axis, and M is the N x N cosine matrix (DCT-II forward, DCT-III inverse).
// One CTA computes a 128 x N tile of D with N <= 256 in one TMEM accumulator
// (128 lanes x N columns of FP32), so every input voxel is read from HBM once.
//
// Operands are staged by the CTA's 256 threads: FP32 voxels are read from global
// memory (coalesced along whichever index is contiguous), converted, and written
// to shared memory in the canonical K-major layout without swizzle: 8-row x 16-byte
// core matrices, K-adjacent core matrices 128 bytes apart (LBO) and 8-row groups
// 1024 bytes apart (SBO).  A K chunk is 128 bytes of every row (64 BF16 or 32
// TF32 values), i.e. four MMAs of K = 16 (BF16) or K = 8 (TF32).  Two stages
// alternate: while the tensor core consumes one, the threads fill the other; a
// tcgen05.commit on the stage's mbarrier tells the threads when it is free.
//
// Precision modes:
//   TF32    one kind::tf32 product of TF32-rounded operands;
//   BF16X3  x = hi + lo with hi = bf16(x), lo = bf16(x - hi) for data and matrix,
//           D += A_hi M_hi + A_hi M_lo + A_lo M_hi with FP32 accumulation
//           (kind::f16), which keeps about 16 significant bits of every product.
//
// Every wait on an mbarrier is bounded by a wall-clock limit; on timeout the
// kernel raises a device error flag, skips the rest of its work, frees its TMEM
// and returns, and the host reports the flag.
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "common.cuh"

namespace tgvdct {

enum TcMode { TC_BF16X3 = 0, TC_TF32 = 1 };
enum TcEpi { TCE_NONE = 0, TCE_SCALE = 1, TCE_POISSON_REF = 2, TCE_POISSON_ACC = 3 };

namespace {

constexpr int TC_M = 128;        // lines per CTA (MMA M)
constexpr int TC_THREADS = 256;  // 8 warps
constexpr int ROW_BYTES = 128;   // K chunk per stage and row
constexpr uint64_t WAIT_LIMIT_NS = 200000000ull;  // 200 ms

struct TcArgs {
    const float* in;
    float* out;
    int L;          // lines per batch
    long long SL;   // line stride (elements)
    long long SB;   // batch stride (elements)
    int NA;         // axis length: contraction length and number of output frequencies
    int NP;         // NA rounded up to a multiple of 16 (MMA N)
    long long sn;   // element stride along the axis
    const uint16_t* m_hi;  // BF16 matrix (NA x NA, row k, column n)
    const uint16_t* m_lo;
    const float* m_tf;     // TF32-rounded matrix
    // divergence operand (x pass of the integration): A[m][n] = B.v at (x = n, row m)
    const float* vx;
    const float* vy;
    const float* vz;
    int W, H, D;
    // epilogue
    float scale;
    int pz_layout;  // 1: (kx = line, ky = k); 2: (kx = line % W, ky = line / W, kz = k)
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
};

// ---- PTX wrappers -------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t globaltimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the completion of the phase with the given parity.
__device__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err) {
    if (mbar_test(bar, parity)) return true;
    const uint64_t t0 = globaltimer();
    while (true) {
        if (mbar_test(bar, parity)) return true;
        if (globaltimer() - t0 > WAIT_LIMIT_NS) {
            atomicExch(err, 1);
            return false;
        }
        __nanosleep(64);
    }
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

template <int MODE>
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                    uint32_t idesc, uint32_t accumulate) {
    if constexpr (MODE == TC_BF16X3) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
            : "memory");
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
            : "memory");
    }
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
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

// Shared-memory matrix descriptor, K-major, no swizzle: start address, LBO (bytes
// between K-adjacent core matrices), SBO (bytes between 8-row groups), version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;  // layout type (bits 61-63) 0: no swizzle
}

// Instruction descriptor: D FP32, A/B BF16 (kind::f16) or TF32 (kind::tf32),
// both K-major, M = 128, N = n.
template <int MODE>
__host__ __device__ constexpr uint32_t instr_desc(int n) {
    const uint32_t ab = MODE == TC_BF16X3 ? 1u : 2u;
    return (1u << 4) | (ab << 7) | (ab << 10) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(TC_M >> 4) << 24);
}

// byte offset of (row r, byte cb of the 128-byte K chunk) in a staged tile
__device__ __forceinline__ uint32_t tile_off(int r, int cb) {
    return (uint32_t)((r >> 3) * 1024 + (cb >> 4) * 128 + (r & 7) * 16 + (cb & 15));
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const uint32_t lo = __bfloat16_as_ushort(__float2bfloat16_rn(a));
    const uint32_t hi = __bfloat16_as_ushort(__float2bfloat16_rn(b));
    return lo | (hi << 16);
}

__device__ __forceinline__ float tf32_round(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ float divergence_at(const TcArgs& g, long long line, int n) {
    const int y = (int)(line % g.H), z = (int)(line / g.H);
    const size_t W = (size_t)g.W, WH = (size_t)g.W * g.H;
    const size_t idx = (size_t)line * W + n;
    const float bx = (n > 0 ? g.vx[idx - 1] : 0.f) - g.vx[idx];  // divergence.cu:38-55
    const float by = (y > 0 ? g.vy[idx - W] : 0.f) - g.vy[idx];
    float s = bx + by;
    if (g.D > 1) s = s + ((z > 0 ? g.vz[idx - WH] : 0.f) - g.vz[idx]);
    return s;
}

// Stage sizes: A tile 128 rows, B tile NP (<= 256) rows, 128 bytes each row.
constexpr uint32_t A_BYTES = TC_M * ROW_BYTES;   // 16 KB
constexpr uint32_t B_BYTES = 256 * ROW_BYTES;    // 32 KB (max)

template <int MODE>
constexpr uint32_t stage_bytes() {
    return MODE == TC_BF16X3 ? 2 * A_BYTES + 2 * B_BYTES : A_BYTES + B_BYTES;
}

template <int MODE, bool DIV, int EPI>
__global__ void __launch_bounds__(TC_THREADS, 1) dct_tc_kernel(TcArgs g) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // 1024-byte aligned staging area
    uint8_t* base = align_shared<1024>(smem_raw);
    constexpr uint32_t SB = stage_bytes<MODE>();
    __shared__ uint64_t bar_free[2];
    __shared__ uint32_t tmem_base_s;

    // an earlier pass timed out: do nothing more (one read shared by the block)
    if (__syncthreads_or(threadIdx.x == 0 ? *(volatile int*)g.err : 0)) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int batch = blockIdx.y;
    const long long line0 = (long long)blockIdx.x * TC_M;
    const float* in = g.in + (long long)batch * g.SB;
    const int NP = g.NP;
    constexpr int KC = MODE == TC_BF16X3 ? 64 : 32;  // elements per K chunk
    const int nchunks = (g.NA + KC - 1) / KC;
    // TMEM columns: power of two >= 32 covering NP
    uint32_t ncols = 32;
    while (ncols < (uint32_t)NP) ncols <<= 1;

    if (tid == 0) {
        mbar_init(&bar_free[0], 1);
        mbar_init(&bar_free[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(&tmem_base_s, ncols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_s;
    const uint32_t idesc = instr_desc<MODE>(NP);
    bool ok = true;

    for (int c = 0; c < nchunks && ok; ++c) {
        const int st = c & 1;
        uint8_t* sA = base + st * SB;
        uint8_t* sAlo = sA + A_BYTES;                                      // BF16X3 only
        uint8_t* sB = sA + (MODE == TC_BF16X3 ? 2 * A_BYTES : A_BYTES);
        uint8_t* sBlo = sB + B_BYTES;                                      // BF16X3 only
        if (c >= 2) ok = mbar_wait(&bar_free[st], ((c - 2) >> 1) & 1, g.err);
        ok = __syncthreads_and(ok);
        if (!ok) break;
        const int k0 = c * KC;
        // ---- A: 128 lines x KC values, 8 values (BF16) / 4 values (TF32) per 16 bytes
        constexpr int VPC = MODE == TC_BF16X3 ? 8 : 4;   // values per 16-byte chunk
        constexpr int CPR = ROW_BYTES / 16;              // chunks per row: 8
        for (int e = tid; e < TC_M * CPR; e += TC_THREADS) {
            int m, j;
            if (g.SL == 1 && !DIV) { m = e % TC_M; j = e / TC_M; }   // lines contiguous
            else { j = e % CPR; m = e / CPR; }                       // axis contiguous
            const long long line = line0 + m;
            float v[VPC];
#pragma unroll
            for (int t = 0; t < VPC; ++t) {
                const int n = k0 + j * VPC + t;
                float x = 0.f;
                if (line < g.L && n < g.NA) {
                    if constexpr (DIV) x = divergence_at(g, line, n);
                    else x = in[line * g.SL + (long long)n * g.sn];
                }
                v[t] = x;
            }
            const uint32_t off = tile_off(m, j * 16);
            if constexpr (MODE == TC_BF16X3) {
                uint32_t hi[4], lo[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const float a = v[2 * t], b = v[2 * t + 1];
                    const float ah = __bfloat162float(__float2bfloat16_rn(a));
                    const float bh = __bfloat162float(__float2bfloat16_rn(b));
                    hi[t] = pack_bf16(ah, bh);
                    lo[t] = pack_bf16(a - ah, b - bh);
                }
                *(uint4*)(sA + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
                *(uint4*)(sAlo + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
            } else {
                *(float4*)(sA + off) = make_float4(tf32_round(v[0]), tf32_round(v[1]),
                                                   tf32_round(v[2]), tf32_round(v[3]));
            }
        }
        // ---- B: NP matrix rows (frequencies) x KC values, from the row-major matrix
        for (int e = tid; e < NP * CPR; e += TC_THREADS) {
            const int j = e % CPR, k = e / CPR;
            const uint32_t off = tile_off(k, j * 16);
            const int n0 = k0 + j * VPC;
            if constexpr (MODE == TC_BF16X3) {
                uint4 h = make_uint4(0, 0, 0, 0), l = make_uint4(0, 0, 0, 0);
                if (k < g.NA) {
                    uint16_t hv[8], lv[8];
#pragma unroll
                    for (int t = 0; t < 8; ++t) {
                        const int n = n0 + t;
                        hv[t] = n < g.NA ? g.m_hi[(size_t)k * g.NA + n] : 0;
                        lv[t] = n < g.NA ? g.m_lo[(size_t)k * g.NA + n] : 0;
                    }
                    h = make_uint4(hv[0] | (hv[1] << 16), hv[2] | (hv[3] << 16),
                                   hv[4] | (hv[5] << 16), hv[6] | (hv[7] << 16));
                    l = make_uint4(lv[0] | (lv[1] << 16), lv[2] | (lv[3] << 16),
                                   lv[4] | (lv[5] << 16), lv[6] | (lv[7] << 16));
                }
                *(uint4*)(sB + off) = h;
                *(uint4*)(sBlo + off) = l;
            } else {
                float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
                if (k < g.NA) {
                    float t4[4];
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        const int n = n0 + t;
                        t4[t] = n < g.NA ? g.m_tf[(size_t)k * g.NA + n] : 0.f;
                    }
                    f = make_float4(t4[0], t4[1], t4[2], t4[3]);
                }
                *(float4*)(sB + off) = f;
            }
        }
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {  // 32 bytes of K per MMA
                const uint32_t ko = kk * 256;   // two core matrices along K
                const uint64_t ad = smem_desc(smem_u32(sA) + ko, 128, 1024);
                const uint64_t bd = smem_desc(smem_u32(sB) + ko, 128, 1024);
                const uint32_t acc0 = (c > 0 || kk > 0) ? 1u : 0u;
                mma<MODE>(tmem, ad, bd, idesc, acc0);
                if constexpr (MODE == TC_BF16X3) {
                    const uint64_t bdl = smem_desc(smem_u32(sBlo) + ko, 128, 1024);
                    const uint64_t adl = smem_desc(smem_u32(sAlo) + ko, 128, 1024);
                    mma<MODE>(tmem, ad, bdl, idesc, 1u);
                    mma<MODE>(tmem, adl, bd, idesc, 1u);
                }
            }
            mma_commit(&bar_free[st]);
        }
    }
    // all MMAs done: the last commit covers every earlier MMA of the issuing thread
    if (ok && nchunks > 0) ok = mbar_wait(&bar_free[(nchunks - 1) & 1], ((nchunks - 1) >> 1) & 1,
                                         g.err);
    ok = __syncthreads_and(ok);
    tc_fence_after();

    if (ok) {
        // ---- epilogue: warp w reads TMEM lanes 32*(w%4).., columns of half w/4
        const int q = warp & 3, half = warp >> 2;
        const int m = q * 32 + lane;
        const long long line = line0 + m;
        const int cols_half = NP / 2;  // multiple of 8
        float* out = g.out + (long long)batch * g.SB;
        for (int c0 = half * cols_half; c0 < (half + 1) * cols_half; c0 += 8) {
            float v[8];
            tmem_ld8(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
            if (line >= g.L) continue;
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int k = c0 + t;
                if (k >= g.NA) continue;
                float x = v[t];
                if constexpr (EPI == TCE_SCALE) {
                    x = x * g.scale;
                } else if constexpr (EPI == TCE_POISSON_REF || EPI == TCE_POISSON_ACC) {
                    int kx, ky, kz;
                    if (g.pz_layout == 1) { kx = (int)line; ky = k; kz = 0; }
                    else { kx = (int)(line % g.W); ky = (int)(line / g.W); kz = k; }
                    x = x * 8.f;
                    if (kx == 0 && ky == 0 && kz == 0) {
                        x = 0.f;
                    } else if constexpr (EPI == TCE_POISSON_REF) {
                        x = x / poisson_den_ref(g.D > 1, g.fx0, g.fx1, g.fx2, g.cosk0, g.cosk1,
                                                g.cosk2, kx, ky, kz);
                    } else {
                        float den = g.eig0[kx] + g.eig1[ky];
                        if (g.D > 1) den = den + g.eig2[kz];
                        x = x / den;
                    }
                }
                out[line * g.SL + (long long)k * g.sn] = x;
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, ncols);
}

template <int MODE, bool DIV, int EPI>
void launch(const TcArgs& g, int batches, cudaStream_t st) {
    constexpr size_t smem = 2 * (size_t)stage_bytes<MODE>() + 1024;
    auto k = dct_tc_kernel<MODE, DIV, EPI>;
    static std::atomic<uint64_t> configured{0};
    smem_attr_once((const void*)k, smem, configured);
    const dim3 grid(ceil_div((size_t)g.L, TC_M), batches);
    k<<<grid, TC_THREADS, smem, st>>>(g);
    TGV_CHECK_LAUNCH();
}

template <int MODE>
void launch_mode(const TcArgs& g, int batches, bool div, int epi, cudaStream_t st) {
    if (div) {
        launch<MODE, true, TCE_NONE>(g, batches, st);
        return;
    }
    switch (epi) {
        case TCE_NONE: launch<MODE, false, TCE_NONE>(g, batches, st); break;
        case TCE_SCALE: launch<MODE, false, TCE_SCALE>(g, batches, st); break;
        case TCE_POISSON_REF: launch<MODE, false, TCE_POISSON_REF>(g, batches, st); break;
        case TCE_POISSON_ACC: launch<MODE, false, TCE_POISSON_ACC>(g, batches, st); break;
    }
}

uint16_t bf16_bits(float x) {
    __nv_bfloat16 b = __float2bfloat16_rn(x);
    return __bfloat16_as_ushort(b);
}
float bf16_float(uint16_t h) { return __bfloat162float(__ushort_as_bfloat16(h)); }

// round to TF32 (10 explicit mantissa bits), nearest, ties away from zero
float tf32_host(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;
    u += 0x1000u;
    u &= 0xffffe000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

double cospi_h(double a) {
    double r = std::fmod(std::fabs(a), 2.0);
    if (r > 1.0) r = 2.0 - r;
    const double pi = 3.14159265358979323846;
    if (r <= 0.25) return std::cos(pi * r);
    if (r <= 0.75) return std::sin(pi * (0.5 - r));
    return -std::cos(pi * (1.0 - r));
}

}  // namespace

bool dct_tc_supported(const DctPlan* p) { return p->W <= 256 && p->H <= 256 && p->D <= 256; }

void dct_plan_prepare_tc(DctPlan* p) {
    if (p->tc_block) return;
    TGV_REQUIRE(dct_tc_supported(p), "tensor-core DCT modes need every side <= 256");
    const int N[3] = {p->W, p->H, p->D};
    size_t bytes = 256;  // error flag
    for (int a = 0; a < 3; ++a) bytes += 2 * ((size_t)N[a] * N[a] * (2 + 2 + 4) + 256 * 3);
    TGV_CUDA(cudaMalloc(&p->tc_block, bytes));
    char* c = (char*)p->tc_block;
    p->dev_err = (int*)c;
    c += 256;
    TGV_CUDA(cudaMemset(p->dev_err, 0, sizeof(int)));
    for (int a = 0; a < 3; ++a) {
        const size_t n = (size_t)N[a];
        for (int dir = 0; dir < 2; ++dir) {
            std::vector<uint16_t> hi(n * n), lo(n * n);
            std::vector<float> tf(n * n);
            for (size_t k = 0; k < n; ++k)
                for (size_t m = 0; m < n; ++m) {
                    // forward: row = frequency k, column = sample m;
                    // inverse: row = sample m, column = frequency k (weight 2 for k >= 1)
                    const double cv = cospi_h(((double)m + 0.5) * (double)k / (double)n);
                    size_t row, col;
                    double val;
                    if (dir == 0) { row = k; col = m; val = cv; }
                    else { row = m; col = k; val = k == 0 ? cv : 2.0 * cv; }
                    const float fv = (float)val;
                    const uint16_t h = bf16_bits(fv);
                    hi[row * n + col] = h;
                    lo[row * n + col] = bf16_bits((float)(val - (double)bf16_float(h)));
                    tf[row * n + col] = tf32_host(fv);
                }
            auto take = [&](size_t b) {
                char* r = c;
                c += (b + 255) & ~size_t(255);
                return r;
            };
            p->bf_hi[dir][a] = (uint16_t*)take(n * n * 2);
            p->bf_lo[dir][a] = (uint16_t*)take(n * n * 2);
            p->tf[dir][a] = (float*)take(n * n * 4);
            TGV_CUDA(cudaMemcpy(p->bf_hi[dir][a], hi.data(), n * n * 2, cudaMemcpyHostToDevice));
            TGV_CUDA(cudaMemcpy(p->bf_lo[dir][a], lo.data(), n * n * 2, cudaMemcpyHostToDevice));
            TGV_CUDA(cudaMemcpy(p->tf[dir][a], tf.data(), n * n * 4, cudaMemcpyHostToDevice));
        }
    }
}

bool dct_tc_check(DctPlan* p, cudaStream_t st) {
    if (!p->dev_err) return true;
    int h = 0;
    TGV_CUDA(cudaMemcpyAsync(&h, p->dev_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    TGV_CUDA(cudaStreamSynchronize(st));
    if (h) TGV_CUDA(cudaMemsetAsync(p->dev_err, 0, sizeof(int), st));
    return h == 0;
}

// One separable pass on the tensor cores (see dct_kernels.cu for the axis layouts).
void pass_tc(DctPlan* p, int axis, bool inverse, const float* in, float* out, int epi,
             float scale, bool div, const float* vx, const float* vy, const float* vz,
             int dct_mode, cudaStream_t st) {
    dct_plan_prepare_tc(p);
    const long long W = p->W, H = p->H, D = p->D, WH = W * H;
    TcArgs g{};
    g.in = in;
    g.out = out;
    g.W = p->W;
    g.H = p->H;
    g.D = p->D;
    g.vx = vx;
    g.vy = vy;
    g.vz = vz;
    g.scale = scale;
    g.cosk0 = p->cosk[0];
    g.cosk1 = p->cosk[1];
    g.cosk2 = p->cosk[2];
    g.eig0 = p->eig[0];
    g.eig1 = p->eig[1];
    g.eig2 = p->eig[2];
    g.err = p->dev_err;
    g.fx0 = p->cosk_fx[0];
    g.fx1 = p->cosk_fx[1];
    g.fx2 = p->cosk_fx[2];
    const int dir = inverse ? 1 : 0;
    g.m_hi = p->bf_hi[dir][axis];
    g.m_lo = p->bf_lo[dir][axis];
    g.m_tf = p->tf[dir][axis];
    int batches = 1;
    if (axis == 0) {
        g.L = (int)(H * D);
        g.SL = W;
        g.SB = 0;
        g.NA = (int)W;
        g.sn = 1;
    } else if (axis == 1) {
        g.L = (int)W;
        g.SL = 1;
        g.SB = WH;
        g.NA = (int)H;
        g.sn = W;
        batches = (int)D;
        g.pz_layout = 1;
    } else {
        g.L = (int)WH;
        g.SL = 1;
        g.SB = 0;
        g.NA = (int)D;
        g.sn = WH;
        g.pz_layout = 2;
    }
    g.NP = (g.NA + 15) / 16 * 16;
    if (dct_mode == TGVDCT_DCT_BF16X3) launch_mode<TC_BF16X3>(g, batches, div, epi, st);
    else launch_mode<TC_TF32>(g, batches, div, epi, st);
}

}  // namespace tgvdct
