// TGV2 primal-dual iteration on sm_103a: two fused stencil passes per iteration.
//
// The reference runs one iteration as 36 kernel launches with 7 device-wide
// synchronisations, most of them thread-per-line directional differences with
// uncoalesced x/y access (tgv_deshade/tgv2_l1_deshade.cu:169-272).  Here one
// iteration is two coalesced passes over the volume:
//
//   dual pass   (tgv_cuda/tgv2_common.cu:96-131 and :174-276)
//       p <- proj_{alpha1}( p + sigma (F ubar - vbar) )
//       q <- proj_{alpha0}( q + sigma E(vbar) ),  E from negated backward differences
//   primal pass (tgv_cuda/tgv2_l1.cu:27-60 / tgv2_l2.cu:27-56 and tgv2_common.cu:279-354)
//       u <- prox( u - tau B.p ),  ubar = u + theta (u - u_old)
//       v <- v - tau (div_F q - p), vbar = v + theta (v - v_old)
//
// The dual pass reads ubar and vbar with a one-voxel stencil and p, q only at the
// voxel it writes; the primal pass reads p and q with a stencil and u, v only at
// the voxel it writes.  So every field is updated in place without a race, and
// u_prev / v_prev (separate arrays in the reference) live in registers.
//
// Per voxel and iteration the two passes move 27 loads + 17 stores of the state
// (176 bytes in FP32); stencil neighbours are served from L1/L2.  Arithmetic
// follows the reference's operation order (explicit fmaf where it calls fmaf, no
// other contraction: this file is compiled with -fmad=false), so in FP32 the
// result differs from the reference's float code only by the rounding of norm3df.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"

// first bad index of a bounds-checking build (see TGV_IN_BOUNDS)
static __device__ unsigned long long g_bounds_tgv;
#define TGV_BOUNDS_WORD g_bounds_tgv

namespace tgvdct {
namespace {

// ---- storage of the dual fields p and q ------------------------------------------
template <int PREC>
struct Dual;

template <>
struct Dual<TGVDCT_STATE_FP32> {
    using T = float;
    static __device__ __forceinline__ float ld(const T* p, size_t i, float) { return p[i]; }
    static __device__ __forceinline__ void st(T* p, size_t i, float v, float) { p[i] = v; }
    // streaming store (evict-first): the next read of the field is an iteration away
    static __device__ __forceinline__ void st_cs(T* p, size_t i, float v, float) {
        __stcs(p + i, v);
    }
};

template <>
struct Dual<TGVDCT_STATE_BF16_DUAL> {
    using T = __nv_bfloat16;
    static __device__ __forceinline__ float ld(const T* p, size_t i, float) {
        return __bfloat162float(p[i]);
    }
    static __device__ __forceinline__ void st(T* p, size_t i, float v, float) {
        p[i] = __float2bfloat16_rn(v);
    }
    static __device__ __forceinline__ void st_cs(T* p, size_t i, float v, float) {
        __stcs((unsigned short*)p + i, __bfloat16_as_ushort(__float2bfloat16_rn(v)));
    }
};

// 16-bit fixed point: value = code * (alpha / 32767).  After the projections every
// component of p satisfies |p_c| <= |p| <= alpha1 and every component of q
// satisfies |q_c| <= alpha0, so the code range covers the field exactly.
// Conversions use the 1.5 * 2^23 bias: for |c| < 2^22 the float 12582912 + c holds
// c in its low mantissa bits, so an integer add and a float add (full-rate
// instructions) replace the slower int<->float conversion instructions, with the
// same round-to-nearest-even result.
template <>
struct Dual<TGVDCT_STATE_FX16_DUAL> {
    using T = int16_t;
    static __device__ __forceinline__ float ld(const T* p, size_t i, float dec) {
        const float c = __int_as_float(0x4B400000 + (int)p[i]) - 12582912.f;  // exact
        return c * dec;
    }
    static __device__ __forceinline__ void st(T* p, size_t i, float v, float enc) {
        const float c = fminf(fmaxf(v * enc, -32767.f), 32767.f);
        p[i] = (T)__float_as_int(c + 12582912.f);  // low 16 bits: the rounded code
    }
    static __device__ __forceinline__ void st_cs(T* p, size_t i, float v, float enc) {
        const float c = fminf(fmaxf(v * enc, -32767.f), 32767.f);
        __stcs((short*)p + i, (short)__float_as_int(c + 12582912.f));
    }
};

// Fields of the two-pass kernels.  The dual pass reads ubar, vbar, p_in, q_in and
// writes p, q; the primal pass reads p, q (the new duals), u_in, f, v_in and writes
// u, ubar_out, v, vbar_out.  The forward loop passes the same buffers for in and out
// (every field read at the voxel that writes it); the adjoint's segment recompute
// passes one stored state as input and the next as output.
template <class T>
struct TgvArgs {
    int W, H, D;
    size_t WH;
    const float* f;
    const float* u_in;
    float* u;
    const float* ubar;     // input ubar
    float* ubar_out;
    const float* v_in[3];
    float* v0;
    float* v1;
    float* v2;
    const float* vb0;      // input vbar
    const float* vb1;
    const float* vb2;
    float* vbo[3];         // output vbar
    const T* pin[3];
    const T* qin[6];       // xx yy zz xy xz yz
    T* p0;
    T* p1;
    T* p2;
    T* qxx;
    T* qyy;
    T* qzz;
    T* qxy;
    T* qxz;
    T* qyz;
    float tau, sigma, theta, tau_lambda, alpha0, alpha1;
    float penc, pdec, qenc, qdec;
    int skip_bz;  // L2 data term with depth == 1 drops B_z p (tgv_cuda/tgv2_l2.cu:39-42)
    const uint8_t* dom;  // masked deshade: update only voxels with dom[i] != 0 (null: all)
};

constexpr int BX = 32, BY = 8;

// Dual pass.  THREE: 3-D operators (also for D == 1); otherwise the 2-D launcher.
template <int PREC, bool THREE>
__global__ void __launch_bounds__(BX* BY) tgv_dual_kernel(TgvArgs<typename Dual<PREC>::T> a) {
    using S = Dual<PREC>;
    const int x = blockIdx.x * BX + threadIdx.x;
    const int y = blockIdx.y * BY + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= a.W || y >= a.H) return;
    const size_t W = (size_t)a.W, WH = a.WH;
    const size_t i = ((size_t)z * a.H + y) * W + x;
    if (!TGV_IN_BOUNDS(i, WH * a.D, 1)) return;
    // outside the masked deshade's domain nothing is updated (tgv2_masked_common.cu)
    if (a.dom && !a.dom[i]) return;

    // p <- proj(p + sigma (F ubar - vbar))          (tgv2_common.cu:118-130)
    const float ub = a.ubar[i];
    const float gx = (x + 1 < a.W) ? a.ubar[i + 1] - ub : 0.f;
    const float gy = (y + 1 < a.H) ? a.ubar[i + W] - ub : 0.f;
    const float vbx = a.vb0[i], vby = a.vb1[i];
    float px = __fmaf_rn(a.sigma, gx - vbx, S::ld(a.pin[0], i, a.pdec));
    float py = __fmaf_rn(a.sigma, gy - vby, S::ld(a.pin[1], i, a.pdec));
    float pz = 0.f, vbz = 0.f, nrm;
    if constexpr (THREE) {
        const float gz = (z + 1 < a.D) ? a.ubar[i + WH] - ub : 0.f;
        vbz = a.vb2[i];
        pz = __fmaf_rn(a.sigma, gz - vbz, S::ld(a.pin[2], i, a.pdec));
        nrm = norm3df(px, py, pz);
    } else {
        nrm = sqrtf(px * px + py * py);  // tgv2_common_2d.cu:113
    }
    nrm = fmaxf(1.f, nrm / a.alpha1);
    S::st(a.p0, i, px / nrm, a.penc);
    S::st(a.p1, i, py / nrm, a.penc);
    if constexpr (THREE) S::st(a.p2, i, pz / nrm, a.penc);

    // q <- proj(q + sigma E vbar), E from negated backward differences
    // B w = w[i-e] - w[i], and -w[i] on the first slice   (tgv_common.cu:133-197)
    const float vbx_x = x > 0 ? a.vb0[i - 1] : 0.f;
    const float vby_x = x > 0 ? a.vb1[i - 1] : 0.f;
    const float vbx_y = y > 0 ? a.vb0[i - W] : 0.f;
    const float vby_y = y > 0 ? a.vb1[i - W] : 0.f;
    const float exx = vbx_x - vbx;
    const float eyy = vby_y - vby;
    const float exy = ((vby_x - vby) + (vbx_y - vbx)) * 0.5f;  // tgv2_common.cu:191-199
    float qxx = __fmaf_rn(a.sigma, exx, S::ld(a.qin[0], i, a.qdec));
    float qyy = __fmaf_rn(a.sigma, eyy, S::ld(a.qin[1], i, a.qdec));
    float qxy = __fmaf_rn(a.sigma, exy, S::ld(a.qin[3], i, a.qdec));
    float s = qxx * qxx + qyy * qyy + 2.f * qxy * qxy;
    float qzz = 0.f, qxz = 0.f, qyz = 0.f;
    if constexpr (THREE) {
        const float vbz_x = x > 0 ? a.vb2[i - 1] : 0.f;
        const float vbz_y = y > 0 ? a.vb2[i - W] : 0.f;
        const float vbx_z = z > 0 ? a.vb0[i - WH] : 0.f;
        const float vby_z = z > 0 ? a.vb1[i - WH] : 0.f;
        const float vbz_z = z > 0 ? a.vb2[i - WH] : 0.f;
        const float ezz = vbz_z - vbz;
        const float exz = ((vbz_x - vbz) + (vbx_z - vbx)) * 0.5f;
        const float eyz = ((vbz_y - vbz) + (vby_z - vby)) * 0.5f;
        qzz = __fmaf_rn(a.sigma, ezz, S::ld(a.qin[2], i, a.qdec));
        qxz = __fmaf_rn(a.sigma, exz, S::ld(a.qin[4], i, a.qdec));
        qyz = __fmaf_rn(a.sigma, eyz, S::ld(a.qin[5], i, a.qdec));
        s = s + qzz * qzz + 2.f * qxz * qxz + 2.f * qyz * qyz;  // tgv2_common.cu:255-261
    }
    const float qn = fmaxf(1.f, sqrtf(s) / a.alpha0);
    S::st(a.qxx, i, qxx / qn, a.qenc);
    S::st(a.qyy, i, qyy / qn, a.qenc);
    S::st(a.qxy, i, qxy / qn, a.qenc);
    if constexpr (THREE) {
        S::st(a.qzz, i, qzz / qn, a.qenc);
        S::st(a.qxz, i, qxz / qn, a.qenc);
        S::st(a.qyz, i, qyz / qn, a.qenc);
    }
}

// Primal pass.
template <int PREC, bool THREE, int DATA>
__global__ void __launch_bounds__(BX* BY) tgv_primal_kernel(TgvArgs<typename Dual<PREC>::T> a) {
    using S = Dual<PREC>;
    const int x = blockIdx.x * BX + threadIdx.x;
    const int y = blockIdx.y * BY + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= a.W || y >= a.H) return;
    const size_t W = (size_t)a.W, WH = a.WH;
    const size_t i = ((size_t)z * a.H + y) * W + x;
    if (!TGV_IN_BOUNDS(i, WH * a.D, 2)) return;
    const bool xl = x + 1 < a.W, yl = y + 1 < a.H;
    if (a.dom && !a.dom[i]) return;

    // u <- prox(u - tau B.p), ubar                       (tgv2_l1.cu:39-52)
    const float pxi = S::ld(a.p0, i, a.pdec);
    const float pyi = S::ld(a.p1, i, a.pdec);
    const float bx = (x > 0 ? S::ld(a.p0, i - 1, a.pdec) : 0.f) - pxi;
    const float by = (y > 0 ? S::ld(a.p1, i - W, a.pdec) : 0.f) - pyi;
    float div = bx + by;
    float pzi = 0.f;
    if constexpr (THREE) {
        pzi = S::ld(a.p2, i, a.pdec);
        const float bz = (z > 0 ? S::ld(a.p2, i - WH, a.pdec) : 0.f) - pzi;
        if (!a.skip_bz) div = div + bz;
    }
    const float uo = a.u_in[i];
    const float fi = a.f[i];
    float uu = uo - a.tau * div;
    if constexpr (DATA == TGVDCT_DATA_L1) {
        const float umf = uu - fi;
        if (umf > a.tau_lambda) uu = uu - a.tau_lambda;
        else if (umf < -a.tau_lambda) uu = uu + a.tau_lambda;
        else uu = fi;
    } else {
        uu = (uu + a.tau_lambda * fi) / (1.f + a.tau_lambda);
    }
    a.u[i] = uu;
    a.ubar_out[i] = uu + a.theta * (uu - uo);

    // div q with Neumann forward differences          (tgv2_common.cu:290-318)
    const float qxx = S::ld(a.qxx, i, a.qdec);
    const float qyy = S::ld(a.qyy, i, a.qdec);
    const float qxy = S::ld(a.qxy, i, a.qdec);
    const float fx_qxx = xl ? S::ld(a.qxx, i + 1, a.qdec) - qxx : 0.f;
    const float fy_qxy = yl ? S::ld(a.qxy, i + W, a.qdec) - qxy : 0.f;
    const float fy_qyy = yl ? S::ld(a.qyy, i + W, a.qdec) - qyy : 0.f;
    const float fx_qxy = xl ? S::ld(a.qxy, i + 1, a.qdec) - qxy : 0.f;
    float dx = fx_qxx + fy_qxy;
    float dy = fy_qyy + fx_qxy;
    float dz = 0.f;
    if constexpr (THREE) {
        const bool zl = z + 1 < a.D;
        const float qzz = S::ld(a.qzz, i, a.qdec);
        const float qxz = S::ld(a.qxz, i, a.qdec);
        const float qyz = S::ld(a.qyz, i, a.qdec);
        const float fz_qxz = zl ? S::ld(a.qxz, i + WH, a.qdec) - qxz : 0.f;
        const float fz_qyz = zl ? S::ld(a.qyz, i + WH, a.qdec) - qyz : 0.f;
        const float fz_qzz = zl ? S::ld(a.qzz, i + WH, a.qdec) - qzz : 0.f;
        const float fx_qxz = xl ? S::ld(a.qxz, i + 1, a.qdec) - qxz : 0.f;
        const float fy_qyz = yl ? S::ld(a.qyz, i + W, a.qdec) - qyz : 0.f;
        dx = dx + fz_qxz;
        dy = dy + fz_qyz;
        dz = (fz_qzz + fx_qxz) + fy_qyz;
    }

    // v <- v - tau (div q - p), vbar                     (tgv2_common.cu:338-347)
    {
        const float vo = a.v_in[0][i];
        const float vn = vo - a.tau * (dx - pxi);
        a.v0[i] = vn;
        a.vbo[0][i] = vn + a.theta * (vn - vo);
    }
    {
        const float vo = a.v_in[1][i];
        const float vn = vo - a.tau * (dy - pyi);
        a.v1[i] = vn;
        a.vbo[1][i] = vn + a.theta * (vn - vo);
    }
    if constexpr (THREE) {
        const float vo = a.v_in[2][i];
        const float vn = vo - a.tau * (dz - pzi);
        a.v2[i] = vn;
        a.vbo[2][i] = vn + a.theta * (vn - vo);
    }
}

// ---- fused single-pass iteration ---------------------------------------------------------
//
// One block owns an FX x TY column tile and marches along z through `zchunk`
// planes.  Its threads cover the tile plus a one-voxel halo, E = (FX+2) x (TY+2):
// every thread loads ubar and vbar of its own position, the halo threads
// recompute the dual updates the tile's stencils need (p on the -x/-y side, q on
// the +x/+y side), and the interior threads do the primal update.  Per plane s:
//
//   registers   ubar(s+1), vbar(s+1), p(s), q(s+1), u(s), f(s), v(s) own, loaded one
//               plane ahead (the loads of plane s+1 are in flight during plane s)
//   smem        ubar/vbar planes s, s+1 over E; p_new(s) over E; q_new planes s, s+1
//   barrier A   ubar/vbar(s+1) in smem
//   dual        p_new(s) on [x0-1, x0+FX) x [y0-1, y0+TY), q_new(s+1) on
//               [x0, x0+FX] x [y0, y0+TY]
//   barrier B
//   primal      u, ubar', v, vbar' at (x, y, s); p_new(s), q_new(s) written out
//
// The fields read with a stencil are double-buffered (in: set cur, out: set cur^1)
// because a neighbouring block may advance a voxel this block still recomputes.
// Per voxel and iteration the kernel moves 18 loads + 17 stores of the state
// (140 bytes in FP32) plus halo re-reads that L2 serves.  The arithmetic of every
// dual and primal update is the same sequence as in the two-pass kernels, so the
// two give identical results.
constexpr int FX = 32;

template <class T>
struct FusedArgs {
    int W, H, D, zchunk;
    size_t WH;
    const float* __restrict__ f;
    float* __restrict__ u;
    float* __restrict__ v[3];
    const float* __restrict__ ubar_in;
    const float* __restrict__ vbar_in[3];
    const T* __restrict__ p_in[3];
    const T* __restrict__ q_in[6];
    float* __restrict__ ubar_out;
    float* __restrict__ vbar_out[3];
    T* __restrict__ p_out[3];
    T* __restrict__ q_out[6];
    float tau, sigma, theta, tau_lambda, alpha0, alpha1;
    float penc, pdec, qenc, qdec;
    int skip_bz;
};

// q component slots in the fused kernel's arrays: xx yy xy (2-D) then zz xz yz
enum { QXX = 0, QYY = 1, QXY = 2, QZZ = 3, QXZ = 4, QYZ = 5 };

template <int NC, int NQ>
struct Prefetch {
    float ub, vb[NC], p[NC], q[NQ], u, f, v[NC];
};

template <int TY>
constexpr int fused_threads() {
    return ((FX + 2) * (TY + 2) + 31) / 32 * 32;
}

template <int TY, bool THREE>
constexpr size_t fused_smem_floats() {
    constexpr int NE = (FX + 2) * (TY + 2);
    constexpr int NC = THREE ? 3 : 2, NQ = THREE ? 6 : 3;
    return (size_t)NE * (2 + 2 * NC + NC + 2 * NQ);
}

template <int PREC, bool THREE, int DATA, int TY>
__global__ void __launch_bounds__(fused_threads<TY>())
    tgv_fused_kernel(FusedArgs<typename Dual<PREC>::T> a) {
    using S = Dual<PREC>;
    constexpr int EX = FX + 2, EY = TY + 2, NE = EX * EY;
    constexpr int NC = THREE ? 3 : 2, NQ = THREE ? 6 : 3;
    extern __shared__ float smem[];
    float* s_ub = smem;                  // [2][NE]
    float* s_vb = s_ub + 2 * NE;         // [2][NC][NE]
    float* s_p = s_vb + 2 * NC * NE;     // [NC][NE]
    float* s_q = s_p + NC * NE;          // [2][NQ][NE]
    auto UB = [&](int slot) { return s_ub + slot * NE; };
    auto VB = [&](int slot, int c) { return s_vb + (slot * NC + c) * NE; };
    auto QS = [&](int slot, int k) { return s_q + (slot * NQ + k) * NE; };
    // q component -> storage slot of the state (xx yy zz xy xz yz)
    constexpr int qmap[6] = {0, 1, 3, 2, 4, 5};

    const int tid = threadIdx.x;
    const bool active = tid < NE;
    const int ex = tid % EX, ey = tid / EX;
    const int x = (int)blockIdx.x * FX + ex - 1;
    const int y = (int)blockIdx.y * TY + ey - 1;
    const bool in_dom = active && x >= 0 && x < a.W && y >= 0 && y < a.H;
    const bool in_rp = in_dom && ex < EX - 1 && ey < EY - 1;
    const bool in_rq = in_dom && ex >= 1 && ey >= 1;
    const bool interior = in_rp && in_rq;
    const bool xl = x + 1 < a.W, yl = y + 1 < a.H;
    const int D = a.D;
    const int z0 = (int)blockIdx.z * a.zchunk;
    const int z1 = min(D, z0 + a.zchunk);
    const size_t col = in_dom ? (size_t)y * a.W + x : 0;
    auto idx = [&](int z) { return (size_t)z * a.WH + col; };
    if constexpr (kCheckBounds) {  // the column, its last plane, the staging position
        bool ok = true;
        if (in_dom) {
            ok = TGV_IN_BOUNDS(col, a.WH, 3) && ok;
            ok = TGV_IN_BOUNDS(idx(z1 - 1), a.WH * (size_t)D, 4) && ok;
        }
        if (active) ok = TGV_IN_BOUNDS(ey * EX + ex, NE, 5) && ok;
        if (__syncthreads_or(!ok)) return;
    }

    auto load = [&](Prefetch<NC, NQ>& r, int s) {
        if (in_dom && s + 1 < D) {
            const size_t i = idx(s + 1);
            r.ub = a.ubar_in[i];
#pragma unroll
            for (int c = 0; c < NC; ++c) r.vb[c] = a.vbar_in[c][i];
        }
        if (in_rp) {
            const size_t i = idx(s);
#pragma unroll
            for (int c = 0; c < NC; ++c) r.p[c] = S::ld(a.p_in[c], i, a.pdec);
        }
        if (in_rq && s + 1 < D) {
            const size_t i = idx(s + 1);
#pragma unroll
            for (int k = 0; k < NQ; ++k) r.q[k] = S::ld(a.q_in[qmap[k]], i, a.qdec);
        }
        if (interior) {
            const size_t i = idx(s);
            r.u = a.u[i];
            r.f = a.f[i];
#pragma unroll
            for (int c = 0; c < NC; ++c) r.v[c] = a.v[c][i];
        }
    };
    // the value the state stores (and the next iteration reads back)
    auto qp = [&](float v) {
        if constexpr (PREC == TGVDCT_STATE_FP32) return v;
        typename S::T t[1];
        S::st(t, 0, v, a.penc);
        return S::ld(t, 0, a.pdec);
    };
    auto qq = [&](float v) {
        if constexpr (PREC == TGVDCT_STATE_FP32) return v;
        typename S::T t[1];
        S::st(t, 0, v, a.qenc);
        return S::ld(t, 0, a.qdec);
    };
    // q <- proj(q + sigma E vbar) at plane z of this position; vb = vbar(z) own,
    // vbz = vbar(z-1) own (0 below the volume), neighbours from smem slot `slot`
    auto dual_q = [&](const float* qold, const float* vb, const float* vbz, int slot, int z,
                      int out_slot) {
        const float vbx_x = x > 0 ? VB(slot, 0)[tid - 1] : 0.f;
        const float vby_x = x > 0 ? VB(slot, 1)[tid - 1] : 0.f;
        const float vbx_y = y > 0 ? VB(slot, 0)[tid - EX] : 0.f;
        const float vby_y = y > 0 ? VB(slot, 1)[tid - EX] : 0.f;
        const float exx = vbx_x - vb[0];
        const float eyy = vby_y - vb[1];
        const float exy = ((vby_x - vb[1]) + (vbx_y - vb[0])) * 0.5f;
        float qxx = __fmaf_rn(a.sigma, exx, qold[QXX]);
        float qyy = __fmaf_rn(a.sigma, eyy, qold[QYY]);
        float qxy = __fmaf_rn(a.sigma, exy, qold[QXY]);
        float sq = qxx * qxx + qyy * qyy + 2.f * qxy * qxy;
        float qzz = 0.f, qxz = 0.f, qyz = 0.f;
        if constexpr (THREE) {
            const float vbz_x = x > 0 ? VB(slot, 2)[tid - 1] : 0.f;
            const float vbz_y = y > 0 ? VB(slot, 2)[tid - EX] : 0.f;
            const float ezz = vbz[2] - vb[2];
            const float exz = ((vbz_x - vb[2]) + (vbz[0] - vb[0])) * 0.5f;
            const float eyz = ((vbz_y - vb[2]) + (vbz[1] - vb[1])) * 0.5f;
            qzz = __fmaf_rn(a.sigma, ezz, qold[QZZ]);
            qxz = __fmaf_rn(a.sigma, exz, qold[QXZ]);
            qyz = __fmaf_rn(a.sigma, eyz, qold[QYZ]);
            sq = sq + qzz * qzz + 2.f * qxz * qxz + 2.f * qyz * qyz;
        }
        (void)z;
        const float qn = fmaxf(1.f, sqrtf(sq) / a.alpha0);
        QS(out_slot, QXX)[tid] = qq(qxx / qn);
        QS(out_slot, QYY)[tid] = qq(qyy / qn);
        QS(out_slot, QXY)[tid] = qq(qxy / qn);
        if constexpr (THREE) {
            QS(out_slot, QZZ)[tid] = qq(qzz / qn);
            QS(out_slot, QXZ)[tid] = qq(qxz / qn);
            QS(out_slot, QYZ)[tid] = qq(qyz / qn);
        }
    };

    // ---- prologue: ubar/vbar(z0) into smem, p_new(z0-1) own, q_new(z0) over R_q
    float ub_cur = 0.f, vb_cur[NC], p_prev[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) vb_cur[c] = 0.f, p_prev[c] = 0.f;
    if (in_dom) {
        const size_t i = idx(z0);
        ub_cur = a.ubar_in[i];
#pragma unroll
        for (int c = 0; c < NC; ++c) vb_cur[c] = a.vbar_in[c][i];
    }
    if (active) {
        UB(z0 & 1)[tid] = ub_cur;
#pragma unroll
        for (int c = 0; c < NC; ++c) VB(z0 & 1, c)[tid] = vb_cur[c];
    }
    if constexpr (THREE) {
        if (interior && z0 > 0) {
            // p_new(z0 - 1) at this column, for B_z p at plane z0
            const size_t i = idx(z0 - 1);
            const float ubm = a.ubar_in[i];
            const float gx = xl ? a.ubar_in[i + 1] - ubm : 0.f;
            const float gy = yl ? a.ubar_in[i + a.W] - ubm : 0.f;
            const float gz = ub_cur - ubm;
            float px = __fmaf_rn(a.sigma, gx - a.vbar_in[0][i], S::ld(a.p_in[0], i, a.pdec));
            float py = __fmaf_rn(a.sigma, gy - a.vbar_in[1][i], S::ld(a.p_in[1], i, a.pdec));
            float pz = __fmaf_rn(a.sigma, gz - a.vbar_in[2][i], S::ld(a.p_in[2], i, a.pdec));
            const float nrm = fmaxf(1.f, norm3df(px, py, pz) / a.alpha1);
            p_prev[0] = qp(px / nrm);
            p_prev[1] = qp(py / nrm);
            p_prev[2] = qp(pz / nrm);
        }
    }
    Prefetch<NC, NQ> pre;
    load(pre, z0);
    __syncthreads();
    if (in_rq) {
        float qold[NQ], vbz[NC];
        const size_t i = idx(z0);
#pragma unroll
        for (int k = 0; k < NQ; ++k) qold[k] = S::ld(a.q_in[qmap[k]], i, a.qdec);
#pragma unroll
        for (int c = 0; c < NC; ++c) vbz[c] = (THREE && z0 > 0) ? a.vbar_in[c][i - a.WH] : 0.f;
        dual_q(qold, vb_cur, vbz, z0 & 1, z0, z0 & 1);
    }

    // ---- march through the planes of the chunk
    for (int s = z0; s < z1; ++s) {
        const int cs = s & 1, ns = cs ^ 1;
        const bool has_next = s + 1 < D;
        const Prefetch<NC, NQ> cur = pre;
        if (s + 1 < z1) load(pre, s + 1);
        if (active) {
            UB(ns)[tid] = (in_dom && has_next) ? cur.ub : 0.f;
#pragma unroll
            for (int c = 0; c < NC; ++c) VB(ns, c)[tid] = (in_dom && has_next) ? cur.vb[c] : 0.f;
        }
        __syncthreads();  // A

        if (in_rp) {  // p_new(s)
            const float ubs = ub_cur;
            const float gx = xl ? UB(cs)[tid + 1] - ubs : 0.f;
            const float gy = yl ? UB(cs)[tid + EX] - ubs : 0.f;
            float px = __fmaf_rn(a.sigma, gx - vb_cur[0], cur.p[0]);
            float py = __fmaf_rn(a.sigma, gy - vb_cur[1], cur.p[1]);
            float nrm;
            float pz = 0.f;
            if constexpr (THREE) {
                const float gz = has_next ? cur.ub - ubs : 0.f;
                pz = __fmaf_rn(a.sigma, gz - vb_cur[2], cur.p[2]);
                nrm = norm3df(px, py, pz);
            } else {
                nrm = sqrtf(px * px + py * py);
            }
            nrm = fmaxf(1.f, nrm / a.alpha1);
            s_p[tid] = qp(px / nrm);
            s_p[NE + tid] = qp(py / nrm);
            if constexpr (THREE) s_p[2 * NE + tid] = qp(pz / nrm);
        }
        if (in_rq && has_next) dual_q(cur.q, cur.vb, vb_cur, ns, s + 1, ns);  // q_new(s+1)
        __syncthreads();  // B

        if (interior) {
            const size_t i = idx(s);
            const float pxi = s_p[tid], pyi = s_p[NE + tid];
            const float bx = (x > 0 ? s_p[tid - 1] : 0.f) - pxi;
            const float by = (y > 0 ? s_p[NE + tid - EX] : 0.f) - pyi;
            float div = bx + by;
            float pzi = 0.f;
            if constexpr (THREE) {
                pzi = s_p[2 * NE + tid];
                const float bz = p_prev[2] - pzi;
                if (!a.skip_bz) div = div + bz;
            }
            const float uo = cur.u, fi = cur.f;
            float uu = uo - a.tau * div;
            if constexpr (DATA == TGVDCT_DATA_L1) {
                const float umf = uu - fi;
                if (umf > a.tau_lambda) uu = uu - a.tau_lambda;
                else if (umf < -a.tau_lambda) uu = uu + a.tau_lambda;
                else uu = fi;
            } else {
                uu = (uu + a.tau_lambda * fi) / (1.f + a.tau_lambda);
            }
            a.u[i] = uu;
            a.ubar_out[i] = uu + a.theta * (uu - uo);

            const float qxx = QS(cs, QXX)[tid], qyy = QS(cs, QYY)[tid], qxy = QS(cs, QXY)[tid];
            const float fx_qxx = xl ? QS(cs, QXX)[tid + 1] - qxx : 0.f;
            const float fy_qxy = yl ? QS(cs, QXY)[tid + EX] - qxy : 0.f;
            const float fy_qyy = yl ? QS(cs, QYY)[tid + EX] - qyy : 0.f;
            const float fx_qxy = xl ? QS(cs, QXY)[tid + 1] - qxy : 0.f;
            float d[3];
            d[0] = fx_qxx + fy_qxy;
            d[1] = fy_qyy + fx_qxy;
            d[2] = 0.f;
            float qzz = 0.f, qxz = 0.f, qyz = 0.f;
            if constexpr (THREE) {
                qzz = QS(cs, QZZ)[tid];
                qxz = QS(cs, QXZ)[tid];
                qyz = QS(cs, QYZ)[tid];
                const float fz_qxz = has_next ? QS(ns, QXZ)[tid] - qxz : 0.f;
                const float fz_qyz = has_next ? QS(ns, QYZ)[tid] - qyz : 0.f;
                const float fz_qzz = has_next ? QS(ns, QZZ)[tid] - qzz : 0.f;
                const float fx_qxz = xl ? QS(cs, QXZ)[tid + 1] - qxz : 0.f;
                const float fy_qyz = yl ? QS(cs, QYZ)[tid + EX] - qyz : 0.f;
                d[0] = d[0] + fz_qxz;
                d[1] = d[1] + fz_qyz;
                d[2] = (fz_qzz + fx_qxz) + fy_qyz;
            }
            const float pv[3] = {pxi, pyi, pzi};
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const float vo = cur.v[c];
                const float vn = vo - a.tau * (d[c] - pv[c]);
                a.v[c][i] = vn;
                a.vbar_out[c][i] = vn + a.theta * (vn - vo);
            }
#pragma unroll
            for (int c = 0; c < NC; ++c) S::st(a.p_out[c], i, pv[c], a.penc);
            S::st(a.q_out[0], i, qxx, a.qenc);
            S::st(a.q_out[1], i, qyy, a.qenc);
            S::st(a.q_out[3], i, qxy, a.qenc);
            if constexpr (THREE) {
                S::st(a.q_out[2], i, qzz, a.qenc);
                S::st(a.q_out[4], i, qxz, a.qenc);
                S::st(a.q_out[5], i, qyz, a.qenc);
            }
#pragma unroll
            for (int c = 0; c < NC; ++c) p_prev[c] = pv[c];
        }
        ub_cur = cur.ub;
#pragma unroll
        for (int c = 0; c < NC; ++c) vb_cur[c] = cur.vb[c];
    }
}

// ---- fused single pass, TMA pipeline -------------------------------------------------
//
// Same tile decomposition and update sequence as tgv_fused_kernel, software-
// pipelined across planes.  Step t of a block computes, in one phase,
//   the primal update at plane t                (needs p_new(t), p_new(t-1), q_new(t), q_new(t+1))
//   the dual update p_new(t+1) on the -x/-y rim (ubar, vbar, p of planes t+1, t+2)
//   the dual update q_new(t+2) on the +x/+y rim (vbar, q of planes t+1, t+2)
// and ends with the block's single barrier; p_new lives in a 2-deep and q_new in a
// 3-deep shared-memory ring.  The stencil fields (ubar, vbar, p, q) of every plane
// arrive through the tensor memory accelerator: one thread issues 13 box loads
// (tile plus one-voxel halo) per plane into a ring of NS stages, completing on the
// stage's mbarrier (expect_tx); step t reads planes t+1 and t+2, so NS - 2 planes are
// in flight while it computes.  The tile fields u, f, v (read only at a thread's
// own voxel) are loaded into registers two planes ahead and prefetched into L2 three
// planes ahead: without the L2 prefetch the primal update waited on those loads and
// the iteration took 334 us at 256 x 256 x 192 instead of 292 us.  Interior voxels
// are one warp per tile row (aligned, coalesced stores); three halo warps take the
// rim.
namespace tma {

constexpr int TX = 32, TY = 8;
constexpr int EXW = TX + 2, EYH = TY + 2, NE = EXW * EYH;  // 34 x 10 positions
constexpr int NTHREADS = 352;                              // 8 interior + 3 halo warps
constexpr int PRODUCER = 256;                              // first halo thread issues TMA
// 200 ms: a plane normally lands in microseconds.  The consumers' waits take their
// limit from the launch (tgvdct_set_pipeline_wait_limit; this is the default); the
// drain of a block's own copies on an error exit always waits up to this long.
constexpr uint64_t WAIT_NS = 200000000ull;
// u, f and v of plane t + TILE_PREFETCH are prefetched into L2 at step t
constexpr int TILE_PREFETCH = 3;

__host__ __device__ constexpr int a128(int b) { return (b + 127) / 128 * 128; }

template <int PREC>
struct Geo {
    static constexpr int DES = PREC == TGVDCT_STATE_FP32 ? 4 : 2;  // dual element bytes
    // ubar / vbar boxes: x0-4 .. x0+35, rows y0-1 .. y0+8 (the dual steps read the
    // +x/+y neighbours of ubar and the -x/-y neighbours of vbar)
    static constexpr int XO_F = 4, BW_F = TX + 8;
    // p is read only at R_p (x0-1 .. x0+31, y0-1 .. y0+7) and q only at R_q
    // (x0 .. x0+32, y0 .. y0+8): nine rows each, x start and width rounded to 16 bytes
    static constexpr int PQ_ROWS = TY + 1;
    static constexpr int XO_P = DES == 4 ? 4 : 8;
    static constexpr int BW_P = DES == 4 ? TX + 4 : TX + 8;  // x0-XO_P .. x0+31
    static constexpr int BW_Q = DES == 4 ? TX + 4 : TX + 8;  // x0 .. x0+35 (x0+39)
    static constexpr int BOX_F = a128(BW_F * EYH * 4);
    static constexpr int BOX_P = a128(BW_P * PQ_ROWS * DES);
    static constexpr int BOX_Q = a128(BW_Q * PQ_ROWS * DES);
    // stage: ubar, vbar[3] | p[3] | q[6]
    static constexpr int OFF_P = 4 * BOX_F;
    static constexpr int OFF_Q = OFF_P + 3 * BOX_P;
    static constexpr int STAGE = OFF_Q + 6 * BOX_Q;
    // bytes the TMA delivers per plane (what expect_tx must announce)
    static constexpr uint32_t tx_bytes(bool three) {
        const int nc = three ? 3 : 2, nq = three ? 6 : 3;
        return (uint32_t)((1 + nc) * BW_F * EYH * 4 + nc * BW_P * PQ_ROWS * DES +
                          nq * BW_Q * PQ_ROWS * DES);
    }
};

struct alignas(64) Maps {
    CUtensorMap ub, vb[3], p[3], q[6];  // q in kernel slot order
};

template <class T>
struct Args {
    Maps maps;
    int W, H, D, zchunk;
    size_t WH;
    const float* f;
    const float* u;  // u and v of the input state
    const float* v[3];
    float* u_out;  // u and v of the output state (the same buffers in the loop)
    float* v_out[3];
    float* ubar_out;
    float* vbar_out[3];
    T* p_out[3];
    T* q_out[6];  // state order: xx yy zz xy xz yz
    float tau, sigma, theta, tau_lambda, alpha0, alpha1;
    float thr_p, thr_q;  // squared-norm bounds below which the projections are skipped
    float penc, pdec, qenc, qdec;
    int skip_bz;
    int* err;
    unsigned long long wait_ns;  // limit of the consumers' pipeline waits (0: one test)
    const uint8_t* dom;  // masked deshade domain (null: every voxel)
    // per-block plane ranges of this grid for that domain (null: whole chunks)
    const uint32_t* tile_active;
};

__device__ __forceinline__ uint32_t su32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
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
// One potentially blocking test: the thread is suspended until the phase completes
// or a hardware time window ends, so a waiting warp neither spins nor oversleeps.
__device__ __forceinline__ bool mtry(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(su32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait; limit_ns == 0 gives up at the first test that finds the phase open.
__device__ bool mwait(uint64_t* bar, uint32_t parity, int* err, uint64_t limit_ns) {
    if (mtest(bar, parity)) return true;
    if (limit_ns == 0) {
        atomicExch(err, 1);
        return false;
    }
    uint64_t t0, t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    while (true) {
        if (mtry(bar, parity)) return true;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        if (t - t0 > limit_ns) {
            atomicExch(err, 1);
            return false;
        }
    }
}
__device__ __forceinline__ void tma_load(void* dst, const CUtensorMap* map, int x, int y, int z,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(su32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(su32(bar))
        : "memory");
}

}  // namespace tma

// p <- proj_{alpha1}(p + sigma (g - vb)), the reference's tgv_kernel_part22 arithmetic.
// The division by max(1, |p|/alpha1) is skipped when that factor is 1 (x / 1 == x).
// thr = alpha1^2 (1 - 2^-19): while the float sum of squares stays at or below it,
// |p| / alpha1 rounds to at most 1 whatever the last-bit errors of the sum (5
// roundings) and of norm3df (a few ulp), so the projection is the identity and the
// norm is not evaluated; the result is bit-identical to evaluating it.
template <bool THREE>
__device__ __forceinline__ void dual_p_update(const float* g, const float* vb, float* p,
                                              float sigma, float alpha1, float thr) {
    p[0] = __fmaf_rn(sigma, g[0] - vb[0], p[0]);
    p[1] = __fmaf_rn(sigma, g[1] - vb[1], p[1]);
    float ss = p[0] * p[0] + p[1] * p[1];  // also the 2-D norm's argument (tgv2_common_2d.cu:113)
    if constexpr (THREE) {
        p[2] = __fmaf_rn(sigma, g[2] - vb[2], p[2]);
        ss = ss + p[2] * p[2];
    }
    if (!(ss > thr)) return;  // inside the ball (NaN: the reference divides by 1 as well)
    float nrm;
    if constexpr (THREE) nrm = norm3df(p[0], p[1], p[2]);
    else nrm = sqrtf(ss);
    nrm = fmaxf(1.f, nrm / alpha1);
    if (nrm > 1.f) {
        p[0] = p[0] / nrm;
        p[1] = p[1] / nrm;
        if constexpr (THREE) p[2] = p[2] / nrm;
    }
}

// q <- proj_{alpha0}(q + sigma E vbar); xm/ym/zm: vbar at x-1 / y-1 / z-1 (0 outside);
// q in slot order xx yy xy zz xz yz (tgv_kernel_part5 arithmetic)
// thr = alpha0^2 (1 - 2^-19): at or below it sqrtf(sq) / alpha0 rounds to at most 1.
template <bool THREE>
__device__ __forceinline__ void dual_q_update(const float* vb, const float* xm, const float* ym,
                                              const float* zm, float* q, float sigma,
                                              float alpha0, float thr) {
    const float exx = xm[0] - vb[0];
    const float eyy = ym[1] - vb[1];
    const float exy = ((xm[1] - vb[1]) + (ym[0] - vb[0])) * 0.5f;
    q[0] = __fmaf_rn(sigma, exx, q[0]);
    q[1] = __fmaf_rn(sigma, eyy, q[1]);
    q[2] = __fmaf_rn(sigma, exy, q[2]);
    float sq = q[0] * q[0] + q[1] * q[1] + 2.f * q[2] * q[2];
    if constexpr (THREE) {
        const float ezz = zm[2] - vb[2];
        const float exz = ((xm[2] - vb[2]) + (zm[0] - vb[0])) * 0.5f;
        const float eyz = ((ym[2] - vb[2]) + (zm[1] - vb[1])) * 0.5f;
        q[3] = __fmaf_rn(sigma, ezz, q[3]);
        q[4] = __fmaf_rn(sigma, exz, q[4]);
        q[5] = __fmaf_rn(sigma, eyz, q[5]);
        sq = sq + q[3] * q[3] + 2.f * q[4] * q[4] + 2.f * q[5] * q[5];
    }
    if (!(sq > thr)) return;
    const float qn = fmaxf(1.f, sqrtf(sq) / alpha0);
    constexpr int NQ = THREE ? 6 : 3;
    if (qn > 1.f) {
#pragma unroll
        for (int k = 0; k < NQ; ++k) q[k] = q[k] / qn;
    }
}

template <int PREC, bool THREE, int DATA, int NS, bool MASKED>
__global__ void __launch_bounds__(tma::NTHREADS, 2)
    tgv_fused_tma_kernel(const __grid_constant__ tma::Args<typename Dual<PREC>::T> a) {
    using namespace tma;
    using S = Dual<PREC>;
    using G = Geo<PREC>;
    using T = typename S::T;
    constexpr int NC = THREE ? 3 : 2, NQ = THREE ? 6 : 3;
    extern __shared__ __align__(128) uint8_t smem_raw[];
    uint8_t* smem = align_shared<128>(smem_raw);
    uint8_t* stages = smem;                                  // NS x STAGE
    float* sP = (float*)(smem + NS * G::STAGE);              // [2][3][NE]
    float* sQ = sP + 2 * 3 * NE;                             // [3][6][NE]
    __shared__ uint64_t full[NS];

    int zr0 = (int)blockIdx.z * a.zchunk, zr1 = min(a.D, zr0 + a.zchunk);
    if constexpr (MASKED) {
        // Only the planes in which some of this block's own voxels are in the domain
        // have anything to update; none: the block leaves.  The other planes are frozen,
        // and both stencil sets hold the values the neighbours read there.  One entry
        // per block, so the whole block takes the same branch, before any barrier.
        if (a.tile_active) {
            const uint32_t r = a.tile_active[((size_t)blockIdx.z * gridDim.y + blockIdx.y) *
                                                 gridDim.x + blockIdx.x];
            if (r == 0) return;
            zr0 = (int)(r >> 16);
            zr1 = (int)(r & 0xffffu);
        }
    }
    // a pipeline wait of an earlier block or launch timed out: do nothing more
    // (one read, shared by the whole block, so every thread takes the same branch)
    if (__syncthreads_or(threadIdx.x == 0 ? *(volatile int*)a.err : 0)) return;
    const int tid = threadIdx.x;
    int ex, ey;
    bool interior = false, active = true;
    if (tid < 256) {
        ex = (tid & 31) + 1;
        ey = (tid >> 5) + 1;
        interior = true;
    } else if (tid < 256 + NE - TX * TY) {
        const int h = tid - 256;
        if (h < EXW) { ex = h; ey = 0; }
        else if (h < 2 * EXW) { ex = h - EXW; ey = EYH - 1; }
        else if (h < 2 * EXW + TY) { ex = 0; ey = 1 + (h - 2 * EXW); }
        else { ex = EXW - 1; ey = 1 + (h - 2 * EXW - TY); }
    } else {
        ex = 0;
        ey = 0;
        active = false;
    }
    const int e = ey * EXW + ex;
    const int x0 = (int)blockIdx.x * TX, y0 = (int)blockIdx.y * TY;
    const int x = x0 - 1 + ex, y = y0 - 1 + ey;
    const bool in_dom = active && x >= 0 && x < a.W && y >= 0 && y < a.H;
    const bool in_rp = in_dom && ex < EXW - 1 && ey < EYH - 1;
    const bool in_rq = in_dom && ex >= 1 && ey >= 1;
    interior = interior && in_dom;
    const bool xl = x + 1 < a.W, yl = y + 1 < a.H;
    const int D = a.D;
    const int z0 = zr0, z1 = zr1;      // this block's planes
    const int pbase = max(z0 - 1, 0);  // first plane this block loads; slots count from it
    const int plast = min(D - 1, z1);  // last plane this block reads
    // 32-bit voxel indices: the host runs this kernel only on volumes of < 2^32 voxels
    const uint32_t wh = (uint32_t)a.WH;
    const uint32_t col = in_dom ? (uint32_t)y * (uint32_t)a.W + (uint32_t)x : 0u;

    const int of = ey * G::BW_F + ex + G::XO_F - 1;  // offset in FP32 stencil boxes
    const int odp = ey * G::BW_P + ex + G::XO_P - 1;  // offset in p boxes (R_p only)
    const int odq = (ey - 1) * G::BW_Q + ex - 1;      // offset in q boxes (R_q only)
    if constexpr (kCheckBounds) {
        // every index this thread's role uses: its column over the chunk, the staged
        // boxes (with the neighbours the dual steps read) and the p/q rings
        constexpr int nF = G::BW_F * EYH, nP = G::BW_P * G::PQ_ROWS, nQ = G::BW_Q * G::PQ_ROWS;
        bool ok = true;
        if (in_dom) {
            ok = TGV_IN_BOUNDS(col, a.WH, 10) && ok;
            ok = TGV_IN_BOUNDS((size_t)(z1 - 1) * a.WH + col, a.WH * (size_t)D, 11) && ok;
        }
        if (in_rp) {
            ok = TGV_IN_BOUNDS(of, nF, 12) && ok;
            if (xl) ok = TGV_IN_BOUNDS(of + 1, nF, 13) && ok;
            if (yl) ok = TGV_IN_BOUNDS(of + G::BW_F, nF, 14) && ok;
            ok = TGV_IN_BOUNDS(odp, nP, 15) && ok;
            ok = TGV_IN_BOUNDS(e, NE, 16) && ok;
        }
        if (in_rq) {
            ok = TGV_IN_BOUNDS(of, nF, 17) && ok;
            if (x > 0) ok = TGV_IN_BOUNDS(of - 1, nF, 18) && ok;
            if (y > 0) ok = TGV_IN_BOUNDS(of - G::BW_F, nF, 19) && ok;
            ok = TGV_IN_BOUNDS(odq, nQ, 20) && ok;
            ok = TGV_IN_BOUNDS(e, NE, 21) && ok;
        }
        if (interior) {
            if (x > 0) ok = TGV_IN_BOUNDS(e - 1, NE, 22) && ok;
            if (y > 0) ok = TGV_IN_BOUNDS(e - EXW, NE, 23) && ok;
            if (xl) ok = TGV_IN_BOUNDS(e + 1, NE, 24) && ok;
            if (yl) ok = TGV_IN_BOUNDS(e + EXW, NE, 25) && ok;
        }
        if (__syncthreads_or(!ok)) return;
    }
    auto st_of = [&](int plane) { return stages + ((plane - pbase) % NS) * G::STAGE; };
    // field views of a stage (st: the stage's base)
    auto fb = [&](const uint8_t* st, int field) -> const float* {  // 0 ubar, 1-3 vbar
        return (const float*)(st + field * G::BOX_F);
    };
    auto pb = [&](const uint8_t* st, int c) -> const T* {
        return (const T*)(st + G::OFF_P + c * G::BOX_P);
    };
    auto qb = [&](const uint8_t* st, int k) -> const T* {
        return (const T*)(st + G::OFF_Q + k * G::BOX_Q);
    };
    auto Pslot = [&](int plane) { return sP + (plane & 1) * 3 * NE; };  // [3][NE]
    auto Qslot = [&](int plane) { return sQ + (plane % 3) * 6 * NE; };  // [6][NE]
    auto dec_p = [&](T v) { T t[1] = {v}; return S::ld(t, 0, a.pdec); };
    auto dec_q = [&](T v) { T t[1] = {v}; return S::ld(t, 0, a.qdec); };
    auto rq_p = [&](float v) {
        if constexpr (PREC == TGVDCT_STATE_FP32) return v;
        T t[1];
        S::st(t, 0, v, a.penc);
        return S::ld(t, 0, a.pdec);
    };
    auto rq_q = [&](float v) {
        if constexpr (PREC == TGVDCT_STATE_FP32) return v;
        T t[1];
        S::st(t, 0, v, a.qenc);
        return S::ld(t, 0, a.qdec);
    };
    auto issue = [&](int plane) {  // producer thread only
        if (plane < 0 || plane > plast) return;
        uint8_t* st = st_of(plane);
        uint64_t* bar = &full[(plane - pbase) % NS];
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)),
                     "r"(G::tx_bytes(THREE))
                     : "memory");
        const int xf = x0 - G::XO_F, xp = x0 - G::XO_P, yb = y0 - 1;
        tma_load(st, &a.maps.ub, xf, yb, plane, bar);
        for (int c = 0; c < NC; ++c) tma_load(st + (1 + c) * G::BOX_F, &a.maps.vb[c], xf, yb, plane, bar);
        for (int c = 0; c < NC; ++c) tma_load(st + G::OFF_P + c * G::BOX_P, &a.maps.p[c], xp, yb, plane, bar);
        for (int k = 0; k < NQ; ++k) tma_load(st + G::OFF_Q + k * G::BOX_Q, &a.maps.q[k], x0, y0, plane, bar);
    };
    bool ok = true;
    int waited_upto = pbase - 1;  // every plane <= this one has landed
    auto wait_plane = [&](int plane) {
        if (plane < 0 || plane > plast || plane <= waited_upto) return;
        const int j = (plane - pbase) / NS;
        if (!mwait(&full[(plane - pbase) % NS], j & 1, a.err, a.wait_ns)) ok = false;
        else waited_upto = plane;
    };
    // p_new over R_p from stage sz (plane z) and sn (plane z+1, or null past the volume):
    // ubar(z) own/+x/+y, ubar(z+1) own, vbar(z) own, p(z)
    // a voxel outside the masked deshade's domain keeps p = q = 0 and u, v unchanged
    auto live = [&](int plane) {
        if constexpr (MASKED) return a.dom[(uint32_t)plane * wh + col] != 0;
        else return true;
    };
    auto dual_p_at = [&](const uint8_t* sz, const uint8_t* sn, bool lv) {
        if (!lv) return make_float3(0.f, 0.f, 0.f);
        const float* ub = fb(sz, 0);
        const float u0 = ub[of];
        float g[3] = {xl ? ub[of + 1] - u0 : 0.f, yl ? ub[of + G::BW_F] - u0 : 0.f, 0.f};
        if constexpr (THREE) g[2] = sn ? fb(sn, 0)[of] - u0 : 0.f;
        float vb[3] = {fb(sz, 1)[of], fb(sz, 2)[of], THREE ? fb(sz, 3)[of] : 0.f};
        float pp[3];
#pragma unroll
        for (int c = 0; c < NC; ++c) pp[c] = dec_p(pb(sz, c)[odp]);
        dual_p_update<THREE>(g, vb, pp, a.sigma, a.alpha1, a.thr_p);
#pragma unroll
        for (int c = 0; c < NC; ++c) pp[c] = rq_p(pp[c]);
        return make_float3(pp[0], pp[1], THREE ? pp[2] : 0.f);
    };
    // q_new over R_q from stage sz (plane z) and sm (plane z-1, or null below the
    // volume): vbar(z) own/-x/-y, vbar(z-1) own, q(z); written to ring slot out
    auto dual_q_at = [&](const uint8_t* sz, const uint8_t* sm, float* out, bool lv) {
        if (!lv) {
#pragma unroll
            for (int k = 0; k < NQ; ++k) out[k * NE + e] = 0.f;
            return;
        }
        float vb[3], xm[3], ym[3], zm[3], q[6];
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const float* box = fb(sz, 1 + c);
            vb[c] = box[of];
            xm[c] = x > 0 ? box[of - 1] : 0.f;
            ym[c] = y > 0 ? box[of - G::BW_F] : 0.f;
            zm[c] = (THREE && sm) ? fb(sm, 1 + c)[of] : 0.f;
        }
#pragma unroll
        for (int k = 0; k < NQ; ++k) q[k] = dec_q(qb(sz, k)[odq]);
        dual_q_update<THREE>(vb, xm, ym, zm, q, a.sigma, a.alpha0, a.thr_q);
#pragma unroll
        for (int k = 0; k < NQ; ++k) out[k * NE + e] = rq_q(q[k]);
    };
    // u, f, v of the next two primal planes: a two-deep register queue, so each load
    // has two planes of work (about the DRAM latency under load) to land
    float tu = 0.f, tf = 0.f, tv[3] = {0.f, 0.f, 0.f};
    float nu = 0.f, nf = 0.f, nv[3] = {0.f, 0.f, 0.f};
    auto load_tile = [&](int z) {  // into the second slot
        if (interior && z < z1) {
            const uint32_t i = (uint32_t)z * wh + col;
            nu = __ldcs(a.u + i);  // read once per iteration: evict-first
            nf = __ldcs(a.f + i);
            for (int c = 0; c < NC; ++c) nv[c] = __ldcs(a.v[c] + i);
        }
    };
    auto advance_tile = [&]() {
        tu = nu;
        tf = nf;
        for (int c = 0; c < 3; ++c) tv[c] = nv[c];
    };
    // and a plane further ahead into L2 (no register waits on a prefetch)
    auto prefetch_tile = [&](int z) {
        if (interior && z < z1) {
            const uint32_t i = (uint32_t)z * wh + col;
            asm volatile("prefetch.global.L2 [%0];" ::"l"(a.u + i));
            asm volatile("prefetch.global.L2 [%0];" ::"l"(a.f + i));
            for (int c = 0; c < NC; ++c) asm volatile("prefetch.global.L2 [%0];" ::"l"(a.v[c] + i));
            if constexpr (MASKED) asm volatile("prefetch.global.L2 [%0];" ::"l"(a.dom + i));
        }
    };

    if (tid == 0) {
        for (int k = 0; k < NS; ++k)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&full[k])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == PRODUCER)
        for (int k = 0; k < NS; ++k) issue(pbase + k);
    int issued_upto = pbase + NS - 1;  // meaningful in the producer only
    load_tile(z0);
    advance_tile();
    load_tile(z0 + 1);
    for (int k = 2; k < TILE_PREFETCH; ++k) prefetch_tile(z0 + k);

    // ---- prologue: p_new(z0-1) own, p_new(z0) over R_p, q_new(z0), q_new(z0+1) over R_q
    wait_plane(z0 - 1);
    wait_plane(z0);
    if (z0 + 1 < D) wait_plane(z0 + 1);
    float p_prev[3] = {0.f, 0.f, 0.f};
    if (ok) {
        const uint8_t* s0 = st_of(z0);
        const uint8_t* s1 = z0 + 1 < D ? st_of(z0 + 1) : nullptr;
        const uint8_t* sm = z0 > 0 ? st_of(z0 - 1) : nullptr;
        if constexpr (THREE) {
            if (interior && z0 > 0) {  // p_new(z0 - 1) at this column
                const float3 pp = dual_p_at(sm, s0, live(z0 - 1));
                p_prev[0] = pp.x;
                p_prev[1] = pp.y;
                p_prev[2] = pp.z;
            }
        }
        if (in_rp) {
            const float3 pp = dual_p_at(s0, s1, live(z0));
            float* Pz = Pslot(z0);
            Pz[e] = pp.x;
            Pz[NE + e] = pp.y;
            if constexpr (THREE) Pz[2 * NE + e] = pp.z;
        }
        if (in_rq) {
            dual_q_at(s0, sm, Qslot(z0), live(z0));
            if (s1) dual_q_at(s1, s0, Qslot(z0 + 1), live(z0 + 1));
        }
    }
    ok = __syncthreads_and(ok);
    if (ok && tid == PRODUCER) {
        // planes z0-1 and z0 are no longer read: their slots take the next planes
        if (z0 > 0) issue(++issued_upto);
        issue(++issued_upto);
    }

    // masked runs: the domain flags of planes t, t + 1, t + 2 of this thread's column,
    // one new flag read per step
    auto live_at = [&](int plane) { return plane < D && live(plane); };
    bool lq0 = true, lq1 = true, lq2 = true;
    if constexpr (MASKED) {
        lq0 = live_at(z0);
        lq1 = live_at(z0 + 1);
        lq2 = live_at(z0 + 2);
    }
    // ring positions of plane t + 1 (stage) and of plane t (p ring) / t (q ring)
    int slot1 = (z0 + 1 - pbase) % NS;
    int pslot = z0 & 1, qslot = z0 % 3;
    for (int t = z0; t < z1 && ok; ++t) {
        const bool p_next = t + 1 < z1;                  // p_new(t+1) feeds primal(t+1)
        const bool q_next = t + 2 <= z1 && t + 2 < D;    // q_new(t+2) feeds primal(t+1)
        if (p_next || q_next) wait_plane(min(t + 2, plast));
        const int slot2 = slot1 + 1 == NS ? 0 : slot1 + 1;
        const uint8_t* S1 = stages + slot1 * G::STAGE;   // plane t + 1
        const uint8_t* S2 = stages + slot2 * G::STAGE;   // plane t + 2
        const float* Pt = sP + pslot * 3 * NE;           // p_new(t)
        float* Pn = sP + (pslot ^ 1) * 3 * NE;           // p_new(t + 1)
        const int q1 = qslot + 1 == 3 ? 0 : qslot + 1, q2 = q1 + 1 == 3 ? 0 : q1 + 1;
        const float* Qt = sQ + qslot * 6 * NE;           // q_new(t)
        const float* Qn = sQ + q1 * 6 * NE;              // q_new(t + 1)
        float* Qnn = sQ + q2 * 6 * NE;                   // q_new(t + 2)
        // A thread whose wait gave up skips the plane; the barrier below shares the
        // outcome and the whole block leaves together.
        if (ok) {
        const float pu = tu, pf = tf, pv0 = tv[0], pv1 = tv[1], pv2 = tv[2];
        advance_tile();
        load_tile(t + 2);
        prefetch_tile(t + TILE_PREFETCH);
        bool lq3 = true;
        if constexpr (MASKED) lq3 = live_at(t + 3);
        // ---- duals for the next planes
        float3 pn = make_float3(0.f, 0.f, 0.f);
        if (in_rp && p_next) pn = dual_p_at(S1, t + 2 < D ? S2 : nullptr, lq1);
        if (in_rq && q_next) dual_q_at(S2, S1, Qnn, lq2);
        // ---- primal at (x, y, t)
        if (interior) {
            const uint32_t i = (uint32_t)t * wh + col;
            float pv[3] = {Pt[e], Pt[NE + e], THREE ? Pt[2 * NE + e] : 0.f};
            const float bx = (x > 0 ? Pt[e - 1] : 0.f) - pv[0];
            const float by = (y > 0 ? Pt[NE + e - EXW] : 0.f) - pv[1];
            float div = bx + by;
            if constexpr (THREE) {
                const float bz = p_prev[2] - pv[2];
                if (!a.skip_bz) div = div + bz;
            }
            float uu = pu - a.tau * div;
            if constexpr (DATA == TGVDCT_DATA_L1) {
                const float umf = uu - pf;
                if (umf > a.tau_lambda) uu = uu - a.tau_lambda;
                else if (umf < -a.tau_lambda) uu = uu + a.tau_lambda;
                else uu = pf;
            } else {
                uu = (uu + a.tau_lambda * pf) / (1.f + a.tau_lambda);
            }
            // outside the domain the stored state is already the frozen one
            const bool lt = lq0;
            if (lt) {
                __stcs(a.u_out + i, uu);
                __stcs(a.ubar_out + i, uu + a.theta * (uu - pu));
            }
            const bool has_next = t + 1 < D;
            const float qxx = Qt[e], qyy = Qt[NE + e], qxy = Qt[2 * NE + e];
            float d[3];
            d[0] = (xl ? Qt[e + 1] - qxx : 0.f) + (yl ? Qt[2 * NE + e + EXW] - qxy : 0.f);
            d[1] = (yl ? Qt[NE + e + EXW] - qyy : 0.f) + (xl ? Qt[2 * NE + e + 1] - qxy : 0.f);
            d[2] = 0.f;
            float qzz = 0.f, qxz = 0.f, qyz = 0.f;
            if constexpr (THREE) {
                qzz = Qt[3 * NE + e];
                qxz = Qt[4 * NE + e];
                qyz = Qt[5 * NE + e];
                d[0] = d[0] + (has_next ? Qn[4 * NE + e] - qxz : 0.f);
                d[1] = d[1] + (has_next ? Qn[5 * NE + e] - qyz : 0.f);
                d[2] = ((has_next ? Qn[3 * NE + e] - qzz : 0.f) +
                        (xl ? Qt[4 * NE + e + 1] - qxz : 0.f)) +
                       (yl ? Qt[5 * NE + e + EXW] - qyz : 0.f);
            }
            const float vo[3] = {pv0, pv1, pv2};
            if (lt) {
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    const float vn = vo[c] - a.tau * (d[c] - pv[c]);
                    __stcs(a.v_out[c] + i, vn);
                    __stcs(a.vbar_out[c] + i, vn + a.theta * (vn - vo[c]));
                    S::st_cs(a.p_out[c], i, pv[c], a.penc);
                }
                S::st_cs(a.q_out[0], i, qxx, a.qenc);
                S::st_cs(a.q_out[1], i, qyy, a.qenc);
                S::st_cs(a.q_out[3], i, qxy, a.qenc);
                if constexpr (THREE) {
                    S::st_cs(a.q_out[2], i, qzz, a.qenc);
                    S::st_cs(a.q_out[4], i, qxz, a.qenc);
                    S::st_cs(a.q_out[5], i, qyz, a.qenc);
                }
            }
#pragma unroll
            for (int c = 0; c < NC; ++c) p_prev[c] = pv[c];
        }
        // p_new(t+1) goes to the other slot of the p ring (primal(t-1) read it before
        // the last barrier)
        if (in_rp && p_next) {
            Pn[e] = pn.x;
            Pn[NE + e] = pn.y;
            if constexpr (THREE) Pn[2 * NE + e] = pn.z;
        }
        lq0 = lq1;
        lq1 = lq2;
        lq2 = lq3;
        }  // ok
        // The block's one barrier per plane: the rings written above become readable,
        // and the stage of plane t + 1 is no longer read.
        ok = __syncthreads_and(ok);
        if (!ok) break;
        if (tid == PRODUCER) issue(++issued_upto);  // plane t+1 is dead: its slot takes t+1+NS
        slot1 = slot2;
        pslot ^= 1;
        qslot = q1;
    }
    // On an error exit, let every load this block issued land before the block's
    // shared memory goes away (bounded waits; the flag is already raised).
    if (!ok && tid == PRODUCER) {
        for (int pl = max(waited_upto + 1, 0); pl <= min(issued_upto, plast); ++pl) {
            const int j = (pl - pbase) / NS;
            mwait(&full[(pl - pbase) % NS], j & 1, a.err, WAIT_NS);
        }
    }
    __syncthreads();
}

// ---- shifted pass: the primal step of iteration n, then the dual step of n + 1 --------
//
// Between two passes the loop keeps (u^n, v^n, p^(n+1), q^(n+1)): the duals run half an
// iteration ahead of the primals.  One pass computes the primal step of iteration n
// (u, ubar, v, vbar from u^n, v^n, f and the stencils of p^(n+1), q^(n+1)) and then the
// dual step of iteration n + 1 (p^(n+2), q^(n+2) from the stencils of ubar^(n+1),
// vbar^(n+1) and the own p^(n+1), q^(n+1)).  ubar and vbar never leave the chip, so a
// voxel-iteration moves u, v, p, q, f in (14 values) and u, v, p, q out (13): 108 bytes
// in FP32 (72 with p, q in 16 bits), against 140 for the pass that starts with the dual
// step.  Every update is the same arithmetic in the same order as in the other kernels
// (bit-identical results).  A dual step (tgv_dual_kernel) before the first pass and a
// primal step (tgv_primal_kernel) after the last convert the loop state to this form
// and back.
//
// A block owns a 32 x 8 column tile and marches along z through its planes.  Step t
// computes the primal of plane t + 1, then the dual of plane t:
//   256 tile threads   primal (u, ubar, v, vbar; u and v stored) and dual (p, q stored)
//   40 rim threads     ubar only, on the +x column and the +y row the dual's forward
//                      differences read
//   40 rim threads     vbar only, on the -x column and the -y row its backward
//                      differences read
// ubar and vbar pass through a two-plane shared-memory ring: the dual of plane t reads
// plane t's, written one step earlier; the own values of planes t - 1 .. t + 1 stay in
// registers.  p and q of every plane arrive by TMA as boxes of rows y0 - 1 .. y0 + 8
// and columns x0 - 4 .. x0 + 35 (FP32) or x0 - 8 .. x0 + 39 (16-bit) into a ring of NS
// stages, completing on the stage's mbarrier; step t reads planes t .. t + 2, so NS - 3
// planes are in flight while it computes.  u, f and v arrive the same way (40 x 10 FP32
// boxes) into a ring of NU stages of their own (step t reads plane t + 1, so NU - 1
// planes are in flight); no thread loads from global memory.  The block meets one
// barrier per plane.  The masked instance reads each voxel's domain flag per plane:
// outside the domain the primal step passes the frozen ubar = u, vbar = 0 to the ring
// and stores nothing, and the dual step is skipped (p = q = 0 already).
namespace shp {

constexpr int TX = 32, TY = 8;
constexpr int EXW = TX + 2, EYH = TY + 2, NE = EXW * EYH;  // tile and rim: 34 x 10
constexpr int NTHREADS = 352;                              // 8 tile warps, 80 rim threads
constexpr int PRODUCER = 256;                              // first rim thread issues TMA
// FP32 boxes (u, f, v): x0-4 .. x0+35, rows y0-1 .. y0+8
constexpr int XO = 4, BW = TX + 8, BH = TY + 2;
constexpr int BOX = (BW * BH * 4 + 127) / 128 * 128;       // bytes per box in a stage
constexpr int BOXF = BOX / 4;                              // floats per box
constexpr int RING = 2 * 4 * NE;                           // [plane & 1][ubar, vbar x3][NE]
// p, q boxes in the state's dual element type: the same rows, x from a 16-byte boundary
// (x0-4 for FP32, x0-8 for 16-bit elements) to at least x0+32
template <int PREC>
struct PQ {
    static constexpr int DES = PREC == TGVDCT_STATE_FP32 ? 4 : 2;
    static constexpr int XO = DES == 4 ? 4 : 8;
    static constexpr int BW = DES == 4 ? TX + 8 : TX + 16;
    static constexpr int BOX = (BW * BH * DES + 127) / 128 * 128;  // bytes per box
    static constexpr int BOXE = BOX / DES;                          // elements per box
    static constexpr int STAGE = 9 * BOX;                           // p[3] | q[6], slot order
    static constexpr uint32_t TX_BYTES = 9u * BW * BH * DES;        // what expect_tx announces
};
constexpr int NU = 3;                                      // stages of u, f, v
constexpr int USTAGE = 5 * BOX;                            // u | f | v[3], same boxes
constexpr uint32_t UTX_BYTES = 5u * BW * BH * 4;

enum Role { IDLE = 0, TILE = 1, RIM_U = 2, RIM_V = 3 };

struct alignas(64) Maps {
    CUtensorMap p[3], q[6];  // q in kernel slot order: xx yy xy zz xz yz
    CUtensorMap uf[5];       // u, f, v_x, v_y, v_z
};

struct Args {
    Maps maps;
    int W, H, D, zchunk;
    size_t WH;
    const float* f;
    const float* u;  // u^n, v^n of the input
    const float* v[3];
    float* u_out;    // u^(n+1), v^(n+1), p^(n+2), q^(n+2) (distinct from the inputs)
    float* v_out[3];
    void* p_out[3];  // the state's dual element type
    void* q_out[6];  // state order: xx yy zz xy xz yz
    float tau, sigma, theta, tau_lambda, alpha0, alpha1;
    float penc, pdec, qenc, qdec;  // 16-bit fixed-point scales (Dual<FX16>)
    float thr_p, thr_q;  // squared-norm bounds below which the projections are skipped
    int skip_bz;
    int* err;
    unsigned long long wait_ns;  // limit of the consumers' pipeline waits (0: one test)
    const uint8_t* dom;          // masked deshade domain (the MASKED instance only)
    // per-block plane ranges of this grid for that domain (null: whole chunks)
    const uint32_t* tile_active;
};

template <int NS, int PREC>
constexpr size_t smem_bytes() {
    return (size_t)NS * PQ<PREC>::STAGE + (size_t)NU * USTAGE + (size_t)RING * 4 + 128;
}

}  // namespace shp

template <int PREC, int DATA, int NS, bool MASKED>
__device__ __forceinline__ void shifted_pass(const shp::Args& a, uint8_t* stages,
                                             uint8_t* ustages, float* ring, uint64_t* full,
                                             uint64_t* ufull) {
    using namespace shp;
    using tma::su32;
    using DS = Dual<PREC>;
    using T = typename DS::T;
    using G = PQ<PREC>;
    static_assert(NS >= 4, "step t reads three planes; one more must be in flight");
    int z0 = (int)blockIdx.z * a.zchunk, z1 = min(a.D, z0 + a.zchunk);
    if constexpr (MASKED) {
        // Only the planes in which some of the tile's voxels are in the domain have
        // anything to update; none: the block leaves.  A voxel outside the domain keeps
        // u = ubar = f, v = vbar = 0, p = q = 0, in both slots of the shifted form, so
        // the frozen planes need no work.  One entry per block (a uniform branch).
        if (a.tile_active) {
            const uint32_t r = a.tile_active[((size_t)blockIdx.z * gridDim.y + blockIdx.y) *
                                                 gridDim.x + blockIdx.x];
            if (r == 0) return;
            z0 = (int)(r >> 16);
            z1 = (int)(r & 0xffffu);
        }
    }
    const int tid = threadIdx.x;
    int ex = 0, ey = 0, role = IDLE;
    if (tid < 256) {
        ex = (tid & 31) + 1;
        ey = (tid >> 5) + 1;
        role = TILE;
    } else {
        const int h = tid - 256;
        if (h < 32) { ex = h + 1; ey = 0; role = RIM_V; }                 // -y row
        else if (h < 64) { ex = h - 31; ey = EYH - 1; role = RIM_U; }     // +y row
        else if (h < 72) { ex = 0; ey = h - 63; role = RIM_V; }           // -x column
        else if (h < 80) { ex = EXW - 1; ey = h - 71; role = RIM_U; }     // +x column
    }
    const int x0 = (int)blockIdx.x * TX, y0 = (int)blockIdx.y * TY;
    const int x = x0 - 1 + ex, y = y0 - 1 + ey;
    if (!(x >= 0 && x < a.W && y >= 0 && y < a.H)) role = IDLE;
    const bool tile = role == TILE;
    const bool need_u = tile || role == RIM_U, need_v = tile || role == RIM_V;
    const bool xl = x + 1 < a.W, yl = y + 1 < a.H;
    const bool xg = x > 0, yg = y > 0;
    const int e = ey * EXW + ex;            // position in the ubar / vbar ring
    const int ob = ey * BW + ex + XO - 1;        // position in the u, f, v boxes
    const int oq = ey * G::BW + ex + G::XO - 1;  // position in the p and q boxes
    const int D = a.D;
    const int pbase = max(z0 - 1, 0);       // first plane of p, q this block loads
    const int plast = min(D - 1, z1);       // last one
    const int qlast = min(D - 1, z1);       // last plane of a primal step here
    // 32-bit voxel indices: the host runs this kernel only on volumes of < 2^32 voxels
    const uint32_t wh = (uint32_t)a.WH;
    const uint32_t col = role != IDLE ? (uint32_t)y * (uint32_t)a.W + (uint32_t)x : 0u;
    // whether this thread's voxel of plane z is in the masked deshade's domain
    auto live = [&](int z) {
        if constexpr (MASKED) return a.dom[(uint32_t)z * wh + col] != 0;
        else return true;
    };
    if constexpr (kCheckBounds) {
        // every index this thread's role uses: its column over the chunk, the staged
        // boxes with the neighbours the primal reads, and the ring
        constexpr int nB = BW * BH, nQ = G::BW * BH;
        bool ok = true;
        if (role != IDLE) {
            ok = TGV_IN_BOUNDS(col, a.WH, 40) && ok;
            ok = TGV_IN_BOUNDS((size_t)qlast * a.WH + col, a.WH * (size_t)D, 41) && ok;
            ok = TGV_IN_BOUNDS(ob, nB, 42) && ok;
            ok = TGV_IN_BOUNDS(oq, nQ, 52) && ok;
            ok = TGV_IN_BOUNDS(e, NE, 43) && ok;
        }
        if (need_u) {
            if (xg) ok = TGV_IN_BOUNDS(oq - 1, nQ, 44) && ok;
            if (yg) ok = TGV_IN_BOUNDS(oq - G::BW, nQ, 45) && ok;
        }
        if (need_v) {
            if (xl) ok = TGV_IN_BOUNDS(oq + 1, nQ, 46) && ok;
            if (yl) ok = TGV_IN_BOUNDS(oq + G::BW, nQ, 47) && ok;
        }
        if (tile) {
            if (xl) ok = TGV_IN_BOUNDS(e + 1, NE, 48) && ok;
            if (yl) ok = TGV_IN_BOUNDS(e + EXW, NE, 49) && ok;
            if (xg) ok = TGV_IN_BOUNDS(e - 1, NE, 50) && ok;
            if (yg) ok = TGV_IN_BOUNDS(e - EXW, NE, 51) && ok;
        }
        if (__syncthreads_or(!ok)) return;
    }
    auto stage_at = [&](int plane) {
        return (const T*)(stages + ((plane - pbase) % NS) * G::STAGE);
    };
    // p component c and q slot k of a stage at a box position, decoded to float
    auto pval = [&](const T* st, int c, int off) { return DS::ld(st, c * G::BOXE + off, a.pdec); };
    auto qval = [&](const T* st, int k, int off) {
        return DS::ld(st, (3 + k) * G::BOXE + off, a.qdec);
    };
    auto issue = [&](int plane) {  // producer thread only
        if (plane < 0 || plane > plast) return;
        const int slot = (plane - pbase) % NS;
        uint8_t* st = stages + slot * G::STAGE;
        uint64_t* bar = &full[slot];
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)),
                     "r"(G::TX_BYTES)
                     : "memory");
        const int xb = x0 - G::XO, yb = y0 - 1;
        for (int c = 0; c < 3; ++c)
            tma::tma_load(st + c * G::BOX, &a.maps.p[c], xb, yb, plane, bar);
        for (int k = 0; k < 6; ++k)
            tma::tma_load(st + (3 + k) * G::BOX, &a.maps.q[k], xb, yb, plane, bar);
    };
    bool ok = true;
    int waited_upto = pbase - 1;  // every plane <= this one has landed
    auto wait_plane = [&](int plane) {
        if (plane < 0 || plane > plast || plane <= waited_upto) return;
        const int j = (plane - pbase) / NS;
        if (!tma::mwait(&full[(plane - pbase) % NS], j & 1, a.err, a.wait_ns)) ok = false;
        else waited_upto = plane;
    };

    // u, f, v of the primal planes qfirst .. qlast: a ring of NU stages of their own
    const int qfirst = z0 > 0 ? z0 - 1 : z0;
    auto issue_u = [&](int plane) {  // producer thread only
        if (plane < qfirst || plane > qlast) return;
        const int slot = (plane - qfirst) % NU;
        uint8_t* st = ustages + slot * USTAGE;
        uint64_t* bar = &ufull[slot];
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)),
                     "r"(UTX_BYTES)
                     : "memory");
        for (int k = 0; k < 5; ++k)
            tma::tma_load(st + k * BOX, &a.maps.uf[k], x0 - XO, y0 - 1, plane, bar);
    };
    int uwaited_upto = qfirst - 1;
    auto wait_u = [&](int plane) {
        if (plane < qfirst || plane > qlast || plane <= uwaited_upto) return;
        const int j = (plane - qfirst) / NU;
        if (!tma::mwait(&ufull[(plane - qfirst) % NU], j & 1, a.err, a.wait_ns)) ok = false;
        else uwaited_upto = plane;
    };
    auto ustage_at = [&](int plane) {
        return (const float*)(ustages + ((plane - qfirst) % NU) * USTAGE);
    };

    // ---- the primal step of this thread's role at plane z (stage S; Sn: plane z + 1,
    // read when has_next).  pzm: p_z of plane z - 1 here (0 under the volume).  full:
    // the plane is one of the block's (u and v stored); otherwise only the tile's own
    // ubar is wanted (the dual of the block's last plane reads it).
    float pzm = 0.f;
    auto primal_at = [&](const T* S, const T* Sn, bool has_next, float* R,
                         const float* Us, uint32_t i, bool full, float& ub_out,
                         float* vb_out, bool lv) {
        const float pv[3] = {pval(S, 0, oq), pval(S, 1, oq), pval(S, 2, oq)};
        if (!lv) {  // frozen: ubar = u, vbar = 0 (p = 0 here), nothing stored
            const float ub = Us[ob];
            ub_out = ub;
            if (full) {
                if (need_u) R[e] = ub;
                if (need_v)
                    for (int c = 0; c < 3; ++c) R[(1 + c) * NE + e] = 0.f;
            }
            pzm = pv[2];
            return;
        }
        if (need_u) {
            // u <- prox(u - tau B.p), ubar                (tgv2_l1.cu:39-52)
            const float pu = Us[ob], pf = Us[BOXF + ob];
            const float bx = (xg ? pval(S, 0, oq - 1) : 0.f) - pv[0];
            const float by = (yg ? pval(S, 1, oq - G::BW) : 0.f) - pv[1];
            float div = bx + by;
            const float bz = pzm - pv[2];
            if (!a.skip_bz) div = div + bz;
            float uu = pu - a.tau * div;
            if constexpr (DATA == TGVDCT_DATA_L1) {
                const float umf = uu - pf;
                if (umf > a.tau_lambda) uu = uu - a.tau_lambda;
                else if (umf < -a.tau_lambda) uu = uu + a.tau_lambda;
                else uu = pf;
            } else {
                uu = (uu + a.tau_lambda * pf) / (1.f + a.tau_lambda);
            }
            const float ub = uu + a.theta * (uu - pu);
            ub_out = ub;
            if (full) {
                R[e] = ub;
                if (tile) __stcs(a.u_out + i, uu);
            }
        }
        if (need_v && full) {
            // v <- v - tau (div q - p), vbar               (tgv2_common.cu:290-347)
            const float qxx = qval(S, 0, oq), qyy = qval(S, 1, oq), qxy = qval(S, 2, oq);
            const float qzz = qval(S, 3, oq), qxz = qval(S, 4, oq), qyz = qval(S, 5, oq);
            float d[3];
            d[0] = (xl ? qval(S, 0, oq + 1) - qxx : 0.f) + (yl ? qval(S, 2, oq + G::BW) - qxy : 0.f);
            d[1] = (yl ? qval(S, 1, oq + G::BW) - qyy : 0.f) + (xl ? qval(S, 2, oq + 1) - qxy : 0.f);
            d[0] = d[0] + (has_next ? qval(Sn, 4, oq) - qxz : 0.f);
            d[1] = d[1] + (has_next ? qval(Sn, 5, oq) - qyz : 0.f);
            d[2] = ((has_next ? qval(Sn, 3, oq) - qzz : 0.f) +
                    (xl ? qval(S, 4, oq + 1) - qxz : 0.f)) +
                   (yl ? qval(S, 5, oq + G::BW) - qyz : 0.f);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float vo = Us[(2 + c) * BOXF + ob];
                const float vn = vo - a.tau * (d[c] - pv[c]);
                const float vb = vn + a.theta * (vn - vo);
                R[(1 + c) * NE + e] = vb;
                vb_out[c] = vb;
                if (tile) __stcs(a.v_out[c] + i, vn);
            }
        }
        pzm = pv[2];
    };
    // ---- the dual step at plane t (stage S, ring slot R of plane t), tile threads:
    // ubar own of planes t, t + 1 and vbar own of planes t - 1, t from registers, the
    // neighbours from the ring
    auto dual_at = [&](const T* S, const float* R, float ubc, float ubn, bool has_next,
                       const float* vbc, const float* vbm, bool has_prev, uint32_t i, bool lv) {
        if (!lv) return;  // p = q = 0 already, in both slots
        float g[3] = {xl ? R[e + 1] - ubc : 0.f, yl ? R[e + EXW] - ubc : 0.f,
                      has_next ? ubn - ubc : 0.f};
        float vb[3] = {vbc[0], vbc[1], vbc[2]};
        float pp[3] = {pval(S, 0, oq), pval(S, 1, oq), pval(S, 2, oq)};
        dual_p_update<true>(g, vb, pp, a.sigma, a.alpha1, a.thr_p);
        float xm[3], ym[3], zm[3], q[6];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float* V = R + (1 + c) * NE;
            xm[c] = xg ? V[e - 1] : 0.f;
            ym[c] = yg ? V[e - EXW] : 0.f;
            zm[c] = has_prev ? vbm[c] : 0.f;
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) q[k] = qval(S, k, oq);
        dual_q_update<true>(vb, xm, ym, zm, q, a.sigma, a.alpha0, a.thr_q);
#pragma unroll
        for (int c = 0; c < 3; ++c) DS::st_cs((T*)a.p_out[c], i, pp[c], a.penc);
        const int qmap[6] = {0, 1, 3, 2, 4, 5};  // slot -> state order
#pragma unroll
        for (int k = 0; k < 6; ++k) DS::st_cs((T*)a.q_out[qmap[k]], i, q[k], a.qenc);
    };

    if (tid == 0) {
        for (int k = 0; k < NS; ++k)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&full[k])) : "memory");
        for (int k = 0; k < NU; ++k)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&ufull[k])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == PRODUCER) {
        for (int k = 0; k < NS; ++k) issue(pbase + k);
        for (int k = 0; k < NU; ++k) issue_u(qfirst + k);
    }
    int issued_upto = pbase + NS - 1;    // meaningful in the producer only
    int uissued_upto = qfirst + NU - 1;  // likewise

    // ---- prologue: vbar own at plane z0 - 1 (tile), the primal of plane z0 (all roles)
    wait_plane(z0 - 1);
    wait_plane(z0);
    wait_plane(z0 + 1);
    wait_u(z0 - 1);
    wait_u(z0);
    float ubc = 0.f, vbc[3] = {0.f, 0.f, 0.f}, vbm[3] = {0.f, 0.f, 0.f};
    if (ok) {
        if (z0 > 0) {
            const T* S = stage_at(z0 - 1);
            if (tile && live(z0 - 1)) {
                const float* Us = ustage_at(z0 - 1);
                const T* Sn = stage_at(z0);
                const float pv[3] = {pval(S, 0, oq), pval(S, 1, oq), pval(S, 2, oq)};
                const float qxx = qval(S, 0, oq), qyy = qval(S, 1, oq), qxy = qval(S, 2, oq);
                const float qzz = qval(S, 3, oq), qxz = qval(S, 4, oq), qyz = qval(S, 5, oq);
                float d[3];
                d[0] = (xl ? qval(S, 0, oq + 1) - qxx : 0.f) +
                       (yl ? qval(S, 2, oq + G::BW) - qxy : 0.f);
                d[1] = (yl ? qval(S, 1, oq + G::BW) - qyy : 0.f) +
                       (xl ? qval(S, 2, oq + 1) - qxy : 0.f);
                d[0] = d[0] + (qval(Sn, 4, oq) - qxz);
                d[1] = d[1] + (qval(Sn, 5, oq) - qyz);
                d[2] = ((qval(Sn, 3, oq) - qzz) + (xl ? qval(S, 4, oq + 1) - qxz : 0.f)) +
                       (yl ? qval(S, 5, oq + G::BW) - qyz : 0.f);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float vo = Us[(2 + c) * BOXF + ob];
                    const float vn = vo - a.tau * (d[c] - pv[c]);
                    vbm[c] = vn + a.theta * (vn - vo);
                }
            }
            if (role != IDLE) pzm = pval(S, 2, oq);
        }
        const bool hn = z0 + 1 < D;
        const T* S = stage_at(z0);
        if (role != IDLE)
            primal_at(S, hn ? stage_at(z0 + 1) : S, hn, ring + (z0 & 1) * 4 * NE, ustage_at(z0),
                      (uint32_t)z0 * wh + col, true, ubc, vbc, live(z0));
    }
    ok = __syncthreads_and(ok);
    if (ok && tid == PRODUCER) {  // planes z0 - 1 (if any) and z0 are done
        if (z0 > 0) {
            issue(++issued_upto);
            issue_u(++uissued_upto);
        }
        issue_u(++uissued_upto);
    }

    int s0 = (z0 - pbase) % NS;        // stage slot of plane t
    int us = (z0 + 1 - qfirst) % NU;   // u stage slot of plane t + 1
    for (int t = z0; t < z1 && ok; ++t) {
        wait_plane(min(t + 2, plast));
        wait_u(t + 1);
        const int s1 = s0 + 1 == NS ? 0 : s0 + 1;
        const int s2 = s1 + 1 == NS ? 0 : s1 + 1;
        const T* St = (const T*)(stages + s0 * G::STAGE);  // plane t
        const T* S1 = (const T*)(stages + s1 * G::STAGE);  // plane t + 1
        const T* S2 = (const T*)(stages + s2 * G::STAGE);  // plane t + 2
        // A thread whose wait gave up skips the plane; the barrier below shares the
        // outcome and the whole block leaves together.
        if (ok) {
            float ubn = 0.f, vbn[3] = {0.f, 0.f, 0.f};
            const bool p1 = t + 1 < D;  // there is a plane t + 1
            if (p1) {
                const bool full = t + 1 < z1;
                const bool hn = t + 2 < D;
                if (role != IDLE && (full || tile))
                    primal_at(S1, hn ? S2 : S1, hn, ring + ((t + 1) & 1) * 4 * NE,
                              (const float*)(ustages + us * USTAGE),
                              (uint32_t)(t + 1) * wh + col, full, ubn, vbn, live(t + 1));
                if constexpr (MASKED) {  // the flags two planes ahead into L2
                    if (role != IDLE && t + 3 <= qlast) {
                        const uint8_t* fl = a.dom + (uint32_t)(t + 3) * wh + col;
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(fl));
                    }
                }
            }
            if (tile)
                dual_at(St, ring + (t & 1) * 4 * NE, ubc, ubn, p1, vbc, vbm, t > 0,
                        (uint32_t)t * wh + col, live(t));
            ubc = ubn;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                vbm[c] = vbc[c];
                vbc[c] = vbn[c];
            }
        }
        // The block's one barrier per plane: the ring slot written above becomes
        // readable, and the stage of plane t is no longer read.
        ok = __syncthreads_and(ok);
        if (!ok) break;
        if (tid == PRODUCER) {
            issue(++issued_upto);                  // plane t's slot takes t + NS
            if (t + 1 < D) issue_u(++uissued_upto);  // plane t + 1's, t + 1 + NU
        }
        s0 = s1;
        us = us + 1 == NU ? 0 : us + 1;
    }
    // On an error exit, let every load this block issued land before the block's
    // shared memory goes away (bounded waits; the flag is already raised).
    if (!ok && tid == PRODUCER) {
        for (int pl = max(waited_upto + 1, 0); pl <= min(issued_upto, plast); ++pl) {
            const int j = (pl - pbase) / NS;
            tma::mwait(&full[(pl - pbase) % NS], j & 1, a.err, tma::WAIT_NS);
        }
        for (int pl = uwaited_upto + 1; pl <= min(uissued_upto, qlast); ++pl) {
            const int j = (pl - qfirst) / NU;
            tma::mwait(&ufull[(pl - qfirst) % NU], j & 1, a.err, tma::WAIT_NS);
        }
    }
    __syncthreads();
}

template <int PREC, int DATA, int NS, bool MASKED>
__global__ void __launch_bounds__(shp::NTHREADS, 2)
    tgv_shifted_tma_kernel(const __grid_constant__ shp::Args a) {
    extern __shared__ __align__(128) uint8_t smem_raw[];
    uint8_t* smem = align_shared<128>(smem_raw);
    __shared__ uint64_t full[NS + shp::NU];
    // a pipeline wait of an earlier block or launch timed out: do nothing more
    if (__syncthreads_or(threadIdx.x == 0 ? *(volatile int*)a.err : 0)) return;
    uint8_t* ustages = smem + NS * shp::PQ<PREC>::STAGE;
    float* ring = (float*)(ustages + shp::NU * shp::USTAGE);
    shifted_pass<PREC, DATA, NS, MASKED>(a, smem, ustages, ring, full, full + NS);
}

size_t elem_bytes(int precision) { return precision == TGVDCT_STATE_FP32 ? 4 : 2; }
size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

template <int PREC>
TgvArgs<typename Dual<PREC>::T> make_args(const TgvState& s, const TgvStep& k,
                                          const TgvStencilFields& I, const float* u_in,
                                          float* const* v_in, const TgvStencilFields& O,
                                          float* u_out, float* const* v_out) {
    using T = typename Dual<PREC>::T;
    TgvArgs<T> a;
    a.W = s.W;
    a.H = s.H;
    a.D = s.D;
    a.WH = (size_t)s.W * s.H;
    a.f = s.f;
    a.u_in = u_in;
    a.u = u_out;
    a.ubar = I.ubar;
    a.ubar_out = O.ubar;
    for (int c = 0; c < 3; ++c) {
        a.v_in[c] = v_in[c];
        a.vbo[c] = O.vbar[c];
        a.pin[c] = (const T*)I.p[c];
    }
    for (int c = 0; c < 6; ++c) a.qin[c] = (const T*)I.q[c];
    a.v0 = v_out[0];
    a.v1 = v_out[1];
    a.v2 = v_out[2];
    a.vb0 = I.vbar[0];
    a.vb1 = I.vbar[1];
    a.vb2 = I.vbar[2];
    a.p0 = (T*)O.p[0];
    a.p1 = (T*)O.p[1];
    a.p2 = (T*)O.p[2];
    a.qxx = (T*)O.q[0];
    a.qyy = (T*)O.q[1];
    a.qzz = (T*)O.q[2];
    a.qxy = (T*)O.q[3];
    a.qxz = (T*)O.q[4];
    a.qyz = (T*)O.q[5];
    a.tau = k.tau;
    a.sigma = k.sigma;
    a.theta = k.theta;
    a.tau_lambda = k.tau * k.lambda;
    a.alpha0 = k.alpha0;
    a.alpha1 = k.alpha1;
    a.penc = 32767.f / k.alpha1;
    a.pdec = k.alpha1 / 32767.f;
    a.qenc = 32767.f / k.alpha0;
    a.qdec = k.alpha0 / 32767.f;
    a.skip_bz = (k.data_term == TGVDCT_DATA_L2 && s.D == 1) ? 1 : 0;
    a.dom = s.domain;
    return a;
}

template <int PREC>
void launch_two_pass(const TgvState& s, const TgvStep& k,
                     const TgvArgs<typename Dual<PREC>::T>& a, cudaStream_t st) {
    const dim3 block(BX, BY, 1);
    const dim3 grid(ceil_div(s.W, BX), ceil_div(s.H, BY), s.D);
    if (s.three) {
        tgv_dual_kernel<PREC, true><<<grid, block, 0, st>>>(a);
        if (k.data_term == TGVDCT_DATA_L1)
            tgv_primal_kernel<PREC, true, TGVDCT_DATA_L1><<<grid, block, 0, st>>>(a);
        else
            tgv_primal_kernel<PREC, true, TGVDCT_DATA_L2><<<grid, block, 0, st>>>(a);
    } else {
        tgv_dual_kernel<PREC, false><<<grid, block, 0, st>>>(a);
        if (k.data_term == TGVDCT_DATA_L1)
            tgv_primal_kernel<PREC, false, TGVDCT_DATA_L1><<<grid, block, 0, st>>>(a);
        else
            tgv_primal_kernel<PREC, false, TGVDCT_DATA_L2><<<grid, block, 0, st>>>(a);
    }
    TGV_CHECK_LAUNCH();
}

template <int PREC>
void iterate_two_pass(const TgvState& s, const TgvStep& k, cudaStream_t st) {
    const TgvStencilFields& F = s.now();  // in place on the current set
    float* const v[3] = {s.v[0], s.v[1], s.v[2]};
    const auto a = make_args<PREC>(s, k, F, s.u, v, F, s.u, v);
    launch_two_pass<PREC>(s, k, a, st);
}

constexpr int FUSED_TY = 8;

template <int PREC, bool THREE, int DATA>
void launch_fused(const FusedArgs<typename Dual<PREC>::T>& a, int D, cudaStream_t st) {
    constexpr int TY = FUSED_TY;
    constexpr size_t smem = fused_smem_floats<TY, THREE>() * sizeof(float);
    auto kern = tgv_fused_kernel<PREC, THREE, DATA, TY>;
    static std::atomic<uint64_t> configured{0};  // per template instance
    smem_attr_once((const void*)kern, smem, configured);
    const dim3 grid(ceil_div(a.W, FX), ceil_div(a.H, TY), ceil_div(D, a.zchunk));
    kern<<<grid, fused_threads<TY>(), smem, st>>>(a);
    TGV_CHECK_LAUNCH();
}


// ---- TMA launch plumbing -----------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
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

void encode_box(CUtensorMap* m, const void* base, int es, const TgvState& s, int bw, int bh) {
    const cuuint64_t dims[3] = {(cuuint64_t)s.W, (cuuint64_t)s.H, (cuuint64_t)s.D};
    const cuuint64_t strides[2] = {(cuuint64_t)s.W * es, (cuuint64_t)s.W * s.H * es};
    const cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)bh, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUtensorMapDataType dt =
        es == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16;
    const CUresult r = tensor_map_encoder()(m, dt, 3, const_cast<void*>(base), dims, strides, box,
                                            estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                            CU_TENSOR_MAP_SWIZZLE_NONE,
                                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    TGV_REQUIRE(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled rejected a state field");
}

// TMA needs 16-byte row and plane strides: width a multiple of 4 (FP32 fields) and
// of 8 (16-bit dual fields).
bool tma_shape_ok(const TgvState& s) {
    const int need = s.precision == TGVDCT_STATE_FP32 ? 4 : 8;
    // (and 32-bit voxel indices)
    return s.W % need == 0 && (s.kernel == TGV_KERNEL_FUSED || s.kernel == TGV_KERNEL_SHIFTED) &&
           (uint64_t)s.W * s.H * s.D < (1ull << 32);
}

template <int PREC>
struct TmaCache {
    tma::Args<typename Dual<PREC>::T> args[2];  // [cur]: reads set cur, writes set cur ^ 1
};

template <int PREC>
constexpr int tma_stages() {
    return PREC == TGVDCT_STATE_FP32 ? 4 : 5;
}

template <int PREC>
size_t tma_smem_bytes() {
    // stages + the p_new ring (2 x 3 fields) and the q_new ring (3 x 6 fields)
    return (size_t)tma_stages<PREC>() * tma::Geo<PREC>::STAGE + 24 * tma::NE * 4 + 128;
}

// Tensor maps of the input stencil set I and the pointers of one iteration
// (u, v, I) -> (u_out, v_out, O).
template <class T, int PREC>
void fill_tma_args(tma::Args<T>& a, const TgvState& s, const TgvStencilFields& I,
                   const float* u, const float* const* v, const TgvStencilFields& O,
                   float* u_out, float* const* v_out) {
    using G = tma::Geo<PREC>;
    std::memset(&a, 0, sizeof(a));
    const int NC = s.three ? 3 : 2, NQ = s.three ? 6 : 3;
    const int qmap[6] = {0, 1, 3, 2, 4, 5};  // kernel slot -> state order
    encode_box(&a.maps.ub, I.ubar, 4, s, G::BW_F, tma::EYH);
    for (int c2 = 0; c2 < NC; ++c2) {
        encode_box(&a.maps.vb[c2], I.vbar[c2], 4, s, G::BW_F, tma::EYH);
        encode_box(&a.maps.p[c2], I.p[c2], G::DES, s, G::BW_P, G::PQ_ROWS);
    }
    for (int k = 0; k < NQ; ++k)
        encode_box(&a.maps.q[k], I.q[qmap[k]], G::DES, s, G::BW_Q, G::PQ_ROWS);
    a.f = s.f;
    a.W = s.W;
    a.H = s.H;
    a.D = s.D;
    a.WH = (size_t)s.W * s.H;
    a.u = u;
    a.u_out = u_out;
    a.ubar_out = O.ubar;
    for (int c2 = 0; c2 < 3; ++c2) {
        a.v[c2] = v[c2];
        a.v_out[c2] = v_out[c2];
        a.vbar_out[c2] = O.vbar[c2];
        a.p_out[c2] = (T*)O.p[c2];
    }
    for (int k = 0; k < 6; ++k) a.q_out[k] = (T*)O.q[k];
}

template <int PREC>
TmaCache<PREC>* tma_cache(TgvState& s) {
    if (!s.tma_cache) {
        using T = typename Dual<PREC>::T;
        auto c = std::make_shared<TmaCache<PREC>>();
        for (int cur = 0; cur < 2; ++cur)
            fill_tma_args<T, PREC>(c->args[cur], s, s.set[cur], s.u, s.v, s.set[cur ^ 1], s.u,
                                   s.v);
        s.tma_cache = c;
    }
    return (TmaCache<PREC>*)s.tma_cache.get();
}

template <int PREC, bool THREE, int DATA>
void launch_tma(const tma::Args<typename Dual<PREC>::T>& a, cudaStream_t st) {
    constexpr int NS = tma_stages<PREC>();
    // the domain test is compiled only into the masked instances
    auto kern = a.dom ? tgv_fused_tma_kernel<PREC, THREE, DATA, NS, true>
                      : tgv_fused_tma_kernel<PREC, THREE, DATA, NS, false>;
    const size_t smem = tma_smem_bytes<PREC>();
    static std::atomic<uint64_t> configured[2] = {};
    smem_attr_once((const void*)kern, smem, configured[a.dom ? 1 : 0]);
    const dim3 grid(ceil_div(a.W, tma::TX), ceil_div(a.H, tma::TY), ceil_div(a.D, a.zchunk));
    kern<<<grid, tma::NTHREADS, smem, st>>>(a);
    TGV_CHECK_LAUNCH();
}

// planes per block of the fused TMA kernel's grid
int tma_zchunk(const TgvState& s) { return s.three ? (s.zchunk > 0 ? s.zchunk : s.D) : 1; }

// alpha^2 (1 - 2^-19), or -1 (never skip) where alpha^2 would leave the normal range
float projection_skip_bound(float alpha) {
    const double a2 = (double)alpha * alpha;
    if (!(a2 > 1e-30 && a2 < 1e30)) return -1.f;
    return (float)(a2 * (1.0 - 1.0 / (1 << 19)));
}

template <int PREC, class T>
void launch_tma_step(tma::Args<T> a, const TgvState& s, const TgvStep& k, int* err,
                     cudaStream_t st) {
    a.zchunk = tma_zchunk(s);
    a.tau = k.tau;
    a.sigma = k.sigma;
    a.theta = k.theta;
    a.tau_lambda = k.tau * k.lambda;
    a.alpha0 = k.alpha0;
    a.alpha1 = k.alpha1;
    a.penc = 32767.f / k.alpha1;
    a.pdec = k.alpha1 / 32767.f;
    a.qenc = 32767.f / k.alpha0;
    a.qdec = k.alpha0 / 32767.f;
    a.thr_p = projection_skip_bound(k.alpha1);
    a.thr_q = projection_skip_bound(k.alpha0);
    a.skip_bz = (k.data_term == TGVDCT_DATA_L2 && s.D == 1) ? 1 : 0;
    a.err = err;
    a.wait_ns = s.wait_ns;
    a.dom = s.domain;
    a.tile_active =
        (s.domain && s.tile_active && s.tile_zchunk == a.zchunk) ? s.tile_active : nullptr;
    if (s.three) {
        if (k.data_term == TGVDCT_DATA_L1) launch_tma<PREC, true, TGVDCT_DATA_L1>(a, st);
        else launch_tma<PREC, true, TGVDCT_DATA_L2>(a, st);
    } else {
        if (k.data_term == TGVDCT_DATA_L1) launch_tma<PREC, false, TGVDCT_DATA_L1>(a, st);
        else launch_tma<PREC, false, TGVDCT_DATA_L2>(a, st);
    }
}

template <int PREC>
void iterate_tma(TgvState& s, const TgvStep& k, int* err, cudaStream_t st) {
    launch_tma_step<PREC>(tma_cache<PREC>(s)->args[s.cur], s, k, err, st);
    s.cur ^= 1;
}

template <int PREC>
void iterate_fused(TgvState& s, const TgvStep& k, cudaStream_t st) {
    using T = typename Dual<PREC>::T;
    const TgvStencilFields& I = s.set[s.cur];
    const TgvStencilFields& O = s.set[s.cur ^ 1];
    FusedArgs<T> a;
    a.W = s.W;
    a.H = s.H;
    a.D = s.D;
    a.zchunk = s.three ? (s.zchunk > 0 ? s.zchunk : s.D) : 1;
    a.WH = (size_t)s.W * s.H;
    a.f = s.f;
    a.u = s.u;
    a.ubar_in = I.ubar;
    a.ubar_out = O.ubar;
    for (int c = 0; c < 3; ++c) {
        a.v[c] = s.v[c];
        a.vbar_in[c] = I.vbar[c];
        a.vbar_out[c] = O.vbar[c];
        a.p_in[c] = (const T*)I.p[c];
        a.p_out[c] = (T*)O.p[c];
    }
    for (int c = 0; c < 6; ++c) {
        a.q_in[c] = (const T*)I.q[c];
        a.q_out[c] = (T*)O.q[c];
    }
    a.tau = k.tau;
    a.sigma = k.sigma;
    a.theta = k.theta;
    a.tau_lambda = k.tau * k.lambda;
    a.alpha0 = k.alpha0;
    a.alpha1 = k.alpha1;
    a.penc = 32767.f / k.alpha1;
    a.pdec = k.alpha1 / 32767.f;
    a.qenc = 32767.f / k.alpha0;
    a.qdec = k.alpha0 / 32767.f;
    a.skip_bz = (k.data_term == TGVDCT_DATA_L2 && s.D == 1) ? 1 : 0;
    if (s.three) {
        if (k.data_term == TGVDCT_DATA_L1) launch_fused<PREC, true, TGVDCT_DATA_L1>(a, s.D, st);
        else launch_fused<PREC, true, TGVDCT_DATA_L2>(a, s.D, st);
    } else {
        if (k.data_term == TGVDCT_DATA_L1) launch_fused<PREC, false, TGVDCT_DATA_L1>(a, s.D, st);
        else launch_fused<PREC, false, TGVDCT_DATA_L2>(a, s.D, st);
    }
    s.cur ^= 1;
}

// ---- the shifted passes: host side ----------------------------------------------------
// Stages of p and q in flight: step t reads planes t .. t + 2, so SHIFTED_NS - 3 planes
// land while it computes.
// Stages of p and q in flight: step t reads planes t .. t + 2, so shifted_stages() - 3
// planes land while it computes (two CTAs per SM: 110.8 KB of shared memory in FP32,
// 91.0 KB with 16-bit duals).
template <int PREC>
constexpr int shifted_stages() {
    return PREC == TGVDCT_STATE_FP32 ? 5 : 6;
}

bool shifted_ok(const TgvState& s) {
    const int need = s.precision == TGVDCT_STATE_FP32 ? 4 : 8;  // 16-byte TMA strides
    return s.kernel == TGV_KERNEL_SHIFTED && s.three && s.D >= 2 && s.W % need == 0 && s.err &&
           (uint64_t)s.W * s.H * s.D < (1ull << 32);  // 32-bit voxel indices
}

// Where the shifted form (u^n, v^n, p^(n+1), q^(n+1)) of a run that started from stencil
// set c lives after an even or odd number of passes.  Even: u, v in their own buffers,
// p, q in set c ^ 1 (the dual step before the first pass writes there).  Odd: u, v in
// set c's ubar and vbar (dead while the duals run ahead), p, q in set c.  A pass reads
// one and writes the other, so no block overwrites what another still reads.
struct ShiftedSlot {
    float* u;
    float* v[3];
    void* p[3];  // the state's dual element type
    void* q[6];  // state order
};

ShiftedSlot shifted_slot(const TgvState& s, int c, int parity) {
    ShiftedSlot r;
    const TgvStencilFields& F = s.set[parity ? c : c ^ 1];
    r.u = parity ? s.set[c].ubar : s.u;
    for (int k = 0; k < 3; ++k) {
        r.v[k] = parity ? s.set[c].vbar[k] : s.v[k];
        r.p[k] = F.p[k];
    }
    for (int k = 0; k < 6; ++k) r.q[k] = F.q[k];
    return r;
}

struct ShiftedCache {
    shp::Args args[2][2];  // [c][parity of the input]: tensor maps and pointers of a pass
};

template <int PREC>
ShiftedCache* shifted_cache(TgvState& s) {
    if (!s.shifted_cache) {
        using G = shp::PQ<PREC>;
        auto cache = std::make_shared<ShiftedCache>();
        const int qmap[6] = {0, 1, 3, 2, 4, 5};  // kernel slot -> state order
        for (int c = 0; c < 2; ++c)
            for (int par = 0; par < 2; ++par) {
                shp::Args& a = cache->args[c][par];
                std::memset(&a, 0, sizeof(a));
                const ShiftedSlot in = shifted_slot(s, c, par), out = shifted_slot(s, c, par ^ 1);
                for (int k = 0; k < 3; ++k)
                    encode_box(&a.maps.p[k], in.p[k], G::DES, s, G::BW, shp::BH);
                for (int k = 0; k < 6; ++k)
                    encode_box(&a.maps.q[k], in.q[qmap[k]], G::DES, s, G::BW, shp::BH);
                const float* uf[5] = {in.u, s.f, in.v[0], in.v[1], in.v[2]};
                for (int k = 0; k < 5; ++k)
                    encode_box(&a.maps.uf[k], uf[k], 4, s, shp::BW, shp::BH);
                a.W = s.W;
                a.H = s.H;
                a.D = s.D;
                a.WH = (size_t)s.W * s.H;
                a.f = s.f;
                a.u = in.u;
                a.u_out = out.u;
                for (int k = 0; k < 3; ++k) {
                    a.v[k] = in.v[k];
                    a.v_out[k] = out.v[k];
                    a.p_out[k] = out.p[k];
                }
                for (int k = 0; k < 6; ++k) a.q_out[k] = out.q[k];
            }
        s.shifted_cache = cache;
    }
    return (ShiftedCache*)s.shifted_cache.get();
}

// Raises the shared-memory limit of the shifted kernel on the current device, once.
template <int PREC, int DATA, bool MASKED>
void shifted_attr() {
    constexpr int NS = shifted_stages<PREC>();
    static std::atomic<uint64_t> configured{0};  // per template instance
    smem_attr_once((const void*)tgv_shifted_tma_kernel<PREC, DATA, NS, MASKED>,
                   shp::smem_bytes<NS, PREC>(), configured);
}

template <int PREC, int DATA, bool MASKED>
void launch_shifted(const shp::Args& a, cudaStream_t st) {
    constexpr int NS = shifted_stages<PREC>();
    auto kern = tgv_shifted_tma_kernel<PREC, DATA, NS, MASKED>;
    constexpr size_t smem = shp::smem_bytes<NS, PREC>();
    static_assert(smem <= 113 * 1024, "two CTAs per SM");
    shifted_attr<PREC, DATA, MASKED>();
    const dim3 grid(ceil_div(a.W, shp::TX), ceil_div(a.H, shp::TY), ceil_div(a.D, a.zchunk));
    kern<<<grid, shp::NTHREADS, smem, st>>>(a);
    TGV_CHECK_LAUNCH();
}

// n >= 2 iterations from the standard state of set c = s.cur: the dual step of the
// first, n - 1 shifted passes, the primal step of the last.  The standard state ends in
// set c when n is even and in set c ^ 1 when n is odd (as after n single passes).
// Returns the number of kernel launches.
template <int PREC>
int iterate_shifted(TgvState& s, const TgvStep& k, uint32_t n, cudaStream_t st) {
    const int c = s.cur;
    ShiftedCache* cache = shifted_cache<PREC>(s);
    const dim3 block(BX, BY, 1);
    const dim3 grid(ceil_div(s.W, BX), ceil_div(s.H, BY), s.D);
    {   // p^(n+1), q^(n+1) of the current state into set c ^ 1
        float* const v[3] = {s.v[0], s.v[1], s.v[2]};
        const auto a = make_args<PREC>(s, k, s.set[c], s.u, v, s.set[c ^ 1], s.u, v);
        tgv_dual_kernel<PREC, true><<<grid, block, 0, st>>>(a);
        TGV_CHECK_LAUNCH();
    }
    for (uint32_t j = 0; j + 1 < n; ++j) {
        shp::Args a = cache->args[c][j & 1];
        a.zchunk = tma_zchunk(s);
        a.tau = k.tau;
        a.sigma = k.sigma;
        a.theta = k.theta;
        a.tau_lambda = k.tau * k.lambda;
        a.alpha0 = k.alpha0;
        a.alpha1 = k.alpha1;
        a.penc = 32767.f / k.alpha1;
        a.pdec = k.alpha1 / 32767.f;
        a.qenc = 32767.f / k.alpha0;
        a.qdec = k.alpha0 / 32767.f;
        a.thr_p = projection_skip_bound(k.alpha1);
        a.thr_q = projection_skip_bound(k.alpha0);
        a.skip_bz = (k.data_term == TGVDCT_DATA_L2 && s.D == 1) ? 1 : 0;
        a.err = s.err;
        a.wait_ns = s.wait_ns;
        a.dom = s.domain;
        a.tile_active = (s.domain && s.tile_active && s.tile_zchunk == a.zchunk) ? s.tile_active
                                                                                  : nullptr;
        const bool m = a.dom != nullptr;
        if (k.data_term == TGVDCT_DATA_L1) {
            if (m) launch_shifted<PREC, TGVDCT_DATA_L1, true>(a, st);
            else launch_shifted<PREC, TGVDCT_DATA_L1, false>(a, st);
        } else {
            if (m) launch_shifted<PREC, TGVDCT_DATA_L2, true>(a, st);
            else launch_shifted<PREC, TGVDCT_DATA_L2, false>(a, st);
        }
    }
    {   // the primal step of the last iteration, into the standard state: u, v to their
        // own buffers, ubar, vbar to the set that holds the last p, q
        const int par = (int)((n - 1) & 1);
        const ShiftedSlot d = shifted_slot(s, c, par);
        const int set = par ? c : c ^ 1;
        float* const v_in[3] = {d.v[0], d.v[1], d.v[2]};
        float* const v_out[3] = {s.v[0], s.v[1], s.v[2]};
        const auto a = make_args<PREC>(s, k, s.set[set], d.u, v_in, s.set[set], s.u, v_out);
        if (k.data_term == TGVDCT_DATA_L1)
            tgv_primal_kernel<PREC, true, TGVDCT_DATA_L1><<<grid, block, 0, st>>>(a);
        else
            tgv_primal_kernel<PREC, true, TGVDCT_DATA_L2><<<grid, block, 0, st>>>(a);
        TGV_CHECK_LAUNCH();
        s.cur = set;
    }
    return (int)n + 1;
}

}  // namespace

size_t tgv_state_bytes(int W, int H, int D, bool three, int precision, int kernel) {
    const size_t n = (size_t)W * H * D;
    const size_t f32 = align256(n * 4), dual = align256(n * elem_bytes(precision));
    const int ncomp = three ? 3 : 2, nq = three ? 6 : 3;
    const int sets = kernel == TGV_KERNEL_TWO_PASS ? 1 : 2;
    // u, f, v + per set: ubar, vbar, p, q; plus a device error flag
    return f32 * (2 + ncomp) + sets * (f32 * (1 + ncomp) + dual * (ncomp + nq)) + 256;
}

void tgv_state_bind(TgvState& s, char* base) {
    const size_t n = (size_t)s.W * s.H * s.D;
    const size_t f32 = align256(n * 4), dual = align256(n * elem_bytes(s.precision));
    char* c = base;
    auto take = [&](size_t b) {
        char* r = c;
        c += b;
        return r;
    };
    const int ncomp = s.three ? 3 : 2, nq = s.three ? 6 : 3;
    s.u = (float*)take(f32);
    s.f = (float*)take(f32);
    for (int k = 0; k < 3; ++k) s.v[k] = k < ncomp ? (float*)take(f32) : nullptr;
    const int sets = s.kernel == TGV_KERNEL_TWO_PASS ? 1 : 2;
    s.tma_cache.reset();
    s.shifted_cache.reset();
    // q order: xx yy zz xy xz yz; the 2-D launcher keeps xx yy xy
    const int order2[3] = {0, 1, 3};
    for (int t = 0; t < 2; ++t) {
        TgvStencilFields& F = s.set[t];
        F = TgvStencilFields();
        if (t >= sets) continue;
        F.ubar = (float*)take(f32);
        for (int k = 0; k < ncomp; ++k) F.vbar[k] = (float*)take(f32);
        for (int k = 0; k < ncomp; ++k) F.p[k] = (void*)take(dual);
        for (int k = 0; k < nq; ++k) F.q[s.three ? k : order2[k]] = (void*)take(dual);
    }
    s.err = (int*)take(256);
    s.cur = 0;
}

void tgv_state_init(TgvState& s, cudaStream_t st) {
    const size_t n = (size_t)s.W * s.H * s.D;
    s.cur = 0;
    const TgvStencilFields& F = s.set[0];
    TGV_CUDA(cudaMemcpyAsync(s.u, s.f, n * 4, cudaMemcpyDeviceToDevice, st));
    TGV_CUDA(cudaMemcpyAsync(F.ubar, s.f, n * 4, cudaMemcpyDeviceToDevice, st));
    const size_t e = elem_bytes(s.precision);
    for (int k = 0; k < 3; ++k) {
        if (s.v[k]) TGV_CUDA(cudaMemsetAsync(s.v[k], 0, n * 4, st));
        if (F.vbar[k]) TGV_CUDA(cudaMemsetAsync(F.vbar[k], 0, n * 4, st));
        if (F.p[k]) TGV_CUDA(cudaMemsetAsync(F.p[k], 0, n * e, st));
    }
    for (int k = 0; k < 6; ++k)
        if (F.q[k]) TGV_CUDA(cudaMemsetAsync(F.q[k], 0, n * e, st));
    // masked runs skip the voxels outside the domain, so the second set must hold
    // the frozen values as well
    const TgvStencilFields& G = s.set[1];
    if (s.domain && G.ubar) {
        TGV_CUDA(cudaMemcpyAsync(G.ubar, s.f, n * 4, cudaMemcpyDeviceToDevice, st));
        for (int k = 0; k < 3; ++k) {
            if (G.vbar[k]) TGV_CUDA(cudaMemsetAsync(G.vbar[k], 0, n * 4, st));
            if (G.p[k]) TGV_CUDA(cudaMemsetAsync(G.p[k], 0, n * e, st));
        }
        for (int k = 0; k < 6; ++k)
            if (G.q[k]) TGV_CUDA(cudaMemsetAsync(G.q[k], 0, n * e, st));
    }
    TGV_CUDA(cudaMemsetAsync(s.err, 0, sizeof(int), st));
}

namespace {
__global__ void domain_kernel(const float* mask, size_t n, uint8_t* domain) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        domain[i] = mask[i] >= 1.f ? 1 : 0;
}
}  // namespace

void build_domain(const float* mask, size_t n, uint8_t* domain, cudaStream_t st) {
    const int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
    domain_kernel<<<blocks, 256, 0, st>>>(mask, n, domain);
    TGV_CHECK_LAUNCH();
}

namespace {
// flags[(cz * gridDim.y + by) * gridDim.x + bx] for the fused TMA kernel's block
// (bx, by, cz) -- columns [TX bx, TX bx + TX) x [TY by, TY by + TY), planes
// [cz zchunk, (cz + 1) zchunk) -- is (first << 16) | (last + 1) over the planes in
// which one of those columns is in the domain, or 0.  One thread per column.
__global__ void tile_flags_kernel(const uint8_t* domain, int W, int H, int D, int zchunk,
                                  uint32_t* flags) {
    __shared__ int lo, hi;
    if (threadIdx.x == 0) {
        lo = D;
        hi = -1;
    }
    __syncthreads();
    const int x = blockIdx.x * tma::TX + (int)(threadIdx.x % tma::TX);
    const int y = blockIdx.y * tma::TY + (int)(threadIdx.x / tma::TX);
    if (x < W && y < H) {
        const int z0 = (int)blockIdx.z * zchunk, z1 = min(D, z0 + zchunk);
        int first = D, last = -1;
        for (int z = z0; z < z1; ++z)
            if (domain[((size_t)z * H + y) * W + x]) {
                first = min(first, z);
                last = z;
            }
        if (last >= 0) {
            atomicMin(&lo, first);
            atomicMax(&hi, last);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0)
        flags[((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] =
            hi >= 0 ? ((uint32_t)lo << 16) | (uint32_t)(hi + 1) : 0u;
}
}  // namespace

size_t tgv_tile_flags_bytes(const TgvState& s) {
    return (size_t)ceil_div(s.W, tma::TX) * ceil_div(s.H, tma::TY) * (size_t)s.D *
           sizeof(uint32_t);
}

void tgv_build_tile_flags(TgvState& s, uint32_t* flags, cudaStream_t st) {
    s.tile_active = nullptr;
    if (!s.domain || !flags) return;
    const int ez = tma_zchunk(s);
    const dim3 grid(ceil_div(s.W, tma::TX), ceil_div(s.H, tma::TY), ceil_div(s.D, ez));
    tile_flags_kernel<<<grid, tma::TX * tma::TY, 0, st>>>(s.domain, s.W, s.H, s.D, ez, flags);
    TGV_CHECK_LAUNCH();
    s.tile_active = flags;
    s.tile_zchunk = ez;
}

bool tgv_uses_tma(const TgvState& s) { return tma_shape_ok(s); }

namespace {
TgvStencilFields stencil_view(const TgvFullDev& d) {
    TgvStencilFields F;
    F.ubar = d.ubar;
    for (int c = 0; c < 3; ++c) F.vbar[c] = d.vbar[c], F.p[c] = d.p[c];
    for (int c = 0; c < 6; ++c) F.q[c] = d.q[c];
    return F;
}
}  // namespace

namespace {
// TMA arguments of the recompute steps, one entry per (input, output) state pair.
struct StepCacheFp32 {
    struct Entry {
        TgvFullDev in, out;
        tma::Args<float> args;
    };
    std::vector<std::unique_ptr<Entry>> entries;
};

bool same_state(const TgvFullDev& a, const TgvFullDev& b) {
    bool same = a.u == b.u && a.ubar == b.ubar;
    for (int c = 0; c < 3; ++c)
        same = same && a.v[c] == b.v[c] && a.vbar[c] == b.vbar[c] && a.p[c] == b.p[c];
    for (int c = 0; c < 6; ++c) same = same && a.q[c] == b.q[c];
    return same;
}
}  // namespace

void tgv_step_fp32(const TgvState& s, const TgvStep& k, const TgvFullDev& in,
                   const TgvFullDev& out, std::shared_ptr<void>& cache, cudaStream_t st) {
    TGV_REQUIRE(s.precision == TGVDCT_STATE_FP32 && s.three,
                "the reverse mode needs FP32 state and 3-D geometry");
    if (tma_shape_ok(s) && s.err) {
        if (!cache) cache = std::make_shared<StepCacheFp32>();
        auto& ents = static_cast<StepCacheFp32*>(cache.get())->entries;
        StepCacheFp32::Entry* e = nullptr;
        for (auto& x : ents)
            if (same_state(x->in, in) && same_state(x->out, out)) e = x.get();
        if (!e) {
            ents.emplace_back(new StepCacheFp32::Entry);
            e = ents.back().get();
            e->in = in;
            e->out = out;
            fill_tma_args<float, TGVDCT_STATE_FP32>(e->args, s, stencil_view(in), in.u, in.v,
                                                    stencil_view(out), out.u, out.v);
        }
        launch_tma_step<TGVDCT_STATE_FP32>(e->args, s, k, s.err, st);
        return;
    }
    float* const vi[3] = {in.v[0], in.v[1], in.v[2]};
    float* const vo[3] = {out.v[0], out.v[1], out.v[2]};
    const auto a = make_args<TGVDCT_STATE_FP32>(s, k, stencil_view(in), in.u, vi,
                                                stencil_view(out), out.u, vo);
    launch_two_pass<TGVDCT_STATE_FP32>(s, k, a, st);
}

void tgv_save_state(const TgvState& s, const TgvFullDev& out, cudaStream_t st) {
    TGV_REQUIRE(s.precision == TGVDCT_STATE_FP32 && s.three,
                "the reverse mode needs FP32 state and 3-D geometry");
    const size_t b = (size_t)s.W * s.H * s.D * 4;
    const TgvStencilFields& F = s.now();
    TGV_CUDA(cudaMemcpyAsync(out.u, s.u, b, cudaMemcpyDeviceToDevice, st));
    TGV_CUDA(cudaMemcpyAsync(out.ubar, F.ubar, b, cudaMemcpyDeviceToDevice, st));
    for (int c = 0; c < 3; ++c) {
        TGV_CUDA(cudaMemcpyAsync(out.v[c], s.v[c], b, cudaMemcpyDeviceToDevice, st));
        TGV_CUDA(cudaMemcpyAsync(out.vbar[c], F.vbar[c], b, cudaMemcpyDeviceToDevice, st));
        TGV_CUDA(cudaMemcpyAsync(out.p[c], F.p[c], b, cudaMemcpyDeviceToDevice, st));
    }
    for (int c = 0; c < 6; ++c)
        TGV_CUDA(cudaMemcpyAsync(out.q[c], F.q[c], b, cudaMemcpyDeviceToDevice, st));
}

namespace {
// The fields of a snapshot, in order: f, u, v[..] (FP32), then ubar, vbar[..] (FP32),
// p[..], q[..] (dual element size) of stencil set `set`; only the allocated ones.
template <class Fn>
void for_each_snapshot_field(const TgvState& s, int set, Fn&& fn) {
    const size_t n = (size_t)s.W * s.H * s.D, e = elem_bytes(s.precision);
    const TgvStencilFields& F = s.set[set];
    fn((void*)s.f, n * 4);
    fn((void*)s.u, n * 4);
    for (int k = 0; k < 3; ++k)
        if (s.v[k]) fn((void*)s.v[k], n * 4);
    fn((void*)F.ubar, n * 4);
    for (int k = 0; k < 3; ++k)
        if (F.vbar[k]) fn((void*)F.vbar[k], n * 4);
    for (int k = 0; k < 3; ++k)
        if (F.p[k]) fn((void*)F.p[k], n * e);
    for (int k = 0; k < 6; ++k)
        if (F.q[k]) fn((void*)F.q[k], n * e);
}
}  // namespace

size_t tgv_snapshot_bytes(const TgvState& s) {
    size_t b = 0;
    for_each_snapshot_field(s, 0, [&](void*, size_t bytes) { b += bytes; });
    return b;
}

void tgv_snapshot_save(const TgvState& s, void* dst, cudaStream_t st) {
    char* d = (char*)dst;
    for_each_snapshot_field(s, s.cur, [&](void* field, size_t bytes) {
        TGV_CUDA(cudaMemcpyAsync(d, field, bytes, cudaMemcpyDeviceToDevice, st));
        d += bytes;
    });
}

void tgv_snapshot_load(TgvState& s, const void* src, cudaStream_t st) {
    // both stencil sets get the snapshot (a masked run reads the frozen outside
    // values from either set), and the loop continues from set 0
    for (int set = 0; set < 2; ++set) {
        if (!s.set[set].ubar) continue;
        const char* p = (const char*)src;
        for_each_snapshot_field(s, set, [&](void* field, size_t bytes) {
            TGV_CUDA(cudaMemcpyAsync(field, p, bytes, cudaMemcpyDeviceToDevice, st));
            p += bytes;
        });
    }
    s.cur = 0;
}

uint64_t tgv_kernels_bounds_take() {
    unsigned long long w = 0;
    TGV_CUDA(cudaMemcpyFromSymbol(&w, g_bounds_tgv, sizeof(w)));
    if (w) {
        const unsigned long long zero = 0;
        TGV_CUDA(cudaMemcpyToSymbol(g_bounds_tgv, &zero, sizeof(zero)));
    }
    return w;
}

void tgv_iterate(TgvState& s, const TgvStep& k, cudaStream_t st) {
    if (tma_shape_ok(s)) {
        TGV_REQUIRE(s.err != nullptr, "TMA kernel needs a device error flag");
        switch (s.precision) {
            case TGVDCT_STATE_FP32: iterate_tma<TGVDCT_STATE_FP32>(s, k, s.err, st); return;
            case TGVDCT_STATE_BF16_DUAL: iterate_tma<TGVDCT_STATE_BF16_DUAL>(s, k, s.err, st); return;
            case TGVDCT_STATE_FX16_DUAL: iterate_tma<TGVDCT_STATE_FX16_DUAL>(s, k, s.err, st); return;
        }
    }
    // The register-staged fused kernel has no domain support: a masked run whose
    // shape rules out TMA uses the two-pass kernels in place on the current set.
    if (s.kernel == TGV_KERNEL_TWO_PASS || s.domain) {
        switch (s.precision) {
            case TGVDCT_STATE_FP32: iterate_two_pass<TGVDCT_STATE_FP32>(s, k, st); return;
            case TGVDCT_STATE_BF16_DUAL: iterate_two_pass<TGVDCT_STATE_BF16_DUAL>(s, k, st); return;
            case TGVDCT_STATE_FX16_DUAL: iterate_two_pass<TGVDCT_STATE_FX16_DUAL>(s, k, st); return;
        }
    } else {
        switch (s.precision) {
            case TGVDCT_STATE_FP32: iterate_fused<TGVDCT_STATE_FP32>(s, k, st); return;
            case TGVDCT_STATE_BF16_DUAL: iterate_fused<TGVDCT_STATE_BF16_DUAL>(s, k, st); return;
            case TGVDCT_STATE_FX16_DUAL: iterate_fused<TGVDCT_STATE_FX16_DUAL>(s, k, st); return;
        }
    }
    TGV_REQUIRE(false, "unknown state precision");
}

int tgv_kernels_per_iteration(const TgvState& s) { return s.kernel == TGV_KERNEL_TWO_PASS ? 2 : 1; }

bool tgv_uses_shifted(const TgvState& s) { return shifted_ok(s); }

int tgv_iterate_n(TgvState& s, const TgvStep& k, uint32_t n, cudaStream_t st) {
    if (n >= 2 && shifted_ok(s)) {
        switch (s.precision) {
            case TGVDCT_STATE_FP32: return iterate_shifted<TGVDCT_STATE_FP32>(s, k, n, st);
            case TGVDCT_STATE_BF16_DUAL: return iterate_shifted<TGVDCT_STATE_BF16_DUAL>(s, k, n, st);
            case TGVDCT_STATE_FX16_DUAL: return iterate_shifted<TGVDCT_STATE_FX16_DUAL>(s, k, n, st);
        }
    }
    for (uint32_t i = 0; i < n; ++i) tgv_iterate(s, k, st);
    return (int)n * tgv_kernels_per_iteration(s);
}

template <int PREC>
void prepare_shifted() {
    shifted_attr<PREC, TGVDCT_DATA_L1, false>();
    shifted_attr<PREC, TGVDCT_DATA_L2, false>();
    shifted_attr<PREC, TGVDCT_DATA_L1, true>();
    shifted_attr<PREC, TGVDCT_DATA_L2, true>();
}

void tgv_prepare_launches(const TgvState& s) {
    if (!shifted_ok(s)) return;
    switch (s.precision) {
        case TGVDCT_STATE_FP32: prepare_shifted<TGVDCT_STATE_FP32>(); break;
        case TGVDCT_STATE_BF16_DUAL: prepare_shifted<TGVDCT_STATE_BF16_DUAL>(); break;
        case TGVDCT_STATE_FX16_DUAL: prepare_shifted<TGVDCT_STATE_FX16_DUAL>(); break;
    }
}

}  // namespace tgvdct
