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
#include "common.cuh"

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
};

// 16-bit fixed point: value = code * (alpha / 32767).  After the projections every
// component of p satisfies |p_c| <= |p| <= alpha1 and every component of q
// satisfies |q_c| <= alpha0, so the code range covers the field exactly.
template <>
struct Dual<TGVDCT_STATE_FX16_DUAL> {
    using T = int16_t;
    static __device__ __forceinline__ float ld(const T* p, size_t i, float dec) {
        return (float)p[i] * dec;
    }
    static __device__ __forceinline__ void st(T* p, size_t i, float v, float enc) {
        float c = rintf(v * enc);
        c = fminf(fmaxf(c, -32767.f), 32767.f);
        p[i] = (T)(int)c;
    }
};

template <class T>
struct TgvArgs {
    int W, H, D;
    size_t WH;
    const float* __restrict__ f;
    float* __restrict__ u;
    float* __restrict__ ubar;
    float* __restrict__ v0;
    float* __restrict__ v1;
    float* __restrict__ v2;
    float* __restrict__ vb0;
    float* __restrict__ vb1;
    float* __restrict__ vb2;
    T* __restrict__ p0;
    T* __restrict__ p1;
    T* __restrict__ p2;
    T* __restrict__ qxx;
    T* __restrict__ qyy;
    T* __restrict__ qzz;
    T* __restrict__ qxy;
    T* __restrict__ qxz;
    T* __restrict__ qyz;
    float tau, sigma, theta, tau_lambda, alpha0, alpha1;
    float penc, pdec, qenc, qdec;
    int skip_bz;  // L2 data term with depth == 1 drops B_z p (tgv_cuda/tgv2_l2.cu:39-42)
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

    // p <- proj(p + sigma (F ubar - vbar))          (tgv2_common.cu:118-130)
    const float ub = a.ubar[i];
    const float gx = (x + 1 < a.W) ? a.ubar[i + 1] - ub : 0.f;
    const float gy = (y + 1 < a.H) ? a.ubar[i + W] - ub : 0.f;
    const float vbx = a.vb0[i], vby = a.vb1[i];
    float px = __fmaf_rn(a.sigma, gx - vbx, S::ld(a.p0, i, a.pdec));
    float py = __fmaf_rn(a.sigma, gy - vby, S::ld(a.p1, i, a.pdec));
    float pz = 0.f, vbz = 0.f, nrm;
    if constexpr (THREE) {
        const float gz = (z + 1 < a.D) ? a.ubar[i + WH] - ub : 0.f;
        vbz = a.vb2[i];
        pz = __fmaf_rn(a.sigma, gz - vbz, S::ld(a.p2, i, a.pdec));
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
    float qxx = __fmaf_rn(a.sigma, exx, S::ld(a.qxx, i, a.qdec));
    float qyy = __fmaf_rn(a.sigma, eyy, S::ld(a.qyy, i, a.qdec));
    float qxy = __fmaf_rn(a.sigma, exy, S::ld(a.qxy, i, a.qdec));
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
        qzz = __fmaf_rn(a.sigma, ezz, S::ld(a.qzz, i, a.qdec));
        qxz = __fmaf_rn(a.sigma, exz, S::ld(a.qxz, i, a.qdec));
        qyz = __fmaf_rn(a.sigma, eyz, S::ld(a.qyz, i, a.qdec));
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
    const bool xl = x + 1 < a.W, yl = y + 1 < a.H;

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
    const float uo = a.u[i];
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
    a.ubar[i] = uu + a.theta * (uu - uo);

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
        const float vo = a.v0[i];
        const float vn = vo - a.tau * (dx - pxi);
        a.v0[i] = vn;
        a.vb0[i] = vn + a.theta * (vn - vo);
    }
    {
        const float vo = a.v1[i];
        const float vn = vo - a.tau * (dy - pyi);
        a.v1[i] = vn;
        a.vb1[i] = vn + a.theta * (vn - vo);
    }
    if constexpr (THREE) {
        const float vo = a.v2[i];
        const float vn = vo - a.tau * (dz - pzi);
        a.v2[i] = vn;
        a.vb2[i] = vn + a.theta * (vn - vo);
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

size_t elem_bytes(int precision) { return precision == TGVDCT_STATE_FP32 ? 4 : 2; }
size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

template <int PREC>
TgvArgs<typename Dual<PREC>::T> make_args(const TgvState& s, const TgvStep& k) {
    using T = typename Dual<PREC>::T;
    const TgvStencilFields& F = s.set[0];
    TgvArgs<T> a;
    a.W = s.W;
    a.H = s.H;
    a.D = s.D;
    a.WH = (size_t)s.W * s.H;
    a.f = s.f;
    a.u = s.u;
    a.ubar = F.ubar;
    a.v0 = s.v[0];
    a.v1 = s.v[1];
    a.v2 = s.v[2];
    a.vb0 = F.vbar[0];
    a.vb1 = F.vbar[1];
    a.vb2 = F.vbar[2];
    a.p0 = (T*)F.p[0];
    a.p1 = (T*)F.p[1];
    a.p2 = (T*)F.p[2];
    a.qxx = (T*)F.q[0];
    a.qyy = (T*)F.q[1];
    a.qzz = (T*)F.q[2];
    a.qxy = (T*)F.q[3];
    a.qxz = (T*)F.q[4];
    a.qyz = (T*)F.q[5];
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
    return a;
}

template <int PREC>
void iterate_two_pass(const TgvState& s, const TgvStep& k, cudaStream_t st) {
    const auto a = make_args<PREC>(s, k);
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

constexpr int FUSED_TY = 8;

template <int PREC, bool THREE, int DATA>
void launch_fused(const FusedArgs<typename Dual<PREC>::T>& a, int D, cudaStream_t st) {
    constexpr int TY = FUSED_TY;
    constexpr size_t smem = fused_smem_floats<TY, THREE>() * sizeof(float);
    auto kern = tgv_fused_kernel<PREC, THREE, DATA, TY>;
    static bool configured = false;  // per template instance
    if (!configured) {
        TGV_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured = true;
    }
    const dim3 grid(ceil_div(a.W, FX), ceil_div(a.H, TY), ceil_div(D, a.zchunk));
    kern<<<grid, fused_threads<TY>(), smem, st>>>(a);
    TGV_CHECK_LAUNCH();
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

}  // namespace

size_t tgv_state_bytes(int W, int H, int D, bool three, int precision, int kernel) {
    const size_t n = (size_t)W * H * D;
    const size_t f32 = align256(n * 4), dual = align256(n * elem_bytes(precision));
    const int ncomp = three ? 3 : 2, nq = three ? 6 : 3;
    const int sets = kernel == TGV_KERNEL_FUSED ? 2 : 1;
    // u, f, v + per set: ubar, vbar, p, q
    return f32 * (2 + ncomp) + sets * (f32 * (1 + ncomp) + dual * (ncomp + nq));
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
    const int sets = s.kernel == TGV_KERNEL_FUSED ? 2 : 1;
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
}

void tgv_iterate(TgvState& s, const TgvStep& k, cudaStream_t st) {
    if (s.kernel == TGV_KERNEL_TWO_PASS) {
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

int tgv_kernels_per_iteration(const TgvState& s) { return s.kernel == TGV_KERNEL_FUSED ? 1 : 2; }

}  // namespace tgvdct
