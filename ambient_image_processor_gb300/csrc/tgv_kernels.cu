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

size_t elem_bytes(int precision) { return precision == TGVDCT_STATE_FP32 ? 4 : 2; }
size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

template <int PREC>
TgvArgs<typename Dual<PREC>::T> make_args(const TgvState& s, const TgvStep& k) {
    using T = typename Dual<PREC>::T;
    TgvArgs<T> a;
    a.W = s.W;
    a.H = s.H;
    a.D = s.D;
    a.WH = (size_t)s.W * s.H;
    a.f = s.f;
    a.u = s.u;
    a.ubar = s.ubar;
    a.v0 = s.v[0];
    a.v1 = s.v[1];
    a.v2 = s.v[2];
    a.vb0 = s.vbar[0];
    a.vb1 = s.vbar[1];
    a.vb2 = s.vbar[2];
    a.p0 = (T*)s.p[0];
    a.p1 = (T*)s.p[1];
    a.p2 = (T*)s.p[2];
    a.qxx = (T*)s.q[0];
    a.qyy = (T*)s.q[1];
    a.qzz = (T*)s.q[2];
    a.qxy = (T*)s.q[3];
    a.qxz = (T*)s.q[4];
    a.qyz = (T*)s.q[5];
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
void iterate_prec(const TgvState& s, const TgvStep& k, cudaStream_t st) {
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

}  // namespace

size_t tgv_state_bytes(int W, int H, int D, bool three, int precision) {
    const size_t n = (size_t)W * H * D;
    const size_t f32 = align256(n * 4), dual = align256(n * elem_bytes(precision));
    const int ncomp = three ? 3 : 2, nq = three ? 6 : 3;
    return f32 * (3 + 2 * ncomp) + dual * (ncomp + nq);
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
    s.u = (float*)take(f32);
    s.ubar = (float*)take(f32);
    s.f = (float*)take(f32);
    const int ncomp = s.three ? 3 : 2, nq = s.three ? 6 : 3;
    for (int k = 0; k < 3; ++k) s.v[k] = k < ncomp ? (float*)take(f32) : nullptr;
    for (int k = 0; k < 3; ++k) s.vbar[k] = k < ncomp ? (float*)take(f32) : nullptr;
    for (int k = 0; k < 3; ++k) s.p[k] = k < ncomp ? (void*)take(dual) : nullptr;
    // q order: xx yy zz xy xz yz; the 2-D launcher keeps xx yy xy
    const int order3[6] = {0, 1, 2, 3, 4, 5};
    const int order2[3] = {0, 1, 3};
    for (int k = 0; k < 6; ++k) s.q[k] = nullptr;
    for (int k = 0; k < nq; ++k) s.q[s.three ? order3[k] : order2[k]] = (void*)take(dual);
}

void tgv_state_init(const TgvState& s, cudaStream_t st) {
    const size_t n = (size_t)s.W * s.H * s.D;
    TGV_CUDA(cudaMemcpyAsync(s.u, s.f, n * 4, cudaMemcpyDeviceToDevice, st));
    TGV_CUDA(cudaMemcpyAsync(s.ubar, s.f, n * 4, cudaMemcpyDeviceToDevice, st));
    const size_t e = elem_bytes(s.precision);
    for (int k = 0; k < 3; ++k) {
        if (s.v[k]) TGV_CUDA(cudaMemsetAsync(s.v[k], 0, n * 4, st));
        if (s.vbar[k]) TGV_CUDA(cudaMemsetAsync(s.vbar[k], 0, n * 4, st));
        if (s.p[k]) TGV_CUDA(cudaMemsetAsync(s.p[k], 0, n * e, st));
    }
    for (int k = 0; k < 6; ++k)
        if (s.q[k]) TGV_CUDA(cudaMemsetAsync(s.q[k], 0, n * e, st));
}

void tgv_iterate(const TgvState& s, const TgvStep& k, cudaStream_t st) {
    switch (s.precision) {
        case TGVDCT_STATE_FP32: iterate_prec<TGVDCT_STATE_FP32>(s, k, st); break;
        case TGVDCT_STATE_BF16_DUAL: iterate_prec<TGVDCT_STATE_BF16_DUAL>(s, k, st); break;
        case TGVDCT_STATE_FX16_DUAL: iterate_prec<TGVDCT_STATE_FX16_DUAL>(s, k, st); break;
        default: TGV_REQUIRE(false, "unknown state precision");
    }
}

int tgv_kernels_per_iteration() { return 2; }

}  // namespace tgvdct
