// Reverse mode of the TGV2 loop: the adjoint of one primal-dual iteration as three
// passes, and the checkpointed driver that runs it backwards through K iterations.
//
// One forward iteration S_k -> S_{k+1} (state u, ubar, v, vbar, p, q; tgv_kernels.cu):
//   y_p = p + sigma (F ubar - vbar),  p' = P_{alpha1}(y_p)
//   y_q = q + sigma E vbar,           q' = Q_{alpha0}(y_q)
//   u~  = u - tau B.p',  u' = prox(u~; f, tau lambda),  ubar' = u' + theta (u' - u)
//   v'  = v - tau (divF q' - p'),  vbar' = v' + theta (v' - v)
// Reverse (adjoints a(.) of S_{k+1} in, of S_k out; lambda, alpha0, alpha1, f accumulated):
//   R1  a(v') = a(v)+(1+theta) a(vbar);  a(u') = a(u)+(1+theta) a(ubar)
//       prox branch of u~ (recomputed bit for bit from S_k.u and S_{k+1}.p): a(u~), d/df,
//       d/dlambda;  out: a(u) = -theta a(ubar) + a(u~),  a(v) = a(v') - theta a(vbar)
//   R2  a(p') = a(p) + tau a(v') - tau B^T a(u~);  a(q') = a(q) - tau divF^T a(v')
//       projection Jacobians at y_p, y_q (recomputed from S_k):
//       J^T g = (alpha/n) g - (alpha/n^3) w.y (y.g) when |y| > alpha, d/dalpha += y.g/n
//       out: a(p) = J_P^T a(p'),  a(q) = J_Q^T a(q')
//   R3  out: a(ubar) = sigma F^T a(p),  a(vbar) = -sigma a(p) + sigma E^T a(q)
// with (F_a^T g)[j] = g[j-e] (j_a >= 1) - g[j] (j_a < N-1) and
// (B_a^T g)[j] = g[j+e] (j_a < N-1) - g[j].  R3 of iteration k and R1 of iteration
// k-1 are pointwise in a(ubar), a(vbar), so inside a segment they run as one kernel
// (adjoint_r3r1) and those four fields never reach memory: per voxel and iteration
// the adjoint moves 63 fields (252 bytes).  An FP64 restatement of the same algebra
// in the oracle gives the reference gradient (central differences pin it).
#include <algorithm>

#include "common.cuh"

// first bad index of a bounds-checking build (see TGV_IN_BOUNDS)
static __device__ unsigned long long g_bounds_adj;
#define TGV_BOUNDS_WORD g_bounds_adj

namespace tgvdct {
namespace {

constexpr int BX = 32, BY = 8;

struct AdjArgs {
    int W, H, D;
    size_t WH;
    const float* f;
    TgvFullDev S;   // S_k
    TgvFullDev S1;  // S_{k+1}
    TgvFullDev A;   // in: adjoint of S_{k+1}; out: adjoint of S_k (in place)
    float* uta;     // a(u~)
    float* va[3];   // a(v')
    float* grad_f;
    double* gp;     // d/dlambda, d/dalpha0, d/dalpha1
    float tau, sigma, theta, tau_lambda, alpha0, alpha1;
    int data_term, skip_bz;
    int zm;  // planes per thread of the z-marching kernels
};

__device__ __forceinline__ void block_add(double* dst, float v) {
    __shared__ float red[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    if ((t & 31) == 0) red[t >> 5] = v;
    __syncthreads();
    if (t == 0) {
        float s = 0.f;
        const int warps = (int)(blockDim.x * blockDim.y) / 32;
        for (int w = 0; w < warps; ++w) s += red[w];
        if (s != 0.f) atomicAdd(dst, (double)s);
    }
    __syncthreads();
}

// The per-voxel arithmetic takes the neighbour values it needs as arguments, so that
// the one-voxel-per-thread kernels (used once per segment) and the z-marching kernels
// (used every iteration; z neighbours carried in registers) share it.  A neighbour
// outside the volume is passed as 0, as the forward operators read it.

// R1 inputs at voxel i: p' = S1.p (centre and the -x, -y, -z neighbours), u and f.
struct R1In {
    float p0, p1, p2;   // S1.p[c][i]
    float px, py, pz;   // S1.p[0][i-1], S1.p[1][i-W], S1.p[2][i-WH]
    float uo, fi;       // S.u[i], f[i]
};

// R1 at voxel i, with a(ubar) and a(vbar) of S_{k+1} given: returns the d/dlambda term.
__device__ __forceinline__ float r1_vals(const AdjArgs& a, size_t i, const R1In& in, float aub,
                                         const float* avb) {
    float glam = 0.f;
    // u~ exactly as the forward primal pass computed it
    const float bx = in.px - in.p0;
    const float by = in.py - in.p1;
    float div = bx + by;
    const float bz = in.pz - in.p2;
    if (!a.skip_bz) div = div + bz;
    const float ut = in.uo - a.tau * div;
    const float ua = a.A.u[i] + (1.f + a.theta) * aub;
    float uta, gf = 0.f;
    if (a.data_term == TGVDCT_DATA_L1) {
        const float dd = ut - in.fi;
        if (dd > a.tau_lambda) {
            uta = ua;
            glam = -a.tau * ua;
        } else if (dd < -a.tau_lambda) {
            uta = ua;
            glam = a.tau * ua;
        } else {
            uta = 0.f;
            gf = ua;
        }
    } else {
        const float den = 1.f + a.tau_lambda;
        uta = ua / den;
        gf = a.tau_lambda * ua / den;
        glam = ua * a.tau * (in.fi - ut) / (den * den);
    }
    a.A.u[i] = -a.theta * aub + uta;
    a.uta[i] = uta;
    if (gf != 0.f) a.grad_f[i] += gf;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float va = a.A.v[c][i] + (1.f + a.theta) * avb[c];
        a.va[c][i] = va;
        a.A.v[c][i] = va - a.theta * avb[c];
    }
    return glam;
}

// R3 inputs at voxel i: a(p) with its -x, -y, -z neighbours, a(q) with the +x, +y, +z
// neighbours the transposed backward differences read.
struct R3In {
    float p0, p1, p2;      // A.p[c][i]
    float px, py, pz;      // A.p[0][i-1], A.p[1][i-W], A.p[2][i-WH]
    float q[6];            // A.q[k][i], xx yy zz xy xz yz
    float qx0, qx3, qx4;   // A.q[0], A.q[3], A.q[4] at i+1
    float qy3, qy1, qy5;   // A.q[3], A.q[1], A.q[5] at i+W
    float qz4, qz5, qz2;   // A.q[4], A.q[5], A.q[2] at i+WH
};

// R3 at voxel i: a(ubar) and a(vbar) of S_k from a(p), a(q) (after R2).
__device__ __forceinline__ void r3_vals(const AdjArgs& a, bool xl, bool yl, bool zl,
                                        const R3In& in, float& aub, float* avb) {
    // a(ubar) = sigma sum_c F_c^T a(p)_c
    const float ftx = in.px - (xl ? in.p0 : 0.f);
    const float fty = in.py - (yl ? in.p1 : 0.f);
    const float ftz = in.pz - (zl ? in.p2 : 0.f);
    aub = a.sigma * ((ftx + fty) + ftz);
    // a(vbar)_c = -sigma a(p)_c + sigma sum_a w B_a^T a(q)_{c a}
    const float* q = in.q;  // xx yy zz xy xz yz
    const float ex = (in.qx0 - q[0]) + 0.5f * (in.qy3 - q[3]) + 0.5f * (in.qz4 - q[4]);
    const float ey = 0.5f * (in.qx3 - q[3]) + (in.qy1 - q[1]) + 0.5f * (in.qz5 - q[5]);
    const float ez = 0.5f * (in.qx4 - q[4]) + 0.5f * (in.qy5 - q[5]) + (in.qz2 - q[2]);
    avb[0] = -a.sigma * in.p0 + a.sigma * ex;
    avb[1] = -a.sigma * in.p1 + a.sigma * ey;
    avb[2] = -a.sigma * in.p2 + a.sigma * ez;
}

// The in-plane loads of R1 and R3 (the z neighbours are passed in).
__device__ __forceinline__ void r1_load(const AdjArgs& a, size_t i, bool xf, bool yf, R1In& in) {
    const size_t W = a.W;
    in.p0 = a.S1.p[0][i];
    in.p1 = a.S1.p[1][i];
    in.p2 = a.S1.p[2][i];
    in.px = xf ? a.S1.p[0][i - 1] : 0.f;
    in.py = yf ? a.S1.p[1][i - W] : 0.f;
    in.uo = a.S.u[i];
    in.fi = a.f[i];
}
__device__ __forceinline__ void r3_load(const AdjArgs& a, size_t i, bool xf, bool yf, bool xl,
                                        bool yl, R3In& in) {
    const size_t W = a.W;
    const float* const* P = a.A.p;
    const float* const* Q = a.A.q;
    in.p0 = P[0][i];
    in.p1 = P[1][i];
    in.p2 = P[2][i];
    in.px = xf ? P[0][i - 1] : 0.f;
    in.py = yf ? P[1][i - W] : 0.f;
#pragma unroll
    for (int k = 0; k < 6; ++k) in.q[k] = Q[k][i];
    in.qx0 = xl ? Q[0][i + 1] : 0.f;
    in.qx3 = xl ? Q[3][i + 1] : 0.f;
    in.qx4 = xl ? Q[4][i + 1] : 0.f;
    in.qy3 = yl ? Q[3][i + W] : 0.f;
    in.qy1 = yl ? Q[1][i + W] : 0.f;
    in.qy5 = yl ? Q[5][i + W] : 0.f;
}

__device__ __forceinline__ void prefetch_l2(const float* p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__global__ void __launch_bounds__(BX* BY) adjoint_r1(AdjArgs a) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
    const int z = blockIdx.z;
    float glam = 0.f;
    const size_t i = ((size_t)z * a.H + y) * a.W + x;
    if (x < a.W && y < a.H && TGV_IN_BOUNDS(i, a.WH * a.D, 30)) {
        R1In in;
        r1_load(a, i, x > 0, y > 0, in);
        in.pz = z > 0 ? a.S1.p[2][i - a.WH] : 0.f;
        const float avb[3] = {a.A.vbar[0][i], a.A.vbar[1][i], a.A.vbar[2][i]};
        glam = r1_vals(a, i, in, a.A.ubar[i], avb);
    }
    block_add(&a.gp[0], glam);
}

__global__ void __launch_bounds__(BX* BY) adjoint_r3(AdjArgs a) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= a.W || y >= a.H) return;
    const size_t i = ((size_t)z * a.H + y) * a.W + x, WH = a.WH;
    if (!TGV_IN_BOUNDS(i, WH * a.D, 31)) return;
    const bool zl = z + 1 < a.D;
    R3In in;
    r3_load(a, i, x > 0, y > 0, x + 1 < a.W, y + 1 < a.H, in);
    in.pz = z > 0 ? a.A.p[2][i - WH] : 0.f;
    in.qz4 = zl ? a.A.q[4][i + WH] : 0.f;
    in.qz5 = zl ? a.A.q[5][i + WH] : 0.f;
    in.qz2 = zl ? a.A.q[2][i + WH] : 0.f;
    float aub, avb[3];
    r3_vals(a, x + 1 < a.W, y + 1 < a.H, zl, in, aub, avb);
    a.A.ubar[i] = aub;
#pragma unroll
    for (int c = 0; c < 3; ++c) a.A.vbar[c][i] = avb[c];
}

// The projection pass (R2, 26 loads per voxel) marches up to ZM_MAX planes per
// thread.  Its fields are prefetched into L2 ZPF planes ahead, and the 18 pointwise
// fields (a(p), a(q), p, q) of the next plane are loaded into registers while the
// current plane computes, at three blocks per SM.  At 256 x 256 x 192 the one-voxel
// kernel took 429 us per launch, the march with the L2 prefetch 367 us and the
// register queue 324 us (standalone, the same inputs).  Small volumes get fewer
// planes per thread so that a launch keeps about two waves of blocks (zm_for); at
// one plane the one-voxel kernel runs.  The march made R3.R1 (19 loads per voxel)
// slower (262 -> 288 us), so it stays one voxel per thread.
constexpr int ZM_MAX = 4, ZPF = 1;

// R3 of iteration k followed by R1 of iteration k-1 (S = S_{k-1}, S1 = S_k): a(ubar)
// and a(vbar) stay in registers.  One voxel per thread, TBX x (256 / TBX) blocks:
// rows of 128 or 256 voxels per block read each field in longer runs, which at
// 256 x 256 x 192 took it from 241 to 230 us; narrow volumes keep 32 x 8.
template <int TBX>
__global__ void __launch_bounds__(BX* BY) adjoint_r3r1(AdjArgs a) {
    constexpr int TBY = BX * BY / TBX;
    const int x = blockIdx.x * TBX + threadIdx.x, y = blockIdx.y * TBY + threadIdx.y;
    const int z = blockIdx.z;
    float glam = 0.f;
    const size_t i = ((size_t)z * a.H + y) * a.W + x, WH = a.WH;
    if (x < a.W && y < a.H && TGV_IN_BOUNDS(i, WH * a.D, 32)) {
        const bool xl = x + 1 < a.W, yl = y + 1 < a.H, zl = z + 1 < a.D;
        const bool xf = x > 0, yf = y > 0, zf = z > 0;
        R3In r3;
        r3_load(a, i, xf, yf, xl, yl, r3);
        r3.pz = zf ? a.A.p[2][i - WH] : 0.f;
        r3.qz4 = zl ? a.A.q[4][i + WH] : 0.f;
        r3.qz5 = zl ? a.A.q[5][i + WH] : 0.f;
        r3.qz2 = zl ? a.A.q[2][i + WH] : 0.f;
        float aub, avb[3];
        r3_vals(a, xl, yl, zl, r3, aub, avb);
        R1In r1;
        r1_load(a, i, xf, yf, r1);
        r1.pz = zf ? a.S1.p[2][i - WH] : 0.f;
        glam = r1_vals(a, i, r1, aub, avb);
    }
    block_add(&a.gp[0], glam);
}

// R2's pointwise inputs at voxel i: a(p), a(q) (adjoints of S_{k+1}) and p, q of S_k.
struct R2Pw {
    float ap[3], aq[6], sp[3], sq[6];
};
__device__ __forceinline__ void r2_pw_load(const AdjArgs& a, size_t i, R2Pw& P) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        P.ap[c] = a.A.p[c][i];
        P.sp[c] = a.S.p[c][i];
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        P.aq[k] = a.A.q[k][i];
        P.sq[k] = a.S.q[k][i];
    }
}

// R2's stencil inputs at voxel i: a(u~) and ubar with their +x, +y, +z neighbours,
// a(v') and vbar with their -x, -y, -z neighbours.
struct R2In {
    float ut0, utx, uty, utz;
    float va0[3], vax[3], vay[3], vaz[3];
    float u0, ubx, uby, ubz;
    float vb0[3], vbx[3], vby[3], vbz[3];
};

// R2 at voxel i: the projection Jacobians; accumulates d/dalpha0, d/dalpha1.
__device__ __forceinline__ void r2_vals(const AdjArgs& a, size_t i, const R2Pw& P, bool xl,
                                        bool yl, bool zl, bool xf, bool yf, bool zf,
                                        const R2In& L, float& ga0, float& ga1) {
    // a(p') = a(p) + tau a(v') - tau B^T a(u~)
    const float bt[3] = {(xl ? L.utx : 0.f) - L.ut0, (yl ? L.uty : 0.f) - L.ut0,
                         (zl ? L.utz : 0.f) - L.ut0};
    float pa[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        pa[c] = P.ap[c] + a.tau * L.va0[c];
        if (!(c == 2 && a.skip_bz)) pa[c] = pa[c] - a.tau * bt[c];
    }
    // a(q') = a(q) - tau divF^T a(v'): (F_a^T g)[i] = g[i-e] (if >= 1) - g[i] (if < N-1)
    float fx[3], fy[3], fz[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float g0 = L.va0[c];
        fx[c] = (xf ? L.vax[c] : 0.f) - (xl ? g0 : 0.f);
        fy[c] = (yf ? L.vay[c] : 0.f) - (yl ? g0 : 0.f);
        fz[c] = (zf ? L.vaz[c] : 0.f) - (zl ? g0 : 0.f);
    }
    float qa[6];  // xx yy zz xy xz yz
    qa[0] = P.aq[0] - a.tau * fx[0];
    qa[1] = P.aq[1] - a.tau * fy[1];
    qa[2] = P.aq[2] - a.tau * fz[2];
    qa[3] = P.aq[3] - a.tau * (fy[0] + fx[1]);
    qa[4] = P.aq[4] - a.tau * (fz[0] + fx[2]);
    qa[5] = P.aq[5] - a.tau * (fz[1] + fy[2]);
    // y_p of the forward dual pass, bit for bit
    const float gx = xl ? L.ubx - L.u0 : 0.f;
    const float gy = yl ? L.uby - L.u0 : 0.f;
    const float gz = zl ? L.ubz - L.u0 : 0.f;
    const float* vb = L.vb0;
    const float yp[3] = {__fmaf_rn(a.sigma, gx - vb[0], P.sp[0]),
                         __fmaf_rn(a.sigma, gy - vb[1], P.sp[1]),
                         __fmaf_rn(a.sigma, gz - vb[2], P.sp[2])};
    const float np = norm3df(yp[0], yp[1], yp[2]);
    if (fmaxf(1.f, np / a.alpha1) > 1.f) {
        const float yg = yp[0] * pa[0] + yp[1] * pa[1] + yp[2] * pa[2];
        const float s = a.alpha1 / np, s3 = s / (np * np);
#pragma unroll
        for (int c = 0; c < 3; ++c) pa[c] = s * pa[c] - s3 * yp[c] * yg;
        ga1 += yg / np;
    }
    // y_q of the forward dual pass, bit for bit
    const float vbx_x = xf ? L.vbx[0] : 0.f, vby_x = xf ? L.vbx[1] : 0.f;
    const float vbz_x = xf ? L.vbx[2] : 0.f;
    const float vbx_y = yf ? L.vby[0] : 0.f, vby_y = yf ? L.vby[1] : 0.f;
    const float vbz_y = yf ? L.vby[2] : 0.f;
    const float vbx_z = zf ? L.vbz[0] : 0.f, vby_z = zf ? L.vbz[1] : 0.f;
    const float vbz_z = zf ? L.vbz[2] : 0.f;
    const float e[6] = {vbx_x - vb[0], vby_y - vb[1], vbz_z - vb[2],
                        ((vby_x - vb[1]) + (vbx_y - vb[0])) * 0.5f,
                        ((vbz_x - vb[2]) + (vbx_z - vb[0])) * 0.5f,
                        ((vbz_y - vb[2]) + (vby_z - vb[1])) * 0.5f};
    float yq[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) yq[k] = __fmaf_rn(a.sigma, e[k], P.sq[k]);
    float sq = yq[0] * yq[0] + yq[1] * yq[1] + 2.f * yq[3] * yq[3];
    sq = sq + yq[2] * yq[2] + 2.f * yq[4] * yq[4] + 2.f * yq[5] * yq[5];
    const float nq = sqrtf(sq);
    if (fmaxf(1.f, nq / a.alpha0) > 1.f) {
        float yg = 0.f;
#pragma unroll
        for (int k = 0; k < 6; ++k) yg += yq[k] * qa[k];
        const float s = a.alpha0 / nq, s3 = s / (nq * nq);
#pragma unroll
        for (int k = 0; k < 6; ++k) qa[k] = s * qa[k] - s3 * (k < 3 ? 1.f : 2.f) * yq[k] * yg;
        ga0 += yg / nq;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) a.A.p[c][i] = pa[c];
#pragma unroll
    for (int k = 0; k < 6; ++k) a.A.q[k][i] = qa[k];
}

// The in-plane loads of R2 (the z neighbours are set by the caller).
__device__ __forceinline__ void r2_load(const AdjArgs& a, size_t i, bool xl, bool yl, bool xf,
                                        bool yf, R2In& L) {
    const size_t W = a.W;
    L.utx = xl ? a.uta[i + 1] : 0.f;
    L.uty = yl ? a.uta[i + W] : 0.f;
    L.ubx = xl ? a.S.ubar[i + 1] : 0.f;
    L.uby = yl ? a.S.ubar[i + W] : 0.f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        L.va0[c] = a.va[c][i];
        L.vax[c] = xf ? a.va[c][i - 1] : 0.f;
        L.vay[c] = yf ? a.va[c][i - W] : 0.f;
        L.vb0[c] = a.S.vbar[c][i];
        L.vbx[c] = xf ? a.S.vbar[c][i - 1] : 0.f;
        L.vby[c] = yf ? a.S.vbar[c][i - W] : 0.f;
    }
}

// R2 one voxel per thread (small volumes).
__global__ void __launch_bounds__(BX* BY) adjoint_r2(AdjArgs a) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
    const int z = blockIdx.z;
    float ga0 = 0.f, ga1 = 0.f;
    const size_t i = ((size_t)z * a.H + y) * a.W + x, WH = a.WH;
    if (x < a.W && y < a.H && TGV_IN_BOUNDS(i, WH * a.D, 33)) {
        const bool xl = x + 1 < a.W, yl = y + 1 < a.H, zl = z + 1 < a.D;
        const bool xf = x > 0, yf = y > 0, zf = z > 0;
        R2In L;
        r2_load(a, i, xl, yl, xf, yf, L);
        L.ut0 = a.uta[i];
        L.utz = zl ? a.uta[i + WH] : 0.f;
        L.u0 = a.S.ubar[i];
        L.ubz = zl ? a.S.ubar[i + WH] : 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            L.vaz[c] = zf ? a.va[c][i - WH] : 0.f;
            L.vbz[c] = zf ? a.S.vbar[c][i - WH] : 0.f;
        }
        R2Pw P;
        r2_pw_load(a, i, P);
        r2_vals(a, i, P, xl, yl, zl, xf, yf, zf, L, ga0, ga1);
    }
    block_add(&a.gp[1], ga0);
    block_add(&a.gp[2], ga1);
}

// R2 marching a.zm planes per thread: the fields prefetched into L2 ZPF planes ahead,
// the pointwise fields of the next plane queued in registers.
__global__ void __launch_bounds__(BX* BY, 3) adjoint_r2_zm(AdjArgs a) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
    const int z0 = (int)blockIdx.z * a.zm, z1 = min(a.D, z0 + a.zm);
    float ga0 = 0.f, ga1 = 0.f;
    const size_t n = a.WH * a.D, i0 = ((size_t)z0 * a.H + y) * a.W + x;
    if (x < a.W && y < a.H && TGV_IN_BOUNDS(i0, n, 34) &&
        TGV_IN_BOUNDS(i0 + (size_t)(z1 - 1 - z0) * a.WH, n, 35)) {
        const size_t W = a.W, WH = a.WH;
        const bool xl = x + 1 < a.W, yl = y + 1 < a.H, xf = x > 0, yf = y > 0;
        size_t i = ((size_t)z0 * a.H + y) * W + x;
        auto prefetch_plane = [&](int z) {
            if (z >= a.D) return;
            const size_t j = ((size_t)z * a.H + y) * W + x;
            prefetch_l2(a.uta + j);
            prefetch_l2(a.S.ubar + j);
            for (int c = 0; c < 3; ++c) {
                prefetch_l2(a.va[c] + j);
                prefetch_l2(a.S.vbar[c] + j);
                prefetch_l2(a.A.p[c] + j);
                prefetch_l2(a.S.p[c] + j);
            }
            for (int k = 0; k < 6; ++k) {
                prefetch_l2(a.A.q[k] + j);
                prefetch_l2(a.S.q[k] + j);
            }
        };
        for (int k = 1; k < ZPF; ++k) prefetch_plane(z0 + k);
        // carried: a(u~) and ubar of this plane, a(v') and vbar of the plane below
        R2In L;
        L.ut0 = a.uta[i];
        L.u0 = a.S.ubar[i];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            L.vaz[c] = z0 > 0 ? a.va[c][i - WH] : 0.f;
            L.vbz[c] = z0 > 0 ? a.S.vbar[c][i - WH] : 0.f;
        }
        R2Pw P, Pn;
        r2_pw_load(a, i, P);
        for (int z = z0; z < z1; ++z, i += WH) {
            prefetch_plane(z + ZPF);
            if (z + 1 < z1) r2_pw_load(a, i + WH, Pn);
            const bool zl = z + 1 < a.D, zf = z > 0;
            r2_load(a, i, xl, yl, xf, yf, L);
            L.utz = zl ? a.uta[i + WH] : 0.f;
            L.ubz = zl ? a.S.ubar[i + WH] : 0.f;
            r2_vals(a, i, P, xl, yl, zl, xf, yf, zf, L, ga0, ga1);
            P = Pn;
            L.ut0 = L.utz;
            L.u0 = L.ubz;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                L.vaz[c] = L.va0[c];
                L.vbz[c] = L.vb0[c];
            }
        }
    }
    block_add(&a.gp[1], ga0);
    block_add(&a.gp[2], ga1);
}

__global__ void finish_grad_f(float* gf, const float* au, const float* aub, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        gf[i] += au[i] + aub[i];  // u_0 = ubar_0 = f
}

size_t a256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

uint64_t adjoint_bounds_take() {
    unsigned long long w = 0;
    TGV_CUDA(cudaMemcpyFromSymbol(&w, g_bounds_adj, sizeof(w)));
    if (w) {
        const unsigned long long zero = 0;
        TGV_CUDA(cudaMemcpyToSymbol(g_bounds_adj, &zero, sizeof(zero)));
    }
    return w;
}

namespace {

// Planes per thread: about (tiles x D) / (16 blocks per SM), between 1 and ZM_MAX.
int zm_for(const TgvState& s) {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        sms = 152;
    }
    const long long tiles = (long long)ceil_div(s.W, BX) * ceil_div(s.H, BY);
    const long long zm = tiles * s.D / (16LL * sms);
    return (int)std::max(1LL, std::min<long long>(ZM_MAX, zm));
}

}  // namespace

size_t tgv_full_state_bytes(size_t n) { return 17 * a256(n * 4); }

void tgv_full_state_bind(TgvFullDev& s, char* base, size_t n) {
    const size_t b = a256(n * 4);
    char* c = base;
    auto take = [&]() {
        float* r = (float*)c;
        c += b;
        return r;
    };
    s.u = take();
    s.ubar = take();
    for (int k = 0; k < 3; ++k) s.v[k] = take();
    for (int k = 0; k < 3; ++k) s.vbar[k] = take();
    for (int k = 0; k < 3; ++k) s.p[k] = take();
    for (int k = 0; k < 6; ++k) s.q[k] = take();
}

void tgv_full_state_zero(const TgvFullDev& s, size_t n, cudaStream_t st) {
    // the 17 fields are contiguous (tgv_full_state_bind)
    TGV_CUDA(cudaMemsetAsync(s.u, 0, tgv_full_state_bytes(n), st));
}

void tgv_adjoint_segment(const TgvState& s, const TgvStep& k, const TgvFullDev* states,
                         int len, const TgvFullDev& A, float* uta, float* const* va,
                         float* grad_f, double* gp, cudaStream_t st) {
    AdjArgs a;
    a.W = s.W;
    a.H = s.H;
    a.D = s.D;
    a.WH = (size_t)s.W * s.H;
    a.f = s.f;
    a.A = A;
    a.uta = uta;
    for (int c = 0; c < 3; ++c) a.va[c] = va[c];
    a.grad_f = grad_f;
    a.gp = gp;
    a.tau = k.tau;
    a.sigma = k.sigma;
    a.theta = k.theta;
    a.tau_lambda = k.tau * k.lambda;
    a.alpha0 = k.alpha0;
    a.alpha1 = k.alpha1;
    a.data_term = k.data_term;
    a.skip_bz = (k.data_term == TGVDCT_DATA_L2 && s.D == 1) ? 1 : 0;
    const dim3 block(BX, BY, 1);
    const dim3 grid(ceil_div(s.W, BX), ceil_div(s.H, BY), s.D);
    a.zm = zm_for(s);
    const dim3 zgrid(ceil_div(s.W, BX), ceil_div(s.H, BY), ceil_div(s.D, a.zm));
    // R3.R1 block rows: the widest of 256, 128, 32 voxels that W fills
    const int tbx = s.W >= 256 ? 256 : (s.W >= 128 ? 128 : 32);
    const dim3 rblock(tbx, BX * BY / tbx, 1);
    const dim3 rgrid(ceil_div(s.W, tbx), ceil_div(s.H, BX * BY / tbx), s.D);
    // iteration j of the segment maps states[j] -> states[j + 1]
    a.S = states[len - 1];
    a.S1 = states[len];
    adjoint_r1<<<grid, block, 0, st>>>(a);
    for (int j = len - 1; j >= 0; --j) {
        a.S = states[j];
        a.S1 = states[j + 1];
        if (a.zm > 1) adjoint_r2_zm<<<zgrid, block, 0, st>>>(a);
        else adjoint_r2<<<grid, block, 0, st>>>(a);
        if (j > 0) {
            a.S = states[j - 1];
            a.S1 = states[j];
            if (tbx == 256) adjoint_r3r1<256><<<rgrid, rblock, 0, st>>>(a);
            else if (tbx == 128) adjoint_r3r1<128><<<rgrid, rblock, 0, st>>>(a);
            else adjoint_r3r1<32><<<rgrid, rblock, 0, st>>>(a);
        } else {
            adjoint_r3<<<grid, block, 0, st>>>(a);
        }
    }
    TGV_CHECK_LAUNCH();
}

void tgv_adjoint_finish(float* grad_f, const TgvFullDev& A, size_t n, cudaStream_t st) {
    size_t b = (n + 255) / 256;
    if (b > 152 * 32) b = 152 * 32;
    finish_grad_f<<<(unsigned)(b ? b : 1), 256, 0, st>>>(grad_f, A.u, A.ubar, n);
    TGV_CHECK_LAUNCH();
}

}  // namespace tgvdct
