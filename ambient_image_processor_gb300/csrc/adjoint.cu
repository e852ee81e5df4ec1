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
// the adjoint moves 63 fields (252 bytes).  For large volumes R2 of iteration k-1 joins
// them (adjoint_fused), so that a(u~) and a(v') stay on chip as well: 44 fields
// (176 bytes).  An FP64 restatement of the same algebra in the oracle gives the
// reference gradient (central differences pin it).
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
    TgvFullDev Ao;  // the fused pass's output: a(u), a(v), a(p), a(q) of S_k (A is its input)
    float* uta;     // a(u~)
    float* va[3];   // a(v')
    float* grad_f;
    double* gp;     // d/dlambda, d/dalpha0, d/dalpha1
    float tau, sigma, theta, tau_lambda, alpha0, alpha1;
    int data_term, skip_bz;
    int zm;  // planes per thread of the z-marching kernels
    int zc;  // planes per block of the fused pass
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

// R1's u part at one voxel, from a(u) and a(ubar) of S_{k+1}: a(u~), the new a(u), the
// d/df term and the d/dlambda term.
struct R1U {
    float uta, au, gf, glam;
};
__device__ __forceinline__ R1U r1_u(const AdjArgs& a, const R1In& in, float au_in, float aub) {
    R1U o;
    o.glam = 0.f;
    o.gf = 0.f;
    // u~ exactly as the forward primal pass computed it
    const float bx = in.px - in.p0;
    const float by = in.py - in.p1;
    float div = bx + by;
    const float bz = in.pz - in.p2;
    if (!a.skip_bz) div = div + bz;
    const float ut = in.uo - a.tau * div;
    const float ua = au_in + (1.f + a.theta) * aub;
    float uta;
    if (a.data_term == TGVDCT_DATA_L1) {
        const float dd = ut - in.fi;
        if (dd > a.tau_lambda) {
            uta = ua;
            o.glam = -a.tau * ua;
        } else if (dd < -a.tau_lambda) {
            uta = ua;
            o.glam = a.tau * ua;
        } else {
            uta = 0.f;
            o.gf = ua;
        }
    } else {
        const float den = 1.f + a.tau_lambda;
        uta = ua / den;
        o.gf = a.tau_lambda * ua / den;
        o.glam = ua * a.tau * (in.fi - ut) / (den * den);
    }
    o.au = -a.theta * aub + uta;
    o.uta = uta;
    return o;
}
// R1's v part, one component: a(v') from a(v) and a(vbar) of S_{k+1}, then the new a(v).
__device__ __forceinline__ float r1_va(const AdjArgs& a, float av_in, float avb) {
    return av_in + (1.f + a.theta) * avb;
}
__device__ __forceinline__ float r1_av(const AdjArgs& a, float va, float avb) {
    return va - a.theta * avb;
}

// R1 at voxel i, with a(ubar) and a(vbar) of S_{k+1} given: returns the d/dlambda term.
__device__ __forceinline__ float r1_vals(const AdjArgs& a, size_t i, const R1In& in, float aub,
                                         const float* avb) {
    const R1U o = r1_u(a, in, a.A.u[i], aub);
    a.A.u[i] = o.au;
    a.uta[i] = o.uta;
    if (o.gf != 0.f) a.grad_f[i] += o.gf;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float va = r1_va(a, a.A.v[c][i], avb[c]);
        a.va[c][i] = va;
        a.A.v[c][i] = r1_av(a, va, avb[c]);
    }
    return o.glam;
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
// a(ubar) = sigma sum_c F_c^T a(p)_c (reads p0..p2 and px, py, pz)
__device__ __forceinline__ float r3_aub(const AdjArgs& a, bool xl, bool yl, bool zl,
                                        const R3In& in) {
    const float ftx = in.px - (xl ? in.p0 : 0.f);
    const float fty = in.py - (yl ? in.p1 : 0.f);
    const float ftz = in.pz - (zl ? in.p2 : 0.f);
    return a.sigma * ((ftx + fty) + ftz);
}
// a(vbar)_c = -sigma a(p)_c + sigma sum_a w B_a^T a(q)_{c a} (reads p0..p2 and the q values)
__device__ __forceinline__ void r3_avb(const AdjArgs& a, const R3In& in, float* avb) {
    const float* q = in.q;  // xx yy zz xy xz yz
    const float ex = (in.qx0 - q[0]) + 0.5f * (in.qy3 - q[3]) + 0.5f * (in.qz4 - q[4]);
    const float ey = 0.5f * (in.qx3 - q[3]) + (in.qy1 - q[1]) + 0.5f * (in.qz5 - q[5]);
    const float ez = 0.5f * (in.qx4 - q[4]) + 0.5f * (in.qy5 - q[5]) + (in.qz2 - q[2]);
    avb[0] = -a.sigma * in.p0 + a.sigma * ex;
    avb[1] = -a.sigma * in.p1 + a.sigma * ey;
    avb[2] = -a.sigma * in.p2 + a.sigma * ez;
}
__device__ __forceinline__ void r3_vals(const AdjArgs& a, bool xl, bool yl, bool zl,
                                        const R3In& in, float& aub, float* avb) {
    aub = r3_aub(a, xl, yl, zl, in);
    r3_avb(a, in, avb);
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

// R2 at voxel i: the projection Jacobians, written to `out`; accumulates d/dalpha0,
// d/dalpha1.
__device__ __forceinline__ void r2_vals(const AdjArgs& a, size_t i, const R2Pw& P, bool xl,
                                        bool yl, bool zl, bool xf, bool yf, bool zf,
                                        const R2In& L, float& ga0, float& ga1,
                                        const TgvFullDev& out) {
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
    for (int c = 0; c < 3; ++c) out.p[c][i] = pa[c];
#pragma unroll
    for (int k = 0; k < 6; ++k) out.q[k][i] = qa[k];
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
        r2_vals(a, i, P, xl, yl, zl, xf, yf, zf, L, ga0, ga1, a.A);
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
            r2_vals(a, i, P, xl, yl, zl, xf, yf, zf, L, ga0, ga1, a.A);
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

// ---- the fused pass: R3 of iteration k, then R1 and R2 of iteration k - 1 ----------
//
// R2 at voxel i reads a(u~) at i and its +x, +y, +z neighbours and a(v') at i and its
// -x, -y, -z neighbours, both made by R1 of the same iteration; R1 is pointwise in the
// a(ubar), a(vbar) that R3 of the iteration after makes.  One block owns a 32 x 8 column
// tile and marches its planes along z: at step s it runs R3.R1 on plane s and R2 on
// plane s - 1, so a(u~) and a(v') stay on chip (a three-plane shared ring for the
// in-plane neighbours, registers for the z neighbours).  Three more warps run the
// R3.R1 parts that the tile's R2 needs just outside it: a(u~) on the +x column and the
// +y row, a(v') on the -x column and the -y row.  A block's first step makes a(v') of
// the plane below its chunk and its last a(u~) of the plane above.  The pass reads the
// adjoint state A and writes a second one, Ao, because the rim threads read A at voxels
// that a neighbouring block updates.  Per voxel it moves 44 fields: A (13) and S_k.p (3),
// S_{k-1}'s u, ubar, vbar, p, q (14) and f read, Ao (13) written, d/df updated where
// the prox is inactive; R3.R1 and R2 as separate passes moved 61.  Each update is the
// same sequence of operations as in adjoint_r3r1 and adjoint_r2, so the results are
// bit-identical.
//
// Loads are plain global loads, each phase's issued before its first store (R2's before
// the plane barrier), with the fields of the next plane prefetched into L2.  The pass
// is bound by load latency at two blocks (22 warps) per SM: at 256 x 256 x 192 it takes
// 0.55 ms against 0.57 ms for R3.R1 and R2 as separate passes.  Staging the inputs in
// shared memory with per-thread 4-byte asynchronous copies (cp.async) was slower (0.89
// ms): the copies cost as many memory instructions as the loads and queued behind the
// shared-memory reads.
namespace fz {
constexpr int TX = 32, TY = 8;
constexpr int NTHREADS = TX * TY + 96;  // eight tile warps, three rim warps
constexpr int SX = TX + 1, SY = TY + 1;   // a plane of the tile with one rim row and column
constexpr int RING = 3;
enum Role { TILE, RIM_U, RIM_V, IDLE };
}  // namespace fz

// a(u~) at voxel i of A and S_{k-1} (R3's a(ubar) part, R1's u part), nothing stored.
__device__ __forceinline__ float fused_uta(const AdjArgs& a, size_t i, bool xf, bool yf,
                                           bool zf, bool xl, bool yl, bool zl) {
    const size_t W = a.W, WH = a.WH;
    R3In r3;
    r3.p0 = a.A.p[0][i];
    r3.p1 = a.A.p[1][i];
    r3.p2 = a.A.p[2][i];
    r3.px = xf ? a.A.p[0][i - 1] : 0.f;
    r3.py = yf ? a.A.p[1][i - W] : 0.f;
    r3.pz = zf ? a.A.p[2][i - WH] : 0.f;
    const float aub = r3_aub(a, xl, yl, zl, r3);
    R1In r1;
    r1_load(a, i, xf, yf, r1);
    r1.pz = zf ? a.S1.p[2][i - WH] : 0.f;
    return r1_u(a, r1, a.A.u[i], aub).uta;
}

// a(v') at voxel i (R3's a(vbar) part, R1's v part), nothing stored.
__device__ __forceinline__ void fused_va(const AdjArgs& a, size_t i, bool xl, bool yl, bool zl,
                                         float* va) {
    const size_t W = a.W, WH = a.WH;
    const float* const* P = a.A.p;
    const float* const* Q = a.A.q;
    R3In r3;
    r3.p0 = P[0][i];
    r3.p1 = P[1][i];
    r3.p2 = P[2][i];
#pragma unroll
    for (int k = 0; k < 6; ++k) r3.q[k] = Q[k][i];
    r3.qx0 = xl ? Q[0][i + 1] : 0.f;
    r3.qx3 = xl ? Q[3][i + 1] : 0.f;
    r3.qx4 = xl ? Q[4][i + 1] : 0.f;
    r3.qy3 = yl ? Q[3][i + W] : 0.f;
    r3.qy1 = yl ? Q[1][i + W] : 0.f;
    r3.qy5 = yl ? Q[5][i + W] : 0.f;
    r3.qz4 = zl ? Q[4][i + WH] : 0.f;
    r3.qz5 = zl ? Q[5][i + WH] : 0.f;
    r3.qz2 = zl ? Q[2][i + WH] : 0.f;
    float avb[3];
    r3_avb(a, r3, avb);
#pragma unroll
    for (int c = 0; c < 3; ++c) va[c] = r1_va(a, a.A.v[c][i], avb[c]);
}

// The fields a tile thread reads at plane z, prefetched into L2 one plane ahead.
__device__ __forceinline__ void fused_prefetch(const AdjArgs& a, uint32_t j) {
    prefetch_l2(a.A.u + j);
    prefetch_l2(a.S.u + j);
    prefetch_l2(a.f + j);
    prefetch_l2(a.grad_f + j);
    prefetch_l2(a.S.ubar + j);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        prefetch_l2(a.A.v[c] + j);
        prefetch_l2(a.A.p[c] + j);
        prefetch_l2(a.S1.p[c] + j);
        prefetch_l2(a.S.vbar[c] + j);
        prefetch_l2(a.S.p[c] + j);
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        prefetch_l2(a.A.q[k] + j);
        prefetch_l2(a.S.q[k] + j);
    }
}

__global__ void __launch_bounds__(fz::NTHREADS, 2) adjoint_fused(AdjArgs a) {
    __shared__ float s_ut[fz::RING][fz::SY][fz::SX];     // a(u~) at (tx, ty), tx, ty >= 0
    __shared__ float s_va[fz::RING][3][fz::SY][fz::SX];  // a(v') at (tx + 1, ty + 1)
    const int w = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    fz::Role role;
    int tx = lane, ty = w;
    if (w < fz::TY) {
        role = fz::TILE;
    } else if (w == fz::TY) {
        role = fz::RIM_U;
        ty = fz::TY;
    } else if (w == fz::TY + 1) {
        role = fz::RIM_V;
        ty = -1;
    } else if (lane < fz::TY) {
        role = fz::RIM_U;
        tx = fz::TX;
        ty = lane;
    } else if (lane < 2 * fz::TY) {
        role = fz::RIM_V;
        tx = -1;
        ty = lane - fz::TY;
    } else {
        role = fz::IDLE;
        tx = 0;
        ty = 0;
    }
    const int W = a.W, H = a.H, D = a.D;
    const int x = (int)blockIdx.x * fz::TX + tx, y = (int)blockIdx.y * fz::TY + ty;
    const int z0 = (int)blockIdx.z * a.zc, z1 = min(D, z0 + a.zc);
    const bool inside = role != fz::IDLE && x >= 0 && x < W && y >= 0 && y < H;
    const bool tile = role == fz::TILE && inside;
    const bool xl = x + 1 < W, yl = y + 1 < H, xf = x > 0, yf = y > 0;
    const uint32_t WH = (uint32_t)a.WH, n = WH * (uint32_t)D;
    // the voxel (x, y) of plane z (meaningful where `inside`)
    auto at = [&](int z) {
        return ((uint32_t)z * (uint32_t)H + (uint32_t)y) * (uint32_t)W + (uint32_t)x;
    };
    float glam = 0.f, ga0 = 0.f, ga1 = 0.f;
    float va_m1[3] = {0.f, 0.f, 0.f}, va_m2[3] = {0.f, 0.f, 0.f};  // a(v') at s - 1, s - 2
    if (tile && z0 - 1 >= 0 && TGV_IN_BOUNDS(at(z0 - 1), n, 44)) fused_prefetch(a, at(z0 - 1));
    if (tile && TGV_IN_BOUNDS(at(z0), n, 44)) fused_prefetch(a, at(z0));
    for (int s = z0 - 1; s <= z1; ++s) {
        const int slot = (s - z0 + 1) % fz::RING;
        float ut_s = 0.f, va_s[3] = {0.f, 0.f, 0.f};  // a(u~), a(v') at (x, y, s)
        if (tile && s + 1 <= z1 && s + 1 < D && TGV_IN_BOUNDS(at(s + 1), n, 44))
            fused_prefetch(a, at(s + 1));
        if (s >= 0 && s < D) {
            const uint32_t i = at(s);
            const bool zl = s + 1 < D, zf = s > 0;
            const bool own = s >= z0 && s < z1;
            if (role == fz::TILE) {
                if (inside && TGV_IN_BOUNDS(i, n, 40)) {
                    if (own) {
                        // R3 of iteration k and R1 of iteration k - 1, stored to Ao; every
                        // load comes before the first store
                        R3In r3;
                        r3_load(a, i, xf, yf, xl, yl, r3);
                        r3.pz = zf ? a.A.p[2][i - WH] : 0.f;
                        r3.qz4 = zl ? a.A.q[4][i + WH] : 0.f;
                        r3.qz5 = zl ? a.A.q[5][i + WH] : 0.f;
                        r3.qz2 = zl ? a.A.q[2][i + WH] : 0.f;
                        R1In r1;
                        r1_load(a, i, xf, yf, r1);
                        r1.pz = zf ? a.S1.p[2][i - WH] : 0.f;
                        const float au_in = a.A.u[i];
                        float av_in[3];
#pragma unroll
                        for (int c = 0; c < 3; ++c) av_in[c] = a.A.v[c][i];
                        const float gf_in = a.grad_f[i];
                        float aub, avb[3];
                        r3_vals(a, xl, yl, zl, r3, aub, avb);
                        const R1U o = r1_u(a, r1, au_in, aub);
                        ut_s = o.uta;
                        glam += o.glam;
                        float av_out[3];
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            va_s[c] = r1_va(a, av_in[c], avb[c]);
                            av_out[c] = r1_av(a, va_s[c], avb[c]);
                        }
                        a.Ao.u[i] = o.au;
#pragma unroll
                        for (int c = 0; c < 3; ++c) a.Ao.v[c][i] = av_out[c];
                        if (o.gf != 0.f) a.grad_f[i] = gf_in + o.gf;
                    } else if (s < z0) {
                        fused_va(a, i, xl, yl, zl, va_s);  // the plane below the chunk
                    } else {
                        ut_s = fused_uta(a, i, xf, yf, zf, xl, yl, zl);  // the plane above
                    }
                }
                s_ut[slot][ty][tx] = ut_s;
#pragma unroll
                for (int c = 0; c < 3; ++c) s_va[slot][c][ty + 1][tx + 1] = va_s[c];
            } else if (role == fz::RIM_U && own) {
                float u = 0.f;
                if (inside && TGV_IN_BOUNDS(i, n, 41)) u = fused_uta(a, i, xf, yf, zf, xl, yl, zl);
                s_ut[slot][ty][tx] = u;
            } else if (role == fz::RIM_V && own) {
                float v[3] = {0.f, 0.f, 0.f};
                if (inside && TGV_IN_BOUNDS(i, n, 42)) fused_va(a, i, xl, yl, zl, v);
#pragma unroll
                for (int c = 0; c < 3; ++c) s_va[slot][c][ty + 1][tx + 1] = v[c];
            }
        }
        // R2 of iteration k - 1 on plane t = s - 1: its global loads before the plane
        // barrier, its a(u~), a(v') neighbours from the ring after it
        const int t = s - 1;
        const bool r2 = tile && t >= z0 && t < z1 && TGV_IN_BOUNDS(at(t), n, 43);
        const bool zl = t + 1 < D, zf = t > 0;
        R2In L;
        R2Pw P;
        if (r2) {
            const uint32_t i = at(t);
            L.u0 = a.S.ubar[i];
            L.ubx = xl ? a.S.ubar[i + 1] : 0.f;
            L.uby = yl ? a.S.ubar[i + W] : 0.f;
            L.ubz = zl ? a.S.ubar[i + WH] : 0.f;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                L.vb0[c] = a.S.vbar[c][i];
                L.vbx[c] = xf ? a.S.vbar[c][i - 1] : 0.f;
                L.vby[c] = yf ? a.S.vbar[c][i - W] : 0.f;
                L.vbz[c] = zf ? a.S.vbar[c][i - WH] : 0.f;
            }
            r2_pw_load(a, i, P);
        }
        __syncthreads();
        if (r2) {
            const int ts = (t - z0 + 1) % fz::RING;
            L.ut0 = s_ut[ts][ty][tx];
            L.utx = xl ? s_ut[ts][ty][tx + 1] : 0.f;
            L.uty = yl ? s_ut[ts][ty + 1][tx] : 0.f;
            L.utz = zl ? ut_s : 0.f;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                L.va0[c] = s_va[ts][c][ty + 1][tx + 1];
                L.vax[c] = xf ? s_va[ts][c][ty + 1][tx] : 0.f;
                L.vay[c] = yf ? s_va[ts][c][ty][tx + 1] : 0.f;
                L.vaz[c] = zf ? va_m2[c] : 0.f;
            }
            r2_vals(a, at(t), P, xl, yl, zl, xf, yf, zf, L, ga0, ga1, a.Ao);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            va_m2[c] = va_m1[c];
            va_m1[c] = va_s[c];
        }
    }
    block_add(&a.gp[0], glam);
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

int sm_count() {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        sms = 152;
    }
    return sms;
}

// Planes per thread: about (tiles x D) / (16 blocks per SM), between 1 and ZM_MAX.
int zm_for(const TgvState& s) {
    const int sms = sm_count();
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
                         int len, AdjointPasses passes, TgvFullDev& A, TgvFullDev& A2,
                         float* uta, float* const* va, float* grad_f, double* gp,
                         cudaStream_t st) {
    AdjArgs a;
    a.W = s.W;
    a.H = s.H;
    a.D = s.D;
    a.WH = (size_t)s.W * s.H;
    a.f = s.f;
    a.A = A;
    a.Ao = A2;
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
    // the fused pass's z-chunk: the iteration kernels' (same tile, two blocks per SM)
    a.zc = s.zchunk > 0 ? std::min(s.zchunk, s.D) : s.D;
    const dim3 fgrid(ceil_div(s.W, fz::TX), ceil_div(s.H, fz::TY), ceil_div(s.D, a.zc));
    // the fused pass indexes voxels in 32 bits
    const size_t fblocks = (size_t)fgrid.x * fgrid.y * fgrid.z;
    const bool fused = a.WH * (size_t)s.D < (size_t(1) << 32) &&
                       (passes == ADJ_FUSED ||
                        (passes == ADJ_FUSED_LARGE && fblocks >= 3 * 2 * (size_t)sm_count()));
    // R3.R1 block rows: the widest of 256, 128, 32 voxels that W fills
    const int tbx = s.W >= 256 ? 256 : (s.W >= 128 ? 128 : 32);
    const dim3 rblock(tbx, BX * BY / tbx, 1);
    const dim3 rgrid(ceil_div(s.W, tbx), ceil_div(s.H, BX * BY / tbx), s.D);
    auto r2 = [&] {
        if (a.zm > 1) adjoint_r2_zm<<<zgrid, block, 0, st>>>(a);
        else adjoint_r2<<<grid, block, 0, st>>>(a);
    };
    // iteration j of the segment maps states[j] -> states[j + 1]
    a.S = states[len - 1];
    a.S1 = states[len];
    adjoint_r1<<<grid, block, 0, st>>>(a);
    r2();
    for (int j = len - 1; j > 0; --j) {
        a.S = states[j - 1];
        a.S1 = states[j];
        if (fused) {
            // R3 of iteration j, R1 and R2 of iteration j - 1, from A into A2
            a.A = A;
            a.Ao = A2;
            adjoint_fused<<<fgrid, fz::NTHREADS, 0, st>>>(a);
            std::swap(A, A2);
            a.A = A;
        } else {
            if (tbx == 256) adjoint_r3r1<256><<<rgrid, rblock, 0, st>>>(a);
            else if (tbx == 128) adjoint_r3r1<128><<<rgrid, rblock, 0, st>>>(a);
            else adjoint_r3r1<32><<<rgrid, rblock, 0, st>>>(a);
            r2();
        }
    }
    adjoint_r3<<<grid, block, 0, st>>>(a);
    TGV_CHECK_LAUNCH();
}

void tgv_adjoint_finish(float* grad_f, const TgvFullDev& A, size_t n, cudaStream_t st) {
    size_t b = (n + 255) / 256;
    if (b > 152 * 32) b = 152 * 32;
    finish_grad_f<<<(unsigned)(b ? b : 1), 256, 0, st>>>(grad_f, A.u, A.ubar, n);
    TGV_CHECK_LAUNCH();
}

}  // namespace tgvdct
