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
#include "common.cuh"

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
};

__device__ __forceinline__ void block_add(double* dst, float v) {
    __shared__ float red[BX * BY / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int t = threadIdx.y * BX + threadIdx.x;
    if ((t & 31) == 0) red[t >> 5] = v;
    __syncthreads();
    if (t == 0) {
        float s = 0.f;
        for (int w = 0; w < BX * BY / 32; ++w) s += red[w];
        if (s != 0.f) atomicAdd(dst, (double)s);
    }
    __syncthreads();
}

// R1 at voxel i, with a(ubar) and a(vbar) of S_{k+1} given: returns the d/dlambda term.
__device__ __forceinline__ float r1_at(const AdjArgs& a, int x, int y, int z, size_t i,
                                       float aub, const float* avb) {
    const size_t W = a.W, WH = a.WH;
    float glam = 0.f;
    // u~ exactly as the forward primal pass computed it
    const float pxi = a.S1.p[0][i], pyi = a.S1.p[1][i], pzi = a.S1.p[2][i];
    const float bx = (x > 0 ? a.S1.p[0][i - 1] : 0.f) - pxi;
    const float by = (y > 0 ? a.S1.p[1][i - W] : 0.f) - pyi;
    float div = bx + by;
    const float bz = (z > 0 ? a.S1.p[2][i - WH] : 0.f) - pzi;
    if (!a.skip_bz) div = div + bz;
    const float uo = a.S.u[i], fi = a.f[i];
    const float ut = uo - a.tau * div;
    const float ua = a.A.u[i] + (1.f + a.theta) * aub;
    float uta, gf = 0.f;
    if (a.data_term == TGVDCT_DATA_L1) {
        const float dd = ut - fi;
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
        glam = ua * a.tau * (fi - ut) / (den * den);
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

// R3 at voxel i: a(ubar) and a(vbar) of S_k from a(p), a(q) (after R2).
__device__ __forceinline__ void r3_at(const AdjArgs& a, int x, int y, int z, size_t i,
                                      float& aub, float* avb) {
    const size_t W = a.W, WH = a.WH;
    const bool xl = x + 1 < a.W, yl = y + 1 < a.H, zl = z + 1 < a.D;
    const bool xf = x > 0, yf = y > 0, zf = z > 0;
    // a(ubar) = sigma sum_c F_c^T a(p)_c
    const float* P0 = a.A.p[0];
    const float* P1 = a.A.p[1];
    const float* P2 = a.A.p[2];
    const float p0 = P0[i], p1 = P1[i], p2 = P2[i];
    const float ftx = (xf ? P0[i - 1] : 0.f) - (xl ? p0 : 0.f);
    const float fty = (yf ? P1[i - W] : 0.f) - (yl ? p1 : 0.f);
    const float ftz = (zf ? P2[i - WH] : 0.f) - (zl ? p2 : 0.f);
    aub = a.sigma * ((ftx + fty) + ftz);
    // a(vbar)_c = -sigma a(p)_c + sigma sum_a w B_a^T a(q)_{c a}
    auto bt = [&](const float* g, int axis) {
        const float g0 = g[i];
        if (axis == 0) return (xl ? g[i + 1] : 0.f) - g0;
        if (axis == 1) return (yl ? g[i + W] : 0.f) - g0;
        return (zl ? g[i + WH] : 0.f) - g0;
    };
    const float* const* Q = a.A.q;  // xx yy zz xy xz yz
    const float ex = bt(Q[0], 0) + 0.5f * bt(Q[3], 1) + 0.5f * bt(Q[4], 2);
    const float ey = 0.5f * bt(Q[3], 0) + bt(Q[1], 1) + 0.5f * bt(Q[5], 2);
    const float ez = 0.5f * bt(Q[4], 0) + 0.5f * bt(Q[5], 1) + bt(Q[2], 2);
    avb[0] = -a.sigma * p0 + a.sigma * ex;
    avb[1] = -a.sigma * p1 + a.sigma * ey;
    avb[2] = -a.sigma * p2 + a.sigma * ez;
}

__global__ void __launch_bounds__(BX* BY) adjoint_r1(AdjArgs a) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
    const int z = blockIdx.z;
    float glam = 0.f;
    if (x < a.W && y < a.H) {
        const size_t i = ((size_t)z * a.H + y) * a.W + x;
        const float avb[3] = {a.A.vbar[0][i], a.A.vbar[1][i], a.A.vbar[2][i]};
        glam = r1_at(a, x, y, z, i, a.A.ubar[i], avb);
    }
    block_add(&a.gp[0], glam);
}

// R3 of iteration k followed by R1 of iteration k-1 (S = S_{k-1}, S1 = S_k): a(ubar)
// and a(vbar) stay in registers.
__global__ void __launch_bounds__(BX* BY) adjoint_r3r1(AdjArgs a) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
    const int z = blockIdx.z;
    float glam = 0.f;
    if (x < a.W && y < a.H) {
        const size_t i = ((size_t)z * a.H + y) * a.W + x;
        float aub, avb[3];
        r3_at(a, x, y, z, i, aub, avb);
        glam = r1_at(a, x, y, z, i, aub, avb);
    }
    block_add(&a.gp[0], glam);
}

__global__ void __launch_bounds__(BX* BY) adjoint_r2(AdjArgs a) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
    const int z = blockIdx.z;
    float ga0 = 0.f, ga1 = 0.f;
    if (x < a.W && y < a.H) {
        const size_t W = a.W, WH = a.WH, i = ((size_t)z * a.H + y) * W + x;
        const bool xl = x + 1 < a.W, yl = y + 1 < a.H, zl = z + 1 < a.D;
        const bool xf = x > 0, yf = y > 0, zf = z > 0;
        // a(p') = a(p) + tau a(v') - tau B^T a(u~)
        const float ut0 = a.uta[i];
        const float bt[3] = {(xl ? a.uta[i + 1] : 0.f) - ut0, (yl ? a.uta[i + W] : 0.f) - ut0,
                             (zl ? a.uta[i + WH] : 0.f) - ut0};
        float pa[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            pa[c] = a.A.p[c][i] + a.tau * a.va[c][i];
            if (!(c == 2 && a.skip_bz)) pa[c] = pa[c] - a.tau * bt[c];
        }
        // a(q') = a(q) - tau divF^T a(v'): (F_a^T g)[i] = g[i-e] (if >= 1) - g[i] (if < N-1)
        float fx[3], fy[3], fz[3];  // F_a^T va_c
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float* g = a.va[c];
            const float g0 = g[i];
            fx[c] = (xf ? g[i - 1] : 0.f) - (xl ? g0 : 0.f);
            fy[c] = (yf ? g[i - W] : 0.f) - (yl ? g0 : 0.f);
            fz[c] = (zf ? g[i - WH] : 0.f) - (zl ? g0 : 0.f);
        }
        float qa[6];  // xx yy zz xy xz yz
        qa[0] = a.A.q[0][i] - a.tau * fx[0];
        qa[1] = a.A.q[1][i] - a.tau * fy[1];
        qa[2] = a.A.q[2][i] - a.tau * fz[2];
        qa[3] = a.A.q[3][i] - a.tau * (fy[0] + fx[1]);
        qa[4] = a.A.q[4][i] - a.tau * (fz[0] + fx[2]);
        qa[5] = a.A.q[5][i] - a.tau * (fz[1] + fy[2]);
        // y_p of the forward dual pass, bit for bit
        const float* ub = a.S.ubar;
        const float u0 = ub[i];
        const float gx = xl ? ub[i + 1] - u0 : 0.f;
        const float gy = yl ? ub[i + W] - u0 : 0.f;
        const float gz = zl ? ub[i + WH] - u0 : 0.f;
        const float vb[3] = {a.S.vbar[0][i], a.S.vbar[1][i], a.S.vbar[2][i]};
        const float yp[3] = {__fmaf_rn(a.sigma, gx - vb[0], a.S.p[0][i]),
                             __fmaf_rn(a.sigma, gy - vb[1], a.S.p[1][i]),
                             __fmaf_rn(a.sigma, gz - vb[2], a.S.p[2][i])};
        const float np = norm3df(yp[0], yp[1], yp[2]);
        if (fmaxf(1.f, np / a.alpha1) > 1.f) {
            const float yg = yp[0] * pa[0] + yp[1] * pa[1] + yp[2] * pa[2];
            const float s = a.alpha1 / np, s3 = s / (np * np);
#pragma unroll
            for (int c = 0; c < 3; ++c) pa[c] = s * pa[c] - s3 * yp[c] * yg;
            ga1 = yg / np;
        }
        // y_q of the forward dual pass, bit for bit
        const float vbx_x = xf ? a.S.vbar[0][i - 1] : 0.f, vby_x = xf ? a.S.vbar[1][i - 1] : 0.f;
        const float vbz_x = xf ? a.S.vbar[2][i - 1] : 0.f;
        const float vbx_y = yf ? a.S.vbar[0][i - W] : 0.f, vby_y = yf ? a.S.vbar[1][i - W] : 0.f;
        const float vbz_y = yf ? a.S.vbar[2][i - W] : 0.f;
        const float vbx_z = zf ? a.S.vbar[0][i - WH] : 0.f, vby_z = zf ? a.S.vbar[1][i - WH] : 0.f;
        const float vbz_z = zf ? a.S.vbar[2][i - WH] : 0.f;
        const float e[6] = {vbx_x - vb[0], vby_y - vb[1], vbz_z - vb[2],
                            ((vby_x - vb[1]) + (vbx_y - vb[0])) * 0.5f,
                            ((vbz_x - vb[2]) + (vbx_z - vb[0])) * 0.5f,
                            ((vbz_y - vb[2]) + (vby_z - vb[1])) * 0.5f};
        float yq[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) yq[k] = __fmaf_rn(a.sigma, e[k], a.S.q[k][i]);
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
            ga0 = yg / nq;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) a.A.p[c][i] = pa[c];
#pragma unroll
        for (int k = 0; k < 6; ++k) a.A.q[k][i] = qa[k];
    }
    block_add(&a.gp[1], ga0);
    block_add(&a.gp[2], ga1);
}

__global__ void __launch_bounds__(BX* BY) adjoint_r3(AdjArgs a) {
    const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= a.W || y >= a.H) return;
    const size_t i = ((size_t)z * a.H + y) * a.W + x;
    float aub, avb[3];
    r3_at(a, x, y, z, i, aub, avb);
    a.A.ubar[i] = aub;
#pragma unroll
    for (int c = 0; c < 3; ++c) a.A.vbar[c][i] = avb[c];
}

__global__ void finish_grad_f(float* gf, const float* au, const float* aub, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        gf[i] += au[i] + aub[i];  // u_0 = ubar_0 = f
}

size_t a256(size_t b) { return (b + 255) & ~size_t(255); }

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
    // iteration j of the segment maps states[j] -> states[j + 1]
    a.S = states[len - 1];
    a.S1 = states[len];
    adjoint_r1<<<grid, block, 0, st>>>(a);
    for (int j = len - 1; j >= 0; --j) {
        a.S = states[j];
        a.S1 = states[j + 1];
        adjoint_r2<<<grid, block, 0, st>>>(a);
        if (j > 0) {
            a.S = states[j - 1];
            a.S1 = states[j];
            adjoint_r3r1<<<grid, block, 0, st>>>(a);
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
