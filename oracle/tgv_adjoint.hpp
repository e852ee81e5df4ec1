// TEST INFRASTRUCTURE — FP64 unrolled reverse mode of the TGV2 loop (the reference
// gradient the CUDA adjoint is checked against).  Not product code.
//
// One iteration S_k -> S_{k+1} of the 3-D loop (tgv_deshade/tgv2_l1_deshade.cu:169-272,
// the arithmetic of tgv_oracle.hpp), state S = (u, ubar, v, vbar, p, q):
//   p' = P_a1(p + sigma (F ubar - vbar))          P: scale by 1 / max(1, |y| / a1)
//   q' = Q_a0(q + sigma E vbar)                    Q: same with the weighted norm
//                                                  |y|^2 = yxx^2+yyy^2+yzz^2+2(yxy^2+yxz^2+yyz^2)
//   u~ = u - tau B.p'                              B.p' = sum_c B_c p'_c
//   u' = prox(u~; f, tau lambda)                   L1 shrink toward f, or L2 average
//   ubar' = u' + theta (u' - u)
//   v' = v - tau (divF q' - p'),  vbar' = v' + theta (v' - v)
// with F (Neumann forward difference) and B (the reference's negated backward
// difference) as in tgv_oracle.hpp.  The adjoint step maps the adjoint of S_{k+1}
// to the adjoint of S_k and accumulates d/df, d/dlambda, d/dalpha0, d/dalpha1.
// Transposes: (F_a^T g)[j] = g[j-e] (j_a >= 1) - g[j] (j_a < N-1);
//             (B_a^T g)[j] = g[j+e] (j_a < N-1) - g[j].
// Projection Jacobians (active when |y| > a): J^T g = (a/n) g - (a/n^3) w.y (y.g),
// d P / d a = y / n; inactive: identity, 0.
#pragma once

#include <cmath>
#include <vector>

#include "tgv_oracle.hpp"

namespace oracle {

template <class T>
struct TgvFullState {
    std::vector<T> u, ub, v[3], vb[3], p[3], q[6];  // q: xx yy zz xy xz yz
    explicit TgvFullState(index_t n = 0) { resize(n); }
    void resize(index_t n) {
        u.assign(n, T(0));
        ub.assign(n, T(0));
        for (int c = 0; c < 3; ++c) v[c].assign(n, T(0)), vb[c].assign(n, T(0)), p[c].assign(n, T(0));
        for (int c = 0; c < 6; ++c) q[c].assign(n, T(0));
    }
};

template <class T>
void forward_transpose(int axis, const T* g, T* out, Dims d) {
    const index_t e = axis == 0 ? 1 : axis == 1 ? d.w : d.w * d.h;
    const index_t na = axis == 0 ? d.w : axis == 1 ? d.h : d.d;
#pragma omp parallel for schedule(static)
    for (index_t z = 0; z < d.d; ++z)
        for (index_t y = 0; y < d.h; ++y)
            for (index_t x = 0; x < d.w; ++x) {
                const index_t i = d.idx(x, y, z);
                const index_t c = axis == 0 ? x : axis == 1 ? y : z;
                T r = c >= 1 ? g[i - e] : T(0);
                if (c < na - 1) r -= g[i];
                out[i] = r;
            }
}

template <class T>
void backward_transpose(int axis, const T* g, T* out, Dims d) {
    const index_t e = axis == 0 ? 1 : axis == 1 ? d.w : d.w * d.h;
    const index_t na = axis == 0 ? d.w : axis == 1 ? d.h : d.d;
#pragma omp parallel for schedule(static)
    for (index_t z = 0; z < d.d; ++z)
        for (index_t y = 0; y < d.h; ++y)
            for (index_t x = 0; x < d.w; ++x) {
                const index_t i = d.idx(x, y, z);
                const index_t c = axis == 0 ? x : axis == 1 ? y : z;
                out[i] = (c < na - 1 ? g[i + e] : T(0)) - g[i];
            }
}

struct StepParams {
    double tau, sigma, theta, lambda, alpha0, alpha1;
    int data_term;
    bool skip_bz;  // L2 data term with depth == 1 (tgv_cuda/tgv2_l2.cu:39-42)
};

// Pre-projection duals and the primal pre-prox value of one iteration.
template <class T>
struct StepInternals {
    std::vector<T> yp[3], yq[6], ut;
    explicit StepInternals(index_t n) {
        for (int c = 0; c < 3; ++c) yp[c].assign(n, T(0));
        for (int c = 0; c < 6; ++c) yq[c].assign(n, T(0));
        ut.assign(n, T(0));
    }
};

template <class T>
void tgv2_step(const T* f, const TgvFullState<T>& S, TgvFullState<T>& O, StepInternals<T>& I,
               Dims d, const StepParams& k) {
    const index_t n = d.n();
    std::vector<T> t0(n), t1(n), t2(n);
    const T tau = T(k.tau), sigma = T(k.sigma), theta = T(k.theta);
    // p' = P(p + sigma (F ubar - vbar))
    forward_diff(0, S.ub.data(), t0.data(), d);
    forward_diff(1, S.ub.data(), t1.data(), d);
    forward_diff(2, S.ub.data(), t2.data(), d);
    const T* g[3] = {t0.data(), t1.data(), t2.data()};
    for (int c = 0; c < 3; ++c)
        for (index_t i = 0; i < n; ++i) I.yp[c][i] = S.p[c][i] + sigma * (g[c][i] - S.vb[c][i]);
    for (index_t i = 0; i < n; ++i) {
        const T nr = std::sqrt(I.yp[0][i] * I.yp[0][i] + I.yp[1][i] * I.yp[1][i] +
                               I.yp[2][i] * I.yp[2][i]);
        const T s = nr > T(k.alpha1) ? T(k.alpha1) / nr : T(1);
        for (int c = 0; c < 3; ++c) O.p[c][i] = I.yp[c][i] * s;
    }
    // u~ = u - tau B.p', prox, ubar
    std::vector<T> bp(n, T(0));
    for (int c = 0; c < 3; ++c) {
        if (c == 2 && k.skip_bz) continue;
        backward_diff(c, O.p[c].data(), t0.data(), d);
        for (index_t i = 0; i < n; ++i) bp[i] += t0[i];
    }
    const T tl = T(k.tau * k.lambda);
    for (index_t i = 0; i < n; ++i) {
        const T ut = S.u[i] - tau * bp[i];
        I.ut[i] = ut;
        T uu;
        if (k.data_term == L1) {
            const T dd = ut - f[i];
            uu = dd > tl ? ut - tl : (dd < -tl ? ut + tl : f[i]);
        } else {
            uu = (ut + tl * f[i]) / (T(1) + tl);
        }
        O.u[i] = uu;
        O.ub[i] = uu + theta * (uu - S.u[i]);
    }
    // q' = Q(q + sigma E vbar)
    std::vector<T> bvx[3], bvy[3], bvz[3];  // B_a vbar_c
    for (int c = 0; c < 3; ++c) {
        bvx[c].resize(n), bvy[c].resize(n), bvz[c].resize(n);
        backward_diff(0, S.vb[c].data(), bvx[c].data(), d);
        backward_diff(1, S.vb[c].data(), bvy[c].data(), d);
        backward_diff(2, S.vb[c].data(), bvz[c].data(), d);
    }
    for (index_t i = 0; i < n; ++i) {
        const T e[6] = {bvx[0][i], bvy[1][i], bvz[2][i], T(0.5) * (bvx[1][i] + bvy[0][i]),
                        T(0.5) * (bvx[2][i] + bvz[0][i]), T(0.5) * (bvy[2][i] + bvz[1][i])};
        T nr2 = 0;
        for (int c = 0; c < 6; ++c) {
            I.yq[c][i] = S.q[c][i] + sigma * e[c];
            nr2 += (c < 3 ? T(1) : T(2)) * I.yq[c][i] * I.yq[c][i];
        }
        const T nr = std::sqrt(nr2);
        const T s = nr > T(k.alpha0) ? T(k.alpha0) / nr : T(1);
        for (int c = 0; c < 6; ++c) O.q[c][i] = I.yq[c][i] * s;
    }
    // v' = v - tau (divF q' - p'), vbar'
    std::vector<T> dv[3];
    const int qi[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};  // component c: F_a q_{c a}
    for (int c = 0; c < 3; ++c) {
        dv[c].assign(n, T(0));
        for (int a = 0; a < 3; ++a) {
            forward_diff(a, O.q[qi[c][a]].data(), t0.data(), d);
            for (index_t i = 0; i < n; ++i) dv[c][i] += t0[i];
        }
        for (index_t i = 0; i < n; ++i) {
            const T vn = S.v[c][i] - tau * (dv[c][i] - O.p[c][i]);
            O.v[c][i] = vn;
            O.vb[c][i] = vn + theta * (vn - S.v[c][i]);
        }
    }
}

template <class T>
struct ParamGrads {
    double lambda = 0, alpha0 = 0, alpha1 = 0;
};

// Adjoint of one iteration: A1 (adjoint of S_{k+1}) -> A0 (adjoint of S_k).
template <class T>
void tgv2_step_adjoint(const T* f, const TgvFullState<T>& S, const TgvFullState<T>& O,
                       const StepInternals<T>& I, const TgvFullState<T>& A1, TgvFullState<T>& A0,
                       T* grad_f, ParamGrads<T>& pg, Dims d, const StepParams& k) {
    (void)S;  // the internals I hold everything the adjoint needs from the forward step
    (void)O;
    const index_t n = d.n();
    const T tau = T(k.tau), sigma = T(k.sigma), theta = T(k.theta), tl = T(k.tau * k.lambda);
    std::vector<T> va[3], ua(n), uta(n), t0(n);
    // vbar' = v' + theta (v' - v);  v' = v - tau divF q' + tau p'
    for (int c = 0; c < 3; ++c) {
        va[c].resize(n);
        for (index_t i = 0; i < n; ++i) {
            va[c][i] = A1.v[c][i] + (T(1) + theta) * A1.vb[c][i];
            A0.v[c][i] = va[c][i] - theta * A1.vb[c][i];
        }
    }
    // ubar' = u' + theta (u' - u);  u' = prox(u~);  u~ = u - tau B.p'
    for (index_t i = 0; i < n; ++i) {
        ua[i] = A1.u[i] + (T(1) + theta) * A1.ub[i];
        T a_ut;
        if (k.data_term == L1) {
            const T dd = I.ut[i] - f[i];
            if (dd > tl) {
                a_ut = ua[i];
                pg.lambda -= (double)(tau * ua[i]);
            } else if (dd < -tl) {
                a_ut = ua[i];
                pg.lambda += (double)(tau * ua[i]);
            } else {
                a_ut = 0;
                grad_f[i] += ua[i];
            }
        } else {
            const T den = T(1) + tl;
            a_ut = ua[i] / den;
            grad_f[i] += tl * ua[i] / den;
            pg.lambda += (double)(ua[i] * tau * (f[i] - I.ut[i]) / (den * den));
        }
        uta[i] = a_ut;
        A0.u[i] = -theta * A1.ub[i] + a_ut;
    }
    // adjoint of p' and q'
    std::vector<T> pa[3], qa[6];
    for (int c = 0; c < 3; ++c) {
        pa[c].resize(n);
        for (index_t i = 0; i < n; ++i) pa[c][i] = A1.p[c][i] + tau * va[c][i];
        if (c == 2 && k.skip_bz) continue;
        backward_transpose(c, uta.data(), t0.data(), d);
        for (index_t i = 0; i < n; ++i) pa[c][i] -= tau * t0[i];
    }
    for (int c = 0; c < 6; ++c) qa[c] = A1.q[c];
    // divF^T: q_{c a} gets F_a^T va_c
    const int qi[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
    for (int c = 0; c < 3; ++c)
        for (int a = 0; a < 3; ++a) {
            forward_transpose(a, va[c].data(), t0.data(), d);
            for (index_t i = 0; i < n; ++i) qa[qi[c][a]][i] -= tau * t0[i];
        }
    // projections
    std::vector<T> ypa[3], yqa[6];
    for (int c = 0; c < 3; ++c) ypa[c].resize(n);
    for (int c = 0; c < 6; ++c) yqa[c].resize(n);
    for (index_t i = 0; i < n; ++i) {
        T nr = std::sqrt(I.yp[0][i] * I.yp[0][i] + I.yp[1][i] * I.yp[1][i] + I.yp[2][i] * I.yp[2][i]);
        if (nr > T(k.alpha1)) {
            const T a = T(k.alpha1);
            T yg = 0;
            for (int c = 0; c < 3; ++c) yg += I.yp[c][i] * pa[c][i];
            for (int c = 0; c < 3; ++c)
                ypa[c][i] = a / nr * pa[c][i] - a / (nr * nr * nr) * I.yp[c][i] * yg;
            pg.alpha1 += (double)(yg / nr);
        } else {
            for (int c = 0; c < 3; ++c) ypa[c][i] = pa[c][i];
        }
        T nr2 = 0;
        for (int c = 0; c < 6; ++c) nr2 += (c < 3 ? T(1) : T(2)) * I.yq[c][i] * I.yq[c][i];
        nr = std::sqrt(nr2);
        if (nr > T(k.alpha0)) {
            const T a = T(k.alpha0);
            T yg = 0;
            for (int c = 0; c < 6; ++c) yg += I.yq[c][i] * qa[c][i];
            for (int c = 0; c < 6; ++c)
                yqa[c][i] = a / nr * qa[c][i] -
                            a / (nr * nr * nr) * (c < 3 ? T(1) : T(2)) * I.yq[c][i] * yg;
            pg.alpha0 += (double)(yg / nr);
        } else {
            for (int c = 0; c < 6; ++c) yqa[c][i] = qa[c][i];
        }
    }
    // y_p = p + sigma (F ubar - vbar);  y_q = q + sigma E vbar
    for (int c = 0; c < 3; ++c) A0.p[c] = ypa[c];
    for (int c = 0; c < 6; ++c) A0.q[c] = yqa[c];
    std::fill(A0.ub.begin(), A0.ub.end(), T(0));
    for (int c = 0; c < 3; ++c) {
        forward_transpose(c, ypa[c].data(), t0.data(), d);
        for (index_t i = 0; i < n; ++i) A0.ub[i] += sigma * t0[i];
        for (index_t i = 0; i < n; ++i) A0.vb[c][i] = -sigma * ypa[c][i];
    }
    // E^T: vbar_x += B_x^T g_xx + 1/2 B_y^T g_xy + 1/2 B_z^T g_xz, and so on
    const int et[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};  // q index for (component c, axis a)
    for (int c = 0; c < 3; ++c)
        for (int a = 0; a < 3; ++a) {
            const int qq = et[c][a];
            const T w = qq < 3 ? T(1) : T(0.5);
            backward_transpose(a, yqa[qq].data(), t0.data(), d);
            for (index_t i = 0; i < n; ++i) A0.vb[c][i] += sigma * w * t0[i];
        }
}

// Gradient of a loss L(u_K, v_K) through K iterations from u = ubar = f:
// given dL/du_K (and dL/dv_K, may be null), returns dL/df and dL/d(lambda, alpha0,
// alpha1).  Stores every state (small volumes only).
template <class T>
void tgv2_gradient(const T* f, Dims d, const StepParams& k, unsigned K, const T* gu,
                   const T* gv[3], T* grad_f, double grad_params[3], T* u_out) {
    const index_t n = d.n();
    std::vector<TgvFullState<T>> S(K + 1, TgvFullState<T>(n));
    std::vector<StepInternals<T>> I(K, StepInternals<T>(n));
    for (index_t i = 0; i < n; ++i) S[0].u[i] = S[0].ub[i] = f[i];
    for (unsigned it = 0; it < K; ++it) tgv2_step(f, S[it], S[it + 1], I[it], d, k);
    if (u_out) std::copy(S[K].u.begin(), S[K].u.end(), u_out);
    TgvFullState<T> A1(n), A0(n);
    for (index_t i = 0; i < n; ++i) A1.u[i] = gu ? gu[i] : T(0);
    for (int c = 0; c < 3; ++c)
        if (gv && gv[c])
            for (index_t i = 0; i < n; ++i) A1.v[c][i] = gv[c][i];
    std::fill(grad_f, grad_f + n, T(0));
    ParamGrads<T> pg;
    for (int it = (int)K - 1; it >= 0; --it) {
        tgv2_step_adjoint(f, S[it], S[it + 1], I[it], A1, A0, grad_f, pg, d, k);
        std::swap(A1, A0);
    }
    for (index_t i = 0; i < n; ++i) grad_f[i] += A1.u[i] + A1.ub[i];  // u_0 = ubar_0 = f
    grad_params[0] = pg.lambda;
    grad_params[1] = pg.alpha0;
    grad_params[2] = pg.alpha1;
}

}  // namespace oracle
