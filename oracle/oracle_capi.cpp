// TEST INFRASTRUCTURE — extern "C" entry points of the CPU oracle (tgv_oracle.hpp),
// loaded by tests/ and bench.py's CPU-baseline leg through ctypes.  Not product code.
#include <algorithm>
#include <vector>

#include "tgv_adjoint.hpp"
#include "tgv_oracle.hpp"
#include "resize_oracle.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

using oracle::Dims;
using oracle::index_t;

namespace {
oracle::Params make_params(double lambda, double alpha0, double alpha1, unsigned iterations,
                           double tau, double sigma, double theta, int data_term, int two_d) {
    oracle::Params p;
    p.lambda = lambda;
    p.alpha0 = alpha0;
    p.alpha1 = alpha1;
    p.iterations = iterations;
    p.tau = tau;
    p.sigma = sigma;
    p.theta = theta;
    p.data_term = data_term;
    p.two_d = two_d != 0;
    return p;
}
Dims dims(unsigned w, unsigned h, unsigned d) { return Dims{(index_t)w, (index_t)h, (index_t)d}; }
}  // namespace

extern "C" {

int oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

#define ORACLE_TYPED(T, SUF)                                                                      \
    unsigned oracle_tgv2_deshade_##SUF(const T* f, unsigned w, unsigned h, unsigned d,            \
                                       double lambda, double alpha0, double alpha1,               \
                                       unsigned iterations, double tau, double sigma,             \
                                       double theta, int data_term, int two_d, T* u, T* vx,       \
                                       T* vy, T* vz) {                                            \
        return oracle::tgv2_deshade<T>(f, dims(w, h, d),                                          \
                                       make_params(lambda, alpha0, alpha1, iterations, tau,       \
                                                   sigma, theta, data_term, two_d),               \
                                       u, vx, vy, vz);                                            \
    }                                                                                             \
    void oracle_divergence_##SUF(const T* vx, const T* vy, const T* vz, unsigned w, unsigned h,   \
                                 unsigned d, T* out) {                                            \
        oracle::divergence<T>(vx, vy, vz, dims(w, h, d), out);                                    \
    }                                                                                             \
    void oracle_cosine_transform_##SUF(const T* in, unsigned w, unsigned h, unsigned d, T* out) { \
        oracle::cosine_transform<T>(in, dims(w, h, d), out);                                      \
    }                                                                                             \
    void oracle_inverse_cosine_transform_##SUF(const T* in, unsigned w, unsigned h, unsigned d,   \
                                               T* out) {                                          \
        oracle::inverse_cosine_transform<T>(in, dims(w, h, d), out);                              \
    }                                                                                             \
    void oracle_solve_poisson_##SUF(const T* in, unsigned w, unsigned h, unsigned d, T* out) {    \
        oracle::solve_poisson_in_cosine_domain<T>(in, dims(w, h, d), out);                        \
    }                                                                                             \
    void oracle_integrate_poisson_dct_##SUF(const T* vx, const T* vy, const T* vz, unsigned w,    \
                                            unsigned h, unsigned d, T* l) {                       \
        oracle::integrate_poisson_dct<T>(vx, vy, vz, dims(w, h, d), l);                           \
    }                                                                                             \
    void oracle_deshade_epilogue_##SUF(const T* u, T* l, const T* mask, int clamp, int add_back,  \
                                       unsigned long long n, T* r) {                              \
        oracle::deshade_epilogue<T>(u, l, mask, clamp != 0, add_back != 0, (index_t)n, r);        \
    }                                                                                             \
    void oracle_masked_deshade_epilogue_##SUF(const T* u, T* l, const T* mask, int clamp,         \
                                              int add_back, unsigned long long n, T* r) {         \
        oracle::masked_deshade_epilogue<T>(u, l, mask, clamp != 0, add_back != 0, (index_t)n, r); \
    }                                                                                             \
    unsigned oracle_tgv2_deshade_masked_##SUF(                                                    \
        const T* f, const T* mask, unsigned w, unsigned h, unsigned d, double lambda,             \
        double alpha0, double alpha1, unsigned iterations, double tau, double sigma,              \
        double theta, int data_term, int two_d, T* u, T* vx, T* vy, T* vz) {                      \
        const size_t n = (size_t)w * h * d;                                                       \
        std::vector<unsigned char> dom(n);                                                        \
        for (size_t i = 0; i < n; ++i) dom[i] = mask[i] >= T(1) ? 1 : 0;                          \
        return oracle::tgv2_deshade<T>(f, dims(w, h, d),                                          \
                                       make_params(lambda, alpha0, alpha1, iterations, tau,       \
                                                   sigma, theta, data_term, two_d),               \
                                       u, vx, vy, vz, nullptr, dom.data());                       \
    }

// Iterations on an explicit loop state, in place: the 17 persistent fields (f is
// read only) in the order f, u, u_bar, p_x, p_y, p_z, v_x, v_y, v_z, vbar_x, vbar_y,
// vbar_z, q_xx, q_yy, q_zz, q_xy, q_xz, q_yz; each w*h*d values.  The same iteration
// as oracle_tgv2_deshade_*, which starts from u = u_bar = f and zeros.
#define ORACLE_STEP(T, SUF)                                                                       \
    void oracle_tgv2_step_##SUF(T* const* fields, unsigned w, unsigned h, unsigned d,            \
                                double lambda, double alpha0, double alpha1,                      \
                                unsigned iterations, double tau, double sigma, double theta,      \
                                int data_term, int two_d) {                                       \
        const Dims g = dims(w, h, d);                                                             \
        const index_t n = g.n();                                                                  \
        oracle::LoopState<T> st(fields[0], n);                                                    \
        std::vector<T>* v[18] = {&st.f,   &st.u,   &st.u_bar, &st.px,  &st.py,  &st.pz,          \
                                 &st.vx,  &st.vy,  &st.vz,    &st.vbx, &st.vby, &st.vbz,         \
                                 &st.qxx, &st.qyy, &st.qzz,   &st.qxy, &st.qxz, &st.qyz};        \
        for (int k = 1; k < 18; ++k) std::copy(fields[k], fields[k] + n, v[k]->begin());        \
        const oracle::Params prm = make_params(lambda, alpha0, alpha1, iterations, tau, sigma,    \
                                               theta, data_term, two_d);                          \
        for (unsigned it = 0; it < iterations; ++it) oracle::tgv2_iteration(st, g, prm);         \
        for (int k = 1; k < 18; ++k) std::copy(v[k]->begin(), v[k]->end(), fields[k]);          \
    }
ORACLE_STEP(float, f32)
ORACLE_STEP(double, f64)
#undef ORACLE_STEP

#define ORACLE_CONVERGENCE(T, SUF)                                                                \
    unsigned oracle_convergence_test_##SUF(const T* f, const T* mask, unsigned w, unsigned h,    \
                                           unsigned d, double lambda, double alpha0,             \
                                           double alpha1, unsigned iterations, unsigned interval, \
                                           T* ncc, T* tv, unsigned capacity, T* metric_tv) {      \
        auto r = oracle::convergence_test<T>(                                                     \
            f, mask, dims(w, h, d),                                                               \
            make_params(lambda, alpha0, alpha1, iterations, 0, 0, 1, oracle::L1, 0), interval);   \
        for (size_t i = 0; i < r.ncc.size() && i < capacity; ++i) {                              \
            ncc[i] = r.ncc[i];                                                                    \
            tv[i] = r.tv[i];                                                                      \
        }                                                                                         \
        metric_tv[0] = r.metric_tv[0];                                                            \
        metric_tv[1] = r.metric_tv[1];                                                            \
        return (unsigned)r.ncc.size();                                                            \
    }
ORACLE_CONVERGENCE(float, f32)
ORACLE_CONVERGENCE(double, f64)
#undef ORACLE_CONVERGENCE

ORACLE_TYPED(float, f32)
ORACLE_TYPED(double, f64)

#undef ORACLE_TYPED

// FP64 reverse mode through K iterations (tgv_adjoint.hpp).  gu / gv* may be null.
// grad_params: d/dlambda, d/dalpha0, d/dalpha1.
void oracle_tgv2_gradient_f64(const double* f, unsigned w, unsigned h, unsigned d, double lambda,
                              double alpha0, double alpha1, unsigned K, double tau, double sigma,
                              double theta, int data_term, const double* gu, const double* gvx,
                              const double* gvy, const double* gvz, double* grad_f,
                              double* grad_params, double* u_out) {
    oracle::StepParams k;
    k.tau = tau > 0 ? tau : oracle::default_step();
    k.sigma = sigma > 0 ? sigma : oracle::default_step();
    k.theta = theta;
    k.lambda = lambda;
    k.alpha0 = alpha0;
    k.alpha1 = alpha1;
    k.data_term = data_term;
    k.skip_bz = data_term == oracle::L2 && d == 1;
    const double* gv[3] = {gvx, gvy, gvz};
    oracle::tgv2_gradient<double>(f, dims(w, h, d), k, K, gu, gv, grad_f, grad_params, u_out);
}

// Cubic B-spline resize as ResizeProcessor runs it through ITK (resize_oracle.hpp).
void oracle_resize_bspline3_f32(const float* in, unsigned w, unsigned h, unsigned d, float* out,
                                unsigned W, unsigned H, unsigned D) {
    oracle::resize_bspline3<float>(in, w, h, d, out, W, H, D);
}

unsigned oracle_resize_factor_extent(unsigned n, float factor) {
    return oracle::resize_factor_extent(n, factor);
}

}  // extern "C"
