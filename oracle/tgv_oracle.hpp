// TEST INFRASTRUCTURE — the CPU oracle for the TGV-DCT deshade path.
//
// This header checks the product and is not part of it: only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg may call it.  It restates, step by step, the
// reference's CUDA kernel sequence of josefkoller/ambient_image_processor as plain
// C++ loops (OpenMP over voxels), templated on the pixel type:
//   * T = float  restates the reference's float instantiation (FP32 stores,
//                explicit fmaf where the reference calls fmaf, FP64 cosine basis
//                with a float accumulator in the DCT passes);
//   * T = double is the FP64 oracle that every error figure is measured against.
//
// Layout: x-fastest, index = z*W*H + y*W + x (source/modules/itk/ITKImage.cpp:84).
//
// Parity pin: tests/golden/ holds outputs of the reference's own .cu kernels,
// compiled for the CPU by oracle/ref_cpu/ and run in the build container;
// tests/test_oracle_golden.py checks this header against them.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <functional>
#include <vector>

namespace oracle {

using index_t = std::ptrdiff_t;

// ---------------------------------------------------------------------------
// cos(pi * a), written from the definition: exact reduction of a modulo 2 and
// the symmetries of cosine, then the C library's cos/sin on |pi*r| <= pi/4.
// The reference calls CUDA's cospi on these same arguments
// (cuda_image_operations/cosine_transform.cu:160-165,
//  solve_poisson_in_cosine_domain.cu:48-53).
inline double cospi_d(double a) {
    double r = std::fmod(std::fabs(a), 2.0);  // exact
    if (r > 1.0) r = 2.0 - r;                 // exact (Sterbenz)
    const double pi = 3.14159265358979323846;
    if (r <= 0.25) return std::cos(pi * r);
    if (r <= 0.75) return std::sin(pi * (0.5 - r));
    return -std::cos(pi * (1.0 - r));
}
inline float cospi_f(float a) { return (float)cospi_d((double)a); }
inline double cospi_t(double a) { return cospi_d(a); }
inline float cospi_t(float a) { return cospi_f(a); }

// sqrt(a^2+b^2+c^2) for norm3df (tgv_cuda/tgv2_common.cu:121)
inline float norm3_t(float a, float b, float c) {
    return (float)std::sqrt((double)a * a + (double)b * b + (double)c * c);
}
inline double norm3_t(double a, double b, double c) { return std::sqrt(a * a + b * b + c * c); }

inline float fma_t(float a, float b, float c) { return std::fmaf(a, b, c); }
inline double fma_t(double a, double b, double c) { return std::fma(a, b, c); }

struct Dims {
    index_t w, h, d;
    index_t n() const { return w * h * d; }
    index_t idx(index_t x, index_t y, index_t z) const { return (z * h + y) * w + x; }
};

// ---------------------------------------------------------------------------
// Difference operators (Appendix-A semantics of the reference).
//
// F_a: Neumann forward difference, (F w)[i] = w[i+e] - w[i], 0 on the last slice
//      (tgv_cuda/tgv_common.cu:66-130).
// B_a: the reference's "backward difference", negated: (B w)[i] = w[i-e] - w[i],
//      and -w[i] on the first slice (tgv_cuda/tgv_common.cu:133-197).
template <class T>
void forward_diff(int axis, const T* in, T* out, Dims g) {
    const index_t e = axis == 0 ? 1 : axis == 1 ? g.w : g.w * g.h;
    const index_t na = axis == 0 ? g.w : axis == 1 ? g.h : g.d;
#pragma omp parallel for schedule(static)
    for (index_t z = 0; z < g.d; ++z)
        for (index_t y = 0; y < g.h; ++y)
            for (index_t x = 0; x < g.w; ++x) {
                const index_t i = g.idx(x, y, z);
                const index_t c = axis == 0 ? x : axis == 1 ? y : z;
                out[i] = (c == na - 1) ? T(0) : T(in[i + e] - in[i]);
            }
}

template <class T>
void backward_diff(int axis, const T* in, T* out, Dims g) {
    const index_t e = axis == 0 ? 1 : axis == 1 ? g.w : g.w * g.h;
#pragma omp parallel for schedule(static)
    for (index_t z = 0; z < g.d; ++z)
        for (index_t y = 0; y < g.h; ++y)
            for (index_t x = 0; x < g.w; ++x) {
                const index_t i = g.idx(x, y, z);
                const index_t c = axis == 0 ? x : axis == 1 ? y : z;
                out[i] = (c == 0) ? T(-in[i]) : T(-in[i] + in[i - e]);
            }
}

enum DataTerm { L1 = 0, L2 = 1 };

struct Params {
    double lambda = 1.0, alpha0 = 2.0, alpha1 = 1.0;
    unsigned iterations = 0;
    // reference step sizes: tau = sigma = 1/sqrt(20), theta = 1
    // (tgv_deshade/tgv2_l1_deshade.cu:148-150)
    double tau = 0.0, sigma = 0.0, theta = 1.0;
    int data_term = L1;
    // true: the 2-D launcher (tgv_deshade/tgv2_l1_deshade_2d.cu), two gradient
    // components; false: the 3-D launcher, also when depth == 1.
    bool two_d = false;
    unsigned paint_interval = 0;
};

inline double default_step() { return 1.0 / std::sqrt(20.0); }

// Callback: (iteration_index, iteration_count, u, v_x, v_y, v_z) -> stop?
template <class T>
using IterCallback = std::function<bool(unsigned, unsigned, const T*, const T*, const T*, const T*)>;

// ---------------------------------------------------------------------------
// TGV2 primal-dual loop: restates tgv_deshade/tgv2_l1_deshade.cu:148-272 (3-D),
// tgv_deshade/tgv2_l1_deshade_2d.cu:84-183 (2-D), with the kernels
// tgv_cuda/tgv2_common.cu:96-354, tgv_cuda/tgv2_l1.cu:27-60,
// tgv_cuda/tgv2_l2.cu:27-56, tgv_cuda/tgv2_common_2d.cu:55-279.
// Writes u (denoised) and v (the bias gradient field).  v_z may be null for 2-D.
// Returns the number of iterations run (a callback may stop the loop early).
//
// domain (optional): the masked deshade of tgv_deshade_masked/tgv2_l1_deshade_masked.cu
// (and _2d.cu), whose kernels (tgv2_masked_common.cu, tgv_masked_common.cu) update
// only the voxels with mask >= 1 (index lists built by
// TGVDeshadeMaskedProcessor.cpp:337-385).  Voxels with domain[i] == 0 are never
// updated: they keep u = u_bar = f and p = v = v_bar = q = 0, and the differences
// taken at updated voxels read those values.
// The loop state of tgv2_deshade: the persistent fields (f, u, u_bar, p, v, v_bar, q)
// and the temporaries one iteration uses.
template <class T>
struct LoopState {
    std::vector<T> f, u, u_prev, u_bar;
    std::vector<T> gx, gy, gz;                                  // p_x, p_y, p_z temporaries
    std::vector<T> px, py, pz;                                  // p dual (p_xx, p_yy, p_zz)
    std::vector<T> vx, vy, vz, vbx, vby, vbz, vpx, vpy, vpz;
    std::vector<T> qxx, qyy, qzz, qxy, qxz, qyz;                // q dual
    std::vector<T> exx, eyy, ezz, exy, exz, eyz, tmp;           // temps
    explicit LoopState(const T* f_in, index_t n)
        : f(f_in, f_in + n), u(f), u_prev(n), u_bar(f), gx(n), gy(n), gz(n), px(n, 0),
          py(n, 0), pz(n, 0), vx(n, 0), vy(n, 0), vz(n, 0), vbx(n, 0), vby(n, 0), vbz(n, 0),
          vpx(n), vpy(n), vpz(n), qxx(n, 0), qyy(n, 0), qzz(n, 0), qxy(n, 0), qxz(n, 0),
          qyz(n, 0), exx(n), eyy(n), ezz(n), exy(n), exz(n), eyz(n), tmp(n) {}
};

// One iteration of the loop below, in place on the state.
template <class T>
void tgv2_iteration(LoopState<T>& st, Dims g, const Params& prm,
                    const unsigned char* domain = nullptr) {
    const index_t n = g.n();
    const bool three = !prm.two_d;
    const T tau = T(prm.tau > 0 ? prm.tau : default_step());
    const T sigma = T(prm.sigma > 0 ? prm.sigma : default_step());
    const T theta = T(prm.theta);
    const T lambda = T(prm.lambda), alpha0 = T(prm.alpha0), alpha1 = T(prm.alpha1);
    auto& f = st.f;
    auto& u = st.u;
    auto& u_prev = st.u_prev;
    auto& u_bar = st.u_bar;
    auto &gx = st.gx, &gy = st.gy, &gz = st.gz;
    auto &px = st.px, &py = st.py, &pz = st.pz;
    auto &vx = st.vx, &vy = st.vy, &vz = st.vz;
    auto &vbx = st.vbx, &vby = st.vby, &vbz = st.vbz;
    auto &vpx = st.vpx, &vpy = st.vpy, &vpz = st.vpz;
    auto &qxx = st.qxx, &qyy = st.qyy, &qzz = st.qzz, &qxy = st.qxy, &qxz = st.qxz,
         &qyz = st.qyz;
    auto &exx = st.exx, &eyy = st.eyy, &ezz = st.ezz, &exy = st.exy, &exz = st.exz,
         &eyz = st.eyz, &tmp = st.tmp;
    {
        // 1. forward differences of u_bar, p update and projection, u_prev = u
        forward_diff(0, u_bar.data(), gx.data(), g);
        forward_diff(1, u_bar.data(), gy.data(), g);
        if (three) forward_diff(2, u_bar.data(), gz.data(), g);
#pragma omp parallel for schedule(static)
        for (index_t i = 0; i < n; ++i) {
            if (domain && !domain[i]) continue;
            px[i] = fma_t(sigma, T(gx[i] - vbx[i]), px[i]);
            py[i] = fma_t(sigma, T(gy[i] - vby[i]), py[i]);
            T nrm;
            if (three) {
                pz[i] = fma_t(sigma, T(gz[i] - vbz[i]), pz[i]);
                nrm = norm3_t(px[i], py[i], pz[i]);
            } else {
                nrm = T(std::sqrt(T(T(px[i] * px[i]) + T(py[i] * py[i]))));
            }
            nrm = std::fmax(T(1), T(nrm / alpha1));
            px[i] = px[i] / nrm;
            py[i] = py[i] / nrm;
            if (three) pz[i] = pz[i] / nrm;
            u_prev[i] = u[i];
        }
        // 2. negated backward differences of p, primal u step, prox, over-relaxation
        backward_diff(0, px.data(), gx.data(), g);
        backward_diff(1, py.data(), gy.data(), g);
        if (three) backward_diff(2, pz.data(), gz.data(), g);
        const T tl = T(tau * lambda);
#pragma omp parallel for schedule(static)
        for (index_t i = 0; i < n; ++i) {
            if (domain && !domain[i]) continue;
            T div;
            if (!three) div = T(gx[i] + gy[i]);
            else if (prm.data_term == L2 && g.d == 1) div = T(gx[i] + gy[i]);  // tgv2_l2.cu:39-42
            else div = T(T(gx[i] + gy[i]) + gz[i]);
            T uu = T(u[i] - T(tau * div));
            if (prm.data_term == L1) {
                const T umf = T(uu - f[i]);
                if (umf > tl) uu = T(uu - tl);
                else if (umf < -tl) uu = T(uu + tl);
                else uu = f[i];
            } else {
                uu = T(T(uu + T(tl * f[i])) / T(T(1) + tl));
            }
            u[i] = uu;
            u_bar[i] = T(uu + T(theta * T(uu - u_prev[i])));
        }
        // 3. symmetric gradient of v_bar from negated backward differences
        backward_diff(0, vbx.data(), exx.data(), g);
        backward_diff(1, vby.data(), eyy.data(), g);
        backward_diff(0, vby.data(), exy.data(), g);
        backward_diff(1, vbx.data(), tmp.data(), g);
#pragma omp parallel for schedule(static)
        for (index_t i = 0; i < n; ++i) exy[i] = T(T(exy[i] + tmp[i]) * T(0.5));
        if (three) {
            backward_diff(2, vbz.data(), ezz.data(), g);
            backward_diff(0, vbz.data(), exz.data(), g);
            backward_diff(2, vbx.data(), tmp.data(), g);
#pragma omp parallel for schedule(static)
            for (index_t i = 0; i < n; ++i) exz[i] = T(T(exz[i] + tmp[i]) * T(0.5));
            backward_diff(1, vbz.data(), eyz.data(), g);
            backward_diff(2, vby.data(), tmp.data(), g);
#pragma omp parallel for schedule(static)
            for (index_t i = 0; i < n; ++i) eyz[i] = T(T(eyz[i] + tmp[i]) * T(0.5));
        }
        // 4. q update and projection, v_prev = v
#pragma omp parallel for schedule(static)
        for (index_t i = 0; i < n; ++i) {
            if (domain && !domain[i]) continue;
            qxx[i] = fma_t(sigma, exx[i], qxx[i]);
            qyy[i] = fma_t(sigma, eyy[i], qyy[i]);
            qxy[i] = fma_t(sigma, exy[i], qxy[i]);
            T s = T(T(qxx[i] * qxx[i]) + T(qyy[i] * qyy[i]));
            s = T(s + T(T(2 * qxy[i]) * qxy[i]));
            if (three) {
                qzz[i] = fma_t(sigma, ezz[i], qzz[i]);
                qxz[i] = fma_t(sigma, exz[i], qxz[i]);
                qyz[i] = fma_t(sigma, eyz[i], qyz[i]);
                s = T(s + T(qzz[i] * qzz[i]));
                s = T(s + T(T(2 * qxz[i]) * qxz[i]));
                s = T(s + T(T(2 * qyz[i]) * qyz[i]));
            }
            const T nrm = std::fmax(T(1), T(T(std::sqrt(s)) / alpha0));
            qxx[i] = qxx[i] / nrm;
            qyy[i] = qyy[i] / nrm;
            qxy[i] = qxy[i] / nrm;
            if (three) {
                qzz[i] = qzz[i] / nrm;
                qxz[i] = qxz[i] / nrm;
                qyz[i] = qyz[i] / nrm;
            }
            vpx[i] = vx[i];
            vpy[i] = vy[i];
            if (three) vpz[i] = vz[i];
        }
        // 5. divergence of q with forward differences (off-diagonals not halved)
        forward_diff(0, qxx.data(), exx.data(), g);
        forward_diff(1, qxy.data(), tmp.data(), g);
#pragma omp parallel for schedule(static)
        for (index_t i = 0; i < n; ++i) exx[i] = T(exx[i] + tmp[i]);
        forward_diff(1, qyy.data(), eyy.data(), g);
        forward_diff(0, qxy.data(), tmp.data(), g);
#pragma omp parallel for schedule(static)
        for (index_t i = 0; i < n; ++i) eyy[i] = T(eyy[i] + tmp[i]);
        if (three) {
            forward_diff(2, qxz.data(), tmp.data(), g);
#pragma omp parallel for schedule(static)
            for (index_t i = 0; i < n; ++i) exx[i] = T(exx[i] + tmp[i]);
            forward_diff(2, qyz.data(), tmp.data(), g);
#pragma omp parallel for schedule(static)
            for (index_t i = 0; i < n; ++i) eyy[i] = T(eyy[i] + tmp[i]);
            forward_diff(2, qzz.data(), ezz.data(), g);
            forward_diff(0, qxz.data(), tmp.data(), g);
#pragma omp parallel for schedule(static)
            for (index_t i = 0; i < n; ++i) ezz[i] = T(ezz[i] + tmp[i]);
            forward_diff(1, qyz.data(), tmp.data(), g);
#pragma omp parallel for schedule(static)
            for (index_t i = 0; i < n; ++i) ezz[i] = T(ezz[i] + tmp[i]);
        }
        // 6. primal v step and over-relaxation
#pragma omp parallel for schedule(static)
        for (index_t i = 0; i < n; ++i) {
            if (domain && !domain[i]) continue;
            vx[i] = T(vx[i] - T(tau * T(exx[i] - px[i])));
            vy[i] = T(vy[i] - T(tau * T(eyy[i] - py[i])));
            vbx[i] = T(vx[i] + T(theta * T(vx[i] - vpx[i])));
            vby[i] = T(vy[i] + T(theta * T(vy[i] - vpy[i])));
            if (three) {
                vz[i] = T(vz[i] - T(tau * T(ezz[i] - pz[i])));
                vbz[i] = T(vz[i] + T(theta * T(vz[i] - vpz[i])));
            }
        }
    }
}

template <class T>
unsigned tgv2_deshade(const T* f_in, Dims g, const Params& prm, T* u_out, T* vx_out,
                      T* vy_out, T* vz_out, IterCallback<T> cb = nullptr,
                      const unsigned char* domain = nullptr) {
    const index_t n = g.n();
    const bool three = !prm.two_d;
    LoopState<T> st(f_in, n);
    auto& u = st.u;
    auto &vx = st.vx, &vy = st.vy, &vz = st.vz;

    unsigned it = 0;
    for (; it < prm.iterations; ++it) {
        tgv2_iteration(st, g, prm, domain);
        // 7. iteration callback (tgv_cuda/tgv2_common.cu:374-408)
        if (cb && prm.paint_interval > 0 && it > 0 && it % prm.paint_interval == 0) {
            if (cb(it, prm.iterations, u.data(), vx.data(), vy.data(), three ? vz.data() : nullptr)) {
                ++it;
                break;
            }
        }
    }
    std::memcpy(u_out, u.data(), sizeof(T) * n);
    std::memcpy(vx_out, vx.data(), sizeof(T) * n);
    std::memcpy(vy_out, vy.data(), sizeof(T) * n);
    if (vz_out) {
        if (three) std::memcpy(vz_out, vz.data(), sizeof(T) * n);
        else std::memset(vz_out, 0, sizeof(T) * n);
    }
    return it;
}

// ---------------------------------------------------------------------------
// Poisson right-hand side: rhs = B_x v_x + B_y v_y (+ B_z v_z when depth > 1)
// (cuda_image_operations/divergence.cu:26-56; depth == 1 goes through
//  divergence_2d.cu:37-56, CudaImageOperationsProcessor.cpp:290-291).
template <class T>
void divergence(const T* vx, const T* vy, const T* vz, Dims g, T* out) {
    const index_t n = g.n();
    std::vector<T> a(n), b(n), c(n);
    backward_diff(0, vx, a.data(), g);
    backward_diff(1, vy, b.data(), g);
#pragma omp parallel for schedule(static)
    for (index_t i = 0; i < n; ++i) a[i] = T(a[i] + b[i]);
    if (g.d > 1) {
        backward_diff(2, vz, c.data(), g);
#pragma omp parallel for schedule(static)
        for (index_t i = 0; i < n; ++i) a[i] = T(a[i] + c[i]);
    }
    std::memcpy(out, a.data(), sizeof(T) * n);
}

// Cosine table  C[k*N + m] = cospi((m + 0.5) * k / N), evaluated in double like
// the reference's `cospi((x2 + 0.5) * x / size)` with size a Pixel-typed N
// (cosine_transform.cu:160-165; inverse_cosine_transform.cu:96-101).
inline std::vector<double> cosine_table(index_t N) {
    std::vector<double> c((size_t)(N * N));
    for (index_t k = 0; k < N; ++k)
        for (index_t m = 0; m < N; ++m)
            c[(size_t)(k * N + m)] = cospi_d(((double)m + 0.5) * (double)k / (double)N);
    return c;
}

// One separable pass along `axis`.  Forward (DCT-II, cosine_transform.cu:142-223):
//   out[k] = sum_m in[m] * cospi((m+.5)k/N), times `scale_mul` at the end.
// Inverse (DCT-III, inverse_cosine_transform.cu:79-164):
//   out[m] = 2 * sum_{k>=1} in[k] * cospi((m+.5)k/N) + in[0], then / `scale_div`.
// The accumulator is the Pixel-typed output element: every term is added in double
// and rounded back to T, as `result[index] += image[...] * cospi(double)` does.
template <class T>
void dct_pass(int axis, bool inverse, const T* in, T* out, Dims g, double scale_mul,
              double scale_div) {
    const index_t N = axis == 0 ? g.w : axis == 1 ? g.h : g.d;
    const index_t e = axis == 0 ? 1 : axis == 1 ? g.w : g.w * g.h;
    const std::vector<double> C = cosine_table(N);
#pragma omp parallel for schedule(static)
    for (index_t z = 0; z < g.d; ++z)
        for (index_t y = 0; y < g.h; ++y)
            for (index_t x = 0; x < g.w; ++x) {
                const index_t i = g.idx(x, y, z);
                const index_t c = axis == 0 ? x : axis == 1 ? y : z;
                const index_t base = i - c * e;
                T acc = T(0);
                if (!inverse) {
                    for (index_t m = 0; m < N; ++m)
                        acc = T((double)acc + (double)in[base + m * e] * C[(size_t)(c * N + m)]);
                    if (scale_mul != 1.0) acc = T(acc * T(scale_mul));
                } else {
                    for (index_t k = 1; k < N; ++k)
                        acc = T((double)acc + (double)in[base + k * e] * C[(size_t)(k * N + c)]);
                    acc = T(acc * T(2));
                    acc = T(acc + in[base]);
                    if (scale_div != 1.0) acc = T((double)acc / scale_div);
                }
                out[i] = acc;
            }
}

// cosine_transform_kernel_launch (cosine_transform.cu:226-293): x, y (, z) passes,
// the last pass multiplies by 8.
template <class T>
void cosine_transform(const T* in, Dims g, T* out) {
    std::vector<T> a(g.n()), b(g.n());
    if (g.d == 1) {
        dct_pass(0, false, in, a.data(), g, 1.0, 1.0);
        dct_pass(1, false, a.data(), out, g, 8.0, 1.0);
    } else {
        dct_pass(0, false, in, a.data(), g, 1.0, 1.0);
        dct_pass(1, false, a.data(), b.data(), g, 1.0, 1.0);
        dct_pass(2, false, b.data(), out, g, 8.0, 1.0);
    }
}

// inverse_cosine_transform_kernel_launch (inverse_cosine_transform.cu:167-227):
// the last pass divides by 8*W*H(*D).
template <class T>
void inverse_cosine_transform(const T* in, Dims g, T* out) {
    std::vector<T> a(g.n()), b(g.n());
    const double s = (double)(g.w * g.h * g.d) * 8.0;
    if (g.d == 1) {
        dct_pass(0, true, in, a.data(), g, 1.0, 1.0);
        dct_pass(1, true, a.data(), out, g, 1.0, s);
    } else {
        dct_pass(0, true, in, a.data(), g, 1.0, 1.0);
        dct_pass(1, true, a.data(), b.data(), g, 1.0, 1.0);
        dct_pass(2, true, b.data(), out, g, 1.0, s);
    }
}

// solve_poisson_in_cosine_domain_kernel(_2D) (solve_poisson_in_cosine_domain.cu:27-83):
// divide by 6 - 2cospi(kx/W) - 2cospi(ky/H) - 2cospi(kz/D) (4 - ... when depth == 1),
// with the cosines of Pixel-typed arguments and the sum in double; DC -> 0.
template <class T>
void solve_poisson_in_cosine_domain(const T* in, Dims g, T* out) {
#pragma omp parallel for schedule(static)
    for (index_t z = 0; z < g.d; ++z)
        for (index_t y = 0; y < g.h; ++y)
            for (index_t x = 0; x < g.w; ++x) {
                const index_t i = g.idx(x, y, z);
                if (x == 0 && y == 0 && z == 0) {
                    out[i] = T(0);
                    continue;
                }
                const double cx = (double)cospi_t(T(T(x) / T(g.w)));
                const double cy = (double)cospi_t(T(T(y) / T(g.h)));
                double den;
                if (g.d == 1) {
                    den = 4.0 - 2.0 * cx - 2.0 * cy;
                } else {
                    const double cz = (double)cospi_t(T(T(z) / T(g.d)));
                    den = 6.0 - 2.0 * cx - 2.0 * cy - 2.0 * cz;
                }
                out[i] = T((double)in[i] / den);
            }
}

// integrate_image_gradients_poisson_cosine_transform (tgv_deshade/TGVDeshadeProcessor.cpp:386-431)
template <class T>
void integrate_poisson_dct(const T* vx, const T* vy, const T* vz, Dims g, T* l_out) {
    std::vector<T> a(g.n()), b(g.n());
    divergence(vx, vy, vz, g, a.data());
    cosine_transform(a.data(), g, b.data());
    solve_poisson_in_cosine_domain(b.data(), g, a.data());
    inverse_cosine_transform(a.data(), g, l_out);
}

// deshade_poisson_cosine_transform (TGVDeshadeProcessor.cpp:71-95) plus the optional
// background add-back r += u * (1 - mask) (TGVDeshadeProcessor.cpp:275-279).
// l is multiplied by the mask in place when a mask is given, like the reference.
template <class T>
void deshade_epilogue(const T* u, T* l, const T* mask, bool set_negative_values_to_zero,
                      bool add_background_back, index_t n, T* r_out) {
#pragma omp parallel for schedule(static)
    for (index_t i = 0; i < n; ++i) {
        T r = T(u[i] - l[i]);
        if (mask) {
            l[i] = T(l[i] * mask[i]);
            r = T(r * mask[i]);
        }
        if (set_negative_values_to_zero && r < 0) r = T(0);
        if (add_background_back && mask) r = T(r + T(u[i] * T(T(1) - mask[i])));
        r_out[i] = r;
    }
}

// The tail of TGVDeshadeMaskedProcessor::processTGV2L1GPUCuda
// (TGVDeshadeMaskedProcessor.cpp:186-211): deshade_epilogue with the mask applied to l
// and r, then either the background add-back or a second multiply by the mask.
template <class T>
void masked_deshade_epilogue(const T* u, T* l, const T* mask, bool set_negative_values_to_zero,
                             bool add_background_back, index_t n, T* r_out) {
#pragma omp parallel for schedule(static)
    for (index_t i = 0; i < n; ++i) {
        T r = T(u[i] - l[i]);
        l[i] = T(l[i] * mask[i]);
        r = T(r * mask[i]);
        if (set_negative_values_to_zero && r < 0) r = T(0);
        if (add_background_back) r = T(r + T(u[i] * T(T(1) - mask[i])));
        else r = T(r * mask[i]);
        r_out[i] = r;
    }
}

// ---------------------------------------------------------------------------
// Convergence metrics of TGVDeshadeProcessor::processTGV2L1DeshadeCuda_convergenceTest
// and ..._convergenceTestMetric (TGVDeshadeProcessor.cpp:479-568), with the image
// statistics of :168-220 accumulated in T in the images' linear order (the
// reference's ITK iteration order, x fastest; T = float is its own arithmetic).
// The deshade loop calls back every `interval` iterations; each call integrates l
// from v (times the mask when one is given); from the second call on it records
// the normalised cross-correlation of l with the previous l and their time total
// variation sum |l - l_before|.  The normalisation uses the mean of the current l
// for both images, as the reference's normalized_cross_correlation does (:190-193).
template <class T>
T linear_mean(const std::vector<T>& a) {
    T m = 0;
    for (const T v : a) m = T(m + v);
    return T(m / T(a.size()));
}
template <class T>
T linear_std(const std::vector<T>& a, T mean) {
    T s = 0;
    for (const T v : a) {
        const T d = T(v - mean);
        s = T(s + T(d * d));
    }
    return T(std::sqrt(T(s / T(a.size() - 1))));
}
template <class T>
T normalized_cross_correlation(const std::vector<T>& a, const std::vector<T>& b) {
    const T m1 = linear_mean(a), s1 = linear_std(a, m1);
    const T m2 = linear_mean(a), s2 = linear_std(b, m2);
    T acc = 0;
    for (size_t i = 0; i < a.size(); ++i) acc = T(acc + T(T(a[i] - m1) * T(b[i] - m2)));
    return T(acc / T(T(s1 * s2) * T(a.size())));
}
template <class T>
T time_tv(const std::vector<T>& a, const std::vector<T>& b) {
    T s = 0;
    for (size_t i = 0; i < a.size(); ++i) s = T(s + std::fabs(T(a[i] - b[i])));
    return s;
}

template <class T>
struct ConvergenceHistory {
    std::vector<T> ncc, tv;
    T metric_tv[2] = {0, 0};
};

template <class T>
ConvergenceHistory<T> convergence_test(const T* f, const T* mask, Dims g, Params prm,
                                       unsigned interval) {
    const index_t n = g.n();
    ConvergenceHistory<T> h;
    std::vector<T> l_before;
    prm.paint_interval = interval;
    std::vector<T> u(n), vx(n), vy(n), vz(n);
    tgv2_deshade<T>(f, g, prm, u.data(), vx.data(), vy.data(), vz.data(),
                    [&](unsigned, unsigned, const T*, const T* px, const T* py, const T* pz) {
                        std::vector<T> l(n);
                        integrate_poisson_dct<T>(px, py, pz, g, l.data());
                        if (mask)
                            for (index_t i = 0; i < n; ++i) l[i] = T(l[i] * mask[i]);
                        if (!l_before.empty()) {
                            h.ncc.push_back(normalized_cross_correlation(l, l_before));
                            h.tv.push_back(time_tv(l, l_before));
                        }
                        l_before.swap(l);
                        return false;
                    });
    // :556-566: sum of |h[i+1] - h[i]| for i < size - 2 (the last difference is left out)
    const std::vector<T>* series[2] = {&h.ncc, &h.tv};
    for (int m = 0; m < 2; ++m) {
        T acc = 0;
        const std::vector<T>& v = *series[m];
        for (size_t i = 0; i + 2 < v.size(); ++i) acc = T(acc + std::fabs(T(v[i + 1] - v[i])));
        h.metric_tv[m] = acc;
    }
    return h;
}

}  // namespace oracle
