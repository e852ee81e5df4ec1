// The reference's launcher templates (include/tgvdct_reference_api.hpp) over the
// tgvdct C ABI.  Host code only: every device step happens inside libtgvdct.
#include "tgvdct_reference_api.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "tgvdct.h"

namespace {

bool g_throw = false;

// The reference's cudaCheckError prints the failure and exits the process
// (source/modules/cuda/cuda_helper.in:11-21).
[[noreturn]] void fail(tgvdct_status st) {
    std::string msg = std::string("tgvdct: ") + tgvdct_status_string(st) + ": " + tgvdct_last_error();
    if (g_throw) throw std::runtime_error(msg);
    std::fprintf(stderr, "%s\n", msg.c_str());
    std::exit((int)st);
}

void check(tgvdct_status st) {
    // TGVDCT_STOPPED: the callback asked to stop; the outputs hold the state then,
    // as in the reference, which breaks out of its loop and copies out.
    if (st != TGVDCT_OK && st != TGVDCT_STOPPED) fail(st);
}

size_t count(uint w, uint h, uint d) { return (size_t)w * h * d; }

// Pixel buffers as float: the float instantiation uses the caller's memory, the
// double one converts.
template <typename Pixel>
struct AsFloat {
    std::vector<float> buf;
    const float* p = nullptr;
    AsFloat(const Pixel* src, size_t n) {
        if constexpr (std::is_same<Pixel, float>::value) {
            p = src;
        } else {
            buf.assign(src, src + n);
            p = buf.data();
        }
    }
};

template <typename Pixel>
Pixel* to_new(const float* src, size_t n) {
    Pixel* out = new Pixel[n];
    for (size_t i = 0; i < n; ++i) out[i] = (Pixel)src[i];
    return out;
}

// Host copies the C callback hands over are read-only views owned by the
// library; the reference's callbacks take Pixel* to its own temporary copies, so
// they get a private copy here (float: the view's bytes, double: converted).
template <typename Pixel>
struct CallbackCopies {
    std::vector<Pixel> u, vx, vy, vz;
    Pixel* take(std::vector<Pixel>& dst, const float* src, size_t n) {
        if (!src) return nullptr;
        dst.resize(n);
        for (size_t i = 0; i < n; ++i) dst[i] = (Pixel)src[i];
        return dst.data();
    }
};

template <typename Pixel>
struct DeshadeBridge {
    DeshadeIterationCallback<Pixel>* cb3 = nullptr;
    DeshadeIterationCallback2D<Pixel>* cb2 = nullptr;
    IterationCallback<Pixel>* cbu = nullptr;
    size_t n = 0;
    CallbackCopies<Pixel> copies;

    static int call(uint32_t it, uint32_t total, const float* u, const float* vx, const float* vy,
                    const float* vz, void* user) {
        auto* b = (DeshadeBridge*)user;
        auto& c = b->copies;
        Pixel* pu = c.take(c.u, u, b->n);
        if (b->cbu) return (*b->cbu)(it, total, pu) ? 1 : 0;
        Pixel* px = c.take(c.vx, vx, b->n);
        Pixel* py = c.take(c.vy, vy, b->n);
        if (b->cb2) return (*b->cb2)(it, total, pu, px, py) ? 1 : 0;
        Pixel* pz = c.take(c.vz, vz, b->n);
        return (*b->cb3)(it, total, pu, px, py, pz) ? 1 : 0;
    }
};

tgvdct_params loop_params(uint w, uint h, uint d, float lambda, uint iterations, uint paint,
                          float alpha0, float alpha1) {
    tgvdct_params p;
    tgvdct_params_init(&p);
    p.width = w;
    p.height = h;
    p.depth = d;
    p.lambda = lambda;
    p.alpha0 = alpha0;
    p.alpha1 = alpha1;
    p.iteration_count = iterations;
    p.paint_iteration_interval = paint;
    return p;
}

template <typename Pixel>
Pixel* denoise(Pixel* f_host, uint w, uint h, uint d, Pixel lambda, uint iterations, uint paint,
               IterationCallback<Pixel>& cb, Pixel alpha0, Pixel alpha1, int data_term) {
    const size_t n = count(w, h, d);
    tgvdct_params p = loop_params(w, h, d, (float)lambda, iterations, paint, (float)alpha0,
                                  (float)alpha1);
    p.data_term = data_term;
    AsFloat<Pixel> f(f_host, n);
    std::vector<float> u(n);
    DeshadeBridge<Pixel> bridge;
    bridge.cbu = &cb;
    bridge.n = n;
    const bool with_cb = (bool)cb && paint > 0;
    check(tgvdct_tgv2_run(&p, f.p, u.data(), nullptr, nullptr, nullptr,
                          with_cb ? &DeshadeBridge<Pixel>::call : nullptr,
                          with_cb ? &bridge : nullptr));
    return to_new<Pixel>(u.data(), n);
}

template <typename Pixel>
Pixel* image_op(Pixel* in_host, uint w, uint h, uint d, int which) {
    const size_t n = count(w, h, d);
    AsFloat<Pixel> in(in_host, n);
    std::vector<float> out(n);
    tgvdct_status st;
    if (which == 0) st = tgvdct_cosine_transform_launch(in.p, w, h, d, TGVDCT_DCT_FP32, out.data());
    else if (which == 1)
        st = tgvdct_inverse_cosine_transform_launch(in.p, w, h, d, TGVDCT_DCT_FP32, out.data());
    else
        st = tgvdct_solve_poisson_in_cosine_domain_launch(in.p, w, h, d, TGVDCT_EIGEN_REFERENCE,
                                                          out.data());
    check(st);
    return to_new<Pixel>(out.data(), n);
}

}  // namespace

void tgvdct_refapi_throw_on_error(bool enable) { g_throw = enable; }

template <typename Pixel>
Pixel* tgv2_l1_deshade_launch(Pixel* f_host, uint width, uint height, uint depth, Pixel lambda,
                              uint iteration_count, uint paint_iteration_interval,
                              const int cuda_block_dimension,
                              DeshadeIterationCallback<Pixel> iteration_finished_callback,
                              Pixel alpha0, Pixel alpha1, Pixel** v_x_host, Pixel** v_y_host,
                              Pixel** v_z_host) {
    (void)cuda_block_dimension;
    const size_t n = count(width, height, depth);
    AsFloat<Pixel> f(f_host, n);
    std::vector<float> u(n), vx(n), vy(n), vz(n);
    DeshadeBridge<Pixel> bridge;
    bridge.cb3 = &iteration_finished_callback;
    bridge.n = n;
    const bool with_cb = (bool)iteration_finished_callback && paint_iteration_interval > 0;
    check(tgvdct_tgv2_l1_deshade_launch(f.p, width, height, depth, (float)lambda, iteration_count,
                                        paint_iteration_interval, cuda_block_dimension,
                                        with_cb ? &DeshadeBridge<Pixel>::call : nullptr,
                                        with_cb ? &bridge : nullptr, (float)alpha0, (float)alpha1,
                                        u.data(), vx.data(), vy.data(), vz.data()));
    *v_x_host = to_new<Pixel>(vx.data(), n);
    *v_y_host = to_new<Pixel>(vy.data(), n);
    *v_z_host = to_new<Pixel>(vz.data(), n);
    return to_new<Pixel>(u.data(), n);
}

template <typename Pixel>
Pixel* tgv2_l1_deshade_launch_2d(Pixel* f_host, uint width, uint height, Pixel lambda,
                                 uint iteration_count, uint paint_iteration_interval,
                                 DeshadeIterationCallback2D<Pixel> iteration_finished_callback,
                                 Pixel alpha0, Pixel alpha1, Pixel** v_x_host, Pixel** v_y_host) {
    const size_t n = count(width, height, 1);
    AsFloat<Pixel> f(f_host, n);
    std::vector<float> u(n), vx(n), vy(n);
    DeshadeBridge<Pixel> bridge;
    bridge.cb2 = &iteration_finished_callback;
    bridge.n = n;
    const bool with_cb = (bool)iteration_finished_callback && paint_iteration_interval > 0;
    check(tgvdct_tgv2_l1_deshade_launch_2d(f.p, width, height, (float)lambda, iteration_count,
                                           paint_iteration_interval,
                                           with_cb ? &DeshadeBridge<Pixel>::call : nullptr,
                                           with_cb ? &bridge : nullptr, (float)alpha0,
                                           (float)alpha1, u.data(), vx.data(), vy.data()));
    *v_x_host = to_new<Pixel>(vx.data(), n);
    *v_y_host = to_new<Pixel>(vy.data(), n);
    return to_new<Pixel>(u.data(), n);
}

template <typename Pixel>
Pixel* tgv2_l1_launch(Pixel* f_host, uint width, uint height, uint depth, Pixel lambda,
                      uint iteration_count, uint paint_iteration_interval,
                      IterationCallback<Pixel> iteration_finished_callback, Pixel alpha0,
                      Pixel alpha1) {
    return denoise<Pixel>(f_host, width, height, depth, lambda, iteration_count,
                          paint_iteration_interval, iteration_finished_callback, alpha0, alpha1,
                          TGVDCT_DATA_L1);
}

template <typename Pixel>
Pixel* tgv2_l2_launch(Pixel* f_host, uint width, uint height, uint depth, Pixel lambda,
                      uint iteration_count, uint paint_iteration_interval,
                      IterationCallback<Pixel> iteration_finished_callback, Pixel alpha0,
                      Pixel alpha1) {
    return denoise<Pixel>(f_host, width, height, depth, lambda, iteration_count,
                          paint_iteration_interval, iteration_finished_callback, alpha0, alpha1,
                          TGVDCT_DATA_L2);
}

template <typename Pixel>
Pixel* divergence_kernel_launch(Pixel* dx, Pixel* dy, Pixel* dz, const uint width,
                                const uint height, const uint depth, bool is_host_data) {
    const size_t n = count(width, height, depth);
    std::vector<float> out(n);
    if (is_host_data) {
        AsFloat<Pixel> a(dx, n), b(dy, n), c(depth > 1 ? dz : nullptr, depth > 1 ? n : 0);
        check(tgvdct_divergence_launch(a.p, b.p, depth > 1 ? c.p : nullptr, width, height, depth,
                                       out.data()));
        return to_new<Pixel>(out.data(), n);
    }
    if constexpr (std::is_same<Pixel, float>::value) {
        // device inputs: the result still comes back as a new[] host buffer
        float* out_dev = nullptr;
        check(tgvdct_device_alloc(n * sizeof(float), (void**)&out_dev));
        const tgvdct_status st =
            tgvdct_divergence_dev(dx, dy, depth > 1 ? dz : nullptr, width, height, depth, out_dev,
                                  nullptr);
        const tgvdct_status st2 =
            st == TGVDCT_OK ? tgvdct_device_to_host(out.data(), out_dev, n * sizeof(float)) : st;
        tgvdct_device_free(out_dev);
        check(st2);
        return to_new<Pixel>(out.data(), n);
    } else {
        // double device buffers: bring them to the host and take the host path
        std::vector<double> h[3];
        Pixel* src[3] = {dx, dy, dz};
        for (int k = 0; k < (depth > 1 ? 3 : 2); ++k) {
            h[k].resize(n);
            check(tgvdct_device_to_host(h[k].data(), src[k], n * sizeof(double)));
        }
        return divergence_kernel_launch<Pixel>(h[0].data(), h[1].data(),
                                               depth > 1 ? h[2].data() : nullptr, width, height,
                                               depth, true);
    }
}

template <typename Pixel>
Pixel* cosine_transform_kernel_launch(Pixel* image_host, uint width, uint height, uint depth) {
    return image_op<Pixel>(image_host, width, height, depth, 0);
}

template <typename Pixel>
Pixel* inverse_cosine_transform_kernel_launch(Pixel* image_host, uint width, uint height,
                                              uint depth) {
    return image_op<Pixel>(image_host, width, height, depth, 1);
}

template <typename Pixel>
Pixel* solve_poisson_in_cosine_domain_kernel_launch(Pixel* image_host, uint width, uint height,
                                                    uint depth) {
    return image_op<Pixel>(image_host, width, height, depth, 2);
}

namespace {
std::vector<float> mask_of(const std::vector<uint>& inside, size_t n) {
    std::vector<float> m(n, 0.f);
    for (uint i : inside)
        if (i < n) m[i] = 1.f;
    return m;
}
}  // namespace

template <typename Pixel>
Pixel* tgv2_l1_deshade_masked_launch(
    Pixel* f_host, uint width, uint height, uint depth, Pixel lambda, uint iteration_count,
    uint paint_iteration_interval, const int cuda_block_dimension,
    DeshadeIterationCallback<Pixel> iteration_finished_callback, Pixel alpha0, Pixel alpha1,
    Pixel** v_x_host, Pixel** v_y_host, Pixel** v_z_host,
    const std::vector<uint>& masked_pixel_indices, const std::vector<uint>&,
    const std::vector<uint>&, const std::vector<uint>&, const std::vector<uint>&,
    const std::vector<uint>&, const std::vector<uint>&, const std::vector<uint>&,
    const std::vector<uint>&, const std::vector<uint>&, const std::vector<uint>&,
    const std::vector<uint>&, const std::vector<uint>&) {
    const size_t n = count(width, height, depth);
    AsFloat<Pixel> f(f_host, n);
    const std::vector<float> m = mask_of(masked_pixel_indices, n);
    std::vector<float> u(n), vx(n), vy(n), vz(n);
    DeshadeBridge<Pixel> bridge;
    bridge.cb3 = &iteration_finished_callback;
    bridge.n = n;
    const bool with_cb = (bool)iteration_finished_callback && paint_iteration_interval > 0;
    check(tgvdct_tgv2_l1_deshade_masked_launch(
        f.p, m.data(), width, height, depth, (float)lambda, iteration_count,
        paint_iteration_interval, cuda_block_dimension,
        with_cb ? &DeshadeBridge<Pixel>::call : nullptr, with_cb ? &bridge : nullptr,
        (float)alpha0, (float)alpha1, u.data(), vx.data(), vy.data(), vz.data()));
    *v_x_host = to_new<Pixel>(vx.data(), n);
    *v_y_host = to_new<Pixel>(vy.data(), n);
    *v_z_host = to_new<Pixel>(vz.data(), n);
    return to_new<Pixel>(u.data(), n);
}

template <typename Pixel>
Pixel* tgv2_l1_deshade_masked_2d_launch(
    Pixel* f_host, uint width, uint height, Pixel lambda, uint iteration_count,
    uint paint_iteration_interval, const int cuda_block_dimension,
    DeshadeIterationCallback2D<Pixel> iteration_finished_callback, Pixel alpha0, Pixel alpha1,
    Pixel** v_x_host, Pixel** v_y_host, const std::vector<uint>& masked_pixel_indices,
    const std::vector<uint>&, const std::vector<uint>&, const std::vector<uint>&,
    const std::vector<uint>&, const std::vector<uint>&, const std::vector<uint>&,
    const std::vector<uint>&, const std::vector<uint>&) {
    const size_t n = count(width, height, 1);
    AsFloat<Pixel> f(f_host, n);
    const std::vector<float> m = mask_of(masked_pixel_indices, n);
    std::vector<float> u(n), vx(n), vy(n);
    DeshadeBridge<Pixel> bridge;
    bridge.cb2 = &iteration_finished_callback;
    bridge.n = n;
    const bool with_cb = (bool)iteration_finished_callback && paint_iteration_interval > 0;
    check(tgvdct_tgv2_l1_deshade_masked_launch(
        f.p, m.data(), width, height, 1, (float)lambda, iteration_count, paint_iteration_interval,
        cuda_block_dimension, with_cb ? &DeshadeBridge<Pixel>::call : nullptr,
        with_cb ? &bridge : nullptr, (float)alpha0, (float)alpha1, u.data(), vx.data(), vy.data(),
        nullptr));
    *v_x_host = to_new<Pixel>(vx.data(), n);
    *v_y_host = to_new<Pixel>(vy.data(), n);
    return to_new<Pixel>(u.data(), n);
}

#define TGVDCT_INSTANTIATE(P)                                                                     \
    template P* tgv2_l1_deshade_launch<P>(P*, uint, uint, uint, P, uint, uint, const int,         \
                                          DeshadeIterationCallback<P>, P, P, P**, P**, P**);      \
    template P* tgv2_l1_deshade_launch_2d<P>(P*, uint, uint, P, uint, uint,                       \
                                             DeshadeIterationCallback2D<P>, P, P, P**, P**);      \
    template P* tgv2_l1_launch<P>(P*, uint, uint, uint, P, uint, uint, IterationCallback<P>, P,  \
                                  P);                                                             \
    template P* tgv2_l2_launch<P>(P*, uint, uint, uint, P, uint, uint, IterationCallback<P>, P,  \
                                  P);                                                             \
    template P* divergence_kernel_launch<P>(P*, P*, P*, const uint, const uint, const uint,      \
                                            bool);                                                \
    template P* cosine_transform_kernel_launch<P>(P*, uint, uint, uint);                          \
    template P* inverse_cosine_transform_kernel_launch<P>(P*, uint, uint, uint);                  \
    template P* solve_poisson_in_cosine_domain_kernel_launch<P>(P*, uint, uint, uint);          \
    template P* tgv2_l1_deshade_masked_launch<P>(                                                 \
        P*, uint, uint, uint, P, uint, uint, const int, DeshadeIterationCallback<P>, P, P, P**,   \
        P**, P**, const std::vector<uint>&, const std::vector<uint>&, const std::vector<uint>&,  \
        const std::vector<uint>&, const std::vector<uint>&, const std::vector<uint>&,            \
        const std::vector<uint>&, const std::vector<uint>&, const std::vector<uint>&,            \
        const std::vector<uint>&, const std::vector<uint>&, const std::vector<uint>&,            \
        const std::vector<uint>&);                                                                \
    template P* tgv2_l1_deshade_masked_2d_launch<P>(                                              \
        P*, uint, uint, P, uint, uint, const int, DeshadeIterationCallback2D<P>, P, P, P**, P**, \
        const std::vector<uint>&, const std::vector<uint>&, const std::vector<uint>&,            \
        const std::vector<uint>&, const std::vector<uint>&, const std::vector<uint>&,            \
        const std::vector<uint>&, const std::vector<uint>&, const std::vector<uint>&);

TGVDCT_INSTANTIATE(float)
TGVDCT_INSTANTIATE(double)
