// TEST INFRASTRUCTURE — extern "C" driver around the reference's own launchers,
// built for the CPU by build_ref_cpu.py (the launchers come from the reference's
// unmodified .cu sources, compiled by g++ against shim/cuda.h).  The few lines of
// ITK-level glue that call them are restated here from
// source/modules/tgv_deshade/TGVDeshadeProcessor.cpp:122-166,386-408 and
// source/modules/cuda_image_operations/CudaImageOperationsProcessor.cpp:286-294.
#include <cmath>
#include <cstring>
#include <functional>
#include <vector>

#include "cuda.h"

uint3_ blockIdx;
uint3_ threadIdx;
dim3 blockDim;
dim3 gridDim;

template <typename Pixel>
using DeshadeIterationCallback =
    std::function<bool(uint, uint, Pixel*, Pixel*, Pixel*, Pixel*)>;
template <typename Pixel>
using DeshadeIterationCallback2D = std::function<bool(uint, uint, Pixel*, Pixel*, Pixel*)>;
template <typename Pixel>
using IterationCallback = std::function<bool(uint, uint, Pixel*)>;

// Declarations of the reference's explicit instantiations.
template <typename Pixel>
Pixel* tgv2_l1_deshade_launch(Pixel* f_host, uint width, uint height, uint depth, Pixel lambda,
                              uint iteration_count, uint paint_iteration_interval,
                              const int cuda_block_dimension,
                              DeshadeIterationCallback<Pixel> iteration_finished_callback,
                              Pixel alpha0, Pixel alpha1, Pixel** v_x, Pixel** v_y, Pixel** v_z);
template <typename Pixel>
Pixel* tgv2_l1_deshade_launch_2d(Pixel* f_host, uint width, uint height, Pixel lambda,
                                 uint iteration_count, uint paint_iteration_interval,
                                 DeshadeIterationCallback2D<Pixel> iteration_finished_callback,
                                 Pixel alpha0, Pixel alpha1, Pixel** v_x, Pixel** v_y);
template <typename Pixel>
Pixel* tgv2_l1_launch(Pixel* f_host, uint width, uint height, uint depth, Pixel lambda,
                      uint iteration_count, uint paint_iteration_interval,
                      IterationCallback<Pixel> iteration_finished_callback, Pixel alpha0,
                      Pixel alpha1);
template <typename Pixel>
Pixel* tgv2_l2_launch(Pixel* f_host, uint width, uint height, uint depth, Pixel lambda,
                      uint iteration_count, uint paint_iteration_interval,
                      IterationCallback<Pixel> iteration_finished_callback, Pixel alpha0,
                      Pixel alpha1);
template <typename Pixel>
Pixel* divergence_kernel_launch(Pixel* dx, Pixel* dy, Pixel* dz, const uint width,
                                const uint height, const uint depth, bool is_host_data);
template <typename Pixel>
Pixel* divergence_2d_kernel_launch(Pixel* dx, Pixel* dy, const uint width, const uint height,
                                   bool is_host_data);
template <typename Pixel>
Pixel* cosine_transform_kernel_launch(Pixel* image_host, uint width, uint height, uint depth);
template <typename Pixel>
Pixel* inverse_cosine_transform_kernel_launch(Pixel* image_host, uint width, uint height,
                                              uint depth);
template <typename Pixel>
Pixel* solve_poisson_in_cosine_domain_kernel_launch(Pixel* image_host, uint width, uint height,
                                                    uint depth);
template <typename Pixel>
Pixel* subtract_kernel_launch(Pixel* image1, Pixel* image2, uint width, uint height, uint depth);
template <typename Pixel>
Pixel* clamp_negative_values_kernel_launch(Pixel* image, uint width, uint height, uint depth,
                                           Pixel value);

template <typename Pixel>
Pixel* multiply_kernel_launch(Pixel* image1, Pixel* image2, uint width, uint height, uint depth);
template <typename Pixel>
Pixel* add_kernel_launch(Pixel* image1, Pixel* image2, uint width, uint height, uint depth);
template <typename Pixel>
Pixel* invert_kernel_launch(Pixel* image, uint width, uint height, uint depth);

using RefIndices = const std::vector<uint>&;
template <typename Pixel>
Pixel* tgv2_l1_deshade_masked_launch(
    Pixel* f_host, uint width, uint height, uint depth, Pixel lambda, uint iteration_count,
    uint paint_iteration_interval, const int cuda_block_dimension,
    DeshadeIterationCallback<Pixel> iteration_finished_callback, Pixel alpha0, Pixel alpha1,
    Pixel** v_x_host, Pixel** v_y_host, Pixel** v_z_host, RefIndices masked, RefIndices left,
    RefIndices not_left, RefIndices right, RefIndices not_right, RefIndices top,
    RefIndices not_top, RefIndices bottom, RefIndices not_bottom, RefIndices front,
    RefIndices not_front, RefIndices back, RefIndices not_back);
template <typename Pixel>
Pixel* tgv2_l1_deshade_masked_2d_launch(
    Pixel* f_host, uint width, uint height, Pixel lambda, uint iteration_count,
    uint paint_iteration_interval, const int cuda_block_dimension,
    DeshadeIterationCallback2D<Pixel> iteration_finished_callback, Pixel alpha0, Pixel alpha1,
    Pixel** v_x_host, Pixel** v_y_host, RefIndices masked, RefIndices left, RefIndices not_left,
    RefIndices right, RefIndices not_right, RefIndices top, RefIndices not_top,
    RefIndices bottom, RefIndices not_bottom);

namespace {
template <class P>
void take(P* src, P* dst, size_t n) {
    std::memcpy(dst, src, sizeof(P) * n);
    delete[] src;
}

// CudaImageOperationsProcessor::divergence: depth == 1 goes to the 2-D kernels.
template <class P>
P* divergence_any(P* vx, P* vy, P* vz, uint w, uint h, uint d) {
    if (d == 1) return divergence_2d_kernel_launch<P>(vx, vy, w, h, true);
    return divergence_kernel_launch<P>(vx, vy, vz, w, h, d, true);
}

// integrate_image_gradients_poisson_cosine_transform (TGVDeshadeProcessor.cpp:386-408)
template <class P>
P* integrate(P* vx, P* vy, P* vz, uint w, uint h, uint d) {
    P* div = divergence_any<P>(vx, vy, vz, w, h, d);
    P* dct = cosine_transform_kernel_launch<P>(div, w, h, d);
    delete[] div;
    P* sol = solve_poisson_in_cosine_domain_kernel_launch<P>(dct, w, h, d);
    delete[] dct;
    P* l = inverse_cosine_transform_kernel_launch<P>(sol, w, h, d);
    delete[] sol;
    return l;
}
// The index lists of TGVDeshadeMaskedProcessor::buildMaskIndices
// (tgv_deshade_masked/TGVDeshadeMaskedProcessor.cpp:337-385): voxels with mask >= 1,
// split by whether they lie on each face of the volume.
struct MaskIndices {
    std::vector<uint> inside, edge[6], not_edge[6];  // left right top bottom front back
};
MaskIndices mask_indices(const float* mask, uint w, uint h, uint d) {
    MaskIndices m;
    for (uint z = 0; z < d; ++z)
        for (uint y = 0; y < h; ++y)
            for (uint x = 0; x < w; ++x) {
                const uint i = (z * h + y) * w + x;
                if (mask[i] < 1) continue;
                m.inside.push_back(i);
                const bool on[6] = {x == 0, x == w - 1, y == 0, y == h - 1, z == 0, z == d - 1};
                for (int k = 0; k < 6; ++k) (on[k] ? m.edge[k] : m.not_edge[k]).push_back(i);
            }
    return m;
}

// tgv2_l1_deshade_masked_launch (3-D) or its 2-D twin (depth == 1), as
// TGVDeshadeMaskedProcessor.cpp:77-212 / :214-330 call them without a callback.
float* masked_launch(const float* f, const float* mask, uint w, uint h, uint d, float lambda,
                     float alpha0, float alpha1, uint iterations, float** vx, float** vy,
                     float** vz) {
    const size_t n = (size_t)w * h * d;
    float* fin = new float[n];
    std::memcpy(fin, f, sizeof(float) * n);
    const MaskIndices m = mask_indices(mask, w, h, d);
    float* u;
    if (d > 1) {
        u = tgv2_l1_deshade_masked_launch<float>(
            fin, w, h, d, lambda, iterations, iterations + 1, -1, nullptr, alpha0, alpha1, vx, vy,
            vz, m.inside, m.edge[0], m.not_edge[0], m.edge[1], m.not_edge[1], m.edge[2],
            m.not_edge[2], m.edge[3], m.not_edge[3], m.edge[4], m.not_edge[4], m.edge[5],
            m.not_edge[5]);
    } else {
        u = tgv2_l1_deshade_masked_2d_launch<float>(
            fin, w, h, lambda, iterations, iterations + 1, -1, nullptr, alpha0, alpha1, vx, vy,
            m.inside, m.edge[0], m.not_edge[0], m.edge[1], m.not_edge[1], m.edge[2],
            m.not_edge[2], m.edge[3], m.not_edge[3]);
        *vz = new float[n]();
    }
    delete[] fin;
    return u;
}
}  // namespace

extern "C" {

// tgv2_l1_deshade_launch<float> as TGVDeshadeProcessor.cpp:137-145 calls it
// (paint interval = iterations + 1, so no callback).
void ref_tgv2_l1_deshade_f32(const float* f, uint w, uint h, uint d, float lambda, float alpha0,
                             float alpha1, uint iterations, float* u, float* vx, float* vy,
                             float* vz) {
    const size_t n = (size_t)w * h * d;
    float* fin = new float[n];
    std::memcpy(fin, f, sizeof(float) * n);
    float *ox, *oy, *oz;
    float* ou = tgv2_l1_deshade_launch<float>(fin, w, h, d, lambda, iterations, iterations + 1,
                                              -1, nullptr, alpha0, alpha1, &ox, &oy, &oz);
    delete[] fin;
    take(ou, u, n);
    take(ox, vx, n);
    take(oy, vy, n);
    take(oz, vz, n);
}

void ref_tgv2_l1_deshade_2d_f32(const float* f, uint w, uint h, float lambda, float alpha0,
                                float alpha1, uint iterations, float* u, float* vx, float* vy) {
    const size_t n = (size_t)w * h;
    float* fin = new float[n];
    std::memcpy(fin, f, sizeof(float) * n);
    float *ox, *oy;
    float* ou = tgv2_l1_deshade_launch_2d<float>(fin, w, h, lambda, iterations, iterations + 1,
                                                 nullptr, alpha0, alpha1, &ox, &oy);
    delete[] fin;
    take(ou, u, n);
    take(ox, vx, n);
    take(oy, vy, n);
}

// The TGV filter's denoise launchers (tgv_cuda/tgv2_l1.cu:64, tgv_cuda/tgv2_l2.cu:60).
void ref_tgv2_denoise_f32(int data_term, const float* f, uint w, uint h, uint d, float lambda,
                          float alpha0, float alpha1, uint iterations, float* u) {
    const size_t n = (size_t)w * h * d;
    float* fin = new float[n];
    std::memcpy(fin, f, sizeof(float) * n);
    float* ou = data_term == 0
                    ? tgv2_l1_launch<float>(fin, w, h, d, lambda, iterations, iterations + 1,
                                            nullptr, alpha0, alpha1)
                    : tgv2_l2_launch<float>(fin, w, h, d, lambda, iterations, iterations + 1,
                                            nullptr, alpha0, alpha1);
    delete[] fin;
    take(ou, u, n);
}

#define REF_TYPED(P, SUF)                                                                        \
    void ref_divergence_##SUF(const P* vx, const P* vy, const P* vz, uint w, uint h, uint d,    \
                              P* out) {                                                          \
        const size_t n = (size_t)w * h * d;                                                      \
        P* r = divergence_any<P>(const_cast<P*>(vx), const_cast<P*>(vy), const_cast<P*>(vz), w, \
                                 h, d);                                                          \
        take(r, out, n);                                                                         \
    }                                                                                            \
    void ref_cosine_transform_##SUF(const P* in, uint w, uint h, uint d, P* out) {               \
        take(cosine_transform_kernel_launch<P>(const_cast<P*>(in), w, h, d), out,                \
             (size_t)w * h * d);                                                                 \
    }                                                                                            \
    void ref_inverse_cosine_transform_##SUF(const P* in, uint w, uint h, uint d, P* out) {       \
        take(inverse_cosine_transform_kernel_launch<P>(const_cast<P*>(in), w, h, d), out,        \
             (size_t)w * h * d);                                                                 \
    }                                                                                            \
    void ref_solve_poisson_##SUF(const P* in, uint w, uint h, uint d, P* out) {                  \
        take(solve_poisson_in_cosine_domain_kernel_launch<P>(const_cast<P*>(in), w, h, d), out,  \
             (size_t)w * h * d);                                                                 \
    }                                                                                            \
    void ref_integrate_poisson_dct_##SUF(const P* vx, const P* vy, const P* vz, uint w, uint h, \
                                         uint d, P* out) {                                       \
        take(integrate<P>(const_cast<P*>(vx), const_cast<P*>(vy), const_cast<P*>(vz), w, h, d), \
             out, (size_t)w * h * d);                                                            \
    }

REF_TYPED(float, f32)
REF_TYPED(double, f64)
#undef REF_TYPED

// TGVDeshadeProcessor::processTGV2L1GPUCuda, the terminal-program overload
// (TGVDeshadeProcessor.cpp:122-166) with no mask and set_negative_values_to_zero
// as the CLI passes it (terminal_programs/tgv2_deshade_main.cpp:57-68).
void ref_process_tgv2_l1_f32(const float* f, uint w, uint h, uint d, float lambda, float alpha0,
                             float alpha1, uint iterations, int set_negative_values_to_zero,
                             float* denoised, float* shading, float* deshaded) {
    const size_t n = (size_t)w * h * d;
    float* fin = new float[n];
    std::memcpy(fin, f, sizeof(float) * n);
    float *vx, *vy, *vz;
    float* u = tgv2_l1_deshade_launch<float>(fin, w, h, d, lambda, iterations, iterations + 1, -1,
                                             nullptr, alpha0, alpha1, &vx, &vy, &vz);
    delete[] fin;
    float* l = integrate<float>(vx, vy, vz, w, h, d);
    delete[] vx;
    delete[] vy;
    delete[] vz;
    float* r = subtract_kernel_launch<float>(u, l, w, h, d);
    if (set_negative_values_to_zero) {
        float* r2 = clamp_negative_values_kernel_launch<float>(r, w, h, d, 0.0f);
        delete[] r;
        r = r2;
    }
    take(u, denoised, n);
    take(l, shading, n);
    take(r, deshaded, n);
}

// The masked TGV loop alone (v_z is zero for depth == 1).
void ref_tgv2_l1_deshade_masked_f32(const float* f, const float* mask, uint w, uint h, uint d,
                                    float lambda, float alpha0, float alpha1, uint iterations,
                                    float* u, float* vx, float* vy, float* vz) {
    const size_t n = (size_t)w * h * d;
    float *ox, *oy, *oz;
    float* ou = masked_launch(f, mask, w, h, d, lambda, alpha0, alpha1, iterations, &ox, &oy, &oz);
    take(ou, u, n);
    take(ox, vx, n);
    take(oy, vy, n);
    take(oz, vz, n);
}

// TGVDeshadeMaskedProcessor::processTGV2L1GPUCuda (TGVDeshadeMaskedProcessor.cpp:77-212,
// 2-D :214-330) without a callback: the masked loop, then
// TGVDeshadeProcessor::deshade_poisson_cosine_transform (TGVDeshadeProcessor.cpp:71-95)
// with the mask, then the background add-back or a second mask multiply.
void ref_process_tgv2_l1_masked_f32(const float* f, const float* mask, uint w, uint h, uint d,
                                    float lambda, float alpha0, float alpha1, uint iterations,
                                    int set_negative_values_to_zero, int add_background_back,
                                    float* denoised, float* shading, float* deshaded) {
    const size_t n = (size_t)w * h * d;
    float *vx, *vy, *vz;
    float* u = masked_launch(f, mask, w, h, d, lambda, alpha0, alpha1, iterations, &vx, &vy, &vz);
    float* mk = new float[n];
    std::memcpy(mk, mask, sizeof(float) * n);
    float* l = integrate<float>(vx, vy, vz, w, h, d);
    delete[] vx;
    delete[] vy;
    delete[] vz;
    float* r = subtract_kernel_launch<float>(u, l, w, h, d);
    float* t = multiply_kernel_launch<float>(l, mk, w, h, d);
    delete[] l;
    l = t;
    t = multiply_kernel_launch<float>(r, mk, w, h, d);
    delete[] r;
    r = t;
    if (set_negative_values_to_zero) {
        t = clamp_negative_values_kernel_launch<float>(r, w, h, d, 0.0f);
        delete[] r;
        r = t;
    }
    if (add_background_back) {
        float* inv = invert_kernel_launch<float>(mk, w, h, d);
        float* bg = multiply_kernel_launch<float>(u, inv, w, h, d);
        t = add_kernel_launch<float>(r, bg, w, h, d);
        delete[] inv;
        delete[] bg;
    } else {
        t = multiply_kernel_launch<float>(r, mk, w, h, d);
    }
    delete[] r;
    r = t;
    delete[] mk;
    take(u, denoised, n);
    take(l, shading, n);
    take(r, deshaded, n);
}

// processTGV2L1DeshadeCuda_convergenceTest / ..._convergenceTestMetric
// (TGVDeshadeProcessor.cpp:479-568) on the reference's launcher and Poisson chain,
// with the float image statistics of :168-220 restated (ITK order: x fastest).
unsigned ref_convergence_test_f32(const float* f, const float* mask, uint w, uint h, uint d,
                                  float lambda, float alpha0, float alpha1, uint iterations,
                                  uint interval, float* ncc, float* tv, unsigned capacity,
                                  float* metric_tv) {
    const size_t n = (size_t)w * h * d;
    std::vector<float> l_before;
    std::vector<float> hn, ht;
    auto mean = [&](const std::vector<float>& a) {
        float m = 0;
        for (float v : a) m += v;
        return m /= (float)n;
    };
    auto stdev = [&](const std::vector<float>& a, float m) {
        float s = 0;
        for (float v : a) {
            const float dd = v - m;
            s += dd * dd;
        }
        return std::sqrt(s / (float)(n - 1));
    };
    DeshadeIterationCallback<float> cb = [&](uint, uint, float*, float* vx, float* vy,
                                             float* vz) {
        float* l = integrate<float>(vx, vy, vz, w, h, d);
        if (mask) {
            float* mk = new float[n];
            std::memcpy(mk, mask, sizeof(float) * n);
            float* t = multiply_kernel_launch<float>(l, mk, w, h, d);
            delete[] mk;
            delete[] l;
            l = t;
        }
        std::vector<float> cur(l, l + n);
        delete[] l;
        if (!l_before.empty()) {
            const float m1 = mean(cur), s1 = stdev(cur, m1);
            const float m2 = mean(cur), s2 = stdev(l_before, m2);
            float acc = 0;
            for (size_t i = 0; i < n; ++i) acc += (cur[i] - m1) * (l_before[i] - m2);
            hn.push_back(acc / (s1 * s2 * (float)n));
            float* a = new float[n];
            float* b = new float[n];
            std::memcpy(a, cur.data(), sizeof(float) * n);
            std::memcpy(b, l_before.data(), sizeof(float) * n);
            float* diff = subtract_kernel_launch<float>(a, b, w, h, d);
            float t = 0;
            for (size_t i = 0; i < n; ++i) t += std::fabs(diff[i]);
            delete[] a;
            delete[] b;
            delete[] diff;
            ht.push_back(t);
        }
        l_before.swap(cur);
        return false;
    };
    float* fin = new float[n];
    std::memcpy(fin, f, sizeof(float) * n);
    float *ox, *oy, *oz;
    float* ou = tgv2_l1_deshade_launch<float>(fin, w, h, d, lambda, iterations, interval, -1, cb,
                                              alpha0, alpha1, &ox, &oy, &oz);
    delete[] fin;
    delete[] ou;
    delete[] ox;
    delete[] oy;
    delete[] oz;
    const std::vector<float>* series[2] = {&hn, &ht};
    for (int m = 0; m < 2; ++m) {
        float acc = 0;
        for (size_t i = 0; i + 2 < series[m]->size(); ++i)
            acc += std::fabs((*series[m])[i + 1] - (*series[m])[i]);
        metric_tv[m] = acc;
    }
    for (size_t i = 0; i < hn.size() && i < capacity; ++i) {
        ncc[i] = hn[i];
        tv[i] = ht[i];
    }
    return (unsigned)hn.size();
}

}  // extern "C"
