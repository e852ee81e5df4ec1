// TEST INFRASTRUCTURE — CPU restatement of the cubic B-spline resize that the
// reference's ResizeProcessor::process(image, width, height, depth, BSpline3)
// (source/modules/resize/ResizeProcessor.cpp:49-143) and ::process(image, factor, ...)
// (:35-47) run through ITK 4.8.1 (README.md:37): itk::ResampleImageFilter with an
// identity transform and itk::BSplineInterpolateImageFunction of order 3, whose
// coefficients come from itk::BSplineDecompositionImageFilter.  ITK is not part of
// the reference tree, so this restates the published algorithm ITK implements
// (Unser, Aldroubi & Eden, IEEE TSP 41(2), 1993; Unser, IEEE SPM 16(6), 1999;
// Thevenaz, Blu & Unser, IEEE TMI 19(7), 2000): the recursive prefilter with one pole
// z = sqrt(3) - 2, mirror (whole-sample symmetric) boundaries, a truncated causal
// initialisation at tolerance 1e-10, and the 4 x 4 x 4 tensor-product evaluation.
// Parity against ITK itself is unpinned (no ITK here); the reference's own call
// sites fix the geometry.  Arithmetic is double, like ITK's coefficient type, and
// the result is cast to float, like the resample filter's float output.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace oracle {

// ResizeProcessor.cpp:38-45: ceil(n * factor) in float, at least 1.
inline unsigned resize_factor_extent(unsigned n, float factor) {
    const float e = std::ceil((float)n * factor);
    const unsigned u = (unsigned)e;
    return u < 1u ? 1u : u;
}

struct BSplineAxis {
    // per output index: the four mirrored input indices, their weights, and whether
    // the sample point lies inside the input's continuous region
    std::vector<int> idx;        // 4 per output index
    std::vector<double> wt;      // 4 per output index
    std::vector<uint8_t> inside;
};

// itk::BSplineInterpolateImageFunction::ApplyMirrorBoundaryConditions
inline int bspline_mirror(int k, int n) {
    if (n == 1) return 0;
    const int n2 = 2 * n - 2;
    if (k < 0) {
        k = -k;
        k -= n2 * (k / n2);
        if (k >= n) k = n2 - k;
    } else if (k >= n) {
        k -= n2 * (k / n2);
        if (k >= n) k = n2 - k;
    }
    return k;
}

// One axis of the resample: out samples 0 .. out_keep-1 of an out_grid-long grid whose
// spacing is in_spacing / (out_grid / n as float), origin 0 (ResizeProcessor.cpp:70-90).
inline BSplineAxis bspline_axis(unsigned n, unsigned out_grid, unsigned out_keep) {
    BSplineAxis a;
    a.idx.resize(4 * (size_t)out_keep);
    a.wt.resize(4 * (size_t)out_keep);
    a.inside.resize(out_keep);
    const float size_factor = (float)out_grid / (float)n;
    const double in_spacing = 1.0;
    const double out_spacing = in_spacing / (double)size_factor;
    for (unsigned i = 0; i < out_keep; ++i) {
        // physical point i * out_spacing, continuous input index point / in_spacing
        const double x = ((double)i * out_spacing) * (1.0 / in_spacing);
        // itk::ImageFunction::IsInsideBuffer: [-0.5, n - 0.5)
        a.inside[i] = (x >= -0.5 && x < (double)n - 0.5) ? 1 : 0;
        const double fl = std::floor(x);
        const int base = (int)fl - 1;
        const double t = x - fl;
        double w[4];
        w[3] = (1.0 / 6.0) * t * t * t;
        w[0] = (1.0 / 6.0) + 0.5 * t * (t - 1.0) - w[3];
        w[2] = t + w[0] - 2.0 * w[3];
        w[1] = 1.0 - w[0] - w[2] - w[3];
        for (int k = 0; k < 4; ++k) {
            a.idx[4 * (size_t)i + k] = bspline_mirror(base + k, (int)n);
            a.wt[4 * (size_t)i + k] = w[k];
        }
    }
    return a;
}

// The prefilter constants of the cubic spline.
struct BSplinePole {
    double z, gain;
    long horizon;
};
inline BSplinePole bspline_pole() {
    BSplinePole p;
    p.z = std::sqrt(3.0) - 2.0;
    p.gain = (1.0 - p.z) * (1.0 - 1.0 / p.z);
    p.horizon = (long)std::ceil(std::log(1e-10) / std::log(std::fabs(p.z)));
    return p;
}

// itk::BSplineDecompositionImageFilter::DataToCoefficients1D on one line of length n
// with element stride s; z2n = z^(n-1) (used only when n <= horizon).
inline void bspline_prefilter_line(double* c, long n, size_t s, const BSplinePole& p, double z2n) {
    if (n == 1) return;
    const double z = p.z;
    for (long k = 0; k < n; ++k) c[k * s] = c[k * s] * p.gain;
    // causal initialisation
    if (p.horizon < n) {
        double zn = z, sum = c[0];
        for (long k = 1; k < p.horizon; ++k) {
            sum = sum + zn * c[k * s];
            zn = zn * z;
        }
        c[0] = sum;
    } else {
        double zn = z;
        const double iz = 1.0 / z;
        double z2 = z2n;
        double sum = c[0] + z2 * c[(n - 1) * s];
        z2 = z2 * z2 * iz;
        for (long k = 1; k <= n - 2; ++k) {
            sum = sum + (zn + z2) * c[k * s];
            zn = zn * z;
            z2 = z2 * iz;
        }
        c[0] = sum / (1.0 - zn * zn);
    }
    for (long k = 1; k < n; ++k) c[k * s] = c[k * s] + z * c[(k - 1) * s];
    // anti-causal initialisation and recursion
    c[(n - 1) * s] = (z / (z * z - 1.0)) * (z * c[(n - 2) * s] + c[(n - 1) * s]);
    for (long k = n - 2; k >= 0; --k) c[k * s] = z * (c[(k + 1) * s] - c[k * s]);
}

// ResizeProcessor::process(image, width, height, depth, BSpline3): out is W x H x D.
template <class In>
void resize_bspline3(const In* in, unsigned w, unsigned h, unsigned d, float* out, unsigned W,
                     unsigned H, unsigned D) {
    // ResizeProcessor.cpp:55-63: upsampling adds two samples per axis, then keeps the
    // first W x H x D (the Extract at :136-141)
    const bool up = W > w || H > h || D > d;
    const unsigned gW = up ? W + 2 : W, gH = up ? H + 2 : H, gD = up ? D + 2 : D;
    const size_t n = (size_t)w * h * d, wh = (size_t)w * h;
    std::vector<double> c(n);
    for (size_t i = 0; i < n; ++i) c[i] = (double)in[i];
    const BSplinePole p = bspline_pole();
    // the decomposition filters along x, then y, then z
    if (w > 1) {
        const double z2n = std::pow(p.z, (double)(w - 1));
        for (size_t line = 0; line < (size_t)h * d; ++line)
            bspline_prefilter_line(c.data() + line * w, w, 1, p, z2n);
    }
    if (h > 1) {
        const double z2n = std::pow(p.z, (double)(h - 1));
        for (unsigned zz = 0; zz < d; ++zz)
            for (unsigned x = 0; x < w; ++x)
                bspline_prefilter_line(c.data() + zz * wh + x, h, w, p, z2n);
    }
    if (d > 1) {
        const double z2n = std::pow(p.z, (double)(d - 1));
        for (size_t col = 0; col < wh; ++col)
            bspline_prefilter_line(c.data() + col, d, wh, p, z2n);
    }
    const BSplineAxis ax = bspline_axis(w, gW, W), ay = bspline_axis(h, gH, H),
                      az = bspline_axis(d, gD, D);
#pragma omp parallel for schedule(static)
    for (long zo = 0; zo < (long)D; ++zo)
        for (unsigned yo = 0; yo < H; ++yo)
            for (unsigned xo = 0; xo < W; ++xo) {
                float v = 0.f;  // the resample filter's default pixel value outside
                if (ax.inside[xo] && ay.inside[yo] && az.inside[zo]) {
                    // the 64 points with x fastest, weight = ((1 * wx) * wy) * wz
                    double acc = 0.0;
                    for (int k = 0; k < 4; ++k)
                        for (int j = 0; j < 4; ++j)
                            for (int i = 0; i < 4; ++i) {
                                double wgt = 1.0;
                                wgt = wgt * ax.wt[4 * (size_t)xo + i];
                                wgt = wgt * ay.wt[4 * (size_t)yo + j];
                                wgt = wgt * az.wt[4 * (size_t)zo + k];
                                const size_t q = (size_t)az.idx[4 * (size_t)zo + k] * wh +
                                                 (size_t)ay.idx[4 * (size_t)yo + j] * w +
                                                 (size_t)ax.idx[4 * (size_t)xo + i];
                                acc = acc + wgt * c[q];
                            }
                    v = (float)acc;
                }
                out[((size_t)zo * H + yo) * W + xo] = v;
            }
}

}  // namespace oracle
