// Test driver for libtgvdct_refapi.so: calls the reference-signature templates the
// way the reference's processors do and writes every result as raw float32 into
// an output directory, for tests/test_refapi_gpu.py to compare.
//
//   refapi_driver <in_dir> <out_dir> <width> <height> <depth> <lambda> <alpha0> <alpha1>
//                 <iterations>
// in_dir holds f.raw and mask.raw (float32, x fastest).
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "tgvdct_reference_api.hpp"

namespace {

std::vector<float> read_raw(const std::string& path, size_t n) {
    std::vector<float> v(n);
    std::ifstream in(path, std::ios::binary);
    in.read((char*)v.data(), (std::streamsize)(n * 4));
    if ((size_t)in.gcount() != n * 4) {
        std::fprintf(stderr, "short read: %s\n", path.c_str());
        std::exit(2);
    }
    return v;
}

template <class P>
void write_raw(const std::string& path, const P* data, size_t n) {
    std::vector<float> v(data, data + n);
    std::ofstream out(path, std::ios::binary);
    out.write((const char*)v.data(), (std::streamsize)(n * 4));
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 10) {
        std::fprintf(stderr, "usage: refapi_driver in out w h d lambda alpha0 alpha1 iterations\n");
        return 1;
    }
    tgvdct_refapi_throw_on_error(true);
    const std::string in = argv[1], out = argv[2];
    const uint w = (uint)std::atoi(argv[3]), h = (uint)std::atoi(argv[4]), d = (uint)std::atoi(argv[5]);
    const float lambda = (float)std::atof(argv[6]), a0 = (float)std::atof(argv[7]),
                a1 = (float)std::atof(argv[8]);
    const uint it = (uint)std::atoi(argv[9]);
    const size_t n = (size_t)w * h * d;
    std::vector<float> f = read_raw(in + "/f.raw", n), mask = read_raw(in + "/mask.raw", n);

    // the 3-D deshade loop, float, with a callback counting its calls
    uint calls = 0, last = 0;
    DeshadeIterationCallback<float> cb = [&](uint i, uint count, float* u, float*, float*, float* vz) {
        ++calls;
        last = i;
        return i >= count && u && vz;  // never stops
    };
    float *vx, *vy, *vz;
    float* u = tgv2_l1_deshade_launch<float>(f.data(), w, h, d, lambda, it, 7, 16, cb, a0, a1, &vx,
                                             &vy, &vz);
    write_raw(out + "/u.raw", u, n);
    write_raw(out + "/vx.raw", vx, n);
    write_raw(out + "/vy.raw", vy, n);
    write_raw(out + "/vz.raw", vz, n);
    std::printf("callbacks %u last %u\n", calls, last);

    // the same loop through the double instantiation
    std::vector<double> fd(f.begin(), f.end());
    double *dx, *dy, *dz;
    double* ud = tgv2_l1_deshade_launch<double>(fd.data(), w, h, d, lambda, it, it + 1, 16, nullptr,
                                                a0, a1, &dx, &dy, &dz);
    write_raw(out + "/u_double.raw", ud, n);

    // Poisson integration as TGVDeshadeProcessor chains the launchers
    float* div = divergence_kernel_launch<float>(vx, vy, vz, w, h, d, true);
    float* c = cosine_transform_kernel_launch<float>(div, w, h, d);
    float* s = solve_poisson_in_cosine_domain_kernel_launch<float>(c, w, h, d);
    float* l = inverse_cosine_transform_kernel_launch<float>(s, w, h, d);
    write_raw(out + "/l.raw", l, n);

    // the TGV filter's denoise loops
    float* u1 = tgv2_l1_launch<float>(f.data(), w, h, d, lambda, it, 0, nullptr, a0, a1);
    float* u2 = tgv2_l2_launch<float>(f.data(), w, h, d, lambda, it, 0, nullptr, a0, a1);
    write_raw(out + "/u_l1.raw", u1, n);
    write_raw(out + "/u_l2.raw", u2, n);

    // the masked loop with the index lists TGVDeshadeMaskedProcessor builds
    std::vector<uint> inside, e[6], ne[6];
    for (uint z = 0; z < d; ++z)
        for (uint y = 0; y < h; ++y)
            for (uint x = 0; x < w; ++x) {
                const uint i = (z * h + y) * w + x;
                if (mask[i] < 1) continue;
                inside.push_back(i);
                const bool on[6] = {x == 0, x == w - 1, y == 0, y == h - 1, z == 0, z == d - 1};
                for (int k = 0; k < 6; ++k) (on[k] ? e[k] : ne[k]).push_back(i);
            }
    float *mx, *my, *mz;
    float* um;
    if (d > 1) {
        um = tgv2_l1_deshade_masked_launch<float>(f.data(), w, h, d, lambda, it, it + 1, 16,
                                                  nullptr, a0, a1, &mx, &my, &mz, inside, e[0],
                                                  ne[0], e[1], ne[1], e[2], ne[2], e[3], ne[3],
                                                  e[4], ne[4], e[5], ne[5]);
    } else {
        um = tgv2_l1_deshade_masked_2d_launch<float>(f.data(), w, h, lambda, it, it + 1, 16,
                                                     nullptr, a0, a1, &mx, &my, inside, e[0],
                                                     ne[0], e[1], ne[1], e[2], ne[2], e[3], ne[3]);
        mz = new float[n]();
    }
    write_raw(out + "/u_masked.raw", um, n);
    write_raw(out + "/vx_masked.raw", mx, n);

    for (float* p : {u, vx, vy, vz, div, c, s, l, u1, u2, um, mx, my, mz}) delete[] p;
    for (double* p : {ud, dx, dy, dz}) delete[] p;
    return 0;
}
