// tgv2_deshade_application: the reference's terminal program
// (source/terminal_programs/tgv2_deshade_main.cpp) on libtgvdct.
//
//   tgv2_deshade_application input lambda alpha0 alpha1 iteration_count
//       cuda_block_dimension [mask] output_denoised output_shading output_deshaded
//
// Same positional arguments, defaults and exit codes (1 usage, 2 missing input,
// 3 missing mask).  Negative deshaded values are set to zero, as the reference
// program does; with a mask it runs the masked deshade with the background added
// back.  Options (anywhere on the line):
//   --data-term=l1|l2     data term of the TGV loop (l1)
//   --tau=T --sigma=S     primal / dual steps (1/sqrt(20))
//   --log-domain          deshade log(f) and exponentiate u, l, r
//   --precision=fp32|bf16|fx16   storage of the dual fields p, q (fp32)
//   --dct=fp32|tf32|bf16x3       DCT contractions (fp32)
//   --eigen=reference|accurate   Laplacian eigenvalues (reference)
//   --no-clamp            keep negative deshaded values
//   --raw=WxHxD           read input (and mask) as headerless float32
// Files: .mha / .mhd MetaImage (uncompressed), or .raw float32.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "metaimage.hpp"
#include "tgvdct.h"

namespace {

void print_usage() {
    std::cout << "parameter: input_image_path lambda alpha0 alpha1 iteration_count "
                 "cuda_block_dimension [mask] output_denoised_path output_shading_path "
                 "output_deshaded_path [--data-term=l1|l2] [--tau=T] [--sigma=S] [--log-domain] "
                 "[--precision=fp32|bf16|fx16] [--dct=fp32|tf32|bf16x3] "
                 "[--eigen=reference|accurate] [--no-clamp] [--raw=WxHxD]"
              << std::endl;
}

bool option(const std::string& arg, const char* name, std::string& value) {
    const std::string key = std::string("--") + name + "=";
    if (arg.compare(0, key.size(), key) != 0) return false;
    value = arg.substr(key.size());
    return true;
}

}  // namespace

int main(int argc, char* argv[]) {
    std::vector<std::string> pos;
    tgvdct_params p;
    tgvdct_params_init(&p);
    bool log_domain = false, clamp = true;
    std::string raw_dims;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        std::string v;
        if (a.compare(0, 2, "--") != 0) pos.push_back(a);
        else if (option(a, "data-term", v)) p.data_term = v == "l2" ? TGVDCT_DATA_L2 : TGVDCT_DATA_L1;
        else if (option(a, "tau", v)) p.tau = std::stof(v);
        else if (option(a, "sigma", v)) p.sigma = std::stof(v);
        else if (a == "--log-domain") log_domain = true;
        else if (a == "--no-clamp") clamp = false;
        else if (option(a, "precision", v))
            p.state_precision = v == "bf16"   ? TGVDCT_STATE_BF16_DUAL
                                : v == "fx16" ? TGVDCT_STATE_FX16_DUAL
                                              : TGVDCT_STATE_FP32;
        else if (option(a, "dct", v))
            p.dct_mode = v == "tf32" ? TGVDCT_DCT_TF32 : v == "bf16x3" ? TGVDCT_DCT_BF16X3 : TGVDCT_DCT_FP32;
        else if (option(a, "eigen", v))
            p.poisson_eigen = v == "accurate" ? TGVDCT_EIGEN_ACCURATE : TGVDCT_EIGEN_REFERENCE;
        else if (option(a, "raw", v)) raw_dims = v;
        else {
            std::cerr << "unknown option " << a << std::endl;
            print_usage();
            return 1;
        }
    }
    // argc < 9 in the reference counts the program name: 8 positional values
    if (pos.size() < 8) {
        print_usage();
        return 1;
    }
    const bool mask_given = pos.size() == 10;
    const std::string input_path = pos[0];
    p.lambda = std::stof(pos[1]);
    p.alpha0 = std::stof(pos[2]);
    p.alpha1 = std::stof(pos[3]);
    p.iteration_count = (uint32_t)std::stoi(pos[4]);
    (void)std::stoi(pos[5]);  // cuda_block_dimension: launch shapes are chosen for sm_103a
    const std::string mask_path = mask_given ? pos[6] : "";
    const std::string out_u = pos[mask_given ? 7 : 6];
    const std::string out_l = pos[mask_given ? 8 : 7];
    const std::string out_r = pos[mask_given ? 9 : 8];

    tgvdct_io::Volume f, mask;
    try {
        f = tgvdct_io::read_volume(input_path, raw_dims);
    } catch (const std::exception& e) {
        std::cerr << "input image file does not exist: " << input_path << " (" << e.what() << ")"
                  << std::endl;
        return 2;
    }
    if (mask_given) {
        try {
            mask = tgvdct_io::read_volume(mask_path, raw_dims);
        } catch (const std::exception& e) {
            std::cerr << "mask image file does not exist: " << mask_path << " (" << e.what() << ")"
                      << std::endl;
            return 3;
        }
        if (mask.count() != f.count()) {
            std::cerr << "mask size differs from the input size" << std::endl;
            return 3;
        }
    }
    p.width = f.width;
    p.height = f.height;
    p.depth = f.depth;

    tgvdct_io::Volume u = f, l = f, r = f;
    tgvdct_status st;
    if (mask_given) {
        // the masked processor as the reference program calls it: clamp and
        // background add-back on (tgv2_deshade_main.cpp:73-86)
        st = tgvdct_process_tgv2_l1_masked(&p, f.voxels.data(), mask.voxels.data(), clamp ? 1 : 0,
                                           1, log_domain ? 1 : 0, nullptr, nullptr,
                                           u.voxels.data(), l.voxels.data(), r.voxels.data());
    } else {
        st = tgvdct_process_tgv2_l1(&p, f.voxels.data(), nullptr, clamp ? 1 : 0, 0,
                                    log_domain ? 1 : 0, nullptr, nullptr, u.voxels.data(),
                                    l.voxels.data(), r.voxels.data());
    }
    if (st != TGVDCT_OK) {
        std::cerr << "tgvdct: " << tgvdct_status_string(st) << ": " << tgvdct_last_error()
                  << std::endl;
        return 10 + (int)st;
    }
    try {
        tgvdct_io::write_volume(out_u, u);
        tgvdct_io::write_volume(out_l, l);
        tgvdct_io::write_volume(out_r, r);
    } catch (const std::exception& e) {
        std::cerr << e.what() << std::endl;
        return 4;
    }
    return 0;
}
