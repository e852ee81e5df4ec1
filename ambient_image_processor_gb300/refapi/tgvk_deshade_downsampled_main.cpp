// tgvk_deshade_downsampled_application: the reference's down-sampled deshade program
// (source/terminal_programs/tgvk_deshade_downsampled_main.cpp) on libtgvdct.
//
//   tgvk_deshade_downsampled_application input f_downsampling order lambda iteration_count
//       [mask] output_image_prefix [--raw=WxHxD]
//
// Resizes the input (times the mask) and the mask by f_downsampling with cubic
// B-splines, deshades there with alpha = (1, 2, ..., order), the clamp and the
// background add-back, resizes the shading back and writes
// <prefix>_shading.mha and <prefix>_deshaded.mha, as the reference does with
// TGVKDeshadeDownsampledProcessor.  Order 2 is what this library builds; other
// orders exit with an error.  Exit codes as the reference: 1 usage, 2 missing
// input, 3 missing mask; 10 + status for a library error, 4 for a write error.
#include <chrono>
#include <iostream>
#include <string>
#include <vector>

#include "metaimage.hpp"
#include "tgvdct.h"

int main(int argc, char* argv[]) {
    std::cout << "started program: " << argv[0] << std::endl;
    std::vector<std::string> pos;
    std::string raw_dims;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a.compare(0, 6, "--raw=") == 0) raw_dims = a.substr(6);
        else pos.push_back(a);
    }
    if (pos.size() < 6) {  // argc < 7 in the reference, which counts the program name
        std::cout << "parameter: input_image_path f_downsampling order lambda iteration_count "
                     "[mask] output_image_prefix [--raw=WxHxD]"
                  << std::endl;
        return 1;
    }
    const float f_downsampling = std::stof(pos[1]);
    const uint32_t order = (uint32_t)std::stoi(pos[2]);
    const float lambda = std::stof(pos[3]);
    const uint32_t iteration_count = (uint32_t)std::stoi(pos[4]);
    const bool mask_given = pos.size() == 7;
    const std::string prefix = pos[mask_given ? 6 : 5];
    tgvdct_io::Volume f, mask;
    try {
        f = tgvdct_io::read_volume(pos[0], raw_dims);
    } catch (const std::exception& e) {
        std::cerr << "input image file does not exist: " << pos[0] << " (" << e.what() << ")"
                  << std::endl;
        return 2;
    }
    if (mask_given) {
        try {
            mask = tgvdct_io::read_volume(pos[5], raw_dims);
        } catch (const std::exception& e) {
            std::cerr << "mask image file does not exist: " << pos[5] << " (" << e.what() << ")"
                      << std::endl;
            return 3;
        }
        if (mask.count() != f.count()) {
            std::cerr << "mask size differs from the input size" << std::endl;
            return 3;
        }
    }
    std::vector<float> alpha(order);
    for (uint32_t i = 0; i < order; ++i) alpha[i] = (float)(i + 1);
    tgvdct_io::Volume shading = f, deshaded = f, denoised = f;
    const auto start = std::chrono::system_clock::now();
    const tgvdct_status st = tgvdct_process_tgvk_l1_downsampled(
        f.voxels.data(), mask_given ? mask.voxels.data() : nullptr, f.width, f.height, f.depth,
        f_downsampling, lambda, order, alpha.data(), iteration_count, 1, 1, 0,
        iteration_count + 1, nullptr, nullptr, denoised.voxels.data(), shading.voxels.data(),
        deshaded.voxels.data(), nullptr);
    const std::chrono::duration<double> elapsed = std::chrono::system_clock::now() - start;
    if (st != TGVDCT_OK) {
        std::cerr << "tgvdct: " << tgvdct_status_string(st) << ": " << tgvdct_last_error()
                  << std::endl;
        return 10 + (int)st;
    }
    std::cout << "elapsed time: " << elapsed.count() << "s" << std::endl;
    try {
        tgvdct_io::write_volume(prefix + "_shading.mha", shading);
        tgvdct_io::write_volume(prefix + "_deshaded.mha", deshaded);
    } catch (const std::exception& e) {
        std::cerr << e.what() << std::endl;
        return 4;
    }
    return 0;
}
