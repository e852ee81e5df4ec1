// tgv2_deshade_convergence_test_application: the reference's convergence test
// program (source/terminal_programs/tgv2_deshade_convergence_test_main.cpp) on
// libtgvdct.
//
//   tgv2_deshade_convergence_test_application input lambda alpha0 alpha1 iteration_count
//       [mask] output_metric_file
//
// Runs the deshade loop with a check after every iteration and writes the total
// variation of the two metric series (normalised cross-correlation of the shading
// field between checks, and its time total variation), one value per line, as
// TGVDeshadeProcessor::processTGV2L1DeshadeCuda_convergenceTestToFile does.  Exit
// codes as the reference: 1 usage, 2 missing input, 3 missing mask.
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "metaimage.hpp"
#include "tgvdct.h"

int main(int argc, char* argv[]) {
    std::vector<std::string> pos;
    std::string raw_dims;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a.compare(0, 6, "--raw=") == 0) raw_dims = a.substr(6);
        else pos.push_back(a);
    }
    if (pos.size() < 6) {  // argc < 8 in the reference, which counts the program name
        std::cout << "parameter: input_image_path lambda alpha0 alpha1 iteration_count [mask] "
                     "output_metric_file_name [--raw=WxHxD]"
                  << std::endl;
        return 1;
    }
    const bool mask_given = pos.size() == 7;
    tgvdct_params p;
    tgvdct_params_init(&p);
    p.lambda = std::stof(pos[1]);
    p.alpha0 = std::stof(pos[2]);
    p.alpha1 = std::stof(pos[3]);
    p.iteration_count = (uint32_t)std::stoi(pos[4]);
    const std::string out_path = pos[mask_given ? 6 : 5];
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
    p.width = f.width;
    p.height = f.height;
    p.depth = f.depth;
    double metric_tv[2] = {0, 0};
    const tgvdct_status st = tgvdct_convergence_test(&p, f.voxels.data(),
                                                     mask_given ? mask.voxels.data() : nullptr, 1,
                                                     nullptr, nullptr, 0, nullptr, metric_tv);
    if (st != TGVDCT_OK) {
        std::cerr << "tgvdct: " << tgvdct_status_string(st) << ": " << tgvdct_last_error()
                  << std::endl;
        return 10 + (int)st;
    }
    std::ofstream out(out_path);
    out.precision(9);
    out << metric_tv[0] << std::endl << metric_tv[1] << std::endl;
    return out ? 0 : 4;
}
