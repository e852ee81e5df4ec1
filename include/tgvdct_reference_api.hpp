// tgvdct_reference_api.hpp — the reference's launcher templates, with their exact
// signatures, implemented over the tgvdct C ABI (libtgvdct_refapi.so).
//
// A C++ program written against josefkoller/ambient_image_processor's launchers
// keeps its call sites: it includes this header (or keeps its own forward
// declarations, which these match) and links libtgvdct_refapi.so instead of the
// reference's .cu objects.  Each template below is explicitly instantiated for
// float and double, as the reference instantiates its own.
//
// Semantics kept from the reference:
//   - host buffers in, new[] host buffers out (the caller delete[]s them);
//   - tgv2_l1_deshade_launch allocates *v_z even when depth == 1
//     (tgv_deshade/tgv2_l1_deshade.cu:289) and runs the 3-D operators then;
//   - the iteration callback gets host copies of u (and v) after iteration i
//     when i > 0 and i % paint_iteration_interval == 0
//     (tgv_cuda/tgv2_common.cu:381-384); returning true stops the loop;
//   - on a failure the reference prints and exits (cudaCheckError,
//     source/modules/cuda/cuda_helper.in:11-21); these do the same unless
//     tgvdct_refapi_throw_on_error(true) was called, after which they throw
//     std::runtime_error instead.
// Differences:
//   - the computation is FP32 on the GPU for both instantiations (the double one
//     converts in and out: the reference's double instantiation narrows its
//     steps and cosines to float as well);
//   - cuda_block_dimension is accepted and ignored (launch shapes are sm_103a's).
#ifndef TGVDCT_REFERENCE_API_HPP
#define TGVDCT_REFERENCE_API_HPP

#include <sys/types.h>

#include <functional>
#include <vector>

// tgv_deshade/tgv2_l1_deshade.cu:28-30
template <typename Pixel>
using DeshadeIterationCallback = std::function<bool(uint iteration_index, uint iteration_count,
                                                    Pixel* u, Pixel* v_x, Pixel* v_y, Pixel* v_z)>;
// tgv_cuda/tgv_common_2d.cu:34-36
template <typename Pixel>
using DeshadeIterationCallback2D =
    std::function<bool(uint iteration_index, uint iteration_count, Pixel* u, Pixel* v_x, Pixel* v_y)>;
// tgv_cuda/tgv_common.cu:29-30
template <typename Pixel>
using IterationCallback = std::function<bool(uint iteration_index, uint iteration_count, Pixel* u)>;

// tgv_deshade/tgv2_l1_deshade.cu:33-41
template <typename Pixel>
Pixel* tgv2_l1_deshade_launch(Pixel* f_host, uint width, uint height, uint depth, Pixel lambda,
                              uint iteration_count, uint paint_iteration_interval,
                              const int cuda_block_dimension,
                              DeshadeIterationCallback<Pixel> iteration_finished_callback,
                              Pixel alpha0, Pixel alpha1, Pixel** v_x_host, Pixel** v_y_host,
                              Pixel** v_z_host);

// tgv_deshade/tgv2_l1_deshade_2d.cu:29-36
template <typename Pixel>
Pixel* tgv2_l1_deshade_launch_2d(Pixel* f_host, uint width, uint height, Pixel lambda,
                                 uint iteration_count, uint paint_iteration_interval,
                                 DeshadeIterationCallback2D<Pixel> iteration_finished_callback,
                                 Pixel alpha0, Pixel alpha1, Pixel** v_x_host, Pixel** v_y_host);

// tgv_cuda/tgv2_l1.cu:64-72
template <typename Pixel>
Pixel* tgv2_l1_launch(Pixel* f_host, uint width, uint height, uint depth, Pixel lambda,
                      uint iteration_count, uint paint_iteration_interval,
                      IterationCallback<Pixel> iteration_finished_callback, Pixel alpha0,
                      Pixel alpha1);

// tgv_cuda/tgv2_l2.cu:60-68
template <typename Pixel>
Pixel* tgv2_l2_launch(Pixel* f_host, uint width, uint height, uint depth, Pixel lambda,
                      uint iteration_count, uint paint_iteration_interval,
                      IterationCallback<Pixel> iteration_finished_callback, Pixel alpha0,
                      Pixel alpha1);

// cuda_image_operations/divergence.cu:59-61 (is_host_data == false: dx, dy, dz
// are device buffers; the result is a new[] host buffer either way)
template <typename Pixel>
Pixel* divergence_kernel_launch(Pixel* dx, Pixel* dy, Pixel* dz, const uint width,
                                const uint height, const uint depth, bool is_host_data = false);

// cuda_image_operations/cosine_transform.cu:226-227
template <typename Pixel>
Pixel* cosine_transform_kernel_launch(Pixel* image_host, uint width, uint height, uint depth);

// cuda_image_operations/inverse_cosine_transform.cu:167-168
template <typename Pixel>
Pixel* inverse_cosine_transform_kernel_launch(Pixel* image_host, uint width, uint height,
                                              uint depth);

// cuda_image_operations/solve_poisson_in_cosine_domain.cu:86-87
template <typename Pixel>
Pixel* solve_poisson_in_cosine_domain_kernel_launch(Pixel* image_host, uint width, uint height,
                                                    uint depth);

// tgv_deshade_masked/tgv2_l1_deshade_masked.cu and tgv2_l1_deshade_masked_2d.cu: the
// masked loop over the voxels listed in masked_pixel_indices.  The face lists are
// accepted for signature compatibility; they follow from the shape.
template <typename Pixel>
Pixel* tgv2_l1_deshade_masked_launch(
    Pixel* f_host, uint width, uint height, uint depth, Pixel lambda, uint iteration_count,
    uint paint_iteration_interval, const int cuda_block_dimension,
    DeshadeIterationCallback<Pixel> iteration_finished_callback, Pixel alpha0, Pixel alpha1,
    Pixel** v_x_host, Pixel** v_y_host, Pixel** v_z_host,
    const std::vector<uint>& masked_pixel_indices, const std::vector<uint>& left_edge_pixel_indices,
    const std::vector<uint>& not_left_edge_pixel_indices,
    const std::vector<uint>& right_edge_pixel_indices,
    const std::vector<uint>& not_right_edge_pixel_indices,
    const std::vector<uint>& top_edge_pixel_indices,
    const std::vector<uint>& not_top_edge_pixel_indices,
    const std::vector<uint>& bottom_edge_pixel_indices,
    const std::vector<uint>& not_bottom_edge_pixel_indices,
    const std::vector<uint>& front_edge_pixel_indices,
    const std::vector<uint>& not_front_edge_pixel_indices,
    const std::vector<uint>& back_edge_pixel_indices,
    const std::vector<uint>& not_back_edge_pixel_indices);

template <typename Pixel>
Pixel* tgv2_l1_deshade_masked_2d_launch(
    Pixel* f_host, uint width, uint height, Pixel lambda, uint iteration_count,
    uint paint_iteration_interval, const int cuda_block_dimension,
    DeshadeIterationCallback2D<Pixel> iteration_finished_callback, Pixel alpha0, Pixel alpha1,
    Pixel** v_x_host, Pixel** v_y_host, const std::vector<uint>& masked_pixel_indices,
    const std::vector<uint>& left_edge_pixel_indices,
    const std::vector<uint>& not_left_edge_pixel_indices,
    const std::vector<uint>& right_edge_pixel_indices,
    const std::vector<uint>& not_right_edge_pixel_indices,
    const std::vector<uint>& top_edge_pixel_indices,
    const std::vector<uint>& not_top_edge_pixel_indices,
    const std::vector<uint>& bottom_edge_pixel_indices,
    const std::vector<uint>& not_bottom_edge_pixel_indices);

// Failure handling of the functions above: false (default) prints the error and
// exits like the reference; true throws std::runtime_error.
void tgvdct_refapi_throw_on_error(bool enable);

#endif  // TGVDCT_REFERENCE_API_HPP
