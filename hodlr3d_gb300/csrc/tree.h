// Host launchers of the device tree build (tree.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace h3d {

void launch_leaf_keys(cudaStream_t s, int64_t n, const double* xyz, int levels, const double* radii,
                      uint32_t* keys, int32_t* vals);
// stable sort of (key, value) by key; counts needs 256 * ceil(n / 1024) ints
void radix_sort_pairs(cudaStream_t s, int64_t n, int key_bits, uint32_t* keys, int32_t* vals,
                      uint32_t* keys_tmp, int32_t* vals_tmp, int32_t* counts, int* launches);
void launch_leaf_offsets(cudaStream_t s, int64_t n, const uint32_t* keys, int64_t nleaf,
                         int32_t* leaf_off);
void launch_gather_points(cudaStream_t s, int64_t n, const double* xyz, const int32_t* perm,
                          const uint32_t* leaf_of, int levels, const double* radii, double* xs,
                          double* ys, double* zs, float* xl, float* yl, float* zl);
void launch_leaf_centres(cudaStream_t s, int64_t nleaf, int levels, const double* radii, double* c);
void launch_box_lists(cudaStream_t s, int j, int mode, int32_t* nbr_all, int32_t* il_count,
                      const int64_t* il_ptr, int32_t* pair_tgt, int32_t* pair_src);
void launch_reverse_pairs(cudaStream_t s, int64_t npairs, const int32_t* pair_tgt,
                          const int32_t* pair_src, const int64_t* il_ptr, int32_t* rev,
                          int32_t* err);

}  // namespace h3d
