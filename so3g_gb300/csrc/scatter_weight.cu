// scatter_weight.cu -- the to_weight_map entry point (the kernel is in
// scatter_kernel.cuh, its launch in scatter_launch.cuh).

#include "scatter_launch.cuh"

extern "C" {

int so3g_proj_to_weight_map(const so3g_pixelization *pz, const double *boresight,
                            int32_t n_time, const double *dets, int32_t n_det,
                            const float *response, const float *det_weights,
                            const so3g_ranges *ranges, const so3g_map *map, int32_t accum,
                            int32_t *err, void *stream) {
    return so3g::scatter_entry<true>(pz, boresight, n_time, dets, n_det, response, nullptr, 0,
                                     det_weights, ranges, map, accum, err, stream);
}

}  // extern "C"
