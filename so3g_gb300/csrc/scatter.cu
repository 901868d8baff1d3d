// scatter.cu -- the to_map entry point: per-sample pointing, float32
// products and float64 accumulation into the map (the kernel is in
// scatter_kernel.cuh, its launch in scatter_launch.cuh).

#include "scatter_launch.cuh"

extern "C" {

int so3g_proj_to_map(const so3g_pixelization *pz, const double *boresight, int32_t n_time,
                     const double *dets, int32_t n_det, const float *response,
                     const float *signal, int64_t sig_det_stride, const float *det_weights,
                     const so3g_ranges *ranges, const so3g_map *map, int32_t accum,
                     int32_t *err, void *stream) {
    return so3g::scatter_entry<false>(pz, boresight, n_time, dets, n_det, response, signal,
                                      sig_det_stride, det_weights, ranges, map, accum, err,
                                      stream);
}

}  // extern "C"
