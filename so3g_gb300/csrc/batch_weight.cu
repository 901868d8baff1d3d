// batch_weight.cu -- the batched to_weight_map entry point (the kernel and
// its launch are in batch_launch.cuh).

#include "batch_launch.cuh"

extern "C" {

int so3g_proj_to_weight_map_batch(const so3g_pixelization *pz, const so3g_obs *obs,
                                  int32_t n_obs, const int64_t *work_offset, int64_t n_work,
                                  int32_t piece, int32_t blocks, const so3g_map *map,
                                  int32_t accum, int32_t *err, void *stream) {
    return so3g::batch_entry<true>(pz, obs, n_obs, work_offset, n_work, piece, blocks, map,
                                   accum, err, stream);
}

}  // extern "C"
