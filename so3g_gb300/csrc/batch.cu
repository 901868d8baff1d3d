// batch.cu -- the batched to_map entry point and the work-item offsets
// (the kernel and its launch are in batch_launch.cuh).

#include "batch_launch.cuh"

extern "C" {

int64_t so3g_batch_work_offsets(const so3g_obs *obs, int32_t n_obs, int32_t piece,
                                int64_t *work_offset) {
    if (!obs || !work_offset || n_obs < 0 || piece <= 0) return -1;
    int64_t total = 0;
    for (int o = 0; o < n_obs; o++) {
        work_offset[o] = total;
        const int64_t pieces = ((int64_t)obs[o].n_time + piece - 1) / piece;
        total += (int64_t)obs[o].n_det * pieces;
    }
    work_offset[n_obs] = total;
    return total;
}

int so3g_proj_to_map_batch(const so3g_pixelization *pz, const so3g_obs *obs, int32_t n_obs,
                           const int64_t *work_offset, int64_t n_work, int32_t piece,
                           int32_t blocks, const so3g_map *map, int32_t accum, int32_t *err,
                           void *stream) {
    return so3g::batch_entry<false>(pz, obs, n_obs, work_offset, n_work, piece, blocks, map,
                                    accum, err, stream);
}

}  // extern "C"
