// scatter_launch.cuh -- launch of the to_map / to_weight_map kernels for
// the entry points of scatter.cu (to_map) and scatter_weight.cu
// (to_weight_map): two translation units, so that each compiles only its
// own kernel instantiations.
#pragma once

#include "mixed_launch.cuh"

namespace so3g {

namespace {

template <bool WEIGHT>
struct ScatterLaunch {
    ScatterArgs a;
    dim3 grid;
    cudaStream_t stream;
    template <int C, int P>
    struct Go {
        ScatterLaunch *L;
        template <int MODE>
        int go() {
            if constexpr (MODE == SO3G_POINTING_MIXED) {
                // Untiled nearest-neighbour maps: the float32 tier alone, its
                // fallback in a second pass (mixed_launch.cuh).
                const int rc = scatter_mixed<C, P, WEIGHT>(L->a, L->grid, L->stream);
                if (rc != 1) return rc;
            }
            k_scatter<C, P, WEIGHT, MODE><<<L->grid, kBlock, 0, L->stream>>>(L->a);
            return after_launch(WEIGHT ? "to_weight_map" : "to_map");
        }
    };
    template <int C, int P>
    int run() {
        Go<C, P> g{this};
        return by_mode<C, P>(a.fast, g);
    }
};

template <bool WEIGHT>
int scatter_entry(const so3g_pixelization *pz, const double *bore, int32_t n_time,
                  const double *dets, int32_t n_det, const float *response,
                  const float *signal, int64_t sig_det_stride, const float *det_weights,
                  const so3g_ranges *ranges, const so3g_map *map, int32_t accum, int32_t *err,
                  void *stream) {
    clear_error();
    ScatterLaunch<WEIGHT> L;
    int rc = make_geom(pz, &L.a.g);
    if (rc) return rc;
    rc = attach_map(pz, map, &L.a.g);
    if (rc) return rc;
    if (n_det < 0 || n_time < 0) return set_error(SO3G_ERR_ARGUMENT, "negative n_det or n_time");
    if (accum != SO3G_ACCUM_ATOMIC && accum != SO3G_ACCUM_WARP_RUNS)
        return set_error(SO3G_ERR_ARGUMENT, "unknown accumulation mode %d", accum);
    long long n_seg = ranges ? ranges->n_seg : n_det;
    long long max_len = ranges ? ranges->max_len : n_time;
    if (n_seg <= 0 || max_len <= 0) return SO3G_OK;
    if (ranges && !ranges->seg) return set_error(SO3G_ERR_ARGUMENT, "ranges->seg is NULL");
    if (!bore || !dets || !response || (!WEIGHT && !signal))
        return set_error(SO3G_ERR_ARGUMENT, "NULL input array");
    L.a.bore = bore;
    L.a.dets = dets;
    L.a.resp = response;
    L.a.signal = signal;
    L.a.sig_stride = sig_det_stride;
    L.a.det_weights = det_weights;
    L.a.segs = Segs{ranges ? ranges->seg : nullptr, n_time};
    L.a.piece = piece_len(max_len, n_seg);
    L.a.accum = accum;
    L.a.err = err;
    L.a.map = map->data;
    L.a.ft = device_fast_tables();
    L.a.fc = make_fast_const(L.a.g);
    L.a.mc = make_mixed_const(L.a.g);
    L.a.fast = fast_mode(pz, L.a.ft);
    L.grid = dim3((unsigned)n_seg, (unsigned)((max_len + L.a.piece - 1) / L.a.piece));
    L.stream = (cudaStream_t)stream;
    L.a.bore32 = bore_f32(pz, L.a.fast, bore, n_time, L.stream);
    rc = dispatch_cp(pz->coord_sys, pix_kind(pz), L);
    bore_f32_free(L.a.bore32, L.stream);
    return rc;
}

}  // namespace

}  // namespace so3g

