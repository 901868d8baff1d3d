// batch_launch.cuh -- to_map / to_weight_map of many observations into one
// map in one persistent launch.
//
// The work items of all observations -- (observation, piece of `piece`
// samples, detector), numbered observation by observation and piece by
// piece -- are shared out statically over the resident blocks (item w goes
// to block w mod gridDim.x).  Each item runs the same per-piece code as
// so3g_proj_to_map.
//
// Shared by the entry points of batch.cu (to_map) and batch_weight.cu
// (to_weight_map): two translation units, so that each compiles only its
// own kernel instantiations.
#pragma once

#include "scatter_kernel.cuh"

namespace so3g {

namespace {

template <int C, int P, bool WEIGHT, int MODE>
__global__ void __launch_bounds__(kBlock, PointingVariant<C, P, MODE>::mixed && MODE == 2
                                              ? kMixedBlocksPerSM
                                              : kScatterBlocksPerSM)
    k_scatter_batch(ScatterArgs base, const so3g_obs *obs, int n_obs,
                    const long long *work_off, long long n_work) {
    __shared__ int s_queue[QueueInts<C, P, MODE>::value];
    __shared__ WarpPiece s_wp[kBlock / 32];
    for (long long w = blockIdx.x; w < n_work; w += gridDim.x) {
        // The observation holding item w: largest o with work_off[o] <= w.
        int lo = 0, hi = n_obs - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(work_off + mid) <= w) lo = mid;
            else hi = mid - 1;
        }
        const so3g_obs ob = obs[lo];
        const long long item = w - __ldg(work_off + lo);
        const int pieces = (ob.n_time + base.piece - 1) / base.piece;
        if (pieces <= 0 || ob.n_det <= 0) continue;   // never for a consistent plan
        // Piece-major: consecutive items are different detectors over the
        // same samples, so the blocks running at once spread their atomics
        // over the focal plane's footprint instead of one detector's track.
        const int pc = (int)(item / ob.n_det);
        const int det = (int)(item - (long long)pc * ob.n_det);
        const int t0 = pc * base.piece;
        const int t1 = min(ob.n_time, t0 + base.piece);
        if (pc >= pieces || t0 >= t1) continue;   // never for a consistent plan
        ScatterArgs a = base;
        a.bore = ob.boresight;
        a.dets = ob.dets;
        a.resp = ob.response;
        a.signal = ob.signal;
        a.sig_stride = ob.sig_det_stride;
        a.det_weights = ob.det_weights;
        scatter_piece<C, P, WEIGHT, MODE>(a, det, t0, t1, s_queue, s_wp);
    }
}

template <bool WEIGHT>
struct BatchLaunch {
    ScatterArgs a;
    const so3g_obs *obs;
    int n_obs;
    const long long *work_off;
    long long n_work;
    int blocks;
    cudaStream_t stream;
    int sms;
    template <int C, int P>
    struct Go {
        BatchLaunch *L;
        template <int MODE>
        int go() {
            long long grid = L->blocks;
            if (L->blocks < 0) {
                // One block per work item, scheduled by the hardware.
                grid = L->n_work;
            } else if (L->blocks == 0) {
                // One full wave: every block resident at once.
                int per_sm = 0;
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    &per_sm, k_scatter_batch<C, P, WEIGHT, MODE>, kBlock, 0);
                grid = (long long)(per_sm > 0 ? per_sm : 1) * L->sms;
            }
            if (grid > L->n_work) grid = L->n_work;
            if (grid > 0x7fffffffLL)
                return set_error(SO3G_ERR_RANGE, "batch of %lld work items: too many blocks",
                                 grid);
            k_scatter_batch<C, P, WEIGHT, MODE><<<(unsigned)grid, kBlock, 0, L->stream>>>(
                L->a, L->obs, L->n_obs, L->work_off, L->n_work);
            return after_launch(WEIGHT ? "to_weight_map batch" : "to_map batch");
        }
    };
    template <int C, int P>
    int run() {
        Go<C, P> g{this};
        return by_mode<C, P>(a.fast, g);
    }
};

template <bool WEIGHT>
int batch_entry(const so3g_pixelization *pz, const so3g_obs *obs, int32_t n_obs,
                const int64_t *work_offset, int64_t n_work, int32_t piece, int32_t blocks,
                const so3g_map *map, int32_t accum, int32_t *err, void *stream) {
    clear_error();
    BatchLaunch<WEIGHT> L;
    int rc = make_geom(pz, &L.a.g);
    if (rc) return rc;
    rc = attach_map(pz, map, &L.a.g);
    if (rc) return rc;
    if (accum != SO3G_ACCUM_ATOMIC && accum != SO3G_ACCUM_WARP_RUNS)
        return set_error(SO3G_ERR_ARGUMENT, "unknown accumulation mode %d", accum);
    if (n_obs < 0 || n_work < 0) return set_error(SO3G_ERR_ARGUMENT, "negative size");
    if (n_obs == 0 || n_work == 0) return SO3G_OK;
    if (!obs || !work_offset) return set_error(SO3G_ERR_ARGUMENT, "NULL observation table");
    if (piece < 256 || piece % 256)
        return set_error(SO3G_ERR_ARGUMENT, "piece must be a positive multiple of 256");
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    L.blocks = blocks;
    L.sms = sms > 0 ? sms : 1;
    L.a.bore = nullptr;
    L.a.dets = nullptr;
    L.a.resp = nullptr;
    L.a.signal = nullptr;
    L.a.sig_stride = 0;
    L.a.det_weights = nullptr;
    L.a.segs = Segs{nullptr, 0};
    L.a.piece = piece;
    L.a.accum = accum;
    L.a.err = err;
    L.a.map = map->data;
    L.a.ft = device_fast_tables();
    L.a.fc = make_fast_const(L.a.g);
    L.a.mc = make_mixed_const(L.a.g);
    L.a.bore32 = nullptr;   // per-observation boresights: converted in the kernel
    L.a.fast = fast_mode(pz, L.a.ft);
    L.obs = obs;
    L.n_obs = n_obs;
    L.work_off = reinterpret_cast<const long long *>(work_offset);
    L.n_work = n_work;
    L.stream = (cudaStream_t)stream;
    return dispatch_cp(pz->coord_sys, pix_kind(pz), L);
}

}  // namespace

}  // namespace so3g

