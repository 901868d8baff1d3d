// gather.cu -- from_map: per-sample float64 pointing and a gather from the
// map, accumulated into the float32 signal exactly as the reference does
// (each term added in float64 and rounded to float32).

#include "host.h"

namespace so3g {

namespace {

struct GatherArgs {
    DGeom g;
    const double *bore;
    const double *dets;
    const float *resp;
    const double *map;
    float *signal;
    long long sig_stride;
    Segs segs;
    int piece;
    int *err;
};

template <int C, int P>
__global__ void __launch_bounds__(kBlock) k_from_map(GatherArgs a) {
    int det, t0, t1;
    if (!seg_piece(a.segs, a.piece, det, t0, t1)) return;
    const QuatD ofs = load_quat(a.dets + 4LL * det);
    const float T = __ldg(a.resp + 2 * det), Pr = __ldg(a.resp + 2 * det + 1);
    const int nc = a.g.ncomp;
    constexpr int NT = PixTraits<P>::taps;
    for (int t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
        double coords[4];
        float pf[3];
        int pix[NT][3];
        float w[NT];
        const QuatD qb = load_quat(a.bore + 4LL * t);
        get_coords<C>(a.g.lut, qb, ofs, coords);
        spin_factors(nc, coords, T, Pr, pf);
        float *sp = a.signal + det * a.sig_stride + t;
        float sig = *sp;
        int n = get_pixels<P>(a.g, coords, pix, w);
#pragma unroll
        for (int k = 0; k < NT; k++) {
            if (k >= n) break;
            long long off, plane;
            int bad = locate<P>(a.g, pix[k], &off, &plane);
            if (bad >= 0) {
                record_missing_tile(a.err, bad);
                continue;
            }
            // src/Projection.cxx:1763-1765
#pragma unroll
            for (int c = 0; c < 3; c++)
                if (c < nc) sig += __ldg(a.map + off + c * plane) * pf[c] * w[k];
        }
        *sp = sig;
    }
}

struct GatherLaunch {
    GatherArgs a;
    dim3 grid;
    cudaStream_t stream;
    template <int C, int P>
    int run() {
        k_from_map<C, P><<<grid, kBlock, 0, stream>>>(a);
        return after_launch("from_map");
    }
};

}  // namespace

}  // namespace so3g

extern "C" int so3g_proj_from_map(const so3g_pixelization *pz, const double *boresight,
                                  int32_t n_time, const double *dets, int32_t n_det,
                                  const float *response, const so3g_map *map, float *signal,
                                  int64_t sig_det_stride, int32_t *err, void *stream) {
    using namespace so3g;
    clear_error();
    GatherLaunch L;
    int rc = make_geom(pz, &L.a.g);
    if (rc) return rc;
    rc = attach_map(pz, map, &L.a.g);
    if (rc) return rc;
    if (n_det < 0 || n_time < 0) return set_error(SO3G_ERR_ARGUMENT, "negative n_det or n_time");
    if (n_det == 0 || n_time == 0) return SO3G_OK;
    if (!boresight || !dets || !response || !signal)
        return set_error(SO3G_ERR_ARGUMENT, "NULL input array");
    L.a.bore = boresight;
    L.a.dets = dets;
    L.a.resp = response;
    L.a.map = map->data;
    L.a.signal = signal;
    L.a.sig_stride = sig_det_stride;
    L.a.segs = Segs{nullptr, n_time};
    L.a.piece = piece_len(n_time);
    L.a.err = err;
    L.grid = dim3((unsigned)n_det, (unsigned)((n_time + L.a.piece - 1) / L.a.piece));
    L.stream = (cudaStream_t)stream;
    return dispatch_cp(pz->coord_sys, pix_kind(pz), L);
}
