// gather.cu -- from_map: per-sample pointing and a gather from the map,
// accumulated into the float32 signal exactly as the reference does (each
// term added in float64 and rounded to float32).
//
// CAR, TAN, ZEA and SIN with flat pixelizors use the certified double-float
// pointing of fastpoint.cuh (when GatherArgs::fast is set);
// samples it cannot certify are queued in shared memory (per warp) and
// finished by the exact float64 pointing, so every sample's result equals
// the exact path's.

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
    int fast;
    FastTables ft;
    FastConst fc;
};

// Adds the sample's map terms to its signal (src/Projection.cxx:1763-1765).
template <int P, int NT>
__device__ __forceinline__ void gather_taps(const GatherArgs &a, float *sp, int n,
                                            const int (*pix)[3], const float *w,
                                            const float *pf) {
    float sig = *sp;
    const int nc = a.g.ncomp;
#pragma unroll
    for (int k = 0; k < NT; k++) {
        if (k >= n) break;
        long long off, plane;
        int bad = locate<P>(a.g, pix[k], &off, &plane);
        if (bad >= 0) {
            record_missing_tile(a.err, bad);
            continue;
        }
#pragma unroll
        for (int c = 0; c < 3; c++)
            if (c < nc) sig += __ldg(a.map + off + c * plane) * pf[c] * w[k];
    }
    *sp = sig;
}

template <int C, int P>
__device__ void exact_gather(const GatherArgs &a, int det, int t, const QuatD &ofs, float T,
                             float Pr) {
    constexpr int NT = PixTraits<P>::taps;
    double coords[4];
    float pf[3];
    int pix[NT][3];
    float w[NT];
    get_coords<C>(a.g.lut, load_quat(a.bore + 4LL * t), ofs, coords);
    spin_factors(a.g.ncomp, coords, T, Pr, pf);
    const int n = get_pixels<P>(a.g, coords, pix, w);
    gather_taps<P, NT>(a, a.signal + det * a.sig_stride + t, n, pix, w, pf);
}

template <int C, int P>
// Compiled for 5 resident blocks per SM (at most 51 registers).
__global__ void __launch_bounds__(kBlock, 5) k_from_map(GatherArgs a) {
    constexpr bool kFastOK =
        (C == SO3G_COORD_CAR || C == SO3G_COORD_TAN || C == SO3G_COORD_ZEA ||
         C == SO3G_COORD_SIN) &&
        (P == PX_FLAT_NT_NN || P == PX_FLAT_T_NN || P == PX_FLAT_NT_BL ||
         P == PX_FLAT_T_BL) ||
        (C == SO3G_COORD_CAR && (P == PX_HP_NT || P == PX_HP_T));
    __shared__ int s_queue[kFastOK ? (kBlock / 32) * kWarpQueue : 1];
    int det, t0, t1;
    if (!seg_piece(a.segs, a.piece, det, t0, t1)) return;
    const QuatD ofs = load_quat(a.dets + 4LL * det);
    const float T = __ldg(a.resp + 2 * det), Pr = __ldg(a.resp + 2 * det + 1);
    const int nc = a.g.ncomp;
    constexpr int NT = PixTraits<P>::taps;
    if (!(kFastOK && a.fast)) {
        for (int t = t0 + threadIdx.x; t < t1; t += blockDim.x) exact_gather<C, P>(a, det, t, ofs, T, Pr);
        return;
    }
    dfl qd[4] = {df_from_double(ofs.a), df_from_double(ofs.b), df_from_double(ofs.c),
                 df_from_double(ofs.d)};
    int *wq = s_queue + (threadIdx.x >> 5) * kWarpQueue;
    int qn = 0;
    const int rounds = (t1 - t0 + blockDim.x - 1) / blockDim.x;
    for (int r = 0; r < rounds; r++) {
        const int t = t0 + r * blockDim.x + threadIdx.x;
        bool push = false;
        if (t < t1) {
            const double *bp = a.bore + 4LL * t;
            const double2 lo = __ldg(reinterpret_cast<const double2 *>(bp));
            const double2 hi = __ldg(reinterpret_cast<const double2 *>(bp) + 1);
            dfl qb[4];
            bool ok = df_split(lo.x, qb[0]) & df_split(lo.y, qb[1]) & df_split(hi.x, qb[2]) &
                      df_split(hi.y, qb[3]);
            int pix[NT][3];
            float pf[3], w[NT];
            int n = 0;
            ok = ok && fast_pointing<C, P>(a.g, a.ft, a.fc, qb, qd, nc, T, Pr, pix, w, n, pf);
            if (ok && n > 0) {
                // src/Projection.cxx:1763-1765 with certified float32
                // roundings, tap by tap and component by component.
                float *sp = a.signal + det * a.sig_stride + t;
                float s = *sp;
#pragma unroll
                for (int k = 0; k < NT; k++) {
                    if (k >= n || !ok) break;
                    long long off, plane;
                    const int bad = locate<P>(a.g, pix[k], &off, &plane);
                    if (bad >= 0) {
                        record_missing_tile(a.err, bad);
                        continue;
                    }
#pragma unroll
                    for (int c = 0; c < 3; c++)
                        if (ok && c < nc)
                            ok = fast_accum(s, __ldg(a.map + off + c * plane), pf[c], w[k]);
                }
                if (ok) *sp = s;
            }
            push = !ok;
        }
        qn = warp_enqueue(wq, qn, push, t);
        if (qn > kWarpQueue - 32 || r == rounds - 1) {
            __syncwarp();
            for (int i = threadIdx.x & 31; i < qn; i += 32)
                exact_gather<C, P>(a, det, wq[i], ofs, T, Pr);
            __syncwarp();
            qn = 0;
        }
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
    L.a.ft = device_fast_tables();
    L.a.fc = make_fast_const(L.a.g);
    L.a.fast = (pz->pointing == SO3G_POINTING_CERTIFIED && L.a.ft.asin_t) ? 1 : 0;
    L.grid = dim3((unsigned)n_det, (unsigned)((n_time + L.a.piece - 1) / L.a.piece));
    L.stream = (cudaStream_t)stream;
    return dispatch_cp(pz->coord_sys, pix_kind(pz), L);
}
