// pointing.cu -- pointing-only queries: coords, pixels, pointing_matrix,
// tile_hits and the domain edges behind pixel_ranges / tile_ranges.

#include <climits>
#include "host.h"

namespace so3g {

namespace {

constexpr int kSentinel = INT_MIN;  // "slot not set yet" (never a pixel index)

struct PointArgs {
    DGeom g;
    const double *bore;
    const double *dets;
    const float *resp;
    int n_time;
    int piece;
    double *coords;         // coords()
    int *pixel;             // pixels() / pointing_matrix()
    float *proj;            // pointing_matrix()
    unsigned long long *hits;  // tile_hits()
    int n_tile;
    // domain edges
    int mode, n_domain;
    const double *dmap;
    const int *tile_domain;
    int *edges;
    long long max_edges;
    unsigned long long *n_edges;
    int *err;
    int fast;               // certified pointing for pixels()/pointing_matrix()
    FastTables ft;
    FastConst fc;
};

// ---- coords ---------------------------------------------------------------

template <int C>
__global__ void __launch_bounds__(kBlock) k_coords(PointArgs a) {
    const int det = blockIdx.x;
    const long long p0 = (long long)blockIdx.y * a.piece;
    const int t1 = (int)min((long long)a.n_time, p0 + a.piece);
    const QuatD ofs = load_quat(a.dets + 4LL * det);
    for (int t = (int)p0 + threadIdx.x; t < t1; t += blockDim.x) {
        double c[4];
        get_coords<C>(a.g.lut, load_quat(a.bore + 4LL * t), ofs, c);
        double2 *out = reinterpret_cast<double2 *>(a.coords + ((long long)det * a.n_time + t) * 4);
        out[0] = make_double2(c[0], c[1]);
        out[1] = make_double2(c[2], c[3]);
    }
}

// ---- pixels / pointing_matrix -------------------------------------------
// Off-map samples keep the previous sample's slots 1.. (GetPixel writes only
// slot 0).  Each warp walks a contiguous sub-range of `sub` samples,
// carrying the last complete tuple across its 32-sample steps; samples that
// precede the first complete tuple of their sub-range get kSentinel, which
// k_pixels_fix then replaces with the tuple carried from earlier sub-ranges.

// Pixelizations whose pixels() / pointing_matrix() use the certified
// double-float pointing.
template <int C, int P>
struct PixCert {
    static constexpr bool value =
        (P == PX_HP_NT || P == PX_HP_T)
            ? C == SO3G_COORD_CAR
            : (C == SO3G_COORD_CAR || C == SO3G_COORD_TAN || C == SO3G_COORD_ZEA ||
               C == SO3G_COORD_SIN || C == SO3G_COORD_ARC);
};

// GetPixel of one sample (and, with PROJ, its spin factors) through the
// certified double-float pointing; false when a decision or a spin factor
// is not certain, and the caller takes the exact path.  GetPixel is the
// nearest pixel with [0, n) bounds for every flat pixelizor, interpolating
// or not, tiled or not (:845-863, :1029-1051): the NonTiled nearest pixel
// is certified and the tile tuple formed from it.
template <int C, int P, bool PROJ>
__device__ __forceinline__ bool cert_pixel(const PointArgs &a, const dfl (&qb)[4],
                                           const dfl (&qd)[4], int nc, float T, float Pr,
                                           int *idx, bool &full, float *pf) {
    dfl Nc, Ns, D;
    int pix[1][3];
    float w[4];
    int n = 0;
    if (P == PX_HP_NT || P == PX_HP_T) {
        dfl qa, qb2, qc, qd2;
        df_qmul(qb, qd, qa, qb2, qc, qd2);
        const dfl cos_t = df_dot<4>({qa, qb2, qc, qd2}, {qa, df_neg(qb2), df_neg(qc), qd2});
        if (!(fabsf(cos_t.hi) < 0.998f)) return false;
        dfl lon;
        if (!fast_lon_spin(a.ft, a.fc, qa, qb2, qc, qd2, cos_t, lon, Nc, Ns, D)) return false;
        if (!fast_healpix<P>(a.g, a.ft, a.fc, cos_t, lon, pix, n) || n != 1) return false;
        idx[0] = pix[0][0];
        if (P == PX_HP_T) idx[1] = pix[0][1];
        full = true;
    } else {
        dfl X, Y;
        if (!fast_native<C>(a.ft, a.fc, qb, qd, X, Y, Nc, Ns, D)) return false;
        const dfl x = df_add(df_mul(X, a.fc.inv_cdx), a.fc.off_x);
        const dfl y = df_add(df_mul(Y, a.fc.inv_cdy), a.fc.off_y);
        if (!fast_pixels<PX_FLAT_NT_NN>(a.g, x, y, pix, w, n)) return false;
        full = n > 0;
        if (!full) {
            idx[0] = -1;
        } else if (P == PX_FLAT_NT_NN || P == PX_FLAT_NT_BL) {
            idx[0] = pix[0][0];
            idx[1] = pix[0][1];
        } else {
            const int iy = pix[0][0], ix = pix[0][1];
            const int sub_y = iy / a.g.ty, sub_x = ix / a.g.tx;
            idx[0] = sub_y * a.g.ntx + sub_x;
            idx[1] = iy - sub_y * a.g.ty;
            idx[2] = ix - sub_x * a.g.tx;
        }
    }
    if (PROJ) return fast_spin<true>(nc, T, Pr, Nc, Ns, D, pf);
    return true;
}

template <int C, int P, bool PROJ>
__global__ void __launch_bounds__(kBlock) k_pixels(PointArgs a, int sub) {
    constexpr int IC = PixTraits<P>::index_count;
    const int det = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long s0 = (long long)blockIdx.y * a.piece + (long long)warp * sub;
    if (s0 >= a.n_time) return;
    const int s1 = (int)min((long long)a.n_time, s0 + sub);
    const QuatD ofs = load_quat(a.dets + 4LL * det);
    float T = 0.f, Pr = 0.f;
    if (PROJ) { T = __ldg(a.resp + 2 * det); Pr = __ldg(a.resp + 2 * det + 1); }
    const int nc = a.g.ncomp;
    int carry[IC];
#pragma unroll
    for (int j = 0; j < IC; j++) carry[j] = kSentinel;
    dfl qd[4];
    if (PixCert<C, P>::value && a.fast) {
        qd[0] = df_of(ofs.a);
        qd[1] = df_of(ofs.b);
        qd[2] = df_of(ofs.c);
        qd[3] = df_of(ofs.d);
    }
    for (int base = (int)s0; base < s1; base += 32) {
        const int t = base + lane;
        const bool live = t < s1;
        int idx[IC];
#pragma unroll
        for (int j = 0; j < IC; j++) idx[j] = kSentinel;
        bool full = false;
        float pf[3] = {0.f, 0.f, 0.f};
        if (live) {
            bool done = false;
            if constexpr (PixCert<C, P>::value) {
                if (a.fast) {
                    const double2 lo = __ldg(reinterpret_cast<const double2 *>(a.bore + 4LL * t));
                    const double2 hi =
                        __ldg(reinterpret_cast<const double2 *>(a.bore + 4LL * t) + 1);
                    dfl qb[4];
                    done = df_split(lo.x, qb[0]) & df_split(lo.y, qb[1]) &
                           df_split(hi.x, qb[2]) & df_split(hi.y, qb[3]);
                    done = done && cert_pixel<C, P, PROJ>(a, qb, qd, nc, T, Pr, idx, full, pf);
                }
            }
            if (!done) {
                // The exact float64 path: the pixelizations above for the
                // few samples the certified pointing leaves, all others.
#pragma unroll
                for (int j = 0; j < IC; j++) idx[j] = kSentinel;
                double c[4];
                get_coords<C>(a.g.lut, load_quat(a.bore + 4LL * t), ofs, c);
                full = get_pixel<P>(a.g, c, idx);
                if (PROJ) spin_factors(nc, c, T, Pr, pf);
            }
        }
        const unsigned vm = __ballot_sync(kFull, live && full);
        const unsigned before = vm & ((1u << lane) - 1u);
        const int src = before ? 31 - __clz(before) : lane;
#pragma unroll
        for (int j = 1; j < IC; j++) {
            int v = __shfl_sync(kFull, idx[j], src);
            if (live && !full) idx[j] = before ? v : carry[j];
        }
        if (vm) {
            const int hi = 31 - __clz(vm);
#pragma unroll
            for (int j = 1; j < IC; j++) carry[j] = __shfl_sync(kFull, idx[j], hi);
        }
        if (live) {
            int *out = a.pixel + ((long long)det * a.n_time + t) * IC;
#pragma unroll
            for (int j = 0; j < IC; j++) out[j] = idx[j];
            if (PROJ) {
                float *pout = a.proj + ((long long)det * a.n_time + t) * nc;
#pragma unroll
                for (int k = 0; k < 3; k++)
                    if (k < nc) pout[k] = pf[k];
            }
        }
    }
}

// One warp per detector: walk the sub-ranges in time order, fill leading
// sentinels with the carried tuple, then carry the sub-range's last tuple.
template <int IC>
__global__ void k_pixels_fix(int *pixel, int n_det, int n_time, int sub) {
    const int det = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (det >= n_det) return;
    int *row = pixel + (long long)det * n_time * IC;
    int carry[IC];
#pragma unroll
    for (int j = 0; j < IC; j++) carry[j] = 0;  // initial tuple {-1, 0, ...}
    for (long long s0 = 0; s0 < n_time; s0 += sub) {
        const int s1 = (int)min((long long)n_time, s0 + sub);
        if (row[s0 * IC + 1] == kSentinel) {
            for (int tt = (int)s0 + lane;; tt += 32) {
                const bool in = tt < s1;
                const bool sent = in && row[(long long)tt * IC + 1] == kSentinel;
                if (sent) {
#pragma unroll
                    for (int j = 1; j < IC; j++) row[(long long)tt * IC + j] = carry[j];
                }
                const unsigned m = __ballot_sync(kFull, sent);
                if (m != kFull) break;
            }
        }
        __syncwarp();
#pragma unroll
        for (int j = 1; j < IC; j++) carry[j] = row[(long long)(s1 - 1) * IC + j];
    }
}

// ---- taps of one sample --------------------------------------------------------

// The GetPixels taps of one sample (Pixelizor*::GetPixels): the certified
// double-float pointing where it applies and decides -- its pixel
// decisions are the exact path's; no spin factors are formed -- else the
// exact float64 path.  qd: the detector's double-float split (a.fast).
template <int C, int P>
__device__ __forceinline__ int sample_taps(const PointArgs &a, const QuatD &ofs,
                                           const dfl (&qd)[4], int t, int (*pix)[3], float *w) {
    if constexpr (FastEligible<C, P>::value) {
        if (a.fast) {
            const double2 lo = __ldg(reinterpret_cast<const double2 *>(a.bore + 4LL * t));
            const double2 hi = __ldg(reinterpret_cast<const double2 *>(a.bore + 4LL * t) + 1);
            dfl qb[4];
            const bool ok = df_split(lo.x, qb[0]) & df_split(lo.y, qb[1]) &
                            df_split(hi.x, qb[2]) & df_split(hi.y, qb[3]);
            int n = 0;
            float pf[3];
            if (ok && fast_pointing<C, P, false>(a.g, a.ft, a.fc, qb, qd, 1, 1.f, 0.f, pix, w, n,
                                                 pf))
                return n;
        }
    }
    double c[4];
    get_coords<C>(a.g.lut, load_quat(a.bore + 4LL * t), ofs, c);
    return get_pixels<P>(a.g, c, pix, w);
}

// The detector's double-float split, where the certified pointing is used.
template <int C, int P>
__device__ __forceinline__ void det_split(const PointArgs &a, const QuatD &ofs, dfl (&qd)[4]) {
    if (FastEligible<C, P>::value && a.fast) {
        qd[0] = df_of(ofs.a);
        qd[1] = df_of(ofs.b);
        qd[2] = df_of(ofs.c);
        qd[3] = df_of(ofs.d);
    }
}

// ---- tile_hits ------------------------------------------------------------

template <int C, int P>
__global__ void __launch_bounds__(kBlock) k_tile_hits(PointArgs a) {
    constexpr int NT = PixTraits<P>::taps;
    const int det = blockIdx.x;
    const int lane = threadIdx.x & 31;
    const long long p0 = (long long)blockIdx.y * a.piece;
    const int t1 = (int)min((long long)a.n_time, p0 + a.piece);
    const QuatD ofs = load_quat(a.dets + 4LL * det);
    dfl qd[4];
    det_split<C, P>(a, ofs, qd);
    for (int base = (int)p0 + (threadIdx.x & ~31); base < t1; base += blockDim.x) {
        const int t = base + lane;
        int pix[NT][3];
        float w[NT];
        int n = 0;
        if (t < t1) n = sample_taps<C, P>(a, ofs, qd, t, pix, w);
#pragma unroll
        for (int k = 0; k < NT; k++) {
            int key = (k < n && pix[k][0] >= 0 && pix[k][0] < a.n_tile) ? pix[k][0] : -1;
            // One atomic per run of equal tiles across the warp.
            int prev = __shfl_up_sync(kFull, key, 1);
            bool head = lane == 0 || key != prev;
            unsigned heads = __ballot_sync(kFull, head);
            unsigned after = heads & ~((2u << lane) - 1u);
            int end = after ? (__ffs(after) - 1) : 32;
            if (head && key >= 0) atomicAdd(a.hits + key, (unsigned long long)(end - lane));
        }
    }
}

// ---- domain edges -----------------------------------------------------------

template <int C, int P>
__device__ __forceinline__ int sample_domain(const PointArgs &a, const QuatD &ofs,
                                             const dfl (&qd)[4], int t) {
    // pixel_ranges :1489-1506, tile_ranges :1655-1670
    constexpr int NT = PixTraits<P>::taps;
    int pix[NT][3];
    float w[NT];
    int n = sample_taps<C, P>(a, ofs, qd, t, pix, w);
    long long samp = -1;
#pragma unroll
    for (int k = 0; k < NT; k++) {
        if (k >= n) break;
        long long pd;
        if (a.mode == 0) {
            pd = stripe<P>(a.g, pix[k], a.n_domain);
        } else if (a.mode == 1) {
            long long off, plane;
            int bad = locate<P>(a.g, pix[k], &off, &plane);
            if (bad >= 0) {
                record_missing_tile(a.err, bad);
                pd = -1;
            } else {
                double v = __ldg(a.dmap + off);
                pd = (v > -2147483648.0 && v < 2147483648.0) ? (long long)(int)v : -1;
            }
        } else {
            int tile = pix[k][0];
            pd = (tile >= 0 && tile < a.n_tile) ? __ldg(a.tile_domain + tile) : -1;
        }
        if (k > 0 && pd != samp) { samp = a.n_domain; break; }
        samp = pd;
    }
    return (int)max(min(samp, (long long)INT_MAX), (long long)INT_MIN + 1);
}

// Lane 0 of each warp step recomputes the label of the sample before the
// step, so every edge is found without a label array: 31 new samples per
// 32-lane step.
template <int C, int P>
__global__ void __launch_bounds__(kBlock) k_domain_edges(PointArgs a) {
    const int det = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long p0 = (long long)blockIdx.y * a.piece;
    const int t1 = (int)min((long long)a.n_time, p0 + a.piece);
    const QuatD ofs = load_quat(a.dets + 4LL * det);
    dfl qd[4];
    det_split<C, P>(a, ofs, qd);
    const int nwarp = blockDim.x >> 5;
    for (long long s = p0 + (long long)warp * 31; s < t1; s += (long long)nwarp * 31) {
        const long long t = s - 1 + lane;
        int lab = INT_MIN;  // "before the first sample"
        if (t >= 0 && t < t1) lab = sample_domain<C, P>(a, ofs, qd, (int)t);
        const int prev = __shfl_up_sync(kFull, lab, 1);
        const bool edge = lane > 0 && t < t1 && (t == 0 || lab != prev);
        if (edge) {
            unsigned long long k = atomicAdd(a.n_edges, 1ull);
            if ((long long)k < a.max_edges) {
                a.edges[3 * k] = det;
                a.edges[3 * k + 1] = (int)t;
                a.edges[3 * k + 2] = lab;
            }
        }
    }
}

// ---- launchers ----------------------------------------------------------------

enum { L_COORDS, L_PIXELS, L_PMAT, L_HITS, L_EDGES };

struct PointLaunch {
    PointArgs a;
    dim3 grid;
    cudaStream_t stream;
    int what;
    int n_det;
    template <int C, int P>
    int run() {
        if (what == L_COORDS) {
            k_coords<C><<<grid, kBlock, 0, stream>>>(a);
            return after_launch("coords");
        }
        if (what == L_PIXELS || what == L_PMAT) {
            constexpr int IC = PixTraits<P>::index_count;
            const int sub = a.piece / (kBlock / 32);
            if (what == L_PIXELS) k_pixels<C, P, false><<<grid, kBlock, 0, stream>>>(a, sub);
            else k_pixels<C, P, true><<<grid, kBlock, 0, stream>>>(a, sub);
            int rc = after_launch(what == L_PIXELS ? "pixels" : "pointing_matrix");
            if (rc || IC < 2) return rc;
            k_pixels_fix<IC><<<(n_det + 7) / 8, 256, 0, stream>>>(a.pixel, n_det, a.n_time, sub);
            return after_launch("pixels fix-up");
        }
        if (what == L_HITS) {
            k_tile_hits<C, P><<<grid, kBlock, 0, stream>>>(a);
            return after_launch("tile_hits");
        }
        k_domain_edges<C, P><<<grid, kBlock, 0, stream>>>(a);
        return after_launch("domain_edges");
    }
};

int point_common(PointLaunch &L, const so3g_pixelization *pz, const double *bore, int n_time,
                 const double *dets, int n_det, void *stream, int what) {
    clear_error();
    int rc = make_geom(pz, &L.a.g);
    if (rc) return rc;
    if (n_det < 0 || n_time < 0) return set_error(SO3G_ERR_ARGUMENT, "negative n_det or n_time");
    if (n_det > 0 && n_time > 0 && (!bore || !dets))
        return set_error(SO3G_ERR_ARGUMENT, "NULL boresight or detector array");
    L.a.bore = bore;
    L.a.dets = dets;
    L.a.n_time = n_time;
    L.a.piece = piece_len(n_time);
    L.grid = dim3((unsigned)n_det, (unsigned)((n_time + L.a.piece - 1) / L.a.piece));
    L.stream = (cudaStream_t)stream;
    L.what = what;
    L.n_det = n_det;
    L.a.ft = device_fast_tables();
    L.a.fc = make_fast_const(L.a.g);
    L.a.fast = fast_mode(pz, L.a.ft) != SO3G_POINTING_EXACT;
    return SO3G_OK;
}

}  // namespace

}  // namespace so3g

using namespace so3g;

extern "C" {

int so3g_proj_coords(const so3g_pixelization *pz, const double *boresight, int32_t n_time,
                     const double *dets, int32_t n_det, double *coords, void *stream) {
    PointLaunch L{};
    int rc = point_common(L, pz, boresight, n_time, dets, n_det, stream, L_COORDS);
    if (rc || n_det == 0 || n_time == 0) return rc;
    if (!coords) return set_error(SO3G_ERR_ARGUMENT, "NULL coords");
    L.a.coords = coords;
    // coords() does not depend on the pixelizor.
    return dispatch_cp(pz->coord_sys, PX_FLAT_NT_NN, L);
}

int so3g_proj_pixels(const so3g_pixelization *pz, const double *boresight, int32_t n_time,
                     const double *dets, int32_t n_det, int32_t *pixel, void *stream) {
    PointLaunch L{};
    int rc = point_common(L, pz, boresight, n_time, dets, n_det, stream, L_PIXELS);
    if (rc || n_det == 0 || n_time == 0) return rc;
    if (!pixel) return set_error(SO3G_ERR_ARGUMENT, "NULL pixel");
    L.a.pixel = pixel;
    return dispatch_cp(pz->coord_sys, pix_kind(pz), L);
}

int so3g_proj_pointing_matrix(const so3g_pixelization *pz, const double *boresight,
                              int32_t n_time, const double *dets, int32_t n_det,
                              const float *response, int32_t *pixel, float *proj,
                              void *stream) {
    PointLaunch L{};
    int rc = point_common(L, pz, boresight, n_time, dets, n_det, stream, L_PMAT);
    if (rc || n_det == 0 || n_time == 0) return rc;
    if (!pixel || !proj || !response) return set_error(SO3G_ERR_ARGUMENT, "NULL output or response");
    L.a.pixel = pixel;
    L.a.proj = proj;
    L.a.resp = response;
    return dispatch_cp(pz->coord_sys, pix_kind(pz), L);
}

int so3g_proj_tile_hits(const so3g_pixelization *pz, const double *boresight, int32_t n_time,
                        const double *dets, int32_t n_det, int64_t *hits, int32_t n_tile,
                        void *stream) {
    PointLaunch L{};
    int rc = point_common(L, pz, boresight, n_time, dets, n_det, stream, L_HITS);
    if (rc) return rc;
    if (!pz->tiled || L.a.g.n_tile <= 0)
        return set_error(SO3G_ERR_ARGUMENT, "No tiles in this pixelization.");
    if (n_tile != L.a.g.n_tile)
        return set_error(SO3G_ERR_ARGUMENT, "hits has %d entries; the pixelization has %d tiles",
                         n_tile, L.a.g.n_tile);
    if (n_det == 0 || n_time == 0) return SO3G_OK;
    if (!hits) return set_error(SO3G_ERR_ARGUMENT, "NULL hits");
    L.a.hits = reinterpret_cast<unsigned long long *>(hits);
    L.a.n_tile = n_tile;
    return dispatch_cp(pz->coord_sys, pix_kind(pz), L);
}

int so3g_proj_domain_edges(const so3g_pixelization *pz, const double *boresight,
                           int32_t n_time, const double *dets, int32_t n_det, int32_t mode,
                           int32_t n_domain, const so3g_map *dmap, const int32_t *tile_domain,
                           int32_t n_tile, int32_t *edges, int64_t max_edges,
                           int64_t *n_edges, int32_t *err, void *stream) {
    PointLaunch L{};
    int rc = point_common(L, pz, boresight, n_time, dets, n_det, stream, L_EDGES);
    if (rc) return rc;
    if (mode < 0 || mode > 2) return set_error(SO3G_ERR_ARGUMENT, "unknown domain mode %d", mode);
    if (mode == 0 && n_domain <= 0) return set_error(SO3G_ERR_ARGUMENT, "n_domain must be positive");
    if (mode == 1) {
        rc = attach_map(pz, dmap, &L.a.g);
        if (rc) return rc;
        L.a.dmap = dmap->data;
    }
    if (mode == 2) {
        if (!pz->tiled || L.a.g.n_tile <= 0)
            return set_error(SO3G_ERR_ARGUMENT, "No tiles in this pixelization.");
        if (n_tile != L.a.g.n_tile || !tile_domain)
            return set_error(SO3G_ERR_ARGUMENT, "tile_domain must have one entry per tile");
        L.a.tile_domain = tile_domain;
        L.a.n_tile = n_tile;
    }
    if (n_det == 0 || n_time == 0) return SO3G_OK;
    if (!edges || !n_edges) return set_error(SO3G_ERR_ARGUMENT, "NULL edges");
    L.a.mode = mode;
    L.a.n_domain = n_domain;
    L.a.edges = edges;
    L.a.max_edges = max_edges;
    L.a.n_edges = reinterpret_cast<unsigned long long *>(n_edges);
    L.a.err = err;
    return dispatch_cp(pz->coord_sys, pix_kind(pz), L);
}

}  // extern "C"
