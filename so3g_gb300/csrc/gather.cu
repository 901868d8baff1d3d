// gather.cu -- from_map: per-sample pointing and a gather from the map,
// accumulated into the float32 signal exactly as the reference does (each
// term added in float64 and rounded to float32).
//
// CAR, TAN, ZEA and SIN with flat pixelizors and CAR HEALPix use the
// certified double-float pointing of fastpoint.cuh (when GatherArgs::fast
// is set), their nearest-neighbour forms behind the float32 tier of
// mixedpoint.cuh (certified mode: the pixel from it, spin factors and
// terms certified in double-float; mixed mode: float32 spin factors and
// terms).  Samples a tier cannot certify are queued in shared memory (per
// warp) and go, 32 at a time, to the double-float and then the exact
// float64 pointing; in certified mode every sample's result equals the
// exact path's.

#include "host.h"
#include "interp_point.cuh"
#include "mx_common.cuh"

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
    int fast;           // SO3G_POINTING_*: 0 exact, 1 certified, 2 mixed
    FastTables ft;
    FastConst fc;
    MixedConst mc;
    const float4 *bore32;   // float32 boresight (mixed pointing), or NULL
    const float4 *map32;    // float32 (T, Q, U, 0) per pixel (mixed pointing), or NULL
};

// Largest parent map (pixels) that gets the float32 copy when tiled: the
// copy spans the parent map (16 bytes per pixel), present tiles or not.
constexpr long long kMap32TiledMaxPixels = 1LL << 28;

// Index of a located sample's pixel in the float32 map copy: its element
// offset for an untiled map; for a tiled map its pixel in the parent map
// (flat: row-major over (ny, nx); HEALPix: the NEST index tile * nppt + sub).
template <int P>
__device__ __forceinline__ long long map32_index(const DGeom &g, const int *pix, long long off) {
    if (P == PX_FLAT_T_NN || P == PX_FLAT_T_BL) {
        const int t = pix[0], row = div_small(t, g.ntx, g.inv_ntx), col = t - row * g.ntx;
        return (long long)(row * g.ty + pix[1]) * g.nx + (long long)col * g.tx + pix[2];
    }
    if (P == PX_HP_T) return (long long)pix[0] * g.nppt + pix[1];
    return off;
}

// Tile tuple of a parent-map pixel in the float32 tier's PARENT form.
template <int P>
__device__ __forceinline__ void parent_to_tile(const DGeom &g, const int *par, int *tp) {
    if (P == PX_HP_T) {
        hp_tile_split(g.nppt, par[0], tp[0], tp[1]);
    } else {
        flat_tile_tuple(g, par[0], par[1], tp);
    }
}

// The float32 copy of a tiled map over its parent map's pixels, .w = 1 on
// present tiles and 0 on absent ones (whose samples raise the missing-tile
// error).
template <int P>
__global__ void k_map_f32_tiled(DGeom g, const double *map, long long npix, float4 *out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    int pix[3];
    if (P == PX_HP_T) {
        hp_tile_split(g.nppt, i, pix[0], pix[1]);
        pix[2] = 0;
    } else {
        const int gy = (int)(i / g.nx), gx = (int)(i - (long long)gy * g.nx);
        flat_tile_tuple(g, gy, gx, pix);
    }
    float v[3] = {0.f, 0.f, 0.f};
    long long off, plane;
    const bool present = locate<P>(g, pix, &off, &plane) < 0;
    if (present)
        for (int c = 0; c < g.ncomp && c < 3; c++)
            v[c] = __double2float_rn(__ldg(map + off + c * plane));
    out[i] = make_float4(v[0], v[1], v[2], present ? 1.f : 0.f);
}

// The untiled map's components as float32, pixel by pixel (one 16-byte
// load per sample in the mixed from_map).
__global__ void k_map_f32(const double *map, int nc, long long npix, float4 *out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    float v[3] = {0.f, 0.f, 0.f};
    for (int c = 0; c < nc; c++) v[c] = __double2float_rn(__ldg(map + c * npix + i));
    out[i] = make_float4(v[0], v[1], v[2], 0.f);
}

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
__device__ __noinline__ void exact_gather(const GatherArgs &a, int det, int t, const QuatD &ofs, float T,
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

// One sample of the mixed-pointing fallback through the double-float
// pointing; false (signal untouched) when its pixel is not certified.  Its
// spin factors and terms, like the float32 tier's, are float32 evaluations
// (the mixed-precision contract).
template <int C, int P>
__device__ __forceinline__ bool df_gather(const GatherArgs &a, int det, int t, const dfl (&qd)[4], float T,
                          float Pr) {
    constexpr int NT = PixTraits<P>::taps;
    const double *bp = a.bore + 4LL * t;
    const double2 lo = __ldg(reinterpret_cast<const double2 *>(bp));
    const double2 hi = __ldg(reinterpret_cast<const double2 *>(bp) + 1);
    dfl qb[4];
    if (!(df_split(lo.x, qb[0]) & df_split(lo.y, qb[1]) & df_split(hi.x, qb[2]) &
          df_split(hi.y, qb[3])))
        return false;
    int pix[NT][3];
    float pf[3], w[NT];
    int n = 0;
    const int nc = a.g.ncomp;
    if (!fast_pointing<C, P, false>(a.g, a.ft, a.fc, qb, qd, nc, T, Pr, pix, w, n, pf))
        return false;
    if (n == 0) return true;
    float *sp = a.signal + det * a.sig_stride + t;
    float s = *sp;
#pragma unroll
    for (int k = 0; k < NT; k++) {
        if (k >= n) break;
        long long off, plane;
        const int bad = locate<P>(a.g, pix[k], &off, &plane);
        if (bad >= 0) {
            record_missing_tile(a.err, bad);
            continue;
        }
        if (a.map32) {
            const float4 m = __ldg(a.map32 + map32_index<P>(a.g, pix[k], off));
            s = fmaf(m.x, pf[0] * w[k], s);
            if (nc > 1) s = fmaf(m.y, pf[1] * w[k], s);
            if (nc > 2) s = fmaf(m.z, pf[2] * w[k], s);
        } else {
#pragma unroll
            for (int c = 0; c < 3; c++)
                if (c < nc) s = fmaf(d2f_round(__ldg(a.map + off + c * plane)), pf[c] * w[k], s);
        }
    }
    *sp = s;
    return true;
}

// One sample of the certified float32 tier's fallback through the full
// certified double-float pointing and certified float32 roundings of the
// reference's float64 sums; false (signal untouched) when any of them is
// not certain.
template <int C, int P>
__device__ __forceinline__ bool df_gather_cert(const GatherArgs &a, int det, int t,
                                               const dfl (&qd)[4], float T, float Pr) {
    constexpr int NT = PixTraits<P>::taps;
    const double *bp = a.bore + 4LL * t;
    const double2 lo = __ldg(reinterpret_cast<const double2 *>(bp));
    const double2 hi = __ldg(reinterpret_cast<const double2 *>(bp) + 1);
    dfl qb[4];
    if (!(df_split(lo.x, qb[0]) & df_split(lo.y, qb[1]) & df_split(hi.x, qb[2]) &
          df_split(hi.y, qb[3])))
        return false;
    int pix[NT][3];
    float pf[3], w[NT];
    int n = 0;
    const int nc = a.g.ncomp;
    if (!fast_pointing<C, P>(a.g, a.ft, a.fc, qb, qd, nc, T, Pr, pix, w, n, pf)) return false;
    if (n == 0) return true;
    float *sp = a.signal + det * a.sig_stride + t;
    float s = *sp;
    bool ok = true;
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
            if (ok && c < nc) ok = fast_accum(s, __ldg(a.map + off + c * plane), pf[c], w[k]);
    }
    if (ok) *sp = s;
    return ok;
}

// Compiled for 5 resident blocks per SM (at most 51 registers; mixed
// pointing: 7), one variant per pointing mode (0 exact, 1 certified, 2
// mixed).  The certified and mixed variants of the nearest-neighbour
// CAR/TAN/ZEA/SIN and HEALPix pixelizations take the float32 tier first.
template <int C, int P, int MODE>
__global__ void __launch_bounds__(kBlock, MixedEligible<C, P>::value && MODE == 2 ? 7 : 5)
    k_from_map(GatherArgs a) {
    constexpr bool kFastOK = FastEligible<C, P>::value && MODE >= 1;
    constexpr bool kMixedOK = MixedEligible<C, P>::value && MODE >= 1;
    constexpr bool kCert = MODE == 1;
    __shared__ int s_queue[!kFastOK ? 1 : (kMixedOK ? 2 : 1) * (kBlock / 32) * kWarpQueue];
    __shared__ WarpPiece s_wp[kFastOK ? kBlock / 32 : 1];
    int det, t0, t1;
    if (!seg_piece(a.segs, a.piece, det, t0, t1)) return;
    const QuatD ofs = load_quat(a.dets + 4LL * det);
    const float T = __ldg(a.resp + 2 * det), Pr = __ldg(a.resp + 2 * det + 1);
    const int nc = a.g.ncomp;
    constexpr int NT = PixTraits<P>::taps;
    if (!kFastOK) {
        for (int t = t0 + threadIdx.x; t < t1; t += blockDim.x) exact_gather<C, P>(a, det, t, ofs, T, Pr);
        return;
    }
    dfl qd[4] = {df_of(ofs.a), df_of(ofs.b), df_of(ofs.c), df_of(ofs.d)};
    constexpr bool mixed = kMixedOK;
    float qd32[4];
    if (kMixedOK && mixed) {
        qd32[0] = d2f_round(ofs.a);
        qd32[1] = d2f_round(ofs.b);
        qd32[2] = d2f_round(ofs.c);
        qd32[3] = d2f_round(ofs.d);
    }
    int *wq = s_queue + (threadIdx.x >> 5) * kWarpQueue;
    int *wdf = s_queue + ((kBlock >> 5) + (threadIdx.x >> 5)) * kWarpQueue;
    int qn = 0, qdf = 0;
    WarpPiece *wp = s_wp + (threadIdx.x >> 5);
    if ((threadIdx.x & 31) == 0) {
        wp->ofs = ofs;
#pragma unroll
        for (int k = 0; k < 4; k++) wp->qd[k] = qd[k];
    }
    __syncwarp();
    auto drain_exact = [&]() {
        __syncwarp();
        for (int i = threadIdx.x & 31; i < qn; i += 32)
            exact_gather<C, P>(a, det, wq[i], wp->ofs, T, Pr);
        __syncwarp();
        qn = 0;
    };
    const int rounds = (t1 - t0 + blockDim.x - 1) / blockDim.x;
    for (int r = 0; r < rounds; r++) {
        const int t = t0 + r * blockDim.x + threadIdx.x;
        bool push = false, push_df = false;
        if constexpr (MODE == 2 && !kMixedOK) {
            // Mixed pointing where the float32 tier does not apply
            // (bilinear): the double-float pointing with certified taps,
            // float32 spin factors, weights and terms (df_gather); the exact
            // path for the samples it leaves.
            if (t < t1) push = !df_gather<C, P>(a, det, t, qd, T, Pr);
            qn = warp_enqueue(wq, qn, push, t);
            if (qn > kWarpQueue - 32 || r == rounds - 1) drain_exact();
            continue;
        }
        if (kMixedOK && mixed && kCert) {
            if (t < t1) {
                float *sp = a.signal + det * a.sig_stride + t;
                const float s_in = *sp;
                // The float32 tier's pixel from the float64 boresight's
                // double-float split, the certified spin factors from the
                // split itself, and certified float32 roundings of the
                // reference's float64 sums.
                const double *bp = a.bore + 4LL * t;
                const double2 lo = __ldg(reinterpret_cast<const double2 *>(bp));
                const double2 hi = __ldg(reinterpret_cast<const double2 *>(bp) + 1);
                dfl qb[4];
                bool ok = df_split(lo.x, qb[0]) & df_split(lo.y, qb[1]) &
                          df_split(hi.x, qb[2]) & df_split(hi.y, qb[3]);
                const float qbf[4] = {qb[0].hi, qb[1].hi, qb[2].hi, qb[3].hi};
                int pix[3];
                float pf[3];
                bool on = false;
                ok = ok && mixed_pointing<C, P, false>(a.g, a.ft, a.mc, qbf, qd32, nc, T, Pr,
                                                       pix, on, pf);
                if (ok && on) ok = df_spin_only<C>(qb, qd, nc, T, Pr, pf);
                if (!ok) {
                    push_df = true;
                } else if (on) {
                    long long off, plane;
                    const int bad = locate<P>(a.g, pix, &off, &plane);
                    if (bad >= 0) {
                        record_missing_tile(a.err, bad);
                    } else {
                        // src/Projection.cxx:1763-1765, component by component.
                        float s = s_in;
#pragma unroll
                        for (int c = 0; c < 3; c++)
                            if (ok && c < nc)
                                ok = fast_accum(s, __ldg(a.map + off + c * plane), pf[c]);
                        if (ok) *sp = s;
                        push = !ok;
                    }
                }
            }
            qn = warp_enqueue(wq, qn, push, t);
            if (qn > kWarpQueue - 32) drain_exact();
            qdf = warp_enqueue(wdf, qdf, push_df, t);
            if (qdf >= 32 || (r == rounds - 1 && qdf > 0)) {
                __syncwarp();
                for (int base = 0; base < qdf; base += 32) {
                    const int i = base + (threadIdx.x & 31);
                    const int ts = i < qdf ? wdf[i] : 0;
                    const bool px = i < qdf && !df_gather_cert<C, P>(a, det, ts, wp->qd, T, Pr);
                    qn = warp_enqueue(wq, qn, px, ts);
                    if (qn > kWarpQueue - 32) drain_exact();
                }
                __syncwarp();
                qdf = 0;
            }
            if (qn > kWarpQueue - 32 || r == rounds - 1) drain_exact();
            continue;
        }
        if (kMixedOK && mixed) {
            if (t < t1) {
                // The signal is loaded before the pointing is evaluated, so
                // that the load's latency (long for a signal in host memory)
                // overlaps the pointing arithmetic.
                float *sp = a.signal + det * a.sig_stride + t;
                const float s_in = *sp;
                float qb[4];
                load_bore_f32(a.bore32, a.bore, t, qb);
                int pix[3];
                float pf[3];
                bool on = false;
                // Tiled maps: the pixel comes as a parent-map index; with the
                // float32 copy (indexed by it, tile presence in .w) no tile
                // arithmetic is needed.
                constexpr bool kParent = P == PX_FLAT_T_NN || P == PX_HP_T;
                if (mixed_pointing<C, P, true, kParent>(a.g, a.ft, a.mc, qb, qd32, nc, T, Pr, pix,
                                                        on, pf)) {
                    if (kParent && on && a.map32) {
                        const long long gi = P == PX_HP_T
                                                 ? (long long)pix[0]
                                                 : (long long)pix[0] * a.g.nx + pix[1];
                        const float4 m = __ldg(a.map32 + gi);
                        if (m.w != 0.f) {
                            float s = fmaf(m.x, pf[0], s_in);
                            if (nc > 1) s = fmaf(m.y, pf[1], s);
                            if (nc > 2) s = fmaf(m.z, pf[2], s);
                            *sp = s;
                        } else {
                            int tp[3];
                            parent_to_tile<P>(a.g, pix, tp);
                            record_missing_tile(a.err, tp[0]);
                        }
                    } else if (on) {
                        if (kParent) {
                            const int par[2] = {pix[0], pix[1]};
                            parent_to_tile<P>(a.g, par, pix);
                        }
                        long long off, plane;
                        const int bad = locate<P>(a.g, pix, &off, &plane);
                        if (bad >= 0) {
                            record_missing_tile(a.err, bad);
                        } else {
                            // float32 terms (the mixed-precision contract).
                            float s = s_in;
                            if (a.map32) {
                                const float4 m = __ldg(a.map32 + map32_index<P>(a.g, pix, off));
                                s = fmaf(m.x, pf[0], s);
                                if (nc > 1) s = fmaf(m.y, pf[1], s);
                                if (nc > 2) s = fmaf(m.z, pf[2], s);
                            } else {
#pragma unroll
                                for (int c = 0; c < 3; c++)
                                    if (c < nc)
                                        s = fmaf(d2f_round(__ldg(a.map + off + c * plane)), pf[c],
                                                 s);
                            }
                            *sp = s;
                        }
                    }
                } else {
                    push_df = true;
                }
            }
            qdf = warp_enqueue(wdf, qdf, push_df, t);
            if (qdf >= 32 || (r == rounds - 1 && qdf > 0)) {
                __syncwarp();
                for (int base = 0; base < qdf; base += 32) {
                    const int i = base + (threadIdx.x & 31);
                    const int ts = i < qdf ? wdf[i] : 0;
                    const bool px = i < qdf && !df_gather<C, P>(a, det, ts, wp->qd, T, Pr);
                    qn = warp_enqueue(wq, qn, px, ts);
                    if (qn > kWarpQueue - 32) drain_exact();
                }
                __syncwarp();
                qdf = 0;
            }
            if (qn > kWarpQueue - 32 || r == rounds - 1) drain_exact();
            continue;
        }
        if (t < t1) {
            float *sp = a.signal + det * a.sig_stride + t;
            const float s_in = *sp;   // loaded early, as in the mixed branch
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
                float s = s_in;
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
        if (qn > kWarpQueue - 32 || r == rounds - 1) drain_exact();
    }
}

// The two-pass mixed from_map of untiled nearest-neighbour maps (see
// mx_common.cuh).  Main pass: the float32 tier on every sample, the map
// read from its float32 copy (one 16-byte load), the signal updated where
// the sample is certified and on the map; the samples it cannot certify
// are left untouched and marked in the mask.
template <int C, int P>
__global__ void __launch_bounds__(kBlock, kMxBlocksPerSM) k_from_map_mx(GatherArgs a, MxMask mm) {
    int det, t0, t1;
    if (!seg_piece(a.segs, a.piece, det, t0, t1)) return;
    const double *dq = a.dets + 4LL * det;
    const float qd[4] = {d2f_round(__ldg(dq)), d2f_round(__ldg(dq + 1)), d2f_round(__ldg(dq + 2)),
                         d2f_round(__ldg(dq + 3))};
    const float T = __ldg(a.resp + 2 * det), Pr = __ldg(a.resp + 2 * det + 1);
    const int nc = a.g.ncomp;
    float *sig = a.signal + det * a.sig_stride;
    unsigned *mw = mm.words + ((long long)blockIdx.x * gridDim.y + blockIdx.y) * mm.wpp +
                   (threadIdx.x >> 5);
    const int rounds = (t1 - t0 + kBlock - 1) / kBlock;
    for (int r = 0; r < rounds; r++) {
        const int t = t0 + r * kBlock + threadIdx.x;
        const bool live = t < t1;
        // Loaded before the pointing, so that its latency overlaps it.
        const float s_in = live ? sig[t] : 0.f;
        float qb[4] = {1.f, 0.f, 0.f, 0.f};
        if (live) {
            const float4 b = __ldg(a.bore32 + t);
            qb[0] = b.x;
            qb[1] = b.y;
            qb[2] = b.z;
            qb[3] = b.w;
        }
        int pix[2] = {0, 0};
        float pf[3] = {0.f, 0.f, 0.f};
        bool on = false;
        const bool ok = live && mixed_pointing<C, P, true, false>(a.g, a.ft, a.mc, qb, qd, nc, T,
                                                                  Pr, pix, on, pf);
        const unsigned fails = __ballot_sync(kFull, live && !ok);
        if (fails && (threadIdx.x & 31) == 0) mw[r * (kBlock / 32)] = fails;
        if (ok && on) {
            const int key = P == PX_HP_NT ? pix[0] : pix[0] * a.g.nx + pix[1];
            const float4 m = __ldg(a.map32 + key);
            // float32 terms (the mixed-precision contract).
            float s = fmaf(m.x, pf[0], s_in);
            if (nc > 1) s = fmaf(m.y, pf[1], s);
            if (nc > 2) s = fmaf(m.z, pf[2], s);
            sig[t] = s;
        }
    }
}

// Fallback passes of k_from_map_mx, by tier: 1 the double-float pointing
// (float32 spin factors and terms), 2 the exact float64 pointing for the
// samples tier 1 could not certify.
template <int C, int P, int TIER>
__global__ void __launch_bounds__(kBlock) k_from_map_mx_fix(GatherArgs a, MxMask mm) {
    mx_for_each<TIER == 1>(a.segs, a.piece, mm, [&](int det, int t) -> bool {
        const QuatD ofs = load_quat(a.dets + 4LL * det);
        const float T = __ldg(a.resp + 2 * det), Pr = __ldg(a.resp + 2 * det + 1);
        if constexpr (TIER == 1) {
            const dfl qd[4] = {df_of(ofs.a), df_of(ofs.b), df_of(ofs.c), df_of(ofs.d)};
            return df_gather<C, P>(a, det, t, qd, T, Pr);
        } else {
            exact_gather<C, P>(a, det, t, ofs, T, Pr);
            return true;
        }
    });
}

template <int C, int P>
struct GatherMxFix {
    const GatherArgs &a;
    const MxMask &mm;
    template <int T>
    void launch(unsigned nb, cudaStream_t st) const {
        if constexpr (T > 0) k_from_map_mx_fix<C, P, T><<<nb, kBlock, 0, st>>>(a, mm);
    }
};

// The chunked from_map for CAR maps (interp_point.cuh), NC-component map,
// with four consecutive samples per lane (the layout of k_scatter_ix4), the
// map read from its float32 copy: one float4 of signal read and written per
// lane where the row is 16-byte aligned, four independent map reads.
// Samples it cannot certify keep their value (the fallback passes add
// theirs) and are marked in the mask.
template <int P, int NC>
__global__ void __launch_bounds__(kBlock, kIxBlocksPerSM)
    k_from_map_ix4(GatherArgs a, MxMask mm, const IxBore *ixb) {
    __shared__ IxParams sp[kBlock / 32][32];
    int det, t0, t1;
    if (!seg_piece(a.segs, a.piece, det, t0, t1)) return;
    const QuatD ofs = load_quat(a.dets + 4LL * det);
    const dfl qd[4] = {df_of(ofs.a), df_of(ofs.b), df_of(ofs.c), df_of(ofs.d)};
    const float q32[4] = {d2f_round(ofs.a), d2f_round(ofs.b), d2f_round(ofs.c),
                          d2f_round(ofs.d)};
    const float T = __ldg(a.resp + 2 * det), Pr = __ldg(a.resp + 2 * det + 1);
    float *sig = a.signal + det * a.sig_stride;
    const bool vec = (reinterpret_cast<unsigned long long>(sig) & 15) == 0;
    unsigned *mwb = mm.words + ((long long)blockIdx.x * gridDim.y + blockIdx.y) * mm.wpp;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tsh = P == PX_HP_T ? __ffsll(a.g.nppt) - 1 : 0;
    const int j0 = t0 / kIxLen, j1 = (t1 - 1) / kIxLen + 1;
    for (int g = j0 + warp * 32; g < j1; g += (kBlock / 32) * 32) {
        if (g + lane < j1)
            ix_setup<P == PX_HP_NT || P == PX_HP_T>(a, ixb, g + lane, a.segs.n_time, qd, q32,
                                                    sp[warp][lane]);
        __syncwarp();
        const int nch = min(32, j1 - g);
        const int rounds = (nch + 1) / 2;
        for (int r = 0; r < rounds; r++) {
            const int ck = 2 * r + (lane >> 4);
            const int tq = (g + ck) * kIxLen + (lane & 15) * 4;
            const bool lane_live = ck < nch;
            const bool whole = vec && lane_live && tq + 3 < t1;
            // Loaded before the pointing, so that its latency overlaps it.
            float sv[4] = {0.f, 0.f, 0.f, 0.f};
            if (whole) {
                const float4 v = *reinterpret_cast<const float4 *>(sig + tq);
                sv[0] = v.x;
                sv[1] = v.y;
                sv[2] = v.z;
                sv[3] = v.w;
            } else if (lane_live) {
#pragma unroll
                for (int i = 0; i < 4; i++)
                    if (tq + i < t1) sv[i] = sig[tq + i];
            }
            const IxParams &pp = sp[warp][min(ck, nch - 1)];
            unsigned f4 = 0u;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int t = tq + i;
                const bool live = lane_live && t < t1;
                int key = 0;
                bool on = false;
                float pf[3];
                const bool ok = ix_sample<P, NC>(pp, ix_s(pp, tq, i), a.g, T, Pr, key, on, pf);
                if (live && !ok) f4 |= 1u << i;
                if (live && ok && on) {
                    // Tiled: the float32 copy spans the parent map, .w = 0
                    // on the pixels of absent tiles.
                    const float4 m = __ldg(a.map32 + key);
                    if ((P == PX_HP_T || P == PX_FLAT_T_NN) && m.w == 0.f) {
                        if (P == PX_HP_T) {
                            record_missing_tile(a.err, key >> tsh);
                        } else {
                            int tp[3];
                            flat_tile_tuple(a.g, key / a.g.nx, key % a.g.nx, tp);
                            record_missing_tile(a.err, tp[0]);
                        }
                    } else {
                        // float32 terms (the mixed-precision contract).
                        float x = fmaf(m.x, pf[0], sv[i]);
                        if constexpr (NC > 1) x = fmaf(m.y, pf[1], x);
                        if constexpr (NC > 2) x = fmaf(m.z, pf[2], x);
                        sv[i] = x;
                    }
                }
            }
            if (__any_sync(kFull, f4 != 0u)) {
                unsigned x = f4 << (4 * (lane & 7));
                x |= __shfl_xor_sync(kFull, x, 1);
                x |= __shfl_xor_sync(kFull, x, 2);
                x |= __shfl_xor_sync(kFull, x, 4);
                if ((lane & 7) == 0 && x)
                    mwb[((g + 2 * r) * kIxLen - t0) / 32 + (lane >> 3)] = x;
            }
            if (whole) {
                *reinterpret_cast<float4 *>(sig + tq) = make_float4(sv[0], sv[1], sv[2], sv[3]);
            } else if (lane_live) {
#pragma unroll
                for (int i = 0; i < 4; i++)
                    if (tq + i < t1) sig[tq + i] = sv[i];
            }
        }
        __syncwarp();
    }
}

// Fallback passes of k_from_map_ix4, by tier: 0 the float32 tier, 1 the
// double-float pointing (float32 spin factors and terms), 2 the exact
// float64 pointing, each on the samples the previous tier left.
template <int P, int TIER>
__global__ void __launch_bounds__(kBlock) k_from_map_ix_fix(GatherArgs a, MxMask mm) {
    constexpr int C = SO3G_COORD_CAR;
    const int nc = a.g.ncomp;
    mx_for_each<TIER < 2>(a.segs, a.piece, mm, [&](int det, int t) -> bool {
        const QuatD ofs = load_quat(a.dets + 4LL * det);
        const float T = __ldg(a.resp + 2 * det), Pr = __ldg(a.resp + 2 * det + 1);
        if constexpr (TIER == 0) {
            const float q32[4] = {d2f_round(ofs.a), d2f_round(ofs.b), d2f_round(ofs.c),
                                  d2f_round(ofs.d)};
            float qb[4];
            load_bore_f32(a.bore32, a.bore, t, qb);
            // Tiled maps: the parent map's pixel (the float32 copy's
            // index, .w = 0 on absent tiles).
            constexpr bool kParent = P == PX_HP_T || P == PX_FLAT_T_NN;
            int pix[2];
            float pf[3] = {0.f, 0.f, 0.f};
            bool on = false;
            if (!mixed_pointing<C, P, true, kParent>(a.g, a.ft, a.mc, qb, q32, nc, T, Pr, pix, on,
                                                     pf))
                return false;
            if (on) {
                float *sp = a.signal + det * a.sig_stride + t;
                const bool hp = P == PX_HP_NT || P == PX_HP_T;
                const float4 m = __ldg(a.map32 + (hp ? (long long)pix[0]
                                                     : (long long)pix[0] * a.g.nx + pix[1]));
                if (kParent && m.w == 0.f) {
                    int tp[3];
                    parent_to_tile<P>(a.g, pix, tp);
                    record_missing_tile(a.err, tp[0]);
                    return true;
                }
                float sv = fmaf(m.x, pf[0], *sp);
                if (nc > 1) sv = fmaf(m.y, pf[1], sv);
                if (nc > 2) sv = fmaf(m.z, pf[2], sv);
                *sp = sv;
            }
            return true;
        } else if constexpr (TIER == 1) {
            const dfl qd[4] = {df_of(ofs.a), df_of(ofs.b), df_of(ofs.c), df_of(ofs.d)};
            return df_gather<C, P>(a, det, t, qd, T, Pr);
        } else {
            exact_gather<C, P>(a, det, t, ofs, T, Pr);
            return true;
        }
    });
}

template <int P>
struct GatherIxFix {
    const GatherArgs &a;
    const MxMask &mm;
    template <int T>
    void launch(unsigned nb, cudaStream_t st) const {
        k_from_map_ix_fix<P, T><<<nb, kBlock, 0, st>>>(a, mm);
    }
};

// The chunked from_map for CAR maps with the nearest-neighbour pixelizors
// and for HEALPix maps (tiled maps: the float32 copy spans the parent map);
// returns 1 (nothing launched) where it does not apply.
template <int C, int P>
int gather_interp(const GatherArgs &a, dim3 grid, cudaStream_t stream) {
    if constexpr (!(C == SO3G_COORD_CAR && (P == PX_FLAT_NT_NN || P == PX_FLAT_T_NN ||
                                            P == PX_HP_NT || P == PX_HP_T))) {
        return 1;
    } else {
        const long long npix =
            (P == PX_FLAT_NT_NN || P == PX_FLAT_T_NN) ? (long long)a.g.ny * a.g.nx : a.g.npix;
        if (a.segs.seg || a.segs.n_time < 2 || !a.map32 || npix >= (1LL << 31) ||
            a.g.ncomp < 1 || a.g.ncomp > 3 || a.piece % kIxLen ||
            (long long)grid.x * a.segs.n_time < chunked_min_samples())
            return 1;
        IxBore *ixb = ix_bore_models(a.bore, a.segs.n_time, stream);
        if (!ixb) return 1;
        MxMask mm;
        if (!mx_mask_alloc(mm, grid, a.piece, stream)) {
            cudaFreeAsync(ixb, stream);
            return 1;
        }
        if (a.g.ncomp == 1)
            k_from_map_ix4<P, 1><<<grid, kBlock, 0, stream>>>(a, mm, ixb);
        else if (a.g.ncomp == 2)
            k_from_map_ix4<P, 2><<<grid, kBlock, 0, stream>>>(a, mm, ixb);
        else
            k_from_map_ix4<P, 3><<<grid, kBlock, 0, stream>>>(a, mm, ixb);
        int rc = after_launch("from_map (chunked)");
        if (rc == SO3G_OK)
            rc = fix_tiers<0>(GatherIxFix<P>{a, mm}, mm, stream, "from_map (chunked fallback)");
        cudaFreeAsync(mm.words, stream);
        cudaFreeAsync(ixb, stream);
        return rc;
    }
}

// Runs the two passes; returns 1 (nothing launched: the caller runs
// k_from_map) when the pixelization is not eligible, the map has 2^31
// pixels or more, a float32 copy is missing, or the mask cannot be
// allocated.
template <int C, int P>
int gather_mixed(const GatherArgs &a, dim3 grid, cudaStream_t stream) {
    const int ri = gather_interp<C, P>(a, grid, stream);
    if (ri != 1) return ri;
    if constexpr (!MxEligible<C, P>::value) {
        return 1;
    } else {
        const long long npix = P == PX_HP_NT ? a.g.npix : (long long)a.g.ny * a.g.nx;
        if (!a.bore32 || !a.map32 || npix >= (1LL << 31)) return 1;
        MxMask mm;
        if (!mx_mask_alloc(mm, grid, a.piece, stream)) return 1;
        k_from_map_mx<C, P><<<grid, kBlock, 0, stream>>>(a, mm);
        int rc = after_launch("from_map (mixed)");
        if (rc == SO3G_OK)
            rc = fix_tiers<1>(GatherMxFix<C, P>{a, mm}, mm, stream, "from_map (mixed fallback)");
        cudaFreeAsync(mm.words, stream);
        return rc;
    }
}

struct GatherLaunch {
    GatherArgs a;
    dim3 grid;
    cudaStream_t stream;
    template <int C, int P>
    struct Go {
        GatherLaunch *L;
        template <int MODE>
        int go() {
            if constexpr (MODE == SO3G_POINTING_MIXED) {
                const int rc = gather_mixed<C, P>(L->a, L->grid, L->stream);
                if (rc != 1) return rc;
            }
            k_from_map<C, P, MODE><<<L->grid, kBlock, 0, L->stream>>>(L->a);
            return after_launch("from_map");
        }
    };
    template <int C, int P>
    int run() {
        Go<C, P> g{this};
        return by_mode<C, P>(a.fast, g);
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
    L.a.piece = piece_len(n_time, n_det);
    L.a.err = err;
    L.a.ft = device_fast_tables();
    L.a.fc = make_fast_const(L.a.g);
    L.a.mc = make_mixed_const(L.a.g);
    L.a.fast = fast_mode(pz, L.a.ft);
    L.grid = dim3((unsigned)n_det, (unsigned)((n_time + L.a.piece - 1) / L.a.piece));
    L.stream = (cudaStream_t)stream;
    L.a.bore32 = bore_f32(pz, L.a.fast, boresight, n_time, L.stream);
    // Mixed pointing: a float32 copy of the map, pixel by pixel (over the
    // parent map when tiled), read with one 16-byte load per sample.
    float4 *map32 = nullptr;
    const long long npix = pz->pix_sys == SO3G_PIX_HEALPIX ? L.a.g.npix
                                                           : (long long)L.a.g.ny * L.a.g.nx;
    const int kind = pix_kind(pz);
    const bool tiled_ok = kind == PX_FLAT_T_NN || kind == PX_HP_T;
    const bool mixed_bl = L.a.fast == SO3G_POINTING_MIXED && !pz->tiled &&
                          pz->pix_sys == SO3G_PIX_FLAT && pz->interp == SO3G_INTERP_BILINEAR;
    if ((L.a.bore32 || mixed_bl) &&
        (!pz->tiled || (tiled_ok && npix <= kMap32TiledMaxPixels))) {
        if (cudaMallocAsync(reinterpret_cast<void **>(&map32), sizeof(float4) * (size_t)npix,
                            L.stream) == cudaSuccess) {
            const unsigned blocks = (unsigned)((npix + kBlock - 1) / kBlock);
            if (!pz->tiled)
                k_map_f32<<<blocks, kBlock, 0, L.stream>>>(map->data, pz->n_comp, npix, map32);
            else if (kind == PX_HP_T)
                k_map_f32_tiled<PX_HP_T><<<blocks, kBlock, 0, L.stream>>>(L.a.g, map->data,
                                                                          npix, map32);
            else
                k_map_f32_tiled<PX_FLAT_T_NN><<<blocks, kBlock, 0, L.stream>>>(
                    L.a.g, map->data, npix, map32);
            if (after_launch("map float32 copy") != SO3G_OK) {
                cudaFreeAsync(map32, L.stream);
                map32 = nullptr;
                clear_error();
            }
        } else {
            cudaGetLastError();
            map32 = nullptr;
        }
    }
    L.a.map32 = map32;
    rc = dispatch_cp(pz->coord_sys, pix_kind(pz), L);
    if (map32) cudaFreeAsync(map32, L.stream);
    bore_f32_free(L.a.bore32, L.stream);
    return rc;
}
