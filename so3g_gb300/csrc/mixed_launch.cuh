// mixed_launch.cuh -- the streamlined to_map / to_weight_map of the mixed
// pointing (SO3G_POINTING_MIXED) for untiled nearest-neighbour maps: CAR,
// TAN, ZEA and SIN flat maps and HEALPix.
//
// Two kernels per call instead of one:
//
// - k_scatter_mx runs the float32 tier of mixedpoint.cuh on every sample
//   (one sample per lane, a detector piece per block, as k_scatter) and
//   accumulates what it certifies.  It keeps no fallback work of its own:
//   each warp records the samples it could not certify as one 32-bit word
//   per round (bit b = lane b) in a mask in global memory.  The loop body is
//   then only the float32 pointing, its certificate, the products and the
//   accumulation, with 32-bit pixel keys -- no per-warp queues, no inlined
//   double-float or float64 code.
// - k_scatter_mx_fix reads the mask warp by warp (32 words = 1024 samples
//   at a time), hands the set bits out to the lanes by prefix sum so that
//   every lane works on a sample, and sends each through the double-float
//   pointing (float32 spin factors: the mixed contract) and, where that
//   cannot certify the pixel either, the exact float64 pointing.
//
// The map is the same as k_scatter's up to the float64 summation order.
#pragma once

#include "mx_common.cuh"
#include "interp_point.cuh"
#include "scatter_kernel.cuh"

namespace so3g {

namespace {

// flush_runs (device.cuh) with a 32-bit pixel key (-1: nothing to add):
// runs of equal keys across the warp are summed in compensated float32 and
// flushed with one float64 atomic per run and value; a warp with at least
// DIRECT runs adds every term with its own atomic.
template <int NV, int DIRECT>
__device__ __forceinline__ void flush_runs32(int key, long long plane, float (&v)[NV],
                                             const int (&mult)[NV], unsigned vmask,
                                             double *map) {
    const int lane = threadIdx.x & 31;
    const int prev = __shfl_up_sync(kFull, key, 1);
    const bool head = (lane == 0) || (key != prev);
    const unsigned heads = __ballot_sync(kFull, head);
    if (__popc(heads) >= DIRECT) {
        if (key >= 0) {
            double *p = map + key;
#pragma unroll
            for (int k = 0; k < NV; k++)
                if ((vmask >> k) & 1u) atomicAdd(p + mult[k] * plane, f2d(v[k]));
        }
        return;
    }
    const unsigned after = heads & ~((2u << lane) - 1u);
    const int end = after ? (__ffs(after) - 1) : 32;
    const int span = head ? end - lane : 1;
    const int maxrun = __reduce_max_sync(kFull, (unsigned)span);
    float e[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) e[k] = 0.f;
    for (int d = 1; d < maxrun; d <<= 1) {
        const bool take = lane + d < end;
#pragma unroll
        for (int k = 0; k < NV; k++) {
            if (!((vmask >> k) & 1u)) continue;
            const float os = __shfl_down_sync(kFull, v[k], d);
            const float oe = __shfl_down_sync(kFull, e[k], d);
            if (take) {
                float s, r;
                two_sum(v[k], os, s, r);
                v[k] = s;
                e[k] += oe + r;
            }
        }
    }
    if (head && key >= 0) {
        double *p = map + key;
#pragma unroll
        for (int k = 0; k < NV; k++)
            if ((vmask >> k) & 1u) atomicAdd(p + mult[k] * plane, f2d(v[k]) + f2d(e[k]));
    }
}

// The main pass.  Block (x, y): piece y of segment x, in rounds of kBlock
// samples (lane = sample).  Needs the float32 boresight copy (a.bore32).
template <int C, int P, bool WEIGHT>
__global__ void __launch_bounds__(kBlock, kMxBlocksPerSM) k_scatter_mx(ScatterArgs a, MxMask mm) {
    int det, t0, t1;
    if (!seg_piece(a.segs, a.piece, det, t0, t1)) return;
    float det_wt = 1.f;
    if (a.det_weights) {
        det_wt = __ldg(a.det_weights + det);
        if (det_wt == 0.f) return;  // src/Projection.cxx:1784-1788
    }
    const double *dq = a.dets + 4LL * det;
    const float qd[4] = {d2f_round(__ldg(dq)), d2f_round(__ldg(dq + 1)), d2f_round(__ldg(dq + 2)),
                         d2f_round(__ldg(dq + 3))};
    const float T = __ldg(a.resp + 2 * det), Pr = __ldg(a.resp + 2 * det + 1);
    const int nc = a.g.ncomp;
    constexpr int NV = WEIGHT ? 6 : 3;
    int mult[NV];
    const unsigned vmask = value_slots<WEIGHT>(nc, mult);
    const long long plane = P == PX_HP_NT ? a.g.npix : (long long)a.g.ny * a.g.nx;
    const float *sig = a.signal + det * a.sig_stride;
    unsigned *mw = mm.words + ((long long)blockIdx.x * gridDim.y + blockIdx.y) * mm.wpp +
                   (threadIdx.x >> 5);
    const int rounds = (t1 - t0 + kBlock - 1) / kBlock;
    for (int r = 0; r < rounds; r++) {
        const int t = t0 + r * kBlock + threadIdx.x;
        const bool live = t < t1;
        const float s = (!WEIGHT && live) ? __ldg(sig + t) : 0.f;
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
        int key = -1;
        if (ok && on) key = P == PX_HP_NT ? pix[0] : pix[0] * a.g.nx + pix[1];
        float v[NV];
        tap_values<WEIGHT, NV, true>(s, pf, 1.f, det_wt, v);
        if (a.accum == SO3G_ACCUM_WARP_RUNS) {
            flush_runs32<NV, kDirectRuns>(key, plane, v, mult, vmask, a.map);
        } else if (key >= 0) {
            double *p = a.map + key;
#pragma unroll
            for (int k = 0; k < NV; k++)
                if ((vmask >> k) & 1u) atomicAdd(p + mult[k] * plane, f2d(v[k]));
        }
    }
}

// The fallback passes of k_scatter_mx, by tier: 1 the double-float
// pointing (float32 spin factors and terms), 2 the exact float64 pointing
// for the samples tier 1 could not certify.
template <int C, int P, bool WEIGHT, int TIER>
__global__ void __launch_bounds__(kBlock) k_scatter_mx_fix(ScatterArgs a, MxMask mm) {
    constexpr int NV = WEIGHT ? 6 : 3;
    int mult[NV];
    const unsigned vmask = value_slots<WEIGHT>(a.g.ncomp, mult);
    mx_for_each<TIER == 1>(a.segs, a.piece, mm, [&](int det, int t) -> bool {
        const float det_wt = a.det_weights ? __ldg(a.det_weights + det) : 1.f;
        const QuatD ofs = load_quat(a.dets + 4LL * det);
        const float T = __ldg(a.resp + 2 * det), Pr = __ldg(a.resp + 2 * det + 1);
        if constexpr (TIER == 1) {
            const dfl qd[4] = {df_of(ofs.a), df_of(ofs.b), df_of(ofs.c), df_of(ofs.d)};
            return df_sample<C, P, WEIGHT, false>(a, det, t, qd, T, Pr, det_wt, mult, vmask);
        } else {
            exact_sample<C, P, WEIGHT>(a, det, t, ofs, T, Pr, det_wt, mult, vmask);
            return true;
        }
    });
}

// Plane offsets (32-bit) and values of one nearest-neighbour sample of an
// NC-component map: to_map adds sig * pf[c] * det_wt to plane c; to_weight_map
// adds pf[i] * pf[j] * det_wt to plane i * NC + j (i <= j), as k_scatter
// (float32 products, left to right).
template <bool WEIGHT, int NC>
struct IxValues {
    static constexpr int NV = WEIGHT ? NC * (NC + 1) / 2 : NC;
    __device__ static void offsets(int plane, int (&off)[NV]) {
        if constexpr (!WEIGHT) {
#pragma unroll
            for (int c = 0; c < NC; c++) off[c] = c * plane;
        } else {
            int k = 0;
#pragma unroll
            for (int i = 0; i < NC; i++)
#pragma unroll
                for (int j = i; j < NC; j++, k++) off[k] = (i * NC + j) * plane;
        }
    }
    __device__ static void values(float sig, const float (&pf)[3], float det_wt,
                                  float (&v)[NV]) {
        if constexpr (!WEIGHT) {
#pragma unroll
            for (int c = 0; c < NC; c++) v[c] = sig * pf[c] * det_wt;
        } else {
            int k = 0;
#pragma unroll
            for (int i = 0; i < NC; i++)
#pragma unroll
                for (int j = i; j < NC; j++, k++) v[k] = pf[i] * pf[j] * det_wt;
        }
    }
};

// Map element of a chunked sample's key (key < 0: none): key itself on an
// untiled map; on a tiled HEALPix map (key = the parent NEST index) the
// element of its tile (tile = key >> tsh, tsh = log2 of the pixels per
// tile), NULL with the missing-tile error recorded when the tile is absent.
// (Tiled flat maps: ix_flush_run.)
template <int P>
__device__ __forceinline__ double *ix_base(const ScatterArgs &a, int key, int tsh) {
    if (key < 0) return nullptr;
    if constexpr (P != PX_HP_T) {
        return a.map + key;
    } else {
        const int tile = key >> tsh;
        const long long toff = __ldg(a.g.tile_offset + tile);
        if (toff < 0) {
            record_missing_tile(a.err, tile);
            return nullptr;
        }
        return a.map + toff + (key & ((1 << tsh) - 1));
    }
}

// One run total of k_scatter_ix4 added to the map (key < 0: nothing); off
// holds the values' plane offsets within the map (or the HEALPix tile).  A
// tiled flat map's key (the parent map's iy * nx + ix) is split into its
// tile tuple when the run is flushed, the tile's own plane size (edge
// tiles are smaller) giving the offsets.  aux: log2 of the pixels per tile
// (tiled HEALPix), the bits of 1/nx as a float (tiled flat).
template <int P, bool WEIGHT, int NC, int NV>
__device__ __forceinline__ void ix_flush_run(const ScatterArgs &a, int key, int aux,
                                             const int (&off)[NV], const float (&v)[NV]) {
    if constexpr (P == PX_FLAT_T_NN) {
        if (key < 0) return;
        const int iy = div_small(key, a.g.nx, __int_as_float(aux)), ix = key - iy * a.g.nx;
        int tp[3];
        flat_tile_tuple(a.g, iy, ix, tp);
        long long o, plane;
        const int bad = locate<P>(a.g, tp, &o, &plane);
        if (bad >= 0) {
            record_missing_tile(a.err, bad);
            return;
        }
        int po[NV];
        IxValues<WEIGHT, NC>::offsets((int)plane, po);
#pragma unroll
        for (int k = 0; k < NV; k++) atomicAdd(a.map + o + po[k], f2d(v[k]));
    } else {
        double *p = ix_base<P>(a, key, aux);
        if (p) {
#pragma unroll
            for (int k = 0; k < NV; k++) atomicAdd(p + off[k], f2d(v[k]));
        }
    }
}

// to_map / to_weight_map of the chunked pass with four consecutive samples
// per lane: round r of a group covers its chunks 2r (lanes 0-15) and 2r + 1
// (lanes 16-31), one float4 of signal per lane (to_map).  A lane sums the
// runs of equal pixels among its four samples (right to left, at most four
// float32 terms: each total within 3u of the exact sum of its terms'
// magnitudes) and packs them into run slots 0..3; slot j of every lane is
// flushed with one float64 atomic per component in one pass, taken only
// when some lane has more than j runs.  Runs are a few samples long, so a
// round of 128 samples takes about two passes of atomics instead of the
// four that one sample per lane needs, and a fraction of the L2 atomics.
// Samples it cannot certify are marked in the mask (bit b of word w = lane
// 8w + b/4, sample b % 4).
template <int P, bool WEIGHT, int NC>
__global__ void __launch_bounds__(kBlock, kIxBlocksPerSM)
    k_scatter_ix4(ScatterArgs a, MxMask mm, const IxBore *ixb) {
    __shared__ IxParams sp[kBlock / 32][32];
    int det, t0, t1;
    if (!seg_piece(a.segs, a.piece, det, t0, t1)) return;
    float det_wt = 1.f;
    if (a.det_weights) {
        det_wt = __ldg(a.det_weights + det);
        if (det_wt == 0.f) return;  // src/Projection.cxx:1784-1788
    }
    const QuatD ofs = load_quat(a.dets + 4LL * det);
    const dfl qd[4] = {df_of(ofs.a), df_of(ofs.b), df_of(ofs.c), df_of(ofs.d)};
    const float q32[4] = {d2f_round(ofs.a), d2f_round(ofs.b), d2f_round(ofs.c),
                          d2f_round(ofs.d)};
    const float T = __ldg(a.resp + 2 * det), Pr = __ldg(a.resp + 2 * det + 1);
    using V = IxValues<WEIGHT, NC>;
    constexpr int NV = V::NV;
    int off[NV];
    V::offsets(P == PX_HP_NT ? (int)a.g.npix : (P == PX_HP_T ? (int)a.g.nppt : a.g.ny * a.g.nx),
               off);
    const int aux = P == PX_HP_T ? __ffsll(a.g.nppt) - 1
                    : (P == PX_FLAT_T_NN ? __float_as_int(1.f / (float)a.g.nx) : 0);
    const float *sig = WEIGHT ? nullptr : a.signal + det * a.sig_stride;
    const bool vec = (reinterpret_cast<unsigned long long>(sig) & 15) == 0;
    unsigned *mwb = mm.words + ((long long)blockIdx.x * gridDim.y + blockIdx.y) * mm.wpp;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j0 = t0 / kIxLen, j1 = (t1 - 1) / kIxLen + 1;
    // The four samples of this lane from tq, zeros past t1.
    auto load4 = [&](int tq) {
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
        if (WEIGHT) return r;
        if (vec && tq + 3 < t1) {
            r = __ldg(reinterpret_cast<const float4 *>(sig + tq));
        } else {
            if (tq < t1) r.x = __ldg(sig + tq);
            if (tq + 1 < t1) r.y = __ldg(sig + tq + 1);
            if (tq + 2 < t1) r.z = __ldg(sig + tq + 2);
            if (tq + 3 < t1) r.w = __ldg(sig + tq + 3);
        }
        return r;
    };
    for (int g = j0 + warp * 32; g < j1; g += (kBlock / 32) * 32) {
        if (g + lane < j1)
            ix_setup<P == PX_HP_NT || P == PX_HP_T>(a, ixb, g + lane, a.segs.n_time, qd, q32,
                                                    sp[warp][lane]);
        __syncwarp();
        const int nch = min(32, j1 - g);
        const int rounds = (nch + 1) / 2;
        const int half = lane >> 4;
        float4 sn = half < nch ? load4((g + half) * kIxLen + (lane & 15) * 4)
                               : make_float4(0.f, 0.f, 0.f, 0.f);
        for (int r = 0; r < rounds; r++) {
            const float4 sc = sn;
            const int ck = 2 * r + half;
            if (r + 1 < rounds && ck + 2 < nch) sn = load4((g + ck + 2) * kIxLen + (lane & 15) * 4);
            const int tq = (g + ck) * kIxLen + (lane & 15) * 4;
            const bool lane_live = ck < nch;
            const IxParams &pp = sp[warp][min(ck, nch - 1)];
            const float sg[4] = {sc.x, sc.y, sc.z, sc.w};
            int key[4];
            float v[4][NV];
            unsigned f4 = 0u;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int t = tq + i;
                const bool live = lane_live && t < t1;
                int kk = 0;
                bool on = false;
                float pf[3];
                const bool ok = ix_sample<P, NC>(pp, ix_s(pp, tq, i), a.g, T, Pr, kk, on, pf);
                if (live && !ok) f4 |= 1u << i;
                key[i] = (live && ok && on) ? kk : -1;
                V::values(sg[i], pf, det_wt, v[i]);
            }
            if (__any_sync(kFull, f4 != 0u)) {
                unsigned x = f4 << (4 * (lane & 7));
                x |= __shfl_xor_sync(kFull, x, 1);
                x |= __shfl_xor_sync(kFull, x, 2);
                x |= __shfl_xor_sync(kFull, x, 4);
                if ((lane & 7) == 0 && x)
                    mwb[((g + 2 * r) * kIxLen - t0) / 32 + (lane >> 3)] = x;
            }
            if (a.accum != SO3G_ACCUM_WARP_RUNS) {
#pragma unroll
                for (int i = 0; i < 4; i++)
                    ix_flush_run<P, WEIGHT, NC, NV>(a, key[i], aux, off, v[i]);
                continue;
            }
            // Run heads and right-to-left run totals (in place: v[i] becomes
            // the total of the run from i while i is in it).
            const bool h1 = key[1] != key[0], h2 = key[2] != key[1], h3 = key[3] != key[2];
#pragma unroll
            for (int k = 0; k < NV; k++) {
                if (!h3) v[2][k] += v[3][k];
                if (!h2) v[1][k] += v[2][k];
                if (!h1) v[0][k] += v[1][k];
            }
            // Slots 1 and 2: the first and second heads among samples 1..3;
            // slot 3: sample 3 when all three are heads.
            const int nruns = 1 + h1 + h2 + h3;
            int ks1 = key[3], ks2 = key[3];
            float s1[NV], s2[NV];
#pragma unroll
            for (int k = 0; k < NV; k++) {
                s1[k] = h1 ? v[1][k] : (h2 ? v[2][k] : v[3][k]);
                s2[k] = (h1 && h2) ? v[2][k] : v[3][k];
            }
            ks1 = h1 ? key[1] : (h2 ? key[2] : key[3]);
            ks2 = (h1 && h2) ? key[2] : key[3];
            ix_flush_run<P, WEIGHT, NC, NV>(a, key[0], aux, off, v[0]);
            if (__any_sync(kFull, nruns > 1) && nruns > 1)
                ix_flush_run<P, WEIGHT, NC, NV>(a, ks1, aux, off, s1);
            if (__any_sync(kFull, nruns > 2) && nruns > 2)
                ix_flush_run<P, WEIGHT, NC, NV>(a, ks2, aux, off, s2);
            if (__any_sync(kFull, nruns > 3) && nruns > 3)
                ix_flush_run<P, WEIGHT, NC, NV>(a, key[3], aux, off, v[3]);
        }
        __syncwarp();
    }
}

// The fallback passes of k_scatter_ix4, by tier: 0 the float32 tier, 1 the
// double-float pointing (float32 spin factors and terms), 2 the exact
// float64 pointing, each on the samples the previous tier left.
template <int P, bool WEIGHT, int TIER>
__global__ void __launch_bounds__(kBlock) k_scatter_ix_fix(ScatterArgs a, MxMask mm) {
    constexpr int C = SO3G_COORD_CAR;
    constexpr int NV = WEIGHT ? 6 : 3;
    int mult[NV];
    const int nc = a.g.ncomp;
    const unsigned vmask = value_slots<WEIGHT>(nc, mult);
    mx_for_each<TIER < 2>(a.segs, a.piece, mm, [&](int det, int t) -> bool {
        const float det_wt = a.det_weights ? __ldg(a.det_weights + det) : 1.f;
        const QuatD ofs = load_quat(a.dets + 4LL * det);
        const float T = __ldg(a.resp + 2 * det), Pr = __ldg(a.resp + 2 * det + 1);
        if constexpr (TIER == 0) {
            const float q32[4] = {d2f_round(ofs.a), d2f_round(ofs.b), d2f_round(ofs.c),
                                  d2f_round(ofs.d)};
            float qb[4];
            load_bore_f32(a.bore32, a.bore, t, qb);
            int pix[3];   // a tiled flat map's tuple: tile, row, column
            float pf[3] = {0.f, 0.f, 0.f};
            bool on = false;
            if (!mixed_pointing<C, P, true, false>(a.g, a.ft, a.mc, qb, q32, nc, T, Pr, pix, on,
                                                   pf))
                return false;
            if (on) {
                long long off, plane;
                const int bad = locate<P>(a.g, pix, &off, &plane);
                if (bad >= 0) {
                    record_missing_tile(a.err, bad);
                    return true;
                }
                const float sg = WEIGHT ? 0.f : __ldg(a.signal + det * a.sig_stride + t);
                float v[NV];
                tap_values<WEIGHT, NV, true>(sg, pf, 1.f, det_wt, v);
#pragma unroll
                for (int q = 0; q < NV; q++)
                    if ((vmask >> q) & 1u) atomicAdd(a.map + off + mult[q] * plane, f2d(v[q]));
            }
            return true;
        } else if constexpr (TIER == 1) {
            const dfl qd[4] = {df_of(ofs.a), df_of(ofs.b), df_of(ofs.c), df_of(ofs.d)};
            return df_sample<C, P, WEIGHT, false>(a, det, t, qd, T, Pr, det_wt, mult, vmask);
        } else {
            exact_sample<C, P, WEIGHT>(a, det, t, ofs, T, Pr, det_wt, mult, vmask);
            return true;
        }
    });
}

template <int P, bool WEIGHT>
struct ScatterIxFix {
    const ScatterArgs &a;
    const MxMask &mm;
    template <int T>
    void launch(unsigned nb, cudaStream_t st) const {
        k_scatter_ix_fix<P, WEIGHT, T><<<nb, kBlock, 0, st>>>(a, mm);
    }
};

template <int C, int P, bool WEIGHT>
struct ScatterMxFix {
    const ScatterArgs &a;
    const MxMask &mm;
    template <int T>
    void launch(unsigned nb, cudaStream_t st) const {
        if constexpr (T > 0) k_scatter_mx_fix<C, P, WEIGHT, T><<<nb, kBlock, 0, st>>>(a, mm);
    }
};

// The chunked pointing for CAR maps with the nearest-neighbour pixelizors
// and for HEALPix maps (untiled or tiled), over whole detectors
// (no sample segments); returns 1 (nothing launched) where it does not
// apply or an allocation fails.
template <int C, int P, bool WEIGHT>
int scatter_interp(const ScatterArgs &a, dim3 grid, cudaStream_t stream) {
    if constexpr (!(C == SO3G_COORD_CAR && (P == PX_FLAT_NT_NN || P == PX_FLAT_T_NN ||
                                            P == PX_HP_NT || P == PX_HP_T))) {
        return 1;
    } else {
        // Keys and plane offsets (key + plane offset untiled; within a tile
        // tiled) in 32 bits.
        const long long nc = a.g.ncomp;
        const long long npix =
            (P == PX_FLAT_NT_NN || P == PX_FLAT_T_NN) ? (long long)a.g.ny * a.g.nx : a.g.npix;
        if (a.segs.seg || a.segs.n_time < 2 || nc < 1 || nc > 3 ||
            (WEIGHT ? nc * nc : nc) * npix >= (1LL << 31) || a.piece % kIxLen ||
            (long long)grid.x * a.segs.n_time < chunked_min_samples())
            return 1;
        IxBore *ixb = ix_bore_models(a.bore, a.segs.n_time, stream);
        if (!ixb) return 1;
        MxMask mm;
        if (!mx_mask_alloc(mm, grid, a.piece, stream)) {
            cudaFreeAsync(ixb, stream);
            return 1;
        }
        if (nc == 1)
            k_scatter_ix4<P, WEIGHT, 1><<<grid, kBlock, 0, stream>>>(a, mm, ixb);
        else if (nc == 2)
            k_scatter_ix4<P, WEIGHT, 2><<<grid, kBlock, 0, stream>>>(a, mm, ixb);
        else
            k_scatter_ix4<P, WEIGHT, 3><<<grid, kBlock, 0, stream>>>(a, mm, ixb);
        int rc = after_launch(WEIGHT ? "to_weight_map (chunked)" : "to_map (chunked)");
        if (rc == SO3G_OK)
            rc = fix_tiers<0>(ScatterIxFix<P, WEIGHT>{a, mm}, mm, stream,
                              WEIGHT ? "to_weight_map (chunked fallback)"
                                     : "to_map (chunked fallback)");
        cudaFreeAsync(mm.words, stream);
        cudaFreeAsync(ixb, stream);
        return rc;
    }
}

// Runs the two passes on a.segs / grid; returns 1 (nothing launched, the
// caller runs k_scatter) when the pixelization is not eligible, the map
// index does not fit 31 bits, or the mask cannot be allocated.
template <int C, int P, bool WEIGHT>
int scatter_mixed(const ScatterArgs &a, dim3 grid, cudaStream_t stream) {
    const int ri = scatter_interp<C, P, WEIGHT>(a, grid, stream);
    if (ri != 1) return ri;
    if constexpr (!MxEligible<C, P>::value) {
        return 1;
    } else {
        const long long npix = P == PX_HP_NT ? a.g.npix : (long long)a.g.ny * a.g.nx;
        if (!a.bore32 || npix >= (1LL << 31)) return 1;
        MxMask mm;
        if (!mx_mask_alloc(mm, grid, a.piece, stream)) return 1;
        k_scatter_mx<C, P, WEIGHT><<<grid, kBlock, 0, stream>>>(a, mm);
        int rc = after_launch(WEIGHT ? "to_weight_map (mixed)" : "to_map (mixed)");
        if (rc == SO3G_OK)
            rc = fix_tiers<1>(ScatterMxFix<C, P, WEIGHT>{a, mm}, mm, stream,
                              WEIGHT ? "to_weight_map (mixed fallback)"
                                     : "to_map (mixed fallback)");
        cudaFreeAsync(mm.words, stream);
        return rc;
    }
}

}  // namespace

}  // namespace so3g
