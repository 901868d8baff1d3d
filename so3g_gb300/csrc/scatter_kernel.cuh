// scatter_kernel.cuh -- the to_map / to_weight_map kernel, shared by the
// entry points of scatter.cu and noalloc.cu.
//
// Work layout: block (x, y) takes piece y of sample segment x (one detector
// and a contiguous range of its samples) in rounds of blockDim.x
// consecutive samples, lane = sample.  Consecutive samples of a scanning
// detector tend to fall in the same pixel, which the WARP_RUNS accumulator
// exploits: runs of equal pixels across the warp are summed in registers
// (compensated float32) and flushed with one float64 atomic per run and
// component.  The ATOMIC accumulator adds every term on its own.
//
// Pointing (ScatterArgs::fast): CAR, TAN, ZEA and SIN with flat pixelizors
// and CAR HEALPix use the certified double-float pointing of fastpoint.cuh.
// Their nearest-neighbour forms take the float32 tier of mixedpoint.cuh
// first: the mixed mode for the pixel and the spin factors, the certified
// mode for the pixel only (its spin factors from df_spin_only).  Samples a
// tier cannot certify are queued in shared memory (per warp) and go, 32 at
// a time, to the double-float path and from there to the exact float64
// pointing, with plain atomics.  Every other case uses the exact pointing.
#pragma once

#include "host.h"
#include "fastpoint.cuh"
#include "mixedpoint.cuh"

namespace so3g {

// Internal linkage: every translation unit that includes this header gets
// its own instantiations.
namespace {

// Resident blocks per SM the scatter kernels are compiled for (caps their
// registers at 65536 / (kBlock * 5) = 51).  The mixed-pointing variants,
// with more memory-latency stalls, run 7 (36 registers): measured 9 %
// faster than 5 despite the extra spills.
constexpr int kScatterBlocksPerSM = 5;
constexpr int kMixedBlocksPerSM = 7;

struct ScatterArgs {
    DGeom g;
    const double *bore;
    const double *dets;
    const float *resp;
    const float *signal;
    long long sig_stride;
    const float *det_weights;
    Segs segs;
    int piece;
    int accum;
    int *err;
    double *map;
    int fast;           // SO3G_POINTING_*: 0 exact, 1 certified, 2 mixed
    FastTables ft;
    FastConst fc;
    MixedConst mc;
    const float4 *bore32;   // float32 boresight (mixed pointing), or NULL
};


// Value slots: to_map slot c = component c; to_weight_map slots are the
// upper-triangle pairs (i, j), j >= i, in row order.
template <bool WEIGHT>
__device__ __forceinline__ unsigned value_slots(int nc, int *mult) {
    unsigned vmask = 0;
    if (!WEIGHT) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            mult[c] = c;
            if (c < nc) vmask |= 1u << c;
        }
    } else {
        int k = 0;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = i; j < 3; j++, k++) {
                mult[k] = i * nc + j;
                if (i < nc && j < nc) vmask |= 1u << k;
            }
    }
    return vmask;
}

// UNIT_W: a nearest-neighbour tap, whose weight is exactly 1 (the
// multiplications by it are exact and are left out).
template <bool WEIGHT, int NV, bool UNIT_W = false>
__device__ __forceinline__ void tap_values(float sig, const float *pf, float w, float det_wt,
                                           float (&v)[NV]) {
    if (!WEIGHT) {
        // src/Projection.cxx:1807 -- float32 product, left to right
#pragma unroll
        for (int c = 0; c < 3; c++) v[c] = UNIT_W ? sig * pf[c] * det_wt : sig * pf[c] * w * det_wt;
    } else {
        // src/Projection.cxx:1850
        int s = 0;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = i; j < 3; j++, s++)
                v[s] = UNIT_W ? pf[i] * pf[j] * det_wt : pf[i] * pf[j] * w * w * det_wt;
    }
}

// One sample through the exact float64 pointing, added with plain atomics.
// Not inlined: it runs for few, compacted samples, and inlined its float64
// registers would weigh on the main loop.
template <int C, int P, bool WEIGHT>
__device__ __noinline__ void exact_sample(const ScatterArgs &a, int det, int t, const QuatD &ofs, float T,
                             float Pr, float det_wt, const int *mult, unsigned vmask) {
    constexpr int NT = PixTraits<P>::taps;
    constexpr int NV = WEIGHT ? 6 : 3;
    double coords[4];
    float pf[3];
    int pix[NT][3];
    float w[NT];
    get_coords<C>(a.g.lut, load_quat(a.bore + 4LL * t), ofs, coords);
    spin_factors(a.g.ncomp, coords, T, Pr, pf);
    const float sig = WEIGHT ? 0.f : __ldg(a.signal + det * a.sig_stride + t);
    const int n = get_pixels<P>(a.g, coords, pix, w);
    for (int k = 0; k < n; k++) {
        long long off, plane;
        int bad = locate<P>(a.g, pix[k], &off, &plane);
        if (bad >= 0) {
            record_missing_tile(a.err, bad);
            continue;
        }
        float v[NV];
        tap_values<WEIGHT>(sig, pf, w[k], det_wt, v);
#pragma unroll
        for (int s = 0; s < NV; s++)
            if ((vmask >> s) & 1u) atomicAdd(a.map + off + mult[s] * plane, f2d(v[s]));
    }
}

// One sample of the float32 tier's fallback through the double-float
// pointing, added with plain atomics; false (nothing added) when its pixel
// (CERT: or a spin factor) is not certified.  Without CERT its spin
// factors, like the float32 tier's, are float32 evaluations (the
// mixed-precision contract).
template <int C, int P, bool WEIGHT, bool CERT = false>
__device__ __forceinline__ bool df_sample(const ScatterArgs &a, int det, int t, const dfl (&qd)[4], float T,
                          float Pr, float det_wt, const int *mult, unsigned vmask) {
    constexpr int NT = PixTraits<P>::taps;
    constexpr int NV = WEIGHT ? 6 : 3;
    const double *bp = a.bore + 4LL * t;
    const double2 lo = __ldg(reinterpret_cast<const double2 *>(bp));
    const double2 hi = __ldg(reinterpret_cast<const double2 *>(bp) + 1);
    dfl qb[4];
    if (!(df_split(lo.x, qb[0]) & df_split(lo.y, qb[1]) & df_split(hi.x, qb[2]) &
          df_split(hi.y, qb[3])))
        return false;
    int pix[NT][3];
    float w[NT], pf[3];
    int n = 0;
    if (!fast_pointing<C, P, CERT>(a.g, a.ft, a.fc, qb, qd, a.g.ncomp, T, Pr, pix, w, n, pf))
        return false;
    const float sig = (!WEIGHT && n > 0) ? __ldg(a.signal + det * a.sig_stride + t) : 0.f;
    for (int k = 0; k < n; k++) {
        long long off, plane;
        int bad = locate<P>(a.g, pix[k], &off, &plane);
        if (bad >= 0) {
            record_missing_tile(a.err, bad);
            continue;
        }
        float v[NV];
        tap_values<WEIGHT>(sig, pf, w[k], det_wt, v);
#pragma unroll
        for (int s = 0; s < NV; s++)
            if ((vmask >> s) & 1u) atomicAdd(a.map + off + mult[s] * plane, f2d(v[s]));
    }
    return true;
}

// Pointing variant a kernel is compiled for: 0 exact, 1 certified, 2 mixed
// (the modes a pixelization does not support fall back to the next lower).
template <int C, int P, int MODE>
struct PointingVariant {
    static constexpr bool fast = FastEligible<C, P>::value && MODE >= 1;
    // The float32 tier decides the pixel (mixed pointing: and the spin
    // factors); the samples it leaves go to the double-float path.
    static constexpr bool mixed = MixedEligible<C, P>::value && MODE >= 1;
    // Certified pointing: spin factors certified in double-float
    // (df_spin_only) after the float32 tier's pixel.
    static constexpr bool cert = MODE == 1;
};

// Shared ints of a block's fallback queues: per warp, one queue for the
// exact path and (mixed pointing) one for the double-float path.
template <int C, int P, int MODE>
struct QueueInts {
    static constexpr int value = !PointingVariant<C, P, MODE>::fast ? 1
                                 : (PointingVariant<C, P, MODE>::mixed ? 2 : 1) *
                                       (kBlock / 32) * kWarpQueue;
};

// Samples [t0, t1) of detector `det`; every thread of the block calls it
// with the same arguments.  s_queue: the block's fallback queues
// (QueueInts<C, P, MODE> ints).
template <int C, int P, bool WEIGHT, int MODE>
__device__ __forceinline__ void scatter_piece(const ScatterArgs &a, int det, int t0, int t1,
                                              int *s_queue, WarpPiece *s_wp) {
    constexpr bool kFastOK = PointingVariant<C, P, MODE>::fast;
    float det_wt = 1.f;
    if (a.det_weights) {
        det_wt = __ldg(a.det_weights + det);
        if (det_wt == 0.f) return;  // src/Projection.cxx:1784-1788
    }
    const QuatD ofs = load_quat(a.dets + 4LL * det);
    const float T = __ldg(a.resp + 2 * det), Pr = __ldg(a.resp + 2 * det + 1);
    const int nc = a.g.ncomp;
    constexpr int NT = PixTraits<P>::taps;
    constexpr int NV = WEIGHT ? 6 : 3;
    int mult[NV];
    const unsigned vmask = value_slots<WEIGHT>(nc, mult);
    constexpr bool kMixedOK = PointingVariant<C, P, MODE>::mixed;
    constexpr bool fast = kFastOK;
    constexpr bool mixed = kMixedOK;
    dfl qd[4];
    float qd32[4];
    int *wq = s_queue + (threadIdx.x >> 5) * kWarpQueue;
    int *wdf = s_queue + ((kBlock >> 5) + (threadIdx.x >> 5)) * kWarpQueue;
    int qn = 0, qdf = 0;
    WarpPiece *wp = s_wp + (threadIdx.x >> 5);
    if (kFastOK && fast) {
        qd[0] = df_of(ofs.a);
        qd[1] = df_of(ofs.b);
        qd[2] = df_of(ofs.c);
        qd[3] = df_of(ofs.d);
        __syncwarp();
        if ((threadIdx.x & 31) == 0) {
            wp->ofs = ofs;
#pragma unroll
            for (int k = 0; k < 4; k++) wp->qd[k] = qd[k];
        }
        __syncwarp();
    }
    if (kMixedOK && mixed) {
        qd32[0] = d2f_round(ofs.a);
        qd32[1] = d2f_round(ofs.b);
        qd32[2] = d2f_round(ofs.c);
        qd32[3] = d2f_round(ofs.d);
    }
    // Recomputes the exact-path queue with the float64 pointing.
    auto drain_exact = [&]() {
        __syncwarp();
        for (int i = threadIdx.x & 31; i < qn; i += 32)
            exact_sample<C, P, WEIGHT>(a, det, wq[i], wp->ofs, T, Pr, det_wt, mult, vmask);
        __syncwarp();
        qn = 0;
    };
    const int rounds = (t1 - t0 + blockDim.x - 1) / blockDim.x;
    for (int r = 0; r < rounds; r++) {
        const int t = t0 + r * blockDim.x + threadIdx.x;
        const bool live = t < t1;
        float pf[3] = {0.f, 0.f, 0.f};
        int pix[NT][3];
        float w[NT];
        int n = 0;
        float sig = 0.f;
        bool push = false, push_df = false;
        // The sample's signal is loaded before its pointing is evaluated, so
        // that the load's latency (long for a signal in host memory, read
        // over the host link) overlaps the pointing arithmetic.
        const float sig_in = (!WEIGHT && live) ? __ldg(a.signal + det * a.sig_stride + t) : 0.f;
        if (live) {
            bool done = false;
            if (kMixedOK && mixed) {
                bool ok, on = false;
                if constexpr (PointingVariant<C, P, MODE>::cert) {
                    // The float32 tier's pixel from the float64 boresight's
                    // double-float split (hi: within u(1 + 2^-22) of it),
                    // the certified spin factors from the split itself.
                    const double *bp = a.bore + 4LL * t;
                    const double2 lo = __ldg(reinterpret_cast<const double2 *>(bp));
                    const double2 hi = __ldg(reinterpret_cast<const double2 *>(bp) + 1);
                    dfl qb[4];
                    ok = df_split(lo.x, qb[0]) & df_split(lo.y, qb[1]) & df_split(hi.x, qb[2]) &
                         df_split(hi.y, qb[3]);
                    const float qbf[4] = {qb[0].hi, qb[1].hi, qb[2].hi, qb[3].hi};
                    ok = ok && mixed_pointing<C, P, false>(a.g, a.ft, a.mc, qbf, qd32, nc, T, Pr,
                                                           pix[0], on, pf);
                    if (ok && on) ok = df_spin_only<C>(qb, qd, nc, T, Pr, pf);
                } else {
                    float qb[4];
                    load_bore_f32(a.bore32, a.bore, t, qb);
                    ok = mixed_pointing<C, P>(a.g, a.ft, a.mc, qb, qd32, nc, T, Pr, pix[0], on,
                                              pf);
                }
                if (ok) {
                    n = on ? 1 : 0;
                    w[0] = 1.f;
                } else {
                    push_df = true;
                    n = 0;
                }
                done = true;
            } else if (kFastOK && fast) {
                const double *bp = a.bore + 4LL * t;
                const double2 lo = __ldg(reinterpret_cast<const double2 *>(bp));
                const double2 hi = __ldg(reinterpret_cast<const double2 *>(bp) + 1);
                dfl qb[4];
                bool ok = df_split(lo.x, qb[0]) & df_split(lo.y, qb[1]) &
                          df_split(hi.x, qb[2]) & df_split(hi.y, qb[3]);
                // Mixed pointing (bilinear): spin factors the nearest floats.
                if (!(ok && fast_pointing<C, P, MODE != 2>(a.g, a.ft, a.fc, qb, qd, nc, T, Pr,
                                                           pix, w, n, pf))) {
                    push = true;
                    n = 0;
                }
                done = true;
            }
            if (!done) {
                double coords[4];
                get_coords<C>(a.g.lut, load_quat(a.bore + 4LL * t), ofs, coords);
                spin_factors(nc, coords, T, Pr, pf);
                n = get_pixels<P>(a.g, coords, pix, w);
            }
            if (!WEIGHT && n > 0) sig = sig_in;
        }
        // (Mixed pointing fills the exact queue from the double-float pass.)
        if (kFastOK && fast && !mixed) qn = warp_enqueue(wq, qn, push, t);
        if (kMixedOK && mixed) qdf = warp_enqueue(wdf, qdf, push_df, t);
#pragma unroll
        for (int k = 0; k < NT; k++) {
            long long off = -1, plane = 0;
            float v[NV];
#pragma unroll
            for (int s = 0; s < NV; s++) v[s] = 0.f;
            if (k < n) {
                int bad = locate<P>(a.g, pix[k], &off, &plane);
                if (bad >= 0) {
                    record_missing_tile(a.err, bad);
                    off = -1;
                } else {
                    tap_values<WEIGHT, NV, NT == 1>(sig, pf, w[k], det_wt, v);
                }
            }
            if (NT > 1 && !__any_sync(kFull, off >= 0)) continue;
            if (a.accum == SO3G_ACCUM_WARP_RUNS) {
                flush_runs<NV>(off, plane, v, mult, vmask, a.map);
            } else if (off >= 0) {
#pragma unroll
                for (int s = 0; s < NV; s++)
                    if ((vmask >> s) & 1u) atomicAdd(a.map + off + mult[s] * plane, f2d(v[s]));
            }
        }
        // Mixed pointing: the samples the float32 tier left, 32 at a time
        // through the double-float path; what that cannot certify goes on
        // to the exact queue.
        if (kMixedOK && mixed && (qdf >= 32 || (r == rounds - 1 && qdf > 0))) {
            __syncwarp();
            for (int base = 0; base < qdf; base += 32) {
                const int i = base + (threadIdx.x & 31);
                const int ts = i < qdf ? wdf[i] : 0;
                const bool px =
                    i < qdf && !df_sample<C, P, WEIGHT, PointingVariant<C, P, MODE>::cert>(
                                   a, det, ts, wp->qd, T, Pr, det_wt, mult, vmask);
                qn = warp_enqueue(wq, qn, px, ts);
                if (qn > kWarpQueue - 32) drain_exact();
            }
            __syncwarp();
            qdf = 0;
        }
        if (kFastOK && fast && (qn > kWarpQueue - 32 || r == rounds - 1)) drain_exact();
    }
}

template <int C, int P, bool WEIGHT, int MODE>
__global__ void __launch_bounds__(kBlock, PointingVariant<C, P, MODE>::mixed && MODE == 2
                                              ? kMixedBlocksPerSM
                                              : kScatterBlocksPerSM)
    k_scatter(ScatterArgs a) {
    __shared__ int s_queue[QueueInts<C, P, MODE>::value];
    __shared__ WarpPiece s_wp[kBlock / 32];
    int det, t0, t1;
    if (!seg_piece(a.segs, a.piece, det, t0, t1)) return;
    scatter_piece<C, P, WEIGHT, MODE>(a, det, t0, t1, s_queue, s_wp);
}



}  // namespace

}  // namespace so3g
