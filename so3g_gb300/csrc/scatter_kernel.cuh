// scatter_kernel.cuh -- the to_map / to_weight_map kernel, shared by the
// entry points of scatter.cu and noalloc.cu.
//
// Work layout: block (x, y) takes piece y of sample segment x (one detector
// and a contiguous range of its samples); each warp handles 32 consecutive
// samples at a time, lane = sample.  Consecutive samples of a scanning
// detector tend to fall in the same pixel, which the WARP_RUNS accumulator
// exploits: runs of equal pixels across the warp are summed in registers
// (compensated float32) and flushed with one float64 atomic per run and
// component.  The ATOMIC accumulator adds every term on its own.
#pragma once

#include "host.h"

namespace so3g {

// Internal linkage: every translation unit that includes this header gets
// its own instantiations.
namespace {

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
};

template <int C, int P, bool WEIGHT>
__global__ void __launch_bounds__(kBlock) k_scatter(ScatterArgs a) {
    int det, t0, t1;
    if (!seg_piece(a.segs, a.piece, det, t0, t1)) return;
    float det_wt = 1.f;
    if (a.det_weights) {
        det_wt = __ldg(a.det_weights + det);
        if (det_wt == 0.f) return;  // src/Projection.cxx:1784-1788
    }
    const QuatD ofs = load_quat(a.dets + 4LL * det);
    const float T = __ldg(a.resp + 2 * det), Pr = __ldg(a.resp + 2 * det + 1);
    const int nc = a.g.ncomp;
    const int lane = threadIdx.x & 31;
    constexpr int NT = PixTraits<P>::taps;
    constexpr int NV = WEIGHT ? 6 : 3;
    // Value slots: to_map slot c = component c; to_weight_map slots are the
    // upper-triangle pairs (i, j), j >= i, in row order.
    int mult[NV];
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

    for (int base = t0 + (threadIdx.x & ~31); base < t1; base += blockDim.x) {
        const int t = base + lane;
        const bool live = t < t1;
        double coords[4];
        float pf[3] = {0.f, 0.f, 0.f};
        int pix[NT][3];
        float w[NT];
        int n = 0;
        float sig = 0.f;
        if (live) {
            const QuatD qb = load_quat(a.bore + 4LL * t);
            get_coords<C>(a.g.lut, qb, ofs, coords);
            spin_factors(nc, coords, T, Pr, pf);
            if (!WEIGHT) sig = __ldg(a.signal + det * a.sig_stride + t);
            n = get_pixels<P>(a.g, coords, pix, w);
        }
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
                } else if (!WEIGHT) {
                    // src/Projection.cxx:1807 -- float32 product, left to right
#pragma unroll
                    for (int c = 0; c < 3; c++) v[c] = sig * pf[c] * w[k] * det_wt;
                } else {
                    // src/Projection.cxx:1850
                    int s = 0;
#pragma unroll
                    for (int i = 0; i < 3; i++)
#pragma unroll
                        for (int j = i; j < 3; j++, s++) v[s] = pf[i] * pf[j] * w[k] * w[k] * det_wt;
                }
            }
            if (NT > 1 && !__any_sync(kFull, off >= 0)) continue;
            if (a.accum == SO3G_ACCUM_WARP_RUNS) {
                flush_runs<NV>(off, plane, v, mult, vmask, a.map);
            } else if (off >= 0) {
#pragma unroll
                for (int s = 0; s < NV; s++)
                    if ((vmask >> s) & 1u) atomicAdd(a.map + off + mult[s] * plane, (double)v[s]);
            }
        }
    }
}

}  // namespace

}  // namespace so3g
