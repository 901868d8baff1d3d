// precomp.cu -- ProjEng_Precomp: projection with precomputed pointing
// (pixel indices and spin projection factors per sample).  No trigonometry:
// these kernels stream the pointing, the signal and the map and are bound by
// HBM bandwidth and atomic throughput.  Untiled maps over whole rows take
// the vectorised kernels (k_pc_scatter4, k_pc_from_map4); everything else
// the per-sample ones.

#include <algorithm>

#include "host.h"

namespace so3g {

namespace {

struct PcArgs {
    int tiled, nc, ny, nx;
    const int *tile_dims;
    const long long *tile_offset;
    int n_tile;
    const int *pixel;
    const float *spin;
    int n_time;
    const float *signal;
    float *signal_out;
    long long sig_stride;
    const float *det_weights;
    Segs segs;
    int piece;
    int accum;
    int *err;
    double *map;
};

// Element offset and plane size of a precomputed pixel tuple; false if it
// is skipped (the error record says why).
template <bool TILED>
__device__ __forceinline__ bool pc_locate(const PcArgs &a, const int *p, int det, int t,
                                          long long *off, long long *plane) {
    if (!TILED) {
        // Pixelizor2_Flat<NonTiled>::pix, src/Projection.cxx:881-886
        if (p[0] >= a.ny || p[1] < 0 || p[1] >= a.nx) {
            record_pixel_range(a.err, 0, det, t);
            return false;
        }
        *off = (long long)p[0] * a.nx + p[1];
        *plane = (long long)a.ny * a.nx;
        return true;
    }
    // Pixelizor2_Flat<Tiled>::pix, src/Projection.cxx:1084-1093
    const int tile = p[0];
    long long toff = tile < a.n_tile ? __ldg(a.tile_offset + tile) : -1;
    if (toff < 0) {
        record_missing_tile(a.err, tile);
        return false;
    }
    const int tny = __ldg(a.tile_dims + 2 * tile), tnx = __ldg(a.tile_dims + 2 * tile + 1);
    if (p[1] < 0 || p[1] >= tny || p[2] < 0 || p[2] >= tnx) {
        record_pixel_range(a.err, tile, det, t);
        return false;
    }
    *off = toff + (long long)p[1] * tnx + p[2];
    *plane = (long long)tny * tnx;
    return true;
}

template <bool TILED>
__device__ __forceinline__ void load_tuple(const PcArgs &a, long long s, int *p) {
    if (!TILED) {
        int2 v = __ldg(reinterpret_cast<const int2 *>(a.pixel) + s);
        p[0] = v.x;
        p[1] = v.y;
    } else {
        const int *q = a.pixel + 3 * s;
        p[0] = __ldg(q);
        p[1] = __ldg(q + 1);
        p[2] = __ldg(q + 2);
    }
}

template <bool TILED, bool WEIGHT>
__global__ void __launch_bounds__(kBlock) k_pc_scatter(PcArgs a) {
    int det, t0, t1;
    if (!seg_piece(a.segs, a.piece, det, t0, t1)) return;
    float det_wt = 1.f;
    if (a.det_weights) {
        det_wt = __ldg(a.det_weights + det);
        if (det_wt == 0.f) return;  // src/Projection.cxx:2101-2105
    }
    const int nc = a.nc;
    const int lane = threadIdx.x & 31;
    constexpr int NV = WEIGHT ? 6 : 3;
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
    // The next round's pointing and signal are loaded before this round's
    // atomics are issued, so that two rounds of loads are in flight.
    int p[3] = {-1, 0, 0}, pn[3] = {-1, 0, 0};
    float pf[3] = {0.f, 0.f, 0.f}, pfn[3] = {0.f, 0.f, 0.f};
    float sg = 0.f, sgn = 0.f;
    auto fetch = [&](int t, int *pp, float *ff, float &ss) {
        if (t < t1) {
            const long long s = (long long)det * a.n_time + t;
            load_tuple<TILED>(a, s, pp);
#pragma unroll
            for (int c = 0; c < 3; c++)
                if (c < nc) ff[c] = __ldg(a.spin + s * nc + c);
            if (!WEIGHT) ss = __ldg(a.signal + det * a.sig_stride + t);
        } else {
            pp[0] = -1;
        }
    };
    fetch(t0 + (threadIdx.x & ~31) + lane, pn, pfn, sgn);
    for (int base = t0 + (threadIdx.x & ~31); base < t1; base += blockDim.x) {
        const int t = base + lane;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            p[c] = pn[c];
            pf[c] = pfn[c];
        }
        sg = sgn;
        fetch(t + blockDim.x, pn, pfn, sgn);
        long long off = -1, plane = 0;
        float v[NV];
#pragma unroll
        for (int k = 0; k < NV; k++) v[k] = 0.f;
        if (t < t1) {
            if (p[0] >= 0 && pc_locate<TILED>(a, p, det, t, &off, &plane)) {
                if (!WEIGHT) {
                    // src/Projection.cxx:2117
                    const float sig = sg;
#pragma unroll
                    for (int c = 0; c < 3; c++) v[c] = det_wt * sig * pf[c];
                } else {
                    // src/Projection.cxx:2151
                    int k = 0;
#pragma unroll
                    for (int i = 0; i < 3; i++)
#pragma unroll
                        for (int j = i; j < 3; j++, k++) v[k] = pf[i] * pf[j] * det_wt;
                }
            }
        }
        if (a.accum == SO3G_ACCUM_WARP_RUNS) {
            flush_runs<NV>(off, plane, v, mult, vmask, a.map);
        } else if (off >= 0) {
#pragma unroll
            for (int k = 0; k < NV; k++)
                if ((vmask >> k) & 1u) atomicAdd(a.map + off + mult[k] * plane, f2d(v[k]));
        }
    }
}

template <bool TILED>
__global__ void __launch_bounds__(kBlock) k_pc_from_map(PcArgs a) {
    // ProjEng_Precomp::from_map, src/Projection.cxx:2066-2082
    int det, t0, t1;
    if (!seg_piece(a.segs, a.piece, det, t0, t1)) return;
    const int nc = a.nc;
    // Four samples per thread and iteration, their pointing loads issued
    // together (more bytes in flight per thread).
    constexpr int U = 4;
    for (int tb = t0 + threadIdx.x; tb < t1; tb += U * blockDim.x) {
        int pu[U][3];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int t = tb + u * blockDim.x;
            pu[u][0] = -1;
            if (t < t1) load_tuple<TILED>(a, (long long)det * a.n_time + t, pu[u]);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int t = tb + u * blockDim.x;
            if (t >= t1) break;
            const long long s = (long long)det * a.n_time + t;
            const int *p = pu[u];
            if (p[0] < 0) continue;
            long long off, plane;
            if (!pc_locate<TILED>(a, p, det, t, &off, &plane)) continue;
            // sig += pf * map, a float64 product and sum rounded to float32 per
            // component: certified double-float roundings (fast_accum), the
            // float64 arithmetic itself for a sample where one is uncertain.
            float pf[3], sig = 0.f;
            double mv[3];
            bool ok = true;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                if (c < nc) {
                    pf[c] = __ldg(a.spin + s * nc + c);
                    mv[c] = __ldg(a.map + off + c * plane);
                    ok = ok && fast_accum(sig, mv[c], pf[c]);
                }
            }
            if (!ok) {
                sig = 0.f;
#pragma unroll
                for (int c = 0; c < 3; c++)
                    if (c < nc) sig += pf[c] * mv[c];
            }
            a.signal_out[det * a.sig_stride + t] += sig;
        }
    }
}

// ---------------------------------------------------------------------------
// Vectorised kernels for the common case: an untiled map, whole detector
// rows (no sample ranges), n_time a multiple of 4 and 16-byte aligned
// arrays.  Each thread takes 4 consecutive samples of its detector per
// iteration and moves them with 16-byte loads: the pixel pairs as two
// int4, the spin factors as NC float4, the signal as one float4 -- six
// load instructions per 4 samples instead of five per sample, so that the
// memory system, not the load issue rate, sets the pace.

// The 4 samples' pixel pairs (iy, ix) and spin factors from sample index s
// (a multiple of 4).
template <int NC>
__device__ __forceinline__ void pc_load4(const PcArgs &a, long long s, int (&p)[8],
                                         float (&f)[4 * NC]) {
    const int4 *pp = reinterpret_cast<const int4 *>(a.pixel) + (s >> 1);
    const int4 u = __ldg(pp), v = __ldg(pp + 1);
    p[0] = u.x; p[1] = u.y; p[2] = u.z; p[3] = u.w;
    p[4] = v.x; p[5] = v.y; p[6] = v.z; p[7] = v.w;
    const float4 *fp = reinterpret_cast<const float4 *>(a.spin + s * NC);
#pragma unroll
    for (int k = 0; k < NC; k++) {
        const float4 w = __ldg(fp + k);
        f[4 * k] = w.x; f[4 * k + 1] = w.y; f[4 * k + 2] = w.z; f[4 * k + 3] = w.w;
    }
}

// Pixelizor2_Flat<NonTiled>::pix (src/Projection.cxx:881-886) for a
// precomputed pair: the element offset, or -1 (iy < 0: skipped; out of
// range: recorded).
__device__ __forceinline__ long long pc_offset(const PcArgs &a, int iy, int ix, int det,
                                               int t) {
    if (iy < 0) return -1;
    if (iy >= a.ny || ix < 0 || ix >= a.nx) {
        record_pixel_range(a.err, 0, det, t);
        return -1;
    }
    return (long long)iy * a.nx + ix;
}

// Upper-triangle pair (i, j), j >= i, of value k of an NC-component
// weight map (NC <= 3), in the order i = 0..NC-1, j = i..NC-1.
template <int NC>
__device__ constexpr int pair_i(int k) {
    return NC == 3 ? (k < 3 ? 0 : (k < 5 ? 1 : 2)) : (NC == 2 ? (k < 2 ? 0 : 1) : 0);
}
template <int NC>
__device__ constexpr int pair_j(int k) {
    return NC == 3 ? (k < 3 ? k : (k < 5 ? k - 2 : 2)) : (NC == 2 ? (k < 2 ? k : 1) : 0);
}

// One run total (hi + lo, at most 3 values from value K0 on) added to the
// map: plane c (to_map) or i * NC + j (to_weight_map); key < 0: nothing.
// hi + lo is added in float64, the exact run sum to ~2^-46, so the map
// differs from the per-sample sums only in float64 summation order.
template <bool WEIGHT, int NC, int K0, int G>
__device__ __forceinline__ void pc_flush_slot(double *map, int key, long long plane,
                                              const float (&hi)[3], const float (&lo)[3]) {
    if (key < 0) return;
    double *p = map + key;
#pragma unroll
    for (int c = 0; c < G; c++) {
        const int k = K0 + c;
        const int pl = WEIGHT ? pair_i<NC>(k) * NC + pair_j<NC>(k) : k;
        double d = f2d(hi[c]);
        if (lo[c] != 0.f) d += f2d(lo[c]);
        atomicAdd(p + pl * plane, d);
    }
}

// Values K0..K0+G-1 of a lane's four samples: the runs of equal pixels
// among them summed right to left with compensated (TwoSum) additions,
// packed into run slots 0..3 and flushed slot by slot, one pass per slot
// taken only when some lane of the warp has that many runs.  A run is ~5
// samples on a 1' scan, so a round of 128 samples takes ~2 passes of
// atomics, where flushing each run as it ends took up to four divergent
// ones that touched the same sectors again (1000 det x 1M, 3x2000x2000:
// to_map 5.64 -> 4.70 ms).
template <bool WEIGHT, int NC, int K0, int G>
__device__ __forceinline__ void pc_runs4(double *map, long long plane, const int (&key)[4],
                                         const float (&sig)[4], const float (&f)[4 * NC],
                                         float det_wt) {
    float v[4][3], lo[4][3];
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const int k = K0 + c;
            const float *pf = f + NC * j;
            if (c >= G) v[j][c] = 0.f;
            else if (WEIGHT) v[j][c] = pf[pair_i<NC>(k)] * pf[pair_j<NC>(k)] * det_wt;  // src/Projection.cxx:2151
            else v[j][c] = det_wt * sig[j] * pf[k];  // src/Projection.cxx:2117
            lo[j][c] = 0.f;
        }
    const bool h1 = key[1] != key[0], h2 = key[2] != key[1], h3 = key[3] != key[2];
#pragma unroll
    for (int c = 0; c < G; c++) {
        float e;
        if (!h3) { two_sum(v[2][c], v[3][c], v[2][c], e); lo[2][c] = e; }
        if (!h2) { two_sum(v[1][c], v[2][c], v[1][c], e); lo[1][c] = lo[2][c] + e; }
        if (!h1) { two_sum(v[0][c], v[1][c], v[0][c], e); lo[0][c] = lo[1][c] + e; }
    }
    // Slots 1 and 2: the first and second heads among samples 1..3; slot
    // 3: sample 3 when all three are heads.
    const int nruns = 1 + h1 + h2 + h3;
    float s1[3], l1[3], s2[3], l2[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        s1[c] = h1 ? v[1][c] : (h2 ? v[2][c] : v[3][c]);
        l1[c] = h1 ? lo[1][c] : (h2 ? lo[2][c] : lo[3][c]);
        s2[c] = (h1 && h2) ? v[2][c] : v[3][c];
        l2[c] = (h1 && h2) ? lo[2][c] : lo[3][c];
    }
    const int k1 = h1 ? key[1] : (h2 ? key[2] : key[3]);
    const int k2 = (h1 && h2) ? key[2] : key[3];
    pc_flush_slot<WEIGHT, NC, K0, G>(map, key[0], plane, v[0], lo[0]);
    if (__any_sync(kFull, nruns > 1) && nruns > 1)
        pc_flush_slot<WEIGHT, NC, K0, G>(map, k1, plane, s1, l1);
    if (__any_sync(kFull, nruns > 2) && nruns > 2)
        pc_flush_slot<WEIGHT, NC, K0, G>(map, k2, plane, s2, l2);
    if (__any_sync(kFull, nruns > 3) && nruns > 3)
        pc_flush_slot<WEIGHT, NC, K0, G>(map, key[3], plane, v[3], lo[3]);
}

// ProjEng_Precomp::to_map / to_weight_map (src/Projection.cxx:2084-2158)
// with 4 consecutive samples per lane (a warp takes 128): the pixel pairs
// as two int4, the spin factors as NC float4 and the signal as one float4.
// The map's element offsets within a plane are 32-bit (the launcher takes
// this kernel for planes below 2^31 pixels).  The values of a weight map are
// summed in groups of three, which keeps them in registers.
template <bool WEIGHT, int NC>
__global__ void __launch_bounds__(kBlock) k_pc_scatter4(PcArgs a) {
    constexpr int NV = WEIGHT ? NC * (NC + 1) / 2 : NC;
    int det, t0, t1;
    if (!seg_piece(a.segs, a.piece, det, t0, t1)) return;
    float det_wt = 1.f;
    if (a.det_weights) {
        det_wt = __ldg(a.det_weights + det);
        if (det_wt == 0.f) return;  // src/Projection.cxx:2101-2105
    }
    const long long plane = (long long)a.ny * a.nx;
    const int lane = threadIdx.x & 31;
    // t1 - t0 is a multiple of 4: a lane's samples are all in or all out.
    for (int tb = t0 + 128 * (threadIdx.x >> 5); tb < t1; tb += 4 * blockDim.x) {
        const int tq = tb + 4 * lane;
        int key[4] = {-1, -1, -1, -1};
        float sig[4] = {0.f, 0.f, 0.f, 0.f};
        float f[4 * NC];
#pragma unroll
        for (int k = 0; k < 4 * NC; k++) f[k] = 0.f;
        if (tq < t1) {
            const long long s = (long long)det * a.n_time + tq;
            int p[8];
            pc_load4<NC>(a, s, p, f);
            if (!WEIGHT) {
                const float4 sg =
                    __ldg(reinterpret_cast<const float4 *>(a.signal + det * a.sig_stride + tq));
                sig[0] = sg.x; sig[1] = sg.y; sig[2] = sg.z; sig[3] = sg.w;
            }
#pragma unroll
            for (int j = 0; j < 4; j++)
                key[j] = (int)pc_offset(a, p[2 * j], p[2 * j + 1], det, tq + j);
        }
        pc_runs4<WEIGHT, NC, 0, (NV < 3 ? NV : 3)>(a.map, plane, key, sig, f, det_wt);
        if constexpr (NV > 3) pc_runs4<WEIGHT, NC, 3, NV - 3>(a.map, plane, key, sig, f, det_wt);
    }
}

// float4 words per pixel of the split map of an NC-component map.
template <int NC>
struct PcSplit {
    static constexpr int W = (NC + 1) / 2;
};

// The map split for k_pc_from_map4: per pixel, component c's float64
// value m as df_split's double-float (h, l) at words 2c, 2c + 1 (h = +-0 for
// m = +-0; NaN where m is not finite or outside df_split's range, which
// sends the sample to the float64 arithmetic), pixel-major: one sample
// reads its pixel's NC components from one or two float4 instead of NC
// float64 planes, and needs no split of its own.
template <int NC>
__global__ void k_pc_map_split(const double *map, long long plane, float4 *split) {
    constexpr int W = PcSplit<NC>::W;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < plane;
         p += (long long)gridDim.x * blockDim.x) {
        float hl[4 * W];
#pragma unroll
        for (int k = 0; k < 4 * W; k++) hl[k] = 0.f;
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const double m = __ldg(map + c * plane + p);
            const unsigned mh = (unsigned)__double2hiint(m);
            float h = __int_as_float(0x7fc00000), l = 0.f;
            if (((mh & 0x7fffffffu) | (unsigned)__double2loint(m)) == 0u) {
                h = __uint_as_float(mh & 0x80000000u);
            } else {
                dfl d;
                if (df_split(m, d)) {
                    h = d.hi;
                    l = d.lo;
                }
            }
            hl[2 * c] = h;
            hl[2 * c + 1] = l;
        }
#pragma unroll
        for (int w = 0; w < W; w++)
            split[p * W + w] = make_float4(hl[4 * w], hl[4 * w + 1], hl[4 * w + 2], hl[4 * w + 3]);
    }
}

// With SPLIT (the form the launcher takes) the map values come from
// k_pc_map_split's copy, the float64 map only for a sample whose rounding is
// not certain: 4.60 ms against 6.15 ms for the kernel that splits each
// value itself (1000 det x 1M samples, 3x2000x2000 map), compiled for 6
// resident blocks (40 registers; 8 blocks spill: 5.23 ms, 5 blocks: 4.70
// ms).  Without SPLIT (no memory for the copy): 8 blocks, 32 registers.
template <int NC, bool SPLIT>
__global__ void __launch_bounds__(kBlock, SPLIT ? 6 : 8)
    k_pc_from_map4(PcArgs a, const float4 *split) {
    // ProjEng_Precomp::from_map, src/Projection.cxx:2066-2082
    int det, t0, t1;
    if (!seg_piece(a.segs, a.piece, det, t0, t1)) return;
    const long long plane = (long long)a.ny * a.nx;
    for (int t = t0 + 4 * threadIdx.x; t < t1; t += 4 * blockDim.x) {
        const long long s = (long long)det * a.n_time + t;
        int p[8];
        float f[4 * NC];
        pc_load4<NC>(a, s, p, f);
        float4 *sp = reinterpret_cast<float4 *>(a.signal_out + det * a.sig_stride + t);
        const float4 sv = *sp;
        float sig[4] = {sv.x, sv.y, sv.z, sv.w};
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const long long off = pc_offset(a, p[2 * j], p[2 * j + 1], det, t + j);
            if (off < 0) continue;
            const float *pf = f + NC * j;
            // The reference sums the components into a float32 sig = 0 (each
            // `sig += pf * map` a float64 product and sum rounded to
            // float32: certified double-float roundings, fast_accum; the
            // float64 arithmetic itself where one is uncertain), then adds
            // sig to the signal.
            float s1 = 0.f;
            bool ok = true;
            if (SPLIT) {
                constexpr int W = PcSplit<NC>::W;
                float hl[4 * W];
#pragma unroll
                for (int w = 0; w < W; w++) {
                    const float4 q = __ldg(split + off * W + w);
                    hl[4 * w] = q.x;
                    hl[4 * w + 1] = q.y;
                    hl[4 * w + 2] = q.z;
                    hl[4 * w + 3] = q.w;
                }
#pragma unroll
                for (int c = 0; c < NC; c++)
                    ok = ok && fast_accum_split(s1, hl[2 * c], hl[2 * c + 1], pf[c]);
                if (!ok) {
                    s1 = 0.f;
#pragma unroll
                    for (int c = 0; c < NC; c++) s1 += pf[c] * __ldg(a.map + off + c * plane);
                }
            } else {
                double mv[NC];
#pragma unroll
                for (int c = 0; c < NC; c++) {
                    mv[c] = __ldg(a.map + off + c * plane);
                    ok = ok && fast_accum(s1, mv[c], pf[c]);
                }
                if (!ok) {
                    s1 = 0.f;
#pragma unroll
                    for (int c = 0; c < NC; c++) s1 += pf[c] * mv[c];
                }
            }
            sig[j] += s1;
        }
        *sp = make_float4(sig[0], sig[1], sig[2], sig[3]);
    }
}

// True when the vectorised kernels apply (see above).
bool pc_vec_ok(const PcArgs &a, const void *sig, long long sig_stride, bool whole_rows) {
    auto al = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
    return !a.tiled && whole_rows && (a.n_time % 4) == 0 && al(a.pixel) && al(a.spin) &&
           (long long)a.ny * a.nx <= 0x7fffffffLL &&
           (!sig || (al(sig) && (sig_stride % 4) == 0));
}

template <bool WEIGHT>
void pc_scatter4_launch(const PcArgs &a, dim3 grid, cudaStream_t st) {
    switch (a.nc) {
    case 1: k_pc_scatter4<WEIGHT, 1><<<grid, kBlock, 0, st>>>(a); break;
    case 2: k_pc_scatter4<WEIGHT, 2><<<grid, kBlock, 0, st>>>(a); break;
    default: k_pc_scatter4<WEIGHT, 3><<<grid, kBlock, 0, st>>>(a); break;
    }
}

template <int NC>
void pc_from_map4_nc(const PcArgs &a, dim3 grid, cudaStream_t st) {
    // The split map (W float4 per pixel) in stream-ordered memory; without
    // it, the kernel splits each map value itself.
    const long long plane = (long long)a.ny * a.nx;
    float4 *split = nullptr;
    if (cudaMallocAsync(reinterpret_cast<void **>(&split),
                        sizeof(float4) * PcSplit<NC>::W * (size_t)plane, st) != cudaSuccess) {
        cudaGetLastError();
        split = nullptr;
    }
    if (split) {
        const long long blocks = std::min<long long>((plane + kBlock - 1) / kBlock, 152LL * 16);
        k_pc_map_split<NC><<<(unsigned)blocks, kBlock, 0, st>>>(a.map, plane, split);
        k_pc_from_map4<NC, true><<<grid, kBlock, 0, st>>>(a, split);
        cudaFreeAsync(split, st);
    } else {
        k_pc_from_map4<NC, false><<<grid, kBlock, 0, st>>>(a, nullptr);
    }
}

void pc_from_map4_launch(const PcArgs &a, dim3 grid, cudaStream_t st) {
    switch (a.nc) {
    case 1: pc_from_map4_nc<1>(a, grid, st); break;
    case 2: pc_from_map4_nc<2>(a, grid, st); break;
    default: pc_from_map4_nc<3>(a, grid, st); break;
    }
}

int pc_common(PcArgs &a, const so3g_precomp_geom *g, const int32_t *pixel,
              const float *spin_proj, int32_t n_det, int32_t n_time, const so3g_map *map) {
    clear_error();
    if (!g) return set_error(SO3G_ERR_ARGUMENT, "geometry is NULL");
    if (g->n_comp < 1 || g->n_comp > 3)
        return set_error(SO3G_ERR_ARGUMENT, "n_comp must be 1, 2 or 3 (got %d)", g->n_comp);
    if (n_det < 0 || n_time < 0) return set_error(SO3G_ERR_ARGUMENT, "negative n_det or n_time");
    if (!map || !map->data) return set_error(SO3G_ERR_ARGUMENT, "map is NULL");
    a.tiled = g->tiled ? 1 : 0;
    a.nc = g->n_comp;
    a.ny = g->naxis[0];
    a.nx = g->naxis[1];
    if (a.tiled) {
        if (!map->tile_offset || !g->tile_dims)
            return set_error(SO3G_ERR_ARGUMENT, "tiled map needs tile_offset and tile_dims");
        a.tile_offset = reinterpret_cast<const long long *>(map->tile_offset);
        a.tile_dims = g->tile_dims;
        a.n_tile = map->n_tile;
    }
    a.pixel = pixel;
    a.spin = spin_proj;
    a.n_time = n_time;
    if (n_det > 0 && n_time > 0 && (!pixel || !spin_proj))
        return set_error(SO3G_ERR_ARGUMENT, "NULL pixel or spin_proj");
    return SO3G_OK;
}

}  // namespace

}  // namespace so3g

using namespace so3g;

extern "C" {

int so3g_precomp_to_map(const so3g_precomp_geom *g, const int32_t *pixel,
                        const float *spin_proj, int32_t n_det, int32_t n_time,
                        const float *signal, int64_t sig_det_stride, const float *det_weights,
                        const so3g_ranges *ranges, const so3g_map *map, int32_t accum,
                        int32_t *err, void *stream) {
    PcArgs a{};
    int rc = pc_common(a, g, pixel, spin_proj, n_det, n_time, map);
    if (rc) return rc;
    if (accum != SO3G_ACCUM_ATOMIC && accum != SO3G_ACCUM_WARP_RUNS)
        return set_error(SO3G_ERR_ARGUMENT, "unknown accumulation mode %d", accum);
    long long n_seg = ranges ? ranges->n_seg : n_det;
    long long max_len = ranges ? ranges->max_len : n_time;
    if (n_seg <= 0 || max_len <= 0 || n_time == 0) return SO3G_OK;
    if (!signal) return set_error(SO3G_ERR_ARGUMENT, "NULL signal");
    a.signal = signal;
    a.sig_stride = sig_det_stride;
    a.det_weights = det_weights;
    a.segs = Segs{ranges ? ranges->seg : nullptr, n_time};
    a.piece = piece_len(max_len);
    a.accum = accum;
    a.err = err;
    a.map = map->data;
    dim3 grid((unsigned)n_seg, (unsigned)((max_len + a.piece - 1) / a.piece));
    if (pc_vec_ok(a, signal, sig_det_stride, !ranges))
        pc_scatter4_launch<false>(a, grid, (cudaStream_t)stream);
    else if (a.tiled) k_pc_scatter<true, false><<<grid, kBlock, 0, (cudaStream_t)stream>>>(a);
    else k_pc_scatter<false, false><<<grid, kBlock, 0, (cudaStream_t)stream>>>(a);
    return after_launch("precomp to_map");
}

int so3g_precomp_to_weight_map(const so3g_precomp_geom *g, const int32_t *pixel,
                               const float *spin_proj, int32_t n_det, int32_t n_time,
                               const float *det_weights, const so3g_ranges *ranges,
                               const so3g_map *map, int32_t accum, int32_t *err, void *stream) {
    PcArgs a{};
    int rc = pc_common(a, g, pixel, spin_proj, n_det, n_time, map);
    if (rc) return rc;
    if (accum != SO3G_ACCUM_ATOMIC && accum != SO3G_ACCUM_WARP_RUNS)
        return set_error(SO3G_ERR_ARGUMENT, "unknown accumulation mode %d", accum);
    long long n_seg = ranges ? ranges->n_seg : n_det;
    long long max_len = ranges ? ranges->max_len : n_time;
    if (n_seg <= 0 || max_len <= 0 || n_time == 0) return SO3G_OK;
    a.det_weights = det_weights;
    a.segs = Segs{ranges ? ranges->seg : nullptr, n_time};
    a.piece = piece_len(max_len);
    a.accum = accum;
    a.err = err;
    a.map = map->data;
    dim3 grid((unsigned)n_seg, (unsigned)((max_len + a.piece - 1) / a.piece));
    if (pc_vec_ok(a, nullptr, 0, !ranges))
        pc_scatter4_launch<true>(a, grid, (cudaStream_t)stream);
    else if (a.tiled) k_pc_scatter<true, true><<<grid, kBlock, 0, (cudaStream_t)stream>>>(a);
    else k_pc_scatter<false, true><<<grid, kBlock, 0, (cudaStream_t)stream>>>(a);
    return after_launch("precomp to_weight_map");
}

int so3g_precomp_from_map(const so3g_precomp_geom *g, const int32_t *pixel,
                          const float *spin_proj, int32_t n_det, int32_t n_time,
                          const so3g_map *map, float *signal, int64_t sig_det_stride,
                          int32_t *err, void *stream) {
    PcArgs a{};
    int rc = pc_common(a, g, pixel, spin_proj, n_det, n_time, map);
    if (rc) return rc;
    if (n_det == 0 || n_time == 0) return SO3G_OK;
    if (!signal) return set_error(SO3G_ERR_ARGUMENT, "NULL signal");
    a.signal_out = signal;
    a.sig_stride = sig_det_stride;
    a.segs = Segs{nullptr, n_time};
    a.piece = piece_len(n_time);
    a.err = err;
    a.map = map->data;
    dim3 grid((unsigned)n_det, (unsigned)((n_time + a.piece - 1) / a.piece));
    if (pc_vec_ok(a, signal, sig_det_stride, true))
        pc_from_map4_launch(a, grid, (cudaStream_t)stream);
    else if (a.tiled) k_pc_from_map<true><<<grid, kBlock, 0, (cudaStream_t)stream>>>(a);
    else k_pc_from_map<false><<<grid, kBlock, 0, (cudaStream_t)stream>>>(a);
    return after_launch("precomp from_map");
}

}  // extern "C"
