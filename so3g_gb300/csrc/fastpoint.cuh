// fastpoint.cuh -- certified fast pointing for the flat pixelizors
// (nearest neighbour and bilinear, NonTiled and Tiled) of the CAR, TAN, ZEA
// and SIN projections.
//
// GB300 executes float64 at 1/64 of the float32 rate, and the exact float64
// pointing (quaternion compose, two table lookups, seven IEEE divisions, one
// square root) is the whole cost of an on-the-fly projection.  This path
// evaluates the same quantities in double-float arithmetic: a value is a
// pair (hi, lo) of float32, carried with error-free transformations (TwoSum,
// and TwoProduct through fmaf), about 44 good bits.  It then decides, for
// each sample, whether its results are certain:
//
//   - the pixel index: the reference computes x = lon/cdelt + crpix - 1
//     + 0.5 and takes its integer part.  If our x is more than kEpsPix from
//     every integer, the reference's x (which differs from ours by far less)
//     has the same integer part, and the same on/off-map decision.
//   - the spin factors float(P * (c*c - s*s)) and float(P * 2*c*s): if our
//     value is farther than the error bound from both float32 rounding
//     boundaries around its float32 rounding, the reference's float64 value
//     rounds to the same float32.
//   - the +-pi seam of atan2 and the regions near the native poles, where
//     the table and the spin factors are ill-conditioned, are not certified.
//
// A sample that is not certified is recomputed by the exact float64 path
// (device.cuh), so every result equals the exact path's bit for bit.  The
// error bounds kEpsPix and kEpsPf exceed the double-float error by orders of
// magnitude; the GPU tests compare both paths sample by sample.
//
// The sums below use the "sloppy" double-float addition, whose error is
// bounded relative to the operands (not the result).  Every certified
// quantity is compared with an absolute bound on that scale.
#pragma once

#include "device.cuh"

namespace so3g {

// Per-warp queue (in shared memory) of the samples the certified path
// leaves to the exact path.  Kept per warp, so that filling and draining it
// needs no block barrier; a warp drains it when another round could
// overflow it and at the end of its piece.
constexpr int kWarpQueue = 64;

// Appends t for the lanes with `push` to the warp's queue q holding qn
// entries; returns the new count.  All 32 lanes must call; qn is the same
// in every lane.
__device__ __forceinline__ int warp_enqueue(int *q, int qn, bool push, int t) {
    const unsigned m = __ballot_sync(0xffffffffu, push);
    if (push) q[qn + __popc(m & ((1u << (threadIdx.x & 31)) - 1u))] = t;
    return qn + __popc(m);
}

// Bounds of |double-float value - reference float64 value|.
constexpr float kEpsPix = 1e-7f;        // pixel coordinate units
constexpr float kEpsPf = 1e-11f;        // spin factors (values of order 1)

struct dfl {
    float hi, lo;
};

__device__ __forceinline__ dfl two_sum(float a, float b) {
    float s = a + b;
    float bb = s - a;
    return dfl{s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ dfl fast_two_sum(float a, float b) {
    float s = a + b;
    return dfl{s, b - (s - a)};
}

__device__ __forceinline__ dfl df_add(dfl x, dfl y) {
    dfl s = two_sum(x.hi, y.hi);
    s.lo += x.lo + y.lo;
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ dfl df_neg(dfl x) { return dfl{-x.hi, -x.lo}; }
__device__ __forceinline__ dfl df_sub(dfl x, dfl y) { return df_add(x, df_neg(y)); }

__device__ __forceinline__ dfl df_mul(dfl x, dfl y) {
    float p = x.hi * y.hi;
    float e = fmaf(x.hi, y.hi, -p);
    e = fmaf(x.hi, y.lo, e);
    e = fmaf(x.lo, y.hi, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ dfl df_mulf(dfl x, float y) {
    float p = x.hi * y;
    float e = fmaf(x.hi, y, -p);
    e = fmaf(x.lo, y, e);
    return fast_two_sum(p, e);
}

// 1/y: float reciprocal and one Newton step in double-float.
__device__ __forceinline__ dfl df_recip(dfl y) {
    const float r = __fdividef(1.0f, y.hi);
    // eps = 1 - y*r, small; 1/y = r (1 + eps + ...) to ~2^-46.
    float p = y.hi * r;
    float pe = fmaf(y.hi, r, -p);
    pe = fmaf(y.lo, r, pe);
    const float eps = (1.0f - p) - pe;
    return fast_two_sum(r, r * eps);
}

// Signed sum of products  sum_k sgn_k x_k y_k  of double-floats, accumulated
// with TwoProduct/TwoSum (a compensated dot product).
template <int N>
__device__ __forceinline__ dfl df_dot(const dfl (&x)[N], const dfl (&y)[N]) {
    float s = x[0].hi * y[0].hi;
    float e = fmaf(x[0].hi, y[0].hi, -s);
    e = fmaf(x[0].hi, y[0].lo, e);
    e = fmaf(x[0].lo, y[0].hi, e);
#pragma unroll
    for (int k = 1; k < N; k++) {
        const float p = x[k].hi * y[k].hi;
        e += fmaf(x[k].hi, y[k].hi, -p);
        e = fmaf(x[k].hi, y[k].lo, e);
        e = fmaf(x[k].lo, y[k].hi, e);
        const dfl u = two_sum(s, p);
        s = u.hi;
        e += u.lo;
    }
    return fast_two_sum(s, e);
}

// Double-float from a double through the conversion instructions.
__device__ __forceinline__ dfl df_from_double(double x) {
    float hi = __double2float_rn(x);
    float lo = __double2float_rn(x - (double)hi);
    return dfl{hi, lo};
}

// Double-float from a double with integer operations only (no float64
// instruction -- GB300 runs float<->double conversions on its slow float64
// pipe): hi is x truncated to 24 significant bits, lo the remaining 29 bits
// truncated to 23, |hi + lo - x| <= 2^-46 |x|.  Zeros are exact.  Returns
// false for magnitudes outside [2^-74, 2^100) and for inf/NaN: the caller
// then takes the exact path.
__device__ __forceinline__ bool df_split(double x, dfl &out) {
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const unsigned ex = (hw >> 20) & 0x7ffu;
    const unsigned sgn = hw & 0x80000000u;
    const float h = __uint_as_float(sgn | ((ex - 896u) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
    // r = low 29 bits of the mantissa, worth r * 2^(e-52); keep its top 23
    // bits exactly through the 2^23 magic number, then scale by 2^(e-46).
    const unsigned r = lw & 0x1fffffffu;
    const float m = __uint_as_float(0x4B000000u | (r >> 6)) - 8388608.0f;
    const float l = m * __uint_as_float((ex - 942u) << 23);
    const bool zero = ((hw & 0x7fffffffu) | lw) == 0u;
    out = zero ? dfl{0.f, 0.f} : fast_two_sum(h, sgn ? -l : l);
    return zero || (ex >= 949u && ex <= 1123u);
}


// Double-float of a float64: integer operations (df_split) where they
// apply, the conversion instructions otherwise.
__device__ __forceinline__ dfl df_of(double x) {
    dfl r;
    if (df_split(x, r)) return r;
    return df_from_double(x);
}

// The integer part of a double-float and the remaining fraction (exact).
__device__ __forceinline__ int df_floor(dfl x, dfl &frac) {
    float f = floorf(x.hi);
    float r = x.hi - f;              // exact: f and x.hi share the exponent range
    if (r == 0.f && x.lo < 0.f) {
        f -= 1.f;
        r = 1.f;
    }
    frac = fast_two_sum(r, x.lo);
    return (int)f;
}

// Half the gap from |v| to the float32 below it (the smaller of the two
// gaps around v): a value within this distance of v rounds to v.
__device__ __forceinline__ float half_gap(float v) {
    const float m = fabsf(v);
    return 0.5f * (m - __int_as_float(__float_as_int(m) - 1));
}

// Table of the asin/atan2 interpolation knots as double-floats, and the
// differences to the next knot: t[i] = (v_hi, v_lo, dv_hi, dv_lo).
struct FastTables {
    const float4 *asin_t;
    const float4 *atan2_t;
    const float4 *asin_sc;   // (sin hi, sin lo, cos hi, cos lo) of the asin knots
};

// Piecewise-linear interpolant of a table at u in [0, 1]: the value of
// LookupTable::get_raw (include/so_linterp.h:20-29) up to float64 rounding.
// The knot below u * (n-1) and the remaining fraction, with the knot
// index kept in [0, n-2]: at u = 1 (the last knot, which get_raw returns
// for d >= n-1) that is knot n-2 with fraction 1.
__device__ __forceinline__ int lut_index(dfl u, dfl &frac) {
    const int i = df_floor(df_mulf(u, (float)(kLutN - 1)), frac);
    const int ic = max(0, min(i, kLutN - 2));
    if (ic != i) frac = df_add(frac, dfl{(float)(i - ic), 0.f});
    return ic;
}

__device__ __forceinline__ dfl lut_df(const float4 *t, dfl u) {
    dfl frac;
    const int i = lut_index(u, frac);
    float4 k = __ldg(t + i);
    return df_add(dfl{k.x, k.y}, df_mul(dfl{k.z, k.w}, frac));
}

struct FastConst {
    dfl inv_cdx, inv_cdy;   // 1/cdelt
    dfl off_x, off_y;       // crpix - 1 + 0.5
    dfl pi, half_pi;
    dfl inv_2pi, third;     // the float64 constants 1/(2 pi) and 1/3
    dfl two_thirds;         // the float64 constant 2/3
};

// Native-frame quantities of one sample, in double-float, from the
// boresight and detector quaternions (Pointer<C>::GetCoords,
// src/Projection.cxx:372-437, 479-507, 337-364):
//   X, Y    the coordinates the flat pixelizor divides by cdelt (CAR: lon,
//           lat; zenithal: the projection-plane coordinates);
//   Nc, Ns, D  with coords[2] = Nc / sqrt(D) and coords[3] = Ns / sqrt(D).
// Returns false where the sample must take the exact path: the CAR
// native poles and atan2 seam, and the zenithal projections far from their
// pole (where the reference's expressions lose conditioning).
// q = qb * qd (Hamilton product).
__device__ __forceinline__ void df_qmul(const dfl (&qb)[4], const dfl (&qd)[4], dfl &a, dfl &b,
                                        dfl &c, dfl &d) {
    a = df_dot<4>({qb[0], qb[1], qb[2], qb[3]},
                  {qd[0], df_neg(qd[1]), df_neg(qd[2]), df_neg(qd[3])});
    b = df_dot<4>({qb[0], qb[1], qb[2], qb[3]}, {qd[1], qd[0], qd[3], df_neg(qd[2])});
    c = df_dot<4>({qb[0], qb[1], qb[2], qb[3]}, {qd[2], df_neg(qd[3]), qd[0], qd[1]});
    d = df_dot<4>({qb[0], qb[1], qb[2], qb[3]}, {qd[3], qd[2], df_neg(qd[1]), qd[0]});
}

// CAR longitude and the spin quantities (Pointer<ProjCAR>::GetCoords,
// :479-507): lon = ATAN2(c*d - a*b, c*a + d*b); c = Nc/h, s = Ns/h with
// h^2 = (1 - cos^2)/4 = D.  False at the +-pi seam (Y ~ 0 with X < 0),
// a discontinuity of atan2.
__device__ __forceinline__ bool fast_lon_spin(const FastTables &ft, const FastConst &fc,
                                              const dfl &a, const dfl &b, const dfl &c,
                                              const dfl &d, const dfl &cos_t, dfl &lon, dfl &Nc,
                                              dfl &Ns, dfl &D) {
    const dfl cd = df_mul(c, d), ab = df_mul(a, b);
    const dfl Yv = df_sub(cd, ab);
    const dfl Xv = df_dot<2>({c, d}, {a, b});
    if (Xv.hi < 0.f && !(fabsf(Yv.hi) > 1e-6f)) return false;
    const bool neg = Yv.hi < 0.f, mirror = Xv.hi < 0.f;
    const dfl ay = neg ? df_neg(Yv) : Yv, ax = mirror ? df_neg(Xv) : Xv;
    if (ax.hi < ay.hi) {
        lon = df_sub(fc.half_pi, lut_df(ft.atan2_t, df_mul(ax, df_recip(ay))));
    } else {
        lon = lut_df(ft.atan2_t, df_mul(ay, df_recip(ax)));
    }
    if (mirror) lon = df_sub(fc.pi, lon);
    if (neg) lon = df_neg(lon);
    // Spin (:1180-1209).
    Nc = df_dot<2>({a, b}, {c, df_neg(d)});
    Ns = df_add(cd, ab);
    D = df_mulf(df_sub(dfl{1.f, 0.f}, df_mul(cos_t, cos_t)), 0.25f);
    return true;
}

template <int C>
__device__ __forceinline__ bool fast_native(const FastTables &ft, const FastConst &fc,
                                            const dfl (&qb)[4], const dfl (&qd)[4], dfl &X,
                                            dfl &Y, dfl &Nc, dfl &Ns, dfl &D) {
    dfl a, b, c, d;
    df_qmul(qb, qd, a, b, c, d);
    if (C == SO3G_COORD_CAR) {
        // cos(theta) = a^2 - b^2 - c^2 + d^2 = sin(lat).
        const dfl cos_t = df_dot<4>({a, b, c, d}, {a, df_neg(b), df_neg(c), d});
        // Near the native poles (|lat| > ~87 deg) the tables' ends and the
        // spin factors are ill-conditioned: exact path.
        if (!(fabsf(cos_t.hi) < 0.998f)) return false;
        // lat = ASIN(cos_t) (odd, continuous at 0).
        const bool south = cos_t.hi < 0.f;
        dfl lat = lut_df(ft.asin_t, south ? df_neg(cos_t) : cos_t);
        if (south) lat = df_neg(lat);
        Y = lat;
        return fast_lon_spin(ft, fc, a, b, c, d, cos_t, X, Nc, Ns, D);
    } else {
        // Zenithal: cos^2(theta/2) = a^2 + d^2; coords[2] = (a^2 - d^2)/n,
        // coords[3] = 2ad/n.
        const dfl n = df_dot<2>({a, d}, {a, d});
        const dfl u = df_dot<2>({a, c}, {b, df_neg(d)});   // a*b - c*d
        const dfl v = df_dot<2>({a, b}, {c, d});           // a*c + b*d
        if (C == SO3G_COORD_TAN) {
            // :372-400: X = 2u / cos(theta), cos(theta) = 2n - 1.
            const dfl ct = df_sub(df_mulf(n, 2.f), dfl{1.f, 0.f});
            if (!(ct.hi > 1e-2f)) return false;
            const dfl r = df_mulf(df_recip(ct), 2.f);
            X = df_mul(u, r);
            Y = df_mul(v, r);
        } else if (C == SO3G_COORD_ZEA) {
            // :408-437: X = 2u / sqrt(n).
            if (!(n.hi > 1e-4f)) return false;
            const float s0 = sqrtf(n.hi);
            const float res = fmaf(-s0, s0, n.hi) + n.lo;   // n - s0^2
            const dfl sq = fast_two_sum(s0, res / (2.f * s0));
            const dfl r = df_mulf(df_recip(sq), 2.f);
            X = df_mul(u, r);
            Y = df_mul(v, r);
        } else if (C == SO3G_COORD_ARC) {
            // :284-326: h = sqrt(sc^2 + ss^2) (sc = a*c + b*d, ss = a*b -
            // c*d), R = ASIN(2 h) / h, or pi / h - R where a^2 + d^2 <
            // b^2 + c^2; X = ss R, Y = sc R.  The exact path takes the
            // reference's series branch (h < 1e-8) and the neighbourhoods
            // of its two decisions: h < 1e-6, |(a^2 + d^2) - (b^2 + c^2)| <=
            // 1e-6, and 2 h near 1 (the table's end, theta near 90 deg).
            if (!(n.hi > 1e-4f)) return false;
            const dfl h2 = df_dot<2>({u, v}, {u, v});
            if (!(h2.hi > 1e-12f)) return false;
            const dfl s2 = df_dot<2>({b, c}, {b, c});
            const dfl dcs = df_sub(n, s2);
            if (!(fabsf(dcs.hi) > 1e-6f)) return false;
            const float h0 = sqrtf(h2.hi);
            const dfl h = fast_two_sum(h0, (fmaf(-h0, h0, h2.hi) + h2.lo) / (2.f * h0));
            const dfl x2 = df_mulf(h, 2.f);
            if (!(x2.hi < 0.998f)) return false;
            const dfl ih = df_recip(h);
            dfl R = df_mul(lut_df(ft.asin_t, x2), ih);
            if (dcs.hi < 0.f) R = df_sub(df_mul(fc.pi, ih), R);
            X = df_mul(u, R);
            Y = df_mul(v, R);
        } else {
            // SIN, :337-364: X = 2u, Y = 2v.
            if (!(n.hi > 1e-4f)) return false;
            X = df_mulf(u, 2.f);
            Y = df_mulf(v, 2.f);
        }
        Nc = df_dot<2>({a, d}, {a, df_neg(d)});
        Ns = df_mulf(df_mul(a, d), 2.f);
        D = df_mul(n, n);
        return true;
    }
}

// Certified flat pixelization (Pixelizor2_Flat<NonTiled|Tiled, NN|Bilinear>
// ::GetPixels, :912-952, :1124-1166) of the pixel coordinates x = X/cdx +
// crx - 1 + 0.5 and y.  Returns false when an integer part is not certain.
// Nearest neighbour: one tap of weight 1 on the map.  Bilinear: the taps
// of the reference (same pixels, same order); each weight is the float32
// nearest to the double-float value of the reference's weight, which is
// the reference's float32 weight or one of its neighbours.
template <int P>
__device__ __forceinline__ bool fast_pixels(const DGeom &g, dfl x, dfl y, int (*pix)[3],
                                            float *w, int &n) {
    n = 0;
    if (P == PX_FLAT_NT_BL || P == PX_FLAT_T_BL) {
        // Far outside the map there is no tap (as in get_pixels).
        if (!(x.hi > -4.f && x.hi < (float)g.nx + 4.f && y.hi > -4.f &&
              y.hi < (float)g.ny + 4.f))
            return x.hi == x.hi && y.hi == y.hi;
    } else {
        if (!(x.hi > -2.f && x.hi < (float)g.nx + 1.f && y.hi > -2.f &&
              y.hi < (float)g.ny + 1.f))
            return x.hi == x.hi && y.hi == y.hi;
    }
    dfl fx, fy;
    const int ix = df_floor(x, fx), iy = df_floor(y, fy);
    if (!(fx.hi > kEpsPix && fx.hi < 1.f - kEpsPix && fy.hi > kEpsPix &&
          fy.hi < 1.f - kEpsPix))
        return false;
    if (P == PX_FLAT_NT_NN) {
        // :912-926 (x not near an integer: floor decides the bounds)
        if (ix >= 0 && ix < g.nx && iy >= 0 && iy < g.ny) {
            pix[0][0] = iy;
            pix[0][1] = ix;
            w[0] = 1.f;
            n = 1;
        }
    } else if (P == PX_FLAT_T_NN) {
        // :1124-1138 (int() truncation: x in (-1, 0) lands in column 0)
        const int tx = (x.hi < 0.f) ? ix + 1 : ix, ty = (y.hi < 0.f) ? iy + 1 : iy;
        if (tx >= 0 && tx < g.nx && ty >= 0 && ty < g.ny) {
            flat_tile_tuple(g, ty, tx, pix[0]);
            w[0] = 1.f;
            n = 1;
        }
    } else {
        // :930-952 (floor) and :1141-1166 (int() truncation, where x1 = ix + 1
        // for negative x and the weight x - x1 is negative).
        int x1 = ix, y1 = iy;
        dfl wx0 = fx, wy0 = fy;
        if (P == PX_FLAT_T_BL) {
            if (x.hi < 0.f) {
                x1 = ix + 1;
                wx0 = df_sub(fx, dfl{1.f, 0.f});
            }
            if (y.hi < 0.f) {
                y1 = iy + 1;
                wy0 = df_sub(fy, dfl{1.f, 0.f});
            }
        }
        const dfl wx[2] = {wx0, df_sub(dfl{1.f, 0.f}, wx0)};
        const dfl wy[2] = {wy0, df_sub(dfl{1.f, 0.f}, wy0)};
#pragma unroll
        for (int dy = 0; dy < 2; dy++) {
            const int yy = y1 + dy;
            if (yy < 0 || yy >= g.ny) continue;
#pragma unroll
            for (int dx = 0; dx < 2; dx++) {
                const int xx = x1 + dx;
                if (xx < 0 || xx >= g.nx) continue;
                if (P == PX_FLAT_NT_BL) {
                    pix[n][0] = yy;
                    pix[n][1] = xx;
                } else {
                    flat_tile_tuple(g, yy, xx, pix[n]);
                }
                w[n] = df_mul(wy[dy], wx[dx]).hi;
                n++;
            }
        }
    }
    return true;
}

// Certified spin factors (spin_proj_factors, :1180-1209): float(P * (c*c -
// s*s)) and float(P * 2*c*s) with c*c - s*s = (Nc^2 - Ns^2)/D and 2*c*s =
// 2 Nc Ns / D.  Returns false when a float32 rounding is not certain.
// CERT = false (the mixed-precision contract, where only pixel indices must
// be the reference's): the floats nearest the double-float values, always
// accepted.
template <bool CERT = true>
__device__ __forceinline__ bool fast_spin(int nc, float T, float Pr, const dfl &Nc,
                                          const dfl &Ns, const dfl &D, float *pf) {
    if (nc == 1) {
        pf[0] = T;
        pf[1] = pf[2] = 0.f;
        return true;
    }
    const dfl invD = df_recip(D);
    const dfl v1 = df_mulf(df_mul(df_dot<2>({Nc, Ns}, {Nc, df_neg(Ns)}), invD), Pr);
    const dfl v2 = df_mulf(df_mul(df_mulf(df_mul(Nc, Ns), 2.f), invD), Pr);
    // Certify the float32 rounding: v.hi is the float nearest v; the
    // reference rounds to the same float unless its value lies beyond the
    // midpoint to a neighbour, i.e. unless |v.lo| + eps reaches half the
    // gap to the nearer neighbour.
    if (CERT) {
        const float e = kEpsPf * fmaxf(1.f, 0.25f / D.hi) * fmaxf(1.f, fabsf(Pr));
        if (!(fabsf(v1.hi) > 1e-30f && fabsf(v1.lo) + e < half_gap(v1.hi))) return false;
        if (!(fabsf(v2.hi) > 1e-30f && fabsf(v2.lo) + e < half_gap(v2.hi))) return false;
    }
    if (nc == 2) {
        pf[0] = v1.hi;
        pf[1] = v2.hi;
        pf[2] = 0.f;
    } else {
        pf[0] = T;
        pf[1] = v1.hi;
        pf[2] = v2.hi;
    }
    return true;
}

// Certified spin factors of a sample whose pixel is already certain (the
// float32 tier of mixedpoint.cuh certified it): the double-float
// quaternion and the spin quantities Nc, Ns, D formed by the same
// operations as fast_native / fast_lon_spin (hence the same values), then
// fast_spin.  False where that path would not apply or the float32
// roundings are not certain.
template <int C>
__device__ __forceinline__ bool df_spin_only(const dfl (&qb)[4], const dfl (&qd)[4], int nc,
                                             float T, float Pr, float *pf) {
    if (nc == 1) {
        pf[0] = T;
        pf[1] = pf[2] = 0.f;
        return true;
    }
    dfl a, b, c, d;
    df_qmul(qb, qd, a, b, c, d);
    dfl Nc, Ns, D;
    if (C == SO3G_COORD_CAR) {
        const dfl cos_t = df_dot<4>({a, b, c, d}, {a, df_neg(b), df_neg(c), d});
        if (!(fabsf(cos_t.hi) < 0.998f)) return false;
        const dfl cd = df_mul(c, d), ab = df_mul(a, b);
        Nc = df_dot<2>({a, b}, {c, df_neg(d)});
        Ns = df_add(cd, ab);
        D = df_mulf(df_sub(dfl{1.f, 0.f}, df_mul(cos_t, cos_t)), 0.25f);
    } else {
        const dfl n = df_dot<2>({a, d}, {a, d});
        if (!(n.hi > 1e-4f)) return false;
        Nc = df_dot<2>({a, d}, {a, df_neg(d)});
        Ns = df_mulf(df_mul(a, d), 2.f);
        D = df_mul(n, n);
    }
    return fast_spin<true>(nc, T, Pr, Nc, Ns, D, pf);
}

// Integer part of a double-float whose fraction is certified to be at
// least e from 0 and 1; false otherwise.
__device__ __forceinline__ bool df_floor_cert(dfl x, float e, int &i) {
    dfl f;
    i = df_floor(x, f);
    return f.hi > e && f.hi < 1.f - e;
}

// Certified HEALPix pixel (Pixelizor_Healpix::GetPixels, :565-574 and
// :713-724, through ang2pix of src/healpix_bare.c:46-78, 271-306) of a
// sample with sin(lat) = cos_t and longitude lon.  The reference forms
// theta = pi/2 - lat from the table value of lat and takes its sin and cos
// with the math library; here sin/cos(lat) come from the tabulated sin/cos
// of the asin knot below lat and the series of the remaining angle
// (|delta| < 1e-3 for |cos_t| < 0.998).  Every integer decision of ang2pix
// (the equatorial/polar split, the wrap of phi, the face, the in-face
// indices) is certified with a margin far above the double-float error;
// false sends the sample to the exact path.  Off-map cannot happen.
template <int P>
__device__ __forceinline__ bool fast_healpix(const DGeom &g, const FastTables &ft,
                                             const FastConst &fc, const dfl &cos_t,
                                             const dfl &lon, int (*pix)[3], int &n) {
    const long long nside = g.nside;
    if (nside > (1LL << 20)) return false;   // in-face indices beyond float's integers
    // lat = v_i + delta (the table's knot and the interpolated remainder).
    const bool south = cos_t.hi < 0.f;
    const dfl u = south ? df_neg(cos_t) : cos_t;
    dfl frac;
    const int i = lut_index(u, frac);
    const float4 k = __ldg(ft.asin_t + i);
    const float4 sc = __ldg(ft.asin_sc + i);
    const dfl delta = df_mul(dfl{k.z, k.w}, frac);
    const dfl d2 = df_mul(delta, delta);
    const float d3 = delta.hi * d2.hi;
    const dfl sin_d = df_add(delta, dfl{d3 * (-1.f / 6.f), 0.f});
    const dfl cos_d = df_add(dfl{1.f, 0.f},
                             df_add(df_mulf(d2, -0.5f), dfl{d2.hi * d2.hi * (1.f / 24.f), 0.f}));
    const dfl S = dfl{sc.x, sc.y}, Cc = dfl{sc.z, sc.w};
    dfl z = df_add(df_mul(S, cos_d), df_mul(Cc, sin_d));     // sin(lat) = cos(theta)
    const dfl s = df_sub(df_mul(Cc, cos_d), df_mul(S, sin_d)); // cos(lat) = sin(theta)
    if (south) z = df_neg(z);
    // The float64 roundings of the reference (theta, sincos) move z and s by
    // ~1e-16; the double-float error is below 1e-12.
    const float ez = 1e-11f;
    const float e = fmaxf(kEpsPix, 1e-10f * (float)nside);
    const dfl za = z.hi < 0.f ? df_neg(z) : z;
    // x = phi / (2 pi) wrapped into [0, 1); tt = 4 x.
    dfl x = df_mul(lon, fc.inv_2pi);
    if (!(fabsf(x.hi) > ez)) return false;
    if (x.hi < 0.f) x = df_add(x, dfl{1.f, 0.f});
    const dfl tt = df_mulf(x, 4.f);
    const float fn = (float)nside;
    int f, ix, iy;
    // za <= 2/3, against the float64 constant 2/3 (a float comparison would
    // misplace the boundary by the float rounding of 2/3).
    const dfl dz = df_sub(za, fc.two_thirds);
    if (!(fabsf(dz.hi) > ez)) return false;
    if (dz.hi < 0.f) {
        // Equatorial belt (za <= 2/3; |za - 2/3| certified above).
        const dfl t1 = df_add(dfl{0.5f, 0.f}, tt);
        const dfl t2 = df_mulf(z, 0.75f);
        const dfl jp = df_sub(t1, t2), jm = df_add(t1, t2);
        int Jp, Jm;
        if (!df_floor_cert(df_mulf(jp, fn), e, Jp)) return false;
        if (!df_floor_cert(df_mulf(jm, fn), e, Jm)) return false;
        // jp*nside and jm*nside are not integers, so floor(jp) is
        // floor(jp*nside) div nside (jp, jm >= 0).
        if (Jp < 0 || Jm < 0) return false;
        const int ifp = Jp / (int)nside, ifm = Jm / (int)nside;
        // hx = jm - ifm, hy = 1 + ifp - jp.
        ix = Jm - ifm * (int)nside;
        iy = (1 + ifp) * (int)nside - Jp - 1;
        f = (ifp == ifm) ? (ifp | 4) : ((ifp < ifm) ? ifp : (ifm + 8));
    } else {
        // Polar caps.
        int ntt;
        if (!df_floor_cert(tt, ez, ntt)) return false;
        if (ntt >= 4) ntt = 3;
        const dfl tp = df_sub(tt, dfl{(float)ntt, 0.f});
        // tmp = s / sqrt((1 + za) * (1/3)).
        const dfl q = df_mul(df_add(dfl{1.f, 0.f}, za), fc.third);
        const float r0 = sqrtf(q.hi);
        const dfl sq = fast_two_sum(r0, (fmaf(-r0, r0, q.hi) + q.lo) / (2.f * r0));
        const dfl tmp = df_mul(s, df_recip(sq));
        const dfl jp = df_mul(tp, tmp), jm = df_mul(df_sub(dfl{1.f, 0.f}, tp), tmp);
        // The clamps at 1 only act within rounding of za = 2/3.
        if (!(jp.hi < 1.f - ez && jm.hi < 1.f - ez)) return false;
        dfl hx, hy;
        if (z.hi >= 0.f) {
            hx = df_sub(dfl{1.f, 0.f}, jm);
            hy = df_sub(dfl{1.f, 0.f}, jp);
            f = ntt;
        } else {
            hx = jp;
            hy = jm;
            f = ntt + 8;
        }
        if (!df_floor_cert(df_mulf(hx, fn), e, ix)) return false;
        if (!df_floor_cert(df_mulf(hy, fn), e, iy)) return false;
    }
    const long long ip = hp_hpd2pix(nside, P == PX_HP_T ? true : (g.nest != 0), f, ix, iy);
    if (ip < 0 || ip >= g.npix) return false;
    if (P == PX_HP_NT) {
        pix[0][0] = (int)ip;
    } else {
        hp_tile_split(g.nppt, ip, pix[0][0], pix[0][1]);
    }
    n = 1;
    return true;
}

// The certified pointing of one sample: taps (pixels, weights) and spin
// factors equal to the exact path's (bilinear weights: see fast_pixels).
// Returns false when the sample must go to the exact path.  SPIN_CERT =
// false: pixels certified, spin factors the nearest floats (fast_spin).
template <int C, int P, bool SPIN_CERT = true>
__device__ __forceinline__ bool fast_pointing(const DGeom &g, const FastTables &ft,
                                              const FastConst &fc, const dfl (&qb)[4],
                                              const dfl (&qd)[4], int nc, float T, float Pr,
                                              int (*pix)[3], float *w, int &n, float *pf) {
    if (P == PX_HP_NT || P == PX_HP_T) {
        dfl a, b, c, d;
        df_qmul(qb, qd, a, b, c, d);
        const dfl cos_t = df_dot<4>({a, b, c, d}, {a, df_neg(b), df_neg(c), d});
        if (!(fabsf(cos_t.hi) < 0.998f)) return false;
        dfl lon, Nc, Ns, D;
        if (!fast_lon_spin(ft, fc, a, b, c, d, cos_t, lon, Nc, Ns, D)) return false;
        if (!fast_healpix<P>(g, ft, fc, cos_t, lon, pix, n)) return false;
        w[0] = 1.f;
        return fast_spin<SPIN_CERT>(nc, T, Pr, Nc, Ns, D, pf);
    }
    dfl X, Y, Nc, Ns, D;
    if (!fast_native<C>(ft, fc, qb, qd, X, Y, Nc, Ns, D)) return false;
    const dfl x = df_add(df_mul(X, fc.inv_cdx), fc.off_x);
    const dfl y = df_add(df_mul(Y, fc.inv_cdy), fc.off_y);
    if (!fast_pixels<P>(g, x, y, pix, w, n)) return false;
    if (n == 0) return true;   // off the map: nothing to add
    return fast_spin<SPIN_CERT>(nc, T, Pr, Nc, Ns, D, pf);
}

// The rounding step of fast_accum from m's double-float split md.
__device__ __forceinline__ bool fast_accum_df(float &sig, dfl md, float pf) {
    const float p = md.hi * pf;
    float pe = fmaf(md.hi, pf, -p);
    pe = fmaf(md.lo, pf, pe);
    dfl s = two_sum(sig, p);
    s.lo += pe;
    s = fast_two_sum(s.hi, s.lo);
    // Error: double-float ~2^-46 and the reference's two float64 roundings,
    // relative to the operands.
    const float e = 5e-13f * (fabsf(p) + fabsf(sig));
    if (!(fabsf(s.hi) > 1e-30f && fabsf(s.lo) + e < half_gap(s.hi))) return false;
    sig = s.hi;
    return true;
}

// sig + m * pf rounded to float32 as the reference's `*sig += map * pf`
// (float64 product and sum, then float32) when that rounding is certain.
// Returns false when it is not (the caller then takes the exact path).
__device__ __forceinline__ bool fast_accum(float &sig, double m, float pf) {
    const int mh = __double2hiint(m);
    if ((((unsigned)mh & 0x7fffffffu) | (unsigned)__double2loint(m)) == 0u ||
        (pf == 0.f && (mh & 0x7ff00000) != 0x7ff00000)) {
        // The term is an exact zero with the product's sign (0 times a
        // finite value); float addition of zeros follows the same sign rules
        // as the reference's float64.
        sig = sig + __int_as_float((mh ^ __float_as_int(pf)) & 0x80000000);
        return true;
    }
    dfl md;
    if (!df_split(m, md)) return false;
    return fast_accum_df(sig, md, pf);
}

// The same with m given by its split (h, l) (k_pc_map_split): h = +-0 for
// m = +-0, NaN where m is not finite or outside df_split's range.
__device__ __forceinline__ bool fast_accum_split(float &sig, float h, float l, float pf) {
    if (h == 0.f || (pf == 0.f && h == h)) {
        sig = sig + __int_as_float((__float_as_int(h) ^ __float_as_int(pf)) & 0x80000000);
        return true;
    }
    return fast_accum_df(sig, dfl{h, l}, pf);
}

// The same for a bilinear tap: sig + m * pf * w as the reference's
// `*sig += map * pf * w` (two float64 products, a float64 sum, then
// float32).
__device__ __forceinline__ bool fast_accum(float &sig, double m, float pf, float w) {
    if (w == 1.f) return fast_accum(sig, m, pf);
    const int mh = __double2hiint(m);
    if ((((unsigned)mh & 0x7fffffffu) | (unsigned)__double2loint(m)) == 0u || pf == 0.f ||
        w == 0.f) {
        sig = sig + __int_as_float((mh ^ __float_as_int(pf) ^ __float_as_int(w)) & 0x80000000);
        return true;
    }
    dfl md;
    if (!df_split(m, md)) return false;
    const float p0 = md.hi * pf;
    float pe = fmaf(md.hi, pf, -p0);
    pe = fmaf(md.lo, pf, pe);
    const dfl t = df_mulf(fast_two_sum(p0, pe), w);
    dfl s = two_sum(sig, t.hi);
    s.lo += t.lo;
    s = fast_two_sum(s.hi, s.lo);
    // Error: double-float ~2^-45 and the reference's three float64
    // roundings, relative to the operands.
    const float e = 5e-13f * (fabsf(t.hi) + fabsf(sig));
    if (!(fabsf(s.hi) > 1e-30f && fabsf(s.lo) + e < half_gap(s.hi))) return false;
    sig = s.hi;
    return true;
}

}  // namespace so3g
