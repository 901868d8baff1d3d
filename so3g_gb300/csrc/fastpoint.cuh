// fastpoint.cuh -- certified fast pointing for CAR with nearest-neighbour
// flat pixelizors.
//
// GB300 executes float64 at 1/64 of the float32 rate, and the exact float64
// pointing (quaternion compose, two table lookups, seven IEEE divisions, one
// square root) is the whole cost of an on-the-fly projection.  This path
// evaluates the same quantities in double-float arithmetic: a value is a
// pair (hi, lo) of float32 with |lo| <= ulp(hi)/2, carried with error-free
// transformations (TwoSum, and TwoProduct through fmaf), about 44 good bits.
// It then decides, for each sample, whether its results are certain:
//
//   - the pixel index: the reference computes x = lon/cdelt + crpix - 1
//     + 0.5 and takes its integer part.  If our x is more than kEpsPix from
//     every integer, the reference's x (which differs from ours by far less)
//     has the same integer part, and the same on/off-map decision.
//   - the spin factors float(P * (c*c - s*s)) and float(P * 2*c*s): if our
//     value is farther than kEpsPf from both float rounding boundaries
//     around its float32 rounding, the reference's float64 value rounds to
//     the same float32.
//   - the branch decisions of the atan2 table near the +-pi seam and the
//     regions near the native poles, where the table and the spin factors
//     are ill-conditioned, are not certified: those samples go to the exact
//     path.
//
// A sample that is not certified is recomputed by the exact float64 path
// (device.cuh), so every result equals the exact path's bit for bit.  The
// error bounds kEpsPix and kEpsPf exceed the worst double-float error by
// well over an order of magnitude (see the measured error study in the GPU
// tests, which compare both paths sample by sample).
#pragma once

#include "device.cuh"

namespace so3g {

// Bounds of |double-float value - reference float64 value|.
constexpr float kEpsPix = 1e-7f;        // pixel coordinate units
constexpr float kEpsPf = 2.0e-12f;      // spin factor (values of order 1)

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
    dfl t = two_sum(x.lo, y.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
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

// x / y with two correction steps.
__device__ __forceinline__ dfl df_div(dfl x, dfl y) {
    float r = 1.0f / y.hi;
    float q1 = x.hi * r;
    dfl rem = df_sub(x, df_mulf(y, q1));
    float q2 = rem.hi * r;
    rem = df_sub(rem, df_mulf(y, q2));
    float q3 = rem.hi * r;
    dfl q = fast_two_sum(q1, q2);
    return df_add(q, dfl{q3, 0.f});
}

// Double-float from a double: hi = x rounded to float, lo = the rest.
__device__ __forceinline__ dfl df_from_double(double x) {
    float hi = __double2float_rn(x);
    float lo = __double2float_rn(x - (double)hi);
    return dfl{hi, lo};
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

// Table of the asin/atan2 interpolation knots as double-floats, and the
// differences to the next knot: t[i] = (v_hi, v_lo, dv_hi, dv_lo).
struct FastTables {
    const float4 *asin_t;
    const float4 *atan2_t;
};

// Piecewise-linear interpolant of a table at u in [0, 1): the value of
// LookupTable::get_raw (include/so_linterp.h:20-29) up to float64 rounding.
__device__ __forceinline__ dfl lut_df(const float4 *t, dfl u) {
    dfl d = df_mulf(u, (float)(kLutN - 1));
    dfl frac;
    int i = df_floor(d, frac);
    i = max(0, min(i, kLutN - 2));
    float4 k = __ldg(t + i);
    return df_add(dfl{k.x, k.y}, df_mul(dfl{k.z, k.w}, frac));
}

struct FastConst {
    dfl inv_cdx, inv_cdy;   // 1/cdelt
    dfl off_x, off_y;       // crpix - 1 + 0.5
    dfl pi, half_pi;
};

// The certified CAR pointing of one sample.  Returns false when the sample
// must go to the exact path.  On success: *on_map, pix (flat nearest-
// neighbour tuple as get_pixels<P> would give) and pf[0..2].
template <int P>
__device__ __forceinline__ bool fast_car(const DGeom &g, const FastTables &ft,
                                         const FastConst &fc, const dfl (&qb)[4],
                                         const dfl (&qd)[4], int nc, float T, float Pr,
                                         int *pix, bool *on_map, float *pf) {
    // q = qb * qd (Hamilton product), double-float.
    const dfl a = df_sub(df_sub(df_sub(df_mul(qb[0], qd[0]), df_mul(qb[1], qd[1])),
                                df_mul(qb[2], qd[2])), df_mul(qb[3], qd[3]));
    const dfl b = df_sub(df_add(df_add(df_mul(qb[0], qd[1]), df_mul(qb[1], qd[0])),
                                df_mul(qb[2], qd[3])), df_mul(qb[3], qd[2]));
    const dfl c = df_add(df_add(df_sub(df_mul(qb[0], qd[2]), df_mul(qb[1], qd[3])),
                                df_mul(qb[2], qd[0])), df_mul(qb[3], qd[1]));
    const dfl d = df_add(df_sub(df_add(df_mul(qb[0], qd[3]), df_mul(qb[1], qd[2])),
                                df_mul(qb[2], qd[1])), df_mul(qb[3], qd[0]));
    // cos(theta) = a^2 - b^2 - c^2 + d^2 = sin(lat).
    const dfl cos_t = df_add(df_sub(df_sub(df_mul(a, a), df_mul(b, b)), df_mul(c, c)),
                             df_mul(d, d));
    // Near the native poles (|lat| > ~87 deg) the tables' ends and the spin
    // factors are ill-conditioned: exact path.
    if (!(fabsf(cos_t.hi) < 0.998f)) return false;
    // lat = ASIN(cos_t) (odd, continuous at 0).
    dfl lat = lut_df(ft.asin_t, cos_t.hi < 0.f ? df_neg(cos_t) : cos_t);
    if (cos_t.hi < 0.f) lat = df_neg(lat);
    // lon = ATAN2(c*d - a*b, c*a + d*b).
    const dfl cd = df_mul(c, d), ab = df_mul(a, b);
    const dfl Y = df_sub(cd, ab);
    const dfl X = df_add(df_mul(c, a), df_mul(d, b));
    // The +-pi seam (Y ~ 0 with X < 0) is a discontinuity of atan2.
    if (X.hi < 0.f && !(fabsf(Y.hi) > 1e-6f)) return false;
    const bool neg = Y.hi < 0.f, mirror = X.hi < 0.f;
    const dfl ay = neg ? df_neg(Y) : Y, ax = mirror ? df_neg(X) : X;
    dfl lon;
    if (ax.hi < ay.hi) {
        lon = df_sub(fc.half_pi, lut_df(ft.atan2_t, df_div(ax, ay)));
    } else {
        lon = lut_df(ft.atan2_t, df_div(ay, ax));
    }
    if (mirror) lon = df_sub(fc.pi, lon);
    if (neg) lon = df_neg(lon);

    // Pixel: x = lon / cdx + crpix_x - 1 + 0.5 (and y), integer part.
    const dfl x = df_add(df_mul(lon, fc.inv_cdx), fc.off_x);
    const dfl y = df_add(df_mul(lat, fc.inv_cdy), fc.off_y);
    dfl fx, fy;
    const int ix = df_floor(x, fx), iy = df_floor(y, fy);
    if (!(fx.hi > kEpsPix && fx.hi < 1.f - kEpsPix && fy.hi > kEpsPix &&
          fy.hi < 1.f - kEpsPix))
        return false;
    if (P == PX_FLAT_NT_NN) {
        // :912-926 (x not near an integer: floor decides the bounds)
        *on_map = ix >= 0 && ix < g.nx && iy >= 0 && iy < g.ny;
        if (*on_map) {
            pix[0] = iy;
            pix[1] = ix;
        }
    } else {
        // :1124-1138 (int() truncation: x in (-1, 0) lands in column 0)
        const int tx = (x.hi < 0.f) ? ix + 1 : ix, ty = (y.hi < 0.f) ? iy + 1 : iy;
        *on_map = tx >= 0 && tx < g.nx && ty >= 0 && ty < g.ny && x.hi > -1.f && y.hi > -1.f;
        if (*on_map) {
            const int sub_y = ty / g.ty, sub_x = tx / g.tx;
            pix[0] = sub_y * g.ntx + sub_x;
            pix[1] = ty - sub_y * g.ty;
            pix[2] = tx - sub_x * g.tx;
        }
    }

    // Spin factors (:1180-1209): c = Nc/h, s = Ns/h with h^2 = (1-cos^2)/4,
    // so c*c - s*s = (Nc^2 - Ns^2)/D and 2*c*s = 2 Nc Ns / D, D = h^2.
    if (nc == 1) {
        pf[0] = T;
        pf[1] = pf[2] = 0.f;
        return true;
    }
    const dfl Nc = df_sub(df_mul(a, c), df_mul(b, d));
    const dfl Ns = df_add(cd, ab);
    const dfl D = df_mulf(df_sub(dfl{1.f, 0.f}, df_mul(cos_t, cos_t)), 0.25f);
    const dfl invD = df_div(dfl{1.f, 0.f}, D);
    const dfl v1 = df_mulf(df_mul(df_sub(df_mul(Nc, Nc), df_mul(Ns, Ns)), invD), Pr);
    const dfl v2 = df_mulf(df_mul(df_mulf(df_mul(Nc, Ns), 2.f), invD), Pr);
    // Certify the float32 rounding: v.hi is the float nearest v; the
    // reference rounds to the same float unless its value lies beyond the
    // midpoint to a neighbour, i.e. unless |v.lo| + eps reaches half the
    // gap to the nearer neighbour (the gap below a power of two is half).
    const float e = kEpsPf * fmaxf(1.f, 0.25f / D.hi) * fmaxf(1.f, fabsf(Pr));
    #pragma unroll
    for (int k = 0; k < 2; k++) {
        const dfl v = k ? v2 : v1;
        const float m = fabsf(v.hi);
        if (m < 1e-30f) return false;
        const float gap = m - __int_as_float(__float_as_int(m) - 1);   // gap to the float below
        if (!(fabsf(v.lo) + e < 0.5f * gap)) return false;
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

}  // namespace so3g
