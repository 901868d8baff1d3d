// fastpoint.cuh -- certified fast pointing for CAR with nearest-neighbour
// flat pixelizors.
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
};

// Piecewise-linear interpolant of a table at u in [0, 1]: the value of
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
    // q = qb * qd (Hamilton product).
    const dfl a = df_dot<4>({qb[0], qb[1], qb[2], qb[3]},
                            {qd[0], df_neg(qd[1]), df_neg(qd[2]), df_neg(qd[3])});
    const dfl b = df_dot<4>({qb[0], qb[1], qb[2], qb[3]},
                            {qd[1], qd[0], qd[3], df_neg(qd[2])});
    const dfl c = df_dot<4>({qb[0], qb[1], qb[2], qb[3]},
                            {qd[2], df_neg(qd[3]), qd[0], qd[1]});
    const dfl d = df_dot<4>({qb[0], qb[1], qb[2], qb[3]},
                            {qd[3], qd[2], df_neg(qd[1]), qd[0]});
    // cos(theta) = a^2 - b^2 - c^2 + d^2 = sin(lat).
    const dfl cos_t = df_dot<4>({a, b, c, d}, {a, df_neg(b), df_neg(c), d});
    // Near the native poles (|lat| > ~87 deg) the tables' ends and the spin
    // factors are ill-conditioned: exact path.
    if (!(fabsf(cos_t.hi) < 0.998f)) return false;
    // lat = ASIN(cos_t) (odd, continuous at 0).
    const bool south = cos_t.hi < 0.f;
    dfl lat = lut_df(ft.asin_t, south ? df_neg(cos_t) : cos_t);
    if (south) lat = df_neg(lat);
    // lon = ATAN2(c*d - a*b, c*a + d*b).
    const dfl cd = df_mul(c, d), ab = df_mul(a, b);
    const dfl Y = df_sub(cd, ab);
    const dfl X = df_dot<2>({c, d}, {a, b});
    // The +-pi seam (Y ~ 0 with X < 0) is a discontinuity of atan2.
    if (X.hi < 0.f && !(fabsf(Y.hi) > 1e-6f)) return false;
    const bool neg = Y.hi < 0.f, mirror = X.hi < 0.f;
    const dfl ay = neg ? df_neg(Y) : Y, ax = mirror ? df_neg(X) : X;
    dfl lon;
    if (ax.hi < ay.hi) {
        lon = df_sub(fc.half_pi, lut_df(ft.atan2_t, df_mul(ax, df_recip(ay))));
    } else {
        lon = lut_df(ft.atan2_t, df_mul(ay, df_recip(ax)));
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
    const dfl Nc = df_dot<2>({a, b}, {c, df_neg(d)});
    const dfl Ns = df_add(cd, ab);
    const dfl D = df_mulf(df_sub(dfl{1.f, 0.f}, df_mul(cos_t, cos_t)), 0.25f);
    const dfl invD = df_recip(D);
    const dfl v1 = df_mulf(df_mul(df_dot<2>({Nc, Ns}, {Nc, df_neg(Ns)}), invD), Pr);
    const dfl v2 = df_mulf(df_mul(df_mulf(df_mul(Nc, Ns), 2.f), invD), Pr);
    // Certify the float32 rounding: v.hi is the float nearest v; the
    // reference rounds to the same float unless its value lies beyond the
    // midpoint to a neighbour, i.e. unless |v.lo| + eps reaches half the
    // gap to the nearer neighbour.
    const float e = kEpsPf * fmaxf(1.f, 0.25f / D.hi) * fmaxf(1.f, fabsf(Pr));
    if (!(fabsf(v1.hi) > 1e-30f && fabsf(v1.lo) + e < half_gap(v1.hi))) return false;
    if (!(fabsf(v2.hi) > 1e-30f && fabsf(v2.lo) + e < half_gap(v2.hi))) return false;
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

// sig + m * pf rounded to float32 as the reference's `*sig += map * pf`
// (float64 product and sum, then float32) when that rounding is certain.
// Returns false when it is not (the caller then takes the exact path).
__device__ __forceinline__ bool fast_accum(float &sig, double m, float pf) {
    const int mh = __double2hiint(m);
    if ((((unsigned)mh & 0x7fffffffu) | (unsigned)__double2loint(m)) == 0u || pf == 0.f) {
        // The term is an exact zero with the product's sign; float addition
        // of zeros follows the same sign rules as the reference's float64.
        sig = sig + __int_as_float((mh ^ __float_as_int(pf)) & 0x80000000);
        return true;
    }
    dfl md;
    if (!df_split(m, md)) return false;
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

}  // namespace so3g
