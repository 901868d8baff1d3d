// mixedpoint.cuh -- float32 pointing with certified pixel indices
// (SO3G_POINTING_MIXED), for CAR with a nearest-neighbour flat pixelizor.
//
// The sample's quaternion product, table lookups, pixel coordinates and
// spin factors are evaluated in plain float32.  Alongside, a bound on the
// error of each pixel coordinate against the reference's float64 value is
// formed from the operands' magnitudes (the derivation is in the comments
// below; u = 2^-24).  A sample whose pixel coordinates are farther than
// their bounds from every integer gets the reference's pixel index; the
// others (a few percent) are handed to the certified double-float path,
// and from there, if needed, to the exact float64 path.  Pixel indices are
// therefore always the reference's.  The spin factors are float32
// evaluations of the same expressions (relative error ~1e-7, at most a few
// 1e-6 where |sin lat| approaches the 0.9 guard): maps and signals agree
// with the float64 path to ~1e-7 of their scale.
#pragma once

#include "fastpoint.cuh"

namespace so3g {

constexpr float kU = 5.9604645e-8f;   // 2^-24

// Pixelizations with the certified double-float pointing.
template <int C, int P>
struct FastEligible {
    static constexpr bool value =
        (C == SO3G_COORD_CAR || C == SO3G_COORD_TAN || C == SO3G_COORD_ZEA ||
         C == SO3G_COORD_SIN) &&
        (P == PX_FLAT_NT_NN || P == PX_FLAT_T_NN || P == PX_FLAT_NT_BL ||
         P == PX_FLAT_T_BL) ||
        (C == SO3G_COORD_CAR && (P == PX_HP_NT || P == PX_HP_T));
};

// Pixelizations with the float32 tier of SO3G_POINTING_MIXED.
template <int C, int P>
struct MixedEligible {
    static constexpr bool value =
        C == SO3G_COORD_CAR && (P == PX_FLAT_NT_NN || P == PX_FLAT_T_NN);
};

struct MixedConst {
    float inv_cdx, inv_cdy;   // 1/cdelt, rounded to float32
    float off_x, off_y;       // crpix - 1 + 0.5
    float pi, half_pi;
};

// Calls f.template go<MODE>() for the kernel variant of pointing mode `fast`.
template <int C, int P, class F>
int by_mode(int fast, F &f) {
    if constexpr (MixedEligible<C, P>::value) {
        if (fast == SO3G_POINTING_MIXED) return f.template go<2>();
    }
    if constexpr (FastEligible<C, P>::value) {
        if (fast != SO3G_POINTING_EXACT) return f.template go<1>();
    }
    return f.template go<0>();
}

// A float64 value truncated to float32 with integer operations (relative
// error < 2^-23 = 2u); 0 outside [2^-126, 2^128).
__device__ __forceinline__ float d2f_trunc(double x) {
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const unsigned ex = (hw >> 20) & 0x7ffu;
    const float v = __uint_as_float((hw & 0x80000000u) | ((ex - 896u) << 23) |
                                    ((hw & 0xfffffu) << 3) | (lw >> 29));
    return (ex > 896u && ex < 1151u) ? v : 0.f;
}

// A float64 value rounded to float32 (half-way cases away from zero) with
// integer operations: relative error <= u.  A carry out of the significand
// moves into the exponent, which is the correct rounding.  0 outside
// [2^-126, 2^127).
__device__ __forceinline__ float d2f_round(double x) {
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const unsigned ex = (hw >> 20) & 0x7ffu;
    const unsigned mag = (((ex - 896u) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29)) +
                         ((lw >> 28) & 1u);
    const float v = __uint_as_float((hw & 0x80000000u) | mag);
    return (ex > 896u && ex < 1150u) ? v : 0.f;
}

// The float32 boresight quaternion of sample t: from the float32 copy
// when there is one, else rounded from the float64 boresight.
__device__ __forceinline__ void load_bore_f32(const float4 *b32, const double *bore, int t,
                                              float (&qb)[4]) {
    if (b32) {
        const float4 v = __ldg(b32 + t);
        qb[0] = v.x;
        qb[1] = v.y;
        qb[2] = v.z;
        qb[3] = v.w;
    } else {
        const double2 lo = __ldg(reinterpret_cast<const double2 *>(bore + 4LL * t));
        const double2 hi = __ldg(reinterpret_cast<const double2 *>(bore + 4LL * t) + 1);
        qb[0] = d2f_round(lo.x);
        qb[1] = d2f_round(lo.y);
        qb[2] = d2f_round(hi.x);
        qb[3] = d2f_round(hi.y);
    }
}

// Piecewise-linear table value in float32: knot i and fraction f of
// u * (n-1); also returns the local slope (table units per unit of u).
__device__ __forceinline__ float lut_f(const float4 *t, float u, float &slope) {
    const float s = u * (float)(kLutN - 1);
    int i = (int)s;
    i = max(0, min(i, kLutN - 2));
    const float f = s - (float)i;
    const float4 k = __ldg(t + i);
    slope = fabsf(k.z) * (float)(kLutN - 1);
    return fmaf(k.z, f, k.x);
}

// The float32 tier.  Returns false when the sample must go to the
// double-float path: near the native poles (|sin lat| >= 0.9, where the
// float32 spin factors lose accuracy), at the atan2 seam, or when a pixel
// coordinate is within its error bound of an integer.
template <int P>
__device__ __forceinline__ bool mixed_car(const DGeom &g, const FastTables &ft,
                                          const MixedConst &mc, const float (&qb)[4],
                                          const float (&qd)[4], int nc, float T, float Pr,
                                          int *pix, bool &on, float *pf) {
    // q = qb * qd with qb and qd rounded to float32 (relative u each).  The
    // error quaternion dq = q~ - q has |dq| <= 2u (inputs: the product of
    // quaternions multiplies norms) + 8u (four roundings per component,
    // each <= u * sum|terms| <= u) = 10u.  A rotation off by dq points
    // <= 2|dq| away, so the exact longitude of q~ is off by <= 20u / cos(lat)
    // and sin(lat) by <= 20u cos(lat); |q~|^2 = 1 +- 20u scales sin(lat).
    const float a = fmaf(qb[0], qd[0], fmaf(-qb[1], qd[1], fmaf(-qb[2], qd[2], -qb[3] * qd[3])));
    const float b = fmaf(qb[0], qd[1], fmaf(qb[1], qd[0], fmaf(qb[2], qd[3], -qb[3] * qd[2])));
    const float c = fmaf(qb[0], qd[2], fmaf(-qb[1], qd[3], fmaf(qb[2], qd[0], qb[3] * qd[1])));
    const float d = fmaf(qb[0], qd[3], fmaf(qb[1], qd[2], fmaf(-qb[2], qd[1], qb[3] * qd[0])));
    // cos(theta) = sin(lat): error <= 20u cos(lat) (rotation) + 20u |sin(lat)|
    // (norm) + 4u (roundings).
    const float cos_t = fmaf(a, a, fmaf(-b, b, fmaf(-c, c, d * d)));
    if (!(fabsf(cos_t) < 0.9f)) return false;
    // lat = ASIN(cos_t): the table's slope times that error, plus u |cos_t|
    // (the index) and 5u (table values and the final fma rounded to
    // float32).  The rotation part times the slope is <= 20.1u (the secant
    // slope of asin on a knot interval is within 1.0003 of 1 / cos(lat) for
    // |sin lat| < 0.9): <= 25.1u + slope (21u |cos_t| + 4u).
    float slope_lat;
    float lat = lut_f(ft.asin_t, fabsf(cos_t), slope_lat);
    if (cos_t < 0.f) lat = -lat;
    // lon = ATAN2(Y, X), Y = c*d - a*b, X = c*a + d*b, |(X, Y)| = cos(lat)/2.
    // Their float32 roundings are <= u each (|ca| + |db| <= 1/2), i.e. an
    // angle <= 2.83u / cos(lat).
    const float Y = fmaf(c, d, -a * b), X = fmaf(c, a, d * b);
    const float ay = fabsf(Y), ax = fabsf(X);
    if (X < 0.f && !(ay > 64.f * kU)) return false;   // the +-pi seam
    const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    const float inv_mx = __frcp_rn(mx);
    // r = mn * (1/mx) rounded twice (2u); atan has slope <= 1.
    float slope_lon;
    float th = lut_f(ft.atan2_t, mn * inv_mx, slope_lon);
    float lon = (ax < ay) ? mc.half_pi - th : th;
    if (X < 0.f) lon = mc.pi - lon;
    if (Y < 0.f) lon = -lon;
    // lon error <= 22.9u / cos(lat) + 2u (r) + 5.4u (table) + 9.5u (the
    // subtractions from pi/2 and pi and those constants' roundings), and
    // 1 / cos(lat) <= 1 / (2 mx): <= 11.5u / mx + 17u.
    const float elon = fmaf(11.5f * kU, inv_mx, 17.f * kU);
    const float elat = fmaf(slope_lat, fmaf(21.f * kU, fabsf(cos_t), 4.f * kU), 25.1f * kU);
    // Pixel coordinates x = lon / cdx + crpix_x - 1 + 0.5 (and y), with the
    // float32 rounding of 1/cdx, of the offset and of the fma; x1.5 safety.
    const float lx = lon * mc.inv_cdx, ly = lat * mc.inv_cdy;
    const float x = fmaf(lon, mc.inv_cdx, mc.off_x), y = fmaf(lat, mc.inv_cdy, mc.off_y);
    const float ex = 1.5f * fmaf(fabsf(mc.inv_cdx), elon,
                                 kU * (fabsf(lx) + fabsf(mc.off_x) + fabsf(x)));
    const float ey = 1.5f * fmaf(fabsf(mc.inv_cdy), elat,
                                 kU * (fabsf(ly) + fabsf(mc.off_y) + fabsf(y)));
    const float fx = floorf(x), fy = floorf(y);
    const float rx = x - fx, ry = y - fy;
    if (!(rx > ex && rx < 1.f - ex && ry > ey && ry < 1.f - ey)) return false;
    const int ix = (int)fx, iy = (int)fy;
    if (P == PX_FLAT_NT_NN) {
        on = ix >= 0 && ix < g.nx && iy >= 0 && iy < g.ny;
        if (on) {
            pix[0] = iy;
            pix[1] = ix;
        }
    } else {
        const int tx = (x < 0.f) ? ix + 1 : ix, ty = (y < 0.f) ? iy + 1 : iy;
        on = tx >= 0 && tx < g.nx && ty >= 0 && ty < g.ny && x > -1.f && y > -1.f;
        if (on) {
            const int sub_y = ty / g.ty, sub_x = tx / g.tx;
            pix[0] = sub_y * g.ntx + sub_x;
            pix[1] = ty - sub_y * g.ty;
            pix[2] = tx - sub_x * g.tx;
        }
    }
    if (!on) return true;
    // Spin factors (:1180-1209) with c = Nc/h, s = Ns/h, h^2 = D
    // = (a^2 + d^2)(b^2 + c^2) (= (1 - cos^2)/4 without cancellation).
    if (nc == 1) {
        pf[0] = T;
        pf[1] = pf[2] = 0.f;
        return true;
    }
    const float Nc = fmaf(a, c, -b * d), Ns = fmaf(c, d, a * b);
    const float D = fmaf(a, a, d * d) * fmaf(b, b, c * c);
    const float k = Pr * __frcp_rn(D);
    const float v1 = fmaf(Nc, Nc, -Ns * Ns) * k, v2 = 2.f * Nc * Ns * k;
    if (nc == 2) {
        pf[0] = v1;
        pf[1] = v2;
        pf[2] = 0.f;
    } else {
        pf[0] = T;
        pf[1] = v1;
        pf[2] = v2;
    }
    return true;
}

}  // namespace so3g
