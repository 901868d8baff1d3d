// mixedpoint.cuh -- float32 pointing with certified pixel indices
// (SO3G_POINTING_MIXED), for CAR, TAN, ZEA and SIN with nearest-neighbour
// flat pixelizors and for HEALPix.
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
// evaluations of the same expressions: the float32 inputs and the
// product's roundings (|dq| <= 10u) turn the polarisation angle by at most
// 4|dq| / cos(lat), so a factor is within 2e-5 of P where |sin lat|
// approaches the 0.9 guard and within ~3e-7 near the native equator, where
// the maps of a scan centred on its map lie (measured on the benchmark
// workloads: <= 3.3e-7 per sample; maps within 1e-7 of each pixel's sum of
// |terms|).
#pragma once

#include "fastpoint.cuh"

namespace so3g {

constexpr float kU = 5.9604645e-8f;   // 2^-24

// Pixelizations with the certified double-float pointing.
template <int C, int P>
struct FastEligible {
    static constexpr bool value =
        (C == SO3G_COORD_CAR || C == SO3G_COORD_TAN || C == SO3G_COORD_ZEA ||
         C == SO3G_COORD_SIN || C == SO3G_COORD_ARC) &&
        (P == PX_FLAT_NT_NN || P == PX_FLAT_T_NN || P == PX_FLAT_NT_BL ||
         P == PX_FLAT_T_BL) ||
        (C == SO3G_COORD_CAR && (P == PX_HP_NT || P == PX_HP_T));
};

// Pixelizations with the float32 tier of SO3G_POINTING_MIXED.
template <int C, int P>
struct MixedEligible {
    static constexpr bool value =
        ((C == SO3G_COORD_CAR || C == SO3G_COORD_TAN || C == SO3G_COORD_ZEA ||
          C == SO3G_COORD_SIN) &&
         (P == PX_FLAT_NT_NN || P == PX_FLAT_T_NN)) ||
        (C == SO3G_COORD_CAR && (P == PX_HP_NT || P == PX_HP_T));
};


// Per-warp copy, in shared memory, of the detector quantities only the
// fallback passes use: kept out of the main loop's registers.
struct WarpPiece {
    QuatD ofs;      // detector offset (exact path)
    dfl qd[4];      // its double-float split (double-float path)
};

struct MixedConst {
    float inv_cdx, inv_cdy;   // 1/cdelt, rounded to float32
    float off_x, off_y;       // crpix - 1 + 0.5
    float pi, half_pi;
};

// Calls f.template go<MODE>() for the kernel variant of pointing mode `fast`.
// Mixed pointing where the float32 tier does not apply (bilinear
// pixelizors) runs the double-float tier with float32 spin factors and
// terms.
template <int C, int P, class F>
int by_mode(int fast, F &f) {
    if constexpr (FastEligible<C, P>::value) {
        if (fast == SO3G_POINTING_MIXED) return f.template go<2>();
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

// Reciprocal by the hardware approximation (PTX rcp.approx.ftz.f32, at most
// 1 ulp = 2u relative error; subnormal inputs flush to zero, which the
// callers exclude): one instruction, against the several of the correctly
// rounded __frcp_rn.
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
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

// The float32 quaternion product and CAR longitude/latitude of a sample,
// with bounds on their errors against the reference's float64 values.
// False where the float32 tier does not apply: near the native poles
// (|sin lat| >= 0.9, where the float32 spin factors lose accuracy) and at
// the atan2 seam.
struct MixedLonLat {
    float a, b, c, d;      // q = qb * qd
    float cos_t;           // sin(lat)
    float lon, lat;
    float elon, elat;      // error bounds (no safety factor)
};

__device__ __forceinline__ bool mixed_lonlat(const FastTables &ft, const MixedConst &mc,
                                             const float (&qb)[4], const float (&qd)[4],
                                             MixedLonLat &o) {
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
    // (the index) and the table's roundings (2u |lat| + 0.01u, as for the
    // longitude).  The rotation part times the slope is <= 20.1u (the
    // secant slope of asin on a knot interval is within 1.0003 of
    // 1 / cos(lat) for |sin lat| < 0.9): <= 20.11u + 2u |lat|
    // + slope (21u |cos_t| + 4u).
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
    // mx >= |(X, Y)| / sqrt(2) > 0.15 here (|sin lat| < 0.9).
    const float inv_mx = rcp_approx(mx);
    // r = mn * (1/mx): the reciprocal's 2u and the product's u (3u);
    // atan has slope <= 1.
    float slope_lon;
    const float th = lut_f(ft.atan2_t, mn * inv_mx, slope_lon);
    float lon = (ax < ay) ? mc.half_pi - th : th;
    if (X < 0.f) lon = mc.pi - lon;
    if (Y < 0.f) lon = -lon;
    // lon error <= 22.9u / cos(lat) + 3u (r) + the table's roundings
    // (u |th| + u |dv f| + u |th|, with |dv f| <= 1e-4: 2u |th| + 0.01u)
    // + 3.2u if th was subtracted from pi/2 + 6.3u if from pi (those
    // constants' roundings and the subtractions'), and 1 / cos(lat) <=
    // 1 / (2 mx).
    o.a = a;
    o.b = b;
    o.c = c;
    o.d = d;
    o.cos_t = cos_t;
    o.lon = lon;
    o.lat = lat;
    o.elon = fmaf(11.5f * kU, inv_mx,
                  fmaf(2.f * kU, th, (3.01f + (ax < ay ? 3.2f : 0.f) + (X < 0.f ? 6.3f : 0.f)) * kU));
    o.elat = fmaf(slope_lat, fmaf(21.f * kU, fabsf(cos_t), 4.f * kU),
                  fmaf(2.f * kU, fabsf(lat), 20.11f * kU));
    return true;
}

// Spin factors (:1180-1209) in float32 with c = Nc/h, s = Ns/h, h^2 = D =
// (a^2 + d^2)(b^2 + c^2) (= (1 - cos^2)/4 without cancellation).
__device__ __forceinline__ void mixed_spin(const MixedLonLat &o, int nc, float T, float Pr,
                                           float *pf) {
    if (nc == 1) {
        pf[0] = T;
        pf[1] = pf[2] = 0.f;
        return;
    }
    const float a = o.a, b = o.b, c = o.c, d = o.d;
    const float Nc = fmaf(a, c, -b * d), Ns = fmaf(c, d, a * b);
    // D = (1 - sin^2 lat) / 4 > 0.04 where the float32 tier applies.
    const float D = fmaf(a, a, d * d) * fmaf(b, b, c * c);
    const float k = Pr * rcp_approx(D);
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
}

// Floor of a float32 value whose error bound is e; false when the value is
// within e of an integer (then the reference's floor is not certain).
__device__ __forceinline__ bool floor_cert(float v, float e, int &i) {
    const float f = floorf(v);
    const float r = v - f;
    i = (int)f;
    return r > e && r < 1.f - e;
}

// The flat pixelizor step of the float32 tier: pixel coordinates x = X /
// cdx + crpix_x - 1 + 0.5 (and y) from projection-plane coordinates (X, Y)
// with error bounds (eX, eY), the float32 roundings of 1/cdx, of the offset
// and of the fma added, x1.5 safety; false when an integer part is not
// certain.  PARENT (tiled): the pixel's parent-map coordinates (iy, ix) in
// pix[0..1] instead of its tile tuple.
template <int P, bool PARENT = false>
__device__ __forceinline__ bool mixed_flat_pixel(const DGeom &g, const MixedConst &mc, float X,
                                                 float Y, float eX, float eY, int *pix,
                                                 bool &on) {
    const float lx = X * mc.inv_cdx, ly = Y * mc.inv_cdy;
    const float x = fmaf(X, mc.inv_cdx, mc.off_x), y = fmaf(Y, mc.inv_cdy, mc.off_y);
    const float ex = 1.5f * fmaf(fabsf(mc.inv_cdx), eX,
                                 kU * (fabsf(lx) + fabsf(mc.off_x) + fabsf(x)));
    const float ey = 1.5f * fmaf(fabsf(mc.inv_cdy), eY,
                                 kU * (fabsf(ly) + fabsf(mc.off_y) + fabsf(y)));
    int ix, iy;
    if (!(floor_cert(x, ex, ix) & floor_cert(y, ey, iy))) return false;
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
            if (PARENT) {
                pix[0] = ty;
                pix[1] = tx;
            } else {
                flat_tile_tuple(g, ty, tx, pix);
            }
        }
    }
    return true;
}

// The float32 tier for CAR with a nearest-neighbour flat pixelizor.
// Returns false when the sample must go to the double-float path.
template <int P, bool SPIN, bool PARENT>
__device__ __forceinline__ bool mixed_car(const DGeom &g, const FastTables &ft,
                                          const MixedConst &mc, const float (&qb)[4],
                                          const float (&qd)[4], int nc, float T, float Pr,
                                          int *pix, bool &on, float *pf) {
    MixedLonLat o;
    if (!mixed_lonlat(ft, mc, qb, qd, o)) return false;
    if (!mixed_flat_pixel<P, PARENT>(g, mc, o.lon, o.lat, o.elon, o.elat, pix, on))
        return false;
    if (SPIN && on) mixed_spin(o, nc, T, Pr, pf);
    return true;
}

// The float32 tier for the zenithal projections (Pointer<ProjTAN|ProjZEA|
// ProjSIN>::GetCoords, :337-437) with a nearest-neighbour flat pixelizor.
// With n = a^2 + d^2 = cos^2(theta/2), u = ab - cd, v = ac + bd ((u, v)
// has length sin(theta)/2): SIN (X, Y) = 2 (u, v), TAN 2 (u, v) / (2n - 1),
// ZEA 2 (u, v) / sqrt(n).  Error bounds: the rotation error 2|dq| <= 20u
// moves the point on the sphere by <= 20u, which moves (X, Y) by <= 20u
// (SIN), 20u / cos(theta)^2 (TAN) or 20u / cos(theta/2) (ZEA); |q~|^2 = 1
// +- 20u scales u, v and n; plus the float32 roundings.  False (double-
// float path) far from the projection's pole: TAN with cos(theta) < 0.1,
// ZEA and SIN with n < 0.25 (theta > 120 deg).
template <int C, int P, bool SPIN, bool PARENT>
__device__ __forceinline__ bool mixed_zen(const DGeom &g, const MixedConst &mc,
                                          const float (&qb)[4], const float (&qd)[4], int nc,
                                          float T, float Pr, int *pix, bool &on, float *pf) {
    const float a = fmaf(qb[0], qd[0], fmaf(-qb[1], qd[1], fmaf(-qb[2], qd[2], -qb[3] * qd[3])));
    const float b = fmaf(qb[0], qd[1], fmaf(qb[1], qd[0], fmaf(qb[2], qd[3], -qb[3] * qd[2])));
    const float c = fmaf(qb[0], qd[2], fmaf(-qb[1], qd[3], fmaf(qb[2], qd[0], qb[3] * qd[1])));
    const float d = fmaf(qb[0], qd[3], fmaf(qb[1], qd[2], fmaf(-qb[2], qd[1], qb[3] * qd[0])));
    const float n = fmaf(a, a, d * d);
    if (!(n > 0.25f)) return false;
    const float u = fmaf(a, b, -c * d), v = fmaf(a, c, b * d);
    float X, Y, e;
    if (C == SO3G_COORD_SIN) {
        X = 2.f * u;
        Y = 2.f * v;
        e = fmaf(21.f * kU, fabsf(X) + fabsf(Y), 24.f * kU);
    } else if (C == SO3G_COORD_TAN) {
        const float ct = fmaf(2.f, n, -1.f);
        if (!(ct > 0.1f)) return false;
        const float r = __frcp_rn(ct);
        X = 2.f * u * r;
        Y = 2.f * v * r;
        // 20u sec^2 (rotation) + 2u sec (u's and v's absolute rounding,
        // <= u) + |P| (24u: their norm scaling and the reciprocal's and
        // products' roundings; 44u sec: the norm and roundings of 2n - 1).
        e = fmaf(fmaf(20.f * kU, r, 2.f * kU), r,
                 (fabsf(X) + fabsf(Y)) * fmaf(44.f * kU, r, 30.f * kU));
    } else {
        const float r = rsqrtf(n) * (1.f + 4.f * kU);   // >= 1/sqrt(n)
        const float sq = sqrtf(n);
        X = 2.f * u / sq;
        Y = 2.f * v / sq;
        // 20u / cos(theta/2) (rotation) + 2u / cos(theta/2) (u's and v's
        // absolute rounding, <= u) + |P| (10u: norm, 6u: roundings).
        e = fmaf(22.f * kU, r, 16.f * kU * (fabsf(X) + fabsf(Y)));
    }
    if (!mixed_flat_pixel<P, PARENT>(g, mc, X, Y, e, e, pix, on)) return false;
    if (!on || !SPIN) return true;
    // Spin factors (:1180-1209) with c = (a^2 - d^2)/n, s = 2ad/n.
    if (nc == 1) {
        pf[0] = T;
        pf[1] = pf[2] = 0.f;
        return true;
    }
    const float N1 = fmaf(a, a, -d * d), N2 = 2.f * a * d;
    const float k = Pr * __frcp_rn(n * n);
    const float v1 = fmaf(N1, N1, -N2 * N2) * k, v2 = 2.f * N1 * N2 * k;
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

// The HEALPix pixel (ang2pix, src/healpix_bare.c:46-78, 271-306) of a
// sample from float32 phi = lon (error <= elon), z = sin(lat) (<= ez) and
// s = cos(lat) (<= es), every integer decision certified against the
// propagated error bound (x1.5 safety).  False when it is not certain (or
// nside is beyond float's integers); the pixel is always on the map.
// FROM_Z: s is not given; the caps' s / sqrt((1 + |z|) / 3) is formed as
// sqrt(3 (1 - |z|)), the same quantity.
template <int P, bool PARENT, bool FROM_Z = false>
__device__ __forceinline__ bool hp_pixel_f32(const DGeom &g, float lon, float elon, float z,
                                             float ez, float s, float es, int *pix) {
    const long long nside = g.nside;
    if (nside > (1LL << 20)) return false;
    constexpr float m = 1.5f;
    // x = phi / (2 pi), wrapped into [0, 1); tt = 4 x.
    constexpr float kInv2Pi = 0.15915494f;
    float x = lon * kInv2Pi;
    float ex = fmaf(elon, kInv2Pi, 2.f * kU * fabsf(x));
    if (!(fabsf(x) > m * ex)) return false;
    if (x < 0.f) {
        x += 1.f;
        ex += kU;
    }
    const float tt = 4.f * x, ett = 4.f * ex;
    const float za = fabsf(z);
    const float fn = (float)(int)nside;   // nside <= 2^20: a 32-bit conversion
    // za <= 2/3 (the float32 2/3 is within 2e-8 of the float64 constant).
    if (!(fabsf(za - 0.6666667f) > fmaf(m, ez, 3e-8f))) return false;
    int f, ix, iy;
    if (za < 0.6666667f) {
        // Equatorial belt: jp = 0.5 + tt - 0.75 z, jm = 0.5 + tt + 0.75 z;
        // ix, iy, the face from floor(jm * nside), floor(jp * nside).
        const float t1 = 0.5f + tt, t2 = 0.75f * z;
        const float jp = t1 - t2, jm = t1 + t2;
        const float ej =
            fmaf(m, fmaf(0.75f, ez, ett), kU * (fabsf(t1) + 1.f + fabsf(jp) + fabsf(jm)));
        const float JP = jp * fn, JM = jm * fn;
        const float eJ = fmaf(ej, fn, kU * fmaxf(fabsf(JP), fabsf(JM)));
        int Jp, Jm;
        if (!(floor_cert(JP, eJ, Jp) & floor_cert(JM, eJ, Jm))) return false;
        if (Jp < 0 || Jm < 0) return false;
        const int ns = (int)nside;
        const int ifp = Jp / ns, ifm = Jm / ns;
        ix = Jm - ifm * ns;
        iy = (1 + ifp) * ns - Jp - 1;
        f = (ifp == ifm) ? (ifp | 4) : ((ifp < ifm) ? ifp : (ifm + 8));
    } else {
        // Polar caps: tmp = s / sqrt((1 + za) / 3), jp = tp tmp, jm = (1 - tp) tmp.
        int ntt;
        if (!floor_cert(tt, m * ett, ntt)) return false;
        if (ntt >= 4) ntt = 3;
        const float tp = tt - (float)ntt;
        float tmp, etmp;
        if (FROM_Z) {
            // 1 - za is exact (za > 1/2); 3 (1 - za) and the root rounded
            // once each; |sqrt(a) - sqrt(b)| <= |a - b| / sqrt(a); the
            // reciprocal's 2u inside the 1.000001.
            const float w1 = 1.f - za;
            tmp = sqrtf(3.f * w1);
            etmp = fmaf(3.f * fmaf(kU, w1, ez) * 1.000001f, rcp_approx(tmp), kU * tmp) + 1e-15f;
        } else {
            const float q = (1.f + za) * 0.33333334f;
            const float eq = fmaf(ez, 0.33333334f, 3.f * kU * q);
            const float sq = sqrtf(q);
            tmp = s / sq;
            etmp = fmaf(es + tmp * eq / (2.f * q), 1.f / sq, 3.f * kU * tmp);
        }
        const float jp = tp * tmp, jm = (1.f - tp) * tmp;
        const float ejp = m * fmaf(ett, tmp, fmaf(tp, etmp, kU * jp));
        const float ejm = m * fmaf(ett, tmp, fmaf(1.f - tp, etmp, 2.f * kU * jm));
        // The clamps at 1 only act within rounding of za = 2/3.
        if (!(jp < 1.f - ejp && jm < 1.f - ejm)) return false;
        float hx, hy, ehx, ehy;
        if (z > 0.f) {
            hx = 1.f - jm;
            hy = 1.f - jp;
            ehx = ejm + kU;
            ehy = ejp + kU;
            f = ntt;
        } else {
            hx = jp;
            hy = jm;
            ehx = ejp;
            ehy = ejm;
            f = ntt + 8;
        }
        const float HX = hx * fn, HY = hy * fn;
        if (!(floor_cert(HX, fmaf(ehx, fn, kU * fabsf(HX)), ix) &
              floor_cert(HY, fmaf(ehy, fn, kU * fabsf(HY)), iy)))
            return false;
    }
    const bool nest = P == PX_HP_T ? true : (g.nest != 0);
    const long long ip = nside <= 8192 ? (long long)hp_hpd2pix32((int)nside, nest, f, ix, iy)
                                       : hp_hpd2pix(nside, nest, f, ix, iy);
    if (ip < 0 || ip >= g.npix) return false;
    if (P == PX_HP_NT || PARENT) {
        pix[0] = (int)ip;
    } else {
        hp_tile_split(g.nppt, ip, pix[0], pix[1]);
    }
    return true;
}

// The float32 tier for HEALPix (Pixelizor_Healpix::GetPixels): z = sin(lat)
// and s = cos(lat) from __sincosf of the float32 latitude (absolute error
// <= 2^-21.41 for |lat| <= pi), then hp_pixel_f32.  Returns false when the
// sample must go to the double-float path.
template <int P, bool SPIN, bool PARENT>
__device__ __forceinline__ bool mixed_healpix(const DGeom &g, const FastTables &ft,
                                              const MixedConst &mc, const float (&qb)[4],
                                              const float (&qd)[4], int nc, float T, float Pr,
                                              int *pix, float *pf) {
    MixedLonLat o;
    if (!mixed_lonlat(ft, mc, qb, qd, o)) return false;
    float z, s;
    __sincosf(o.lat, &z, &s);
    const float ez = fmaf(fabsf(s), o.elat, 3.8e-7f);
    const float es = fmaf(fabsf(z), o.elat, 3.8e-7f);
    if (!hp_pixel_f32<P, PARENT>(g, o.lon, o.elon, z, ez, s, es, pix)) return false;
    if (SPIN) mixed_spin(o, nc, T, Pr, pf);
    return true;
}

// The float32 tier of one sample for pixelization P: one tap (weight 1)
// when `on`.  False hands the sample to the double-float path.  SPIN =
// false: the pixel only (the caller forms certified spin factors).  PARENT
// (tiled pixelizors): the pixel as a parent-map index -- flat (iy, ix) in
// pix[0..1], HEALPix the NEST index in pix[0] -- instead of a tile tuple.
template <int C, int P, bool SPIN = true, bool PARENT = false>
__device__ __forceinline__ bool mixed_pointing(const DGeom &g, const FastTables &ft,
                                               const MixedConst &mc, const float (&qb)[4],
                                               const float (&qd)[4], int nc, float T, float Pr,
                                               int *pix, bool &on, float *pf) {
    if (P == PX_HP_NT || P == PX_HP_T) {
        on = true;
        return mixed_healpix<P, SPIN, PARENT>(g, ft, mc, qb, qd, nc, T, Pr, pix, pf);
    }
    if (C == SO3G_COORD_CAR)
        return mixed_car<P, SPIN, PARENT>(g, ft, mc, qb, qd, nc, T, Pr, pix, on, pf);
    return mixed_zen<C, P, SPIN, PARENT>(g, mc, qb, qd, nc, T, Pr, pix, on, pf);
}

}  // namespace so3g
