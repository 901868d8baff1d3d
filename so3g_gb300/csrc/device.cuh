// device.cuh -- device-side building blocks of the GB300 ProjectionEngine:
// exact float64 pointing (quaternion compose + projection), the asin/atan2
// interpolation tables, the rectangular and HEALPix pixelizors and the spin
// projection factors.
//
// Every translation unit that includes this file is compiled with
// -fmad=false: no multiply-add is fused, IEEE division and square root are
// used, and each expression below is evaluated in the order written.  That
// order is the one of the reference (so3g src/Projection.cxx, cited per
// function), so coordinates and pixel indices equal the reference's bit for
// bit (HEALPix excepted where CUDA's cos/sin differ from the host libm in
// the last bit; see hp_ang2pix).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/so3g_gb300.h"

namespace so3g {

constexpr int kLutN = 1 << 14;  // TRIG_TABLE_SIZE, src/Projection.cxx:34
constexpr double kPi = 3.141592653589793238462643383279502884197;
constexpr unsigned kFull = 0xffffffffu;

// Pixelizor kinds (template parameter P).
enum { PX_FLAT_NT_NN = 0, PX_FLAT_NT_BL = 1, PX_FLAT_T_NN = 2, PX_FLAT_T_BL = 3,
       PX_HP_NT = 4, PX_HP_T = 5 };

template <int P> struct PixTraits;
template <> struct PixTraits<PX_FLAT_NT_NN> { static constexpr int index_count = 2, taps = 1; };
template <> struct PixTraits<PX_FLAT_NT_BL> { static constexpr int index_count = 2, taps = 4; };
template <> struct PixTraits<PX_FLAT_T_NN>  { static constexpr int index_count = 3, taps = 1; };
template <> struct PixTraits<PX_FLAT_T_BL>  { static constexpr int index_count = 3, taps = 4; };
template <> struct PixTraits<PX_HP_NT>      { static constexpr int index_count = 1, taps = 1; };
template <> struct PixTraits<PX_HP_T>       { static constexpr int index_count = 2, taps = 1; };

// Geometry and map description, passed by value to every kernel.
struct DGeom {
    int ny, nx;              // Flat map
    double cdy, cdx;         // cdelt (y, x)
    double cry, crx;         // crpix (y, x)
    int ty, tx;              // Flat tile shape
    int nty, ntx;            // Flat tile grid
    float inv_ty, inv_tx, inv_ntx;   // their reciprocals (div_small)
    long long nside, npix;   // HEALPix
    long long nppt;          // HEALPix pixels per tile
    int n_tile;              // tiles of the pixelization (0 untiled)
    int nest;
    int ncomp;
    const long long *tile_offset;  // per-tile element offsets (tiled maps)
    int n_tile_map;                // entries of tile_offset
    const double *lut;             // asin table at [0, kLutN), atan2 at [kLutN, 2 kLutN)
};

// ---------------------------------------------------------------------------
// Interpolation tables (include/so_linterp.h:8-71).

__device__ __forceinline__ double lut_raw(const double *v, double x) {
    // LookupTable::get_raw, so_linterp.h:20-29 (dx = 1/(n-1)).
    const double dx = 1. / (kLutN - 1);
    double d = x / dx;
    if (x < 0) return __ldg(v);
    if (!(d < (double)(kLutN - 1))) {        // idx >= n-1 (guard: NaN)
        if (d != d) return d;
        return __ldg(v + kLutN - 1);
    }
    int idx = (int)d;
    d -= idx;
    return __ldg(v + idx) * (1 - d) + __ldg(v + idx + 1) * d;
}

__device__ __forceinline__ double asin_lut(const double *lut, double x) {
    // asinTable::get, so_linterp.h:41-45.
    if (x < 0) return -lut_raw(lut, -x);
    return lut_raw(lut, x);
}

__device__ __forceinline__ double atan2_lut(const double *lut, double y, double x) {
    // atan2Table::get, so_linterp.h:57-70.  The recursion folds y < 0 (odd
    // symmetry) and x < 0 (pi - .) before the octant split; the signs are
    // applied afterwards in the same nesting order.
    const double *v = lut + kLutN;
    bool neg = false, mirror = false;
    if (y < 0) { y = -y; neg = true; }
    if (x < 0) { x = -x; mirror = true; }
    double r;
    if (y == 0) r = __ldg(v);
    else if (x < y) r = kPi / 2 - lut_raw(v, x / y);
    else r = lut_raw(v, y / x);
    if (mirror) r = kPi - r;
    if (neg) r = -r;
    return r;
}

// ---------------------------------------------------------------------------
// Quaternion compose: boost::math::quaternion<double> operator* (Hamilton
// product, each component summed left to right), as used by every
// Pointer<C>::GetCoords (src/Projection.cxx:256, 298, 351, 386, 422, 458, 493).

struct QuatD { double a, b, c, d; };

__device__ __forceinline__ QuatD qmul(const QuatD &p, const QuatD &q) {
    QuatD r;
    r.a = p.a * q.a - p.b * q.b - p.c * q.c - p.d * q.d;
    r.b = p.a * q.b + p.b * q.a + p.c * q.d - p.d * q.c;
    r.c = p.a * q.c - p.b * q.d + p.c * q.a + p.d * q.b;
    r.d = p.a * q.d + p.b * q.c - p.c * q.b + p.d * q.a;
    return r;
}

__device__ __forceinline__ QuatD load_quat(const double *p) {
    double2 lo = __ldg(reinterpret_cast<const double2 *>(p));
    double2 hi = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    return QuatD{lo.x, lo.y, hi.x, hi.y};
}

// Pointer<C>::GetCoords (src/Projection.cxx:238-507).  `q` is the boresight
// quaternion of the sample and `o` the detector offset.
template <int C>
__device__ __forceinline__ void get_coords(const double *lut, const QuatD &qb, const QuatD &o,
                                           double *coords) {
    if (C == SO3G_COORD_FLAT) {
        // :262-276 (boresight and offsets live in a flat 2-d space)
        coords[0] = qb.a + o.a;
        coords[1] = qb.b + o.b;
        coords[2] = qb.c * o.c - qb.d * o.d;
        coords[3] = qb.d * o.c + qb.c * o.d;
        return;
    }
    QuatD q = qmul(qb, o);
    const double a = q.a, b = q.b, c = q.c, d = q.d;
    if (C == SO3G_COORD_QUAT) {
        // :241-257
        coords[0] = a; coords[1] = b; coords[2] = c; coords[3] = d;
    } else if (C == SO3G_COORD_CAR) {
        // :479-507
        const double cos_theta = a * a - b * b - c * c + d * d;
        const double half_sin_theta = 0.5 * sqrt(1 - cos_theta * cos_theta);
        coords[0] = atan2_lut(lut, c * d - a * b, c * a + d * b);
        coords[1] = asin_lut(lut, cos_theta);
        coords[2] = (a * c - b * d) / half_sin_theta;
        coords[3] = (c * d + a * b) / half_sin_theta;
    } else if (C == SO3G_COORD_CEA) {
        // :444-472 (uses the math-library atan2, not the table)
        const double cos_theta = a * a - b * b - c * c + d * d;
        const double half_sin_theta = 0.5 * sqrt(1 - cos_theta * cos_theta);
        coords[0] = atan2(c * d - a * b, c * a + d * b);
        coords[1] = cos_theta;
        coords[2] = (a * c - b * d) / half_sin_theta;
        coords[3] = (c * d + a * b) / half_sin_theta;
    } else if (C == SO3G_COORD_ARC) {
        // :284-326
        const double cos_theta2_sq = a * a + d * d;
        const double sin_theta2_sq = b * b + c * c;
        const double sc = c * a + d * b;
        const double ss = a * b - c * d;
        const double half_sin_theta = sqrt(sc * sc + ss * ss);
        double R_factor;
        if (half_sin_theta < 1e-8)
            R_factor = 2 + 1.33333333333 * half_sin_theta * half_sin_theta;
        else
            R_factor = asin_lut(lut, half_sin_theta * 2) / half_sin_theta;
        if (cos_theta2_sq < sin_theta2_sq)
            R_factor = kPi / half_sin_theta - R_factor;
        coords[0] = ss * R_factor;
        coords[1] = sc * R_factor;
        coords[2] = (a * a - d * d) / cos_theta2_sq;
        coords[3] = (2 * a * d) / cos_theta2_sq;
    } else if (C == SO3G_COORD_SIN) {
        // :337-364
        const double cos_theta2_sq = a * a + d * d;
        coords[0] = 2 * (a * b - c * d);
        coords[1] = 2 * (c * a + d * b);
        coords[2] = (a * a - d * d) / cos_theta2_sq;
        coords[3] = (2 * a * d) / cos_theta2_sq;
    } else if (C == SO3G_COORD_TAN) {
        // :372-400
        const double cos_theta2_sq = a * a + d * d;
        const double cos_theta = 2 * cos_theta2_sq - 1;
        coords[0] = (a * b - c * d) * 2 / cos_theta;
        coords[1] = (a * c + b * d) * 2 / cos_theta;
        coords[2] = (a * a - d * d) / cos_theta2_sq;
        coords[3] = (2 * a * d) / cos_theta2_sq;
    } else {  // ZEA, :408-437
        const double cos_theta2_sq = a * a + d * d;
        const double cos_theta2 = sqrt(cos_theta2_sq);
        coords[0] = (a * b - c * d) * 2 / cos_theta2;
        coords[1] = (a * c + b * d) * 2 / cos_theta2;
        coords[2] = (a * a - d * d) / cos_theta2_sq;
        coords[3] = (2 * a * d) / cos_theta2_sq;
    }
}

// ---------------------------------------------------------------------------
// HEALPix ang2ring / ang2nest: the published HEALPix "bare" algorithm the
// reference compiles in (src/healpix_bare.c:46-78, 109-114, 152-211,
// 271-275, 303-306), restated for the device.  cos/sin come from CUDA's
// double sincos, which may differ from the host libm in the last bit; a
// pixel index can change only when the sample lies within ~1e-16 of a
// pixel boundary.

__device__ __forceinline__ int hp_jrll(int f) { return 2 + (f >> 2); }
__device__ __forceinline__ int hp_jpll(int f) {
    // {1,3,5,7, 0,2,4,6, 1,3,5,7}
    return ((f & 3) << 1) + ((f >> 2) == 1 ? 0 : 1);
}

__device__ __forceinline__ long long hp_spread_bits(long long v) {
    long long r = v & 0xffffffffLL;
    r = (r ^ (r << 16)) & 0x0000ffff0000ffffLL;
    r = (r ^ (r << 8)) & 0x00ff00ff00ff00ffLL;
    r = (r ^ (r << 4)) & 0x0f0f0f0f0f0f0f0fLL;
    r = (r ^ (r << 2)) & 0x3333333333333333LL;
    r = (r ^ (r << 1)) & 0x5555555555555555LL;
    return r;
}

// hpd2nest / hpd2ring (src/healpix_bare.c:109-114, 152-211): the pixel of
// face f, in-face coordinates (ix, iy).
__device__ __forceinline__ long long hp_hpd2pix(long long nside, bool nest, int f, long long ix,
                                               long long iy) {
    if (nest)  // hpd2nest
        return (f * nside * nside) + hp_spread_bits(ix) + (hp_spread_bits(iy) << 1);
    // hpd2ring
    long long nl4 = 4 * nside;
    long long jr = (hp_jrll(f) * nside) - ix - iy - 1;
    if (jr < nside) {
        long long jp = (hp_jpll(f) * jr + ix - iy + 1) / 2;
        jp = (jp > nl4) ? jp - nl4 : ((jp < 1) ? jp + nl4 : jp);
        return 2 * jr * (jr - 1) + jp - 1;
    } else if (jr > 3 * nside) {
        jr = nl4 - jr;
        long long jp = (hp_jpll(f) * jr + ix - iy + 1) / 2;
        jp = (jp > nl4) ? jp - nl4 : ((jp < 1) ? jp + nl4 : jp);
        return 12 * nside * nside - 2 * (jr + 1) * jr + jp - 1;
    } else {
        long long jp = (hp_jpll(f) * nside + ix - iy + 1 + ((jr - nside) & 1)) / 2;
        jp = (jp > nl4) ? jp - nl4 : ((jp < 1) ? jp + nl4 : jp);
        return 2 * nside * (nside - 1) + (jr - nside) * nl4 + jp - 1;
    }
}

// hp_hpd2pix in 32-bit integers, for nside <= 8192 (every index, and
// 2 jr (jr - 1) for jr <= 4 nside, below 2^31): the same steps.
__device__ __forceinline__ int hp_spread_bits32(int v) {
    unsigned r = (unsigned)v & 0xffffu;
    r = (r ^ (r << 8)) & 0x00ff00ffu;
    r = (r ^ (r << 4)) & 0x0f0f0f0fu;
    r = (r ^ (r << 2)) & 0x33333333u;
    r = (r ^ (r << 1)) & 0x55555555u;
    return (int)r;
}

__device__ __forceinline__ int hp_hpd2pix32(int nside, bool nest, int f, int ix, int iy) {
    if (nest) return f * nside * nside + hp_spread_bits32(ix) + (hp_spread_bits32(iy) << 1);
    const int nl4 = 4 * nside;
    int jr = hp_jrll(f) * nside - ix - iy - 1;
    if (jr < nside) {
        int jp = (hp_jpll(f) * jr + ix - iy + 1) / 2;
        jp = (jp > nl4) ? jp - nl4 : ((jp < 1) ? jp + nl4 : jp);
        return 2 * jr * (jr - 1) + jp - 1;
    } else if (jr > 3 * nside) {
        jr = nl4 - jr;
        int jp = (hp_jpll(f) * jr + ix - iy + 1) / 2;
        jp = (jp > nl4) ? jp - nl4 : ((jp < 1) ? jp + nl4 : jp);
        return 12 * nside * nside - 2 * (jr + 1) * jr + jp - 1;
    } else {
        int jp = (hp_jpll(f) * nside + ix - iy + 1 + ((jr - nside) & 1)) / 2;
        jp = (jp > nl4) ? jp - nl4 : ((jp < 1) ? jp + nl4 : jp);
        return 2 * nside * (nside - 1) + (jr - nside) * nl4 + jp - 1;
    }
}

// Returns the pixel, or -1 for a NaN/inf angle (the reference converts NaN
// to an integer there, which is undefined).
__device__ __forceinline__ long long hp_ang2pix(long long nside, bool nest, double theta,
                                                double phi) {
    double sth, cth;
    sincos(theta, &sth, &cth);
    if (sth < 0) { sth = -sth; phi += kPi; }
    if (!(cth == cth) || !(sth == sth) || !(fabs(phi) < 1e300)) return -1;
    // loc2hpc
    const double z = cth, s = sth;
    double za = fabs(z);
    double x = phi * (1. / (2. * kPi));
    if (x < 0.)
        x += (long long)x + 1.;
    else if (x >= 1.)
        x -= (long long)x;
    double tt = 4. * x;
    double hx, hy;
    int f;
    if (za <= 2. / 3.) {
        double temp1 = 0.5 + tt;
        double temp2 = z * 0.75;
        double jp = temp1 - temp2;
        double jm = temp1 + temp2;
        int ifp = (int)jp;
        int ifm = (int)jm;
        hx = jm - ifm;
        hy = 1 + ifp - jp;
        f = (ifp == ifm) ? (ifp | 4) : ((ifp < ifm) ? ifp : (ifm + 8));
    } else {
        long long ntt = (long long)tt;
        if (ntt >= 4) ntt = 3;
        double tp = tt - ntt;
        double tmp = s / sqrt((1. + za) * (1. / 3.));
        double jp = tp * tmp;
        double jm = (1.0 - tp) * tmp;
        if (jp > 1.) jp = 1.;
        if (jm > 1.) jm = 1.;
        if (z >= 0) { hx = 1. - jm; hy = 1. - jp; f = (int)ntt; }
        else        { hx = jp;      hy = jm;      f = (int)ntt + 8; }
    }
    // loc2hpd
    long long ix = (long long)(hx * nside), iy = (long long)(hy * nside);
    return hp_hpd2pix(nside, nest, f, ix, iy);
}

// x / d for 0 <= x < 2^24 and 1 <= d < 2^24 from inv_d = 1/d rounded to
// float32: x * inv_d is within one of the quotient (relative error below
// 2^-23, and exact for d = 1), which one remainder test corrects -- a few
// instructions instead of an integer division.
__device__ __forceinline__ int div_small(int x, int d, float inv_d) {
    if (x >= (1 << 24)) return x / d;
    int q = __float2int_rz(__int2float_rn(x) * inv_d);
    const int r = x - q * d;
    q += (r >= d) - (r < 0);
    return q;
}

// Tile tuple (tile, row and column in the tile) of parent-map pixel
// (iy, ix) >= 0 of a flat tiled pixelizor (:1029-1051, :1124-1138).
__device__ __forceinline__ void flat_tile_tuple(const DGeom &g, int iy, int ix, int *t) {
    const int sub_y = div_small(iy, g.ty, g.inv_ty), sub_x = div_small(ix, g.tx, g.inv_tx);
    t[0] = sub_y * g.ntx + sub_x;
    t[1] = iy - sub_y * g.ty;
    t[2] = ix - sub_x * g.tx;
}

// Tile and in-tile index of a HEALPix NEST pixel ip >= 0 with nppt pixels
// per tile: a power of 4 for the power-of-2 nside and nside_tile the
// pixelizor accepts, split with a shift and a mask instead of a 64-bit
// division; a division otherwise.
__device__ __forceinline__ void hp_tile_split(long long nppt, long long ip, int &tile, int &sub) {
    if ((nppt & (nppt - 1)) == 0) {
        const int s = __ffsll(nppt) - 1;
        tile = (int)(ip >> s);
        sub = (int)(ip & (nppt - 1));
    } else {
        tile = (int)(ip / nppt);
        sub = (int)(ip - (long long)tile * nppt);
    }
}

// ---------------------------------------------------------------------------
// Pixelizors.  get_pixel() is GetPixel (used by pixels/pointing_matrix:
// writes only the slots it sets); get_pixels() is GetPixels (interpolation
// taps, returns their count).

// get_pixel() returns false when it set only slot 0 (to -1): the other
// slots then keep the values of the previous sample, as in the reference.
template <int P>
__device__ __forceinline__ bool get_pixel(const DGeom &g, const double *coords, int *idx) {
    if (P == PX_HP_NT || P == PX_HP_T) {
        // Pixelizor_Healpix::GetPixel, src/Projection.cxx:557-564, 703-712
        double phi = coords[0];
        double theta = kPi / 2 - coords[1];
        long long ix = hp_ang2pix(g.nside, P == PX_HP_T ? true : (g.nest != 0), theta, phi);
        if (P == PX_HP_NT) {
            idx[0] = (int)ix;
            return true;
        }
        if (ix < 0) { idx[0] = -1; return false; }
        hp_tile_split(g.nppt, ix, idx[0], idx[1]);
        return true;
    }
    // Pixelizor2_Flat<NonTiled>::GetPixel :845-863 / <Tiled> :1029-1051
    double ix = coords[0] / g.cdx + g.crx - 1 + 0.5;
    if (!(ix >= 0 && ix < g.nx)) { idx[0] = -1; return false; }   // guard: NaN
    double iy = coords[1] / g.cdy + g.cry - 1 + 0.5;
    if (!(iy >= 0 && iy < g.ny)) { idx[0] = -1; return false; }
    if (P == PX_FLAT_NT_NN || P == PX_FLAT_NT_BL) {
        idx[0] = int(iy);
        idx[1] = int(ix);
    } else {
        flat_tile_tuple(g, int(iy), int(ix), idx);
    }
    return true;
}

template <int P>
__device__ __forceinline__ int get_pixels(const DGeom &g, const double *coords, int (*pix)[3],
                                          float *w) {
    if (P == PX_HP_NT || P == PX_HP_T) {
        // Pixelizor_Healpix::GetPixels, :565-574, :713-724
        double phi = coords[0];
        double theta = kPi / 2 - coords[1];
        long long ix = hp_ang2pix(g.nside, P == PX_HP_T ? true : (g.nest != 0), theta, phi);
        // guard: the HEALPix arithmetic is only defined for phi > -2 pi
        if (ix < 0 || ix >= g.npix) return 0;
        if (P == PX_HP_NT) {
            pix[0][0] = (int)ix;
        } else {
            hp_tile_split(g.nppt, ix, pix[0][0], pix[0][1]);
        }
        w[0] = 1;
        return 1;
    }
    double x = coords[0] / g.cdx + g.crx - 1 + 0.5;
    double y = coords[1] / g.cdy + g.cry - 1 + 0.5;
    if (P == PX_FLAT_NT_NN) {
        // :912-926
        if (!(x >= 0 && x < g.nx)) return 0;
        if (!(y >= 0 && y < g.ny)) return 0;
        pix[0][0] = int(y) - int(y < 0);
        pix[0][1] = int(x) - int(x < 0);
        w[0] = 1;
        return 1;
    } else if (P == PX_FLAT_T_NN) {
        // :1124-1138 -- int() truncation before the bounds test, so
        // x in (-1, 0) lands in column 0.
        if (!(x > -1 && x < g.nx)) return 0;
        if (!(y > -1 && y < g.ny)) return 0;
        int ix = int(x), iy = int(y);
        flat_tile_tuple(g, iy, ix, pix[0]);
        w[0] = 1;
        return 1;
    } else {
        // Bilinear, :930-952 (NonTiled, floor) and :1141-1166 (Tiled, int()).
        if (!(x > -4 && x < g.nx + 4 && y > -4 && y < g.ny + 4)) return 0;  // guard
        int x1, y1;
        if (P == PX_FLAT_NT_BL) {
            x1 = int(x) - int(x < 0);
            y1 = int(y) - int(y < 0);
        } else {
            x1 = int(x);
            y1 = int(y);
        }
        double wx[2] = {x - x1, 1 - (x - x1)};
        double wy[2] = {y - y1, 1 - (y - y1)};
        int iout = 0;
#pragma unroll
        for (int dy = 0; dy < 2; dy++) {
            int iy = y1 + dy;
            if (iy < 0 || iy >= g.ny) continue;
#pragma unroll
            for (int dx = 0; dx < 2; dx++) {
                int ix = x1 + dx;
                if (ix < 0 || ix >= g.nx) continue;
                if (P == PX_FLAT_NT_BL) {
                    pix[iout][0] = iy;
                    pix[iout][1] = ix;
                } else {
                    flat_tile_tuple(g, iy, ix, pix[iout]);
                }
                w[iout] = wy[dy] * wx[dx];
                iout++;
            }
        }
        return iout;
    }
}

// Element offset of a tap's pixel in the map and the size of one component
// plane (the pix()/wpix() accessors, :590-600, :755-774, :881-893,
// :1084-1105).  Returns the tile index (>= 0) if the tile is absent, else -1.
template <int P>
__device__ __forceinline__ int locate(const DGeom &g, const int *idx, long long *off,
                                      long long *plane) {
    if (P == PX_FLAT_NT_NN || P == PX_FLAT_NT_BL) {
        *off = (long long)idx[0] * g.nx + idx[1];
        *plane = (long long)g.ny * g.nx;
        return -1;
    } else if (P == PX_HP_NT) {
        *off = idx[0];
        *plane = g.npix;
        return -1;
    } else {
        int t = idx[0];
        long long toff = (t >= 0 && t < g.n_tile_map) ? __ldg(g.tile_offset + t) : -1;
        if (toff < 0) return t < 0 ? 0x7fffffff : t;
        if (P == PX_HP_T) {
            *off = toff + idx[1];
            *plane = g.nppt;
        } else {
            const int row = div_small(t, g.ntx, g.inv_ntx), col = t - row * g.ntx;
            long long tny = min(g.ty, g.ny - row * g.ty);
            long long tnx = min(g.tx, g.nx - col * g.tx);
            *off = toff + idx[1] * tnx + idx[2];
            *plane = tny * tnx;
        }
        return -1;
    }
}

// stripe() of the pixelizors (:601-603, :776-780, :894-898, :1106-1108).
template <int P>
__device__ __forceinline__ long long stripe(const DGeom &g, const int *idx, int n) {
    if (P == PX_FLAT_NT_NN || P == PX_FLAT_NT_BL) {
        if (idx[0] < 0) return -1;
        return (long long)idx[1] * n / g.nx;
    } else if (P == PX_FLAT_T_NN || P == PX_FLAT_T_BL) {
        return idx[0] % n;
    } else if (P == PX_HP_NT) {
        return (long long)idx[0] * n / g.npix;
    } else {
        long long ipix = (long long)idx[0] * g.nppt + idx[1];
        return ipix * n / (g.nppt * g.n_tile);
    }
}

// spin_proj_factors<S>, src/Projection.cxx:1180-1209: computed in float64,
// stored as float32.
__device__ __forceinline__ void spin_factors(int nc, const double *coords, float T, float P,
                                             float *pf) {
    if (nc == 1) {
        pf[0] = T;
        pf[1] = 0.f;
        pf[2] = 0.f;
    } else {
        const double c = coords[2], s = coords[3];
        float f1 = P * (c * c - s * s);
        float f2 = P * (2 * c * s);
        if (nc == 2) { pf[0] = f1; pf[1] = f2; pf[2] = 0.f; }
        else { pf[0] = T; pf[1] = f1; pf[2] = f2; }
    }
}

// ---------------------------------------------------------------------------
// Device error record (4 x int32): see enum so3g_device_error.

__device__ __forceinline__ void record_missing_tile(int *err, int tile) {
    if (!err) return;
    int old = atomicCAS(err, 0, SO3G_DEVERR_MISSING_TILE);
    if (old == 0 || old == SO3G_DEVERR_MISSING_TILE)
        atomicMax(err + 1, 0x7fffffff - tile);  // decoded as the smallest tile
}

__device__ __forceinline__ void record_pixel_range(int *err, int tile, int det, int t) {
    if (!err) return;
    int old = atomicCAS(err, 0, SO3G_DEVERR_PIXEL_RANGE);
    if (old == 0) {
        err[1] = tile;
        err[2] = det;
        err[3] = t;
    }
}

// float -> double by integer operations: exact, and no float64-pipe
// instruction (GB300 runs float<->double conversions on its slow float64
// pipe, at ~0.7 per clock per SM).
static __device__ __noinline__ double f2d_special(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned s = u & 0x80000000u, ef = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    // Subnormal floats: normalise the mantissa (leading one at bit p).
    const int p = 31 - __clz(m | 1u);
    const unsigned mn = (m << (23 - p)) & 0x7fffffu;
    unsigned ed, mant;
    if (ef == 0u) {
        ed = m ? (unsigned)(p - 149 + 1023) : 0u;
        mant = m ? mn : 0u;
    } else if (ef == 255u) {
        ed = 2047u;
        mant = m;
    } else {
        ed = ef - 127u + 1023u;
        mant = m;
    }
    const unsigned hw = s | (ed << 20) | (mant >> 3), lw = mant << 29;
    return __hiloint2double((int)hw, (int)lw);
}

// float -> double with integer instructions only; normal floats take the
// short path (rebias the exponent, move the significand), zeros keep their
// sign, and subnormals, infinities and NaNs go through f2d_special.
__device__ __forceinline__ double f2d(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned a = u & 0x7fffffffu;
    if (a - 0x00800000u < 0x7f000000u)
        return __hiloint2double((int)((u & 0x80000000u) | ((a >> 3) + (896u << 20))),
                                (int)(u << 29));
    if (a == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
    return f2d_special(f);
}

// Compensated float32 addition (Knuth's TwoSum): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// A warp with at least this many runs adds its terms with one atomic each:
// its atomics already spread over many addresses, and the reduction would
// cost more issue slots than the atomics it saves.
constexpr int kDirectRuns = 4;

// Sums the values of each run of equal keys across the warp (lanes in
// order) and adds the run totals to map[key + mult[k] * plane] from the
// run's first lane.  Keys < 0 are not flushed.  All 32 lanes must call.
template <int NV, int DIRECT_RUNS = kDirectRuns>
__device__ __forceinline__ void flush_runs(long long key, long long plane, float (&v)[NV],
                                           const int (&mult)[NV], unsigned vmask, double *map) {
    const int lane = threadIdx.x & 31;
    long long prev = __shfl_up_sync(kFull, key, 1);
    bool head = (lane == 0) || (key != prev);
    unsigned heads = __ballot_sync(kFull, head);
    if (__popc(heads) >= DIRECT_RUNS) {
        if (key >= 0) {
#pragma unroll
            for (int k = 0; k < NV; k++)
                if ((vmask >> k) & 1u) atomicAdd(map + key + mult[k] * plane, f2d(v[k]));
        }
        return;
    }
    unsigned after = heads & ~((2u << lane) - 1u);
    int end = after ? (__ffs(after) - 1) : 32;
    int span = head ? end - lane : 1;
    int maxrun = __reduce_max_sync(kFull, (unsigned)span);
    float e[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) e[k] = 0.f;
    for (int d = 1; d < maxrun; d <<= 1) {
        const bool take = lane + d < end;
#pragma unroll
        for (int k = 0; k < NV; k++) {
            if (!((vmask >> k) & 1u)) continue;
            float os = __shfl_down_sync(kFull, v[k], d);
            float oe = __shfl_down_sync(kFull, e[k], d);
            if (take) {
                float s, r;
                two_sum(v[k], os, s, r);
                v[k] = s;
                e[k] += oe + r;
            }
        }
    }
    if (head && key >= 0) {
#pragma unroll
        for (int k = 0; k < NV; k++)
            if ((vmask >> k) & 1u) atomicAdd(map + key + mult[k] * plane, f2d(v[k]) + f2d(e[k]));
    }
}

// Sample-range work decomposition shared by the projection kernels: block
// (x, y) covers piece y of segment x, `piece` samples long.
struct Segs {
    const int *seg;   // (det, start, end) triples, or NULL
    int n_time;       // used when seg == NULL: segment x = detector x
};

__device__ __forceinline__ bool seg_piece(const Segs &s, int piece, int &det, int &t0, int &t1) {
    int b = blockIdx.x;
    int s0, s1;
    if (s.seg) {
        det = __ldg(s.seg + 3 * b);
        s0 = __ldg(s.seg + 3 * b + 1);
        s1 = __ldg(s.seg + 3 * b + 2);
    } else {
        det = b;
        s0 = 0;
        s1 = s.n_time;
    }
    long long p0 = (long long)s0 + (long long)blockIdx.y * piece;
    if (p0 >= s1) return false;
    t0 = (int)p0;
    t1 = (int)min((long long)s1, p0 + piece);
    return true;
}

}  // namespace so3g
