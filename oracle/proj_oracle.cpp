// proj_oracle.cpp -- CPU oracle (test infrastructure) for the so3g
// ProjectionEngine hot path.  See proj_oracle.h.
//
// Every function restates the reference arithmetic in the same operation
// order (each line cites the so3g source it follows).  Nothing here is
// optimised beyond what the reference does: templates over the coordinate
// system, pixelizor and spin count, as the reference's ProjectionEngine
// template (include/Projection.h:40-66), and OpenMP where the reference
// uses it.  Differences from the reference are limited to inputs for which
// the reference has undefined behaviour (NaN or out-of-range float->int
// conversions, out-of-range tile or pixel indices); those are marked
// "guard" below and turn into "no pixel" or an error record.

#include "proj_oracle.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kPi = 3.141592653589793238462643383279502884197;  // M_PI
constexpr int kTableSize = 1 << 14;  // TRIG_TABLE_SIZE, src/Projection.cxx:34

thread_local std::string g_err;

int fail(const std::string &msg) {
    g_err = msg;
    return SO3G_ERR_ARGUMENT;
}

// ---------------------------------------------------------------------------
// Linear-interpolation trig tables (include/so_linterp.h:8-71).

struct Lut {
    int n = 0;
    double dx = 0.;
    std::vector<double> v;
};
Lut g_asin, g_atan2;
bool g_ready = false;

// LookupTable::get_raw, so_linterp.h:20-29.
inline double lut_raw(const Lut &t, double x) {
    double d = x / t.dx;
    if (x < 0) return t.v[0];
    if (!(d < (double)(t.n - 1))) {          // guard: NaN and huge d
        if (d != d) return d;
        return t.v[t.n - 1];
    }
    int idx = (int)d;                        // idx >= n-1 handled above
    d -= idx;
    return t.v[idx] * (1 - d) + t.v[idx + 1] * d;
}

// asinTable::get, so_linterp.h:41-45.
inline double asin_lut(double x) {
    if (x < 0) return -lut_raw(g_asin, -x);
    return lut_raw(g_asin, x);
}

// atan2Table::get, so_linterp.h:57-70 (recursion unrolled: each level
// applies one fold, in the same order).
inline double atan2_lut(double y, double x) {
    if (y < 0) return -atan2_lut(-y, x);
    if (x < 0) return kPi - atan2_lut(y, -x);
    if (y == 0) return g_atan2.v[0];
    if (x < y) return kPi / 2 - lut_raw(g_atan2, x / y);
    return lut_raw(g_atan2, y / x);
}

void build_tables() {
    // asinTable(n), so_linterp.h:35-39; atan2Table(n), so_linterp.h:51-56.
    g_asin.n = kTableSize;
    g_asin.dx = 1. / (kTableSize - 1);
    g_asin.v.resize(kTableSize);
    for (int i = 0; i < kTableSize; i++) g_asin.v[i] = std::asin(i * g_asin.dx);
    g_atan2.n = kTableSize;
    g_atan2.dx = 1. / (kTableSize - 1);
    g_atan2.v.resize(kTableSize);
    for (int i = 0; i < kTableSize; i++) g_atan2.v[i] = std::atan2(i * g_atan2.dx, 1.);
    g_ready = true;
}

// ---------------------------------------------------------------------------
// Quaternion product: boost::math::quaternion<double> operator* (boost
// 1.87), used at src/Projection.cxx:256,298,351,386,422,458,493.  Hamilton
// product, each component summed left to right.

struct Quat { double a, b, c, d; };

inline Quat qmul(const Quat &p, const Quat &q) {
    Quat r;
    r.a = p.a * q.a - p.b * q.b - p.c * q.c - p.d * q.d;
    r.b = p.a * q.b + p.b * q.a + p.c * q.d - p.d * q.c;
    r.c = p.a * q.c - p.b * q.d + p.c * q.a + p.d * q.b;
    r.d = p.a * q.d + p.b * q.c - p.c * q.b + p.d * q.a;
    return r;
}

// ---------------------------------------------------------------------------
// Pointer<C>::GetCoords, src/Projection.cxx:241-507.

template <int C>
inline void get_coords(const double *bt, const double *dofs, double *coords);

template <> inline void get_coords<SO3G_COORD_QUAT>(const double *bt, const double *dofs, double *coords) {
    // :241-257
    Quat q = qmul(Quat{bt[0], bt[1], bt[2], bt[3]}, Quat{dofs[0], dofs[1], dofs[2], dofs[3]});
    coords[0] = q.a; coords[1] = q.b; coords[2] = q.c; coords[3] = q.d;
}

template <> inline void get_coords<SO3G_COORD_FLAT>(const double *bt, const double *dofs, double *coords) {
    // :262-276
    for (int ic = 0; ic < 4; ic++) coords[ic] = bt[ic];
    coords[0] += dofs[0];
    coords[1] += dofs[1];
    const double c2 = coords[2];
    coords[2] = coords[2] * dofs[2] - coords[3] * dofs[3];
    coords[3] = coords[3] * dofs[2] + c2 * dofs[3];
}

template <> inline void get_coords<SO3G_COORD_ARC>(const double *bt, const double *dofs, double *coords) {
    // :284-326
    Quat q = qmul(Quat{bt[0], bt[1], bt[2], bt[3]}, Quat{dofs[0], dofs[1], dofs[2], dofs[3]});
    const double a = q.a, b = q.b, c = q.c, d = q.d;
    const double cos_theta2_sq = a * a + d * d;
    const double sin_theta2_sq = b * b + c * c;
    const double sc = c * a + d * b;
    const double ss = a * b - c * d;
    const double half_sin_theta = std::sqrt(sc * sc + ss * ss);
    double R_factor;
    if (half_sin_theta < 1e-8)
        R_factor = 2 + 1.33333333333 * half_sin_theta * half_sin_theta;
    else
        R_factor = asin_lut(half_sin_theta * 2) / half_sin_theta;
    if (cos_theta2_sq < sin_theta2_sq)
        R_factor = kPi / half_sin_theta - R_factor;
    coords[0] = ss * R_factor;
    coords[1] = sc * R_factor;
    coords[2] = (a * a - d * d) / cos_theta2_sq;
    coords[3] = (2 * a * d) / cos_theta2_sq;
}

template <> inline void get_coords<SO3G_COORD_SIN>(const double *bt, const double *dofs, double *coords) {
    // :337-364
    Quat q = qmul(Quat{bt[0], bt[1], bt[2], bt[3]}, Quat{dofs[0], dofs[1], dofs[2], dofs[3]});
    const double a = q.a, b = q.b, c = q.c, d = q.d;
    const double cos_theta2_sq = a * a + d * d;
    coords[0] = 2 * (a * b - c * d);
    coords[1] = 2 * (c * a + d * b);
    coords[2] = (a * a - d * d) / cos_theta2_sq;
    coords[3] = (2 * a * d) / cos_theta2_sq;
}

template <> inline void get_coords<SO3G_COORD_TAN>(const double *bt, const double *dofs, double *coords) {
    // :372-400
    Quat q = qmul(Quat{bt[0], bt[1], bt[2], bt[3]}, Quat{dofs[0], dofs[1], dofs[2], dofs[3]});
    const double a = q.a, b = q.b, c = q.c, d = q.d;
    const double cos_theta2_sq = a * a + d * d;
    const double cos_theta = 2 * cos_theta2_sq - 1;
    coords[0] = (a * b - c * d) * 2 / cos_theta;
    coords[1] = (a * c + b * d) * 2 / cos_theta;
    coords[2] = (a * a - d * d) / cos_theta2_sq;
    coords[3] = (2 * a * d) / cos_theta2_sq;
}

template <> inline void get_coords<SO3G_COORD_ZEA>(const double *bt, const double *dofs, double *coords) {
    // :408-437
    Quat q = qmul(Quat{bt[0], bt[1], bt[2], bt[3]}, Quat{dofs[0], dofs[1], dofs[2], dofs[3]});
    const double a = q.a, b = q.b, c = q.c, d = q.d;
    const double cos_theta2_sq = a * a + d * d;
    const double cos_theta2 = std::sqrt(cos_theta2_sq);
    coords[0] = (a * b - c * d) * 2 / cos_theta2;
    coords[1] = (a * c + b * d) * 2 / cos_theta2;
    coords[2] = (a * a - d * d) / cos_theta2_sq;
    coords[3] = (2 * a * d) / cos_theta2_sq;
}

template <> inline void get_coords<SO3G_COORD_CEA>(const double *bt, const double *dofs, double *coords) {
    // :444-472 (libm atan2, not the table)
    Quat q = qmul(Quat{bt[0], bt[1], bt[2], bt[3]}, Quat{dofs[0], dofs[1], dofs[2], dofs[3]});
    const double a = q.a, b = q.b, c = q.c, d = q.d;
    const double cos_theta = a * a - b * b - c * c + d * d;
    const double half_sin_theta = 0.5 * std::sqrt(1 - cos_theta * cos_theta);
    coords[0] = std::atan2(c * d - a * b, c * a + d * b);
    coords[1] = cos_theta;
    coords[2] = (a * c - b * d) / half_sin_theta;
    coords[3] = (c * d + a * b) / half_sin_theta;
}

template <> inline void get_coords<SO3G_COORD_CAR>(const double *bt, const double *dofs, double *coords) {
    // :479-507
    Quat q = qmul(Quat{bt[0], bt[1], bt[2], bt[3]}, Quat{dofs[0], dofs[1], dofs[2], dofs[3]});
    const double a = q.a, b = q.b, c = q.c, d = q.d;
    const double cos_theta = a * a - b * b - c * c + d * d;
    const double half_sin_theta = 0.5 * std::sqrt(1 - cos_theta * cos_theta);
    coords[0] = atan2_lut(c * d - a * b, c * a + d * b);
    coords[1] = asin_lut(cos_theta);
    coords[2] = (a * c - b * d) / half_sin_theta;
    coords[3] = (c * d + a * b) / half_sin_theta;
}

// ---------------------------------------------------------------------------
// HEALPix ang2ring / ang2nest: the published HEALPix "bare" algorithm as
// compiled into the reference (src/healpix_bare.c:46-78 loc2hpc, 109-114
// ang2loc, 152-161 spread_bits, 178-179 hpd2nest, 187-211 hpd2ring,
// 271-275 loc2hpd, 303-306 ang2ring/ang2nest).

const int kJrll[12] = {2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4};
const int kJpll[12] = {1, 3, 5, 7, 0, 2, 4, 6, 1, 3, 5, 7};

struct HpCont { double x, y; int32_t f; };

inline HpCont hp_loc_to_face(double z, double s, double phi) {
    double za = std::fabs(z);
    double x = phi * (1. / (2. * kPi));
    if (x < 0.)
        x += (int64_t)x + 1.;
    else if (x >= 1.)
        x -= (int64_t)x;
    double tt = 4. * x;
    if (za <= 2. / 3.) {
        double temp1 = 0.5 + tt;
        double temp2 = z * 0.75;
        double jp = temp1 - temp2;
        double jm = temp1 + temp2;
        int ifp = (int)jp;
        int ifm = (int)jm;
        HpCont r;
        r.x = jm - ifm;
        r.y = 1 + ifp - jp;
        r.f = (ifp == ifm) ? (ifp | 4) : ((ifp < ifm) ? ifp : (ifm + 8));
        return r;
    }
    int64_t ntt = (int64_t)tt;
    if (ntt >= 4) ntt = 3;
    double tp = tt - ntt;
    double tmp = s / std::sqrt((1. + za) * (1. / 3.));
    double jp = tp * tmp;
    double jm = (1.0 - tp) * tmp;
    if (jp > 1.) jp = 1.;
    if (jm > 1.) jm = 1.;
    HpCont r;
    if (z >= 0) { r.x = 1. - jm; r.y = 1. - jp; r.f = (int32_t)ntt; }
    else        { r.x = jp;      r.y = jm;      r.f = (int32_t)ntt + 8; }
    return r;
}

inline int64_t hp_spread_bits(int64_t v) {
    int64_t r = v & 0xffffffff;
    r = (r ^ (r << 16)) & 0x0000ffff0000ffff;
    r = (r ^ (r << 8)) & 0x00ff00ff00ff00ff;
    r = (r ^ (r << 4)) & 0x0f0f0f0f0f0f0f0f;
    r = (r ^ (r << 2)) & 0x3333333333333333;
    r = (r ^ (r << 1)) & 0x5555555555555555;
    return r;
}

inline int64_t hp_face_to_nest(int64_t nside, int64_t ix, int64_t iy, int32_t f) {
    return (f * nside * nside) + hp_spread_bits(ix) + (hp_spread_bits(iy) << 1);
}

inline int64_t hp_face_to_ring(int64_t nside, int64_t ix, int64_t iy, int32_t f) {
    if (f < 0 || f > 11) return -1;   // guard: only reached for phi <= -2 pi
    int64_t nl4 = 4 * nside;
    int64_t jr = (kJrll[f] * nside) - ix - iy - 1;
    if (jr < nside) {
        int64_t jp = (kJpll[f] * jr + ix - iy + 1) / 2;
        jp = (jp > nl4) ? jp - nl4 : ((jp < 1) ? jp + nl4 : jp);
        return 2 * jr * (jr - 1) + jp - 1;
    } else if (jr > 3 * nside) {
        jr = nl4 - jr;
        int64_t jp = (kJpll[f] * jr + ix - iy + 1) / 2;
        jp = (jp > nl4) ? jp - nl4 : ((jp < 1) ? jp + nl4 : jp);
        return 12 * nside * nside - 2 * (jr + 1) * jr + jp - 1;
    } else {
        int64_t jp = (kJpll[f] * nside + ix - iy + 1 + ((jr - nside) & 1)) / 2;
        jp = (jp > nl4) ? jp - nl4 : ((jp < 1) ? jp + nl4 : jp);
        return 2 * nside * (nside - 1) + (jr - nside) * nl4 + jp - 1;
    }
}

// ang2nest / ang2ring with t_ang {theta, phi}.  Returns -1 for a NaN angle
// (guard: the reference converts NaN to int64).
inline int64_t hp_ang2pix(int64_t nside, bool nest, double theta, double phi) {
    double cth = std::cos(theta), sth = std::sin(theta);
    if (sth < 0) { sth = -sth; phi += kPi; }
    if (!(cth == cth) || !(sth == sth) || !(phi == phi) || std::isinf(phi)) return -1;
    HpCont h = hp_loc_to_face(cth, sth, phi);
    int64_t ix = (int64_t)(h.x * nside), iy = (int64_t)(h.y * nside);
    return nest ? hp_face_to_nest(nside, ix, iy, h.f) : hp_face_to_ring(nside, ix, iy, h.f);
}

// ---------------------------------------------------------------------------
// Pixelizors (src/Projection.cxx:513-1166).

enum { PX_FLAT_NT_NN = 0, PX_FLAT_NT_BL = 1, PX_FLAT_T_NN = 2, PX_FLAT_T_BL = 3,
       PX_HP_NT = 4, PX_HP_T = 5 };

struct Geom {
    // Flat
    int ny, nx;
    double cdy, cdx, cry, crx;
    int ty, tx, nty, ntx;
    // HEALPix
    int64_t nside, npix, nppt;
    int ntile_hp;
    bool nest;
    int ncomp;
    int n_tile() const { return ntile_hp; }
};

Geom make_geom(const so3g_pixelization *pz) {
    Geom g{};
    g.ncomp = pz->n_comp;
    g.ny = pz->naxis[0]; g.nx = pz->naxis[1];
    g.cdy = pz->cdelt[0]; g.cdx = pz->cdelt[1];
    g.cry = pz->crpix[0]; g.crx = pz->crpix[1];
    g.ty = pz->tile_shape[0]; g.tx = pz->tile_shape[1];
    if (pz->pix_sys == SO3G_PIX_FLAT && pz->tiled) {
        g.nty = (g.ny + g.ty - 1) / g.ty;
        g.ntx = (g.nx + g.tx - 1) / g.tx;
        g.ntile_hp = g.nty * g.ntx;
    }
    if (pz->pix_sys == SO3G_PIX_HEALPIX) {
        g.nside = pz->nside;
        g.npix = 12 * g.nside * g.nside;
        g.nest = pz->nest != 0;
        if (pz->tiled) {
            g.ntile_hp = (int)(12 * (int64_t)pz->nside_tile * pz->nside_tile);
            g.nppt = g.npix / g.ntile_hp;
        }
    }
    return g;
}

template <int P> struct Pix;

// Pixelizor2_Flat<NonTiled, NearestNeighbor>
template <> struct Pix<PX_FLAT_NT_NN> {
    static constexpr int index_count = 2, interp_count = 1;
    // GetPixel, :845-863
    static inline void get_pixel(const Geom &g, const double *coords, int *idx) {
        double ix = coords[0] / g.cdx + g.crx - 1 + 0.5;
        if (!(ix >= 0 && ix < g.nx)) { idx[0] = -1; return; }   // guard: NaN
        double iy = coords[1] / g.cdy + g.cry - 1 + 0.5;
        if (!(iy >= 0 && iy < g.ny)) { idx[0] = -1; return; }
        idx[0] = int(iy);
        idx[1] = int(ix);
    }
    // GetPixels, :912-926
    static inline int get_pixels(const Geom &g, const double *coords, int pix[][3], float *w) {
        double x = coords[0] / g.cdx + g.crx - 1 + 0.5;
        double y = coords[1] / g.cdy + g.cry - 1 + 0.5;
        if (!(x >= 0 && x < g.nx)) return 0;                    // guard: NaN
        if (!(y >= 0 && y < g.ny)) return 0;
        pix[0][0] = int(y) - int(y < 0);
        pix[0][1] = int(x) - int(x < 0);
        w[0] = 1;
        return 1;
    }
};

// Pixelizor2_Flat<NonTiled, Bilinear>::GetPixels, :930-952
template <> struct Pix<PX_FLAT_NT_BL> {
    static constexpr int index_count = 2, interp_count = 4;
    static inline void get_pixel(const Geom &g, const double *coords, int *idx) {
        Pix<PX_FLAT_NT_NN>::get_pixel(g, coords, idx);
    }
    static inline int get_pixels(const Geom &g, const double *coords, int pix[][3], float *w) {
        double x = coords[0] / g.cdx + g.crx - 1 + 0.5;
        double y = coords[1] / g.cdy + g.cry - 1 + 0.5;
        if (!(x > -4 && x < g.nx + 4 && y > -4 && y < g.ny + 4)) return 0;  // guard
        int x1 = int(x) - int(x < 0);
        int y1 = int(y) - int(y < 0);
        double wx[2] = {x - x1, 1 - (x - x1)};
        double wy[2] = {y - y1, 1 - (y - y1)};
        int iout = 0;
        for (int iy = y1; iy < y1 + 2; iy++) {
            if (iy < 0 || iy >= g.ny) continue;
            for (int ix = x1; ix < x1 + 2; ix++) {
                if (ix < 0 || ix >= g.nx) continue;
                pix[iout][0] = iy;
                pix[iout][1] = ix;
                w[iout] = wy[iy - y1] * wx[ix - x1];
                iout++;
            }
        }
        return iout;
    }
};

// Pixelizor2_Flat<Tiled, NearestNeighbor>
template <> struct Pix<PX_FLAT_T_NN> {
    static constexpr int index_count = 3, interp_count = 1;
    // GetPixel, :1029-1051
    static inline void get_pixel(const Geom &g, const double *coords, int *idx) {
        double ix = coords[0] / g.cdx + g.crx - 1 + 0.5;
        if (!(ix >= 0 && ix < g.nx)) { idx[0] = -1; return; }
        double iy = coords[1] / g.cdy + g.cry - 1 + 0.5;
        if (!(iy >= 0 && iy < g.ny)) { idx[0] = -1; return; }
        int sub_y = int(iy) / g.ty;
        int sub_x = int(ix) / g.tx;
        idx[0] = sub_y * ((g.nx + g.tx - 1) / g.tx) + sub_x;
        idx[1] = int(iy) - sub_y * g.ty;
        idx[2] = int(ix) - sub_x * g.tx;
    }
    // GetPixels, :1124-1138: truncation before the bounds test, so
    // x in (-1, 0) lands in column 0.
    static inline int get_pixels(const Geom &g, const double *coords, int pix[][3], float *w) {
        double x = coords[0] / g.cdx + g.crx - 1 + 0.5;
        if (!(x > -1 && x < g.nx)) return 0;   // == (int(x) in [0, nx)); guard: NaN
        int ix = int(x);
        double y = coords[1] / g.cdy + g.cry - 1 + 0.5;
        if (!(y > -1 && y < g.ny)) return 0;
        int iy = int(y);
        int sub_y = iy / g.ty;
        int sub_x = ix / g.tx;
        pix[0][0] = sub_y * ((g.nx + g.tx - 1) / g.tx) + sub_x;
        pix[0][1] = iy - sub_y * g.ty;
        pix[0][2] = ix - sub_x * g.tx;
        w[0] = 1;
        return 1;
    }
};

// Pixelizor2_Flat<Tiled, Bilinear>::GetPixels, :1141-1166 (truncation)
template <> struct Pix<PX_FLAT_T_BL> {
    static constexpr int index_count = 3, interp_count = 4;
    static inline void get_pixel(const Geom &g, const double *coords, int *idx) {
        Pix<PX_FLAT_T_NN>::get_pixel(g, coords, idx);
    }
    static inline int get_pixels(const Geom &g, const double *coords, int pix[][3], float *w) {
        double x = coords[0] / g.cdx + g.crx - 1 + 0.5;
        double y = coords[1] / g.cdy + g.cry - 1 + 0.5;
        if (!(x > -4 && x < g.nx + 4 && y > -4 && y < g.ny + 4)) return 0;  // guard
        int x1 = int(x);
        int y1 = int(y);
        double wx[2] = {x - x1, 1 - (x - x1)};
        double wy[2] = {y - y1, 1 - (y - y1)};
        int iout = 0;
        for (int iy = y1; iy < y1 + 2; iy++) {
            if (iy < 0 || iy >= g.ny) continue;
            int sub_y = iy / g.ty;
            for (int ix = x1; ix < x1 + 2; ix++) {
                if (ix < 0 || ix >= g.nx) continue;
                int sub_x = ix / g.tx;
                pix[iout][0] = sub_y * ((g.nx + g.tx - 1) / g.tx) + sub_x;
                pix[iout][1] = iy - sub_y * g.ty;
                pix[iout][2] = ix - sub_x * g.tx;
                w[iout] = wy[iy - y1] * wx[ix - x1];
                iout++;
            }
        }
        return iout;
    }
};

// Pixelizor_Healpix<NonTiled>, :522-620
template <> struct Pix<PX_HP_NT> {
    static constexpr int index_count = 1, interp_count = 1;
    static inline void get_pixel(const Geom &g, const double *coords, int *idx) {
        double phi = coords[0];
        double theta = kPi / 2 - coords[1];
        idx[0] = (int)hp_ang2pix(g.nside, g.nest, theta, phi);
    }
    static inline int get_pixels(const Geom &g, const double *coords, int pix[][3], float *w) {
        double phi = coords[0];
        double theta = kPi / 2 - coords[1];
        int64_t ix = hp_ang2pix(g.nside, g.nest, theta, phi);
        if (ix < 0 || ix >= g.npix) return 0;   // guard: NaN angle, phi <= -2 pi
        pix[0][0] = (int)ix;
        w[0] = 1;
        return 1;
    }
};

// Pixelizor_Healpix<Tiled> (NEST only), :628-800
template <> struct Pix<PX_HP_T> {
    static constexpr int index_count = 2, interp_count = 1;
    static inline void get_pixel(const Geom &g, const double *coords, int *idx) {
        double phi = coords[0];
        double theta = kPi / 2 - coords[1];
        int ix = (int)hp_ang2pix(g.nside, true, theta, phi);
        if (ix < 0) { idx[0] = -1; return; }   // guard: NaN angle
        idx[0] = ix / (int)g.nppt;
        idx[1] = ix % (int)g.nppt;
    }
    static inline int get_pixels(const Geom &g, const double *coords, int pix[][3], float *w) {
        double phi = coords[0];
        double theta = kPi / 2 - coords[1];
        int64_t ix = hp_ang2pix(g.nside, true, theta, phi);
        if (ix < 0 || ix >= g.npix) return 0;
        pix[0][0] = (int)(ix / g.nppt);
        pix[0][1] = (int)(ix % g.nppt);
        w[0] = 1;
        return 1;
    }
};

// Element offset of a pixel tuple in a map (the pix()/wpix() accessors,
// :590-600, :755-774, :881-893, :1084-1105) and the size of one component
// plane.  Returns false and sets *bad_tile for an absent tile.
template <int P>
inline bool locate(const Geom &g, const so3g_map *m, const int *idx, int64_t *off,
                   int64_t *plane, int *bad_tile) {
    if (P == PX_FLAT_NT_NN || P == PX_FLAT_NT_BL) {
        *off = (int64_t)idx[0] * g.nx + idx[1];
        *plane = (int64_t)g.ny * g.nx;
        return true;
    } else if (P == PX_FLAT_T_NN || P == PX_FLAT_T_BL) {
        int t = idx[0];
        if (t < 0 || t >= m->n_tile || m->tile_offset[t] < 0) { *bad_tile = t; return false; }
        int row = t / g.ntx, col = t % g.ntx;
        int64_t tny = std::min(g.ty, g.ny - row * g.ty);
        int64_t tnx = std::min(g.tx, g.nx - col * g.tx);
        *off = m->tile_offset[t] + idx[1] * tnx + idx[2];
        *plane = tny * tnx;
        return true;
    } else if (P == PX_HP_NT) {
        *off = idx[0];
        *plane = g.npix;
        return true;
    } else {
        int t = idx[0];
        if (t < 0 || t >= m->n_tile || m->tile_offset[t] < 0) { *bad_tile = t; return false; }
        *off = m->tile_offset[t] + idx[1];
        *plane = g.nppt;
        return true;
    }
}

// stripe(), :601-603, :776-780, :894-898, :1106-1108.
template <int P>
inline int64_t stripe(const Geom &g, const int *idx, int n) {
    if (P == PX_FLAT_NT_NN || P == PX_FLAT_NT_BL) {
        if (idx[0] < 0) return -1;
        return (int64_t)idx[1] * n / g.nx;
    } else if (P == PX_FLAT_T_NN || P == PX_FLAT_T_BL) {
        return idx[0] % n;
    } else if (P == PX_HP_NT) {
        return (int64_t)idx[0] * n / g.npix;
    } else {
        int64_t ipix = (int64_t)idx[0] * g.nppt + idx[1];
        return ipix * n / (g.nppt * g.ntile_hp);
    }
}

// ---------------------------------------------------------------------------
// Spin projection factors, src/Projection.cxx:1180-1209.

template <int NC>
inline void spin_factors(const double *coords, float T, float P, float *pf) {
    if (NC == 1) {
        pf[0] = T;
    } else if (NC == 2) {
        const double c = coords[2], s = coords[3];
        pf[0] = P * (c * c - s * s);
        pf[1] = P * (2 * c * s);
    } else {
        const double c = coords[2], s = coords[3];
        pf[0] = T;
        pf[1] = P * (c * c - s * s);
        pf[2] = P * (2 * c * s);
    }
}

inline void record_tile_error(int32_t *err, int tile) {
    if (!err) return;
#pragma omp critical(orc_err)
    {
        if (err[0] == 0 || (err[0] == SO3G_DEVERR_MISSING_TILE && tile < err[1])) {
            err[0] = SO3G_DEVERR_MISSING_TILE;
            err[1] = tile;
        }
    }
}

inline void record_range_error(int32_t *err, int tile, int det, int t) {
    if (!err) return;
#pragma omp critical(orc_err)
    {
        if (err[0] == 0) {
            err[0] = SO3G_DEVERR_PIXEL_RANGE;
            err[1] = tile; err[2] = det; err[3] = t;
        }
    }
}

// ---------------------------------------------------------------------------
// Operations.

struct Inputs {
    const double *bore;
    int n_time;
    const double *dets;
    int n_det;
};

template <int C>
void op_coords(const Inputs &in, double *out) {
    // ProjectionEngine::coords, :1316-1349
#pragma omp parallel for
    for (int i_det = 0; i_det < in.n_det; ++i_det) {
        const double *dofs = in.dets + 4 * (int64_t)i_det;
        double *row = out + (int64_t)i_det * in.n_time * 4;
        for (int t = 0; t < in.n_time; ++t)
            get_coords<C>(in.bore + 4 * (int64_t)t, dofs, row + 4 * (int64_t)t);
    }
}

template <int C, int P, int NC>
void op_pointing(const Geom &g, const Inputs &in, const float *resp, int32_t *pixel, float *proj) {
    // ProjectionEngine::pixels (:1351-1385) and pointing_matrix (:1391-1438):
    // the pixel tuple persists across samples of a detector, so slots the
    // pixelizor does not write keep the previous sample's values.
    constexpr int IC = Pix<P>::index_count;
#pragma omp parallel for
    for (int i_det = 0; i_det < in.n_det; ++i_det) {
        const double *dofs = in.dets + 4 * (int64_t)i_det;
        int idx[3] = {-1, 0, 0};
        float T = 0, Pr = 0;
        if (proj) { T = resp[2 * i_det]; Pr = resp[2 * i_det + 1]; }
        for (int t = 0; t < in.n_time; ++t) {
            double coords[4];
            get_coords<C>(in.bore + 4 * (int64_t)t, dofs, coords);
            Pix<P>::get_pixel(g, coords, idx);
            int64_t s = ((int64_t)i_det * in.n_time + t);
            for (int k = 0; k < IC; k++) pixel[s * IC + k] = idx[k];
            if (proj) {
                float pf[3];
                spin_factors<NC>(coords, T, Pr, pf);
                for (int k = 0; k < NC; k++) proj[s * NC + k] = pf[k];
            }
        }
    }
}

template <int C, int P>
void op_tile_hits(const Geom &g, const Inputs &in, int64_t *hits, int n_tile) {
    // ProjectionEngine::tile_hits, :1543-1601
    std::vector<int64_t> total(n_tile, 0);
#pragma omp parallel
    {
        std::vector<int64_t> mine(n_tile, 0);
#pragma omp for
        for (int i_det = 0; i_det < in.n_det; ++i_det) {
            const double *dofs = in.dets + 4 * (int64_t)i_det;
            for (int t = 0; t < in.n_time; ++t) {
                double coords[4];
                int pix[4][3];
                float w[4];
                get_coords<C>(in.bore + 4 * (int64_t)t, dofs, coords);
                int n = Pix<P>::get_pixels(g, coords, pix, w);
                for (int k = 0; k < n; k++)
                    if (pix[k][0] >= 0 && pix[k][0] < n_tile) mine[pix[k][0]]++;
            }
        }
#pragma omp critical(orc_hits)
        for (int k = 0; k < n_tile; k++) total[k] += mine[k];
    }
    for (int k = 0; k < n_tile; k++) hits[k] = total[k];
}

template <int C, int P>
void op_labels(const Geom &g, const Inputs &in, int mode, int n_domain, const so3g_map *dmap,
               const int32_t *tile_domain, int n_tile, int32_t *label, int32_t *err) {
    // Sample domains of pixel_ranges (:1489-1506) and tile_ranges (:1655-1670).
#pragma omp parallel for
    for (int i_det = 0; i_det < in.n_det; ++i_det) {
        const double *dofs = in.dets + 4 * (int64_t)i_det;
        for (int t = 0; t < in.n_time; ++t) {
            double coords[4];
            int pix[4][3];
            float w[4];
            get_coords<C>(in.bore + 4 * (int64_t)t, dofs, coords);
            int n = Pix<P>::get_pixels(g, coords, pix, w);
            int64_t samp = -1;
            for (int k = 0; k < n; k++) {
                int64_t pd;
                if (mode == 0) {
                    pd = stripe<P>(g, pix[k], n_domain);
                } else if (mode == 1) {
                    int64_t off, plane;
                    int bad = 0;
                    if (!locate<P>(g, dmap, pix[k], &off, &plane, &bad)) {
                        record_tile_error(err, bad);
                        pd = -1;
                    } else {
                        double v = dmap->data[off];
                        pd = (v > -2147483648.0 && v < 2147483648.0) ? (int64_t)(int)v : -1;
                    }
                } else {
                    int tile = pix[k][0];
                    pd = (tile >= 0 && tile < n_tile) ? tile_domain[tile] : -1;
                }
                if (k > 0 && pd != samp) { samp = n_domain; break; }
                samp = pd;
            }
            label[(int64_t)i_det * in.n_time + t] = (int32_t)samp;
        }
    }
}

struct SchedView {
    // Flattened schedule; with no sched, one bunch with one thread covering
    // all samples of all detectors.
    std::vector<int32_t> seg_store, toff_store, boff_store;
    const int32_t *seg;
    const int32_t *toff;
    const int32_t *boff;
    int n_bunch;
};

SchedView make_sched(const orc_sched *s, int n_det, int n_time) {
    SchedView v;
    if (s) {
        v.seg = s->seg; v.toff = s->thread_offset; v.boff = s->bunch_offset; v.n_bunch = s->n_bunch;
        return v;
    }
    for (int d = 0; d < n_det; d++) { v.seg_store.push_back(d); v.seg_store.push_back(0); v.seg_store.push_back(n_time); }
    v.toff_store = {0, n_det};
    v.boff_store = {0, 1};
    v.seg = v.seg_store.data(); v.toff = v.toff_store.data(); v.boff = v.boff_store.data(); v.n_bunch = 1;
    return v;
}

template <int C, int P, int NC, bool WEIGHT>
void op_scatter(const Geom &g, const Inputs &in, const float *resp, const float *signal,
                int64_t sig_stride, const float *det_weights, const orc_sched *sched,
                const so3g_map *map, int32_t *err) {
    // to_map (:1924-1966 / :1772-1811) and to_weight_map (:1968-2010 / :1813-1854).
    SchedView sv = make_sched(sched, in.n_det, in.n_time);
    for (int b = 0; b < sv.n_bunch; b++) {
        int th0 = sv.boff[b], th1 = sv.boff[b + 1];
#pragma omp parallel for schedule(dynamic, 1)
        for (int th = th0; th < th1; th++) {
            for (int k = sv.toff[th]; k < sv.toff[th + 1]; k++) {
                int i_det = sv.seg[3 * k], t0 = sv.seg[3 * k + 1], t1 = sv.seg[3 * k + 2];
                float det_wt = 1.;
                if (det_weights) {
                    det_wt = det_weights[i_det];
                    if (det_wt == 0.) continue;
                }
                const double *dofs = in.dets + 4 * (int64_t)i_det;
                const float T = resp[2 * i_det], Pr = resp[2 * i_det + 1];
                for (int t = t0; t < t1; ++t) {
                    double coords[4];
                    float pf[3];
                    int pix[4][3];
                    float w[4];
                    get_coords<C>(in.bore + 4 * (int64_t)t, dofs, coords);
                    spin_factors<NC>(coords, T, Pr, pf);
                    float sig = 0;
                    if (!WEIGHT) sig = signal[(int64_t)i_det * sig_stride + t];
                    int n = Pix<P>::get_pixels(g, coords, pix, w);
                    for (int ip = 0; ip < n; ip++) {
                        int64_t off, plane;
                        int bad = 0;
                        if (!locate<P>(g, map, pix[ip], &off, &plane, &bad)) {
                            record_tile_error(err, bad);
                            continue;
                        }
                        if (!WEIGHT) {
                            for (int c = 0; c < NC; c++)
                                map->data[off + c * plane] += sig * pf[c] * w[ip] * det_wt;
                        } else {
                            for (int i = 0; i < NC; i++)
                                for (int j = i; j < NC; j++)
                                    map->data[off + (i * NC + j) * plane] +=
                                        pf[i] * pf[j] * w[ip] * w[ip] * det_wt;
                        }
                    }
                }
            }
        }
    }
}

template <int C, int P, int NC>
void op_from_map(const Geom &g, const Inputs &in, const float *resp, const so3g_map *map,
                 float *signal, int64_t sig_stride, int32_t *err) {
    // ProjectionEngine::from_map, :1728-1770
#pragma omp parallel for
    for (int i_det = 0; i_det < in.n_det; ++i_det) {
        const double *dofs = in.dets + 4 * (int64_t)i_det;
        const float T = resp[2 * i_det], Pr = resp[2 * i_det + 1];
        for (int t = 0; t < in.n_time; ++t) {
            double coords[4];
            float pf[3];
            int pix[4][3];
            float w[4];
            get_coords<C>(in.bore + 4 * (int64_t)t, dofs, coords);
            spin_factors<NC>(coords, T, Pr, pf);
            float *sig = signal + (int64_t)i_det * sig_stride + t;
            int n = Pix<P>::get_pixels(g, coords, pix, w);
            for (int ip = 0; ip < n; ip++) {
                int64_t off, plane;
                int bad = 0;
                if (!locate<P>(g, map, pix[ip], &off, &plane, &bad)) {
                    record_tile_error(err, bad);
                    continue;
                }
                for (int c = 0; c < NC; c++)
                    *sig += map->data[off + c * plane] * pf[c] * w[ip];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Dispatch.

template <int C, int P>
int dispatch_cp(const so3g_pixelization *pz, int op, void **a);

enum { OP_POINTING = 0, OP_TILE_HITS, OP_LABELS, OP_TO_MAP, OP_TO_WEIGHT, OP_FROM_MAP };

struct Args {
    Inputs in;
    const float *resp;
    int32_t *pixel;
    float *proj;
    int64_t *hits;
    int n_tile;
    int mode, n_domain;
    const so3g_map *dmap;
    const int32_t *tile_domain;
    int32_t *label;
    const float *signal_in;
    float *signal_out;
    int64_t sig_stride;
    const float *det_weights;
    const orc_sched *sched;
    const so3g_map *map;
    int32_t *err;
};

template <int C, int P, int NC>
void run_cpn(const Geom &g, int op, const Args &a) {
    switch (op) {
    case OP_POINTING: op_pointing<C, P, NC>(g, a.in, a.resp, a.pixel, a.proj); break;
    case OP_TO_MAP: op_scatter<C, P, NC, false>(g, a.in, a.resp, a.signal_in, a.sig_stride, a.det_weights, a.sched, a.map, a.err); break;
    case OP_TO_WEIGHT: op_scatter<C, P, NC, true>(g, a.in, a.resp, nullptr, 0, a.det_weights, a.sched, a.map, a.err); break;
    case OP_FROM_MAP: op_from_map<C, P, NC>(g, a.in, a.resp, a.map, a.signal_out, a.sig_stride, a.err); break;
    }
}

template <int C, int P>
void run_cp(const so3g_pixelization *pz, const Geom &g, int op, const Args &a) {
    if (op == OP_TILE_HITS) { op_tile_hits<C, P>(g, a.in, a.hits, a.n_tile); return; }
    if (op == OP_LABELS) { op_labels<C, P>(g, a.in, a.mode, a.n_domain, a.dmap, a.tile_domain, a.n_tile, a.label, a.err); return; }
    switch (pz->n_comp) {
    case 1: run_cpn<C, P, 1>(g, op, a); break;
    case 2: run_cpn<C, P, 2>(g, op, a); break;
    default: run_cpn<C, P, 3>(g, op, a); break;
    }
}

template <int C>
void run_c(const so3g_pixelization *pz, const Geom &g, int op, const Args &a) {
    if (pz->pix_sys == SO3G_PIX_HEALPIX) {
        if (pz->tiled) run_cp<C, PX_HP_T>(pz, g, op, a);
        else run_cp<C, PX_HP_NT>(pz, g, op, a);
        return;
    }
    int p = (pz->tiled ? 2 : 0) + (pz->interp == SO3G_INTERP_BILINEAR ? 1 : 0);
    switch (p) {
    case PX_FLAT_NT_NN: run_cp<C, PX_FLAT_NT_NN>(pz, g, op, a); break;
    case PX_FLAT_NT_BL: run_cp<C, PX_FLAT_NT_BL>(pz, g, op, a); break;
    case PX_FLAT_T_NN: run_cp<C, PX_FLAT_T_NN>(pz, g, op, a); break;
    default: run_cp<C, PX_FLAT_T_BL>(pz, g, op, a); break;
    }
}

int check_pz(const so3g_pixelization *pz) {
    if (!g_ready) build_tables();
    if (!pz) return fail("null pixelization");
    if (pz->n_comp < 1 || pz->n_comp > 3) return fail("n_comp must be 1, 2 or 3");
    if (pz->coord_sys < 0 || pz->coord_sys > 7) return fail("bad coord_sys");
    if (pz->pix_sys == SO3G_PIX_HEALPIX) {
        if (pz->coord_sys != SO3G_COORD_CAR) return fail("HEALPix needs CAR coordinates");
        int ns = pz->nside;
        if (!(ns > 0 && ns < 8192 && (ns & (ns - 1)) == 0)) return fail("Invalid nside");
        if (pz->tiled) {
            int nt = pz->nside_tile;
            if (!(nt > 0 && nt <= ns && (nt & (nt - 1)) == 0)) return fail("Invalid nside_tile");
        }
    } else {
        if (pz->naxis[0] < 0 || pz->naxis[1] < 0) return fail("bad naxis");
        if (pz->tiled && (pz->tile_shape[0] <= 0 || pz->tile_shape[1] <= 0)) return fail("bad tile_shape");
    }
    return 0;
}

int run(const so3g_pixelization *pz, int op, const Args &a) {
    int rc = check_pz(pz);
    if (rc) return rc;
    Geom g = make_geom(pz);
    switch (pz->coord_sys) {
    case SO3G_COORD_FLAT: run_c<SO3G_COORD_FLAT>(pz, g, op, a); break;
    case SO3G_COORD_QUAT: run_c<SO3G_COORD_QUAT>(pz, g, op, a); break;
    case SO3G_COORD_CAR: run_c<SO3G_COORD_CAR>(pz, g, op, a); break;
    case SO3G_COORD_CEA: run_c<SO3G_COORD_CEA>(pz, g, op, a); break;
    case SO3G_COORD_ARC: run_c<SO3G_COORD_ARC>(pz, g, op, a); break;
    case SO3G_COORD_SIN: run_c<SO3G_COORD_SIN>(pz, g, op, a); break;
    case SO3G_COORD_TAN: run_c<SO3G_COORD_TAN>(pz, g, op, a); break;
    default: run_c<SO3G_COORD_ZEA>(pz, g, op, a); break;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// ProjEng_Precomp (src/Projection.cxx:2012-2256).

struct PcMap {
    const so3g_precomp_geom *g;
    const so3g_map *m;
    // Element offset of the (tile,) iy, ix tuple and the plane size.
    inline int locate(const int32_t *idx, int64_t *off, int64_t *plane, int *bad_tile, bool *range) const {
        *range = false;
        if (!g->tiled) {
            int ny = g->naxis[0], nx = g->naxis[1];
            if (idx[0] >= ny || idx[1] < 0 || idx[1] >= nx) { *range = true; return 0; }
            *off = (int64_t)idx[0] * nx + idx[1];
            *plane = (int64_t)ny * nx;
            return 1;
        }
        int t = idx[0];
        if (t >= m->n_tile || m->tile_offset[t] < 0) { *bad_tile = t; return 0; }
        int tny = g->tile_dims[2 * t], tnx = g->tile_dims[2 * t + 1];
        if (idx[1] < 0 || idx[1] >= tny || idx[2] < 0 || idx[2] >= tnx) { *range = true; return 0; }
        *off = m->tile_offset[t] + (int64_t)idx[1] * tnx + idx[2];
        *plane = (int64_t)tny * tnx;
        return 1;
    }
};

template <bool WEIGHT>
void precomp_scatter(const so3g_precomp_geom *g, const int32_t *pixel, const float *spin,
                     int n_det, int n_time, const float *signal, int64_t sig_stride,
                     const float *det_weights, const orc_sched *sched, const so3g_map *map,
                     int32_t *err) {
    // precomp_to_map_single_thread (:2087-2122), precomp_to_weight_map_single_thread (:2124-2155)
    const int NI = g->tiled ? 3 : 2, NC = g->n_comp;
    PcMap pm{g, map};
    SchedView sv = make_sched(sched, n_det, n_time);
    for (int b = 0; b < sv.n_bunch; b++) {
        int th0 = sv.boff[b], th1 = sv.boff[b + 1];
#pragma omp parallel for schedule(dynamic, 1)
        for (int th = th0; th < th1; th++) {
            for (int k = sv.toff[th]; k < sv.toff[th + 1]; k++) {
                int i_det = sv.seg[3 * k], t0 = sv.seg[3 * k + 1], t1 = sv.seg[3 * k + 2];
                float det_wt = 1.;
                if (det_weights) {
                    det_wt = det_weights[i_det];
                    if (det_wt == 0.) continue;
                }
                for (int t = t0; t < t1; ++t) {
                    int64_t s = (int64_t)i_det * n_time + t;
                    const int32_t *po = pixel + s * NI;
                    if (po[0] < 0) continue;
                    const float *pf = spin + s * NC;
                    int64_t off, plane;
                    int bad = 0;
                    bool range;
                    if (!pm.locate(po, &off, &plane, &bad, &range)) {
                        if (range) record_range_error(err, g->tiled ? po[0] : 0, i_det, t);
                        else record_tile_error(err, bad);
                        continue;
                    }
                    if (!WEIGHT) {
                        const float sig = signal[(int64_t)i_det * sig_stride + t];
                        for (int c = 0; c < NC; ++c)
                            map->data[off + c * plane] += det_wt * sig * pf[c];
                    } else {
                        for (int i = 0; i < NC; ++i)
                            for (int j = i; j < NC; ++j)
                                map->data[off + (i * NC + j) * plane] += pf[i] * pf[j] * det_wt;
                    }
                }
            }
        }
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI.

extern "C" {

int orc_init(void) {
    if (!g_ready) build_tables();
    return 0;
}

int orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

const char *orc_last_error(void) { return g_err.c_str(); }

int orc_get_tables(double *asin_vals, double *atan2_vals, int32_t n) {
    if (!g_ready) build_tables();
    if (n != kTableSize) return fail("table size mismatch");
    std::memcpy(asin_vals, g_asin.v.data(), sizeof(double) * n);
    std::memcpy(atan2_vals, g_atan2.v.data(), sizeof(double) * n);
    return 0;
}

double orc_asin(double x) { if (!g_ready) build_tables(); return asin_lut(x); }
double orc_atan2(double y, double x) { if (!g_ready) build_tables(); return atan2_lut(y, x); }
int64_t orc_ang2pix(int64_t nside, int32_t nest, double theta, double phi) {
    return hp_ang2pix(nside, nest != 0, theta, phi);
}

int orc_coords(const so3g_pixelization *pz, const double *bore, int32_t n_time,
               const double *dets, int32_t n_det, double *coords) {
    int rc = check_pz(pz);
    if (rc) return rc;
    Inputs in{bore, n_time, dets, n_det};
    switch (pz->coord_sys) {
    case SO3G_COORD_FLAT: op_coords<SO3G_COORD_FLAT>(in, coords); break;
    case SO3G_COORD_QUAT: op_coords<SO3G_COORD_QUAT>(in, coords); break;
    case SO3G_COORD_CAR: op_coords<SO3G_COORD_CAR>(in, coords); break;
    case SO3G_COORD_CEA: op_coords<SO3G_COORD_CEA>(in, coords); break;
    case SO3G_COORD_ARC: op_coords<SO3G_COORD_ARC>(in, coords); break;
    case SO3G_COORD_SIN: op_coords<SO3G_COORD_SIN>(in, coords); break;
    case SO3G_COORD_TAN: op_coords<SO3G_COORD_TAN>(in, coords); break;
    default: op_coords<SO3G_COORD_ZEA>(in, coords); break;
    }
    return 0;
}

int orc_pixels(const so3g_pixelization *pz, const double *bore, int32_t n_time,
               const double *dets, int32_t n_det, int32_t *pixel) {
    Args a{};
    a.in = Inputs{bore, n_time, dets, n_det};
    a.pixel = pixel;
    a.proj = nullptr;
    return run(pz, OP_POINTING, a);
}

int orc_pointing_matrix(const so3g_pixelization *pz, const double *bore,
                        int32_t n_time, const double *dets, int32_t n_det,
                        const float *response, int32_t *pixel, float *proj) {
    Args a{};
    a.in = Inputs{bore, n_time, dets, n_det};
    a.resp = response;
    a.pixel = pixel;
    a.proj = proj;
    return run(pz, OP_POINTING, a);
}

int orc_tile_hits(const so3g_pixelization *pz, const double *bore, int32_t n_time,
                  const double *dets, int32_t n_det, int64_t *hits, int32_t n_tile) {
    if (!pz->tiled) return fail("No tiles in this pixelization.");
    Args a{};
    a.in = Inputs{bore, n_time, dets, n_det};
    a.hits = hits;
    a.n_tile = n_tile;
    return run(pz, OP_TILE_HITS, a);
}

int orc_domain_labels(const so3g_pixelization *pz, const double *bore,
                      int32_t n_time, const double *dets, int32_t n_det,
                      int32_t mode, int32_t n_domain, const so3g_map *dmap,
                      const int32_t *tile_domain, int32_t n_tile, int32_t *label) {
    Args a{};
    a.in = Inputs{bore, n_time, dets, n_det};
    a.mode = mode;
    a.n_domain = n_domain;
    a.dmap = dmap;
    a.tile_domain = tile_domain;
    a.n_tile = n_tile;
    a.label = label;
    return run(pz, OP_LABELS, a);
}

int orc_to_map(const so3g_pixelization *pz, const double *bore, int32_t n_time,
               const double *dets, int32_t n_det, const float *response,
               const float *signal, int64_t sig_det_stride,
               const float *det_weights, const orc_sched *sched,
               const so3g_map *map, int32_t *err) {
    Args a{};
    a.in = Inputs{bore, n_time, dets, n_det};
    a.resp = response;
    a.signal_in = signal;
    a.sig_stride = sig_det_stride;
    a.det_weights = det_weights;
    a.sched = sched;
    a.map = map;
    a.err = err;
    return run(pz, OP_TO_MAP, a);
}

int orc_to_weight_map(const so3g_pixelization *pz, const double *bore,
                      int32_t n_time, const double *dets, int32_t n_det,
                      const float *response, const float *det_weights,
                      const orc_sched *sched, const so3g_map *map, int32_t *err) {
    Args a{};
    a.in = Inputs{bore, n_time, dets, n_det};
    a.resp = response;
    a.det_weights = det_weights;
    a.sched = sched;
    a.map = map;
    a.err = err;
    return run(pz, OP_TO_WEIGHT, a);
}

int orc_from_map(const so3g_pixelization *pz, const double *bore, int32_t n_time,
                 const double *dets, int32_t n_det, const float *response,
                 const so3g_map *map, float *signal, int64_t sig_det_stride,
                 int32_t *err) {
    Args a{};
    a.in = Inputs{bore, n_time, dets, n_det};
    a.resp = response;
    a.map = map;
    a.signal_out = signal;
    a.sig_stride = sig_det_stride;
    a.err = err;
    return run(pz, OP_FROM_MAP, a);
}

int orc_precomp_to_map(const so3g_precomp_geom *g, const int32_t *pixel,
                       const float *spin_proj, int32_t n_det, int32_t n_time,
                       const float *signal, int64_t sig_det_stride,
                       const float *det_weights, const orc_sched *sched,
                       const so3g_map *map, int32_t *err) {
    precomp_scatter<false>(g, pixel, spin_proj, n_det, n_time, signal, sig_det_stride,
                           det_weights, sched, map, err);
    return 0;
}

int orc_precomp_to_weight_map(const so3g_precomp_geom *g, const int32_t *pixel,
                              const float *spin_proj, int32_t n_det,
                              int32_t n_time, const float *det_weights,
                              const orc_sched *sched, const so3g_map *map,
                              int32_t *err) {
    precomp_scatter<true>(g, pixel, spin_proj, n_det, n_time, nullptr, 0, det_weights,
                          sched, map, err);
    return 0;
}

int orc_precomp_from_map(const so3g_precomp_geom *g, const int32_t *pixel,
                         const float *spin_proj, int32_t n_det, int32_t n_time,
                         const so3g_map *map, float *signal,
                         int64_t sig_det_stride, int32_t *err) {
    // ProjEng_Precomp::from_map, :2036-2085
    const int NI = g->tiled ? 3 : 2, NC = g->n_comp;
    PcMap pm{g, map};
#pragma omp parallel for
    for (int i_det = 0; i_det < n_det; ++i_det) {
        for (int t = 0; t < n_time; ++t) {
            int64_t s = (int64_t)i_det * n_time + t;
            const int32_t *po = pixel + s * NI;
            if (po[0] < 0) continue;
            int64_t off, plane;
            int bad = 0;
            bool range;
            if (!pm.locate(po, &off, &plane, &bad, &range)) {
                if (range) record_range_error(err, g->tiled ? po[0] : 0, i_det, t);
                else record_tile_error(err, bad);
                continue;
            }
            float sig = 0;
            for (int c = 0; c < NC; ++c) {
                float pf = spin_proj[s * NC + c];
                sig += pf * map->data[off + c * plane];
            }
            signal[(int64_t)i_det * sig_det_stride + t] += sig;
        }
    }
    return 0;
}

}  // extern "C"
