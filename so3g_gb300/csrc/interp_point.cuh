// interp_point.cuh -- chunked pointing for the mixed mode of CAR maps with
// the untiled nearest-neighbour pixelizor: the pointing of 64 consecutive
// samples of a detector from one model, with a certified bound.
//
// The boresight of a chunk [ta, tb] (tb = ta + 64, or the last sample) is
// modelled by the quadratic through its samples at ta, the middle and tb,
//   Q(s) = q(ta) + s D1 + s^2 D2,   s = (t - ta) / (tb - ta),
// and E = max over the chunk's samples of |q(t) - Q(s)| is measured from
// the data (k_ix_bore, float64, once per call for all detectors).  For a
// detector q_d, q(t) (x) q_d = A0 + s A1 + s^2 A2 + e, |e| <= E |q_d|, with
// A_k = D_k (x) q_d.  The reference's coordinates are quadratic forms of
// that quaternion (Pointer<ProjCAR>::GetCoords, src/Projection.cxx:479-507):
//   w = X + iY = (ca + db) + i(cd - ab),  lon = atan2(Y, X)
//   Z = a^2 - b^2 - c^2 + d^2,            lat = asin(Z)
//   v = Nc + iNs = (ac - bd) + i(cd + ab), the spin factors P v^2 / |v|^2
// so along the model each is a polynomial in s, of degree 4 with its s^3
// and s^4 coefficients negligible (|A2| ~ 1e-6):
//   lon = lon(ta) + arg(1 + z),  z = c1 s + c2 s^2 (c_k = W_k / W_0)
//         ~ lon(ta) + Im(z - z^2/2 + z^3/3)              (|z| < 0.05)
//   lat = lat(ta) + k1 dZ + k2 dZ^2 + k3 dZ^3,  dZ = s Z1 + s^2 Z2
//         (asin's Taylor series),
// both expanded in s and cut after s^3: per sample a cubic in s for each
// pixel coordinate and a quadratic for each spin component, about 25
// float32 operations, with no boresight load and no table.
// The anchor lon(ta), lat(ta) are the reference's values at ta from the
// certified double-float pointing (fastpoint.cuh), as pixel coordinates
// x(ta), y(ta) split into an integer and a fraction.
//
// Bound (ix_setup): the remainders of the two series (|z|^4 / (4(1-|z|))
// and the asin term |dZ|^4 max|asin''''| / 24), the terms cut from their
// expansions in s, the dropped s^3, s^4 terms
// and the model error E through the forms' norms (|B_w(p, q)| <= |p||q|/
// sqrt(2), |B_Z(p, q)| <= |p||q|), the float32 evaluation of the
// coefficients and of the per-sample polynomials, the reference's table
// interpolation error at both ends (2 x h^2/8 max|f''|) and the anchor's
// double-float error, times a safety factor 1.5.  A sample whose pixel
// coordinates are farther than that from every integer gets the
// reference's pixel; the others (and every sample of a chunk whose model
// does not apply: near the native poles, across the atan2 seam, a chunk
// moving more than 0.05 of a radian, or one whose spin factors the model
// would not give to 1e-7) go to the fallback pass with the double-float and
// exact pointing.  Spin factors are float32 evaluations of the model
// (within ~1e-7 of the reference's), as in the mixed mode's float32 tier.
#pragma once

#include "mx_common.cuh"

namespace so3g {

namespace {

constexpr int kIxLen = 64;            // samples per chunk
constexpr int kIxBlocksPerSM = 4;

// The boresight model of one chunk.
struct IxBore {
    float4 d1, d2;    // Q(s) = q(ta) + s d1 + s^2 d2 (float32-rounded)
    float e;          // max |q(t) - Q(s)| over the chunk's samples (rounded up)
    float pad[3];
};

// Per (detector, chunk): the model's coefficients and bounds, read by the
// lanes of a chunk (six 16-byte words).
struct __align__(16) IxParams {
    float xf, yf, b1, b2;       // x = xb + xf + s (b1 + s (b2 + s b3)) (pixels)
    float b3, e1, e2, e3;       // y = yb + yf + s (e1 + s (e2 + s e3))
    float v0r, v0i, v1r, v1i;   // v = v0 + s (v1 + s (v2 + s v3))
    float v2r, v2i, hx, hy;     // hx, hy: 1/2 - bounds (pixels; < 0: not modelled)
    float v3r, v3i, inv_len;    // inv_len = 1 / (tb - ta)
    int ta;                     // chunk start
    int xb, yb, pad0, pad1;     // the anchor's integer parts
};

// The same six words for a HEALPix map: the sample's phi (radians) and
// z = sin(lat) as polynomials in s, with bounds on their errors against
// the reference's float64 values; the pixel follows from them per sample
// (hp_pixel_f32).
struct __align__(16) IxParamsHp {
    float lon_a, b1, b2, b3;    // lon = lon_a + s (b1 + s (b2 + s b3))
    float z_a, z1, z2, elon;    // z = z_a + s (z1 + s (z2 + s z3)); elon < 0: not modelled
    float v0r, v0i, v1r, v1i;   // v as IxParams
    float v2r, v2i, ez, z3;
    float v3r, v3i, inv_len;
    int ta;
    int pad0, pad1, pad2, pad3;
};
static_assert(sizeof(IxParamsHp) == sizeof(IxParams), "one shared-memory slot for both");

// The chunks' boresight models (one thread per chunk), in float64.
__global__ void k_ix_bore(const double *bore, int n_time, int n_chunks, IxBore *out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_chunks) return;
    const int ta = j * kIxLen, tb = min(ta + kIxLen, n_time - 1), L = tb - ta;
    double qa[4], d1[4], d2[4];
    for (int k = 0; k < 4; k++) qa[k] = __ldg(bore + 4LL * ta + k);
    if (L >= 2) {
        const int tm = ta + L / 2;
        const double sm = (double)(tm - ta) / L;
        for (int k = 0; k < 4; k++) {
            const double qm = __ldg(bore + 4LL * tm + k), qb = __ldg(bore + 4LL * tb + k);
            d2[k] = ((qm - qa[k]) - sm * (qb - qa[k])) / (sm * sm - sm);
            d1[k] = (qb - qa[k]) - d2[k];
        }
    } else {
        for (int k = 0; k < 4; k++) {
            d1[k] = L == 1 ? __ldg(bore + 4LL * tb + k) - qa[k] : 0.;
            d2[k] = 0.;
        }
    }
    float f1[4], f2[4];
    for (int k = 0; k < 4; k++) {
        f1[k] = __double2float_rn(d1[k]);
        f2[k] = __double2float_rn(d2[k]);
    }
    double e = 0.;
    for (int t = ta; t <= tb; t++) {
        const double s = L > 0 ? (double)(t - ta) / L : 0.;
        double n2 = 0.;
        for (int k = 0; k < 4; k++) {
            const double r = __ldg(bore + 4LL * t + k) - (qa[k] + s * (double)f1[k] +
                                                          s * s * (double)f2[k]);
            n2 += r * r;
        }
        e = fmax(e, sqrt(n2));
    }
    IxBore o;
    o.d1 = make_float4(f1[0], f1[1], f1[2], f1[3]);
    o.d2 = make_float4(f2[0], f2[1], f2[2], f2[3]);
    o.e = __double2float_ru(e * (1. + 1e-6) + 1e-30);
    o.pad[0] = o.pad[1] = o.pad[2] = 0.f;
    out[j] = o;
}

__device__ __forceinline__ void qmul32(const float (&p)[4], const float (&q)[4], float (&r)[4]) {
    r[0] = p[0] * q[0] - p[1] * q[1] - p[2] * q[2] - p[3] * q[3];
    r[1] = p[0] * q[1] + p[1] * q[0] + p[2] * q[3] - p[3] * q[2];
    r[2] = p[0] * q[2] - p[1] * q[3] + p[2] * q[0] + p[3] * q[1];
    r[3] = p[0] * q[3] + p[1] * q[2] - p[2] * q[1] + p[3] * q[0];
}

__device__ __forceinline__ float norm4(const float (&q)[4]) {
    return sqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
}

// The three quadratic forms of (a, b, c, d) and twice their polar forms
// B(p, q) (so that F(p + q) = F(p) + 2 B(p, q) + F(q)).
__device__ __forceinline__ void form_w(const float (&q)[4], float &x, float &y) {
    x = q[2] * q[0] + q[3] * q[1];
    y = q[2] * q[3] - q[0] * q[1];
}
__device__ __forceinline__ void form_w2(const float (&p)[4], const float (&q)[4], float &x,
                                        float &y) {
    x = p[2] * q[0] + p[0] * q[2] + p[3] * q[1] + p[1] * q[3];
    y = p[2] * q[3] + p[3] * q[2] - p[0] * q[1] - p[1] * q[0];
}
__device__ __forceinline__ float form_z(const float (&q)[4]) {
    return q[0] * q[0] - q[1] * q[1] - q[2] * q[2] + q[3] * q[3];
}
__device__ __forceinline__ float form_z2(const float (&p)[4], const float (&q)[4]) {
    return 2.f * (p[0] * q[0] - p[1] * q[1] - p[2] * q[2] + p[3] * q[3]);
}
__device__ __forceinline__ void form_v(const float (&q)[4], float &x, float &y) {
    x = q[0] * q[2] - q[1] * q[3];
    y = q[2] * q[3] + q[0] * q[1];
}
__device__ __forceinline__ void form_v2(const float (&p)[4], const float (&q)[4], float &x,
                                        float &y) {
    x = p[0] * q[2] + p[2] * q[0] - p[1] * q[3] - p[3] * q[1];
    y = p[2] * q[3] + p[3] * q[2] + p[0] * q[1] + p[1] * q[0];
}

// The model of chunk j for a detector (double-float qd, float32 q32): the
// anchor from the certified double-float pointing, the coefficients and
// bounds as described above.  Leaves hx = hy = -1 (HP: elon = -1; every
// sample to the fallback pass) where the model does not apply.  HP: the
// HEALPix form (IxParamsHp) -- phi and z instead of pixel coordinates.
template <bool HP, class Args>
__device__ __forceinline__ void ix_setup(const Args &a, const IxBore *ixb, int j, int n_time,
                                         const dfl (&qd)[4], const float (&q32)[4],
                                         IxParams &p) {
    constexpr float u = kU;
    const int ta = j * kIxLen, tb = min(ta + kIxLen, n_time - 1);
    {
        float4 *w = reinterpret_cast<float4 *>(&p);
#pragma unroll
        for (int k = 0; k < (int)(sizeof(IxParams) / 16); k++) w[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    p.ta = ta;
    p.inv_len = tb > ta ? 1.f / (float)(tb - ta) : 0.f;
    p.hx = p.hy = -1.f;   // HP: elon = z1 = -1 (the slot's third word of P1)
    IxParamsHp &ph = reinterpret_cast<IxParamsHp &>(p);
    if (HP) ph.elon = -1.f;
    const double2 lo = __ldg(reinterpret_cast<const double2 *>(a.bore + 4LL * ta));
    const double2 hi = __ldg(reinterpret_cast<const double2 *>(a.bore + 4LL * ta) + 1);
    dfl qb[4];
    if (!(df_split(lo.x, qb[0]) & df_split(lo.y, qb[1]) & df_split(hi.x, qb[2]) &
          df_split(hi.y, qb[3])))
        return;
    // Anchor: CAR, the pixel coordinates (xb + fx, yb + fy); HEALPix, phi
    // and z = sin(lat) (the quaternion's form; the reference's z is
    // sin(ASIN(z)), within the table's error of it).
    dfl X, fx{0.f, 0.f}, fy{0.f, 0.f}, za_df{0.f, 0.f};
    int xb = 0, yb = 0;
    if constexpr (!HP) {
        dfl Y, Nc, Ns, D;
        if (!fast_native<SO3G_COORD_CAR>(a.ft, a.fc, qb, qd, X, Y, Nc, Ns, D)) return;
        const dfl xa = df_add(df_mul(X, a.fc.inv_cdx), a.fc.off_x);
        const dfl ya = df_add(df_mul(Y, a.fc.inv_cdy), a.fc.off_y);
        if (!(fabsf(xa.hi) < 1e7f && fabsf(ya.hi) < 1e7f)) return;
        xb = df_floor(xa, fx);
        yb = df_floor(ya, fy);
    } else {
        dfl qa_, qb_, qc_, qd_, Nc, Ns, D;
        df_qmul(qb, qd, qa_, qb_, qc_, qd_);
        za_df = df_dot<4>({qa_, qb_, qc_, qd_}, {qa_, df_neg(qb_), df_neg(qc_), qd_});
        if (!(fabsf(za_df.hi) < 0.95f)) return;
        if (!fast_lon_spin(a.ft, a.fc, qa_, qb_, qc_, qd_, za_df, X, Nc, Ns, D)) return;
    }

    // The model quaternions, float32.
    const IxBore B = ixb[j];
    const float qa[4] = {qb[0].hi, qb[1].hi, qb[2].hi, qb[3].hi};
    const float d1[4] = {B.d1.x, B.d1.y, B.d1.z, B.d1.w};
    const float d2[4] = {B.d2.x, B.d2.y, B.d2.z, B.d2.w};
    float A0[4], A1[4], A2[4];
    qmul32(qa, q32, A0);
    qmul32(d1, q32, A1);
    qmul32(d2, q32, A2);
    const float n0 = norm4(A0), n1 = norm4(A1), n2 = norm4(A2);
    // Model error through the detector rotation, with the float32 rounding
    // of s (<= 2u s) moving the model by <= 2u (|d1| + 2 |d2|).
    const float E = (B.e + 2.f * u * (n1 + 2.f * n2)) * 1.0001f;
    const float Em = n0 + n1 + n2;
    // Effect of the float32 evaluation of the coefficients (absolute, in
    // the forms' units).  A0 is within 10u n0 of q(ta) (x) q_d (2u from
    // rounding both factors, 2 gamma_4 from the product's four-term sums),
    // A1 and A2 within 9u of their norms (d1, d2 are the model's own).
    // Through the polar forms (|2B_w| <= sqrt2, |2B_Z| <= 2) and their
    // four-term sums: W1 within 33u n0 n1, W2 within 34u n0 n2 + 17u n1^2,
    // W3 within 31u n1 n2, Z1 within 46u n0 n1, Z2 within 47u n0 n2 + 23u
    // n1^2, Z3 within 44u n1 n2.
    const float ecoef = 48.f * u * (n0 * (n1 + n2) + n1 * (n1 + n2));
    // W0 and Z0 are evaluated from A0: W0 to 17u n0^2 (relative 17u n0^2 /
    // |W0| once divided out), Z0 to 24u n0^2 (moving the asin
    // coefficients).
    const float rel0 = 17.f * u * n0 * n0;
    const float dZ0 = 24.f * u * n0 * n0;

    // Longitude: w(s) = W0 + W1 s + W2 s^2 + W3 s^3 (+ W4 s^4).
    float w0x, w0y, w1x, w1y, w2x, w2y, w3x, w3y, t0x, t0y;
    form_w(A0, w0x, w0y);
    form_w2(A0, A1, w1x, w1y);
    form_w(A1, w2x, w2y);
    form_w2(A0, A2, t0x, t0y);
    w2x += t0x;
    w2y += t0y;
    form_w2(A1, A2, w3x, w3y);
    const float w0a2 = w0x * w0x + w0y * w0y;
    const float w0a = sqrtf(w0a2);
    if (!(w0a > 0.1f)) return;                     // |sin lat| >~ 0.98
    const float ir = 1.f / w0a2;
    const float c1r = (w1x * w0x + w1y * w0y) * ir, c1i = (w1y * w0x - w1x * w0y) * ir;
    const float c2r = (w2x * w0x + w2y * w0y) * ir, c2i = (w2y * w0x - w2x * w0y) * ir;
    const float c3r = (w3x * w0x + w3y * w0y) * ir, c3i = (w3y * w0x - w3x * w0y) * ir;
    const float s2 = 1.41421356f;
    // Dropped: W4 = w(A2) (|w(q)| <= |q|^2 / sqrt2) and the model error E.
    const float eta = (n2 * n2 / s2 + s2 * Em * E + E * E / s2) / w0a;
    const float c1a = sqrtf(c1r * c1r + c1i * c1i), c2a = sqrtf(c2r * c2r + c2i * c2i);
    const float c3a = sqrtf(c3r * c3r + c3i * c3i);
    const float zmax = c1a + c2a + c3a + eta + ecoef / w0a;
    if (!(zmax < 0.05f)) return;
    const float dlmax = zmax * (1.f + zmax);
    // atan2 seam: lon stays inside (-pi, pi) over the chunk.
    if (!(fabsf(X.hi) + dlmax < 3.1405f)) return;
    // Per sample the series Im(z - z^2/2 + z^3/3), z = c1 s + c2 s^2 +
    // c3 s^3, is evaluated as its expansion in s cut after s^3 (pixels:
    // x = xf + s (b1 + s (b2 + s b3))):
    //   b1 = Im c1,  b2 = Im c2 - Im(c1^2)/2,
    //   b3 = Im c3 - Im(c1 c2) + Im(c1^3)/3;
    // the cut terms of z^2 / 2 and z^3 / 3 (those of degree >= 4 in s) are
    // within (zc^2 - |c1|(|c1| + 2|c2|)) / 2 + (zc^3 - |c1|^3) / 3, zc =
    // |c1| + |c2| + |c3|.
    const float icxs = HP ? 1.f : a.mc.inv_cdx, icys = HP ? 1.f : a.mc.inv_cdy;
    const float b1 = c1i * icxs;
    const float b2 = (c2i - c1r * c1i) * icxs;
    const float b3 = (c3i + c1i * (c1r * c1r - c1i * c1i * (1.f / 3.f)) -
                      (c1r * c2i + c1i * c2r)) * icxs;
    const float zc = c1a + c2a + c3a;
    const float cut_lon = 0.5f * (zc * zc - c1a * (c1a + 2.f * c2a)) +
                          (zc * zc * zc - c1a * c1a * c1a) * (1.f / 3.f);
    // Series remainder, the cut terms, the dropped terms (eta) and the
    // coefficients' errors through the series' derivative (<= 1 + 2|z|):
    // W1, W2's absolute errors, W0's relative error and the division's
    // roundings (6u |c|); and the ATAN2 table's interpolation error at both
    // ends (h^2/8 max|atan''| = 3.0e-10).
    const float z2m = zmax * zmax;
    const float lon_err = z2m * z2m / (4.f * (1.f - zmax)) + cut_lon + eta * (1.f + 2.f * zmax) +
                          (ecoef / w0a + (rel0 / w0a + 6.f * u) * zmax) * (1.f + 2.f * zmax) +
                          2.f * 3.1e-10f;
    const float icx = fabsf(icxs), icy = fabsf(icys);
    // In pixels: lon_err, the roundings of b1..b3 (<= 5u each, |b1| + |b2|
    // + |b3| <= (zmax + zmax^2 + zmax^3) / cdelt), of the float32 1/cdelt
    // and of the per-sample Horner steps (4u of dlmax / cdelt, u of x).
    const float bx = 1.5f * (lon_err * icx + 1e-7f + 8.f * u * zmax * (1.f + zmax) * icx +
                             u * (4.f * dlmax * icx + 2.f));
    // HEALPix: lon itself per sample (radians), lon_a + the cubic: lon_err,
    // the anchor's float32 rounding (and double-float's 1e-12), b1..b3's
    // roundings, the Horner steps and the final sum.
    const float lon_a = X.hi + X.lo;
    const float elon = lon_err + 8.f * u * zmax * (1.f + zmax) + 4.f * u * dlmax +
                       2.f * u * (fabsf(lon_a) + dlmax) + 1e-12f;

    // Latitude: Z(s) = Z0 + Z1 s + Z2 s^2 + Z3 s^3 (+ Z4 s^4).
    const float Z0 = form_z(A0);
    const float Z1 = form_z2(A0, A1);
    const float Z2 = form_z(A1) + form_z2(A0, A2);
    const float Z3 = form_z2(A1, A2);
    // Dropped: Z4 = Z(A2) (|Z(q)| <= |q|^2) and the model error.
    const float etaZ = n2 * n2 + 2.f * Em * E + E * E;
    const float dzmax = fabsf(Z1) + fabsf(Z2) + fabsf(Z3) + etaZ + ecoef;
    const float Zm = fabsf(Z0) + dzmax + 1e-6f;
    if (!(Zm < 0.95f)) return;

    // asin's Taylor coefficients at Z0: asin' = (1-Z^2)^-1/2, asin'' =
    // Z (1-Z^2)^-3/2, asin''' = (1+2Z^2)(1-Z^2)^-5/2, asin'''' = Z (9+6Z^2)
    // (1-Z^2)^-7/2, all increasing in |Z|; their bounds at Zm.
    const float om = 1.f - Z0 * Z0;
    const float k1 = rsqrtf(om), k1c = k1 * k1 * k1;
    const float k2 = 0.5f * Z0 * k1c;
    const float k3 = (1.f + 2.f * Z0 * Z0) * k1c * k1 * k1 * (1.f / 6.f);
    const float omm = 1.f - Zm * Zm;
    const float r = rsqrtf(omm), r3 = r * r * r, r5 = r3 * r * r;
    const float m4 = Zm * (9.f + 6.f * Zm * Zm) * r5 * r * r;
    const float k1m = r, k2m = 0.5f * Zm * r3, k3m = (1.f + 2.f * Zm * Zm) * r5 * (1.f / 6.f);
    const float dzm = dzmax + etaZ + ecoef;
    const float dlatmax = dzmax * (k1m + dzmax * (k2m + dzmax * k3m));
    // Table interpolation error of ASIN at both ends: h^2 / 8 max|asin''|,
    // h = 1 / (kLutN - 1).
    const float h2_8 = 1.f / (8.f * 16383.f * 16383.f);
    const float dz2 = dzmax * dzmax;
    // Per sample k1 dZ + k2 dZ^2 + k3 dZ^3, dZ = Z1 s + Z2 s^2 + Z3 s^3,
    // is evaluated as its expansion in s cut after s^3 (pixels: y = yf +
    // s (e1 + s (e2 + s e3))):  e1 = k1 Z1,  e2 = k1 Z2 + k2 Z1^2,
    // e3 = k1 Z3 + 2 k2 Z1 Z2 + k3 Z1^3;  the cut terms are within
    // k2 (dc^2 - |Z1|(|Z1| + 2|Z2|)) + k3 (dc^3 - |Z1|^3), dc = |Z1| + |Z2|
    // + |Z3|.
    const float Z1a = fabsf(Z1), Z2a = fabsf(Z2), dc = Z1a + Z2a + fabsf(Z3);
    const float e1 = k1 * Z1 * icys;
    const float e2 = (k1 * Z2 + k2 * Z1 * Z1) * icys;
    const float e3 = (k1 * Z3 + 2.f * k2 * Z1 * Z2 + k3 * Z1 * Z1 * Z1) * icys;
    const float cut_lat =
        k2m * (dc * dc - Z1a * (Z1a + 2.f * Z2a)) + k3m * (dc * dc * dc - Z1a * Z1a * Z1a);
    // Series remainder; the cut terms; dZ's errors through the series'
    // derivative; Z0's error through the coefficients (d k_n / dZ0 = (n + 1)
    // k_(n+1)); the roundings of k1..k3 and e1..e3 (32u |dlat|); the ASIN
    // table at both ends and the anchor.
    const float lat_err = dz2 * dz2 * m4 / 24.f + cut_lat +
                          (etaZ + ecoef) * (k1m + 2.f * k2m * dzm + 3.f * k3m * dzm * dzm) +
                          dZ0 * dzm * (2.f * k2m + dzm * (3.f * k3m + dzm * m4 / 6.f)) +
                          32.f * u * dlatmax + 2.f * (h2_8 * Zm * r3 + 1e-15f);
    // In pixels, with the float32 1/cdelt and the Horner steps.
    const float by = 1.5f * (lat_err * icy + 1e-7f + u * (4.f * dlatmax * icy + 2.f));

    // Spin: v(s) = V0 + V1 s + V2 s^2 + V3 s^3; the dropped V4 = v(A2) and
    // the model error must stay below 1e-7 of |v| for the float32 contract.
    float v0x, v0y, v1x, v1y, v2x, v2y, v3x, v3y;
    form_v(A0, v0x, v0y);
    form_v2(A0, A1, v1x, v1y);
    form_v(A1, v2x, v2y);
    form_v2(A0, A2, t0x, t0y);
    v2x += t0x;
    v2y += t0y;
    form_v2(A1, A2, v3x, v3y);
    const float v0a = sqrtf(v0x * v0x + v0y * v0y);
    if (!((n2 * n2 / s2 + s2 * Em * E + E * E / s2) < 1e-7f * v0a)) return;

    if constexpr (HP) {
        // z itself per sample, z_a + s (Z1 + s Z2): the dropped terms and
        // coefficient errors (etaZ + ecoef), the reference's z =
        // sin(ASIN(z)) against z (the ASIN table's h^2/8 max|asin''|,
        // twice), the anchor's float32 rounding and the Horner steps.
        const float z_a = za_df.hi + za_df.lo;
        const float ez = etaZ + ecoef + 2.f * h2_8 * Zm * r3 + 1e-12f +
                         u * (2.f * fabsf(z_a) + 5.f * dzmax);
        ph.lon_a = lon_a;
        ph.b1 = b1;
        ph.b2 = b2;
        ph.b3 = b3;
        ph.z_a = z_a;
        ph.z1 = Z1;
        ph.z2 = Z2;
        ph.z3 = Z3;
        ph.v3r = v3x;
        ph.v3i = v3y;
        ph.v0r = v0x;
        ph.v0i = v0y;
        ph.v1r = v1x;
        ph.v1i = v1y;
        ph.v2r = v2x;
        ph.v2i = v2y;
        ph.ez = ez;
        ph.elon = elon;
        return;
    }
    p.xf = fx.hi + fx.lo;
    p.yf = fy.hi + fy.lo;
    p.xb = xb;
    p.yb = yb;
    p.b1 = b1;
    p.b2 = b2;
    p.b3 = b3;
    p.e1 = e1;
    p.e2 = e2;
    p.e3 = e3;
    p.v0r = v0x;
    p.v0i = v0y;
    p.v1r = v1x;
    p.v1i = v1y;
    p.v2r = v2x;
    p.v2i = v2y;
    p.v3r = v3x;
    p.v3i = v3y;
    p.hx = 0.5f - bx;
    p.hy = 0.5f - by;
}

// One sample of a modelled chunk at s = (t - ta) / (tb - ta) (computed by
// the caller as (float)(t - ta) * inv_len: within 2u of s): pixel (key =
// iy * nx + ix, on = on the map) and the spin factors of an NC-component
// map (T; Q, U; or T, Q, U); false when its pixel is not certified.  The
// fraction r of a pixel coordinate is certified when |r - 1/2| < 1/2 -
// bound (r - 1/2 and 1/2 - bound are rounded by at most 2^-25, well inside
// the bound's 1e-7 term).  P = PX_FLAT_T_NN: the tiled pixelizor's rule
// (int() truncation, src/Projection.cxx:1124-1138): on for coordinates in
// (-1, n), those in (-1, 0) landing in row or column 0 -- a certified floor
// of -1 lies strictly inside (-1, 0); key is the parent map's iy * nx + ix.
template <int P, int NC>
__device__ __forceinline__ bool ix_eval(const IxParams &p, float s, const DGeom &g, float T,
                                        float Pr, int &key, bool &on, float (&pf)[3]) {
    const float4 *w = reinterpret_cast<const float4 *>(&p);
    const float4 P0 = w[0], P1 = w[1], P3 = w[3], P5 = w[5];
    const float x = fmaf(s, fmaf(s, fmaf(s, P1.x, P0.w), P0.z), P0.x);
    const float y = fmaf(s, fmaf(s, fmaf(s, P1.w, P1.z), P1.y), P0.y);
    const float fxl = floorf(x), fyl = floorf(y);
    const bool ok = fabsf((x - fxl) - 0.5f) < P3.z && fabsf((y - fyl) - 0.5f) < P3.w;
    int ix = __float_as_int(P5.x) + (int)fxl, iy = __float_as_int(P5.y) + (int)fyl;
    if constexpr (P == PX_FLAT_T_NN) {
        on = (unsigned)(ix + 1) < (unsigned)(g.nx + 1) && (unsigned)(iy + 1) < (unsigned)(g.ny + 1);
        ix = max(ix, 0);
        iy = max(iy, 0);
    } else {
        on = (unsigned)ix < (unsigned)g.nx && (unsigned)iy < (unsigned)g.ny;
    }
    key = iy * g.nx + ix;
    if constexpr (NC == 1) {
        pf[0] = T;
        pf[1] = pf[2] = 0.f;
    } else {
        const float4 P2 = w[2], P4 = w[4];
        const float vr = fmaf(s, fmaf(s, fmaf(s, P4.x, P3.x), P2.z), P2.x);
        const float vi = fmaf(s, fmaf(s, fmaf(s, P4.y, P3.y), P2.w), P2.y);
        const float k = Pr * rcp_approx(fmaf(vr, vr, vi * vi));
        const float v1 = fmaf(vr, vr, -vi * vi) * k, v2 = 2.f * vr * vi * k;
        if constexpr (NC == 2) {
            pf[0] = v1;
            pf[1] = v2;
            pf[2] = 0.f;
        } else {
            pf[0] = T;
            pf[1] = v1;
            pf[2] = v2;
        }
    }
    return ok;
}

// The HEALPix form of ix_eval (IxParamsHp): phi and z from their
// polynomials, the pixel index (always on the map) from hp_pixel_f32 --
// for a tiled map (P = PX_HP_T) the parent map's NEST index.
template <int P, int NC>
__device__ __forceinline__ bool ix_eval_hp(const IxParams &pr, float s, const DGeom &g, float T,
                                           float Pr, int &key, float (&pf)[3]) {
    const float4 *w = reinterpret_cast<const float4 *>(&pr);
    const float4 P0 = w[0], P1 = w[1], P3 = w[3];
    const float lon = fmaf(s, fmaf(s, fmaf(s, P0.w, P0.z), P0.y), P0.x);
    const float z = fmaf(s, fmaf(s, fmaf(s, P3.w, P1.z), P1.y), P1.x);
    int pix[1] = {0};
    const bool ok =
        P1.w >= 0.f && hp_pixel_f32<P, P == PX_HP_T, true>(g, lon, P1.w, z, P3.z, 0.f, 0.f, pix);
    key = pix[0];
    if constexpr (NC == 1) {
        pf[0] = T;
        pf[1] = pf[2] = 0.f;
    } else {
        const float4 P2 = w[2], P4 = w[4];
        const float vr = fmaf(s, fmaf(s, fmaf(s, P4.x, P3.x), P2.z), P2.x);
        const float vi = fmaf(s, fmaf(s, fmaf(s, P4.y, P3.y), P2.w), P2.y);
        const float k = Pr * rcp_approx(fmaf(vr, vr, vi * vi));
        const float v1 = fmaf(vr, vr, -vi * vi) * k, v2 = 2.f * vr * vi * k;
        if constexpr (NC == 2) {
            pf[0] = v1;
            pf[1] = v2;
            pf[2] = 0.f;
        } else {
            pf[0] = T;
            pf[1] = v1;
            pf[2] = v2;
        }
    }
    return ok;
}

// One sample of the chunked pointing for pixelizor P (CAR nearest or
// HEALPix): ok (certified), key (map index; tiled maps: the parent map's
// index), on, spin factors.
template <int P, int NC>
__device__ __forceinline__ bool ix_sample(const IxParams &p, float s, const DGeom &g, float T,
                                          float Pr, int &key, bool &on, float (&pf)[3]) {
    if constexpr (P == PX_HP_NT || P == PX_HP_T) {
        on = true;
        return ix_eval_hp<P, NC>(p, s, g, T, Pr, key, pf);
    } else {
        return ix_eval<P, NC>(p, s, g, T, Pr, key, on, pf);
    }
}

// s of sample tq + i of a chunk: (float)(tq + i - ta) * inv_len, the
// difference formed exactly (|tq - ta| < 2^24).
__device__ __forceinline__ float ix_s(const IxParams &p, int tq, int i) {
    const float4 P4 = reinterpret_cast<const float4 *>(&p)[4];
    return ((float)(tq - __float_as_int(P4.w)) + (float)i) * P4.z;
}

// The boresight models of a call's chunks, in stream-ordered memory; NULL
// when the allocation fails (the caller takes the per-sample path).
inline IxBore *ix_bore_models(const double *bore, int n_time, cudaStream_t stream) {
    const int n_chunks = (n_time + kIxLen - 1) / kIxLen;
    IxBore *p = nullptr;
    if (n_chunks <= 0 ||
        cudaMallocAsync(reinterpret_cast<void **>(&p), sizeof(IxBore) * (size_t)n_chunks,
                        stream) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    k_ix_bore<<<(n_chunks + 127) / 128, 128, 0, stream>>>(bore, n_time, n_chunks, p);
    if (after_launch("boresight chunk models") != SO3G_OK) {
        cudaFreeAsync(p, stream);
        clear_error();
        return nullptr;
    }
    return p;
}

}  // namespace

}  // namespace so3g
