// sightline.cu -- boresight quaternions of CelestialSightLine.for_horizon and
// naive_az_el (python/proj/coords.py:99-125, 190-209) on the device, and the
// quat x vector product of Projectionist._cache_q_fp_to_native
// (python/proj/wcs.py:140-148).
//
// The Python layer evaluates these as numpy expressions: euler(axis, angle)
// = (cos(angle/2), .., sin(angle/2) at index axis+1, ..) per sample, then
// Hamilton products left to right.  The kernels repeat those operations in
// the same order, in float64 without fused multiply-adds (the library is
// built with -fmad=false), from the same host-formed constants.  Only the
// device's cos/sin may differ from the host's in the last bit.

#include "host.h"

namespace so3g {

namespace {

// euler(axis, angle) (python/proj/quat.py:15-44): the rotation by `angle`
// about cartesian axis `axis`.
__device__ __forceinline__ QuatD euler_q(int axis, double angle) {
    double s, c;
    sincos(angle / 2, &s, &c);
    QuatD q{c, 0., 0., 0.};
    if (axis == 0) q.b = s;
    else if (axis == 1) q.c = s;
    else q.d = s;
    return q;
}

__device__ __forceinline__ QuatD quat_of(const double (&v)[4]) {
    return QuatD{v[0], v[1], v[2], v[3]};
}

__global__ void k_boresight(so3g_sightline sl, const double *t, const double *az,
                            const double *el, const double *roll, long long n, double *out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double r = roll ? roll[i] : sl.roll;
        QuatD q;
        if (sl.kind == SO3G_SIGHT_NAIVE_AZEL) {
            // J = (t - ERA_EPOCH) / 86400; era = polyval(ERA_POLY, J)
            // (= (0 * J + p0) * J + p1); lst = era + site.lon * DEG.
            const double J = (t[i] - sl.era_epoch) / 86400;
            const double era = (0. * J + sl.era_poly[0]) * J + sl.era_poly[1];
            const double lst = era + sl.site_lon_rad;
            q = qmul(euler_q(2, lst), quat_of(sl.q_site_lat));
            q = qmul(q, quat_of(sl.q_pi));
            q = qmul(q, euler_q(2, -az[i]));
        } else {
            q = euler_q(2, -az[i]);
        }
        q = qmul(q, euler_q(1, M_PI / 2 - el[i]));
        q = qmul(q, euler_q(2, r));
        if (sl.has_left) q = qmul(quat_of(sl.q_left), q);
        double2 *o = reinterpret_cast<double2 *>(out + 4 * i);
        o[0] = make_double2(q.a, q.b);
        o[1] = make_double2(q.c, q.d);
    }
}

__global__ void k_quat_left_multiply(QuatD left, const double *in, long long n, double *out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const QuatD q = qmul(left, load_quat(in + 4 * i));
        double2 *o = reinterpret_cast<double2 *>(out + 4 * i);
        o[0] = make_double2(q.a, q.b);
        o[1] = make_double2(q.c, q.d);
    }
}

// Grid for n samples: at most 8 waves of 152 SMs x 8 blocks of kBlock
// threads; the kernels stride over the rest.
unsigned grid_for(long long n) {
    const long long want = (n + kBlock - 1) / kBlock;
    const long long cap = 8LL * 152 * 8;
    return (unsigned)(want < cap ? want : cap);
}

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

}  // namespace so3g

extern "C" int so3g_boresight(const so3g_sightline *sl, const double *t, const double *az,
                              const double *el, const double *roll, int64_t n, double *q_out,
                              void *stream) {
    using namespace so3g;
    clear_error();
    if (!sl) return set_error(SO3G_ERR_ARGUMENT, "NULL sight line");
    if (sl->kind != SO3G_SIGHT_HORIZON && sl->kind != SO3G_SIGHT_NAIVE_AZEL)
        return set_error(SO3G_ERR_ARGUMENT, "unknown sight-line kind %d", sl->kind);
    if (n < 0) return set_error(SO3G_ERR_ARGUMENT, "negative sample count");
    if (n == 0) return SO3G_OK;
    if (!az || !el || !q_out || (sl->kind == SO3G_SIGHT_NAIVE_AZEL && !t))
        return set_error(SO3G_ERR_ARGUMENT, "NULL input array");
    if (!aligned16(q_out)) return set_error(SO3G_ERR_ARGUMENT, "q_out is not 16-byte aligned");
    k_boresight<<<grid_for(n), kBlock, 0, (cudaStream_t)stream>>>(*sl, t, az, el, roll, n,
                                                                  q_out);
    return after_launch("boresight");
}

extern "C" int so3g_quat_left_multiply(const double *q_left, const double *q_in, int64_t n,
                                       double *q_out, void *stream) {
    using namespace so3g;
    clear_error();
    if (n < 0) return set_error(SO3G_ERR_ARGUMENT, "negative count");
    if (n == 0) return SO3G_OK;
    if (!q_left || !q_in || !q_out) return set_error(SO3G_ERR_ARGUMENT, "NULL array");
    if (!aligned16(q_in) || !aligned16(q_out))
        return set_error(SO3G_ERR_ARGUMENT, "quaternion arrays must be 16-byte aligned");
    const QuatD left{q_left[0], q_left[1], q_left[2], q_left[3]};
    k_quat_left_multiply<<<grid_for(n), kBlock, 0, (cudaStream_t)stream>>>(left, q_in, n,
                                                                           q_out);
    return after_launch("quaternion product");
}
