// api.cu -- library state of the C ABI: trig tables per device, error
// reporting, launch accounting and pixelization validation.

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "host.h"

namespace so3g {

namespace {

thread_local std::string t_err;
std::atomic<long long> g_launches{0};
// Measured on a CAR TQU map of 1' pixels scanned at 1 deg/s, 200 Hz (mixed
// pointing): at 6.4M samples per call the per-sample tier took 0.27 / 0.26
// ms (to_map / from_map) and the chunked kernels 0.37 / 0.38; at 2e7 0.51 /
// 0.41 against 0.52 / 0.55; at 1e8 1.27 / 1.02 against 0.90 / 0.86.
std::atomic<long long> g_chunked_min{30000000};
std::mutex g_mu;
constexpr int kMaxDevices = 64;
double *g_lut[kMaxDevices] = {nullptr};
float4 *g_fast_lut[kMaxDevices] = {nullptr};
double g_host_lut[2 * kLutN];
bool g_host_lut_ready = false;

// Double-float knots of a table and their forward differences, for the
// certified pointing: (v_hi, v_lo, dv_hi, dv_lo) per knot.
void split(double x, float &hi, float &lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

void fast_knots(const double *v, float4 *out) {
    for (int i = 0; i < kLutN; i++) {
        float vh, vl, dh, dl;
        split(v[i], vh, vl);
        split(i + 1 < kLutN ? v[i + 1] - v[i] : 0., dh, dl);
        out[i] = make_float4(vh, vl, dh, dl);
    }
}

// sin and cos of the asin table's knots as double-floats: the HEALPix
// certified pointing evaluates sin/cos(lat) about the knot below lat.
void sincos_knots(const double *v, float4 *out) {
    for (int i = 0; i < kLutN; i++) {
        float sh, sl, ch, cl;
        split(std::sin(v[i]), sh, sl);
        split(std::cos(v[i]), ch, cl);
        out[i] = make_float4(sh, sl, ch, cl);
    }
}

// asinTable / atan2Table construction (include/so_linterp.h:35-39, 51-56),
// with the host math library, as the reference's static tables
// (src/Projection.cxx:36-38).
void build_host_tables() {
    if (g_host_lut_ready) return;
    const double dx = 1. / (kLutN - 1);
    for (int i = 0; i < kLutN; i++) g_host_lut[i] = std::asin(i * dx);
    for (int i = 0; i < kLutN; i++) g_host_lut[kLutN + i] = std::atan2(i * dx, 1.);
    g_host_lut_ready = true;
}

// The knot tables of the certified pointing (asin, atan2, then sin/cos of
// the asin knots), built once from the host tables.
float4 g_host_knots[3 * kLutN];
bool g_host_knots_ready = false;

void build_host_knots() {
    if (g_host_knots_ready) return;
    build_host_tables();
    fast_knots(g_host_lut, g_host_knots);
    fast_knots(g_host_lut + kLutN, g_host_knots + kLutN);
    sincos_knots(g_host_lut, g_host_knots + 2 * kLutN);
    g_host_knots_ready = true;
}

bool pow2(long long v) { return v > 0 && (v & (v - 1)) == 0; }

}  // namespace

int set_error(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_err = buf;
    return code;
}

void clear_error() { t_err.clear(); }

long long chunked_min_samples() { return g_chunked_min.load(std::memory_order_relaxed); }

int after_launch(const char *what) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(SO3G_ERR_CUDA, "%s: launch failed: %s", what, cudaGetErrorString(e));
    return SO3G_OK;
}

const double *device_lut() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
    return g_lut[dev];
}

FastTables device_fast_tables() {
    int dev = 0;
    FastTables t{nullptr, nullptr, nullptr};
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return t;
    if (g_fast_lut[dev]) {
        t.asin_t = g_fast_lut[dev];
        t.atan2_t = g_fast_lut[dev] + kLutN;
        t.asin_sc = g_fast_lut[dev] + 2 * kLutN;
    }
    return t;
}

FastConst make_fast_const(const DGeom &g) {
    FastConst c;
    const double inv_x = g.cdx != 0. ? 1. / g.cdx : 0., inv_y = g.cdy != 0. ? 1. / g.cdy : 0.;
    split(inv_x, c.inv_cdx.hi, c.inv_cdx.lo);
    split(inv_y, c.inv_cdy.hi, c.inv_cdy.lo);
    split(g.crx - 1 + 0.5, c.off_x.hi, c.off_x.lo);
    split(g.cry - 1 + 0.5, c.off_y.hi, c.off_y.lo);
    split(kPi, c.pi.hi, c.pi.lo);
    split(kPi / 2, c.half_pi.hi, c.half_pi.lo);
    split(1. / (2. * kPi), c.inv_2pi.hi, c.inv_2pi.lo);
    split(1. / 3., c.third.hi, c.third.lo);
    split(2. / 3., c.two_thirds.hi, c.two_thirds.lo);
    return c;
}

MixedConst make_mixed_const(const DGeom &g) {
    MixedConst c;
    c.inv_cdx = g.cdx != 0. ? (float)(1. / g.cdx) : 0.f;
    c.inv_cdy = g.cdy != 0. ? (float)(1. / g.cdy) : 0.f;
    c.off_x = (float)(g.crx - 1 + 0.5);
    c.off_y = (float)(g.cry - 1 + 0.5);
    c.pi = (float)kPi;
    c.half_pi = (float)(kPi / 2);
    return c;
}

int fast_mode(const so3g_pixelization *pz, const FastTables &ft) {
    if (!ft.asin_t) return SO3G_POINTING_EXACT;
    return pz->pointing;
}

namespace {
__global__ void k_bore_f32(const double *bore, float4 *out, int n_time) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_time) return;
    const double2 lo = __ldg(reinterpret_cast<const double2 *>(bore + 4LL * t));
    const double2 hi = __ldg(reinterpret_cast<const double2 *>(bore + 4LL * t) + 1);
    out[t] = make_float4(__double2float_rn(lo.x), __double2float_rn(lo.y),
                         __double2float_rn(hi.x), __double2float_rn(hi.y));
}
}  // namespace

const float4 *bore_f32(const so3g_pixelization *pz, int mode, const double *bore, int n_time,
                       cudaStream_t stream) {
    const int kind = pix_kind(pz);
    const int cs = pz->coord_sys;
    const bool flat_nn = kind == PX_FLAT_NT_NN || kind == PX_FLAT_T_NN;
    const bool hp = kind == PX_HP_NT || kind == PX_HP_T;
    const bool eligible = (hp && cs == SO3G_COORD_CAR) ||
                          (flat_nn && (cs == SO3G_COORD_CAR || cs == SO3G_COORD_TAN ||
                                       cs == SO3G_COORD_ZEA || cs == SO3G_COORD_SIN));
    if (mode != SO3G_POINTING_MIXED || !eligible || n_time <= 0 || !bore) return nullptr;
    float4 *p = nullptr;
    if (cudaMallocAsync(reinterpret_cast<void **>(&p), sizeof(float4) * (size_t)n_time,
                        stream) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    k_bore_f32<<<(n_time + kBlock - 1) / kBlock, kBlock, 0, stream>>>(bore, p, n_time);
    if (after_launch("boresight float32 copy") != SO3G_OK) {
        cudaFreeAsync(p, stream);
        clear_error();
        return nullptr;
    }
    return p;
}

void bore_f32_free(const float4 *p, cudaStream_t stream) {
    if (p) cudaFreeAsync(const_cast<float4 *>(p), stream);
}

int pix_kind(const so3g_pixelization *pz) {
    if (pz->pix_sys == SO3G_PIX_HEALPIX) return pz->tiled ? PX_HP_T : PX_HP_NT;
    return (pz->tiled ? 2 : 0) + (pz->interp == SO3G_INTERP_BILINEAR ? 1 : 0);
}

const double *host_lut() {
    std::lock_guard<std::mutex> lk(g_mu);
    build_host_tables();
    return g_host_lut;
}

const float4 *host_fast_knots() {
    std::lock_guard<std::mutex> lk(g_mu);
    build_host_knots();
    return g_host_knots;
}

int make_geom(const so3g_pixelization *pz, DGeom *g) {
    const double *lut = device_lut();
    if (!lut) return set_error(SO3G_ERR_NOT_INIT, "so3g_init() was not called on this device");
    return make_geom_lut(pz, g, lut);
}

int make_geom_lut(const so3g_pixelization *pz, DGeom *g, const double *lut) {
    if (!pz) return set_error(SO3G_ERR_ARGUMENT, "pixelization is NULL");
    std::memset(g, 0, sizeof(*g));
    if (pz->n_comp < 1 || pz->n_comp > 3)
        return set_error(SO3G_ERR_ARGUMENT, "n_comp must be 1, 2 or 3 (got %d)", pz->n_comp);
    if (pz->coord_sys < SO3G_COORD_FLAT || pz->coord_sys > SO3G_COORD_ZEA)
        return set_error(SO3G_ERR_ARGUMENT, "unknown coordinate system %d", pz->coord_sys);
    if (pz->interp != SO3G_INTERP_NEAREST && pz->interp != SO3G_INTERP_BILINEAR)
        return set_error(SO3G_ERR_ARGUMENT, "unknown interpolation %d", pz->interp);
    if (pz->pointing != SO3G_POINTING_EXACT && pz->pointing != SO3G_POINTING_CERTIFIED &&
        pz->pointing != SO3G_POINTING_MIXED)
        return set_error(SO3G_ERR_ARGUMENT, "unknown pointing mode %d", pz->pointing);
    g->ncomp = pz->n_comp;
    g->lut = lut;
    if (pz->pix_sys == SO3G_PIX_HEALPIX) {
        if (pz->coord_sys != SO3G_COORD_CAR)
            return set_error(SO3G_ERR_ARGUMENT, "HEALPix pixelization needs CAR coordinates");
        if (pz->interp != SO3G_INTERP_NEAREST)
            return set_error(SO3G_ERR_ARGUMENT, "HEALPix supports nearest interpolation only");
        // check_nside, src/Projection.cxx:607-614
        if (!(pz->nside > 0 && pz->nside < 8192 && pow2(pz->nside)))
            return set_error(SO3G_ERR_ARGUMENT, "Invalid nside %d", pz->nside);
        g->nside = pz->nside;
        g->npix = 12LL * pz->nside * pz->nside;
        g->nest = pz->nest ? 1 : 0;
        if (pz->tiled) {
            if (!pz->nest) return set_error(SO3G_ERR_ARGUMENT, "RING not supported for tiled maps");
            if (!(pz->nside_tile > 0 && pz->nside_tile < 8192 && pow2(pz->nside_tile)))
                return set_error(SO3G_ERR_ARGUMENT, "Invalid nside %d", pz->nside_tile);
            if (pz->nside_tile > pz->nside)
                return set_error(SO3G_ERR_ARGUMENT, "Invalid nside_tile %d > nside %d",
                                 pz->nside_tile, pz->nside);
            g->n_tile = (int)(12LL * pz->nside_tile * pz->nside_tile);
            g->nppt = g->npix / g->n_tile;
        }
        return SO3G_OK;
    }
    if (pz->pix_sys != SO3G_PIX_FLAT)
        return set_error(SO3G_ERR_ARGUMENT, "unknown pixel system %d", pz->pix_sys);
    if (pz->naxis[0] < 0 || pz->naxis[1] < 0)
        return set_error(SO3G_ERR_ARGUMENT, "negative map shape");
    g->ny = pz->naxis[0];
    g->nx = pz->naxis[1];
    g->cdy = pz->cdelt[0];
    g->cdx = pz->cdelt[1];
    g->cry = pz->crpix[0];
    g->crx = pz->crpix[1];
    if (pz->tiled) {
        if (pz->tile_shape[0] <= 0 || pz->tile_shape[1] <= 0)
            return set_error(SO3G_ERR_ARGUMENT, "tile shape must be positive");
        g->ty = pz->tile_shape[0];
        g->tx = pz->tile_shape[1];
        g->nty = (g->ny + g->ty - 1) / g->ty;
        g->ntx = (g->nx + g->tx - 1) / g->tx;
        g->n_tile = g->nty * g->ntx;
        if (g->ntx == 0) g->ntx = 1;  // empty map: keeps the tile arithmetic defined
        g->inv_ty = 1.0f / (float)g->ty;
        g->inv_tx = 1.0f / (float)g->tx;
        g->inv_ntx = 1.0f / (float)g->ntx;
    }
    return SO3G_OK;
}

int attach_map(const so3g_pixelization *pz, const so3g_map *m, DGeom *g) {
    if (!m || !m->data) return set_error(SO3G_ERR_ARGUMENT, "map is NULL");
    if (pz->tiled) {
        if (!m->tile_offset)
            return set_error(SO3G_ERR_ARGUMENT, "tiled map needs a tile_offset table");
        if (m->n_tile != g->n_tile)
            return set_error(SO3G_ERR_ARGUMENT, "tiled map has %d tiles; the pixelization has %d",
                             m->n_tile, g->n_tile);
        g->tile_offset = reinterpret_cast<const long long *>(m->tile_offset);
        g->n_tile_map = m->n_tile;
    }
    return SO3G_OK;
}

}  // namespace so3g

using namespace so3g;

extern "C" {

int so3g_abi_version(void) { return SO3G_GB300_ABI_VERSION; }

const char *so3g_last_error(void) { return t_err.c_str(); }

int64_t so3g_launch_count(void) { return (int64_t)g_launches.load(); }

int64_t so3g_set_chunked_min_samples(int64_t n) {
    return (int64_t)g_chunked_min.exchange(n < 0 ? 0 : (long long)n);
}

int so3g_init(void) {
    clear_error();
    std::lock_guard<std::mutex> lk(g_mu);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(SO3G_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return set_error(SO3G_ERR_RANGE, "device %d out of range", dev);
    build_host_tables();
    if (g_lut[dev]) return SO3G_OK;
    double *d = nullptr;
    e = cudaMalloc(&d, sizeof(double) * 2 * kLutN);
    if (e != cudaSuccess) return set_error(SO3G_ERR_CUDA, "cudaMalloc: %s", cudaGetErrorString(e));
    e = cudaMemcpy(d, g_host_lut, sizeof(double) * 2 * kLutN, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return set_error(SO3G_ERR_CUDA, "cudaMemcpy: %s", cudaGetErrorString(e));
    }
    g_lut[dev] = d;
    // Double-float knots for the certified pointing.
    build_host_knots();
    float4 *f = nullptr;
    e = cudaMalloc(&f, sizeof(float4) * 3 * kLutN);
    if (e != cudaSuccess) return set_error(SO3G_ERR_CUDA, "cudaMalloc: %s", cudaGetErrorString(e));
    e = cudaMemcpy(f, g_host_knots, sizeof(float4) * 3 * kLutN, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(f);
        return set_error(SO3G_ERR_CUDA, "cudaMemcpy: %s", cudaGetErrorString(e));
    }
    g_fast_lut[dev] = f;
    // Keep freed stream-ordered allocations (the boresight copies of the
    // mixed pointing) in this process's pool instead of returning them to
    // the driver at every synchronisation.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        unsigned long long keep = 1ULL << 30;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
    return SO3G_OK;
}

int so3g_host_access(const void *ptr, int32_t *mode) {
    clear_error();
    if (!mode) return set_error(SO3G_ERR_ARGUMENT, "mode is NULL");
    *mode = SO3G_HOST_NONE;
    if (!ptr) return SO3G_OK;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(SO3G_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    cudaPointerAttributes at{};
    e = cudaPointerGetAttributes(&at, ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(SO3G_ERR_CUDA, "cudaPointerGetAttributes: %s", cudaGetErrorString(e));
    }
    if (at.type == cudaMemoryTypeHost) {
        // Page-locked: usable in kernels when mapped at the same address.
        if (at.devicePointer == ptr) *mode = SO3G_HOST_MAPPED;
        return SO3G_OK;
    }
    if (at.type == cudaMemoryTypeUnregistered) {
        int pageable = 0;
        e = cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_error(SO3G_ERR_CUDA, "cudaDeviceGetAttribute: %s", cudaGetErrorString(e));
        }
        if (pageable == 1) *mode = SO3G_HOST_PAGEABLE;
    }
    return SO3G_OK;
}

int so3g_get_trig_tables(double *asin_vals, double *atan2_vals, int32_t n) {
    clear_error();
    if (n != kLutN) return set_error(SO3G_ERR_ARGUMENT, "table size is %d", kLutN);
    {
        std::lock_guard<std::mutex> lk(g_mu);
        build_host_tables();
    }
    std::memcpy(asin_vals, g_host_lut, sizeof(double) * kLutN);
    std::memcpy(atan2_vals, g_host_lut + kLutN, sizeof(double) * kLutN);
    return SO3G_OK;
}

}  // extern "C"
