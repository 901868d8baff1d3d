// host.h -- host-side helpers shared by the translation units of the C ABI.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/so3g_gb300.h"
#include "fastpoint.cuh"
#include "mixedpoint.cuh"

namespace so3g {

// Records `msg` as this thread's last error and returns `code`.
int set_error(int code, const char *fmt, ...);
// Clears the last error (each entry point starts with it).
void clear_error();
// Checks cudaGetLastError() after a launch; counts the launch.
int after_launch(const char *what);
// Smallest call (detectors x samples) that takes the chunked mixed kernels
// (so3g_set_chunked_min_samples); smaller calls take the per-sample float32
// tier, whose fixed cost per call is lower.
long long chunked_min_samples();
// Per-device trig table (asin then atan2, 2 x kLutN float64), or NULL.
const double *device_lut();

// Validates a pixelization and fills the device geometry (without the map),
// using the trig tables uploaded by so3g_init().
int make_geom(const so3g_pixelization *pz, DGeom *g);
// The same with the caller's device copy of the trig tables.
int make_geom_lut(const so3g_pixelization *pz, DGeom *g, const double *lut);
// The host trig tables (asin then atan2, 2 x kLutN float64).
const double *host_lut();
// The host copy of the certified pointing's knot tables (asin, atan2, then
// sin/cos of the asin knots: 3 x kLutN float4), the layout FastTables
// points into.
const float4 *host_fast_knots();
// Double-float knot tables of the certified pointing on the current device
// (uploaded by so3g_init), or NULL pointers.
FastTables device_fast_tables();
// Double-float pixelizor constants of the certified pointing.
FastConst make_fast_const(const DGeom &g);
// Float32 pixelizor constants of the mixed pointing.
MixedConst make_mixed_const(const DGeom &g);
// The pointing mode a kernel runs for a pixelization (0 exact, 1 certified,
// 2 mixed): the exact path when the double-float tables are missing.
int fast_mode(const so3g_pixelization *pz, const FastTables &ft);
// Float32 copy of a boresight (n_time quaternions, rounded to nearest) for
// the mixed pointing, in stream-ordered device memory; NULL when the
// pixelization does not use it or the allocation fails (the kernels then
// convert the float64 boresight themselves).  Release with bore_f32_free.
const float4 *bore_f32(const so3g_pixelization *pz, int mode, const double *bore,
                       int n_time, cudaStream_t stream);
void bore_f32_free(const float4 *p, cudaStream_t stream);
// Adds the map's tile table to the geometry; checks the tile count.
int attach_map(const so3g_pixelization *pz, const so3g_map *m, DGeom *g);
// Pixelizor kind (PX_*) of a pixelization.
int pix_kind(const so3g_pixelization *pz);

// Block and piece sizes of the per-segment projection kernels.
constexpr int kBlock = 256;
constexpr int kMinPiece = 4096;

// Piece length for n_seg segments of up to max_len samples: at least
// kMinPiece, doubled (up to 32768) while the grid would keep over 16 waves
// of resident blocks (fewer pieces amortise the per-piece set-up), and as
// far as needed to keep a segment within 65535 pieces.
inline int piece_len(long long max_len, long long n_seg = 1) {
    constexpr long long kManyBlocks = 16LL * 152 * 5;
    long long p = kMinPiece;
    while (p < 32768 && n_seg * ((max_len + 2 * p - 1) / (2 * p)) >= kManyBlocks) p *= 2;
    while ((max_len + p - 1) / p > 65535) p *= 2;
    return (int)p;
}

// Launch dispatch over (coordinate system, pixelizor): F is a functor with
// a templated operator()<C, P>() returning int.
template <class F>
int dispatch_cp(int coord, int kind, F &&f) {
#define SO3G_P(C)                                                   \
    switch (kind) {                                                  \
    case PX_FLAT_NT_NN: return f.template run<C, PX_FLAT_NT_NN>();   \
    case PX_FLAT_NT_BL: return f.template run<C, PX_FLAT_NT_BL>();   \
    case PX_FLAT_T_NN: return f.template run<C, PX_FLAT_T_NN>();     \
    case PX_FLAT_T_BL: return f.template run<C, PX_FLAT_T_BL>();     \
    default: break;                                                  \
    }
    if (kind == PX_HP_NT) return f.template run<SO3G_COORD_CAR, PX_HP_NT>();
    if (kind == PX_HP_T) return f.template run<SO3G_COORD_CAR, PX_HP_T>();
    switch (coord) {
    case SO3G_COORD_FLAT: SO3G_P(SO3G_COORD_FLAT) break;
    case SO3G_COORD_QUAT: SO3G_P(SO3G_COORD_QUAT) break;
    case SO3G_COORD_CAR: SO3G_P(SO3G_COORD_CAR) break;
    case SO3G_COORD_CEA: SO3G_P(SO3G_COORD_CEA) break;
    case SO3G_COORD_ARC: SO3G_P(SO3G_COORD_ARC) break;
    case SO3G_COORD_SIN: SO3G_P(SO3G_COORD_SIN) break;
    case SO3G_COORD_TAN: SO3G_P(SO3G_COORD_TAN) break;
    case SO3G_COORD_ZEA: SO3G_P(SO3G_COORD_ZEA) break;
    default: break;
    }
#undef SO3G_P
    return set_error(SO3G_ERR_ARGUMENT, "unsupported coordinate system %d / pixelizor %d",
                     coord, kind);
}

}  // namespace so3g
