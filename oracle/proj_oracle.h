/*
 * proj_oracle.h -- CPU oracle for the so3g ProjectionEngine hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, operation for
 * operation, the arithmetic of so3g's src/Projection.cxx (Pointer<C>,
 * Pixelizor2_Flat, Pixelizor_Healpix, spin_proj_factors, to_map,
 * to_weight_map, from_map, ProjEng_Precomp), include/so_linterp.h and the
 * HEALPix ang2pix routines of src/healpix_bare.c.  It is used by the tests
 * to check the CUDA library, by __graft_entry__.smoke() to check one small
 * projection, and by bench.py as the timed CPU baseline.  The product never links or calls
 * it.  All pointers here are HOST pointers; the parameter structs are the
 * ones of include/so3g_gb300.h.
 *
 * Build: g++ -O2 -ffp-contract=off -fopenmp (no FMA contraction, so the
 * float64 results equal those of an x86-64 build of the reference).
 */
#ifndef SO3G_PROJ_ORACLE_H
#define SO3G_PROJ_ORACLE_H

#include <stdint.h>
#include "../include/so3g_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Thread schedule of to_map/to_weight_map: the [bunch][thread][det] ranges
 * of derive_ranges (src/Projection.cxx:1856-1922).  Segment k is
 * (det, start, end) = seg[3k..3k+2]; thread j owns segments
 * [thread_offset[j], thread_offset[j+1]); bunch b owns threads
 * [bunch_offset[b], bunch_offset[b+1]).  Bunches run one after the other,
 * the threads of a bunch in parallel (OpenMP).  NULL = one bunch, one
 * thread, all samples of all detectors. */
typedef struct orc_sched {
    const int32_t *seg;
    int32_t        n_seg;
    int32_t        n_thread;
    const int32_t *thread_offset;
    int32_t        n_bunch;
    int32_t        _pad;
    const int32_t *bunch_offset;
} orc_sched;

int    orc_init(void);
int    orc_set_threads(int n);
int    orc_get_tables(double *asin_vals, double *atan2_vals, int32_t n);
double orc_asin(double x);
double orc_atan2(double y, double x);
int64_t orc_ang2pix(int64_t nside, int32_t nest, double theta, double phi);
const char *orc_last_error(void);

int orc_coords(const so3g_pixelization *pz, const double *bore, int32_t n_time,
               const double *dets, int32_t n_det, double *coords);
int orc_pixels(const so3g_pixelization *pz, const double *bore, int32_t n_time,
               const double *dets, int32_t n_det, int32_t *pixel);
int orc_pointing_matrix(const so3g_pixelization *pz, const double *bore,
                        int32_t n_time, const double *dets, int32_t n_det,
                        const float *response, int32_t *pixel, float *proj);
int orc_tile_hits(const so3g_pixelization *pz, const double *bore, int32_t n_time,
                  const double *dets, int32_t n_det, int64_t *hits, int32_t n_tile);
int orc_domain_labels(const so3g_pixelization *pz, const double *bore,
                      int32_t n_time, const double *dets, int32_t n_det,
                      int32_t mode, int32_t n_domain, const so3g_map *dmap,
                      const int32_t *tile_domain, int32_t n_tile, int32_t *label);

/* err: 4 x int32 as the device error record of the CUDA library. */
int orc_to_map(const so3g_pixelization *pz, const double *bore, int32_t n_time,
               const double *dets, int32_t n_det, const float *response,
               const float *signal, int64_t sig_det_stride,
               const float *det_weights, const orc_sched *sched,
               const so3g_map *map, int32_t *err);
int orc_to_weight_map(const so3g_pixelization *pz, const double *bore,
                      int32_t n_time, const double *dets, int32_t n_det,
                      const float *response, const float *det_weights,
                      const orc_sched *sched, const so3g_map *map, int32_t *err);
int orc_from_map(const so3g_pixelization *pz, const double *bore, int32_t n_time,
                 const double *dets, int32_t n_det, const float *response,
                 const so3g_map *map, float *signal, int64_t sig_det_stride,
                 int32_t *err);

int orc_precomp_to_map(const so3g_precomp_geom *g, const int32_t *pixel,
                       const float *spin_proj, int32_t n_det, int32_t n_time,
                       const float *signal, int64_t sig_det_stride,
                       const float *det_weights, const orc_sched *sched,
                       const so3g_map *map, int32_t *err);
int orc_precomp_to_weight_map(const so3g_precomp_geom *g, const int32_t *pixel,
                              const float *spin_proj, int32_t n_det,
                              int32_t n_time, const float *det_weights,
                              const orc_sched *sched, const so3g_map *map,
                              int32_t *err);
int orc_precomp_from_map(const so3g_precomp_geom *g, const int32_t *pixel,
                         const float *spin_proj, int32_t n_det, int32_t n_time,
                         const so3g_map *map, float *signal,
                         int64_t sig_det_stride, int32_t *err);

#ifdef __cplusplus
}
#endif

#endif
