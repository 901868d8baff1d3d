/*
 * so3g_gb300.h -- C ABI of the GB300 (sm_103a) ProjectionEngine library.
 *
 * This is the drop-in boundary for so3g's ProjectionEngine hot path:
 * quaternion pointing, pixelisation (Flat/Quat/CAR/CEA/ARC/SIN/TAN/ZEA
 * rectangular maps and HEALPix; NonTiled and Tiled; nearest and bilinear)
 * and the SpinT/SpinQU/SpinTQU operators to_map, to_weight_map and
 * from_map.  Every entry point takes plain pointers and sizes; nothing in
 * a signature is a Python, numpy or torch type.
 *
 * Pointer conventions
 *   - Array arguments of the so3g_proj_* and so3g_precomp_* entry points
 *     are DEVICE pointers (memory of the current CUDA device), except the
 *     structs themselves, which live in host memory and are read before the
 *     call returns.  The signal of so3g_proj_to_map / so3g_proj_from_map
 *     may also be host memory that the device reaches in place (see
 *     so3g_host_access).
 *   - Work is enqueued on `stream` (a cudaStream_t; NULL = legacy default
 *     stream).  Calls return once the kernels are enqueued; results are
 *     ordered on the stream.
 *   - Errors that the host can see (bad arguments) are returned as a
 *     negative status; so3g_last_error() then holds a message.  Errors that
 *     only the kernel can see (a sample that lands on an absent tile) are
 *     recorded in the device error record `err` (4 x int32, see
 *     so3g_device_error) which the caller zeroes before the call and reads
 *     after synchronising.
 *
 * Layouts (all C-contiguous)
 *   boresight     (n_time, 4)  float64   quaternion (1,i,j,k) per sample
 *   dets          (n_det, 4)   float64   detector offset quaternions
 *   response      (n_det, 2)   float32   (T, P) response per detector
 *   det_weights   (n_det,)     float32   optional (NULL = all ones)
 *   signal        n_det rows of n_time float32; row r starts at
 *                 signal + r * sig_det_stride (elements); unit time stride
 *   map           see so3g_map
 *
 * The reference implementation these entry points replace is the
 * ProjectionEngine template of so3g, src/Projection.cxx, bound to Python
 * by the EXPORT_ENGINE macro (src/Projection.cxx:2294-2308).
 */
#ifndef SO3G_GB300_H
#define SO3G_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SO3G_GB300_ABI_VERSION 2

/* Coordinate systems: the CoordSys template parameter (Pointer<C>),
 * src/Projection.cxx:152-159, 238-507. */
enum so3g_coord_sys {
    SO3G_COORD_FLAT = 0,
    SO3G_COORD_QUAT = 1,
    SO3G_COORD_CAR  = 2,
    SO3G_COORD_CEA  = 3,
    SO3G_COORD_ARC  = 4,
    SO3G_COORD_SIN  = 5,
    SO3G_COORD_TAN  = 6,
    SO3G_COORD_ZEA  = 7
};

/* Pixel systems: Pixelizor2_Flat (src/Projection.cxx:802-1166) and
 * Pixelizor_Healpix (src/Projection.cxx:513-800). */
enum so3g_pix_sys {
    SO3G_PIX_FLAT    = 0,
    SO3G_PIX_HEALPIX = 1
};

/* Interpolation: NearestNeighbor / Bilinear (src/Projection.cxx:166-167). */
enum so3g_interp {
    SO3G_INTERP_NEAREST  = 0,
    SO3G_INTERP_BILINEAR = 1
};

/* Accumulation strategy of the scatter operators (to_map, to_weight_map). */
enum so3g_accum {
    /* One float64 atomic add per (sample, tap, component): the plain
     * FP64-accumulate path. */
    SO3G_ACCUM_ATOMIC = 0,
    /* Runs of equal pixels along a warp's samples are pre-reduced in
     * registers (compensated float32 two-sum) and flushed with one float64
     * atomic add per run. */
    SO3G_ACCUM_WARP_RUNS = 1
};

/* Pointing evaluation (so3g_pixelization.pointing). */
enum so3g_pointing {
    /* Float64 throughout, in the reference's operation order. */
    SO3G_POINTING_EXACT = 0,
    /* CAR, TAN, ZEA and SIN with flat pixelizors, and HEALPix:
     * double-float pointing whose pixel indices and float32 spin factors
     * are certified equal to the exact ones, with the exact path for every
     * sample that cannot be certified.  Results are those of
     * SO3G_POINTING_EXACT, except bilinear interpolation weights, which may
     * differ from it by one float32 ulp.  Other pixelizations use the
     * exact path. */
    SO3G_POINTING_CERTIFIED = 1,
    /* Mixed precision (CAR, TAN, ZEA and SIN with nearest-neighbour flat
     * pixelizors, and HEALPix): float32 pointing whose
     * pixel indices are certified equal to the exact ones (samples that
     * cannot be certified take the double-float, then the exact path).
     * With bilinear flat pixelizors: the double-float pointing with the
     * reference's taps.  Spin factors, interpolation weights and from_map
     * terms are float32 evaluations: maps and signals agree with the exact
     * path to ~1e-7 of their scale.  Other pixelizations as
     * SO3G_POINTING_CERTIFIED. */
    SO3G_POINTING_MIXED = 2
};

/* Status codes returned by every entry point. */
enum so3g_status {
    SO3G_OK            = 0,
    SO3G_ERR_ARGUMENT  = -1,  /* bad argument; message in so3g_last_error() */
    SO3G_ERR_CUDA      = -2,  /* a CUDA call failed */
    SO3G_ERR_NOT_INIT  = -3,  /* so3g_init() was not called on this device */
    SO3G_ERR_RANGE     = -4   /* a size is beyond a documented limit */
};

/* Device error record codes (err[0]). */
enum so3g_device_error {
    SO3G_DEVERR_NONE         = 0,
    /* A sample landed on a tile that is absent from the map; err[1] is the
     * smallest such tile index.  Mirrors tiling_exception
     * (include/exceptions.h:103-116, raised at src/Projection.cxx:1084-1088). */
    SO3G_DEVERR_MISSING_TILE = 1,
    /* A precomputed pixel index lies outside its map or tile; err[1] is the
     * tile (or 0), err[2] the detector and err[3] the sample. */
    SO3G_DEVERR_PIXEL_RANGE  = 2
};

/* Pixelisation: the arguments of the ProjEng_* constructor
 * (Pixelizor2_Flat(bp::object), src/Projection.cxx:821-829 and 971-994;
 * Pixelizor_Healpix(bp::object), src/Projection.cxx:534-542 and 640-675)
 * plus the template choices of the class name. */
typedef struct so3g_pixelization {
    int32_t coord_sys;      /* enum so3g_coord_sys */
    int32_t pix_sys;        /* enum so3g_pix_sys */
    int32_t tiled;          /* 0 = NonTiled, 1 = Tiled */
    int32_t interp;         /* enum so3g_interp (HEALPix: nearest only) */
    int32_t n_comp;         /* 1 = SpinT, 2 = SpinQU, 3 = SpinTQU */
    int32_t naxis[2];       /* Flat: (ny, nx) */
    int32_t tile_shape[2];  /* Flat Tiled: (tile_ny, tile_nx) */
    int32_t nside;          /* HEALPix nside */
    int32_t nest;           /* HEALPix: 1 = NEST, 0 = RING */
    int32_t nside_tile;     /* HEALPix Tiled */
    int32_t pointing;       /* enum so3g_pointing */
    double  cdelt[2];       /* Flat: (dy, dx), radians per pixel */
    double  crpix[2];       /* Flat: (crpix_y, crpix_x), FITS 1-based */
} so3g_pixelization;

/* A map, or a weight map.  Untiled: `data` holds (n_comp, <pixels>)
 * (to_map/from_map) or (n_comp, n_comp, <pixels>) (to_weight_map), where
 * <pixels> is (ny, nx) for Flat and (12*nside^2,) for HEALPix.
 * Tiled: tile t holds the same layout over its own pixels, starting at
 * data + tile_offset[t] (elements); tile_offset[t] < 0 marks an absent tile.
 * Flat tiles at the right/bottom edge are cropped to the parent map, as
 * in Pixelizor2_Flat<Tiled>::zeros (src/Projection.cxx:1014-1025). */
typedef struct so3g_map {
    double        *data;
    const int64_t *tile_offset;  /* device array of n_tile, or NULL (untiled) */
    int32_t        n_tile;       /* number of tiles (0 for untiled) */
    int32_t        _pad;
} so3g_map;

/* Sample ranges: the thread_intervals argument (derive_ranges,
 * src/Projection.cxx:1856-1922) flattened to segments.  Segment k covers
 * samples [seg[3k+1], seg[3k+2]) of detector seg[3k].  A sample covered
 * by two segments is projected twice, as in the reference.  NULL means
 * every sample of every detector once. */
typedef struct so3g_ranges {
    const int32_t *seg;   /* device array of n_seg * 3 int32 */
    int32_t        n_seg;
    int32_t        max_len;  /* longest segment (end - start) */
} so3g_ranges;

/* ---- Library state ------------------------------------------------------ */

/* Builds the 16384-entry asin/atan2 interpolation tables on the host (as
 * the reference's static asinTable/atan2Table, src/Projection.cxx:34-40,
 * include/so_linterp.h:32-71) and uploads them to the current device.
 * Must be called once per device before any so3g_proj_* call. */
int so3g_init(void);

/* Message of the last failing call in this thread ("" if none). */
const char *so3g_last_error(void);

/* ABI version (SO3G_GB300_ABI_VERSION). */
int so3g_abi_version(void);

/* Copies the host trig tables (2 x 16384 float64: asin then atan2). */
int so3g_get_trig_tables(double *asin_vals, double *atan2_vals, int32_t n);

/* Number of kernel launches this library has enqueued since load. */
int64_t so3g_launch_count(void);

/* Sets the smallest call (detectors x samples of a call over whole
 * detectors) that takes the chunked mixed-pointing kernels, and returns
 * the previous value (default 30,000,000; no counterpart in the reference,
 * whose pointing has one form).  Smaller calls take the per-sample float32
 * tier, whose fixed cost per call is lower; results agree within the mixed
 * pointing's tolerance either way.  Process-wide; negative values count as
 * 0 (every eligible call chunked). */
int64_t so3g_set_chunked_min_samples(int64_t n);

/* How the current device can reach host memory at `ptr` (no counterpart
 * in the reference, whose arrays are all host memory).  Sets *mode to
 *   SO3G_HOST_NONE     not reachable: copy it to the device first;
 *   SO3G_HOST_MAPPED   page-locked memory mapped into the device's address
 *                      space at the same address (cudaHostAlloc /
 *                      cudaHostRegister under unified addressing);
 *   SO3G_HOST_PAGEABLE ordinary (pageable) memory, which this device reads
 *                      and writes coherently through the host's page
 *                      tables (cudaDevAttrPageableMemoryAccess, e.g. a
 *                      Grace host over NVLink-C2C).
 * The signal pointer of so3g_proj_to_map / so3g_proj_from_map may be such
 * host memory when the mode is not SO3G_HOST_NONE: the kernels then read
 * (and from_map writes) the samples in place, with no staging copy.  A
 * NULL ptr gives SO3G_HOST_NONE. */
enum so3g_host_mode {
    SO3G_HOST_NONE     = 0,
    SO3G_HOST_MAPPED   = 1,
    SO3G_HOST_PAGEABLE = 2
};
int so3g_host_access(const void *ptr, int32_t *mode);

/* ---- Pointing-only queries ----------------------------------------------- */

/* ProjectionEngine::coords (src/Projection.cxx:1316-1349).
 * coords: (n_det, n_time, 4) float64. */
int so3g_proj_coords(const so3g_pixelization *pz,
                     const double *boresight, int32_t n_time,
                     const double *dets, int32_t n_det,
                     double *coords, void *stream);

/* ProjectionEngine::pixels (src/Projection.cxx:1351-1385).
 * pixel: (n_det, n_time, index_count) int32, index_count = 2 (Flat),
 * 3 (Flat Tiled), 1 (HEALPix), 2 (HEALPix Tiled).  Off-map samples get -1
 * in slot 0 and keep the previous sample's other slots, as the reference. */
int so3g_proj_pixels(const so3g_pixelization *pz,
                     const double *boresight, int32_t n_time,
                     const double *dets, int32_t n_det,
                     int32_t *pixel, void *stream);

/* ProjectionEngine::pointing_matrix (src/Projection.cxx:1391-1438).
 * pixel as so3g_proj_pixels; proj: (n_det, n_time, n_comp) float32. */
int so3g_proj_pointing_matrix(const so3g_pixelization *pz,
                              const double *boresight, int32_t n_time,
                              const double *dets, int32_t n_det,
                              const float *response,
                              int32_t *pixel, float *proj, void *stream);

/* ProjectionEngine::tile_hits (src/Projection.cxx:1543-1601).
 * hits: (n_tile,) int64, zeroed by the caller; counts every interpolation
 * tap of every sample (the reference counts in int; int64 cannot wrap). */
int so3g_proj_tile_hits(const so3g_pixelization *pz,
                        const double *boresight, int32_t n_time,
                        const double *dets, int32_t n_det,
                        int64_t *hits, int32_t n_tile, void *stream);

/* Domain changes behind ProjectionEngine::pixel_ranges
 * (src/Projection.cxx:1440-1541) and ::tile_ranges (:1606-1705).  Every
 * sample gets a domain label:
 *   mode 0: stripe(pixel, n_domain)  (pixel_ranges with map = None)
 *   mode 1: (int) dmap[pixel]        (pixel_ranges with a map; dmap holds
 *           the map's first component, laid out as so3g_map)
 *   mode 2: tile_domain[tile]        (tile_ranges; tile_domain is a device
 *           array of n_tile entries, -1 = unassigned)
 * with -1 for a sample with no pixel and n_domain for one whose
 * interpolation taps disagree.  For every sample t whose label differs from
 * that of sample t-1 (and for t = 0) one edge record (det, t, label) of 3
 * int32 is appended to `edges` (capacity max_edges records, unordered).
 * n_edges (device int64, zeroed by the caller) receives the number of
 * edges; when it exceeds max_edges the extra records are dropped and the
 * caller retries with more room.  A run of equal labels >= 0 from one edge
 * to the next is one interval of the reference's ranges. */
int so3g_proj_domain_edges(const so3g_pixelization *pz,
                           const double *boresight, int32_t n_time,
                           const double *dets, int32_t n_det,
                           int32_t mode, int32_t n_domain,
                           const so3g_map *dmap,
                           const int32_t *tile_domain, int32_t n_tile,
                           int32_t *edges, int64_t max_edges,
                           int64_t *n_edges, int32_t *err, void *stream);

/* ---- Projection operators ------------------------------------------------ */

/* ProjectionEngine::to_map (src/Projection.cxx:1924-1966, inner loop
 * to_map_single_thread :1772-1811):
 *   map[c, pix] += sig * pf[c] * w * det_wt   (float32 product, float64 sum)
 * Detectors with det_weights == 0 are skipped.  ranges may be NULL. */
int so3g_proj_to_map(const so3g_pixelization *pz,
                     const double *boresight, int32_t n_time,
                     const double *dets, int32_t n_det,
                     const float *response,
                     const float *signal, int64_t sig_det_stride,
                     const float *det_weights,
                     const so3g_ranges *ranges,
                     const so3g_map *map,
                     int32_t accum, int32_t *err, void *stream);

/* so3g_proj_to_map for callers that cannot allocate device memory (no
 * counterpart in the reference).  Such callers -- an application that owns
 * all device memory through its own pool or budget, or a binding that can
 * only pass buffers it already holds -- cannot provide the small device
 * tables so3g_proj_to_map needs besides its inputs and outputs, nor call the
 * allocating so3g_init().  This entry point keeps the error record, the trig
 * tables (with the double-float knots of the certified and mixed pointing),
 * the tile-offset table and the sample segments in one static device array
 * of 2.25 MiB per GPU (held until the process exits) and allocates nothing.
 * Inputs, signal and map are device pointers as for so3g_proj_to_map; the
 * pointing mode is pz->pointing, as there.  The segments (host_seg: n_seg
 * (det, start, end) int32 triples, or NULL for all samples) and the
 * tile-offset table of a tiled map (host_tile_offset: n_tile int64 element
 * offsets, -1 = absent tile) are HOST arrays, copied into the static array;
 * when either is given the call waits for the stream to consume them, so
 * they may be reused on return.  At most 65536 segments and 65536 tiles;
 * larger requests return SO3G_ERR_RANGE.  If host_err is not NULL the call
 * waits for the stream and copies the device error record (as
 * so3g_device_error) into it; otherwise so3g_noalloc_read_error reads it
 * later.  Every call sets up the static array in the current CUDA context
 * (address lookup, trig-table upload on `stream`).  All calls share the
 * static array: calls that overlap on the GPU race, so serialise them. */
int so3g_proj_to_map_noalloc(const so3g_pixelization *pz,
                             const double *boresight, int32_t n_time,
                             const double *dets, int32_t n_det,
                             const float *response,
                             const float *signal, int64_t sig_det_stride,
                             const float *det_weights,
                             const int32_t *host_seg, int32_t n_seg,
                             double *map_data,
                             const int64_t *host_tile_offset, int32_t n_tile,
                             int32_t accum, int32_t *host_err, void *stream);

/* The device error record (as so3g_device_error) of the last
 * so3g_proj_to_map_noalloc call on the current device, after waiting for
 * `stream` (no counterpart in the reference; allocates nothing). */
int so3g_noalloc_read_error(int32_t *host_err, void *stream);

/* ProjectionEngine::to_weight_map (src/Projection.cxx:1968-2010, inner
 * loop :1813-1854): W[i, j, pix] += pf[i]*pf[j]*w*w*det_wt for j >= i. */
int so3g_proj_to_weight_map(const so3g_pixelization *pz,
                            const double *boresight, int32_t n_time,
                            const double *dets, int32_t n_det,
                            const float *response,
                            const float *det_weights,
                            const so3g_ranges *ranges,
                            const so3g_map *map,
                            int32_t accum, int32_t *err, void *stream);

/* ---- Batches of observations --------------------------------------------
 * Many observations (each its own boresight, focal plane and signal)
 * projected into one map by one persistent launch: the work items
 * (observation, detector, piece of `piece` samples) of all observations
 * are shared out over `blocks` resident blocks.  A caller projecting N
 * observations with so3g_proj_to_map makes N launches; the reference
 * makes N calls of ProjectionEngine::to_map (src/Projection.cxx:1924-1966).
 * The sums are the same; only the float64 summation order differs. */
typedef struct so3g_obs {
    const double *boresight;    /* device (n_time, 4) */
    const double *dets;         /* device (n_det, 4) */
    const float  *response;     /* device (n_det, 2) */
    const float  *signal;       /* device rows (to_map), NULL otherwise */
    const float  *det_weights;  /* device (n_det,), or NULL */
    int64_t       sig_det_stride;
    int32_t       n_time;
    int32_t       n_det;
} so3g_obs;

/* Host helper: work_offset[o] = number of work items of observations
 * 0..o-1 (n_det * ceil(n_time / piece) each), for o = 0..n_obs; returns
 * the total.  obs is read on the host (only n_time and n_det). */
int64_t so3g_batch_work_offsets(const so3g_obs *obs, int32_t n_obs, int32_t piece,
                                int64_t *work_offset);

/* to_map / to_weight_map of a batch.  obs (n_obs entries) and work_offset
 * (n_obs + 1 entries, from so3g_batch_work_offsets with the same piece)
 * are DEVICE arrays.  blocks > 0: a grid of that many blocks, each taking
 * every blocks-th work item; 0: one full wave of resident blocks (as many
 * as fit on the device at once); < 0: one block per work item. */
int so3g_proj_to_map_batch(const so3g_pixelization *pz, const so3g_obs *obs,
                           int32_t n_obs, const int64_t *work_offset,
                           int64_t n_work, int32_t piece, int32_t blocks,
                           const so3g_map *map, int32_t accum, int32_t *err,
                           void *stream);
int so3g_proj_to_weight_map_batch(const so3g_pixelization *pz, const so3g_obs *obs,
                                  int32_t n_obs, const int64_t *work_offset,
                                  int64_t n_work, int32_t piece, int32_t blocks,
                                  const so3g_map *map, int32_t accum, int32_t *err,
                                  void *stream);

/* ProjectionEngine::from_map (src/Projection.cxx:1728-1770):
 *   sig += map[c, pix] * pf[c] * w, rounded to float32 after every term;
 * accumulates into `signal`. */
int so3g_proj_from_map(const so3g_pixelization *pz,
                       const double *boresight, int32_t n_time,
                       const double *dets, int32_t n_det,
                       const float *response,
                       const so3g_map *map,
                       float *signal, int64_t sig_det_stride,
                       int32_t *err, void *stream);

/* ---- Precomputed pointing (ProjEng_Precomp, src/Projection.cxx:2012-2256) -
 * pixel: (n_det, n_time, n_index) int32 with a close-packed last axis;
 * n_index is 2 for NonTiled (iy, ix) and 3 for Tiled (tile, iy, ix).
 * Samples with pixel[..., 0] < 0 are skipped.  spin_proj: (n_det, n_time,
 * n_comp) float32.  The map is (n_comp, ny, nx) (weight map: (n_comp,
 * n_comp, ny, nx)); a tiled map is so3g_map's tile list, tile t being
 * (.., tile_dims[2t], tile_dims[2t+1]).  A pixel outside its map or tile
 * is skipped and recorded as SO3G_DEVERR_PIXEL_RANGE (the reference does
 * not check it).  */
typedef struct so3g_precomp_geom {
    int32_t        tiled;
    int32_t        n_comp;
    int32_t        naxis[2];    /* untiled map (ny, nx) */
    const int32_t *tile_dims;   /* tiled: device array (n_tile, 2) */
} so3g_precomp_geom;

/* ProjEng_Precomp::to_map (src/Projection.cxx:2087-2122, 2157-2206):
 *   map[c, pix] += det_wt * sig * pf[c]   (float32 product, float64 sum) */
int so3g_precomp_to_map(const so3g_precomp_geom *g,
                        const int32_t *pixel, const float *spin_proj,
                        int32_t n_det, int32_t n_time,
                        const float *signal, int64_t sig_det_stride,
                        const float *det_weights,
                        const so3g_ranges *ranges,
                        const so3g_map *map,
                        int32_t accum, int32_t *err, void *stream);

/* ProjEng_Precomp::to_weight_map (src/Projection.cxx:2124-2155, 2208-2253):
 *   W[i, j, pix] += pf[i] * pf[j] * det_wt for j >= i. */
int so3g_precomp_to_weight_map(const so3g_precomp_geom *g,
                               const int32_t *pixel, const float *spin_proj,
                               int32_t n_det, int32_t n_time,
                               const float *det_weights,
                               const so3g_ranges *ranges,
                               const so3g_map *map,
                               int32_t accum, int32_t *err, void *stream);

/* ProjEng_Precomp::from_map (src/Projection.cxx:2036-2085):
 *   sig += sum_c pf[c] * map[c, pix]  (the sum over c in float32) */
int so3g_precomp_from_map(const so3g_precomp_geom *g,
                          const int32_t *pixel, const float *spin_proj,
                          int32_t n_det, int32_t n_time,
                          const so3g_map *map,
                          float *signal, int64_t sig_det_stride,
                          int32_t *err, void *stream);

/* ---- Boresight generation (the step before the path) --------------------- */

/* Sight-line models of CelestialSightLine (python/proj/coords.py). */
enum so3g_sight_kind {
    SO3G_SIGHT_HORIZON    = 0,  /* for_horizon, coords.py:190-209 */
    SO3G_SIGHT_NAIVE_AZEL = 1   /* naive_az_el, coords.py:99-125 */
};

/* Constants of a sight line, formed on the host as the Python layer forms
 * them (so that both sides share their bits):
 *   horizon:    Q = euler(2, -az) * euler(1, pi/2 - el) * euler(2, roll)
 *   naive:      Q = euler(2, lst) * q_site_lat * q_pi * euler(2, -az)
 *                   * euler(1, pi/2 - el) * euler(2, roll),
 *               lst = (era_poly[0] * J + era_poly[1]) + site_lon_rad,
 *               J = (t - era_epoch) / 86400
 * each product taken left to right, as numpy evaluates the expression;
 * then, with has_left, Q = q_left * Q (the Projectionist's
 * q_celestial_to_native * Q, python/proj/wcs.py:140-148). */
typedef struct so3g_sightline {
    int32_t kind;            /* so3g_sight_kind */
    int32_t has_left;        /* apply q_left */
    double roll;             /* roll where the roll array is NULL */
    double site_lon_rad;     /* naive: site.lon * DEG */
    double era_epoch;        /* naive: ERA_EPOCH */
    double era_poly[2];      /* naive: ERA_POLY */
    double q_site_lat[4];    /* naive: euler(1, pi/2 - site.lat * DEG) */
    double q_pi[4];          /* naive: euler(2, pi) */
    double q_left[4];
} so3g_sightline;

/* Boresight quaternions q_out (n, 4) float64 of a sight line from the
 * per-sample arrays t (naive only; NULL for horizon), az, el and roll
 * (NULL: sl->roll), all (n,) float64 device arrays.  Replaces the numpy
 * evaluation of CelestialSightLine.for_horizon / naive_az_el
 * (python/proj/coords.py:99-125, 190-209) and, with has_left, the
 * quat x G3VectorQuat product of Projectionist._cache_q_fp_to_native. */
int so3g_boresight(const so3g_sightline *sl, const double *t, const double *az,
                   const double *el, const double *roll, int64_t n, double *q_out,
                   void *stream);

/* q_out[i] = q_left * q_in[i] for n quaternions (device arrays (n, 4)
 * float64; q_left host, 4 float64): spt3g's quat x G3VectorQuat product,
 * used by Projectionist._cache_q_fp_to_native (python/proj/wcs.py:140-148). */
int so3g_quat_left_multiply(const double *q_left, const double *q_in, int64_t n,
                            double *q_out, void *stream);

/* ---- Cut masks to sample segments ----------------------------------------- */

/* RangesMatrix.from_mask (python/proj/ranges.py:11-297; Ranges built from a
 * boolean mask, src/Ranges.cxx) for an (n_det, n_time) uint8 mask in
 * device memory (nonzero = sample in a range; row d at mask + d *
 * det_stride): counts[d] = the number of runs of set samples in row d
 * (device int32 array of n_det). */
int so3g_mask_count_segments(const uint8_t *mask, int32_t n_det, int32_t n_time,
                             int64_t det_stride, int32_t *counts, void *stream);

/* Writes the runs as so3g_ranges segments: seg (3 int32 per segment, device)
 * receives (d, start, end) for the runs of row d from index first[d] on,
 * first being the exclusive prefix sum of counts (device int64, n_det);
 * *max_len (device int32, zeroed by the caller) becomes the longest run. */
int so3g_mask_fill_segments(const uint8_t *mask, int32_t n_det, int32_t n_time,
                            int64_t det_stride, const int64_t *first, const int32_t *counts,
                            int32_t *seg, int32_t *max_len, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SO3G_GB300_H */
