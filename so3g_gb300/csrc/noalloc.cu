// noalloc.cu -- so3g_proj_to_map_noalloc: to_map for callers that cannot
// allocate device memory.
//
// Some callers own every byte of device memory they use: an application
// with its own memory pool or a fixed device-memory budget, or a foreign-
// language binding that can only hand over buffers it already holds.  They
// cannot let a library call cudaMalloc, and they cannot allocate the small
// device-side tables that so3g_proj_to_map takes besides its inputs and
// outputs: the error record, the tile-offset table of a tiled map, the
// sample segments, and (through so3g_init) the trig tables.
//
// This entry point keeps all of those in one file-scope static device array
// (g_noalloc_scratch, below) of a fixed size, which every GPU that loads
// the library holds until the process exits.  The caller passes the
// inputs and the map in device memory, and the two small tables as HOST
// arrays; the entry point copies them into the scratch before the launch.
// It calls no cudaMalloc, cudaFree or other allocating routine.
//
// Set-up, on every call: the entry point looks up the scratch's device
// address in the current context (cudaGetSymbolAddress) and copies the
// trig tables (and, for the certified and mixed pointing, their
// double-float knots) into it on the caller's stream, so a fresh context
// (after cudaDeviceReset, or a caller's own CUDA context) is set up the
// same way as the first one.  Pointing modes are those of so3g_proj_to_map
// (pz->pointing); the mixed mode converts the float64 boresight itself, as
// there is no room for its float32 copy.
//
// Host arrays: the segment and tile-offset tables are copied from the
// caller's host arrays; the call waits for the stream to consume them, so
// they may be reused or freed as soon as it returns.
//
// Sharing: every call uses the same scratch and leaves its contents there.
// The error record is cleared at the start of each call and can be read
// afterwards with so3g_noalloc_read_error; the tables are rewritten.
// Calls whose work overlaps on the GPU (different streams, or different
// host threads) race on the scratch: serialise them.

#include <climits>

#include "scatter_kernel.cuh"

namespace so3g {

namespace {

// Limits: tiles of a tiled map and sample segments per call.
constexpr int kNoAllocMaxTiles = 1 << 16;
constexpr int kNoAllocMaxSegs = 1 << 16;

// Scratch layout (byte offsets): error record, trig tables, double-float
// knot tables, tile offsets, sample segments.  2.25 MiB in all.
constexpr size_t kOffErr = 0;
constexpr size_t kOffLut = 256;
constexpr size_t kOffKnots = kOffLut + sizeof(double) * 2 * kLutN;
constexpr size_t kOffTiles = kOffKnots + sizeof(float4) * 3 * kLutN;
constexpr size_t kOffSegs = kOffTiles + sizeof(long long) * kNoAllocMaxTiles;
constexpr size_t kScratchBytes = kOffSegs + 3 * sizeof(int) * kNoAllocMaxSegs;
static_assert(kOffKnots % 16 == 0 && kOffTiles % 16 == 0, "scratch alignment");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of the scratch in the current context.
int scratch_address(unsigned char **out) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
        return set_error(SO3G_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    *out = static_cast<unsigned char *>(p);
    return SO3G_OK;
}

// Copies the trig tables (and, for the certified and mixed pointing, the
// knot tables) into the scratch on stream st.  The sources are the
// library's static host tables, valid for the whole process.
int upload_tables(unsigned char *scr, bool knots, cudaStream_t st) {
    cudaError_t e = cudaMemcpyAsync(scr + kOffLut, host_lut(), sizeof(double) * 2 * kLutN,
                                    cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && knots)
        e = cudaMemcpyAsync(scr + kOffKnots, host_fast_knots(), sizeof(float4) * 3 * kLutN,
                            cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess)
        return set_error(SO3G_ERR_CUDA, "trig table upload: %s", cudaGetErrorString(e));
    return SO3G_OK;
}

struct NoAllocLaunch {
    ScatterArgs a;
    dim3 grid;
    cudaStream_t stream;
    template <int C, int P>
    struct Go {
        NoAllocLaunch *L;
        template <int MODE>
        int go() {
            k_scatter<C, P, false, MODE><<<L->grid, kBlock, 0, L->stream>>>(L->a);
            return after_launch("to_map (no-alloc)");
        }
    };
    template <int C, int P>
    int run() {
        Go<C, P> g{this};
        return by_mode<C, P>(a.fast, g);
    }
};

}  // namespace

}  // namespace so3g

using namespace so3g;

extern "C" int so3g_proj_to_map_noalloc(
    const so3g_pixelization *pz, const double *boresight, int32_t n_time, const double *dets,
    int32_t n_det, const float *response, const float *signal, int64_t sig_det_stride,
    const float *det_weights, const int32_t *host_seg, int32_t n_seg, double *map_data,
    const int64_t *host_tile_offset, int32_t n_tile, int32_t accum, int32_t *host_err,
    void *stream) {
    clear_error();
    if (host_err)
        for (int i = 0; i < 4; i++) host_err[i] = 0;
    if (!pz) return set_error(SO3G_ERR_ARGUMENT, "pixelization is NULL");
    if (n_det < 0 || n_time < 0 || n_seg < 0 || n_tile < 0)
        return set_error(SO3G_ERR_ARGUMENT, "negative size");
    if (n_seg > kNoAllocMaxSegs)
        return set_error(SO3G_ERR_RANGE,
                         "no-alloc to_map takes at most %d sample segments (got %d)",
                         kNoAllocMaxSegs, n_seg);
    if (n_tile > kNoAllocMaxTiles)
        return set_error(SO3G_ERR_RANGE, "no-alloc to_map takes at most %d tiles (got %d)",
                         kNoAllocMaxTiles, n_tile);
    if (accum != SO3G_ACCUM_ATOMIC && accum != SO3G_ACCUM_WARP_RUNS)
        return set_error(SO3G_ERR_ARGUMENT, "unknown accumulation mode %d", accum);
    unsigned char *scr = nullptr;
    int rc = scratch_address(&scr);
    if (rc) return rc;

    NoAllocLaunch L{};
    rc = make_geom_lut(pz, &L.a.g, reinterpret_cast<const double *>(scr + kOffLut));
    if (rc) return rc;
    const float4 *knots = reinterpret_cast<const float4 *>(scr + kOffKnots);
    L.a.ft = FastTables{knots, knots + kLutN, knots + 2 * kLutN};
    L.a.fast = fast_mode(pz, L.a.ft);
    if (!map_data) return set_error(SO3G_ERR_ARGUMENT, "map is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    rc = upload_tables(scr, L.a.fast != SO3G_POINTING_EXACT, st);
    if (rc) return rc;
    bool host_tables = false;
    if (pz->tiled) {
        if (!host_tile_offset)
            return set_error(SO3G_ERR_ARGUMENT, "tiled map needs a host tile_offset table");
        if (n_tile != L.a.g.n_tile)
            return set_error(SO3G_ERR_ARGUMENT, "tiled map has %d tiles; the pixelization has %d",
                             n_tile, L.a.g.n_tile);
        cudaError_t e = cudaMemcpyAsync(scr + kOffTiles, host_tile_offset,
                                        sizeof(long long) * n_tile, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess)
            return set_error(SO3G_ERR_CUDA, "tile table copy: %s", cudaGetErrorString(e));
        L.a.g.tile_offset = reinterpret_cast<const long long *>(scr + kOffTiles);
        L.a.g.n_tile_map = n_tile;
        host_tables = true;
    }
    long long n_work = n_det, max_len = n_time;
    const int *dseg = nullptr;
    if (host_seg) {
        max_len = 0;
        for (int k = 0; k < n_seg; k++) {
            const int d = host_seg[3 * k], a = host_seg[3 * k + 1], b = host_seg[3 * k + 2];
            if (d < 0 || d >= n_det || a < 0 || b > n_time)
                return set_error(SO3G_ERR_ARGUMENT, "segment %d (%d, %d, %d) is outside the "
                                 "(n_det, n_time) = (%d, %d) samples", k, d, a, b, n_det, n_time);
            if (b - a > max_len) max_len = b - a;
        }
        n_work = n_seg;
        if (n_seg > 0) {
            cudaError_t e = cudaMemcpyAsync(scr + kOffSegs, host_seg, 3 * sizeof(int) * n_seg,
                                            cudaMemcpyHostToDevice, st);
            if (e != cudaSuccess)
                return set_error(SO3G_ERR_CUDA, "segment copy: %s", cudaGetErrorString(e));
            host_tables = true;
        }
        dseg = reinterpret_cast<const int *>(scr + kOffSegs);
    }
    int *derr = reinterpret_cast<int *>(scr + kOffErr);
    cudaError_t e = cudaMemsetAsync(derr, 0, 4 * sizeof(int), st);
    if (e != cudaSuccess) return set_error(SO3G_ERR_CUDA, "error record clear: %s", cudaGetErrorString(e));
    if (n_work > 0 && max_len > 0) {
        if (!boresight || !dets || !response || !signal)
            return set_error(SO3G_ERR_ARGUMENT, "NULL input array");
        L.a.bore = boresight;
        L.a.dets = dets;
        L.a.resp = response;
        L.a.signal = signal;
        L.a.sig_stride = sig_det_stride;
        L.a.det_weights = det_weights;
        L.a.segs = Segs{dseg, n_time};
        L.a.piece = piece_len(max_len, n_work);
        L.a.accum = accum;
        L.a.err = derr;
        L.a.map = map_data;
        L.a.fc = make_fast_const(L.a.g);
        L.a.mc = make_mixed_const(L.a.g);
        L.a.bore32 = nullptr;   // the kernels round the float64 boresight themselves
        L.grid = dim3((unsigned)n_work, (unsigned)((max_len + L.a.piece - 1) / L.a.piece));
        L.stream = st;
        rc = dispatch_cp(pz->coord_sys, pix_kind(pz), L);
        if (rc) return rc;
    }
    if (host_err) {
        e = cudaMemcpyAsync(host_err, derr, 4 * sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess)
            return set_error(SO3G_ERR_CUDA, "error record read: %s", cudaGetErrorString(e));
    } else if (host_tables) {
        // The caller may reuse host_seg / host_tile_offset on return.
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess)
            return set_error(SO3G_ERR_CUDA, "stream wait: %s", cudaGetErrorString(e));
    }
    return SO3G_OK;
}

extern "C" int so3g_noalloc_read_error(int32_t *host_err, void *stream) {
    clear_error();
    if (!host_err) return set_error(SO3G_ERR_ARGUMENT, "host_err is NULL");
    unsigned char *scr = nullptr;
    int rc = scratch_address(&scr);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(host_err, scr + kOffErr, 4 * sizeof(int),
                                    cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return set_error(SO3G_ERR_CUDA, "error record read: %s", cudaGetErrorString(e));
    return SO3G_OK;
}
