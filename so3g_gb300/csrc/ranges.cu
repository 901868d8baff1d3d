// ranges.cu -- cut masks to sample segments on the device.
//
// RangesMatrix.from_mask (python/proj/ranges.py:11-297; Ranges<int32_t>
// built from a boolean mask, src/Ranges.cxx) for an (n_det, n_time) mask
// held in device memory: each detector row's runs of set samples become
// (det, start, end) segments, in detector then time order -- the
// so3g_ranges form in which the projection kernels take thread_intervals.
// Two passes: so3g_mask_count_segments counts each row's runs; the caller
// forms the exclusive prefix sum of the counts (the rows' first segment
// indices) and so3g_mask_fill_segments writes the segments.
//
// One block per row walks it in rounds of kMaskBlock x 16 samples; each
// thread turns its 16 samples into a 16-bit set mask and counts the run
// starts (set after unset) and ends (unset after set, and the row's end
// after a set sample) in it with bit operations; a block-wide scan of the
// packed (starts, ends) counts places the thread's edges in time order.

#include "host.h"

namespace so3g {

namespace {

constexpr int kMaskBlock = 256;
constexpr int kMaskChunk = 16;

struct MaskRow {
    const uint8_t *row;
    int n_time;
    bool vec;   // row 16-byte aligned: uint4 loads
};

// Bits 0..15: samples t0 .. t0+15 set (0 beyond the row's end); prev: the
// sample before t0 is set.
__device__ __forceinline__ unsigned chunk_bits(const MaskRow &m, int t0, unsigned &prev) {
    prev = (t0 > 0 && m.row[t0 - 1] != 0) ? 1u : 0u;
    unsigned bits = 0;
    if (m.vec && t0 + kMaskChunk <= m.n_time) {
        const uint4 v = *reinterpret_cast<const uint4 *>(m.row + t0);
        const unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int k = 0; k < 4; k++)
#pragma unroll
            for (int b = 0; b < 4; b++)
                if ((w[k] >> (8 * b)) & 0xffu) bits |= 1u << (4 * k + b);
    } else {
        for (int j = 0; j < kMaskChunk && t0 + j < m.n_time; j++)
            if (m.row[t0 + j]) bits |= 1u << j;
    }
    return bits;
}

// Run starts and ends among the chunk's samples.  An end at sample t means
// the run covers up to t - 1; bit j of `ends` is an end at t0 + j, and
// bit 16 the row's end (t0 + 16 == n_time or the chunk's last sample).
__device__ __forceinline__ void chunk_edges(const MaskRow &m, int t0, unsigned &starts,
                                            unsigned &ends) {
    unsigned prev;
    const unsigned bits = chunk_bits(m, t0, prev);
    const unsigned before = ((bits << 1) | prev) & 0xffffu;   // sample t-1 set
    const int n = min(kMaskChunk, m.n_time - t0);
    const unsigned live = n >= 32 ? 0xffffffffu : ((1u << n) - 1u);
    starts = bits & ~before & live;
    ends = ~bits & before & live;
    // The row's end closes a run that reaches it.
    if (t0 + n == m.n_time && ((bits >> (n - 1)) & 1u)) ends |= 1u << n;
}

// Block-wide exclusive scan of v (kMaskBlock threads); total in *total.
__device__ __forceinline__ unsigned block_scan(unsigned v, unsigned *s_warp, unsigned *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned y = __shfl_up_sync(kFull, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned w = lane < kMaskBlock / 32 ? s_warp[lane] : 0u;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned y = __shfl_up_sync(kFull, w, d);
            if (lane >= d) w += y;
        }
        if (lane < kMaskBlock / 32) s_warp[lane] = w;
    }
    __syncthreads();
    const unsigned base = warp ? s_warp[warp - 1] : 0u;
    *total = s_warp[kMaskBlock / 32 - 1];
    __syncthreads();
    return base + x - v;
}

__global__ void __launch_bounds__(kMaskBlock) k_mask_count(const uint8_t *mask, int n_time,
                                                           long long stride, int *counts) {
    __shared__ unsigned s_warp[kMaskBlock / 32];
    const int det = blockIdx.x;
    MaskRow m{mask + det * stride, n_time,
              (reinterpret_cast<uintptr_t>(mask + det * stride) & 15u) == 0};
    unsigned c = 0;
    for (int t0 = threadIdx.x * kMaskChunk; t0 < n_time; t0 += kMaskBlock * kMaskChunk) {
        unsigned s, e;
        chunk_edges(m, t0, s, e);
        c += __popc(s);
    }
    unsigned total;
    block_scan(c, s_warp, &total);
    if (threadIdx.x == 0) counts[det] = (int)total;
}

__global__ void __launch_bounds__(kMaskBlock) k_mask_fill(const uint8_t *mask, int n_time,
                                                          long long stride,
                                                          const long long *first,
                                                          const int *counts, int *seg,
                                                          int *max_len) {
    __shared__ unsigned s_warp[kMaskBlock / 32];
    __shared__ int s_max;
    const int det = blockIdx.x;
    MaskRow m{mask + det * stride, n_time,
              (reinterpret_cast<uintptr_t>(mask + det * stride) & 15u) == 0};
    int *out = seg + 3 * first[det];
    unsigned done_s = 0, done_e = 0;   // edges written by earlier rounds
    const int rounds = (n_time + kMaskBlock * kMaskChunk - 1) / (kMaskBlock * kMaskChunk);
    for (int r = 0; r < rounds; r++) {
        const int t0 = (r * kMaskBlock + threadIdx.x) * kMaskChunk;
        unsigned s = 0, e = 0;
        if (t0 < n_time) chunk_edges(m, t0, s, e);
        // starts in the low 16 bits, ends in the high (at most 4352 each).
        unsigned total;
        const unsigned pre = block_scan(__popc(s) | ((unsigned)__popc(e) << 16), s_warp, &total);
        unsigned ks = done_s + (pre & 0xffffu), ke = done_e + (pre >> 16);
        while (s) {
            const int j = __ffs(s) - 1;
            s &= s - 1;
            out[3 * ks] = det;
            out[3 * ks + 1] = t0 + j;
            ks++;
        }
        while (e) {
            const int j = __ffs(e) - 1;
            e &= e - 1;
            out[3 * ke + 2] = t0 + j;
            ke++;
        }
        done_s += total & 0xffffu;
        done_e += total >> 16;
    }
    // The row's longest segment (the launch extent of the projection
    // kernels): the block reads back what it wrote.
    if (threadIdx.x == 0) s_max = 0;
    __syncthreads();
    int longest = 0;
    for (int k = threadIdx.x; k < counts[det]; k += kMaskBlock)
        longest = max(longest, out[3 * k + 2] - out[3 * k + 1]);
    atomicMax(&s_max, longest);
    __syncthreads();
    if (threadIdx.x == 0 && s_max > 0) atomicMax(max_len, s_max);
}

}  // namespace

}  // namespace so3g

extern "C" int so3g_mask_count_segments(const uint8_t *mask, int32_t n_det, int32_t n_time,
                                        int64_t det_stride, int32_t *counts, void *stream) {
    using namespace so3g;
    clear_error();
    if (n_det < 0 || n_time < 0) return set_error(SO3G_ERR_ARGUMENT, "negative n_det or n_time");
    if (n_det == 0) return SO3G_OK;
    if (!counts || (n_time > 0 && !mask)) return set_error(SO3G_ERR_ARGUMENT, "NULL array");
    if (det_stride < n_time) return set_error(SO3G_ERR_ARGUMENT, "det_stride < n_time");
    k_mask_count<<<(unsigned)n_det, kMaskBlock, 0, (cudaStream_t)stream>>>(mask, n_time,
                                                                          det_stride, counts);
    return after_launch("mask segment count");
}

extern "C" int so3g_mask_fill_segments(const uint8_t *mask, int32_t n_det, int32_t n_time,
                                       int64_t det_stride, const int64_t *first,
                                       const int32_t *counts, int32_t *seg, int32_t *max_len,
                                       void *stream) {
    using namespace so3g;
    clear_error();
    if (n_det < 0 || n_time < 0) return set_error(SO3G_ERR_ARGUMENT, "negative n_det or n_time");
    if (n_det == 0 || n_time == 0) return SO3G_OK;
    if (!mask || !first || !counts || !seg || !max_len)
        return set_error(SO3G_ERR_ARGUMENT, "NULL array");
    if (det_stride < n_time) return set_error(SO3G_ERR_ARGUMENT, "det_stride < n_time");
    k_mask_fill<<<(unsigned)n_det, kMaskBlock, 0, (cudaStream_t)stream>>>(
        mask, n_time, det_stride, reinterpret_cast<const long long *>(first), counts, seg,
        max_len);
    return after_launch("mask segment fill");
}
