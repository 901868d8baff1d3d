// mx_common.cuh -- pieces shared by the two-pass mixed-pointing kernels of
// to_map (mixed_launch.cuh) and from_map (gather.cu): which pixelizations
// take them, and the fallback mask that links the passes.
//
// The main pass handles one sample per lane in rounds of kBlock samples;
// each warp records the samples its float32 tier could not certify as one
// 32-bit word per round (bit b = lane b).  The fallback pass visits the set
// bits (mx_for_each), 32 mask words per warp, dealing the bits out to the
// lanes by prefix sum so that every lane has a sample to work on.
#pragma once

#include "host.h"

namespace so3g {

namespace {

// Resident blocks per SM of k_scatter_mx (registers <= 65536 / (256 * 6)
// = 42 each).
constexpr int kMxBlocksPerSM = 6;

template <int C, int P>
struct MxEligible {
    static constexpr bool value = MixedEligible<C, P>::value &&
                                  (P == PX_FLAT_NT_NN || P == PX_HP_NT);
};

// The fallback mask of one call: one word per (block, round, warp).
struct MxMask {
    unsigned *words;
    long long n_words;
    int wpp;         // words per piece: (piece / kBlock) rounds x (kBlock / 32) warps
    int wpp_shift;   // log2(wpp): pieces are powers of two
    int gy;          // pieces per segment (grid.y of the main kernel)
};

// Position of the k-th (0-based) set bit of w (w has more than k set bits).
__device__ __forceinline__ int nth_bit(unsigned w, int k) {
    for (int i = 0; i < k; i++) w &= w - 1u;
    return __ffs(w) - 1;
}

// (det, t) of bit `bit` of mask word `word`.  Integer shifts and one
// 32-bit division: 64-bit division would run on the float64 pipe.
__device__ __forceinline__ void mx_sample(const Segs &segs, int piece, const MxMask &mm,
                                          long long word, int bit, int &det, int &t) {
    const unsigned blk = (unsigned)(word >> mm.wpp_shift);   // < 2^31 blocks
    const int rem = (int)(word & (long long)(mm.wpp - 1));
    const unsigned x = blk / (unsigned)mm.gy, y = blk - x * (unsigned)mm.gy;
    int s0 = 0;
    if (segs.seg) {
        det = __ldg(segs.seg + 3 * x);
        s0 = __ldg(segs.seg + 3 * x + 1);
    } else {
        det = x;
    }
    t = s0 + y * piece + (rem / (kBlock / 32)) * kBlock + (rem % (kBlock / 32)) * 32 + bit;
}

// Calls f(det, t) once for every set bit of the mask, the bits of each 32
// words dealt out to the 32 lanes of a warp by prefix sum.
template <class F>
__device__ __forceinline__ void mx_for_each(const Segs &segs, int piece, const MxMask &mm, F &&f) {
    const int lane = threadIdx.x & 31;
    const long long n_groups = (mm.n_words + 31) / 32;
    const long long warps = (long long)gridDim.x * (blockDim.x / 32);
    for (long long g = (long long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
         g < n_groups; g += warps) {
        const long long w = g * 32 + lane;
        const unsigned bits = w < mm.n_words ? mm.words[w] : 0u;
        const int cnt = __popc(bits);
        int inc = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int o = __shfl_up_sync(kFull, inc, d);
            if (lane >= d) inc += o;
        }
        const int total = __shfl_sync(kFull, inc, 31);
        const int excl = inc - cnt;
        for (int base = 0; base < total; base += 32) {
            const int k = base + lane;
            // Owner: the last lane whose exclusive prefix is <= k.
            int lo = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const int e = __shfl_sync(kFull, excl, lo + step);
                if (e <= k) lo += step;
            }
            const unsigned ob = __shfl_sync(kFull, bits, lo);
            const int oe = __shfl_sync(kFull, excl, lo);
            if (k < total) {
                int det, t;
                mx_sample(segs, piece, mm, g * 32 + lo, nth_bit(ob, k - oe), det, t);
                f(det, t);
            }
        }
    }
}

// Allocates and clears (stream-ordered) the mask of a main pass over
// `grid` with pieces of `piece` samples; false (nothing allocated) when the
// allocation fails.
inline bool mx_mask_alloc(MxMask &mm, dim3 grid, int piece, cudaStream_t stream) {
    mm.wpp = (piece / kBlock) * (kBlock / 32);
    mm.wpp_shift = 0;
    while ((1 << mm.wpp_shift) < mm.wpp) mm.wpp_shift++;
    if ((1 << mm.wpp_shift) != mm.wpp) return false;   // pieces are powers of two
    mm.gy = (int)grid.y;
    if ((long long)grid.x * grid.y >= (1LL << 31)) return false;   // mx_sample's 32-bit blocks
    mm.n_words = (long long)grid.x * grid.y * mm.wpp;
    mm.words = nullptr;
    if (cudaMallocAsync(reinterpret_cast<void **>(&mm.words),
                        sizeof(unsigned) * (size_t)mm.n_words, stream) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (cudaMemsetAsync(mm.words, 0, sizeof(unsigned) * (size_t)mm.n_words, stream) !=
        cudaSuccess) {
        cudaGetLastError();
        cudaFreeAsync(mm.words, stream);
        return false;
    }
    return true;
}

// Blocks of kBlock threads for a fallback pass over mask mm: one warp per
// 32 words, at most 16 waves of 152 SMs (the warps then stride).
inline unsigned mx_fix_blocks(const MxMask &mm) {
    const long long groups = (mm.n_words + 31) / 32;
    const long long warps_per_block = kBlock / 32;
    long long b = (groups + warps_per_block - 1) / warps_per_block;
    if (b > 152LL * 16) b = 152LL * 16;
    return (unsigned)(b > 0 ? b : 1);
}

}  // namespace

}  // namespace so3g
