// mx_common.cuh -- pieces shared by the two-pass mixed-pointing kernels of
// to_map (mixed_launch.cuh) and from_map (gather.cu): which pixelizations
// take them, and the fallback mask that links the passes.
//
// The main pass handles one sample per lane in rounds of kBlock samples;
// each warp records the samples its float32 tier could not certify as one
// 32-bit word per round (bit b = lane b).  The fallback passes, one per
// tier of pointing, visit the set bits (mx_for_each), 32 mask words per
// warp, dealing the bits out to the lanes by prefix sum so that every lane
// has a sample to work on, and leave in the mask the samples that the next
// tier must take.
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

// Position of the k-th (0-based) set bit of w (w has more than k set bits),
// by bisection on the bit counts of the lower halves.
__device__ __forceinline__ int nth_bit(unsigned w, int k) {
    int pos = 0;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        const int c = __popc(w & ((1u << s) - 1u));
        if (k >= c) {
            k -= c;
            w >>= s;
            pos += s;
        }
    }
    return pos;
}

// Mask words per lane in one window of mx_for_each (a warp reads 32 x this
// many words at once).
constexpr int kMxWin = 8;

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

// Calls f(det, t) once for every set bit of the mask.  A warp reads a
// window of 32 x kMxWin words (kMxWin independent loads per lane) and deals
// its set bits out to the 32 lanes by prefix sum, 32 at a time, so that
// every lane has a sample to work on even where the bits are sparse.  f
// returns true when it has handled the sample.  With REQUEUE the words are
// cleared as they are read and the bits whose f returned false set again,
// so that the next tier's pass over the same mask sees only those: each
// tier then runs on full warps, instead of a warp paying for a costlier
// tier whenever one of its lanes needs it.
template <bool REQUEUE, class F>
__device__ __forceinline__ void mx_for_each(const Segs &segs, int piece, const MxMask &mm, F &&f) {
    const int lane = threadIdx.x & 31;
    constexpr long long kWinWords = 32LL * kMxWin;
    const long long n_win = (mm.n_words + kWinWords - 1) / kWinWords;
    const long long warps = (long long)gridDim.x * (blockDim.x / 32);
    for (long long win = (long long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
         win < n_win; win += warps) {
        const long long w0 = win * kWinWords + lane;
        unsigned bits[kMxWin];
#pragma unroll
        for (int i = 0; i < kMxWin; i++) {
            const long long w = w0 + 32LL * i;
            bits[i] = w < mm.n_words ? mm.words[w] : 0u;
        }
        int cnt = 0;
#pragma unroll
        for (int i = 0; i < kMxWin; i++) {
            cnt += __popc(bits[i]);
            if (REQUEUE && bits[i]) mm.words[w0 + 32LL * i] = 0u;
        }
        if (!__any_sync(kFull, cnt != 0)) continue;
        if (REQUEUE) __syncwarp();
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
            // Owner: the last lane whose exclusive prefix is <= k; then the
            // owner's word that holds its (k - prefix)-th bit.
            int lo = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const int e = __shfl_sync(kFull, excl, lo + step);
                if (e <= k) lo += step;
            }
            int r = k - __shfl_sync(kFull, excl, lo), rank = 0, iw = 0;
            unsigned pick = 0u;
#pragma unroll
            for (int i = 0; i < kMxWin; i++) {
                const unsigned ob = __shfl_sync(kFull, bits[i], lo);
                const int c = __popc(ob);
                if (r >= 0 && r < c) {
                    pick = ob;
                    rank = r;
                    iw = i;
                }
                r -= c;
            }
            if (k < total) {
                const int bit = nth_bit(pick, rank);
                const long long word = win * kWinWords + 32LL * iw + lo;
                int det, t;
                mx_sample(segs, piece, mm, word, bit, det, t);
                const bool done = f(det, t);
                if (REQUEUE && !done) atomicOr(mm.words + word, 1u << bit);
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
// window of 32 x kMxWin words, at most 8 blocks per SM of 152 (the warps
// then stride).
inline unsigned mx_fix_blocks(const MxMask &mm) {
    const long long windows = (mm.n_words + 32LL * kMxWin - 1) / (32LL * kMxWin);
    const long long warps_per_block = kBlock / 32;
    long long b = (windows + warps_per_block - 1) / warps_per_block;
    if (b > 152LL * 8) b = 152LL * 8;
    return (unsigned)(b > 0 ? b : 1);
}

// Launches the fallback passes k.launch<T> for tiers T = FIRST..2 over
// mask mm in stream order; the first error stops the sequence.
template <int FIRST, class K>
int fix_tiers(const K &k, const MxMask &mm, cudaStream_t stream, const char *what) {
    const unsigned nb = mx_fix_blocks(mm);
    int rc = SO3G_OK;
    if constexpr (FIRST <= 0) {
        k.template launch<0>(nb, stream);
        rc = after_launch(what);
    }
    if constexpr (FIRST <= 1) {
        if (rc == SO3G_OK) {
            k.template launch<1>(nb, stream);
            rc = after_launch(what);
        }
    }
    if (rc == SO3G_OK) {
        k.template launch<2>(nb, stream);
        rc = after_launch(what);
    }
    return rc;
}

}  // namespace

}  // namespace so3g
