// Host wrappers of the ahead-of-time kernels (aot.cu).
#pragma once

#include <cuda_runtime.h>

namespace ft {

// out[b] = (T^S)^(2^b), b < nbits; tpow = T^(2^j), j < 64 (1024 words per matrix)
cudaError_t launch_lane_powers(const unsigned long long* tpow, unsigned long long S, int nbits,
                               unsigned long long* out, cudaStream_t st);

// Batches (layouts in aot.cu): item stream states from per-instance item_prep records
// (one warp per instance), and the per-instance sums of the work items plus the FP64
// pass (qacc may be NULL).
cudaError_t launch_batch_item_states(const void* prep, int n, const unsigned long long* tpow,
                                     const unsigned long long* itemM, unsigned long long* out, cudaStream_t st);
cudaError_t launch_batch_finalize(const void* inst, int n, const double* parts, int K,
                                  const unsigned long long* qacc, double* out, cudaStream_t st);

// The FP64 pass of a mixed batch adds each handed-off sample's values exactly into
// per-integral fixed-point accumulators: digit j (a signed 64-bit counter) has weight
// 2^(32 j - 1074), and a double enters as three signed 32-bit digits of its integer
// significand, so the sums are exact and independent of the order of the atomics.
// Per integral: 4K accumulators of kExactDigits words, then 4 counters (kept,
// dropped, robust, spare).  The kernel source gets the same count as FT_XA_DIGITS.
constexpr int kExactDigits = 68;
inline unsigned long long exact_words(int K) { return 4ull * (unsigned long long)K * kExactDigits + 4ull; }

// out[s] = sum over parts of parts[p * slots + s]; slots [0, ndd) are (hi, lo) pairs
cudaError_t launch_finalize(const double* parts, int nparts, int slots, int ndd, double* out, cudaStream_t st);

// Limits of the no-allocation path (ft_integrate_noalloc): per-block partial moments
// for up to 2048 blocks of up to 136 slots (16 eps orders), 65536 FP64 hand-off
// entries, lane skip matrices for up to 2^24 lanes, the stream states of up to 32
// warps per block.  About 7 MB per device.
#define NOALLOC_MAX_BLOCKS 2048
#define NOALLOC_MAX_SLOTS 136
#define NOALLOC_PART_DOUBLES (NOALLOC_MAX_BLOCKS * NOALLOC_MAX_SLOTS)
#define NOALLOC_QUEUE_ENTRIES 65536
#define NOALLOC_MAX_LANE_BITS 24
#define NOALLOC_LANE_WORDS (NOALLOC_MAX_LANE_BITS * 1024)
#define NOALLOC_WARP_WORDS (NOALLOC_MAX_BLOCKS * 32 * 4)
#define NOALLOC_TOTAL_WORDS \
    (2 + NOALLOC_PART_DOUBLES + 5 * NOALLOC_QUEUE_ENTRIES + NOALLOC_LANE_WORDS + NOALLOC_WARP_WORDS)

struct noalloc_layout {
    unsigned int* qcount;
    double* parts;
    unsigned long long* queue;
    unsigned long long* lanepw;
    unsigned long long* warpst;
};

// stream states of the first lane of every warp of a launch: warp w starts at
// (T^S)^(32 w) base, from the lane skip matrices lanepw[b] = (T^S)^(2^b), b < lanebits
cudaError_t launch_warp_states(const unsigned long long* lanepw, int lanebits, const unsigned long long* base,
                               unsigned nwarps, unsigned long long* out, cudaStream_t st);

// device addresses inside the static scratch of the current device (first call per
// device looks the symbol up)
cudaError_t noalloc_scratch(noalloc_layout* out);

// FMA issue-rate probe (TFLOP/s, FMA = 2 flops) of the current device
double fma_peak_tflops(bool fp64);

}  // namespace ft
