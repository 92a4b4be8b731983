// Topology-independent kernels, compiled ahead of time with nvcc for sm_103a.
//
//  ft_gf2_lane_powers  the skip matrices a sampling launch needs: P_b = (T^S)^(2^b)
//                      for b < nbits, where T is one xoshiro256+ step and S the number
//                      of draws per lane; one CTA of 256 threads, thread c owns
//                      column c of the 256x256 GF(2) matrices.
//  ft_finalize_parts   sums the per-block partial moments of one integration into a
//                      single vector: double-double for the moment slots, plain for
//                      the counters.
//  ft_batch_item_states  stream states of the work items of a batch (one warp per
//                      integral, GF(2) skip-ahead).
//  ft_batch_finalize   per-integral sums of a batch's work items and FP64 pass.
//  ft_warp_states      stream states of the warps of a sampling launch (one warp per
//                      warp, GF(2) skip-ahead), so each thread skips only its lane.
#include <cuda_runtime.h>

#include <mutex>

#include "aot.hpp"

typedef unsigned long long u64;

namespace {

// column c of A * B, A in shared memory by columns
__device__ __forceinline__ void gf2_col(const u64* A, const u64* bcol, u64* out)
{
    u64 r0 = 0, r1 = 0, r2 = 0, r3 = 0;
#pragma unroll
    for (int w = 0; w < 4; w++) {
        u64 bits = bcol[w];
        while (bits) {
            const int b = __ffsll((long long)bits) - 1;
            bits &= bits - 1;
            const u64* col = A + (w * 64 + b) * 4;
            r0 ^= col[0];
            r1 ^= col[1];
            r2 ^= col[2];
            r3 ^= col[3];
        }
    }
    out[0] = r0;
    out[1] = r1;
    out[2] = r2;
    out[3] = r3;
}

__global__ void __launch_bounds__(256) ft_gf2_lane_powers(const u64* __restrict__ tpow, u64 S, int nbits,
                                                          u64* __restrict__ out)
{
    __shared__ u64 A[1024];
    __shared__ u64 M[1024];
    const int c = threadIdx.x;
    for (int w = 0; w < 4; w++) M[c * 4 + w] = (w == (c >> 6)) ? (1ull << (c & 63)) : 0ull;
    __syncthreads();
    // M = T^S = product of T^(2^j) over the set bits j of S (powers of T commute)
    for (int j = 0; j < 64; j++) {
        if (!((S >> j) & 1ull)) continue;
        for (int w = 0; w < 4; w++) A[c * 4 + w] = tpow[(size_t)j * 1024 + c * 4 + w];
        __syncthreads();
        u64 r[4];
        gf2_col(A, M + c * 4, r);
        __syncthreads();
        for (int w = 0; w < 4; w++) M[c * 4 + w] = r[w];
        __syncthreads();
    }
    for (int b = 0; b < nbits; b++) {
        for (int w = 0; w < 4; w++) out[(size_t)b * 1024 + c * 4 + w] = M[c * 4 + w];
        if (b + 1 == nbits) break;
        for (int w = 0; w < 4; w++) A[c * 4 + w] = M[c * 4 + w];
        __syncthreads();
        u64 r[4];
        gf2_col(A, A + c * 4, r);
        __syncthreads();
        for (int w = 0; w < 4; w++) M[c * 4 + w] = r[w];
        __syncthreads();
    }
}

__device__ __forceinline__ void dd_add(double& ah, double& al, double bh, double bl)
{
    const double s = ah + bh;
    const double bb = s - ah;
    double err = (ah - (s - bb)) + (bh - bb);
    err += al + bl;
    ah = s + err;
    al = err - (ah - s);
}

// one block per slot pair (moments) or slot (counters): the block's threads take the
// parts in turn, then a double-double (or plain) tree across the block
__global__ void __launch_bounds__(256) ft_finalize_parts(const double* __restrict__ parts, int nparts, int slots,
                                                         int ndd, double* __restrict__ out)
{
    __shared__ double sh[8], sl[8];
    const int u = blockIdx.x;
    const int npairs = ndd / 2;
    const bool pair = u < npairs;
    const int s = pair ? 2 * u : ndd + (u - npairs);
    double h = 0.0, l = 0.0;
    for (int p = threadIdx.x; p < nparts; p += blockDim.x) {
        if (pair)
            dd_add(h, l, parts[(size_t)p * slots + s], parts[(size_t)p * slots + s + 1]);
        else
            h += parts[(size_t)p * slots + s];
    }
    for (int off = 16; off; off >>= 1) {
        const double oh = __shfl_down_sync(0xffffffffu, h, off), ol = __shfl_down_sync(0xffffffffu, l, off);
        if (pair)
            dd_add(h, l, oh, ol);
        else
            h += oh;
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        sh[w] = h;
        sl[w] = l;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double H = sh[0], L = sl[0];
        for (int i = 1; i < (int)(blockDim.x >> 5); i++) {
            if (pair)
                dd_add(H, L, sh[i], sl[i]);
            else
                H += sh[i];
        }
        out[s] = H;
        if (pair) out[s + 1] = L;
    }
}

// ------------------------------------------------------------------ batches
// Device views of the batch descriptors (layouts shared with the batch kernels of the
// sampling module and with batch.cpp).
struct batch_inst_view {
    const void* prm;
    const void* tab;
    u64 nsamples, first_item, nitems, pad[3];
};
struct item_prep {
    u64 s[4];         // seed state of the instance's stream
    u64 skip;         // draws before its first sample
    u64 first_item, nitems, pad;
};

__device__ __forceinline__ u64 word_of(const u64 (&g)[4], int w)
{
    return w == 0 ? g[0] : w == 1 ? g[1] : w == 2 ? g[2] : g[3];
}

// g <- M g over GF(2) by one warp: lane l owns input bits 8l .. 8l+7 (column c of M is
// the four words M[4c .. 4c+3]); the partial results are XOR-reduced across the warp
__device__ __forceinline__ void warp_gf2_apply(const u64* __restrict__ M, u64 (&g)[4], int lane)
{
    u64 r0 = 0, r1 = 0, r2 = 0, r3 = 0;
    const u64 sw = word_of(g, lane >> 3);
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int c = lane * 8 + k;
        const u64 mask = 0ull - ((sw >> (((lane & 7) << 3) + k)) & 1ull);
        const ulonglong2 lo = __ldg((const ulonglong2*)(M + 4 * c)), hi = __ldg((const ulonglong2*)(M + 4 * c + 2));
        r0 ^= lo.x & mask;
        r1 ^= lo.y & mask;
        r2 ^= hi.x & mask;
        r3 ^= hi.y & mask;
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) {
        r0 ^= __shfl_xor_sync(0xffffffffu, r0, off);
        r1 ^= __shfl_xor_sync(0xffffffffu, r1, off);
        r2 ^= __shfl_xor_sync(0xffffffffu, r2, off);
        r3 ^= __shfl_xor_sync(0xffffffffu, r3, off);
    }
    g[0] = r0;
    g[1] = r1;
    g[2] = r2;
    g[3] = r3;
}

// one warp per instance: the stream state of each of its work items' first samples
__global__ void __launch_bounds__(128) ft_batch_item_states(const item_prep* __restrict__ d, int n,
                                                            const u64* __restrict__ tpow,
                                                            const u64* __restrict__ itemM, u64* __restrict__ out)
{
    const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = (int)(threadIdx.x & 31u);
    if (w >= n) return;   // the whole warp
    u64 g[4] = {d[w].s[0], d[w].s[1], d[w].s[2], d[w].s[3]};
    const u64 skip = d[w].skip;
    for (int b = 0; b < 64; b++)
        if ((skip >> b) & 1ull) warp_gf2_apply(tpow + (size_t)b * 1024, g, lane);
    const u64 f = d[w].first_item, m = d[w].nitems;
    for (u64 k = 0; k < m; k++) {
        if (lane < 4) out[(f + k) * 4 + lane] = word_of(g, lane);
        if (k + 1 < m) warp_gf2_apply(itemM, g, lane);
    }
}

// one warp per output warp: the first lane's state of warp w of a sampling launch is
// (T^S)^(32 w) base, i.e. the lane skip matrices of the bits of w shifted by 5
__global__ void __launch_bounds__(128) ft_warp_states(const u64* __restrict__ lanepw, int lanebits, u64 s0, u64 s1,
                                                      u64 s2, u64 s3, unsigned nwarps, u64* __restrict__ out)
{
    const unsigned w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = (int)(threadIdx.x & 31u);
    if (w >= nwarps) return;   // the whole warp
    u64 g[4] = {s0, s1, s2, s3};
    for (int j = 0; j + 5 < lanebits; j++)
        if ((w >> j) & 1u) warp_gf2_apply(lanepw + (size_t)(j + 5) * 1024, g, lane);
    if (lane < 4) out[(size_t)w * 4 + lane] = word_of(g, lane);
}

// An exact fixed-point accumulator (kExactDigits signed 64-bit digits of weight
// 2^(32 j - 1074)) as a double-double: carries normalised from the lowest digit up
// (digits in [0, 2^32), the sign in the final carry), a negative total negated, then
// the digits added from the most significant down.
__device__ void exact_to_dd(const u64* __restrict__ dig, double& h, double& l)
{
    unsigned int d[ft::kExactDigits];
    long long carry = 0;
    for (int j = 0; j < ft::kExactDigits; j++) {
        const long long t = (long long)dig[j] + carry;
        d[j] = (unsigned int)(unsigned long long)t;
        carry = t >> 32;
    }
    const bool neg = carry < 0;
    if (neg) {
        // two's complement of the digit vector: invert, add one
        unsigned long long c = 1;
        for (int j = 0; j < ft::kExactDigits; j++) {
            const unsigned long long t = (unsigned long long)(~d[j]) + c;
            d[j] = (unsigned int)t;
            c = t >> 32;
        }
    }
    h = 0.0;
    l = 0.0;
    for (int j = ft::kExactDigits - 1; j >= 0; j--)
        if (d[j]) dd_add(h, l, ldexp((double)d[j], 32 * j - 1074), 0.0);
    if (neg) {
        h = -h;
        l = -l;
    }
}

// Per instance: the sums of its work items (double-double for the moment pairs) plus
// the FP64 pass's exact sums (qacc, NULL for FP64 batches).  One thread per (instance,
// moment pair or counter).  Slots: 8K moments as 4K (hi, lo) pairs, then kept,
// dropped, queued, exact, robust, 3 spare; qacc: 4K exact accumulators, then kept,
// dropped, robust, spare.
__global__ void ft_batch_finalize(const batch_inst_view* __restrict__ inst, int n, const double* __restrict__ parts,
                                  int K, const u64* __restrict__ qacc, double* __restrict__ out)
{
    const int slots = 8 * K + 8, units = 4 * K + 8;
    const u64 qwords = 4ull * (u64)K * ft::kExactDigits + 4ull;   // ft::exact_words(K)
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * units) return;
    const int m = (int)(t / units), u = (int)(t % units);
    const u64 f = inst[m].first_item, cnt = inst[m].nitems;
    double* o = out + (size_t)m * slots;
    if (u < 4 * K) {
        double h = 0.0, l = 0.0;
        for (u64 k = 0; k < cnt; k++)
            dd_add(h, l, parts[(f + k) * slots + 2 * u], parts[(f + k) * slots + 2 * u + 1]);
        if (qacc) {
            double qh, ql;
            exact_to_dd(qacc + (size_t)m * qwords + (size_t)u * ft::kExactDigits, qh, ql);
            dd_add(h, l, qh, ql);
        }
        o[2 * u] = h;
        o[2 * u + 1] = l;
    } else {
        const int c = u - 4 * K;
        double v = 0.0;
        for (u64 k = 0; k < cnt; k++) v += parts[(f + k) * slots + 8 * K + c];
        if (qacc) {
            const u64* cnt4 = qacc + (size_t)m * qwords + 4ull * K * ft::kExactDigits;
            if (c == 0) v += (double)cnt4[0];
            if (c == 1) v += (double)cnt4[1];
            if (c == 4) v += (double)cnt4[2];
        }
        o[8 * K + c] = v;
    }
}

// Issue-rate probes for the roofline denominators: every thread runs 8 independent
// FMA chains, so the pipe, not the dependency latency, limits the rate.
template <class T>
__global__ void __launch_bounds__(256) ft_fma_probe(T* __restrict__ out, int iters, T a, T b)
{
    T x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = (T)(threadIdx.x + k) * (T)1e-3;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = x[k] * a + b;
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) s += x[k];
    if (s == (T)12345.678) out[threadIdx.x] = s;   // keeps the chains alive
}

}  // namespace

namespace ft {

// FMA issue rate in TFLOP/s (2 flops per FMA), timed with CUDA events
double fma_peak_tflops(bool fp64)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void* buf = nullptr;
    cudaMalloc(&buf, 4096);
    const int blocks = sms * 8, iters = fp64 ? 2048 : 65536;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(e0);
        if (fp64)
            ft_fma_probe<double><<<blocks, 256>>>((double*)buf, iters, 0.999999, 1e-7);
        else
            ft_fma_probe<float><<<blocks, 256>>>((float*)buf, iters, 0.999999f, 1e-7f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    const double flops = 2.0 * 8 * (double)iters * blocks * 256;
    return flops / (best * 1e-3) / 1e12;
}

// ------------------------------------------------------------------ no-allocation scratch
// Scratch of ft_integrate_noalloc, for callers that must not allocate device memory
// during an integration.  It is one file-scope device array per GPU that loads this
// library, held until the process exits:
//   [2 words] FP64 hand-off queue count, [NOALLOC_PART_DOUBLES] per-block partial
//   moments, [5 * NOALLOC_QUEUE_ENTRIES] hand-off queue, [NOALLOC_LANE_WORDS] lane
//   skip matrices, [NOALLOC_WARP_WORDS] warp start states.
// Every call shares it (and it keeps the last call's contents), so calls that overlap
// on the GPU race; the queue count is cleared at the start of each call.
constexpr unsigned long long kNoallocParts = 2, kNoallocQueue = kNoallocParts + NOALLOC_PART_DOUBLES,
                             kNoallocLanes = kNoallocQueue + 5ull * NOALLOC_QUEUE_ENTRIES,
                             kNoallocWarps = kNoallocLanes + NOALLOC_LANE_WORDS;
// the regions end inside the array, and each holds what the host-side checks of
// ft_integrate_noalloc let a call use: 2048 blocks of up to 8K+8 = 136 slots (16 eps
// orders), the stream states of every warp of 2048 blocks of up to 1024 threads, the
// 1024-word skip matrices of up to 24 lane bits
static_assert(kNoallocWarps + NOALLOC_WARP_WORDS <= NOALLOC_TOTAL_WORDS, "no-allocation layout overruns");
static_assert(NOALLOC_PART_DOUBLES >= NOALLOC_MAX_BLOCKS * (8 * 16 + 8), "partial sums of 16 eps orders");
static_assert(NOALLOC_WARP_WORDS >= NOALLOC_MAX_BLOCKS * (1024 / 32) * 4, "warp states of 1024-thread blocks");
static_assert(NOALLOC_LANE_WORDS >= NOALLOC_MAX_LANE_BITS * 1024, "lane skip matrices");
static_assert(kNoallocQueue % 2 == 0 && kNoallocLanes % 2 == 0 && kNoallocWarps % 2 == 0,
              "16-byte aligned regions (ulonglong2 loads)");
static __device__ __align__(256) u64 g_noalloc_scratch[NOALLOC_TOTAL_WORDS];

cudaError_t noalloc_scratch(noalloc_layout* out)
{
    // In host code g_noalloc_scratch names a host-side stand-in; the device address is
    // looked up once per device, with that device current.
    static std::mutex mu;
    static void* addr[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!addr[dev]) {
            e = cudaGetSymbolAddress(&addr[dev], g_noalloc_scratch);
            if (e != cudaSuccess) {
                addr[dev] = nullptr;
                return e;
            }
        }
        base = addr[dev];
    }
    u64* w = (u64*)base;
    out->qcount = (unsigned int*)w;
    out->parts = (double*)(w + kNoallocParts);
    out->queue = w + kNoallocQueue;
    out->lanepw = w + kNoallocLanes;
    out->warpst = w + kNoallocWarps;
    return cudaSuccess;
}

cudaError_t launch_lane_powers(const u64* tpow, u64 S, int nbits, u64* out, cudaStream_t st)
{
    ft_gf2_lane_powers<<<1, 256, 0, st>>>(tpow, S, nbits, out);
    return cudaGetLastError();
}

cudaError_t launch_batch_item_states(const void* prep, int n, const u64* tpow, const u64* itemM, u64* out,
                                     cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    ft_batch_item_states<<<(n + 3) / 4, 128, 0, st>>>((const item_prep*)prep, n, tpow, itemM, out);
    return cudaGetLastError();
}

cudaError_t launch_batch_finalize(const void* inst, int n, const double* parts, int K,
                                  const unsigned long long* qacc, double* out, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const long long threads = (long long)n * (4 * K + 8);
    ft_batch_finalize<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>((const batch_inst_view*)inst, n, parts, K,
                                                                         qacc, out);
    return cudaGetLastError();
}

cudaError_t launch_warp_states(const u64* lanepw, int lanebits, const u64* base, unsigned nwarps, u64* out,
                               cudaStream_t st)
{
    if (nwarps == 0) return cudaSuccess;
    ft_warp_states<<<(nwarps + 3) / 4, 128, 0, st>>>(lanepw, lanebits, base[0], base[1], base[2], base[3], nwarps, out);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const double* parts, int nparts, int slots, int ndd, double* out, cudaStream_t st)
{
    const int units = ndd / 2 + (slots - ndd);
    ft_finalize_parts<<<units, 256, 0, st>>>(parts, nparts, slots, ndd, out);
    return cudaGetLastError();
}

}  // namespace ft
