// Topology-independent kernels, compiled ahead of time with nvcc for sm_103a.
//
//  ft_gf2_lane_powers  the skip matrices a sampling launch needs: P_b = (T^S)^(2^b)
//                      for b < nbits, where T is one xoshiro256+ step and S the number
//                      of draws per lane; one CTA of 256 threads, thread c owns
//                      column c of the 256x256 GF(2) matrices.
//  ft_finalize_parts   sums the per-block partial moments of one integration into a
//                      single vector: double-double for the moment slots, plain for
//                      the counters.
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

// one thread per slot pair (moments) or slot (counters)
__global__ void ft_finalize_parts(const double* __restrict__ parts, int nparts, int slots, int ndd,
                                  double* __restrict__ out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int npairs = ndd / 2;
    if (t < npairs) {
        double h = 0.0, l = 0.0;
        for (int p = 0; p < nparts; p++) dd_add(h, l, parts[(size_t)p * slots + 2 * t], parts[(size_t)p * slots + 2 * t + 1]);
        out[2 * t] = h;
        out[2 * t + 1] = l;
    } else if (t < npairs + (slots - ndd)) {
        const int s = ndd + (t - npairs);
        double v = 0.0;
        for (int p = 0; p < nparts; p++) v += parts[(size_t)p * slots + s];
        out[s] = v;
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
//   skip matrices.
// Every call shares it (and it keeps the last call's contents), so calls that overlap
// on the GPU race; the queue count is cleared at the start of each call.
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
    out->parts = (double*)(w + 2);
    out->queue = w + 2 + NOALLOC_PART_DOUBLES;
    out->lanepw = w + 2 + NOALLOC_PART_DOUBLES + 5 * (size_t)NOALLOC_QUEUE_ENTRIES;
    return cudaSuccess;
}

cudaError_t launch_lane_powers(const u64* tpow, u64 S, int nbits, u64* out, cudaStream_t st)
{
    ft_gf2_lane_powers<<<1, 256, 0, st>>>(tpow, S, nbits, out);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const double* parts, int nparts, int slots, int ndd, double* out, cudaStream_t st)
{
    const int threads = ndd / 2 + (slots - ndd);
    ft_finalize_parts<<<(threads + 127) / 128, 128, 0, st>>>(parts, nparts, slots, ndd, out);
    return cudaGetLastError();
}

}  // namespace ft
