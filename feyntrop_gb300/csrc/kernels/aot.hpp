// Host wrappers of the ahead-of-time kernels (aot.cu).
#pragma once

#include <cuda_runtime.h>

namespace ft {

// out[b] = (T^S)^(2^b), b < nbits; tpow = T^(2^j), j < 64 (1024 words per matrix)
cudaError_t launch_lane_powers(const unsigned long long* tpow, unsigned long long S, int nbits,
                               unsigned long long* out, cudaStream_t st);

// out[s] = sum over parts of parts[p * slots + s]; slots [0, ndd) are (hi, lo) pairs
cudaError_t launch_finalize(const double* parts, int nparts, int slots, int ndd, double* out, cudaStream_t st);

// FMA issue-rate probe (TFLOP/s, FMA = 2 flops) of the current device
double fma_peak_tflops(bool fp64);

}  // namespace ft
