// Launch shapes of the sampling kernels: defaults from sweeps on GB300 and a tuning
// table filled by the autotuner (ft_autotune), persisted next to the kernel cache.
#pragma once

#include <string>

#include "jit.hpp"

namespace ft {

struct launch_shape {
    int block = 256;               // threads per block
    int minb = 1;                  // minimum resident blocks per SM given to the register allocator
    int variant = 0;               // FT_VARIANT code-size options of the kernel body
    unsigned long long chunk = 0;  // batch work item: samples per thread (0: default)
    double rate = 0;               // samples/s measured when tuned (0: default shape)
};

// tuning class of a kernel: topology, eps orders, regime, precision, table placement
std::string tune_class(const kernel_key& k);

// the shape the sampling kernels of key k use: tuned if the table has the class, else
// the defaults (launch fields of k are ignored); FEYNTROP_GB300_BLOCK / _MINB / _VARIANT
// override, and the block shrinks until the shared memory fits an SM
launch_shape choose_shape(const kernel_key& k);

// default shape (no table, no environment)
launch_shape default_shape(const kernel_key& k);

// record a tuned shape for the class of k (in memory and in the table file)
void record_shape(const kernel_key& k, const launch_shape& s);

// forget tuned shapes (in memory; the file is rewritten by the next record)
void clear_shapes();

// applies shape s to k and shrinks the block until its shared memory fits
void apply_shape(kernel_key& k, const launch_shape& s);

// batch work-item size forced on batches created by this thread (0: none); the
// autotuner sets it while it measures candidates
void set_chunk_override(unsigned long long chunk);
unsigned long long chunk_override();

}  // namespace ft
