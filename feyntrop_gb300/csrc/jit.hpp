// Run-time compilation of the sampling kernels for one graph topology.
//
// The kernel body (kernels/sample_body.cuh, embedded in the library at build
// time) is prefixed with the topology as compile-time constants and compiled by
// NVRTC straight to an sm_103a cubin.  Cubins are cached in memory per device
// and on disk (FEYNTROP_GB300_CACHE, else a _jit_cache folder beside the
// library), keyed by a hash of the full source and options.
#pragma once

#include <cuda.h>

#include <string>
#include <vector>

namespace ft {

struct kernel_key {
    int E = 0, V = 0, K = 1, loops = 0, rank = 1;
    int table_global = 0;   // read the table from global memory instead of staging it
    int prec = 0;       // 0 FP64, 1 mixed
    int mode = 0;       // 0 undeformed, 1 deformed
    int only_psi = 0;
    int record = 0;
    int block = 128;
    int minb = 1;           // minimum resident blocks per SM asked of the register allocator
    int variant = 0;        // code-size options of the kernel body (FT_VARIANT)
    int batch = 0;          // 1: the batch kernels (many integrals of the topology per launch)
    int q0 = 0;             // reduced vertices [0, q0) carry no external momentum (zero rows of P~)
    std::vector<int> ek, el;   // endpoints in the kernel's vertex labels, ek > el
};

struct kernel_set {
    CUmodule module = nullptr;
    CUfunction sample = nullptr;   // ft_sample (ft_sample_batch in batch modules)
    CUfunction queue = nullptr;    // ft_sample_queue / ft_sample_queue_batch (FP64 modules only)
    int block = 128;
    int variant = 0;               // FT_VARIANT of the module
    unsigned smem = 0;             // dynamic shared memory per block
    int regs = 0;
    int local_bytes = 0;
    int blocks_per_sm = 0;         // of ft_sample at this block size and smem
    int queue_blocks_per_sm = 0;
    double compile_seconds = 0;
};

std::string kernel_source(const kernel_key& key);

// directory of the compiled-kernel cache (and of the launch-shape tuning table)
std::string cache_dir();

// shared memory the kernel stages the table into (0 when read from global memory)
unsigned table_smem_bytes(const kernel_key& key);

struct driver_api {
    CUresult (*ModuleLoadData)(CUmodule*, const void*);
    CUresult (*ModuleGetFunction)(CUfunction*, CUmodule, const char*);
    CUresult (*FuncSetAttribute)(CUfunction, CUfunction_attribute, int);
    CUresult (*FuncGetAttribute)(int*, CUfunction_attribute, CUfunction);
    CUresult (*OccupancyMaxActiveBlocksPerMultiprocessor)(int*, CUfunction, int, size_t);
    CUresult (*LaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                             CUstream, void**, void**);
    CUresult (*GetErrorString)(CUresult, const char**);
};
driver_api& drv();
void check(CUresult r, const char* what);

// compiled and loaded on the current device (throws std::runtime_error)
const kernel_set& get_kernels(const kernel_key& key);

// already loaded on the current device, else nullptr (never compiles or loads)
const kernel_set* find_kernels(const kernel_key& key);

// compile only (no device needed); returns the cubin size
size_t compile_only(const kernel_key& key, std::string* log = nullptr);

// compile into the on-disk cache unless it is there already
void precompile(const kernel_key& key);
// the cubins of several keys, compiled concurrently on the host's threads
void precompile_all(const std::vector<kernel_key>& keys);

}  // namespace ft
