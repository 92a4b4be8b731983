// Internal to the library: plans, device state and error plumbing shared by the
// single-integral path (runtime.cpp) and the batch path (batch.cpp).
#pragma once

#include <cuda_runtime.h>

#include <exception>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/feyntrop_gb300.h"
#include "jit.hpp"
#include "problem.hpp"
#include "tune.hpp"
#include "xoshiro.hpp"

namespace ftrt {

extern thread_local std::string g_error;

struct cuda_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

inline void cu(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw cuda_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// status code of the exception in flight (sets g_error)
int status_of(const std::exception_ptr& ep);

// throws std::logic_error when there is no CUDA device
void require_device();

// per-device constants: the 64 skip matrices T^(2^b), the SM count
struct device_state {
    unsigned long long* tpow = nullptr;
    int sms = 0;
};
device_state& dev_state();

// the device parameter block of a plan: the FP64 values, then the same as floats,
// then as two-float (hi, lo) pairs (the layout the kernel body reads)
std::vector<double> param_block(const std::vector<double>& prm);

// sums of one integration (8K+8 slots) into the caller's result
void fill_result(const ft::prepared& P, const std::vector<double>& acc, ft_result* r);

}  // namespace ftrt

struct ft_plan {
    ft::prepared P;
    // the kernels' vertex labels: vertices without external momentum first, the external
    // ones last, the last of them the deleted (ground) vertex; kek/kel the edges in these
    // labels and kP the scalar products; reduced vertices [0, q0) carry no momentum
    std::vector<int> kek, kel;
    std::vector<double> kP;
    int q0 = 0;
    std::vector<double> sigma, q, prm;
    std::vector<unsigned char> tab;
    int device = 0;
    double* d_prm = nullptr;
    unsigned char* d_tab = nullptr;
    // scratch reused by launches
    double* d_parts = nullptr;
    size_t parts_cap = 0;
    double* d_final = nullptr;
    double* h_final = nullptr;
    unsigned long long* d_queue = nullptr;
    unsigned int* d_qcount = nullptr;
    size_t qcap = 0;
    // lane skip matrices for the last few per-thread strides S (alternating precisions
    // or sample counts reuse them): 64 matrices of 8 KB each per entry
    struct lane_entry {
        unsigned long long* d = nullptr;
        unsigned long long S = 0;
        int bits = 0;
        unsigned long long used = 0;
    };
    lane_entry lanes[4];
    unsigned long long lane_clock = 0;
    unsigned long long* d_lanepw = nullptr;   // the entry of the current launch
    unsigned long long* d_warpst = nullptr;   // stream states of the warps of the last launch
    size_t warpst_cap = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::mutex mu;
    // a launch shape under measurement by the autotuner (for one precision)
    bool forced = false;
    int forced_prec = 0;
    ft::launch_shape forced_shape;

    ft::kernel_key key(int prec, int record) const
    {
        ft::kernel_key k;
        k.E = P.E;
        k.V = P.V;
        k.K = P.K;
        k.loops = P.loops;
        k.rank = (int)sigma.size();
        k.prec = prec;
        k.mode = P.deformed() ? 1 : 0;
        k.only_psi = P.only_psi() ? 1 : 0;
        k.record = record;
        k.ek = kek;
        k.el = kel;
        k.q0 = q0;
        // tables are staged per block in shared memory up to E = 12 (102 KB FP64, 70 KB
        // mixed, beside one block's per-thread sums: the cube's mixed kernel ran 8 % faster
        // than reading its table through L1); from E = 13 on they are read through L1
        k.table_global = P.E >= 13 ? 1 : 0;
        // launch shape: a shape being measured by the autotuner, else the tuning table's
        // (or the default) for this kernel class
        ft::apply_shape(k, (forced && forced_prec == prec) ? forced_shape : ft::choose_shape(k));
        return k;
    }

    int slots() const { return 8 * P.K + 8; }

    ~ft_plan()
    {
        if (d_prm) cudaFree(d_prm);
        if (d_tab) cudaFree(d_tab);
        if (d_parts) cudaFree(d_parts);
        if (d_final) cudaFree(d_final);
        if (h_final) cudaFreeHost(h_final);
        if (d_queue) cudaFree(d_queue);
        if (d_qcount) cudaFree(d_qcount);
        for (lane_entry& e : lanes)
            if (e.d) cudaFree(e.d);
        if (d_warpst) cudaFree(d_warpst);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }
};
