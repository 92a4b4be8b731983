// ORACLE — test infrastructure only.
//
// A CPU restatement of feyntrop's tropical sampling + integrand evaluation loop,
// used solely as the checker for the GPU path (tests, the smoke check, and the CPU
// baseline leg of the benchmark).  Nothing in the product links, loads or calls it.
//
// What it restates, and where the reference does the same thing:
//   xoshiro256+ / splitmix64 streams ........ srcs/random.hpp:15-139
//   connected components .................... srcs/components.hpp:92-120
//   omega / PGP / reduced Laplacian ......... srcs/tropical_sampling.hpp:26-44,
//                                             srcs/laplacian.hpp:14-99
//   J(gamma) table + regime flags ........... srcs/tropical_sampling.hpp:46-458
//   Euclidean regime decision ............... srcs/feyntrop.cpp:128-133, 233-239
//   sector draw (cut scan + X, psi_tr, xi_tr) srcs/tropical_sampling.hpp:468-564
//   per-sample integrand (both branches) .... srcs/feynman_integral.hpp:162-362
//   x-derivatives of phi/psi ................ srcs/laplacian.hpp:102-215
//   stats / fp_summer / tree merge .......... srcs/stats.hpp:13-134
//
// The dense factorisations are written here from their textbook definitions with
// the pivot rules of the reference's linear-algebra library (LDLT pivoting on the
// largest original diagonal, complete-pivot LU, partial-pivot LU, first maximum
// wins), so that per-sample values track the reference to rounding level.
//
// Pinning: its J(gamma) tables and sector draws are compared bit for bit, and its
// per-sample values and single-thread integrals within a stated tolerance, with
// the reference binary and a harness built from the reference headers
// (tests/golden, made by tests/golden/make_golden.py).
#pragma once

#include <complex>
#include <cstdint>
#include <string>
#include <vector>

namespace fto {

struct xoshiro {
    uint64_t s[4];
    explicit xoshiro(uint64_t seed);
    uint64_t next();
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// advance a stream by `steps` calls of next() (GF(2) matrix power; test helper)
void skip(xoshiro& g, uint64_t steps);

struct problem {
    int E = 0, V = 0;
    std::vector<int> k, l;        // endpoints, normalised so that k > l
    std::vector<double> nu;       // edge weights
    std::vector<double> P;        // V x V scalar products, row major
    std::vector<double> m2;       // squared masses per edge
    double D = 4;
    int K = 1;
    double lambda = 0;
};

struct prepared {
    problem p;
    // table, indexed by the edge bitmask of gamma
    std::vector<double> Jr, r;
    std::vector<uint8_t> mm, L;
    double W = 0, W_ref = 0, IGtr = 0;
    int loops = 0;
    bool euclidean = true, pseudo_euclidean = true, generic = true, gp = true;
    bool W_zero = false;
    double def_ref = 0;           // -lambda when the deformation is active
    bool deformed() const { return def_ref != 0.0; }
};

// throws std::invalid_argument / std::domain_error with the reference's messages
prepared prepare(const problem& p);

struct sector {
    std::vector<int> order;       // removed edge at each step
    std::vector<double> X;        // X per edge (before rescaling)
    double psi_tr = 0, xi_tr = 0;
};

sector draw_sector(const prepared& pr, xoshiro& g);

struct sample_value {
    std::vector<std::complex<double>> R;   // per eps order
    bool dropped = false;
};

sample_value evaluate(const prepared& pr, const sector& s);

struct estimate {
    std::vector<double> re_avg, re_acc, im_avg, im_acc;
    uint64_t kept = 0, dropped = 0;
};

// Integrates N samples of stream `seed`.  Samples are split into `threads`
// contiguous blocks of the single stream, so the result does not depend on the
// thread count beyond summation order.
estimate integrate(const prepared& pr, uint64_t N, uint64_t seed, int threads);

}  // namespace fto
