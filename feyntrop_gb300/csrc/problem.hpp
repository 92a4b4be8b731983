// Host preprocessing for one Feynman integral: input validation, regime
// decision, and the J(gamma) subgraph table that the sampler walks.
//
// Follows, with the same checks, messages and floating-point operation order:
//   graph validation ............... srcs/graph.hpp:169-214
//   input checks ................... srcs/feyntrop.cpp:25-119
//   Euclidean decision ............. srcs/feyntrop.cpp:128-133
//   J(gamma) table, regime flags ... srcs/tropical_sampling.hpp:284-458
//   GP / genericity decisions ...... srcs/feyntrop.cpp:182-239
//   per-integral constants ......... srcs/feynman_integral.hpp:51-140
//
// The table is built in two passes: every subset's structural data (components,
// loop number, mass-momentum-spanning flag, the 2- and 3-cut kinematic tests) is
// independent of the others and is computed on all host threads; the Jr sums and
// the subdivergence / generalised-permutahedron checks then run layer by layer in
// the reference's subset order, which keeps every Jr bit-identical.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace ft {

struct problem_input {
    std::vector<int> v, w;       // edge endpoints as given
    std::vector<double> nu;      // edge weights
    int V = -1;                  // -1: derive from the edges
    std::vector<double> P;       // V x V row major
    std::vector<double> m2;      // E
    double D = 4;
    int K = 1;
    double lambda = 0;
};

struct prepared {
    int E = 0, V = 0, K = 1, loops = 0;
    std::vector<int> ek, el;     // normalised endpoints, ek > el
    std::vector<double> nu, P, m2;
    double D = 4, lambda_in = 0;

    std::vector<double> Jr, r;   // indexed by edge bitmask
    std::vector<uint8_t> mm, L;

    double W = 0, W_ref = 0, IGtr = 0;
    bool euclidean = true, pseudo_euclidean = true, generic = true, gp = true, W_zero = false;
    double lambda = 0;           // the deformation actually used
    double def_ref = 0;          // -lambda when the deformation is active
    std::vector<std::string> log; // stderr lines the reference prints before sampling
    double seconds_preprocessing = 0;

    bool deformed() const { return def_ref != 0.0; }
    bool only_psi() const { return W_zero && K == 1; }
};

// Throws std::invalid_argument, std::domain_error or std::runtime_error with the
// reference's messages on every input the reference rejects.
prepared prepare(const problem_input& in, int threads = 0);

// Eigenvalues of a symmetric matrix (cyclic Jacobi).
std::vector<double> symmetric_eigenvalues(std::vector<double> A, int n);

// glibc random(3) with its default seed, the source of the reference's probe points
struct glibc_random {
    uint32_t t[31];
    int f = 3, b = 0;
    glibc_random();
    int32_t next();
};

}  // namespace ft
