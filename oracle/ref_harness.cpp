// Test-infrastructure harness compiled from the reference's own headers (the
// include path points at the reference checkout at build time; nothing from it
// is copied here).  It exposes reference functions that the stock `feyntrop`
// binary does not print, so that the oracle restatement can be pinned to them:
//
//   ref_harness table   < input.json   -> the J(gamma) table of
//                                          generate_subgraph_table
//                                          (srcs/tropical_sampling.hpp:284-458),
//                                          every double as its IEEE bit pattern
//   ref_harness sectors n < input.json -> n consecutive draws of
//                                          get_random_psi_xi_tropical_sample
//                                          (srcs/tropical_sampling.hpp:503-564)
//                                          from the seed's stream 0, i.e. the
//                                          stream feynman_integral_estimate gives
//                                          thread 0 (srcs/feynman_integral.hpp:85-93)
//
// The regime flag (Euclidean or not) is decided the way srcs/feyntrop.cpp:128-133
// decides it, because generate_subgraph_table takes it as an argument.

#include <cstdio>
#include <cstring>
#include <iostream>
#include <algorithm>
#include <numeric>

#include <Eigen/Eigenvalues>
#include <nlohmann/json.hpp>

#include "graph.hpp"
#include "tropical_sampling.hpp"

using json = nlohmann::json;

static uint64_t bits_of(double x)
{
    uint64_t u;
    std::memcpy(&u, &x, sizeof u);
    return u;
}

static std::string hex(double x)
{
    char buf[32];
    std::snprintf(buf, sizeof buf, "%016llx", (unsigned long long)bits_of(x));
    return buf;
}

struct problem
{
    graph g;
    Eigen::MatrixXd P;
    Eigen::VectorXd m2;
    double D;
    int K;
    uint64_t seed;
    bool euclidean;
};

static graph::edge_vector read_edges(const json& data)
{
    graph::edge_vector edges;
    for (auto& edge : data["graph"])
        edges.push_back({{(int)edge[0][0], (int)edge[0][1]}, (double)edge[1]});
    return edges;
}

static problem read_problem()
{
    json data = json::parse(std::cin);
    graph g(read_edges(data));
    Eigen::MatrixXd P(g._V, g._V);
    for (int k = 0; k < g._V; k++)
        for (int l = 0; l < g._V; l++)
            P(k, l) = data["scalarproducts"][k][l];
    Eigen::VectorXd m2(g._E);
    for (int e = 0; e < g._E; e++)
        m2[e] = data["masses_sqr"][e];

    Eigen::SelfAdjointEigenSolver<Eigen::MatrixXd> es(P);
    Eigen::MatrixXd P_abs = -es.eigenvectors() * es.eigenvalues().cwiseAbs().asDiagonal() * es.eigenvectors().inverse();
    bool euclidean = P.isZero() || P.isApprox(P_abs);

    return problem{g, P, m2, (double)data["dimension"], (int)data["num_eps_terms"],
                   (uint64_t)data["seed"], euclidean};
}

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::fprintf(stderr, "usage: ref_harness table|sectors [n] < input.json\n");
        return 2;
    }
    std::string mode = argv[1];
    problem p = read_problem();

    J_vector table;
    double W, IGtr;
    bool gp, pseudo, generic;
    std::tie(table, W, IGtr, gp, pseudo, generic) =
        generate_subgraph_table(p.g, p.D, p.P, p.m2, p.K > 1, !p.euclidean);

    if (mode == "table") {
        json out;
        out["E"] = p.g._E;
        out["V"] = p.g._V;
        out["W"] = hex(W);
        out["IGtr"] = hex(IGtr);
        out["gp"] = gp;
        out["pseudo_euclidean"] = pseudo;
        out["generic"] = generic;
        out["euclidean"] = p.euclidean;
        std::vector<std::string> Jr, r;
        std::vector<int> mm, L;
        for (auto& t : table) {
            Jr.push_back(hex(std::get<0>(t)));
            r.push_back(hex(std::get<1>(t)));
            mm.push_back((int)std::get<2>(t));
            L.push_back((int)std::get<3>(t));
        }
        out["Jr"] = Jr;
        out["r"] = r;
        out["mm"] = mm;
        out["L"] = L;
        std::cout << out.dump() << std::endl;
        return 0;
    }

    if (mode == "sectors") {
        long n = argc > 2 ? std::atol(argv[2]) : 16;
        true_random::xoshiro256 gen(p.seed);
        Eigen::VectorXd X(p.g._E);
        json out = json::array();
        for (long i = 0; i < n; i++) {
            double psi_tr, xi_tr;
            std::tie(psi_tr, xi_tr) = get_random_psi_xi_tropical_sample(X, p.g, table, gen);
            // X of an edge is the running product at the step that removed it, and that
            // product never grows, so sorting by X (descending) recovers the removal order.
            std::vector<int> order(p.g._E);
            std::iota(order.begin(), order.end(), 0);
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return X[a] > X[b]; });
            std::vector<std::string> xs;
            for (int e = 0; e < p.g._E; e++)
                xs.push_back(hex(X[e]));
            out.push_back({{"order", order}, {"X", xs}, {"psi_tr", hex(psi_tr)}, {"xi_tr", hex(xi_tr)}});
        }
        std::cout << out.dump() << std::endl;
        return 0;
    }

    std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 2;
}
