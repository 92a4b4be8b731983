// The reference's low-level interface in process: JSON in, JSON out
// (srcs/feyntrop.cpp:20-281).  Same keys, the same input checks and messages, the
// same output object; diagnostics go to the log text (stderr in the CLI).
//
// Optional keys beyond the reference's eight (unchanged inputs behave identically):
//   "precision": "fp64" (default) | "mixed"
//   "first_sample": index of the first sample of the seed's stream (sharding)
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/feyntrop_gb300.h"
#include "json.hpp"

namespace {

thread_local std::string g_err;

const char* kGraphMsg = "input graph must be a list of the form [[[v1_1,v2_1],nu_1],[[v1_2,v2_2],nu_2],...]";

struct parsed {
    std::vector<int32_t> edges;
    std::vector<double> nu, P, m2;
    int V = 0;
    double D = 0, lambda = 0;
    int K = 1;
    uint64_t N = 0, seed = 0, first = 0;
    int precision = FT_PRECISION_FP64;
};

parsed parse_input(const std::string& text)
{
    const ftj::value data = ftj::parse(text);
    const char* keys[] = {"N", "graph", "dimension", "scalarproducts", "masses_sqr", "num_eps_terms", "lambda", "seed"};
    for (const char* k : keys)
        if (!data.contains(k))
            throw std::invalid_argument(
                "input json must contain the data fields: N, graph, dimension, scalarproducts, masses_sqr, "
                "num_eps_terms, lambda, seed");
    if (!data["N"].is_number()) throw std::invalid_argument("input N must be a number");
    if (!data["lambda"].is_number()) throw std::invalid_argument("input lambda must be a number");
    if (!data["dimension"].is_number()) throw std::invalid_argument("input dimension must be a number");
    if (!data["num_eps_terms"].is_number()) throw std::invalid_argument("input num_eps_terms must be a number");
    if (!data["seed"].is_number()) throw std::invalid_argument("input seed must be a number");
    parsed p;
    p.N = ftj::as_u64(data["N"]);
    p.seed = ftj::as_u64(data["seed"]);
    p.lambda = data["lambda"].num;
    p.D = data["dimension"].num;
    p.K = ftj::as_int(data["num_eps_terms"]);
    if (!data["graph"].is_array()) throw std::invalid_argument(kGraphMsg);
    int Vmax = 0;
    for (const ftj::value& e : data["graph"].arr) {
        if (!e.is_array() || e.size() != 2 || !e[0].is_array() || e[0].size() != 2) throw std::invalid_argument(kGraphMsg);
        if (!e[0][0].is_number() || !e[0][1].is_number() || !e[1].is_number()) throw std::invalid_argument(kGraphMsg);
        int k = ftj::as_int(e[0][0]), l = ftj::as_int(e[0][1]);
        p.edges.push_back(k);
        p.edges.push_back(l);
        p.nu.push_back(e[1].num);
        Vmax = std::max(Vmax, std::max(k, l) + 1);
    }
    p.V = Vmax;
    const ftj::value& sp = data["scalarproducts"];
    if (!sp.is_array() || (int)sp.size() != p.V) throw std::invalid_argument("input scalarproducts must be a (V x V)-matrix");
    for (int k = 0; k < p.V; k++) {
        if (!sp[k].is_array() || (int)sp[k].size() != p.V)
            throw std::invalid_argument("input scalarproducts must be a (V x V)-matrix");
        for (int l = 0; l < p.V; l++) {
            if (!sp[k][l].is_number()) throw std::invalid_argument("input scalarproducts must be a (V x V)-matrix");
            p.P.push_back(sp[k][l].num);
        }
    }
    const ftj::value& m = data["masses_sqr"];
    const int E = (int)p.nu.size();
    if (!m.is_array() || (int)m.size() != E) throw std::invalid_argument("input masses_sqr must be an array of size E");
    for (int e = 0; e < E; e++) {
        if (!m[e].is_number()) throw std::invalid_argument("input masses_sqr must be an array of size E");
        p.m2.push_back(m[e].num);
    }
    if (data.contains("precision")) {
        const ftj::value& pr = data["precision"];
        if (pr.kind == ftj::value::string_k && pr.str == "mixed")
            p.precision = FT_PRECISION_MIXED;
        else if (pr.kind == ftj::value::string_k && pr.str == "fp64")
            p.precision = FT_PRECISION_FP64;
        else
            throw std::invalid_argument("input precision must be \"fp64\" or \"mixed\"");
    }
    if (data.contains("first_sample")) p.first = ftj::as_u64(data["first_sample"]);
    return p;
}

char* dup(const std::string& s)
{
    char* c = (char*)std::malloc(s.size() + 1);
    std::memcpy(c, s.c_str(), s.size() + 1);
    return c;
}

}  // namespace

extern "C" int ft_run_json(const char* input_json, char** output, char** log)
{
    std::ostringstream lg;
    *output = nullptr;
    if (log) *log = nullptr;
    int rc = FT_OK;
    try {
        parsed in = parse_input(input_json ? input_json : "");
        ft_problem pb;
        pb.num_edges = (int32_t)in.nu.size();
        pb.edges = in.edges.data();
        pb.nu = in.nu.data();
        pb.num_vertices = in.V;
        pb.scalarproducts = in.P.data();
        pb.masses_sqr = in.m2.data();
        pb.dimension = in.D;
        pb.num_eps_terms = in.K;
        pb.lambda = in.lambda;
        ft_plan* plan = nullptr;
        rc = ft_plan_create(&pb, &plan);
        if (rc != FT_OK) {
            lg << ft_last_error() << "\n";
            if (log) *log = dup(lg.str());
            return rc;
        }
        ft_plan_info info;
        ft_plan_get_info(plan, &info);
        for (int i = 0; i < info.num_log_lines; i++) lg << ft_plan_log_line(plan, i) << "\n";
        int dev = 0;
        cudaDeviceProp prop;
        cudaGetDevice(&dev);
        cudaGetDeviceProperties(&prop, dev);
        lg << "Started integrating on " << prop.name << " ("
           << (in.precision == FT_PRECISION_MIXED ? "mixed FP32/FP64" : "FP64") << ") and N = " << (double)in.N
           << " points.\n";
        const int K = in.K;
        std::vector<double> ra(K), rs(K), ia(K), is(K);
        ft_result res;
        std::memset(&res, 0, sizeof res);
        res.re_avg = ra.data();
        res.re_acc = rs.data();
        res.im_avg = ia.data();
        res.im_acc = is.data();
        ft_run_options o;
        o.num_samples = in.N;
        o.seed = in.seed;
        o.first_sample = in.first;
        o.precision = in.precision;
        o.stream = nullptr;
        rc = ft_integrate(plan, &o, &res);
        if (rc != FT_OK) {
            lg << ft_last_error() << "\n";
            ft_plan_destroy(plan);
            if (log) *log = dup(lg.str());
            return rc;
        }
        if (res.dropped)
            lg << "Warning: " << res.dropped
               << " sampled values were not finite - floating point accuracy or numerical stability seem to be "
                  "insufficient - these points were dropped. If this happens often, the result will not be "
                  "reliable.\n";
        lg << "Finished in " << (res.seconds_sampling + info.seconds_preprocessing) << " seconds = "
           << (res.seconds_sampling + info.seconds_preprocessing) / 3600 << " hours.\n";
        std::ostringstream out;
        out << "{\"IGtr\":" << ftj::number(info.IGtr) << ",\"integral\":[";
        for (int j = 0; j < K; j++) {
            if (j) out << ",";
            out << "[[" << ftj::number(ra[j]) << "," << ftj::number(rs[j]) << "],[" << ftj::number(ia[j]) << ","
                << ftj::number(is[j]) << "]]";
        }
        out << "],\"seconds preprocessing\":" << ftj::number(info.seconds_preprocessing)
            << ",\"seconds sampling\":" << ftj::number(res.seconds_sampling) << "}";
        *output = dup(out.str());
        ft_plan_destroy(plan);
    } catch (const std::invalid_argument& e) {
        lg << e.what() << "\n";
        g_err = e.what();
        rc = FT_ERR_INVALID_ARGUMENT;
    } catch (const std::exception& e) {
        lg << e.what() << "\n";
        g_err = e.what();
        rc = FT_ERR_RUNTIME;
    }
    if (log) *log = dup(lg.str());
    return rc;
}
