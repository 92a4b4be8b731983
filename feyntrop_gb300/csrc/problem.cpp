#include "problem.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <sstream>
#include <stdexcept>
#include <thread>

namespace ft {

// ------------------------------------------------------------------ glibc random(3)
// TYPE_3 additive-feedback generator of glibc's random(3) seeded with 1 (the state
// std::rand() starts in when srand was never called).  The reference draws its
// mass-momentum-spanning probe points from std::rand()
// (srcs/tropical_sampling.hpp:356 via Eigen's Random); reproducing the generator
// here keeps the probe points identical without touching the C library's state.
glibc_random::glibc_random()
{
    int32_t word = 1;
    t[0] = 1;
    for (int i = 1; i < 31; i++) {
        // 16807 * word mod (2^31 - 1) without overflow (Schrage)
        int32_t hi = word / 127773, lo = word % 127773;
        word = 16807 * lo - 2836 * hi;
        if (word < 0) word += 2147483647;
        t[i] = (uint32_t)word;
    }
    f = 3;
    b = 0;
    for (int i = 0; i < 310; i++) next();
}

int32_t glibc_random::next()
{
    t[f] += t[b];
    int32_t out = (int32_t)(t[f] >> 1);
    f = (f + 1) % 31;
    b = (b + 1) % 31;
    return out;
}

// ------------------------------------------------------------------ helpers
static std::string graph_string(const prepared& p)
{
    // srcs/graph.hpp:266-288
    std::stringstream os;
    os << "G(";
    for (int j = 0; j < p.E; j++) {
        double c = p.nu[j];
        if (std::fabs(std::nearbyint(c) / c - 1.0) < 1e-12)
            os << "[{" << p.ek[j] << "," << p.el[j] << "}," << std::lrint(c) << "]";
        else
            os << "[{" << p.ek[j] << "," << p.el[j] << "}," << c << "]";
        if (j != p.E - 1) os << ",";
    }
    os << ")";
    return os.str();
}

static std::string matrix_string(const std::vector<double>& M, int n)
{
    std::stringstream s;
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < n; j++) s << (j ? " " : "") << M[i * n + j];
        if (i + 1 < n) s << "\n";
    }
    return s.str();
}

std::vector<double> symmetric_eigenvalues(std::vector<double> A, int n)
{
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0;
        for (int i = 0; i < n; i++)
            for (int j = i + 1; j < n; j++) off += A[i * n + j] * A[i * n + j];
        if (off == 0.0) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                double apq = A[p * n + q];
                if (apq == 0.0) continue;
                double theta = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {
                    double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
            }
    }
    std::vector<double> ev(n);
    for (int i = 0; i < n; i++) ev[i] = A[i * n + i];
    return ev;
}

namespace {

struct structure {
    uint8_t cv, loops, mm, not_pseudo, not_generic;
};

struct builder {
    const prepared& p;
    bool phi_tr;
    double pmsqr_ref;
    std::vector<std::vector<double>> X, Xinv;   // probe points

    // components of the subgraph with edge mask `sub`, numbered by smallest vertex
    // (srcs/components.hpp:92-120)
    int components(uint64_t sub, int* cmap) const
    {
        int stack[64];
        for (int v = 0; v < p.V; v++) cmap[v] = -1;
        int C = 0;
        for (int v0 = 0; v0 < p.V; v0++) {
            if (cmap[v0] >= 0) continue;
            cmap[v0] = C;
            int top = 0;
            stack[top++] = v0;
            while (top) {
                int v = stack[--top];
                for (int e = 0; e < p.E; e++) {
                    if (!((sub >> e) & 1)) continue;
                    int w = p.ek[e] == v ? p.el[e] : (p.el[e] == v ? p.ek[e] : -1);
                    if (w >= 0 && cmap[w] < 0) {
                        cmap[w] = C;
                        stack[top++] = w;
                    }
                }
            }
            C++;
        }
        return C;
    }

    // srcs/laplacian.hpp:70-99
    void pgp(int C, const int* cmap, double* M) const
    {
        int n = C - 1;
        for (int i = 0; i < n * n; i++) M[i] = 0.0;
        for (int i = 0; i < p.V; i++)
            for (int j = 0; j < p.V; j++) {
                int a = cmap[i], b = cmap[j];
                if (a == C - 1 || b == C - 1) continue;
                M[a * n + b] += p.P[i * p.V + j];
            }
    }

    // srcs/tropical_sampling.hpp:46-82: |phi/psi + sum m^2 x| summed over probes,
    // with phi/psi = -trace(L^{-1} PGP) on the contracted graph, compared with
    // 1e-12 pmsqr_ref.  The terms are non-negative and rounded addition is monotone, so
    // once a partial sum reaches the threshold the full sum does too: the loop stops
    // there with the same answer (most subgraphs are decided by the first probe).
    bool mass_momentum_spanning(uint64_t sub, int C, const int* cmap, const double* PGP) const
    {
        const int n = C - 1;
        double L[64 * 64], D[64], col[64];
        double sum = 0.0;
        for (size_t t = 0; t < X.size(); t++) {
            std::fill(L, L + (size_t)n * n, 0.0);
            for (int j = 0; j < p.E; j++) {
                if ((sub >> j) & 1) continue;
                int k = cmap[p.ek[j]], l = cmap[p.el[j]];
                if (k == l) continue;
                if (k < l) std::swap(k, l);
                double x = Xinv[t][j];
                L[l * n + l] += x;
                if (k == C - 1) continue;
                L[k * n + k] += x;
                L[k * n + l] -= x;
            }
            // LDL^T of the (positive definite) lower triangle, in place
            for (int k = 0; k < n; k++) {
                double d = L[k * n + k];
                for (int j = 0; j < k; j++) d -= L[k * n + j] * L[k * n + j] * D[j];
                D[k] = d;
                for (int i = k + 1; i < n; i++) {
                    double s = L[i * n + k];
                    for (int j = 0; j < k; j++) s -= L[i * n + j] * D[j] * L[k * n + j];
                    L[i * n + k] = s / d;
                }
            }
            double tr = 0.0;
            for (int c = 0; c < n; c++) {
                for (int i = 0; i < n; i++) col[i] = PGP[i * n + c];
                for (int i = 0; i < n; i++)
                    for (int j = 0; j < i; j++) col[i] -= L[i * n + j] * col[j];
                for (int i = 0; i < n; i++) col[i] /= D[i];
                for (int i = n - 1; i >= 0; i--)
                    for (int j = i + 1; j < n; j++) col[i] -= L[j * n + i] * col[j];
                tr += col[c];
            }
            double pxi = -tr;
            for (int j = 0; j < p.E; j++)
                if (!((sub >> j) & 1)) pxi += p.m2[j] * X[t][j];
            sum += std::fabs(pxi);
            if (!(sum / pmsqr_ref < 1e-12)) return false;
        }
        return sum / pmsqr_ref < 1e-12;
    }

    // srcs/tropical_sampling.hpp:84-148
    bool generic_3_cut(uint64_t sub, const int* cmap, const double* PGP) const
    {
        bool zero = true;
        for (int i = 0; i < 4; i++) zero = zero && std::fabs(PGP[i]) <= 1e-12;
        if (zero) return true;
        double a = PGP[0], b = PGP[3], gamma = PGP[1];
        double c = a + b + 2 * gamma;
        double A = 0, B = 0, Cc = 0;
        for (int j = 0; j < p.E; j++) {
            if ((sub >> j) & 1) continue;
            int kc = cmap[p.ek[j]], lc = cmap[p.el[j]];
            if (kc == lc) continue;
            if (kc == 0 || lc == 0) A += p.m2[j];
            if (kc == 1 || lc == 1) B += p.m2[j];
            if (kc == 2 || lc == 2) Cc += p.m2[j];
        }
        const double thr = 1e-5;
        double da = std::fabs(a - A) / pmsqr_ref, db = std::fabs(b - B) / pmsqr_ref,
               dc = std::fabs(c - Cc) / pmsqr_ref;
        if (da > 1e-10 && db < thr && dc < thr) return false;
        if (db > 1e-10 && da < thr && dc < thr) return false;
        if (dc > 1e-10 && da < thr && db < thr) return false;
        return true;
    }

    structure analyse(uint64_t sub) const
    {
        int cmap[64];
        structure s{};
        int C = components(sub, cmap);
        int n = __builtin_popcountll(sub);
        s.cv = (uint8_t)C;
        s.loops = (uint8_t)(n - p.V + C);
        bool mm = false;
        if (phi_tr) {
            std::vector<double> M((size_t)(C - 1) * (C - 1) + 4);
            pgp(C, cmap, M.data());
            if (C == 2 && M[0] / pmsqr_ref >= 1e-12) s.not_pseudo = 1;
            if (C == 3 && !generic_3_cut(sub, cmap, M.data())) s.not_generic = 1;
            mm = mass_momentum_spanning(sub, C, cmap, M.data());
        } else if (n == p.E) {
            mm = true;
        }
        s.mm = mm;
        return s;
    }
};

uint64_t next_combination(uint64_t v)
{
    uint64_t t = v | (v - 1);
    return (t + 1) | (((~t & -~t) - 1) >> (__builtin_ctzll(v) + 1));
}

}  // namespace

prepared prepare(const problem_input& in, int threads)
{
    auto t0 = std::chrono::steady_clock::now();
    prepared p;
    const int E = (int)in.v.size();
    p.E = E;
    p.K = in.K;
    p.D = in.D;
    p.lambda_in = in.lambda;

    // srcs/graph.hpp:169-214
    int Vp = 0;
    for (int j = 0; j < E; j++) {
        int k = in.v[j], l = in.w[j];
        double c = in.nu[j];
        int hi = k, lo = l;
        if (k < l) std::swap(hi, lo);
        if (c <= 1e-12) throw std::invalid_argument("graph: edge weights must be larger than 0");
        if (k < 0 || l < 0) throw std::invalid_argument("graph: vertex numbers must start from 0");
        if (k == l)
            throw std::invalid_argument("graph: has a tadpole (selfloop) edge. This program cannot take care of this. ");
        p.ek.push_back(hi);
        p.el.push_back(lo);
        p.nu.push_back(c);
        Vp = std::max(Vp, std::max(k, l) + 1);
    }
    p.V = Vp;
    for (int v = 0; v < p.V; v++) {
        bool seen = false;
        for (int j = 0; j < E && !seen; j++) seen = p.ek[j] == v || p.el[j] == v;
        if (!seen) {
            std::stringstream s;
            s << "graph: the graph has a singleton vertex " << v;
            throw std::invalid_argument(s.str());
        }
    }
    const int V = p.V;
    if ((int)in.P.size() != V * V) throw std::invalid_argument("input scalarproducts must be a (V x V)-matrix");
    if ((int)in.m2.size() != E) throw std::invalid_argument("input masses_sqr must be an array of size E");
    p.P = in.P;
    p.m2 = in.m2;

    // srcs/feyntrop.cpp:98-112 (relative 1e-12 symmetry, absolute 1e-12 column sums)
    {
        double diff = 0, n1 = 0;
        for (int i = 0; i < V; i++)
            for (int j = 0; j < V; j++) {
                double d = p.P[i * V + j] - p.P[j * V + i];
                diff += d * d;
                n1 += p.P[i * V + j] * p.P[i * V + j];
            }
        if (diff > 1e-24 * n1) {
            std::stringstream s;
            s << "integrate_graph: The matrix \n" << matrix_string(p.P, V)
              << "\nof invariants was given as input and it is not symmetric or not a VxV matrix. One row and column "
                 "must be specified for each vertex - representing the momentum flowing into this vertex.";
            throw std::domain_error(s.str());
        }
        for (int j = 0; j < V; j++) {
            double s = 0;
            for (int i = 0; i < V; i++) s += p.P[i * V + j];
            if (std::fabs(s) > 1e-12) {
                std::stringstream m;
                m << "Scalar product (P) matrix has to fulfill momentum conservation. That means all row and column "
                     "sums need to be 0. The matrix \n"
                  << matrix_string(p.P, V) << "\ndoes not fulfill this requirement.";
                throw std::domain_error(m.str());
            }
        }
    }

    // srcs/feyntrop.cpp:128-133: Euclidean iff P == 0 or P is negative semidefinite
    {
        bool zero = true;
        double n2 = 0, pos2 = 0;
        for (double x : p.P) zero = zero && std::fabs(x) <= 1e-12;
        for (double ev : symmetric_eigenvalues(p.P, V)) {
            n2 += ev * ev;
            if (ev > 0) pos2 += 4 * ev * ev;
        }
        p.euclidean = zero || pos2 <= 1e-24 * n2;
    }

    // srcs/tropical_sampling.hpp:284-458
    if (E > 63) {
        std::stringstream s;
        s << "E = " << E << " this graph is too large for this implementation!";
        throw std::domain_error(s.str());
    }
    if (V > 32)
        throw std::runtime_error("Error: stacksize for BFS stack too small. Compile with larger MAX_BFS_STACKSIZE.");

    builder bld{p, false, 0.0, {}, {}};
    const uint64_t full = (1ULL << E) - 1;
    int cmap[64];
    int C = bld.components(full, cmap);
    p.loops = E - V + C;
    if (C != 1) {
        std::stringstream s;
        s << "Error: the graph " << graph_string(p) << " is not connected.";
        throw std::domain_error(s.str());
    }
    auto omega = [&](double D, int L, uint64_t sub) {
        double m = 0.0;
        for (int j = 0; j < E; j++)
            if ((sub >> j) & 1) m += p.nu[j];
        return m - D / 2.0 * L;
    };
    p.W = omega(p.D, p.loops, full);
    p.W_ref = omega(-p.D, p.loops, full);

    {
        int C0 = bld.components(0, cmap);
        std::vector<double> M((size_t)(C0 - 1) * (C0 - 1));
        bld.pgp(C0, cmap, M.data());
        double a = 0, b = 0;
        for (double x : M) a += x * x;
        for (double x : p.m2) b += x * x;
        bld.pmsqr_ref = std::sqrt(a) + std::sqrt(b);
    }
    const bool eps_expansion = p.K > 1;
    bld.phi_tr = eps_expansion || std::fabs(p.W / p.W_ref) > 1e-12;
    if (bld.phi_tr && std::fabs(bld.pmsqr_ref) < 1e-12) {
        std::stringstream s;
        s << "The graph " << graph_string(p) << " has superficial degree of divergence " << p.W
          << " and/or we need higher orders in epsilon. So, kinematics are necessary. The incoming momenta/masses "
             "appear to be too small to get an (numerically effective) non-zero F/Phi polynomial.";
        throw std::domain_error(s.str());
    }
    if (bld.phi_tr) {
        glibc_random rnd;
        for (int i = 0; i < 100; i++) {
            std::vector<double> x(E), xi(E);
            for (int j = 0; j < E; j++) {
                double u = -1.0 + (1.0 - -1.0) * double(rnd.next()) / double(2147483647);
                x[j] = 2.0 * 1.0 + u;
                xi[j] = 1.0 / x[j];
            }
            bld.X.push_back(x);
            bld.Xinv.push_back(xi);
        }
    }

    // pass 1: structural data of every subset, on all threads
    const size_t size = 1ULL << E;
    std::vector<structure> st(size);
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    // at least 1024 subsets per thread: below that, starting threads costs more than it saves
    threads = (int)std::max<size_t>(1, std::min<size_t>((size_t)threads, size / 1024));
    {
        std::atomic<size_t> next{0};
        std::exception_ptr err;
        auto work = [&]() {
            try {
                while (true) {
                    size_t lo = next.fetch_add(64);
                    if (lo >= size) break;
                    size_t hi = std::min(size, lo + 64);
                    for (size_t s = lo; s < hi; s++) st[s] = bld.analyse(s);
                }
            } catch (...) {
                err = std::current_exception();
            }
        };
        std::vector<std::thread> pool;
        for (int t = 1; t < threads; t++) pool.emplace_back(work);
        work();
        for (auto& th : pool) th.join();
        if (err) std::rethrow_exception(err);
    }

    // pass 2: Jr sums, subdivergence and GP checks in the reference's subset order
    p.Jr.assign(size, 0.0);
    p.r.assign(size, 0.0);
    p.mm.assign(size, 0);
    p.L.assign(size, 0);
    for (size_t s = 0; s < size; s++) {
        if (st[s].not_pseudo) p.pseudo_euclidean = false;
        if (st[s].not_generic) p.generic = false;
        p.mm[s] = st[s].mm;
        p.L[s] = st[s].loops;
    }
    const bool check_gp = bld.phi_tr && !p.euclidean;
    for (int n = 0; n <= E; n++) {
        uint64_t sub = (n == 0) ? 0 : ((1ULL << n) - 1);
        while (true) {
            double Jr, r;
            if (n == 0) {
                Jr = 1.0;
                r = 1.0;
            } else {
                Jr = 0.0;
                for (int j = 0; j < E; j++)
                    if ((sub >> j) & 1) {
                        uint64_t c = sub & ~(1ULL << j);
                        Jr += p.Jr[c] / p.r[c];
                    }
                r = omega(p.D, st[sub].loops, sub);
                if (st[sub].mm) r -= p.W;
            }
            if (r / p.W_ref < 1e-12 && n != E) {
                std::stringstream s;
                s << "Error: the graph " << graph_string(p) << " has a UV or IR subdivergence. \nE.g. the subgraph with "
                  << "edge numbers { ";
                for (int j = 0; j < E; j++)
                    if ((sub >> j) & 1) s << j << " ";
                s << "} or, explicitly, with the edges { ";
                for (int j = 0; j < E; j++)
                    if ((sub >> j) & 1) s << "[" << p.ek[j] << "," << p.el[j] << "] ";
                s << "}";
                s << " has an (effective) superficial degree of divergence of " << r << ".";
                throw std::domain_error(s.str());
            }
            if (check_gp && n >= 2 && p.gp) {
                // srcs/tropical_sampling.hpp:152-228
                int z = st[sub].mm ? st[sub].loops + 1 : st[sub].loops;
                auto zof = [&](uint64_t g) { return st[g].mm ? st[g].loops + 1 : st[g].loops; };
                for (int a = 0; a < E && p.gp; a++) {
                    if (!((sub >> a) & 1)) continue;
                    uint64_t A = sub & ~(1ULL << a);
                    int zA = zof(A);
                    for (int b = a + 1; b < E; b++) {
                        if (!((sub >> b) & 1)) continue;
                        if (zA + zof(sub & ~(1ULL << b)) > z + zof(A & ~(1ULL << b))) {
                            p.gp = false;
                            break;
                        }
                    }
                }
            }
            p.Jr[sub] = Jr;
            p.r[sub] = r;
            if (n == 0 || n == E) break;
            sub = next_combination(sub);
            if (sub >> E) break;
        }
    }
    p.IGtr = p.Jr[full];

    // srcs/feyntrop.cpp:165-239
    {
        std::string regime = p.euclidean ? "Euclidean" : (p.pseudo_euclidean ? "Pseudo-Euclidean" : "Minkowski");
        p.log.push_back("(Effective) kinematic regime: " + regime + (p.generic ? " (generic)." : " (exceptional)."));
    }
    auto gp_error = [&](const char* head) {
        std::stringstream s;
        s << head
          << " This is likely a bug and the result of the integration shouldn't be trusted. Please contact the "
             "developers and send them the following data such that they can fix this bug. Thank you!\n"
          << graph_string(p) << "\n";
        for (double m : p.m2) s << m << "\n";
        s << matrix_string(p.P, V) << "\n";
        throw std::domain_error(s.str());
    };
    if (p.generic && !p.gp)
        gp_error("The momenta seem generic, but the generalized permutahedron property is not fulfilled.");
    if (p.euclidean && !p.gp)
        gp_error("The momenta seem Euclidean, but the generalized permutahedron property is not fulfilled.");
    if (!p.generic && !p.euclidean && p.W > 0) {
        p.log.push_back(
            "Warning: Kinematics are non-Euclidean and (very) exceptional. Detailed info on the N[F] polytope is "
            "needed. The integration might fail or be unstable. Check the result by 1) varying the number of sample "
            "points 2) evaluating at multiple kinematic points close to the current one (i.e. by making the "
            "kinematics more generic) 3) increasing the spacetime dimension D0.");
        p.log.push_back(p.gp ? "The generalized permutahedron property seems fulfilled. This is a good sign that the "
                               "integration might succeed anyway."
                             : "The generalized permutahedron property does NOT seem fulfilled. Likely, there are "
                               "singular points in the integration domain that impeed convergence.");
    } else if (p.gp) {
        p.log.push_back("Generalized permutahedron property seems fulfilled.");
    } else if (p.W > 0) {
        gp_error("The momenta seem Euclidean or generic, but the generalized permutahedron property seems not "
                 "fulfilled.");
    } else {
        p.log.push_back("Generalized permutahedron property seems NOT fulfilled. However, the integration should work "
                        "fine as the N[F] polytope is not relevant for the given dimension and edge weights.");
    }
    p.lambda = 0.0;
    if (!p.pseudo_euclidean) {
        std::stringstream s;
        s << "Analytic continuation: activated. Lambda = " << in.lambda << ".";
        p.log.push_back(s.str());
        p.lambda = in.lambda;
    }
    // srcs/feynman_integral.hpp:60-140
    p.W_zero = std::fabs(p.W / p.W_ref) < 1e-12;
    p.def_ref = (p.lambda != 0 && !(p.W_zero && p.K == 1)) ? -p.lambda : 0.0;
    p.seconds_preprocessing =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return p;
}

}  // namespace ft
