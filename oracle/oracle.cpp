// ORACLE — test infrastructure only (see oracle.hpp for what it restates and how
// it is pinned).  Plain C++17, no third-party code; each block cites the reference
// lines it follows.
#include "oracle.hpp"
#include "opcount.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <sstream>
#include <stdexcept>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace fto {

using cd = std::complex<double>;

// complex companion of a real type: std::complex<double> for double, cx for the
// operation-counting scalar
template <class Real> struct cplx_of { using type = std::complex<Real>; };
template <> struct cplx_of<cnt> { using type = cx; };
template <class Real> using cplx_t = typename cplx_of<Real>::type;

// the sampling templates call these unqualified, so that the counting scalar's
// overloads are found beside the standard ones
using std::abs;
using std::arg;
using std::cos;
using std::exp;
using std::fabs;
using std::isfinite;
using std::log;
using std::polar;
using std::pow;
using std::sin;

op_counts& ops()
{
    static thread_local op_counts c;
    return c;
}

// ---------------------------------------------------------------- random streams
// srcs/random.hpp:32-66 (splitmix64 seeding) and :124-139 (xoshiro256+ step)
static uint64_t splitmix_next(uint64_t& x)
{
    uint64_t z = (x += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

xoshiro::xoshiro(uint64_t seed)
{
    uint64_t x = seed;
    for (int i = 0; i < 4; i++) s[i] = splitmix_next(x);
}

static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

uint64_t xoshiro::next()
{
    const uint64_t out = s[0] + s[3];
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return out;
}

// The state update is linear over GF(2); a 256x256 bit matrix (column c = image of
// basis vector c) raised to a power advances a stream by that many steps.
using bitvec = std::array<uint64_t, 4>;
using bitmat = std::vector<bitvec>;  // 256 columns

static bitvec mat_apply(const bitmat& M, const bitvec& v)
{
    bitvec r{0, 0, 0, 0};
    for (int i = 0; i < 256; i++)
        if ((v[i >> 6] >> (i & 63)) & 1)
            for (int w = 0; w < 4; w++) r[w] ^= M[i][w];
    return r;
}

static bitmat mul(const bitmat& A, const bitmat& B)
{
    bitmat C(256);
    for (int c = 0; c < 256; c++) C[c] = mat_apply(A, B[c]);
    return C;
}

// T^(2^b), b = 0..63, built once
static const std::vector<bitmat>& powers()
{
    static const std::vector<bitmat> P = [] {
        std::vector<bitmat> v(64);
        bitmat T(256);
        for (int c = 0; c < 256; c++) {
            xoshiro x(0);
            for (int w = 0; w < 4; w++) x.s[w] = 0;
            x.s[c >> 6] = 1ULL << (c & 63);
            x.next();
            for (int w = 0; w < 4; w++) T[c][w] = x.s[w];
        }
        v[0] = T;
        for (int b = 1; b < 64; b++) v[b] = mul(v[b - 1], v[b - 1]);
        return v;
    }();
    return P;
}

void skip(xoshiro& g, uint64_t steps)
{
    const std::vector<bitmat>& P = powers();
    bitvec v{g.s[0], g.s[1], g.s[2], g.s[3]};
    for (int b = 0; b < 64; b++)
        if ((steps >> b) & 1) v = mat_apply(P[b], v);
    for (int w = 0; w < 4; w++) g.s[w] = v[w];
}

// ---------------------------------------------------------------- graph helpers
static int popcount64(uint64_t v) { return __builtin_popcountll(v); }

// srcs/components.hpp:92-120: components numbered in order of their smallest vertex
static int components(const problem& p, uint64_t sub, std::vector<int>& cmap)
{
    if (p.V > 32)
        throw std::runtime_error("Error: stacksize for BFS stack too small. Compile with larger MAX_BFS_STACKSIZE.");
    cmap.assign(p.V, -1);
    int C = 0;
    std::vector<int> stack;
    for (int v0 = 0; v0 < p.V; v0++) {
        if (cmap[v0] >= 0) continue;
        cmap[v0] = C;
        stack.assign(1, v0);
        while (!stack.empty()) {
            int v = stack.back();
            stack.pop_back();
            for (int e = 0; e < p.E; e++) {
                if (!((sub >> e) & 1)) continue;
                int w = p.k[e] == v ? p.l[e] : (p.l[e] == v ? p.k[e] : -1);
                if (w >= 0 && cmap[w] < 0) {
                    cmap[w] = C;
                    stack.push_back(w);
                }
            }
        }
        C++;
    }
    return C;
}

// srcs/tropical_sampling.hpp:26-44
static double omega(const problem& p, double D, int L, uint64_t sub)
{
    double m = 0.0;
    for (int j = 0; j < p.E; j++)
        if ((sub >> j) & 1) m += p.nu[j];
    return m - D / 2.0 * L;
}

// srcs/laplacian.hpp:70-99 (n x n, n = C-1, row major)
template <class Real = double>
static std::vector<Real> pgp_matrix(const problem& p, int C, const std::vector<int>& cmap)
{
    int n = C - 1;
    std::vector<Real> M((size_t)n * n, Real(0.0));
    for (int i = 0; i < p.V; i++)
        for (int j = 0; j < p.V; j++) {
            int v = cmap[i], w = cmap[j];
            if (v == C - 1 || w == C - 1) continue;
            M[v * n + w] += p.P[i * p.V + j];
        }
    return M;
}

// srcs/laplacian.hpp:14-67 (lower triangle only; edges in `contracted` skipped)
template <class F>
static std::vector<F> reduced_laplacian(const problem& p, uint64_t contracted, int C,
                                        const std::vector<int>& cmap, const std::vector<F>& xinv)
{
    int n = C - 1;
    std::vector<F> La((size_t)n * n, F(0));
    for (int j = 0; j < p.E; j++) {
        if ((contracted >> j) & 1) continue;
        int k = cmap[p.k[j]], l = cmap[p.l[j]];
        if (k == l) continue;
        if (k < l) std::swap(k, l);
        F x = xinv[j];
        La[l * n + l] += x;
        if (k == C - 1) continue;
        La[k * n + k] += x;
        La[k * n + l] += -x;
    }
    return La;
}

// ---------------------------------------------------------------- dense factorisations
// LDL^T with symmetric pivoting; the pivot order is the one a left-looking LDLT
// that picks the largest remaining *original* diagonal entry produces (the rule
// of the library used at srcs/feynman_integral.hpp:216).  Reads the lower triangle.
template <class Real>
struct ldlt_t {
    int n = 0;
    std::vector<int> perm;        // position -> original index
    std::vector<Real> L, D;       // unit lower factor (row major), diagonal
    std::vector<Real> diag, y, col;

    ldlt_t() = default;
    ldlt_t(const std::vector<Real>& A, int n_) { compute(A, n_); }

    void compute(const std::vector<Real>& A, int n_)
    {
        n = n_;
        perm.resize(n);
        diag.resize(n);
        for (int i = 0; i < n; i++) perm[i] = i;
        for (int i = 0; i < n; i++) diag[i] = A[i * n + i];
        for (int k = 0; k < n; k++) {
            int best = k;
            for (int i = k + 1; i < n; i++)
                if (fabs(diag[i]) > fabs(diag[best])) best = i;
            std::swap(diag[k], diag[best]);
            std::swap(perm[k], perm[best]);
        }
        auto a = [&](int i, int j) {  // symmetric access of the permuted matrix
            int pi = perm[i], pj = perm[j];
            return pi >= pj ? A[pi * n + pj] : A[pj * n + pi];
        };
        L.assign((size_t)n * n, Real(0.0));
        D.assign(n, Real(0.0));
        for (int k = 0; k < n; k++) {
            Real d = a(k, k);
            for (int j = 0; j < k; j++) d -= L[k * n + j] * L[k * n + j] * D[j];
            D[k] = d;
            L[k * n + k] = 1.0;
            for (int i = k + 1; i < n; i++) {
                Real s = a(i, k);
                for (int j = 0; j < k; j++) s -= L[i * n + j] * D[j] * L[k * n + j];
                L[i * n + k] = (d != 0.0) ? s / d : Real(0.0);
            }
        }
    }

    // x = A^{-1} b (x and b may not alias)
    void solve_into(const Real* b, Real* x)
    {
        y.resize(n);
        for (int i = 0; i < n; i++) y[i] = b[perm[i]];
        for (int i = 0; i < n; i++)
            for (int j = 0; j < i; j++) y[i] -= L[i * n + j] * y[j];
        for (int i = 0; i < n; i++)
            y[i] = fabs(D[i]) > std::numeric_limits<double>::min() ? y[i] / D[i] : Real(0.0);
        for (int i = n - 1; i >= 0; i--)
            for (int j = i + 1; j < n; j++) y[i] -= L[j * n + i] * y[j];
        for (int i = 0; i < n; i++) x[perm[i]] = y[i];
    }

    std::vector<Real> solve(const std::vector<Real>& b)
    {
        std::vector<Real> x(n);
        solve_into(b.data(), x.data());
        return x;
    }

    Real det() const
    {
        Real p = 1.0;
        for (const Real& d : D) p *= d;
        return p;
    }

    // trace(A^{-1} B), B row major n x n
    Real trace_solve(const std::vector<Real>& B)
    {
        Real t = 0.0;
        col.resize(2 * n);
        for (int j = 0; j < n; j++) {
            for (int i = 0; i < n; i++) col[i] = B[i * n + j];
            solve_into(col.data(), col.data() + n);
            t += col[n + j];
        }
        return t;
    }
};
using ldlt = ldlt_t<double>;

// LU with complete pivoting (largest modulus, first in column-major order), as used
// at srcs/feynman_integral.hpp:305.
template <class Real>
struct full_piv_lu_t {
    using C = cplx_t<Real>;
    int n = 0;
    std::vector<C> lu;
    std::vector<int> rowp, colp;   // transpositions
    int ntransp = 0;

    void compute(const std::vector<C>& A, int n_)
    {
        n = n_;
        lu = A;
        rowp.assign(n, 0);
        colp.assign(n, 0);
        ntransp = 0;
        for (int k = 0; k < n; k++) {
            int br = k, bc = k;
            Real best = -1.0;
            for (int c = k; c < n; c++)
                for (int r = k; r < n; r++) {
                    Real s = abs(lu[r * n + c]);
                    if (s > best) { best = s; br = r; bc = c; }
                }
            rowp[k] = br;
            colp[k] = bc;
            if (best == 0.0) {
                for (int i = k; i < n; i++) rowp[i] = colp[i] = i;
                break;
            }
            if (br != k) {
                for (int c = 0; c < n; c++) std::swap(lu[k * n + c], lu[br * n + c]);
                ntransp++;
            }
            if (bc != k) {
                for (int r = 0; r < n; r++) std::swap(lu[r * n + k], lu[r * n + bc]);
                ntransp++;
            }
            for (int r = k + 1; r < n; r++) lu[r * n + k] /= lu[k * n + k];
            for (int r = k + 1; r < n; r++)
                for (int c = k + 1; c < n; c++) lu[r * n + c] -= lu[r * n + k] * lu[k * n + c];
        }
    }

    C det() const
    {
        C p(1.0);
        for (int i = 0; i < n; i++) p *= lu[i * n + i];
        return (ntransp % 2) ? -p : p;
    }

    std::vector<C> solve(std::vector<C> b) const
    {
        for (int k = 0; k < n; k++) std::swap(b[k], b[rowp[k]]);
        for (int i = 0; i < n; i++)
            for (int j = 0; j < i; j++) b[i] -= lu[i * n + j] * b[j];
        for (int i = n - 1; i >= 0; i--) {
            for (int j = i + 1; j < n; j++) b[i] -= lu[i * n + j] * b[j];
            b[i] /= lu[i * n + i];
        }
        for (int k = n - 1; k >= 0; k--) std::swap(b[k], b[colp[k]]);
        return b;
    }
};

// LU with partial pivoting (largest modulus in the column, first wins), as used at
// srcs/feynman_integral.hpp:314-316; only the determinant is needed.
template <class Real>
static cplx_t<Real> partial_piv_det(std::vector<cplx_t<Real>>& lu, int n)
{
    using C = cplx_t<Real>;
    int ntransp = 0;
    for (int k = 0; k < n; k++) {
        int br = k;
        Real best = abs(lu[k * n + k]);
        for (int r = k + 1; r < n; r++) {
            Real s = abs(lu[r * n + k]);
            if (s > best) { best = s; br = r; }
        }
        if (best != 0.0) {
            if (br != k) {
                for (int c = 0; c < n; c++) std::swap(lu[k * n + c], lu[br * n + c]);
                ntransp++;
            }
            for (int r = k + 1; r < n; r++) lu[r * n + k] /= lu[k * n + k];
        }
        for (int r = k + 1; r < n; r++)
            for (int c = k + 1; c < n; c++) lu[r * n + c] -= lu[r * n + k] * lu[k * n + c];
    }
    C p(1.0);
    for (int i = 0; i < n; i++) p *= lu[i * n + i];
    return (ntransp % 2) ? -p : p;
}

// cyclic Jacobi eigenvalues of a symmetric matrix (for the regime decision)
static std::vector<double> sym_eigenvalues(std::vector<double> A, int n)
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

// ---------------------------------------------------------------- J(gamma) table
// srcs/tropical_sampling.hpp:46-82
static bool mass_momentum_spanning(const problem& p, uint64_t sub, const std::vector<double>& PGP,
                                   const std::vector<std::vector<double>>& Xs,
                                   const std::vector<std::vector<double>>& Xinvs,
                                   const std::vector<int>& cmap, int C, double pmsqr_ref)
{
    double sum = 0;
    for (size_t i = 0; i < Xs.size(); i++) {
        auto La = reduced_laplacian<double>(p, sub, C, cmap, Xinvs[i]);
        static thread_local ldlt f;
        f.compute(La, C - 1);
        double pxi = -f.trace_solve(PGP);
        for (int j = 0; j < p.E; j++)
            if (!((sub >> j) & 1)) pxi += p.m2[j] * Xs[i][j];
        sum += std::fabs(pxi);
    }
    return sum / pmsqr_ref < 1e-12;
}

// srcs/tropical_sampling.hpp:84-148
static bool kinematic_generic_3_cut(const problem& p, uint64_t sub, const std::vector<double>& PGP,
                                    const std::vector<int>& cmap, double pmsqr_ref, double thr)
{
    bool zero = true;
    for (double v : PGP) zero = zero && std::fabs(v) <= 1e-12;
    if (zero) return true;
    double a = PGP[0], b = PGP[3], gamma = PGP[1];
    double c = a + b + 2 * gamma;
    double A = 0, B = 0, Cc = 0;
    for (int j = 0; j < p.E; j++) {
        if ((sub >> j) & 1) continue;
        int kc = cmap[p.k[j]], lc = cmap[p.l[j]];
        if (kc == lc) continue;
        if (kc == 0 || lc == 0) A += p.m2[j];
        if (kc == 1 || lc == 1) B += p.m2[j];
        if (kc == 2 || lc == 2) Cc += p.m2[j];
    }
    double da = std::fabs(a - A) / pmsqr_ref, db = std::fabs(b - B) / pmsqr_ref, dc = std::fabs(c - Cc) / pmsqr_ref;
    if (da > 1e-10 && db < thr && dc < thr) return false;
    if (db > 1e-10 && da < thr && dc < thr) return false;
    if (dc > 1e-10 && da < thr && db < thr) return false;
    return true;
}

// srcs/tropical_sampling.hpp:152-228
static bool subgraph_gp_property(const problem& p, uint64_t sub, const prepared& pr, int L, bool mm)
{
    int z = mm ? L + 1 : L;
    for (int a = 0; a < p.E; a++) {
        if (!((sub >> a) & 1)) continue;
        uint64_t A = sub & ~(1ULL << a);
        int zA = pr.mm[A] ? pr.L[A] + 1 : pr.L[A];
        for (int b = a + 1; b < p.E; b++) {
            if (!((sub >> b) & 1)) continue;
            uint64_t AB = A & ~(1ULL << b), B = sub & ~(1ULL << b);
            int zB = pr.mm[B] ? pr.L[B] + 1 : pr.L[B];
            int zAB = pr.mm[AB] ? pr.L[AB] + 1 : pr.L[AB];
            if (zA + zB > z + zAB) return false;
        }
    }
    return true;
}

static uint64_t next_combination(uint64_t v)
{
    uint64_t t = v | (v - 1);
    return (t + 1) | (((~t & -~t) - 1) >> (__builtin_ctzll(v) + 1));
}

// srcs/graph.hpp:169-214 checks, srcs/feyntrop.cpp:98-119 checks,
// srcs/tropical_sampling.hpp:284-458 table, srcs/feyntrop.cpp:128-239 decisions
prepared prepare(const problem& in)
{
    prepared pr;
    problem& p = pr.p;
    p = in;
    int Vmax = 0;
    for (int j = 0; j < p.E; j++) {
        int k = p.k[j], l = p.l[j];
        if (k < l) std::swap(p.k[j], p.l[j]);
        if (p.nu[j] <= 1e-12) throw std::invalid_argument("graph: edge weights must be larger than 0");
        if (k < 0 || l < 0) throw std::invalid_argument("graph: vertex numbers must start from 0");
        if (k == l)
            throw std::invalid_argument("graph: has a tadpole (selfloop) edge. This program cannot take care of this. ");
        Vmax = std::max(Vmax, std::max(k, l) + 1);
    }
    if (p.V != Vmax) throw std::invalid_argument("oracle: V does not match the edge list");
    for (int v = 0; v < p.V; v++) {
        bool seen = false;
        for (int j = 0; j < p.E; j++) seen = seen || p.k[j] == v || p.l[j] == v;
        if (!seen) {
            std::stringstream s;
            s << "graph: the graph has a singleton vertex " << v;
            throw std::invalid_argument(s.str());
        }
    }
    const int E = p.E, V = p.V;
    // symmetry and momentum conservation (relative / absolute 1e-12)
    {
        double diff = 0, nrm = 0;
        for (int i = 0; i < V; i++)
            for (int j = 0; j < V; j++) {
                double d = p.P[i * V + j] - p.P[j * V + i];
                diff += d * d;
                nrm += p.P[i * V + j] * p.P[i * V + j];
            }
        if (diff > 1e-24 * nrm) throw std::domain_error("integrate_graph: The matrix of invariants is not symmetric");
        for (int j = 0; j < V; j++) {
            double s = 0;
            for (int i = 0; i < V; i++) s += p.P[i * V + j];
            if (std::fabs(s) > 1e-12)
                throw std::domain_error("Scalar product (P) matrix has to fulfill momentum conservation.");
        }
    }
    // Euclidean iff P == 0 or P is negative semidefinite (srcs/feyntrop.cpp:128-133)
    {
        bool zero = true;
        double n2 = 0, pos2 = 0;
        for (double v : p.P) zero = zero && std::fabs(v) <= 1e-12;
        for (double ev : sym_eigenvalues(p.P, V)) {
            n2 += ev * ev;
            if (ev > 0) pos2 += 4 * ev * ev;
        }
        pr.euclidean = zero || pos2 <= 1e-24 * n2;
    }
    if (E > 63) {
        std::stringstream s;
        s << "E = " << E << " this graph is too large for this implementation!";
        throw std::domain_error(s.str());
    }
    const bool eps_expansion = p.K > 1, non_euclidean = !pr.euclidean;
    const uint64_t full = (E == 64) ? ~0ULL : ((1ULL << E) - 1);
    std::vector<int> cmap;
    int C = components(p, full, cmap);
    int L = E - V + C;
    if (C != 1) throw std::domain_error("Error: the graph is not connected.");
    pr.loops = L;
    pr.W = omega(p, p.D, L, full);
    pr.W_ref = omega(p, -p.D, L, full);
    const double W = pr.W, W_ref = pr.W_ref;

    int cV = components(p, 0, cmap);
    std::vector<double> PGP = pgp_matrix(p, cV, cmap);
    double pgp_norm = 0, m_norm = 0;
    for (double v : PGP) pgp_norm += v * v;
    for (double v : p.m2) m_norm += v * v;
    const double pmsqr_ref = std::sqrt(pgp_norm) + std::sqrt(m_norm);
    const bool phi_tr = eps_expansion || std::fabs(W / W_ref) > 1e-12;
    if (phi_tr && std::fabs(pmsqr_ref) < 1e-12)
        throw std::domain_error("The graph has superficial degree of divergence and/or we need higher orders in "
                                "epsilon. So, kinematics are necessary.");

    // probe points: the reference draws 2 + U[-1,1] from std::rand() with its
    // default seed; reproduced here so the probes are the same numbers
    std::vector<std::vector<double>> Xs, Xinvs;
    if (phi_tr) {
        std::srand(1);
        for (int i = 0; i < 100; i++) {
            std::vector<double> x(E), xi(E);
            for (int j = 0; j < E; j++) {
                double rnd = -1.0 + (1.0 - -1.0) * double(std::rand()) / double(RAND_MAX);
                x[j] = 2.0 * 1.0 + rnd;
                xi[j] = 1.0 / x[j];
            }
            Xs.push_back(x);
            Xinvs.push_back(xi);
        }
    }

    const size_t size = 1ULL << E;
    pr.Jr.assign(size, 0.0);
    pr.r.assign(size, 0.0);
    pr.mm.assign(size, 0);
    pr.L.assign(size, 0);
    const double generic_threshold = 1e-5;

    for (int n = 0; n <= E; n++) {
        uint64_t sub = (n == 0) ? 0 : ((n == 64) ? ~0ULL : ((1ULL << n) - 1));
        while (true) {
            int cv = components(p, sub, cmap);
            bool mm = false;
            if (phi_tr) {
                PGP = pgp_matrix(p, cv, cmap);
                if (cv == 2 && PGP[0] / pmsqr_ref >= 1e-12) pr.pseudo_euclidean = false;
                if (cv == 3)
                    pr.generic = pr.generic && kinematic_generic_3_cut(p, sub, PGP, cmap, pmsqr_ref, generic_threshold);
                mm = mass_momentum_spanning(p, sub, PGP, Xs, Xinvs, cmap, cv, pmsqr_ref);
            } else if (n == E) {
                mm = true;
            }
            int Ls = n - V + cv;
            double Jr, r;
            if (n == 0) {
                Jr = 1.0;
                r = 1.0;
            } else {
                Jr = 0.0;
                for (int j = 0; j < E; j++)
                    if ((sub >> j) & 1) {
                        uint64_t c = sub & ~(1ULL << j);
                        Jr += pr.Jr[c] / pr.r[c];
                    }
                r = omega(p, p.D, Ls, sub);
                if (mm) r -= W;
            }
            if (r / W_ref < 1e-12 && n != E) {
                std::stringstream s;
                s << "Error: the graph has a UV or IR subdivergence. E.g. the subgraph with edge numbers { ";
                for (int j = 0; j < E; j++)
                    if ((sub >> j) & 1) s << j << " ";
                s << "} has an (effective) superficial degree of divergence of " << r << ".";
                throw std::domain_error(s.str());
            }
            if (phi_tr && non_euclidean && n >= 2)
                pr.gp = pr.gp && subgraph_gp_property(p, sub, pr, Ls, mm);
            pr.Jr[sub] = Jr;
            pr.r[sub] = r;
            pr.mm[sub] = mm;
            pr.L[sub] = (uint8_t)Ls;
            if (n == 0 || n == E) break;
            sub = next_combination(sub);
            if (sub >> E) break;
        }
    }
    pr.IGtr = pr.Jr[full];

    // srcs/feyntrop.cpp:182-239
    if (pr.generic && !pr.gp)
        throw std::domain_error("The momenta seem generic, but the generalized permutahedron property is not fulfilled.");
    if (pr.euclidean && !pr.gp)
        throw std::domain_error("The momenta seem Euclidean, but the generalized permutahedron property is not fulfilled.");
    if (!(!pr.generic && !pr.euclidean && W > 0) && !pr.gp && W > 0)
        throw std::domain_error("The momenta seem Euclidean or generic, but the generalized permutahedron property seems not fulfilled.");
    double lambda = pr.pseudo_euclidean ? 0.0 : p.lambda;

    // srcs/feynman_integral.hpp:51-140
    pr.W_zero = std::fabs(W / W_ref) < 1e-12;
    pr.def_ref = (lambda != 0 && !(pr.W_zero && p.K == 1)) ? -lambda : 0.0;
    return pr;
}

// ---------------------------------------------------------------- sector draw
// srcs/tropical_sampling.hpp:468-564
template <class Real>
static sector draw_sector_t(const prepared& pr, xoshiro& g)
{
    const int E = pr.p.E;
    sector s;
    s.X.assign(E, 0.0);
    uint64_t sub = (1ULL << E) - 1;
    Real JJr = pr.Jr[sub];
    bool MM = pr.mm[sub];
    int oL = pr.L[sub];
    Real G = 0.0, F = 1.0, XX = 1.0;
    for (int j = 0;; j++) {
        // get_random_cut: first edge (ascending) whose running sum exceeds u*JJr,
        // else the last edge visited
        const Real u = Real((double)(g.next() >> 11)) * (1.0 / 9007199254740992.0);
        Real R = u * JJr;
        Real T = 0.0;
        int e = -1;
        for (int c = 0; c < E; c++) {
            if (!((sub >> c) & 1)) continue;
            uint64_t t = sub & ~(1ULL << c);
            T += Real(pr.Jr[t]) / pr.r[t];
            e = c;
            if (T > R) break;
        }
        sub &= ~(1ULL << e);
        JJr = pr.Jr[sub];
        Real r = pr.r[sub];
        bool mm = pr.mm[sub];
        int L = pr.L[sub];
        s.order.push_back(e);
        if (MM && !mm) G = XX;
        MM = mm;
        s.X[e] = (double)XX;
        if (L < oL) {
            F *= XX;
            oL = L;
        }
        if (j >= E - 1) break;
        const Real U = Real((double)(g.next() >> 11)) * (1.0 / 9007199254740992.0);
        XX *= pow(1. - U, 1. / r);
    }
    s.psi_tr = (double)F;
    s.xi_tr = (double)(G * F);
    return s;
}

sector draw_sector(const prepared& pr, xoshiro& g) { return draw_sector_t<double>(pr, g); }

// ---------------------------------------------------------------- integrand
// srcs/laplacian.hpp:102-215 for an empty contracted subgraph
template <class Real>
static void pphi_derivatives(const problem& p, int C, const std::vector<int>& cmap,
                             const std::vector<Real>& xinv, const std::vector<Real>& xinv2,
                             const std::vector<Real>& Ginv, const std::vector<Real>& M,
                             std::vector<Real>& d, std::vector<Real>& dd)
{
    const int E = p.E, n = C - 1;
    auto LP = [&](int i, int j) { return M[i * n + j]; };
    auto LI = [&](int i, int j) { return Ginv[i * n + j]; };
    for (int a = 0; a < E; a++) {
        int ka = cmap[p.k[a]], la = cmap[p.l[a]];
        if (la > ka) std::swap(la, ka);
        Real s, t;
        if (ka == C - 1) {
            s = LP(la, la);
            t = LI(la, la);
        } else {
            s = LP(ka, ka) + LP(la, la) - 2. * LP(ka, la);
            t = LI(ka, ka) + LI(la, la) - 2. * LI(ka, la);
        }
        Real xa = xinv2[a];
        Real xas = xa * s;
        d[a] = -xas;
        dd[a * E + a] = 2. * xas * (xinv[a] - xa * t);
        for (int b = a + 1; b < E; b++) {
            int kb = cmap[p.k[b]], lb = cmap[p.l[b]];
            if (lb > kb) std::swap(lb, kb);
            Real s2, t2;
            if (kb == C - 1) {
                if (ka == C - 1) {
                    s2 = LP(la, lb);
                    t2 = LI(la, lb);
                } else {
                    s2 = LP(la, lb) - LP(ka, lb);
                    t2 = LI(la, lb) - LI(ka, lb);
                }
            } else {
                if (ka == C - 1) {
                    s2 = LP(la, lb) - LP(la, kb);
                    t2 = LI(la, lb) - LI(la, kb);
                } else {
                    s2 = LP(ka, kb) + LP(la, lb) - LP(ka, lb) - LP(la, kb);
                    t2 = LI(ka, kb) + LI(la, lb) - LI(ka, lb) - LI(la, kb);
                }
            }
            Real xb = xinv2[b];
            dd[a * E + b] = dd[b * E + a] = -2. * xa * xb * s2 * t2;
        }
    }
}

template <class C>
static C cpow(const C& x, double y)
{
    // principal branch, as the standard complex power with a real exponent
    const auto lr = log(abs(x)), th = arg(x);
    return polar(exp(y * lr), y * th);
}

// srcs/feynman_integral.hpp:162-362.  Writes the K eps-order values into `out`;
// returns false when the sample is dropped.
template <class Real>
static bool evaluate_t(const prepared& pr, const sector& sec, std::vector<cplx_t<Real>>& out)
{
    using C = cplx_t<Real>;
    const problem& p = pr.p;
    const int E = p.E, V = p.V, n = V - 1, K = p.K;
    const double D = p.D, W = pr.W;
    const int L = pr.loops;
    out.assign(K, C(0.0));

    std::vector<Real> X(sec.X.begin(), sec.X.end());
    const Real psi_tr = sec.psi_tr, xi_tr = sec.xi_tr;

    // vertex with the smallest incident X becomes the deleted row/column
    std::vector<Real> XV(V, Real(0.0));
    for (int j = 0; j < E; j++) {
        XV[p.k[j]] += X[j];
        XV[p.l[j]] += X[j];
    }
    int minV = 0;
    for (int i = 1; i < V; i++)
        if (XV[minV] > XV[i]) minV = i;
    std::vector<int> cmap(V);
    for (int i = 0; i < V; i++) cmap[i] = i < minV ? i : (i > minV ? i - 1 : V - 1);

    // normalise so that psi_tr^(-D/2) (psi_tr/xi_tr)^W = 1
    Real tgt = pow(psi_tr, -D / 2.) * pow(psi_tr / xi_tr, W);
    Real scale = pow(tgt, 1. / (D / 2. * L + W));
    for (Real& x : X) x *= scale;
    std::vector<Real> Xinv(E);
    for (int j = 0; j < E; j++) Xinv[j] = 1.0 / X[j];

    auto La = reduced_laplacian<Real>(p, 0, V, cmap, Xinv);
    static thread_local ldlt_t<Real> f;
    f.compute(La, n);
    Real Xprod = 1.0;
    for (const Real& x : X) Xprod *= x;

    if (pr.def_ref == 0. || (pr.W_zero && K == 1)) {
        Real psi = f.det() * Xprod;
        Real R = pr.IGtr * pow(psi, -D / 2.);
        if (!isfinite(R)) return false;
        if (pr.W_zero && K == 1) {
            out[0] = C(R);
            return true;
        }
        auto PGP = pgp_matrix<Real>(p, V, cmap);
        Real pphi = -f.trace_solve(PGP);
        Real pxi = pphi;
        for (int j = 0; j < E; j++) pxi += p.m2[j] * X[j];
        R *= pow(pxi, -W);
        if (!isfinite(R)) return false;
        out[0] = C(R);
        if (K > 1) {
            Real eps_fac = log(psi) - L * log(pxi);
            for (int j = 1; j < K; j++) {
                R *= eps_fac / (double)j;
                out[j] = C(R);
            }
        }
        return true;
    }

    // deformed (Minkowski) branch
    auto PGP = pgp_matrix<Real>(p, V, cmap);
    static thread_local std::vector<Real> Ginv;
    Ginv.assign((size_t)n * n, Real(0.0));
    {
        static thread_local std::vector<Real> col;
        col.assign(2 * n, Real(0.0));
        for (int j = 0; j < n; j++) {
            for (int i = 0; i < n; i++) col[i] = (i == j) ? 1.0 : 0.0;
            f.solve_into(col.data(), col.data() + n);
            for (int i = 0; i < n; i++) Ginv[i * n + j] = col[n + i];
        }
    }
    static thread_local std::vector<Real> T1, M;
    T1.assign((size_t)n * n, Real(0.0));
    M.assign((size_t)n * n, Real(0.0));
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            Real s = 0;
            for (int k = 0; k < n; k++) s += Ginv[i * n + k] * PGP[k * n + j];
            T1[i * n + j] = s;
        }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            Real s = 0;
            for (int k = 0; k < n; k++) s += T1[i * n + k] * Ginv[j * n + k];
            M[i * n + j] = s;
        }
    static thread_local std::vector<Real> Xinv2;
    Xinv2.assign(E, Real(0.0));
    for (int j = 0; j < E; j++) Xinv2[j] = Xinv[j] * Xinv[j];
    static thread_local std::vector<Real> d, dd;
    d.assign(E, Real(0.0));
    dd.assign((size_t)E * E, Real(0.0));
    pphi_derivatives<Real>(p, V, cmap, Xinv, Xinv2, Ginv, M, d, dd);
    for (int j = 0; j < E; j++) d[j] = (d[j] + p.m2[j]) * pr.def_ref;

    static thread_local std::vector<C> cX, cXinv;
    cX.assign(E, C(0.0));
    cXinv.assign(E, C(0.0));
    for (int j = 0; j < E; j++) {
        cX[j] = X[j] * C(cos(d[j]), sin(d[j]));
        cXinv[j] = 1.0 / cX[j];
    }
    auto cLa = reduced_laplacian<C>(p, 0, V, cmap, cXinv);
    for (int k = 0; k < n; k++)
        for (int l = k + 1; l < n; l++) cLa[k * n + l] = cLa[l * n + k];
    static thread_local full_piv_lu_t<Real> lu;
    lu.compute(cLa, n);
    C cXprod(1.0);
    for (auto& c : cX) cXprod *= c;
    C cPsi = cXprod * lu.det();
    C cR = pr.IGtr * cpow(cPsi, -D / 2.);

    static thread_local std::vector<C> J;
    J.assign((size_t)E * E, C(0.0));
    for (int a = 0; a < E; a++)
        for (int b = 0; b < E; b++)
            J[a * E + b] = C(0., pr.def_ref) * dd[a * E + b] * X[b] + (a == b ? 1.0 : 0.0);
    C det_jac = partial_piv_det<Real>(J, E);
    Real x_nu = 0;
    for (int j = 0; j < E; j++) x_nu += p.nu[j] * d[j];
    cR *= det_jac * C(cos(x_nu), sin(x_nu));

    C tr(0.0);
    {
        std::vector<C> col(n);
        for (int j = 0; j < n; j++) {
            for (int i = 0; i < n; i++) col[i] = C(PGP[i * n + j]);
            tr += lu.solve(col)[j];
        }
    }
    C cPPhi = -tr;
    C cPXi = cPPhi;
    for (int j = 0; j < E; j++) cPXi += p.m2[j] * cX[j];
    cR *= cpow(cPXi, -W);
    if (!isfinite(cR.real()) || !isfinite(cR.imag())) return false;
    out[0] = cR;
    if (K > 1) {
        C eps_fac = log(cPsi) - (double)L * log(cPXi);
        for (int j = 1; j < K; j++) {
            cR *= eps_fac / (double)j;
            out[j] = cR;
        }
    }
    return true;
}

sample_value evaluate(const prepared& pr, const sector& sec)
{
    sample_value v;
    v.dropped = !evaluate_t<double>(pr, sec, v.R);
    if (v.dropped) v.R.assign(pr.p.K, cd(0, 0));
    return v;
}

// ---------------------------------------------------------------- statistics
// srcs/stats.hpp:13-134
struct summer {
    std::array<double, 64> s{};
    void add(double v)
    {
        if (v == 0.0) return;
        for (double& x : s) {
            if (x == 0.0) {
                x = v;
                return;
            }
            v += x;
            x = 0.0;
        }
        throw std::runtime_error("ERROR: More limbs needed for fp_summer");
    }
    double value() const
    {
        double v = 0.0;
        for (double x : s) v += x;
        return v;
    }
};

static summer merge(const summer& a, const summer& b)
{
    summer m;
    for (int i = 0; i < 63; i++) m.s[i + 1] = a.s[i] + b.s[i];
    m.s[0] = 0.0;
    return m;
}

struct stats {
    uint64_t N = 0;
    summer S1, S2;
    void update(double v)
    {
        N++;
        S1.add(v);
        S2.add(v * v);
    }
    double avg() const { return S1.value() / N; }
    double var() const { return ((double)N / ((double)N - 1)) * (S2.value() / N - std::pow(avg(), 2)); }
    double acc() const { return std::sqrt(var() / N); }
};

static stats merge(const stats& a, const stats& b)
{
    stats m;
    m.N = a.N + b.N;
    m.S1 = merge(a.S1, b.S1);
    m.S2 = merge(a.S2, b.S2);
    return m;
}

static stats merge_all(std::vector<stats> v)
{
    for (size_t e = 0; (1ULL << e) < v.size(); e++)
        for (size_t i = 0; i + (1ULL << e) < v.size(); i += 1ULL << (e + 1)) v[i] = merge(v[i], v[i + (1ULL << e)]);
    return v[0];
}

estimate integrate(const prepared& pr, uint64_t N, uint64_t seed, int threads)
{
    const int K = pr.p.K, E = pr.p.E;
    if (threads < 1) threads = 1;
    std::vector<std::vector<stats>> re(threads, std::vector<stats>(K)), im(threads, std::vector<stats>(K));
    std::vector<uint64_t> dropped(threads, 0);
    const bool real_only = !pr.deformed();
    powers();
    // chunks of the single stream; a chunk's first state is reached by skip-ahead,
    // so every sample is the one the single-threaded reference would draw
    const uint64_t chunk = 10000, nchunks = (N + chunk - 1) / chunk;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
    for (uint64_t c = 0; c < nchunks; c++) {
#ifdef _OPENMP
        const int t = omp_get_thread_num();
#else
        const int t = 0;
#endif
        const uint64_t lo = c * chunk, hi = std::min(N, lo + chunk);
        xoshiro g(seed);
        skip(g, lo * (uint64_t)(2 * E - 1));
        for (uint64_t i = lo; i < hi; i++) {
            sector s = draw_sector(pr, g);
            sample_value v = evaluate(pr, s);
            if (v.dropped) {
                dropped[t]++;
                continue;
            }
            if (real_only) {
                if (pr.W_zero && K == 1) {
                    re[t][0].update(v.R[0].real());
                } else {
                    for (int j = 0; j < K; j++) re[t][j].update(v.R[j].real());
                }
            } else {
                for (int j = 0; j < K; j++) {
                    re[t][j].update(v.R[j].real());
                    im[t][j].update(v.R[j].imag());
                }
            }
        }
    }
    if (real_only)
        for (int t = 0; t < threads; t++)
            for (int j = 0; j < K; j++) {
                im[t][j].update(0);
                im[t][j].update(0);
            }
    estimate est;
    for (int j = 0; j < K; j++) {
        std::vector<stats> rj, ij;
        for (int t = 0; t < threads; t++) {
            rj.push_back(re[t][j]);
            ij.push_back(im[t][j]);
        }
        stats R = merge_all(rj), I = merge_all(ij);
        est.re_avg.push_back(R.avg());
        est.re_acc.push_back(R.acc());
        est.im_avg.push_back(I.avg());
        est.im_acc.push_back(I.acc());
    }
    for (auto d : dropped) est.dropped += d;
    est.kept = N - est.dropped;
    return est;
}

}  // namespace fto

// ---------------------------------------------------------------- C interface (ctypes)
extern "C" {

static thread_local std::string g_err;

const char* fto_last_error() { return g_err.c_str(); }

// One opaque handle per prepared problem.
void* fto_prepare(int E, int V, const int* edges, const double* nu, const double* P, const double* m2, double D,
                  int K, double lambda)
{
    try {
        fto::problem p;
        p.E = E;
        p.V = V;
        for (int j = 0; j < E; j++) {
            p.k.push_back(edges[2 * j]);
            p.l.push_back(edges[2 * j + 1]);
            p.nu.push_back(nu[j]);
            p.m2.push_back(m2[j]);
        }
        p.P.assign(P, P + (size_t)V * V);
        p.D = D;
        p.K = K;
        p.lambda = lambda;
        return new fto::prepared(fto::prepare(p));
    } catch (std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

void fto_free(void* h) { delete (fto::prepared*)h; }

// info: W, W_ref, IGtr, loops, euclidean, pseudo_euclidean, generic, gp, W_zero, def_ref
void fto_info(void* h, double* out)
{
    auto* pr = (fto::prepared*)h;
    double v[10] = {pr->W, pr->W_ref, pr->IGtr, (double)pr->loops, (double)pr->euclidean,
                    (double)pr->pseudo_euclidean, (double)pr->generic, (double)pr->gp, (double)pr->W_zero,
                    pr->def_ref};
    std::memcpy(out, v, sizeof v);
}

void fto_table(void* h, double* Jr, double* r, uint8_t* mm, uint8_t* L)
{
    auto* pr = (fto::prepared*)h;
    size_t n = pr->Jr.size();
    std::memcpy(Jr, pr->Jr.data(), n * sizeof(double));
    std::memcpy(r, pr->r.data(), n * sizeof(double));
    std::memcpy(mm, pr->mm.data(), n);
    std::memcpy(L, pr->L.data(), n);
}

// Samples first..first+count-1 of the stream `seed`: removal order (count x E),
// raw X (count x E), psi_tr, xi_tr, and the integrand per eps order (count x K
// complex as re, im pairs) with a dropped flag.
int fto_samples(void* h, uint64_t seed, uint64_t first, uint64_t count, int32_t* order, double* X, double* psi_tr,
                double* xi_tr, double* R, uint8_t* dropped)
{
    try {
        auto* pr = (fto::prepared*)h;
        const int E = pr->p.E, K = pr->p.K;
        fto::xoshiro g(seed);
        fto::skip(g, first * (uint64_t)(2 * E - 1));
        for (uint64_t i = 0; i < count; i++) {
            fto::sector s = fto::draw_sector(*pr, g);
            fto::sample_value v = fto::evaluate(*pr, s);
            for (int e = 0; e < E; e++) {
                if (order) order[i * E + e] = s.order[e];
                if (X) X[i * E + e] = s.X[e];
            }
            if (psi_tr) psi_tr[i] = s.psi_tr;
            if (xi_tr) xi_tr[i] = s.xi_tr;
            for (int j = 0; j < K; j++) {
                if (R) {
                    R[(i * K + j) * 2] = v.R[j].real();
                    R[(i * K + j) * 2 + 1] = v.R[j].imag();
                }
            }
            if (dropped) dropped[i] = v.dropped;
        }
        return 0;
    } catch (std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

// out: K x 4 (re_avg, re_acc, im_avg, im_acc); counts: kept, dropped
int fto_integrate(void* h, uint64_t N, uint64_t seed, int threads, double* out, uint64_t* counts)
{
    try {
        auto* pr = (fto::prepared*)h;
        fto::estimate est = fto::integrate(*pr, N, seed, threads);
        for (int j = 0; j < pr->p.K; j++) {
            out[4 * j + 0] = est.re_avg[j];
            out[4 * j + 1] = est.re_acc[j];
            out[4 * j + 2] = est.im_avg[j];
            out[4 * j + 3] = est.im_acc[j];
        }
        if (counts) {
            counts[0] = est.kept;
            counts[1] = est.dropped;
        }
        return 0;
    } catch (std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

// Operation counts of samples first..first+count-1 of stream `seed`, run through the
// same restatement with the counting scalar.  out[7]: adds, muls, divs, sqrts,
// transcendentals, comparisons (summed over the samples) and the dropped count;
// R (optional, count x K complex) receives the counted run's values.
int fto_count_ops(void* h, uint64_t seed, uint64_t first, uint64_t count, double* out, double* R)
{
    try {
        auto* pr = (fto::prepared*)h;
        const int E = pr->p.E, K = pr->p.K;
        fto::xoshiro g(seed);
        fto::skip(g, first * (uint64_t)(2 * E - 1));
        fto::op_counts& c = fto::ops();
        c = fto::op_counts();
        double dropped = 0;
        std::vector<fto::cx> v;
        for (uint64_t i = 0; i < count; i++) {
            fto::sector s = fto::draw_sector_t<fto::cnt>(*pr, g);
            const bool kept = fto::evaluate_t<fto::cnt>(*pr, s, v);
            if (!kept) dropped++;
            for (int j = 0; j < K && R; j++) {
                R[(i * K + j) * 2] = kept ? v[j].re.v : 0.0;
                R[(i * K + j) * 2 + 1] = kept ? v[j].im.v : 0.0;
            }
        }
        const double o[7] = {c.add, c.mul, c.div, c.sqrt, c.trans, c.cmp, dropped};
        std::memcpy(out, o, sizeof o);
        return 0;
    } catch (std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

void fto_skip(uint64_t seed, uint64_t steps, uint64_t* state)
{
    fto::xoshiro g(seed);
    fto::skip(g, steps);
    for (int i = 0; i < 4; i++) state[i] = g.s[i];
}

}  // extern "C"
