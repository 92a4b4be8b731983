// Per-sample tropical Monte Carlo kernel body, compiled at run time for one graph
// topology (the host prepends the constants below and compiles with NVRTC for
// sm_103a, so every edge endpoint is a compile-time constant and all matrices live
// in registers).
//
// Required definitions:
//   FT_E, FT_V        edges, vertices            FT_K        eps orders
//   FT_LOOPS          loop number                FT_RANK     rank of the reduced P
//   FT_PREC           0: plain FP64, 1: mixed FP32 with FP64 sampling decisions
//   FT_MODE           0: undeformed integrand (srcs/feynman_integral.hpp:218-276)
//                     1: deformed integrand  (srcs/feynman_integral.hpp:278-362)
//   FT_ONLY_PSI       1 when W = 0 and one eps order (only psi is needed)
//   FT_RECORD         1: write per-sample records
//   FT_BLOCK          threads per block
//   FT_EK[], FT_EL[]  edge endpoints (FT_EK[e] > FT_EL[e])
//
// One thread owns one sample at a time and walks a contiguous block of samples of
// the seed's single xoshiro256+ stream, so the samples are exactly those of the
// reference run with one OpenMP thread (srcs/feynman_integral.hpp:144-164).
//
// Numerical design (the reference's algebra, restated for a GPU thread):
//  * Sector draw (srcs/tropical_sampling.hpp:468-564): the cut scan compares running
//    sums of Jr/r against u*Jr in FP64 in the reference's order, so the removal order
//    is bit-identical.  The mixed form decides each comparison in FP32 with a
//    rigorous error margin and repeats the scan in FP64 when a comparison falls
//    inside the margin.  The mixed form keeps log X in a two-float sum.
//  * The deleted vertex of the reduced Laplacian is always the last one of the
//    kernel's labels (the host numbers the vertices without external momentum first,
//    so it is an external one).  Any choice gives the same psi, phi/psi and
//    derivatives (matrix-tree theorem and momentum conservation); the reference's
//    choice only affects rounding.
//  * The real reduced Laplacian is eliminated in conductance form: pivots are sums
//    of positive conductances and updates add positive products, so psi = det L *
//    prod X has full relative accuracy whatever the spread of X.
//  * phi/psi = -tr(L^-1 P~) with P~ = sum_r sigma_r q_r q_r^T (host eigen-split):
//    each term is a forward substitution with the elimination multipliers.  The
//    mixed form's complex block instead contracts P~'s external block with L(y)^-1
//    directly, one quadratic form of P~ per row of the substitution's triangular map.
//  * Deformed branch: L^-1 from the positive factors, x-derivatives of phi/psi
//    (srcs/laplacian.hpp:102-215), the complex Laplacian eliminated in the same
//    conductance form with a pivot-growth check (the FP64 form's failing samples take
//    a complete-pivoting LU, srcs/feynman_integral.hpp:305; the mixed form runs this
//    elimination and V in two-float and hands the rare failing samples to FP64), and
//    the Jacobian determinant as det(I + i*lambda' X^1/2 H X^1/2) (similar to
//    I + i*lambda' H X, srcs/feynman_integral.hpp:312), whose real part is the
//    identity, so symmetric elimination without pivoting is stable.
//  * Updates on structural zeros of the eliminations (from each topology's fill
//    pattern, generated by the host) and additions to zero are left out.

#ifndef FT_E
#error "topology constants missing"
#endif
#ifndef FT_MINB
#define FT_MINB 1
#endif
// 1: the module holds the batch kernels (many integrals of this topology per launch)
#ifndef FT_BATCH
#define FT_BATCH 0
#endif

typedef unsigned long long u64;
typedef unsigned int u32;

// intermediate values for host-side numerical studies (compiled out on the device)
#ifndef FT_DBG
#define FT_DBG(slot, value)
#endif

// Code size: the per-topology kernel is straight-line code (every loop unrolled so
// that the small matrices stay in registers), and the FP32 library functions carry
// large slow paths.  FT_VARIANT bit 0 keeps one out-of-line copy of each FP32
// transcendental, bit 1 does the same for the two-float primitives, so the code the
// SM streams per sample fits the instruction caches better; bit 2 starts every sample
// with a block-wide barrier, so that the block's warps walk the code together and
// share its instruction fetches; bit 3 keeps one out-of-line copy of each larger
// two-float routine (logarithm, exponential, e^(ix), complex inverse, argument), bit 4
// of the complex two-float product and multiply-add.
#ifndef FT_VARIANT
#define FT_VARIANT 0
#endif
#if (FT_VARIANT & 1) && !defined(FT_HOST_SIM)
#define FT_MATHFN __noinline__
#else
#define FT_MATHFN __forceinline__
#endif
#if (FT_VARIANT & 2) && !defined(FT_HOST_SIM)
#define FT_DFFN __noinline__
#else
#define FT_DFFN __forceinline__
#endif
#if (FT_VARIANT & 8) && !defined(FT_HOST_SIM)
#define FT_BIGFN __noinline__
#else
#define FT_BIGFN __forceinline__
#endif
#if (FT_VARIANT & 16) && !defined(FT_HOST_SIM)
#define FT_CXFN __noinline__
#else
#define FT_CXFN __forceinline__
#endif
static __device__ FT_MATHFN float m_log1p(float x) { return log1pf(x); }
static __device__ FT_MATHFN float m_exp(float x) { return expf(x); }
static __device__ FT_MATHFN float m_exp2(float x) { return exp2f(x); }
static __device__ FT_MATHFN float m_log2(float x) { return log2f(x); }
static __device__ FT_MATHFN float m_atan2(float y, float x) { return atan2f(y, x); }
static __device__ FT_MATHFN float m_hypot(float x, float y) { return hypotf(x, y); }
static __device__ FT_MATHFN void m_sincos(float x, float* s, float* c) { sincosf(x, s, c); }
static __device__ FT_MATHFN float m_atan(float x) { return atanf(x); }

#define FT_N (FT_V - 1)
// reduced vertices [0, FT_Q0) carry no external momentum: the vectors q_r of P~ vanish
// there (the host labels the internal vertices first), so the forward substitutions
// of the quadratic forms start at row FT_Q0
#ifndef FT_Q0
#define FT_Q0 0
#endif
// Structural pattern of the eliminations, generated per topology: NZC(i, j) (i < j) a
// conductance between i and j that can be non-zero when i is eliminated (an edge or
// fill), NZG(i) a conductance to ground, NZM(i, j) an entry of M^-1 that can be
// non-zero.  Updates on structural zeros are left out (without the tables: dense).
#ifdef FT_HAVE_PATTERN
#define NZC(i, j) (FT_NZC[i][j] != 0)
#define NZG(i) (FT_NZG[i] != 0)
#define NZM(i, j) (FT_NZM[i][j] != 0)
#else
#define NZC(i, j) true
#define NZG(i) true
#define NZM(i, j) true
#endif
// edge e is the first to contribute to its conductance slot (the pair of endpoints, or
// the ground slot of its lower endpoint): its conductance is assigned, not added to zero
static __device__ constexpr bool first_in_slot(int e)
{
    for (int f = 0; f < e; f++)
        if (FT_EK[f] == FT_EK[e] && FT_EL[f] == FT_EL[e]) return false;
    return true;
}
#define FT_FULL ((1u << FT_E) - 1u)
#define FT_NPAIR (FT_E * (FT_E - 1) / 2)

// ------------------------------------------------------------------ parameter block
// doubles: 0 D, 1 W, 2 IGtr, 3 def_ref, 4 1/(D/2*L+W), 5 Jr(full), 6 unused, 7 unused,
// then m2[E], nu[E], sigma[RANK], q[RANK][N], then P~ on the external rows [Q0, N)
// (its upper triangle row by row, off-diagonal entries doubled)
#define P_D 0
#define P_W 1
#define P_IGTR 2
#define P_DEF 3
#define P_NORM 4
#define P_JRFULL 5
#define P_M2 8
#define P_NU (8 + FT_E)
#define P_SIG (8 + 2 * FT_E)
#define P_Q (8 + 2 * FT_E + FT_RANK)
#define FT_NE (FT_N - FT_Q0)
#define P_PT (8 + 2 * FT_E + FT_RANK + FT_RANK * FT_N)
#define P_SIZE (P_PT + FT_NE * (FT_NE + 1) / 2)
// entry (j, k), j <= k, of the external block of P~ (indices from Q0)
#define PT_AT(j, k) (P_PT + (j) * FT_NE - (j) * ((j) - 1) / 2 + ((k) - (j)))
// the same block as floats follows at prm + P_SIZE, then as two-float (hi, lo) pairs at
// prm + P_SIZE + (P_SIZE + 1) / 2 (the mixed form reads only those two)

// ------------------------------------------------------------------ table layout
// [w64 | Jr64 | rinv64 : 8 bytes each][meta : 1 byte][pad to 16][w32 | Jr32 : 4 bytes each]
// [rinv32 : (hi, lo) float pairs]
#define T_ENTRIES (1u << FT_E)
#define T_W64 0
#define T_JR64 (8u * T_ENTRIES)
#define T_RI64 (16u * T_ENTRIES)
#define T_META (24u * T_ENTRIES)
#define T_F32 ((25u * T_ENTRIES + 15u) & ~15u)
#define T_W32 (T_F32)
#define T_JR32 (T_F32 + 4u * T_ENTRIES)
#define T_RI32 (T_F32 + 8u * T_ENTRIES)   // (hi, lo) float pairs: 1/r in two-float

// ------------------------------------------------------------------ accumulator slots
// per eps order j: [8j + 0..7] = re S1 (hi, lo), re S2 (hi, lo), im S1 (hi, lo), im S2 (hi, lo)
// then [8K] kept, [8K+1] dropped, [8K+2] queued, [8K+3] exact sampling steps,
// [8K+4] robust factorisations
#define ACC_KEPT (8 * FT_K)
#define ACC_DROPPED (8 * FT_K + 1)
#define ACC_QUEUED (8 * FT_K + 2)
#define ACC_EXACT (8 * FT_K + 3)
#define ACC_ROBUST (8 * FT_K + 4)
#define ACC_SLOTS (8 * FT_K + 8)

// record flags
#define REC_DROPPED 1
#define REC_QUEUED 2
#define REC_EXACT 4
#define REC_ROBUST 8

// ------------------------------------------------------------------ small helpers
static __device__ __forceinline__ u64 rotl64(u64 x, int k) { return (x << k) | (x >> (64 - k)); }

struct xo {
    u64 a, b, c, d;
    __device__ __forceinline__ u64 next()
    {
        const u64 out = a + d;
        const u64 t = b << 17;
        c ^= a;
        d ^= b;
        b ^= c;
        a ^= d;
        c ^= t;
        d = rotl64(d, 45);
        return out;
    }
};

static __device__ __forceinline__ double u01(u64 x) { return (double)(x >> 11) * 0x1.0p-53; }

template <class T>
struct cx {
    T re, im;
};
template <class T>
static __device__ __forceinline__ cx<T> cmk(T r, T i)
{
    cx<T> z;
    z.re = r;
    z.im = i;
    return z;
}
template <class T>
static __device__ __forceinline__ cx<T> operator+(cx<T> a, cx<T> b) { return cmk(a.re + b.re, a.im + b.im); }
template <class T>
static __device__ __forceinline__ cx<T> operator-(cx<T> a, cx<T> b) { return cmk(a.re - b.re, a.im - b.im); }
template <class T>
static __device__ __forceinline__ cx<T> operator*(cx<T> a, cx<T> b)
{
    return cmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <class T>
static __device__ __forceinline__ cx<T> operator*(T s, cx<T> a) { return cmk(s * a.re, s * a.im); }
// reciprocals: IEEE division in FP64; the correctly rounded reciprocal instruction
// sequence in FP32 (a division there expands to a long inline sequence)
static __device__ __forceinline__ double rcp_(double x) { return 1.0 / x; }
#ifdef FT_HOST_SIM
static __device__ __forceinline__ float rcp_(float x) { return 1.0f / x; }
#else
static __device__ __forceinline__ float rcp_(float x) { return __frcp_rn(x); }
#endif
template <class T>
static __device__ __forceinline__ cx<T> crecip(cx<T> z)
{
    // scaled so that |z|^2 cannot overflow in single precision
    const T s = fmax(fabs(z.re), fabs(z.im));
    const T is = rcp_(s);
    const T r = z.re * is, i = z.im * is;
    const T id = rcp_(s * (r * r + i * i));
    return cmk(r * id, -i * id);
}
static __device__ __forceinline__ double cabs_(cx<double> z) { return hypot(z.re, z.im); }
// |z| for the pivots and determinants of the FP32 path (moduli far inside the
// float range there: conductances 1/x of a sector stay below ~1e18)
static __device__ __forceinline__ float cabs_(cx<float> z) { return sqrtf(fmaf(z.re, z.re, z.im * z.im)); }
static __device__ __forceinline__ bool cfinite(cx<double> z) { return isfinite(z.re) && isfinite(z.im); }
static __device__ __forceinline__ bool cfinite(cx<float> z) { return isfinite(z.re) && isfinite(z.im); }

// principal logarithm, exp, real power (the reference's std::log / std::pow on
// complex<double>, srcs/feynman_integral.hpp:310,327,354)
static __device__ __forceinline__ cx<double> clog_(cx<double> z) { return cmk(log(hypot(z.re, z.im)), atan2(z.im, z.re)); }
static __device__ __forceinline__ cx<double> cexp_(cx<double> z)
{
    double s, c, m = exp(z.re);
    sincos(z.im, &s, &c);
    return cmk(m * c, m * s);
}
static __device__ __forceinline__ cx<double> cpow_(cx<double> z, double y)
{
    double lr = log(hypot(z.re, z.im)), th = atan2(z.im, z.re);
    double s, c, m = exp(y * lr);
    sincos(y * th, &s, &c);
    return cmk(m * c, m * s);
}

// ------------------------------------------------------------------ conductance-form elimination
// Reduced Laplacian of the graph with conductances y_e, ground = vertex V-1.
// Fills the pivots d[k] and the elimination multipliers a[k][i] = c_ki / d_k
// (i > k), which define L = M^T diag(d) M with M unit upper triangular and
// M[k][i] = -a[k][i].  Returns the smallest pivot-to-row-size ratio (1 for
// positive conductances).
template <class F, class R>
struct elim {
    F d[FT_N];
    F a[FT_N][FT_N];   // a[k][i], i > k

    __device__ __forceinline__ R factor(const F* y)
    {
        F c[FT_N][FT_N];   // c[i][j], i < j < N: conductance between i and j
        F g[FT_N];         // conductance to ground
#pragma unroll
        for (int i = 0; i < FT_N; i++) {
            g[i] = F{};
#pragma unroll
            for (int j = 0; j < FT_N; j++) c[i][j] = F{};
        }
#pragma unroll
        for (int e = 0; e < FT_E; e++) {
            const int k = FT_EK[e], l = FT_EL[e];
            F& slot = (k == FT_V - 1) ? g[l] : c[l][k];
            slot = first_in_slot(e) ? y[e] : slot + y[e];
        }
        R worst = R(1);
#pragma unroll
        for (int k = 0; k < FT_N; k++) {
            F dk = g[k];
            R mag = mag_of(g[k]);
#pragma unroll
            for (int j = k + 1; j < FT_N; j++) {
                if (!NZC(k, j)) continue;
                dk = dk + c[k][j];
                mag += mag_of(c[k][j]);
            }
            d[k] = dk;
            R ratio = mag_of(dk) * rcp_(mag);
            worst = ratio < worst ? ratio : worst;
            F inv = inv_of(dk);
#pragma unroll
            for (int i = k + 1; i < FT_N; i++) a[k][i] = NZC(k, i) ? c[k][i] * inv : F{};
#pragma unroll
            for (int i = k + 1; i < FT_N; i++) {
                if (!NZC(k, i)) continue;
                if (NZG(k)) g[i] = g[i] + a[k][i] * g[k];
#pragma unroll
                for (int j = i + 1; j < FT_N; j++)
                    if (NZC(k, j)) c[i][j] = c[i][j] + a[k][i] * c[k][j];
            }
        }
        return worst;
    }

    // q^T L^{-1} q for a real vector q (forward substitution y = M^-T q, sum y^2/d;
    // y vanishes on the rows before FT_Q0, where q does)
    template <class Q>
    __device__ __forceinline__ F quad(const Q* q) const
    {
        F y[FT_N];
        F s = F{};
#pragma unroll
        for (int i = FT_Q0; i < FT_N; i++) {
            F yi = from_real((R)q[i]);
#pragma unroll
            for (int k = FT_Q0; k < i; k++)
                if (NZC(k, i)) yi = yi + a[k][i] * y[k];
            y[i] = yi;
            s = s + yi * yi * inv_of(d[i]);
        }
        return s;
    }

    // q^T L^{-1} q as quad(), adding sum_i |y_i|^2 / |d_i| (the magnitude of its terms) to mag
    template <class Q>
    __device__ __forceinline__ F quad_mag(const Q* q, R& mag) const
    {
        F y[FT_N];
        F s = F{};
#pragma unroll
        for (int i = FT_Q0; i < FT_N; i++) {
            F yi = from_real((R)q[i]);
#pragma unroll
            for (int k = FT_Q0; k < i; k++)
                if (NZC(k, i)) yi = yi + a[k][i] * y[k];
            y[i] = yi;
            const F t = yi * yi * inv_of(d[i]);
            s = s + t;
            mag += mag_of(t);
        }
        return s;
    }

    static __device__ __forceinline__ R mag_of(R x) { return fabs(x); }
    static __device__ __forceinline__ R mag_of(cx<R> x) { return fabs(x.re) + fabs(x.im); }
    static __device__ __forceinline__ R inv_of(R x) { return rcp_(x); }
    static __device__ __forceinline__ cx<R> inv_of(cx<R> x) { return crecip(x); }
    static __device__ __forceinline__ F from_real(R x)
    {
        F f{};
        set_real(f, x);
        return f;
    }
    static __device__ __forceinline__ void set_real(R& f, R x) { f = x; }
    static __device__ __forceinline__ void set_real(cx<R>& f, R x) { f = cmk(x, R(0)); }
};

// ------------------------------------------------------------------ robust complex LU
// Complete-pivoting LU of the complex reduced Laplacian (largest modulus, first in
// column-major order), used when the static elimination reports pivot growth.
// Returns det and -tr(L^-1 P~).
static __device__ void robust_complex(const cx<double>* y, const double* prm, cx<double>& det, cx<double>& pphi)
{
    cx<double> A[FT_N * FT_N];
    int rp[FT_N], cp[FT_N];
    for (int i = 0; i < FT_N * FT_N; i++) A[i] = cmk(0.0, 0.0);
    for (int e = 0; e < FT_E; e++) {
        const int k = FT_EK[e], l = FT_EL[e];
        A[l * FT_N + l] = A[l * FT_N + l] + y[e];
        if (k == FT_V - 1) continue;
        A[k * FT_N + k] = A[k * FT_N + k] + y[e];
        A[k * FT_N + l] = A[k * FT_N + l] - y[e];
        A[l * FT_N + k] = A[l * FT_N + k] - y[e];
    }
    int nt = 0;
    for (int k = 0; k < FT_N; k++) {
        int br = k, bc = k;
        double best = -1.0;
        for (int c = k; c < FT_N; c++)
            for (int r = k; r < FT_N; r++) {
                double s = cabs_(A[r * FT_N + c]);
                if (s > best) {
                    best = s;
                    br = r;
                    bc = c;
                }
            }
        rp[k] = br;
        cp[k] = bc;
        if (br != k) {
            for (int c = 0; c < FT_N; c++) {
                cx<double> t = A[k * FT_N + c];
                A[k * FT_N + c] = A[br * FT_N + c];
                A[br * FT_N + c] = t;
            }
            nt++;
        }
        if (bc != k) {
            for (int r = 0; r < FT_N; r++) {
                cx<double> t = A[r * FT_N + k];
                A[r * FT_N + k] = A[r * FT_N + bc];
                A[r * FT_N + bc] = t;
            }
            nt++;
        }
        cx<double> inv = crecip(A[k * FT_N + k]);
        for (int r = k + 1; r < FT_N; r++) A[r * FT_N + k] = A[r * FT_N + k] * inv;
        for (int r = k + 1; r < FT_N; r++)
            for (int c = k + 1; c < FT_N; c++) A[r * FT_N + c] = A[r * FT_N + c] - A[r * FT_N + k] * A[k * FT_N + c];
    }
    det = cmk(1.0, 0.0);
    for (int i = 0; i < FT_N; i++) det = det * A[i * FT_N + i];
    if (nt & 1) det = cmk(-det.re, -det.im);
    // -tr(L^-1 P~), P~ = sum_r sigma_r q_r q_r^T: sum_r sigma_r q_r^T L^-1 q_r
    cx<double> tr = cmk(0.0, 0.0);
    for (int r = 0; r < FT_RANK; r++) {
        cx<double> b[FT_N];
        for (int i = 0; i < FT_N; i++) b[i] = cmk(prm[P_Q + r * FT_N + i], 0.0);
        for (int k = 0; k < FT_N; k++) {
            cx<double> t = b[k];
            b[k] = b[rp[k]];
            b[rp[k]] = t;
        }
        for (int i = 0; i < FT_N; i++)
            for (int j = 0; j < i; j++) b[i] = b[i] - A[i * FT_N + j] * b[j];
        for (int i = FT_N - 1; i >= 0; i--) {
            for (int j = i + 1; j < FT_N; j++) b[i] = b[i] - A[i * FT_N + j] * b[j];
            b[i] = b[i] * crecip(A[i * FT_N + i]);
        }
        for (int k = FT_N - 1; k >= 0; k--) {
            cx<double> t = b[k];
            b[k] = b[cp[k]];
            b[cp[k]] = t;
        }
        cx<double> s = cmk(0.0, 0.0);
        for (int i = 0; i < FT_N; i++) s = s + prm[P_Q + r * FT_N + i] * b[i];
        tr = tr + prm[P_SIG + r] * s;
    }
    pphi = cmk(-tr.re, -tr.im);
}

// ------------------------------------------------------------------ robust derivatives
// x-derivatives of phi/psi by the reference's route (srcs/feynman_integral.hpp:166-194,
// 283-287; srcs/laplacian.hpp:14-99, 102-215), for samples where an edge's conductance
// 1/x_e dwarfs the rest of the network between its ends: the fixed ground of the
// unrolled path then leaves both ends floating together, and the potential and
// resistance differences across the edge cancel.  Grounding the vertex with the
// smallest sum of incident x (the reference's choice) ties such an edge to the ground.
// Reduced Laplacian with that ground, LDL^T with diagonal pivoting, L^-1, L^-1 P L^-T,
// then the derivatives as differences of their entries.  Runtime indices, out of line:
// it runs for a few samples in 1e4 (edge weights below 1 make tiny x more frequent).
static __device__ __noinline__ void robust_derivatives(const double* X, const double* Xi, const double* prm,
                                                       double* dphi, double (*H)[FT_E])
{
    double XV[FT_V];
#pragma unroll 1
    for (int v = 0; v < FT_V; v++) XV[v] = 0.0;
#pragma unroll 1
    for (int e = 0; e < FT_E; e++) {
        XV[FT_EK[e]] += X[e];
        XV[FT_EL[e]] += X[e];
    }
    int gnd = 0;
#pragma unroll 1
    for (int v = 1; v < FT_V; v++)
        if (XV[gnd] > XV[v]) gnd = v;
    int map[FT_V];
#pragma unroll 1
    for (int v = 0; v < FT_V; v++) map[v] = v < gnd ? v : (v > gnd ? v - 1 : FT_N);
    // reduced Laplacian A and contracted scalar products B (P from its rank split; the
    // ground-V-1 row and column follow from momentum conservation)
    double A[FT_N][FT_N], B[FT_N][FT_N];
#pragma unroll 1
    for (int i = 0; i < FT_N; i++)
#pragma unroll 1
        for (int j = 0; j < FT_N; j++) A[i][j] = 0.0;
#pragma unroll 1
    for (int e = 0; e < FT_E; e++) {
        const int k = map[FT_EK[e]], l = map[FT_EL[e]];
        if (k < FT_N) A[k][k] += Xi[e];
        if (l < FT_N) A[l][l] += Xi[e];
        if (k < FT_N && l < FT_N) {
            A[k][l] -= Xi[e];
            A[l][k] -= Xi[e];
        }
    }
    auto Pfull = [&](int i, int j) -> double {
        // P[i][j] of the V x V matrix with zero row and column sums
        double s = 0.0;
#pragma unroll 1
        for (int r = 0; r < FT_RANK; r++) {
            double qi = 0.0, qj = 0.0;
            if (i < FT_N) {
                qi = prm[P_Q + r * FT_N + i];
            } else {
#pragma unroll 1
                for (int m = 0; m < FT_N; m++) qi -= prm[P_Q + r * FT_N + m];
            }
            if (j < FT_N) {
                qj = prm[P_Q + r * FT_N + j];
            } else {
#pragma unroll 1
                for (int m = 0; m < FT_N; m++) qj -= prm[P_Q + r * FT_N + m];
            }
            s += prm[P_SIG + r] * qi * qj;
        }
        return s;
    };
#pragma unroll 1
    for (int v = 0; v < FT_V; v++) {
        if (v == gnd) continue;
#pragma unroll 1
        for (int w = 0; w < FT_V; w++) {
            if (w == gnd) continue;
            B[map[v]][map[w]] = Pfull(v, w);
        }
    }
    // A = P^T L D L^T P (diagonal pivoting); then A^-1 column by column into C
    int perm[FT_N];
#pragma unroll 1
    for (int i = 0; i < FT_N; i++) perm[i] = i;
#pragma unroll 1
    for (int k = 0; k < FT_N; k++) {
        int pk = k;
#pragma unroll 1
        for (int i = k + 1; i < FT_N; i++)
            if (fabs(A[i][i]) > fabs(A[pk][pk])) pk = i;
        if (pk != k) {
#pragma unroll 1
            for (int j = 0; j < FT_N; j++) {
                const double t = A[k][j];
                A[k][j] = A[pk][j];
                A[pk][j] = t;
            }
#pragma unroll 1
            for (int j = 0; j < FT_N; j++) {
                const double t = A[j][k];
                A[j][k] = A[j][pk];
                A[j][pk] = t;
            }
            const int t = perm[k];
            perm[k] = perm[pk];
            perm[pk] = t;
        }
        const double dk = A[k][k];
        // Schur update of the whole (symmetric) trailing block, so that later pivot
        // swaps see current values in both triangles; row k keeps the unscaled column
#pragma unroll 1
        for (int i = k + 1; i < FT_N; i++) {
            const double f = A[i][k] / dk;
#pragma unroll 1
            for (int j = k + 1; j < FT_N; j++) A[i][j] -= f * A[k][j];
        }
#pragma unroll 1
        for (int i = k + 1; i < FT_N; i++) A[i][k] /= dk;
    }
    // columns of the inverse: solve L D L^T y = P e_c; C[perm[i]][c] = y_i
    double C[FT_N][FT_N];
#pragma unroll 1
    for (int c = 0; c < FT_N; c++) {
        double y[FT_N];
#pragma unroll 1
        for (int i = 0; i < FT_N; i++) {
            double t = perm[i] == c ? 1.0 : 0.0;
#pragma unroll 1
            for (int j = 0; j < i; j++) t -= A[i][j] * y[j];
            y[i] = t;
        }
#pragma unroll 1
        for (int i = 0; i < FT_N; i++) y[i] /= A[i][i];
#pragma unroll 1
        for (int i = FT_N - 1; i >= 0; i--)
#pragma unroll 1
            for (int j = i + 1; j < FT_N; j++) y[i] -= A[j][i] * y[j];
#pragma unroll 1
        for (int i = 0; i < FT_N; i++) C[perm[i]][c] = y[i];
    }
    // S = C B C^T (into A, reusing it)
#pragma unroll 1
    for (int i = 0; i < FT_N; i++)
#pragma unroll 1
        for (int j = 0; j < FT_N; j++) {
            double t = 0.0;
#pragma unroll 1
            for (int k = 0; k < FT_N; k++) t += C[i][k] * B[k][j];
            A[i][j] = t;
        }
#pragma unroll 1
    for (int i = 0; i < FT_N; i++)
#pragma unroll 1
        for (int j = 0; j < FT_N; j++) {
            double t = 0.0;
#pragma unroll 1
            for (int k = 0; k < FT_N; k++) t += A[i][k] * C[j][k];
            B[i][j] = t;
        }
    // derivatives (srcs/laplacian.hpp:127-213): differences of S = B and of C
    auto S = [&](int i, int j) -> double { return (i == FT_N || j == FT_N) ? 0.0 : B[i][j]; };
    auto T = [&](int i, int j) -> double { return (i == FT_N || j == FT_N) ? 0.0 : C[i][j]; };
#pragma unroll 1
    for (int a = 0; a < FT_E; a++) {
        const int ka = map[FT_EK[a]], la = map[FT_EL[a]];
        const double s = S(ka, ka) + S(la, la) - 2.0 * S(ka, la);
        const double t = T(ka, ka) + T(la, la) - 2.0 * T(ka, la);
        const double xa = Xi[a] * Xi[a];
        const double xas = xa * s;
        dphi[a] = -xas;
        H[a][a] = 2.0 * xas * (Xi[a] - xa * t);
#pragma unroll 1
        for (int b = a + 1; b < FT_E; b++) {
            const int kb = map[FT_EK[b]], lb = map[FT_EL[b]];
            const double s2 = S(ka, kb) + S(la, lb) - S(ka, lb) - S(la, kb);
            const double t2 = T(ka, kb) + T(la, lb) - T(ka, lb) - T(la, kb);
            H[a][b] = -2.0 * xa * (Xi[b] * Xi[b]) * s2 * t2;
        }
    }
}

// ------------------------------------------------------------------ sector draw, FP64
struct table_ref {
    const void* w;              // staged copies (shared memory): w, Jr, 1/r in the working precision
    const void* Jr;
    const void* ri;
    const unsigned char* meta;  // mm << 7 | loop number
    const unsigned char* gm;    // global copy (FP64 sections for exact re-checks)
};

#if FT_BATCH
// The batch kernels' current work item and its instance's table (global copy), written
// by the block's first thread between items and read where they are used, so that
// neither is held in registers across the per-sample code.
__shared__ unsigned long long s_batch_item;
__shared__ const unsigned char* s_batch_tab;
#define TABLE_GM(t) s_batch_tab
// first word of an FP64-pass queue entry: item << 28 | lane << 18 | offset of the
// sample in the lane's chunk (the other four hold the sample's stream state)
#define BQ_ITEM_SHIFT 28
#define BQ_LANE_SHIFT 18
#define BQ_OFF_MASK ((1ull << BQ_LANE_SHIFT) - 1ull)
#define BQ_LANE_MASK 1023ull
#else
#define TABLE_GM(t) ((t).gm)
#endif

static __device__ __forceinline__ void draw_sector64(xo& g, const table_ref& t, double Jr_full, double* X, double& F,
                                                     double& Gv, unsigned char* ord)
{
    const double* w = (const double*)t.w;
    const double* Jr = (const double*)t.Jr;
    const double* ri = (const double*)t.ri;
    const unsigned char* meta = t.meta;
    u32 sub = FT_FULL;
    double JJr = Jr_full, XX = 1.0;
    bool MM = true;
    int oL = FT_LOOPS;
    F = 1.0;
    Gv = 0.0;
#pragma unroll
    for (int j = 0; j < FT_E; j++) {
        const double R = u01(g.next()) * JJr;
        double T = 0.0;
        int e = 0;
        // the subgraph's edges in ascending order (its set bits) until the running sum
        // passes R, else the last one
        for (u32 left = sub; left != 0u; left &= left - 1u) {
            e = __ffs(left) - 1;
            T += w[sub ^ (1u << e)];
            if (T > R) break;
        }
        sub ^= 1u << e;
        JJr = Jr[sub];
        const double rinv = ri[sub];
        const unsigned m = meta[sub];
        const bool mm = (m >> 7) != 0;
        const int L = (int)(m & 127u);
        if (MM && !mm) Gv = XX;
        MM = mm;
#pragma unroll
        for (int k = 0; k < FT_E; k++)
            if (k == e) X[k] = XX;
        if (L < oL) {
            F *= XX;
            oL = L;
        }
        if (FT_RECORD) ord[j] = (unsigned char)e;
        if (j < FT_E - 1) XX *= pow(1.0 - u01(g.next()), rinv);
    }
}

// ------------------------------------------------------------------ sector draw, mixed
// two-float value hi + lo
struct f2 {
    float hi, lo;
};
static __device__ __forceinline__ f2 f2_add(f2 a, float b)
{
    float s = a.hi + b;
    float bb = s - a.hi;
    float err = (a.hi - (s - bb)) + (b - bb);
    float lo = a.lo + err;
    float h = s + lo;
    f2 r;
    r.hi = h;
    r.lo = lo - (h - s);
    return r;
}
static __device__ __forceinline__ f2 f2_add2(f2 a, f2 b)
{
    f2 r = f2_add(a, b.hi);
    return f2_add(r, b.lo);
}

// log(1 - u) for u = (x >> 11) 2^-53, to about 1e-7 absolute (undeformed integrands), with integer and FP32
// instructions only (64-bit integer to float conversions would run on the FP64 pipe).
// A positive integer v is turned into the float bits of 2^k (1 + f) directly: k from
// the leading-zero count, f from the next 23 bits rounded (a carry bumps k).
static __device__ __forceinline__ int float_bits_of(u64 v, int scale_exp)
{
    const int lz = __clzll(v);
    const u64 frac = ((((v << lz) << 1) >> 40) + 1ull) >> 1;   // 23 bits after the leading 1, rounded
    return ((63 - lz + scale_exp + 127) << 23) + (int)frac;
}

static __device__ __forceinline__ f2 log1m_u32(u64 x)
{
    const u64 m = x >> 11;
    f2 r;
    r.lo = 0.0f;
    if (m < (1ull << 52)) {
        // u < 1/2: log1p(-u)
        r.hi = m ? m_log1p(-__int_as_float(float_bits_of(m, -53))) : 0.0f;
        return r;
    }
    // 1 - u = q 2^-53 exactly (q < 2^52); q = 2^k (1 + f): log(1 - u) = (k - 53) ln2 + log1p(f)
    const int bits = float_bits_of((1ull << 53) - m, 0);
    const int k = (bits >> 23) - 127;
    const float f = __int_as_float((bits & 0x007fffff) | 0x3f800000) - 1.0f;
    const float kk = (float)(k - 53);
    // ln2 split so that kk * LN2_HI is exact
    const float LN2_HI = 0.693145751953125f, LN2_LO = 1.42860682030941723212e-6f;
    f2 a;
    a.hi = kk * LN2_HI;
    a.lo = kk * LN2_LO;
    return f2_add(a, m_log1p(f));
}

static __device__ __forceinline__ f2 f2_two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    f2 r;
    r.hi = s;
    r.lo = (a - (s - bb)) + (b - bb);
    return r;
}

// log(1 - u) for u = (x >> 11) 2^-53 in two-float, to about 1e-12 absolute, with integer
// and FP32 instructions only (64-bit conversions and FP64 would run on the FP64 pipe).
// Table-driven reduction after Tang (ACM TOMS 16, 1990): 1 - u = q 2^-53 with the
// integer q = 2^53 - (x >> 11) exactly, q = 2^k M with M in [1, 2) held as two floats
// (47 fraction bits); c_i = 1 + (i + 1/2)/64 for the top 6 fraction bits i,
// r_i = fl(1/c_i) and -log r_i (two-float) from FT_LOGTAB; z = M r_i - 1 (|z| < 1/100)
// from exact products, log M = -log r_i + log1p(z) with log1p(z) = z - z^2/2 + z^3/3 -
// z^4/4 + z^5/5, the terms past z in FP32.
static __device__ FT_BIGFN f2 log1m_u2(u64 x)
{
    const u64 q = (1ull << 53) - (x >> 11);   // 1 .. 2^53
    const int lz = __clzll(q);
    const u64 mb = q << lz;                    // M = mb / 2^63, leading 1 at bit 63
    const u32 top = (u32)(mb >> 40);           // 1 + 23 fraction bits
    const float m_hi = __int_as_float(0x3f800000 | (int)(top & 0x7fffffu));
    const float m_lo = (float)(u32)((mb >> 16) & 0xffffffull) * 0x1.0p-47f;
    const int i = (int)((top >> 17) & 63u);
    const float r = FT_LOGTAB[3 * i], nl_hi = FT_LOGTAB[3 * i + 1], nl_lo = FT_LOGTAB[3 * i + 2];
    // z = M r - 1: m_hi r = p + e exactly, p - 1 exact (p within 1% of 1)
    const float p = m_hi * r;
    const float e = fmaf(m_hi, r, -p);
    const f2 z = f2_two_sum(p - 1.0f, fmaf(m_lo, r, e));
    const float zh = z.hi;
    const float tail = zh * zh * fmaf(zh, fmaf(zh, fmaf(zh, 0.2f, -0.25f), 0.333333343f), -0.5f);
    // (k - 53) ln2 with ln2 in three parts (LN2_HI has 16 bits: the products are exact)
    const float kk = (float)(10 - lz);          // k - 53 with k = 63 - lz
    const float LN2_HI = 0.693145751953125f, LN2_LO = 1.428606765330187e-06f, LN2_LO2 = 5.497923e-14f;
    f2 acc = f2_two_sum(kk * LN2_HI, nl_hi);
    acc = f2_add(acc, fmaf(kk, LN2_LO, nl_lo));
    acc = f2_add(acc, fmaf(kk, LN2_LO2, z.lo + tail));
    return f2_add(acc, zh);
}

// e^a for a two-float a (|a| < 80) in two-float, about 1e-12 relative; table-driven
// after Tang (ACM TOMS 15, 1989): a = (32 m + j) ln2/32 + s with |s| <= ln2/64,
// e^a = 2^m 2^(j/32) e^s, 2^(j/32) as two floats from FT_EXPTAB, e^s = 1 + s + s^2/2 +
// s^3/6 + s^4/24 with the terms past s in FP32.  ln2/32 = C1 + C2 + C3, C1 with 11
// significant bits so that k C1 is exact for |k| < 2^13.
static __device__ FT_BIGFN f2 exp_f2(f2 a)
{
    const float C1 = 0x1.62cp-6f, C2 = 0x1.217f7ep-17f, C3 = -0x1.c610cap-42f;
    const float kf = rintf(a.hi * 46.1662407f);
    const int k = (int)kf;
    // a - k C1 is exact; k C2 = p2 + e2 exactly
    const float p2 = kf * C2;
    const float e2 = fmaf(kf, C2, -p2);
    f2 sv = f2_two_sum(fmaf(-kf, C1, a.hi), -p2);
    sv = f2_add(sv, fmaf(-kf, C3, a.lo - e2));
    const float sh = sv.hi;
    const float tail = sh * sh * fmaf(sh, fmaf(sh, 0.0416666679f, 0.166666672f), 0.5f);
    // e^s = 1 + es
    f2 es = f2_two_sum(sh, sv.lo + tail);
    es = f2_add(f2_two_sum(1.0f, es.hi), es.lo);
    const int j = k & 31, m = k >> 5;
    const float t_hi = FT_EXPTAB[2 * j], t_lo = FT_EXPTAB[2 * j + 1];
    // (t_hi + t_lo)(es.hi + es.lo) with the product error of the leading term
    const float ph = t_hi * es.hi;
    const float pl = fmaf(t_hi, es.hi, -ph) + fmaf(t_hi, es.lo, t_lo * es.hi);
    const f2 pr = f2_two_sum(ph, pl);
    const float sc = __int_as_float((127 + m) << 23);   // 2^m, |m| < 126
    f2 out;
    out.hi = pr.hi * sc;
    out.lo = pr.lo * sc;
    return out;
}

// The reference's comparison, exactly (FP64, ascending edges, first running sum above
// u * Jr(gamma), else the last edge): used when an FP32 comparison is within its
// error margin.  Out of line: it runs for a few steps per 1e4 samples.
static __device__ __noinline__ int exact_cut(u64 x, u32 sub, const unsigned char* __restrict__ gm)
{
    const double* w64 = (const double*)(gm + T_W64);
    const double* Jr64 = (const double*)(gm + T_JR64);
    const double R = u01(x) * Jr64[sub];
    double TT = 0.0;
    int cut = 0;
    for (int c = 0; c < FT_E; c++) {
        if ((sub >> c) & 1u) {
            TT += w64[sub ^ (1u << c)];
            cut = c;
            if (TT > R) break;
        }
    }
    return cut;
}

static __device__ __forceinline__ int draw_sector32(xo& g, const table_ref& t, const float* pf, f2* lx, f2& lF,
                                                    f2& lG, unsigned char* ord)
{
    const float* w = (const float*)t.w;
    const float* Jr = (const float*)t.Jr;
    const float* ri = (const float*)t.ri;
    const unsigned char* meta = t.meta;
    u32 sub = FT_FULL;
    float JJr = pf[P_JRFULL];
    bool MM = true;
    int oL = FT_LOOPS, exact = 0;
    f2 lxx;
    lxx.hi = lxx.lo = 0.0f;
    lF = lxx;
    lG = lxx;
#pragma unroll
    for (int j = 0; j < FT_E; j++) {
        const u64 x = g.next();
        // FP32 decision with margin: |T32 - T64| <= (2E) 2^-24 Jr, |R32 - R64| <= 4 2^-24 Jr
        const float uf = (float)(u32)(x >> 40) * 0x1.0p-24f;
        const float Rf = uf * JJr;
        const float margin = (float)(2 * FT_E + 8) * 0x1.0p-24f * JJr;
        float T = 0.0f;
        int e = 0, sure = -1;
        bool unsure = false;
        // the edges of the current subgraph in ascending order (its set bits), up to the
        // first sure decision: the same comparisons as a scan over all E edges, without
        // the trips over edges already cut
        for (u32 left = sub; left != 0u; left &= left - 1u) {
            const int c = __ffs(left) - 1;
            T += w[sub ^ (1u << c)];
            e = c;
            const float d = T - Rf;
            if (d > margin) {
                sure = c;
                break;
            }
            if (d >= -margin) unsure = true;
        }
        int cut = sure >= 0 ? sure : e;
        if (unsure) {
            cut = exact_cut(x, sub, TABLE_GM(t));
            exact++;
        }
        sub ^= 1u << cut;
        JJr = Jr[sub];
        const float2 rinv = ((const float2*)ri)[sub];   // 1/r as two floats
        const unsigned m = meta[sub];
        const bool mm = (m >> 7) != 0;
        const int L = (int)(m & 127u);
        if (MM && !mm) lG = lxx;
        MM = mm;
#pragma unroll
        for (int k = 0; k < FT_E; k++)
            if (k == cut) lx[k] = lxx;
        if (L < oL) {
            lF = f2_add2(lF, lxx);
            oL = L;
        }
        if (FT_RECORD) ord[j] = (unsigned char)cut;
        if (j < FT_E - 1) {
#if FT_MODE == 1
            // deformed integrands: the phase moves by |theta| per unit of log X, so the
            // sector point is carried to ~1e-12 (two-float logarithm)
            f2 l = log1m_u2(g.next());
#else
            f2 l = log1m_u32(g.next());
#endif
            // (hi + lo) * (rinv.x + rinv.y) with the product error kept
            float p = l.hi * rinv.x;
            float pe = fmaf(l.hi, rinv.x, -p) + fmaf(l.hi, rinv.y, l.lo * rinv.x);
            f2 inc;
            inc.hi = p;
            inc.lo = pe;
            lxx = f2_add2(lxx, inc);
        }
    }
    return exact;
}

// ------------------------------------------------------------------ integrand, FP64
// X: unnormalised sector point; returns R per eps order, false when dropped.
// `robust` reports that the complete-pivoting LU was needed.
static __device__ __forceinline__ bool integrand64(const double* prm, double* X, double psi_tr, double xi_tr,
                                                   cx<double>* out, bool& robust)
{
    const double D = prm[P_D], W = prm[P_W], IGtr = prm[P_IGTR];
    // normalise so that psi_tr^(-D/2) (psi_tr/xi_tr)^W = 1 (srcs/feynman_integral.hpp:201-204)
    const double tgt = pow(psi_tr, -D / 2.) * pow(psi_tr / xi_tr, W);
    const double scale = pow(tgt, prm[P_NORM]);
    double Xi[FT_E];
    double Xprod = 1.0;
#pragma unroll
    for (int e = 0; e < FT_E; e++) {
        X[e] *= scale;
        Xi[e] = 1.0 / X[e];
        Xprod *= X[e];
    }
    elim<double, double> L;
    L.factor(Xi);
    double det = 1.0;
#pragma unroll
    for (int k = 0; k < FT_N; k++) det *= L.d[k];
    robust = false;
#if FT_MODE == 0
    const double psi = det * Xprod;
    double R = IGtr * pow(psi, -D / 2.);
    if (!isfinite(R)) return false;
#if FT_ONLY_PSI
    out[0] = cmk(R, 0.0);
    return true;
#else
    double tr = 0.0;
#pragma unroll
    for (int r = 0; r < FT_RANK; r++) tr += prm[P_SIG + r] * L.quad(prm + P_Q + r * FT_N);
    double pxi = -tr;
#pragma unroll
    for (int e = 0; e < FT_E; e++) pxi += prm[P_M2 + e] * X[e];
    R *= pow(pxi, -W);
    if (!isfinite(R)) return false;
    out[0] = cmk(R, 0.0);
    if (FT_K > 1) {
        const double ef = log(psi) - FT_LOOPS * log(pxi);
#pragma unroll
        for (int j = 1; j < FT_K; j++) {
            R *= ef / (double)j;
            out[j] = cmk(R, 0.0);
        }
    }
    return true;
#endif
#else
    const double kappa = prm[P_DEF];
    // G = L^-1 = N diag(1/d) N^T with N = M^-1 (entrywise non-negative)
    double Nm[FT_N][FT_N];
#pragma unroll
    for (int i = FT_N - 1; i >= 0; i--) {
#pragma unroll
        for (int j = 0; j < FT_N; j++) Nm[i][j] = 0.0;
        Nm[i][i] = 1.0;
#pragma unroll
        for (int j = i + 1; j < FT_N; j++) {
            if (!NZM(i, j)) continue;
            double s = 0.0;
#pragma unroll
            for (int k = i + 1; k <= j; k++)
                if (NZC(i, k) && (k == j || NZM(k, j))) s += L.a[i][k] * Nm[k][j];
            Nm[i][j] = s;
        }
    }
    double id[FT_N];
#pragma unroll
    for (int k = 0; k < FT_N; k++) id[k] = 1.0 / L.d[k];
    double G[FT_N][FT_N];
#pragma unroll
    for (int i = 0; i < FT_N; i++)
#pragma unroll
        for (int j = i; j < FT_N; j++) {
            double s = 0.0;
#pragma unroll
            for (int k = j; k < FT_N; k++)
                if ((k == i || NZM(i, k)) && (k == j || NZM(j, k))) s += Nm[i][k] * Nm[j][k] * id[k];
            G[i][j] = s;
            G[j][i] = s;
        }
    // h_r = L^-1 q_r; per edge: hb[r][e] = h_r . b_e with b_e = e_k - e_l (ground row zero)
    double hb[FT_RANK][FT_E];
#pragma unroll
    for (int r = 0; r < FT_RANK; r++) {
        double h[FT_N];
#pragma unroll
        for (int i = 0; i < FT_N; i++) {
            double s = 0.0;
#pragma unroll
            for (int j = FT_Q0; j < FT_N; j++) s += G[i][j] * prm[P_Q + r * FT_N + j];
            h[i] = s;
        }
#pragma unroll
        for (int e = 0; e < FT_E; e++) {
            const int k = FT_EK[e], l = FT_EL[e];
            hb[r][e] = (k == FT_V - 1 ? 0.0 : h[k]) - h[l];
        }
    }
    // s_ab = sum_r sigma_r hb_a hb_b, t_ab = b_a^T G b_b
    auto Gx = [&](int i, int j) -> double { return (i == FT_V - 1 || j == FT_V - 1) ? 0.0 : G[i][j]; };
    double dphi[FT_E];
    double H[FT_E][FT_E];
    bool cancel = false;
#pragma unroll
    for (int a = 0; a < FT_E; a++) {
        const int ka = FT_EK[a], la = FT_EL[a];
        double s = 0.0;
#pragma unroll
        for (int r = 0; r < FT_RANK; r++) s += prm[P_SIG + r] * hb[r][a] * hb[r][a];
        const double t = Gx(ka, ka) + Gx(la, la) - 2.0 * Gx(ka, la);
        // an edge whose ends float together: its resistance difference cancels
        cancel |= ka != FT_V - 1 && !(t > 1e-7 * (Gx(ka, ka) + Gx(la, la)));
        const double xa = Xi[a] * Xi[a];
        const double xas = xa * s;
        dphi[a] = -xas;
        H[a][a] = 2.0 * xas * (Xi[a] - xa * t);
#pragma unroll
        for (int b = a + 1; b < FT_E; b++) {
            const int kb = FT_EK[b], lb = FT_EL[b];
            double s2 = 0.0;
#pragma unroll
            for (int r = 0; r < FT_RANK; r++) s2 += prm[P_SIG + r] * hb[r][a] * hb[r][b];
            const double t2 = Gx(ka, kb) + Gx(la, lb) - Gx(ka, lb) - Gx(la, kb);
            H[a][b] = -2.0 * xa * (Xi[b] * Xi[b]) * s2 * t2;
        }
    }
    if (cancel) {
        robust_derivatives(X, Xi, prm, dphi, H);
        robust = true;
    }
    // deformation x -> x exp(i theta), theta = -lambda (d(phi/psi)/dx + m^2)
    double theta[FT_E];
    cx<double> cX[FT_E], cy[FT_E];
    double xnu = 0.0;
    cx<double> cXprod = cmk(1.0, 0.0);
#pragma unroll
    for (int e = 0; e < FT_E; e++) {
        theta[e] = (dphi[e] + prm[P_M2 + e]) * kappa;
        FT_DBG(40 + e, theta[e]);
        double sn, cs;
        sincos(theta[e], &sn, &cs);
        cX[e] = cmk(X[e] * cs, X[e] * sn);
        cy[e] = cmk(Xi[e] * cs, -Xi[e] * sn);   // 1 / cX
        xnu += prm[P_NU + e] * theta[e];
        cXprod = cXprod * cX[e];
    }
    elim<cx<double>, double> CL;
    const double growth = CL.factor(cy);
    cx<double> cdet, cpphi;
    if (growth > 1e-8) {
        cdet = cmk(1.0, 0.0);
#pragma unroll
        for (int k = 0; k < FT_N; k++) cdet = cdet * CL.d[k];
        cx<double> tr = cmk(0.0, 0.0);
#pragma unroll
        for (int r = 0; r < FT_RANK; r++) tr = tr + prm[P_SIG + r] * CL.quad(prm + P_Q + r * FT_N);
        cpphi = cmk(-tr.re, -tr.im);
    } else {
        robust = true;
        robust_complex(cy, prm, cdet, cpphi);
    }
    const cx<double> cPsi = cXprod * cdet;
    cx<double> cR = IGtr * cpow_(cPsi, -D / 2.);
    // det(I + i kappa X^1/2 H X^1/2), symmetric elimination without pivoting
    cx<double> J[FT_E][FT_E];
    double sx[FT_E];
#pragma unroll
    for (int e = 0; e < FT_E; e++) sx[e] = sqrt(X[e]);
#pragma unroll
    for (int a = 0; a < FT_E; a++)
#pragma unroll
        for (int b = a; b < FT_E; b++) J[a][b] = cmk(a == b ? 1.0 : 0.0, kappa * H[a][b] * sx[a] * sx[b]);
    cx<double> detJ = cmk(1.0, 0.0);
#pragma unroll
    for (int k = 0; k < FT_E; k++) {
        const cx<double> piv = J[k][k];
        detJ = detJ * piv;
        const cx<double> inv = crecip(piv);
#pragma unroll
        for (int i = k + 1; i < FT_E; i++) {
            const cx<double> f = J[k][i] * inv;
#pragma unroll
            for (int j = i; j < FT_E; j++) J[i][j] = J[i][j] - f * J[k][j];
        }
    }
    double sn, cs;
    sincos(xnu, &sn, &cs);
    cR = cR * (detJ * cmk(cs, sn));
    cx<double> cPXi = cpphi;
#pragma unroll
    for (int e = 0; e < FT_E; e++) cPXi = cPXi + prm[P_M2 + e] * cX[e];
    FT_DBG(50, log2(hypot(detJ.re, detJ.im)));
    FT_DBG(51, atan2(detJ.im, detJ.re));
    FT_DBG(52, atan2(cPsi.im, cPsi.re));
    FT_DBG(54, atan2(cPXi.im, cPXi.re));
    FT_DBG(55, xnu);
    FT_DBG(56, cpphi.re);
    FT_DBG(57, cpphi.im);
    FT_DBG(58, cPXi.re);
    FT_DBG(59, cPXi.im);
    cR = cR * cpow_(cPXi, -W);
    if (!cfinite(cR)) return false;
    out[0] = cR;
    if (FT_K > 1) {
        const cx<double> lp = clog_(cPsi), lv = clog_(cPXi);
        const cx<double> ef = cmk(lp.re - FT_LOOPS * lv.re, lp.im - FT_LOOPS * lv.im);
#pragma unroll
        for (int j = 1; j < FT_K; j++) {
            cR = cR * ((1.0 / (double)j) * ef);
            out[j] = cR;
        }
    }
    return true;
#endif
}


// ------------------------------------------------------------------ integrand, mixed
#if FT_PREC == 1
#if FT_MODE == 1
// ------------------------------------------------------------------ two-float arithmetic
// Values hi + lo with |lo| <= ulp(hi)/2 (about 48 significant bits) from error-free
// transformations of FP32 operations (Knuth's two-sum, the FMA two-product); they run
// on the FP32 pipe, which is ~60x wider than the FP64 pipe on this GPU.
struct df {
    float hi, lo;
};
static __device__ __forceinline__ df df_mk(float x)
{
    df r;
    r.hi = x;
    r.lo = 0.0f;
    return r;
}
static __device__ __forceinline__ df df_norm(float s, float e)
{
    df r;
    r.hi = s + e;
    r.lo = e - (r.hi - s);
    return r;
}
static __device__ FT_DFFN df df_add(df x, df y)
{
    const float s = x.hi + y.hi;
    const float bb = s - x.hi;
    float e = (x.hi - (s - bb)) + (y.hi - bb);
    e += x.lo + y.lo;
    return df_norm(s, e);
}
static __device__ __forceinline__ df df_neg(df x)
{
    x.hi = -x.hi;
    x.lo = -x.lo;
    return x;
}
static __device__ __forceinline__ df df_sub(df x, df y) { return df_add(x, df_neg(y)); }
// A product cannot cancel: its low part e stays within ~1.5 ulp of p, which every
// consumer (sums, products, the reciprocal, conversions) handles, so it is returned
// without renormalisation.
static __device__ FT_DFFN df df_mul(df x, df y)
{
    const float p = x.hi * y.hi;
    float e = fmaf(x.hi, y.hi, -p);
    e = fmaf(x.hi, y.lo, e);
    e = fmaf(x.lo, y.hi, e);
    df r;
    r.hi = p;
    r.lo = e;
    return r;
}
// x y + z: the leading product exact (FMA residual), one two-sum with z.hi, the small
// terms added once
static __device__ FT_DFFN df df_fma(df x, df y, df z)
{
    const float p = x.hi * y.hi;
    const float pe = fmaf(x.hi, y.hi, -p);
    const float s = p + z.hi;
    const float bb = s - p;
    float e = (p - (s - bb)) + (z.hi - bb);
    e += pe + fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, z.lo));
    return df_norm(s, e);
}
static __device__ FT_DFFN df df_inv(df x)
{
    // one Newton step from the FP32 reciprocal r: 1/x = r (1 + e) with e = 1 - x r;
    // 1 - x.hi r (about 2^-23) is exact to 2^-47 by the FMA, then x.lo r is removed.
    // |r e| stays within about an ulp of r, so the pair needs no renormalisation.
    const float r = rcp_(x.hi);
    const float e = fmaf(-x.lo, r, fmaf(-x.hi, r, 1.0f));
    df o;
    o.hi = r;
    o.lo = r * e;
    return o;
}
static __device__ __forceinline__ float df_f(df x) { return x.hi + x.lo; }
static __device__ __forceinline__ df df_of(f2 x)
{
    df r;
    r.hi = x.hi;
    r.lo = x.lo;
    return r;
}

// ------------------------------------------------------------------ complex two-float
// Complex two-float numbers, and sin / cos of a two-float angle to ~1e-13, table-driven
// after Tang: x = k pi/64 + r with |r| <= pi/128 (pi/64 as three FP32 parts, each
// k * part formed exactly with an FMA); sin(k pi/64), cos(k pi/64) as float pairs from
// FT_SCTAB (k mod 128); sin r = r - r^3/6 + r^5/120 and cos r = 1 - r^2/2 + r^4/24 -
// r^6/720 with r and r^2 in two-float and the terms below 3e-6 in FP32; then
// sin x = sin a cos r + cos a sin r, cos x = cos a cos r - sin a sin r in two-float.
struct cdf {
    df re, im;
};
static __device__ __forceinline__ cdf cdf_mk(df r, df i)
{
    cdf z;
    z.re = r;
    z.im = i;
    return z;
}
static __device__ __forceinline__ cdf cdf_zero() { return cdf_mk(df_mk(0.0f), df_mk(0.0f)); }
static __device__ __forceinline__ cdf operator+(cdf a, cdf b) { return cdf_mk(df_add(a.re, b.re), df_add(a.im, b.im)); }
static __device__ __forceinline__ cdf operator-(cdf a, cdf b) { return cdf_mk(df_sub(a.re, b.re), df_sub(a.im, b.im)); }
static __device__ FT_CXFN cdf operator*(cdf a, cdf b)
{
    return cdf_mk(df_fma(a.re, b.re, df_neg(df_mul(a.im, b.im))), df_fma(a.re, b.im, df_mul(a.im, b.re)));
}
static __device__ __forceinline__ cdf operator*(df s, cdf a) { return cdf_mk(df_mul(s, a.re), df_mul(s, a.im)); }
static __device__ FT_BIGFN cdf cdf_inv(cdf a)
{
    const df m = df_inv(df_fma(a.re, a.re, df_mul(a.im, a.im)));
    return cdf_mk(df_mul(a.re, m), df_neg(df_mul(a.im, m)));
}
// a b + c with four two-float FMAs
static __device__ FT_CXFN cdf cdf_fma(cdf a, cdf b, cdf c)
{
    return cdf_mk(df_fma(a.re, b.re, df_fma(df_neg(a.im), b.im, c.re)), df_fma(a.re, b.im, df_fma(a.im, b.re, c.im)));
}
// z 2^-k for the exponent k of z's larger part (exact), the exponent added to k_acc;
// false when z is zero or not finite
static __device__ __forceinline__ bool cdf_renorm(cdf& z, int& k_acc)
{
    const float mx = fmaxf(fabsf(z.re.hi), fabsf(z.im.hi));
    const int be = (__float_as_int(mx) >> 23) & 0xff;
    const bool ok = be > 0 && be < 255;
    const int k = ok ? be - 127 : 0;
    const float sc = __int_as_float((127 - k) << 23);
    z.re.hi *= sc;
    z.re.lo *= sc;
    z.im.hi *= sc;
    z.im.lo *= sc;
    k_acc += k;
    return ok;
}

// e^(ix) = cos x + i sin x
static __device__ FT_BIGFN cdf expi_df(df x)
{
    const float P1 = 0x1.921fb6p-5f, P2 = -0x1.777a5cp-30f, P3 = -0x1.ee59dap-55f;
    const float k = rintf((x.hi + x.lo) * 0x1.45f306p+4f);
    const float p1 = k * P1, e1 = fmaf(k, P1, -p1);
    const float p2 = k * P2, e2 = fmaf(k, P2, -p2);
    df r = df_add(x, df_norm(-p1, -e1));
    r = df_add(r, df_norm(-p2, -e2));
    r = df_add(r, df_mk(-k * P3));
    const float rh = r.hi, r2 = rh * rh;
    // sin r = r + rh^3 (-1/6 + rh^2/120)
    const df sr = df_add(r, df_mk(rh * r2 * fmaf(r2, 0x1.111112p-7f, -0x1.555556p-3f)));
    // cos r = 1 - (rh^2 + 2 rh r.lo)/2 + rh^4/24 - rh^6/720, with rh^2 = r2 + qe exactly
    const float qe = fmaf(rh, rh, -r2);
    const df cr = df_add(df_norm(1.0f, -0.5f * r2),
                         df_mk(fmaf(-rh, r.lo, -0.5f * qe) + r2 * r2 * fmaf(r2, -0x1.6c16c2p-10f, 0x1.555556p-5f)));
    const float4 t = FT_SCTAB[((int)k) & 127];
    df sa, ca;
    sa.hi = t.x;
    sa.lo = t.y;
    ca.hi = t.z;
    ca.lo = t.w;
    return cdf_mk(df_fma(ca, cr, df_neg(df_mul(sa, sr))), df_fma(sa, cr, df_mul(ca, sr)));
}

// The deformed Laplacian at the sample (srcs/feynman_integral.hpp:293-310) and V there
// (:322-336) in two-float complex arithmetic, for every deformed sample: in FP32 both
// suffer cancellation (the spanning-tree sum with phases, the quadratic forms against
// the mass terms), and their errors enter the integrand as D/2 arg psi and W arg V.
// Conductances y_e = e^(-i theta_e) / X_e from the two-float contour and sector point,
// the conductance-form elimination of `elim`, the product of its pivots (rescaled by
// powers of two as it goes: det L(y) = det * 2^det_e) and
// V = -sum_jk P~_jk (L(y)^-1)_jk + sum_e m2_e X_e e^(i theta_e) (the reference's
// -sum_r sigma_r q_r^T L^-1 q_r, contracted with P~ itself here).
// deformed integrand, the two-float complex block (det L(y) and V): smallest accepted
// pivot-to-row ratio, smallest |V| relative to the sum of its terms' magnitudes, and
// largest W qmag / |V| (qmag: the magnitudes of every term summed into V, through the
// row quadratic forms).  Two-float arithmetic keeps ~1e-14 of these magnitudes and
// the sector point and contour it starts from ~1e-12, so the bounds only catch samples
// whose cancellation would amplify that to ~1e-7.
#ifndef ACC_GROWTH
#define ACC_GROWTH 1e-5f
#endif
#ifndef ACC_V_CANCEL
#define ACC_V_CANCEL 1e-6f
#endif
#ifndef ACC_V_AMPLIFY
#define ACC_V_AMPLIFY 1e5f
#endif
struct cblock {
    cdf V;
    cdf det;
    int det_e;
    bool ok;       // pivots and the determinant finite and non-zero
    bool growth_ok;  // every pivot above ACC_GROWTH of its row's size
    float mag;     // sum of the magnitudes of V's terms: masses, and one term per external row
    float qmag;    // the same through the row quadratic forms: sum_i |1/d_i| sum_jk |P~_jk| |U_ij| |U_ik| + mag
};
static __device__ __forceinline__ float cmag_hi(const cdf& z) { return fabsf(z.re.hi) + fabsf(z.im.hi); }

static __device__ __forceinline__ void complex_block(const df* theta, const f2* Xi2, const float* pd, cblock& o)
{
    auto pdf = [&](int i) -> df {
        df v;
        v.hi = pd[2 * i];
        v.lo = pd[2 * i + 1];
        return v;
    };
    cdf c[FT_N][FT_N], g[FT_N];
#pragma unroll
    for (int i = 0; i < FT_N; i++) {
        g[i] = cdf_zero();
#pragma unroll
        for (int j = 0; j < FT_N; j++) c[i][j] = cdf_zero();
    }
    cdf v = cdf_zero();
    float mag = 0.0f;
#pragma unroll
    for (int e = 0; e < FT_E; e++) {
        const cdf eix = expi_df(theta[e]);
        const df cs = eix.re, sn = eix.im;
        const df xi = df_of(Xi2[e]);
        const cdf y = cdf_mk(df_mul(xi, cs), df_neg(df_mul(xi, sn)));
        const int k = FT_EK[e], l = FT_EL[e];
        cdf& slot = (k == FT_V - 1) ? g[l] : c[l][k];
        slot = first_in_slot(e) ? y : slot + y;
        const df m2x = df_mul(pdf(P_M2 + e), df_inv(xi));
        const cdf mt = cdf_mk(df_mul(m2x, cs), df_mul(m2x, sn));
        v = e == 0 ? mt : v + mt;
        mag += fabsf(m2x.hi);
    }
    cdf a[FT_N][FT_N], dinv[FT_N];
    cdf det = cdf_mk(df_mk(1.0f), df_mk(0.0f));
    int det_e = 0;
    bool ok = true;
    bool growth_ok = true;
#pragma unroll
    for (int k = 0; k < FT_N; k++) {
        cdf dk = g[k];
        float row = cmag_hi(g[k]);
#pragma unroll
        for (int j = k + 1; j < FT_N; j++) {
            if (!NZC(k, j)) continue;
            dk = dk + c[k][j];
            row += cmag_hi(c[k][j]);
        }
        growth_ok &= cmag_hi(dk) > ACC_GROWTH * row;
        det = det * dk;
        ok &= cdf_renorm(det, det_e);
        dinv[k] = cdf_inv(dk);
#pragma unroll
        for (int i = k + 1; i < FT_N; i++)
            if (NZC(k, i)) a[k][i] = c[k][i] * dinv[k];
#pragma unroll
        for (int i = k + 1; i < FT_N; i++) {
            if (!NZC(k, i)) continue;
            if (NZG(k)) g[i] = cdf_fma(a[k][i], g[k], g[i]);
#pragma unroll
            for (int j = i + 1; j < FT_N; j++)
                if (NZC(k, j)) c[i][j] = cdf_fma(a[k][i], c[k][j], c[i][j]);
        }
    }
    // The momentum part, sum_jk P~_jk (L(y)^-1)_jk over the external rows [Q0, N) (P~
    // vanishes elsewhere).  The forward substitution is y = U q with U unit lower
    // triangular, U_ij = sum_{j <= k < i} a_ki U_kj, so L^-1 = U^T diag(1/d) U there and
    // the part is sum_i (u_i^T P~ u_i) / d_i, u_i the i-th row of U: one quadratic form of
    // P~ per row instead of one forward substitution per term of its low-rank split.
    float qmag = 0.0f;
#if FT_NE > 0
    {
        auto ptd = [&](int j, int k) -> df { return pdf(PT_AT(j, k)); };
        cdf U[FT_NE][FT_NE];   // U[i][j], j < i (indices from Q0)
        cdf vq = cdf_zero();
#pragma unroll
        for (int ii = 0; ii < FT_NE; ii++) {
            const int i = FT_Q0 + ii;
#pragma unroll
            for (int jj = 0; jj < ii; jj++) {
                const int j = FT_Q0 + jj;
                cdf u = cdf_zero();
                bool any = false;
                if (NZC(j, i)) {
                    u = a[j][i];
                    any = true;
                }
#pragma unroll
                for (int kk = jj + 1; kk < ii; kk++) {
                    const int k = FT_Q0 + kk;
                    if (!NZC(k, i)) continue;
                    u = any ? cdf_fma(a[k][i], U[kk][jj], u) : a[k][i] * U[kk][jj];
                    any = true;
                }
                U[ii][jj] = u;
            }
            // Q = u^T P~ u with u = (U_i0 .. U_i,i-1, 1): Q = P_ii + sum_j u_j w_j,
            // w_j = sum_{j <= k < i} P_jk u_k + P_ji (off-diagonal P doubled)
            cdf Q = cdf_mk(ptd(ii, ii), df_mk(0.0f));
            float qm = fabsf(ptd(ii, ii).hi);
#pragma unroll
            for (int jj = 0; jj < ii; jj++) {
                cdf w = ptd(jj, jj) * U[ii][jj];
                float wm = fabsf(ptd(jj, jj).hi) * cmag_hi(U[ii][jj]);
#pragma unroll
                for (int kk = jj + 1; kk < ii; kk++) {
                    w = w + ptd(jj, kk) * U[ii][kk];
                    wm += fabsf(ptd(jj, kk).hi) * cmag_hi(U[ii][kk]);
                }
                w.re = df_add(w.re, ptd(jj, ii));
                wm += fabsf(ptd(jj, ii).hi);
                Q = cdf_fma(U[ii][jj], w, Q);
                qm += cmag_hi(U[ii][jj]) * wm;
            }
            const cdf t = Q * dinv[i];
            vq = ii == 0 ? t : vq + t;
            mag += cmag_hi(t);
            qmag += qm * cmag_hi(dinv[i]);
        }
        v = v - vq;
    }
#endif
    o.V = v;
    o.det = det;
    o.det_e = det_e;
    o.ok = ok;
    o.growth_ok = growth_ok;
    o.mag = mag;
    o.qmag = qmag + mag;
}

// x-derivatives of phi/psi at the sample point (srcs/laplacian.hpp:102-215) and the
// deformation angle theta = -lambda (d(phi/psi)/dx + m^2) (srcs/feynman_integral.hpp:290-291).
// Everything here is a difference of entries of L^-1, which cancels in FP32 for a
// sizeable fraction of sectors, so the block runs in two-float arithmetic: the
// conductance-form elimination (all operations on positive values), G = L^-1, the
// potentials h_r = G q_r and their drops across the edges, the effective-resistance
// combinations t, and the Minkowski products s.  Outputs theta and the upper
// triangle of H in FP32.  pd: the parameter block as two-float pairs.
static __device__ __forceinline__ void derivatives_df(const float* Xi32, const f2* XiT, const float* pd, df* theta_out,
                                                      float (*H_out)[FT_E], bool& cancel)
{
    df c[FT_N][FT_N], g[FT_N];
#pragma unroll
    for (int i = 0; i < FT_N; i++) {
        g[i] = df_mk(0.0f);
#pragma unroll
        for (int j = 0; j < FT_N; j++) c[i][j] = df_mk(0.0f);
    }
#pragma unroll
    for (int e = 0; e < FT_E; e++) {
        const int k = FT_EK[e], l = FT_EL[e];
        df& slot = (k == FT_V - 1) ? g[l] : c[l][k];
        slot = first_in_slot(e) ? df_of(XiT[e]) : df_add(slot, df_of(XiT[e]));
    }
    df a[FT_N][FT_N], id[FT_N];
#pragma unroll
    for (int k = 0; k < FT_N; k++) {
        df dk = g[k];
#pragma unroll
        for (int j = k + 1; j < FT_N; j++)
            if (NZC(k, j)) dk = df_add(dk, c[k][j]);
        id[k] = df_inv(dk);
#pragma unroll
        for (int i = k + 1; i < FT_N; i++)
            if (NZC(k, i)) a[k][i] = df_mul(c[k][i], id[k]);
#pragma unroll
        for (int i = k + 1; i < FT_N; i++) {
            if (!NZC(k, i)) continue;
            if (NZG(k)) g[i] = df_fma(a[k][i], g[k], g[i]);
#pragma unroll
            for (int j = i + 1; j < FT_N; j++)
                if (NZC(k, j)) c[i][j] = df_fma(a[k][i], c[k][j], c[i][j]);
        }
    }
    // N = M^-1 (unit upper triangular, non-negative), G = N diag(1/d) N^T
    df Nm[FT_N][FT_N];
#pragma unroll
    for (int i = FT_N - 1; i >= 0; i--) {
#pragma unroll
        for (int j = i + 1; j < FT_N; j++) {
            if (!NZM(i, j)) continue;
            df s = NZC(i, j) ? a[i][j] : df_mk(0.0f);
            bool any = NZC(i, j);
#pragma unroll
            for (int k = i + 1; k < j; k++)
                if (NZC(i, k) && NZM(k, j)) {
                    s = any ? df_fma(a[i][k], Nm[k][j], s) : df_mul(a[i][k], Nm[k][j]);
                    any = true;
                }
            Nm[i][j] = s;
        }
    }
    // Nd[j][k] = N[j][k] / d_k, so that each term of G is one two-float multiply-add
    df Nd[FT_N][FT_N];
#pragma unroll
    for (int j = 0; j < FT_N; j++)
#pragma unroll
        for (int k = j + 1; k < FT_N; k++)
            if (NZM(j, k)) Nd[j][k] = df_mul(Nm[j][k], id[k]);
    df G[FT_N][FT_N];
#pragma unroll
    for (int i = 0; i < FT_N; i++)
#pragma unroll
        for (int j = i; j < FT_N; j++) {
            // k = j term has N[j][j] = 1
            df s = (i == j) ? id[j] : (NZM(i, j) ? Nd[i][j] : df_mk(0.0f));
#pragma unroll
            for (int k = j + 1; k < FT_N; k++)
                if (NZM(i, k) && NZM(j, k)) s = df_fma(Nm[i][k], Nd[j][k], s);
            G[i][j] = s;
            G[j][i] = s;
        }
    df hb[FT_RANK][FT_E];
#pragma unroll
    for (int r = 0; r < FT_RANK; r++) {
        df h[FT_N];
#pragma unroll
        for (int i = 0; i < FT_N; i++) {
            df s = df_mk(0.0f);
#pragma unroll
            for (int j = FT_Q0; j < FT_N; j++) {
                df q;
                q.hi = pd[2 * (P_Q + r * FT_N + j)];
                q.lo = pd[2 * (P_Q + r * FT_N + j) + 1];
                s = j == FT_Q0 ? df_mul(G[i][j], q) : df_fma(G[i][j], q, s);
            }
            h[i] = s;
        }
#pragma unroll
        for (int e = 0; e < FT_E; e++) {
            const int k = FT_EK[e], l = FT_EL[e];
            hb[r][e] = (k == FT_V - 1) ? df_neg(h[l]) : df_sub(h[k], h[l]);
        }
    }
    auto Gx = [&](int i, int j) -> df { return (i == FT_V - 1 || j == FT_V - 1) ? df_mk(0.0f) : G[i][j]; };
    df kappa;
    kappa.hi = pd[2 * P_DEF];
    kappa.lo = pd[2 * P_DEF + 1];
#pragma unroll
    for (int a2 = 0; a2 < FT_E; a2++) {
        const int ka = FT_EK[a2], la = FT_EL[a2];
        // w = row a2 of (edge incidence) L^-1, w_v = G_{ka v} - G_{la v} (the ground's row of
        // L^-1 is zero): edge a2's resistance combination with any edge (k, l),
        // G_ka,k + G_la,l - G_ka,l - G_la,k, is then w_k - w_l.  The entries no edge
        // pair reads are dropped at compile time.
        df w[FT_N];
#pragma unroll
        for (int v = 0; v < FT_N; v++)
            w[v] = ka == FT_V - 1 ? df_neg(G[la][v]) : (la == FT_V - 1 ? G[ka][v] : df_sub(G[ka][v], G[la][v]));
        auto wd = [&](int k, int l) -> df {
            return k == FT_V - 1 ? df_neg(w[l]) : (l == FT_V - 1 ? w[k] : df_sub(w[k], w[l]));
        };
        df sig_hb[FT_RANK];
        df s = df_mk(0.0f);
#pragma unroll
        for (int r = 0; r < FT_RANK; r++) {
            df sg;
            sg.hi = pd[2 * (P_SIG + r)];
            sg.lo = pd[2 * (P_SIG + r) + 1];
            sig_hb[r] = df_mul(sg, hb[r][a2]);
            s = r == 0 ? df_mul(sig_hb[r], hb[r][a2]) : df_fma(sig_hb[r], hb[r][a2], s);
        }
        const df t = wd(ka, la);
        // an edge whose ends float together: the FP64 pass takes the sample
        cancel |= ka != FT_V - 1 && !(df_f(t) > 1e-7f * (df_f(Gx(ka, ka)) + df_f(Gx(la, la))));
        const df xi = df_of(XiT[a2]);
        const df xa = df_mul(xi, xi);
        const df xas = df_mul(xa, s);
        df m2;
        m2.hi = pd[2 * (P_M2 + a2)];
        m2.lo = pd[2 * (P_M2 + a2) + 1];
        theta_out[a2] = df_mul(df_sub(m2, xas), kappa);
        // 2 xa s (1/x - xa t)
        H_out[a2][a2] = 2.0f * df_f(df_mul(xas, df_sub(xi, df_mul(xa, t))));
        // the off-diagonal entries are FP32 products of their (two-float) factors
        const float xaf = df_f(xa);
#pragma unroll
        for (int b = a2 + 1; b < FT_E; b++) {
            const int kb = FT_EK[b], lb = FT_EL[b];
            df s2 = df_mk(0.0f);
#pragma unroll
            for (int r = 0; r < FT_RANK; r++) s2 = r == 0 ? df_mul(sig_hb[r], hb[r][b]) : df_fma(sig_hb[r], hb[r][b], s2);
            const df t2 = wd(kb, lb);
            const float xb = Xi32[b];
            H_out[a2][b] = -2.0f * (xaf * (xb * xb)) * df_f(s2) * df_f(t2);
        }
    }
}
#endif

// positive value m * 2^e with m in [1, 2): products of many pivots and X values
// without overflow, and logarithms split into an exact integer and a small part
struct mexp {
    float m;
    int e;
    bool bad;
};
static __device__ __forceinline__ void mx_mul(mexp& a, float x)
{
    const float p = a.m * x;
    const int b = __float_as_int(p);
    const int be = (b >> 23) & 0xff;
    a.bad |= (be == 0) | (be == 255) | (b < 0);
    a.e += be - 127;
    a.m = __int_as_float((b & 0x007fffff) | 0x3f800000);
}
static __device__ __forceinline__ mexp mx_one()
{
    mexp r;
    r.m = 1.0f;
    r.e = 0;
    r.bad = false;
    return r;
}
static __device__ __forceinline__ f2 f2_make(float h, float l)
{
    f2 r;
    r.hi = h;
    r.lo = l;
    return r;
}
static __device__ __forceinline__ f2 f2_mulf(f2 a, float b)
{
    const float p = a.hi * b;
    const float e = fmaf(a.hi, b, -p) + a.lo * b;
    const float h = p + e;
    return f2_make(h, e - (h - p));
}
static __device__ __forceinline__ f2 f2_mul2(f2 a, f2 b)
{
    const float p = a.hi * b.hi;
    const float e = fmaf(a.hi, b.hi, -p) + (a.hi * b.lo + a.lo * b.hi);
    const float h = p + e;
    return f2_make(h, e - (h - p));
}
static __device__ __forceinline__ f2 f2_neg(f2 a) { return f2_make(-a.hi, -a.lo); }
// undeformed integrand: relative size of V below which the FP32 evaluation hands the
// sample to FP64
#ifndef V_CANCEL
#define V_CANCEL 0.05f
#endif
// smallest pivot-to-row ratio accepted in the FP32 elimination of the Jacobian
#ifndef PIVOT_GROWTH
#define PIVOT_GROWTH 0.02f
#endif
#define RLN2_HI 1.44269502162933349609375f
#define RLN2_LO 1.925963033500011e-8f
#define LN2_F 0.69314718055994531f

// log2(value / exp(lref)) for value = mx and a natural-log reference lref (two-float)
static __device__ __forceinline__ f2 log2_ratio(const mexp& mx, f2 lref)
{
    f2 r = f2_mul2(lref, f2_make(RLN2_HI, RLN2_LO));
    r = f2_add(f2_neg(r), (float)mx.e);
    return f2_add(r, m_log2(mx.m));
}

// principal argument reduced to (-pi, pi]; `edge` reports a value within 1e-5 of
// the branch cut, where FP32 cannot decide the branch the way the reference does
static __device__ __forceinline__ float wrap_pi(float x, bool& edge)
{
    const float TWO_PI_HI = 6.28318548202514648f, TWO_PI_LO = -1.7484555e-7f;
    const float k = rintf(x * 0.159154943091895336f);
    float r = fmaf(-k, TWO_PI_HI, x);
    r = fmaf(-k, TWO_PI_LO, r);
    edge |= fabsf(r) > 3.14158265f;
    return r;
}

// two-float variant of wrap_pi
static __device__ __forceinline__ f2 wrap_pi2(f2 x, bool& edge)
{
    const float TWO_PI_HI = 6.28318548202514648f, TWO_PI_LO = -1.7484555e-7f;
    const float k = rintf((x.hi + x.lo) * 0.159154943091895336f);
    // k * 2pi as an exact two-float product (k * TWO_PI_HI alone is rounded once |k| > 1)
    const float p = k * TWO_PI_HI;
    f2 r = f2_add(x, -p);
    r = f2_add(r, -fmaf(k, TWO_PI_HI, -p));
    r = f2_add(r, -k * TWO_PI_LO);
    edge |= fabsf(r.hi + r.lo) > 3.14158265f;
    return r;
}

// Principal argument of x + i y in two-float to about 1.5e-7 absolute: atanf of the
// ratio of the smaller to the larger part (a result in [0, pi/4], where an ulp is
// 6e-8), the octant restored with multiples of pi/2 in two-float, plus the first-order
// effect of the low parts, (x dy - y dx) / |z|^2.  Zero gives 0.
static __device__ FT_BIGFN f2 arg_f2(float x, float y, float xl, float yl)
{
    const float PIO2_HI = 1.57079637f, PIO2_LO = -4.37113883e-8f;
    const float ax = fabsf(x), ay = fabsf(y);
    const bool sw = ay > ax;
    const float num = sw ? ax : ay, den = sw ? ay : ax;
    // the ratio through the correctly rounded reciprocal (within 1.5 ulp of num / den)
    const float a = den > 0.0f ? m_atan(num * rcp_(den)) : 0.0f;
    f2 r = sw ? f2_add(f2_make(PIO2_HI, PIO2_LO), -a) : f2_make(a, 0.0f);
    if (x < 0.0f) r = f2_add2(f2_make(2.0f * PIO2_HI, 2.0f * PIO2_LO), f2_neg(r));
    if (y < 0.0f) r = f2_neg(r);
    const float n2 = fmaf(x, x, y * y);
    return n2 > 0.0f ? f2_add(r, (x * yl - y * xl) * rcp_(n2)) : r;
}

// Sets need64 when the FP32 / two-float evaluation cannot be trusted (the sample then
// goes to the FP64 pass); returns false for a dropped (non-finite) sample.
static __device__ __forceinline__ bool integrand32(const float* pd, const float* pf, const f2* lx, f2 lF, f2 lG,
                                                   cx<float>* out, bool& need64)
{
    need64 = false;
    const float D2 = 0.5f * pf[P_D], W = pf[P_W];
    // working frame X_e = exp(lx_e - sh), sh an integer near the middle of the range;
    // R and the eps factor are ratios to the tropical approximants and do not depend on it
    float lmin = 0.0f;
#pragma unroll
    for (int e = 0; e < FT_E; e++) lmin = fminf(lmin, lx[e].hi);
    const float sh = rintf(0.5f * lmin);
    float X[FT_E], Xi[FT_E];
#if FT_MODE == 1
    // 1/X in two-float for the derivative block and the complex Laplacian (theta is a
    // function of X whose phase effect grows with |theta|); X and 1/X in FP32 from it;
    // log prod X (in the frame) in two-float
    f2 Xi2[FT_E];
    f2 sumlx = f2_make(0.0f, 0.0f);
    bool xbad = false;
#pragma unroll
    for (int e = 0; e < FT_E; e++) {
        const f2 a = f2_add(lx[e], -sh);
        sumlx = f2_add2(sumlx, a);
        Xi2[e] = exp_f2(f2_make(-a.hi, -a.lo));
        Xi[e] = Xi2[e].hi;
        X[e] = rcp_(Xi[e]);
        xbad |= !(Xi[e] > 1e-30f && Xi[e] < 1e30f);
    }
    if (xbad) {   // outside the two-float exponential's range: the FP64 pass takes it
        need64 = true;
        return false;
    }
#else
#pragma unroll
    for (int e = 0; e < FT_E; e++) {
        const f2 a = f2_add(lx[e], -sh);
        const float ep = m_exp(a.hi), em = m_exp(-a.hi);
        X[e] = fmaf(ep, a.lo, ep);
        Xi[e] = fmaf(em, -a.lo, em);
    }
#endif
    const f2 lFs = f2_add(lF, -(float)FT_LOOPS * sh);   // log psi_tr in the frame
    const f2 lGs = f2_add(lG, -sh);                      // log V_tr = log(xi_tr / psi_tr)
    const float IGtr = pf[P_IGTR];
#if FT_MODE == 0
    elim<float, float> L;
    L.factor(Xi);
    mexp psi = mx_one();
#pragma unroll
    for (int k = 0; k < FT_N; k++) mx_mul(psi, L.d[k]);
#pragma unroll
    for (int e = 0; e < FT_E; e++) mx_mul(psi, X[e]);
    if (psi.bad) {
        need64 = true;
        return false;
    }
    const f2 lpsi = log2_ratio(psi, lFs);   // log2(psi / psi_tr)
#if FT_ONLY_PSI
    const f2 t = f2_mulf(lpsi, -D2);
    const float R = m_exp2(t.hi) * (1.0f + t.lo * LN2_F);
    out[0] = cmk(IGtr * R, 0.0f);
    return true;
#else
    float pphi = 0.0f, mag = 0.0f;
#pragma unroll
    for (int r = 0; r < FT_RANK; r++) {
        const float v = pf[P_SIG + r] * L.quad(pf + P_Q + r * FT_N);
        pphi -= v;
        mag += fabsf(v);
    }
    float pxi = pphi;
#pragma unroll
    for (int e = 0; e < FT_E; e++) {
        const float v = pf[P_M2 + e] * X[e];
        pxi += v;
        mag += fabsf(v);
    }
    if (!(pxi > V_CANCEL * mag)) {   // cancellation, or a sign the FP64 pass must decide
        need64 = true;
        return false;
    }
    mexp V = mx_one();
    mx_mul(V, pxi);
    const f2 lv = log2_ratio(V, lGs);   // log2(V / V_tr)
    const f2 t = f2_add2(f2_mulf(lpsi, -D2), f2_mulf(lv, -W));
    const float Rf = m_exp2(t.hi) * (1.0f + t.lo * LN2_F);
    if (!isfinite(Rf) || V.bad) {
        need64 = true;
        return false;
    }
    float R = IGtr * Rf;
    out[0] = cmk(R, 0.0f);
    if (FT_K > 1) {
        const float ef = LN2_F * ((float)(psi.e - FT_LOOPS * V.e) + (m_log2(psi.m) - (float)FT_LOOPS * m_log2(V.m)));
#pragma unroll
        for (int j = 1; j < FT_K; j++) {
            R *= ef * (1.0f / (float)j);
            out[j] = cmk(R, 0.0f);
        }
    }
    return true;
#endif
#else
    const float kappa = pf[P_DEF];
    // The contour (theta) and its Jacobian come from differences of entries of L^-1,
    // which cancel in FP32 for a sizeable fraction of sectors; this block runs in two-float.
    df theta[FT_E];
    float H[FT_E][FT_E];
    bool cancel = false;
    derivatives_df(Xi, Xi2, pd, theta, H, cancel);
    if (cancel) {
        need64 = true;
        return false;
    }
    // det(I + i kappa X^1/2 H X^1/2) (similar to I + i kappa H X, srcs/feynman_integral.hpp:312-320):
    // the real part is the identity, so the symmetric elimination needs no pivoting; FP32,
    // the pivots' product rescaled by powers of two (det J = pj 2^pj_e).  Before the complex
    // block, so that H is no longer live there.
    cx<float> pj = cmk(1.0f, 0.0f);
    int pj_e = 0;
    bool jok = true;   // pivots above PIVOT_GROWTH of their rows, scaled product finite
    {
        cx<float> J[FT_E][FT_E];
        float sx[FT_E];
#pragma unroll
        for (int e = 0; e < FT_E; e++) sx[e] = sqrtf(X[e]);
#pragma unroll
        for (int a = 0; a < FT_E; a++)
#pragma unroll
            for (int b = a; b < FT_E; b++) J[a][b] = cmk(a == b ? 1.0f : 0.0f, kappa * H[a][b] * sx[a] * sx[b]);
#pragma unroll
        for (int k = 0; k < FT_E; k++) {
            const cx<float> piv = J[k][k];
            const float m = fabsf(piv.re) + fabsf(piv.im);
            float row = m;
#pragma unroll
            for (int j = k + 1; j < FT_E; j++) row += fabsf(J[k][j].re) + fabsf(J[k][j].im);
            jok &= m > PIVOT_GROWTH * row;
            pj = pj * piv;
            {
                const float mx = fmaxf(fabsf(pj.re), fabsf(pj.im));
                const int be = (__float_as_int(mx) >> 23) & 0xff;
                jok &= be > 0 && be < 255;
                const int kk = (be > 0 && be < 255) ? be - 127 : 0;
                const float sc = __int_as_float((127 - kk) << 23);
                pj = cmk(pj.re * sc, pj.im * sc);
                pj_e += kk;
            }
            const cx<float> inv = crecip(piv);
#pragma unroll
            for (int i = k + 1; i < FT_E; i++) {
                const cx<float> f = J[k][i] * inv;
#pragma unroll
                for (int j = i; j < FT_E; j++) J[i][j] = J[i][j] - f * J[k][j];
            }
        }
    }
    if (!jok) {
        need64 = true;
        return false;
    }
    // phase sums in two-float: sum theta and nu . theta
    f2 xnu = f2_make(0.0f, 0.0f), thsum = f2_make(0.0f, 0.0f);
#pragma unroll
    for (int e = 0; e < FT_E; e++) {
        FT_DBG(e, theta[e].hi + theta[e].lo);
        thsum = f2_add2(thsum, f2_make(theta[e].hi, theta[e].lo));
        xnu = f2_add2(xnu, f2_mulf(f2_make(theta[e].hi, theta[e].lo), pf[P_NU + e]));
    }
    cblock cb;
    complex_block(theta, Xi2, pd, cb);
    // two-float pivots lose ~1e-14 / growth
    if (!cb.ok || !cb.growth_ok) {
        need64 = true;
        return false;
    }
    // V = Vn 2^v_e, |Vn| in [1, 2 sqrt 2)
    cdf Vn = cb.V;
    int v_e = 0;
    if (!cdf_renorm(Vn, v_e) || v_e > 126) {
        need64 = true;
        return false;
    }
    const float vsc = __int_as_float((127 - v_e) << 23);   // 2^-v_e
    const float vn2 = fmaf(Vn.re.hi, Vn.re.hi, Vn.im.hi * Vn.im.hi);
    const float vm = sqrtf(vn2);
    FT_DBG(20, Vn.re.hi);
    FT_DBG(21, Vn.im.hi);
    FT_DBG(34, W * cb.qmag * vsc / vm);
    // V in two-float keeps ~1e-14 of its terms' magnitudes (and ~1e-12 from the sector
    // point and contour it is built from): samples where V cancels to below 1e-6 of its
    // terms, or where W qmag / |V| exceeds 1e5, go to the FP64 pass
    if (!(vm > ACC_V_CANCEL * (cb.mag * vsc)) || !(W * (cb.qmag * vsc) < ACC_V_AMPLIFY * vm)) {
        need64 = true;
        return false;
    }
    bool edge = false;
    const f2 av2 = arg_f2(Vn.re.hi, Vn.im.hi, Vn.re.lo, Vn.im.lo);
    const float av = av2.hi + av2.lo;
    edge |= fabsf(av) > 3.14158265f;
    FT_DBG(32, av);
    FT_DBG(33, xnu.hi + xnu.lo);
    // arg cPsi = sum theta + arg det L(y), reduced to the principal branch in two-float
    const float dn2 = fmaf(cb.det.re.hi, cb.det.re.hi, cb.det.im.hi * cb.det.im.hi);
    const f2 apsi2 = wrap_pi2(f2_add2(thsum, arg_f2(cb.det.re.hi, cb.det.im.hi, cb.det.re.lo, cb.det.im.lo)), edge);
    const float apsi = apsi2.hi + apsi2.lo;
    FT_DBG(26, apsi);
    if (edge) {
        need64 = true;
        return false;
    }
    // log2 |cPsi| and log2 |V| (exponents exact, small parts in FP32), then
    // log2 |cR / IGtr| = -D/2 log2(|cPsi| / psi_tr) - W log2(|V| / V_tr) + log2 |det J|
    const float l2dm = 0.5f * m_log2(dn2), l2vm = 0.5f * m_log2(vn2);
    const f2 l2psi_abs = f2_add(f2_add(f2_mul2(sumlx, f2_make(RLN2_HI, RLN2_LO)), (float)cb.det_e), l2dm);
    const f2 lpsi = f2_add2(l2psi_abs, f2_neg(f2_mul2(lFs, f2_make(RLN2_HI, RLN2_LO))));
    const f2 l2v_abs = f2_add(f2_make((float)v_e, 0.0f), l2vm);
    const f2 lv = f2_add2(l2v_abs, f2_neg(f2_mul2(lGs, f2_make(RLN2_HI, RLN2_LO))));
    f2 t = f2_add2(f2_mulf(lpsi, -D2), f2_mulf(lv, -W));
    t = f2_add(t, (float)pj_e);
    t = f2_add(t, 0.5f * m_log2(fmaf(pj.re, pj.re, pj.im * pj.im)));
    // arg cR = -D/2 arg cPsi + arg det J + nu . theta - W arg V (two-float sum)
    f2 angf = f2_add2(f2_mulf(apsi2, -D2), xnu);
    angf = f2_add2(angf, arg_f2(pj.re, pj.im, 0.0f, 0.0f));
    angf = f2_add2(angf, f2_mulf(av2, -W));
    const float ang = angf.hi;
    const float mod = m_exp2(t.hi) * (1.0f + t.lo * LN2_F);
    float sn, cs;
    m_sincos(ang, &sn, &cs);
    {
        const float c2 = fmaf(-angf.lo, sn, cs), s2 = fmaf(angf.lo, cs, sn);
        cs = c2;
        sn = s2;
    }
    if (!isfinite(mod)) {
        need64 = true;
        return false;
    }
    cx<float> c = cmk(IGtr * mod * cs, IGtr * mod * sn);
    out[0] = c;
    if (FT_K > 1) {
        // log cPsi - L log V (srcs/feynman_integral.hpp:336-341): the large parts in two-float
        const f2 dl = f2_add2(l2psi_abs, f2_mulf(l2v_abs, -(float)FT_LOOPS));
        const float er = LN2_F * (dl.hi + dl.lo);
        const float ei = apsi - (float)FT_LOOPS * av;
#pragma unroll
        for (int j = 1; j < FT_K; j++) {
            c = c * cmk(er * (1.0f / (float)j), ei * (1.0f / (float)j));
            out[j] = c;
        }
    }
    return true;
#endif
}
#endif

#ifndef FT_HOST_SIM
// ------------------------------------------------------------------ accumulation
// Neumaier-compensated running sums per thread
struct nsum {
    double s, c;
    __device__ __forceinline__ void add(double v)
    {
        double t = s + v;
        c += (fabs(s) >= fabs(v)) ? ((s - t) + v) : ((v - t) + s);
        s = t;
    }
};

// double-double sum of two (hi, lo) pairs
static __device__ __forceinline__ void dd_add(double& ah, double& al, double bh, double bl)
{
    double s = ah + bh;
    double bb = s - ah;
    double err = (ah - (s - bb)) + (bh - bb);
    err += al + bl;
    ah = s + err;
    al = err - (ah - s);
}

// Block reduction of per-thread (hi, lo) accumulators into o[0 .. ACC_SLOTS)
static __device__ __noinline__ void block_reduce(double* vals /* ACC_SLOTS per thread, (hi,lo) pairs for the first 8K */,
                                                 double* o)
{
    // runs once per thread at the end: kept as loops (small code), not unrolled
    __shared__ double red[FT_BLOCK / 32][ACC_SLOTS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll 1
    for (int s = 0; s < 8 * FT_K; s += 2) {
        double h = vals[s], l = vals[s + 1];
#pragma unroll 1
        for (int off = 16; off; off >>= 1) {
            double oh = __shfl_down_sync(0xffffffffu, h, off), ol = __shfl_down_sync(0xffffffffu, l, off);
            dd_add(h, l, oh, ol);
        }
        if (lane == 0) {
            red[wid][s] = h;
            red[wid][s + 1] = l;
        }
    }
#pragma unroll 1
    for (int s = 8 * FT_K; s < ACC_SLOTS; s++) {
        double v = vals[s];
#pragma unroll 1
        for (int off = 16; off; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) red[wid][s] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll 1
        for (int s = 0; s < 8 * FT_K; s += 2) {
            double h = red[0][s], l = red[0][s + 1];
#pragma unroll 1
            for (int w = 1; w < FT_BLOCK / 32; w++) dd_add(h, l, red[w][s], red[w][s + 1]);
            o[s] = h;
            o[s + 1] = l;
        }
#pragma unroll 1
        for (int s = 8 * FT_K; s < ACC_SLOTS; s++) {
            double v = 0.0;
#pragma unroll 1
            for (int w = 0; w < FT_BLOCK / 32; w++) v += red[w][s];
            o[s] = v;
        }
    }
}

// stream state from 4 words (16-byte aligned)
static __device__ __forceinline__ xo load_state(const u64* __restrict__ s)
{
    const ulonglong2 a = *(const ulonglong2*)s, b = *(const ulonglong2*)(s + 2);
    xo g;
    g.a = a.x;
    g.b = a.y;
    g.c = b.x;
    g.d = b.y;
    return g;
}

// ------------------------------------------------------------------ lane start states
// state <- P_b state for every set bit b of `lane`, with P_b = (T^S)^(2^b) supplied by
// the host (S = draws per lane).  The loop is uniform across the warp so that the
// matrix columns are broadcast loads.
static __device__ __forceinline__ void skip_lanes(xo& g, u32 lane, const u64* __restrict__ pw, int nbits)
{
    for (int b = 0; b < nbits; b++) {
        const bool mine = (lane >> b) & 1u;
        if (!__any_sync(0xffffffffu, mine)) continue;
        const ulonglong2* M = (const ulonglong2*)(pw + (size_t)b * 1024);
        u64 r0 = 0, r1 = 0, r2 = 0, r3 = 0;
        const u64 sv[4] = {g.a, g.b, g.c, g.d};
#pragma unroll 4
        for (int c = 0; c < 256; c++) {
            const u64 mask = 0ull - ((sv[c >> 6] >> (c & 63)) & 1ull);
            const ulonglong2 lo = __ldg(M + 2 * c), hi = __ldg(M + 2 * c + 1);
            r0 ^= lo.x & mask;
            r1 ^= lo.y & mask;
            r2 ^= hi.x & mask;
            r3 ^= hi.y & mask;
        }
        if (mine) {
            g.a = r0;
            g.b = r1;
            g.c = r2;
            g.d = r3;
        }
    }
}

// ------------------------------------------------------------------ table staging
// FP64 form: shared = [w64 | Jr64 | 1/r64 | meta] (25 bytes per entry, the global
// layout's first sections).  Mixed form: shared = [w32 | Jr32 | 1/r32 | meta].
#if FT_TABLE_GLOBAL
#define SM_USED 0u
#elif FT_PREC == 0
#define SM_USED (25u * T_ENTRIES)
#else
#define SM_USED (17u * T_ENTRIES)
#endif
static __device__ __forceinline__ void copy_bytes(unsigned char* dst, const unsigned char* __restrict__ src, u32 bytes)
{
    const u32 n16 = bytes / 16u;
    for (u32 i = threadIdx.x; i < n16; i += blockDim.x) ((uint4*)dst)[i] = ((const uint4*)src)[i];
    for (u32 i = n16 * 16u + threadIdx.x; i < bytes; i += blockDim.x) dst[i] = src[i];
}

// the table's sections: in global memory (large tables, L2 / L1 cached) or the staged
// copy in shared memory
static __device__ __forceinline__ table_ref table_at(unsigned char* sm, const unsigned char* __restrict__ tab)
{
    table_ref t;
    t.gm = tab;
#if FT_TABLE_GLOBAL
    (void)sm;
#if FT_PREC == 0
    t.w = tab + T_W64;
    t.Jr = tab + T_JR64;
    t.ri = tab + T_RI64;
#else
    t.w = tab + T_W32;
    t.Jr = tab + T_JR32;
    t.ri = tab + T_RI32;
#endif
    t.meta = tab + T_META;
#elif FT_PREC == 0
    t.w = sm + T_W64;
    t.Jr = sm + T_JR64;
    t.ri = sm + T_RI64;
    t.meta = sm + T_META;
#else
    t.w = sm;
    t.Jr = sm + 4u * T_ENTRIES;
    t.ri = sm + 8u * T_ENTRIES;
    t.meta = sm + 16u * T_ENTRIES;
#endif
    return t;
}

// the block's copy of a staged table (no barrier)
static __device__ __forceinline__ void copy_table(unsigned char* sm, const unsigned char* __restrict__ tab)
{
#if FT_TABLE_GLOBAL
    (void)sm;
    (void)tab;
#elif FT_PREC == 0
    copy_bytes(sm, tab, 25u * T_ENTRIES);
#else
    copy_bytes(sm, tab + T_F32, 16u * T_ENTRIES);
    copy_bytes(sm + 16u * T_ENTRIES, tab + T_META, T_ENTRIES);
#endif
}

static __device__ __forceinline__ table_ref stage_table(unsigned char* sm, const unsigned char* __restrict__ tab)
{
    copy_table(sm, tab);
#if !FT_TABLE_GLOBAL
    __syncthreads();
#endif
    return table_at(sm, tab);
}

// ------------------------------------------------------------------ per-thread accumulators
// Per-thread sums live in shared memory (slot-major, so a warp touches consecutive
// words), which keeps them out of the register budget of the sampling code:
//   FP64 form: Neumaier-compensated FP64 sums per sample.
//   mixed form: Kahan-compensated FP32 sums per sample, folded into the FP64
//   Neumaier sums every 256 kept samples; the sample counters too (FP32 counts since
//   the last fold, FP64 totals), so that no accumulator state is held in registers
//   across the per-sample code.
// Slots: 4 per eps order (re f, re f^2, im f, im f^2).
#if FT_MODE == 0
#define ACC_PARTS 2   // undeformed integrand: real parts only
#else
#define ACC_PARTS 4
#endif
#define ACC_NS (ACC_PARTS * FT_K)
#define ACC_SMEM_OFFSET ((SM_USED + 15u) & ~15u)
// mixed form, counters: kept, dropped, queued, exact
#define ACC_NC 4

#if FT_PREC == 0
struct accum {
    double* S;   // [slot][thread] sums
    double* C;   // [slot][thread] Neumaier compensations
    double kept, dropped, queued, exact, robust;

    __device__ __forceinline__ void init(unsigned char* smem_acc)
    {
        const int t = threadIdx.x;
        S = (double*)smem_acc + t;
        C = S + ACC_NS * FT_BLOCK;
#pragma unroll
        for (int s = 0; s < ACC_NS; s++) {
            S[s * FT_BLOCK] = 0.0;
            C[s * FT_BLOCK] = 0.0;
        }
        kept = dropped = queued = exact = robust = 0.0;
    }

    __device__ __forceinline__ void nadd(int slot, double v)
    {
        const double s = S[slot * FT_BLOCK];
        const double t = s + v;
        C[slot * FT_BLOCK] += (fabs(s) >= fabs(v)) ? ((s - t) + v) : ((v - t) + s);
        S[slot * FT_BLOCK] = t;
    }

    __device__ __forceinline__ void add64(const cx<double>* R)
    {
        kept += 1;
#pragma unroll
        for (int j = 0; j < FT_K; j++) {
            if (FT_ONLY_PSI && j > 0) break;
            nadd(ACC_PARTS * j + 0, R[j].re);
            nadd(ACC_PARTS * j + 1, R[j].re * R[j].re);
            if (ACC_PARTS == 4) {
                nadd(ACC_PARTS * j + 2, R[j].im);
                nadd(ACC_PARTS * j + 3, R[j].im * R[j].im);
            }
        }
    }

    // block-wide: every thread of the block calls it; the block's sums go to dst[0 .. ACC_SLOTS)
    __device__ __forceinline__ void finish(double* dst)
    {
        double vals[ACC_SLOTS];
#pragma unroll
        for (int s = 0; s < 8 * FT_K; s++) vals[s] = 0.0;
#pragma unroll
        for (int s = 0; s < ACC_NS; s++) {
            const double sv = S[s * FT_BLOCK], cv = C[s * FT_BLOCK];
            const double h = sv + cv;
            // slot s = (order j, part q) -> output pair 4 j + q
            const int o = 4 * (s / ACC_PARTS) + (s % ACC_PARTS);
            vals[2 * o] = h;
            vals[2 * o + 1] = cv - (h - sv);
        }
        vals[ACC_KEPT] = kept;
        vals[ACC_DROPPED] = dropped;
        vals[ACC_QUEUED] = queued;
        vals[ACC_EXACT] = exact;
        vals[ACC_ROBUST] = robust;
#pragma unroll
        for (int s = ACC_ROBUST + 1; s < ACC_SLOTS; s++) vals[s] = 0.0;
        block_reduce(vals, dst);
    }
};
#else
// Shared-memory layout from ACC_SMEM_OFFSET, [slot][thread]: S, C (ACC_NS doubles
// each), N (ACC_NC doubles), then Sf, Cf (ACC_NS floats each), Nf (ACC_NC floats).
// Every address is the block's fixed offset plus the thread index, so the struct holds
// nothing but the base.
#define ACC_D(k) (((double*)base)[(k) * FT_BLOCK + threadIdx.x])
#define ACC_F(k) (((float*)((double*)base + (2 * ACC_NS + ACC_NC) * FT_BLOCK))[(k) * FT_BLOCK + threadIdx.x])
struct accum {
    unsigned char* base;

    __device__ __forceinline__ double& S(int s) { return ACC_D(s); }
    __device__ __forceinline__ double& C(int s) { return ACC_D(ACC_NS + s); }
    __device__ __forceinline__ double& N(int c) { return ACC_D(2 * ACC_NS + c); }
    __device__ __forceinline__ float& Sf(int s) { return ACC_F(s); }
    __device__ __forceinline__ float& Cf(int s) { return ACC_F(ACC_NS + s); }
    __device__ __forceinline__ float& Nf(int c) { return ACC_F(2 * ACC_NS + c); }

    __device__ __forceinline__ void init(unsigned char* smem_acc)
    {
        base = smem_acc;
#pragma unroll
        for (int s = 0; s < ACC_NS; s++) {
            S(s) = 0.0;
            C(s) = 0.0;
            Sf(s) = 0.0f;
            Cf(s) = 0.0f;
        }
#pragma unroll
        for (int c = 0; c < ACC_NC; c++) {
            N(c) = 0.0;
            Nf(c) = 0.0f;
        }
    }

    __device__ __forceinline__ void nadd(int slot, double v)
    {
        const double s = S(slot);
        const double t = s + v;
        C(slot) += (fabs(s) >= fabs(v)) ? ((s - t) + v) : ((v - t) + s);
        S(slot) = t;
    }

    __device__ __forceinline__ void add32(const cx<float>* R)
    {
#pragma unroll
        for (int j = 0; j < FT_K; j++) {
            if (FT_ONLY_PSI && j > 0) break;
            const float re = R[j].re, im = R[j].im;
            const float v[4] = {re, re * re, im, im * im};
#pragma unroll
            for (int q = 0; q < ACC_PARTS; q++) {
                const int o = ACC_PARTS * j + q;
                const float sf = Sf(o);
                const float y = v[q] - Cf(o);
                const float tt = sf + y;
                Cf(o) = (tt - sf) - y;
                Sf(o) = tt;
            }
        }
        const float k = Nf(0) + 1.0f;
        Nf(0) = k;
        if (k == 256.0f) fold();
    }
    // every sample: dropped d, queued q (constants 0 or 1 at the call sites), exact steps e
    __device__ __forceinline__ void note32(float d, float q, float e)
    {
        if (d != 0.0f) Nf(1) += d;
        if (q != 0.0f) Nf(2) += q;
        if (e != 0.0f) Nf(3) += e;
    }
    __device__ __forceinline__ void fold()
    {
#pragma unroll
        for (int s = 0; s < ACC_NS; s++) {
            nadd(s, (double)Sf(s) - (double)Cf(s));
            Sf(s) = 0.0f;
            Cf(s) = 0.0f;
        }
#pragma unroll
        for (int c = 0; c < ACC_NC; c++) {
            N(c) += (double)Nf(c);
            Nf(c) = 0.0f;
        }
    }

    // block-wide: every thread of the block calls it; the block's sums go to dst[0 .. ACC_SLOTS)
    __device__ __forceinline__ void finish(double* dst)
    {
        fold();
        double vals[ACC_SLOTS];
#pragma unroll
        for (int s = 0; s < 8 * FT_K; s++) vals[s] = 0.0;
#pragma unroll
        for (int s = 0; s < ACC_NS; s++) {
            const double sv = S(s), cv = C(s);
            const double h = sv + cv;
            // slot s = (order j, part q) -> output pair 4 j + q
            const int o = 4 * (s / ACC_PARTS) + (s % ACC_PARTS);
            vals[2 * o] = h;
            vals[2 * o + 1] = cv - (h - sv);
        }
        vals[ACC_KEPT] = N(0);
        vals[ACC_DROPPED] = N(1);
        vals[ACC_QUEUED] = N(2);
        vals[ACC_EXACT] = N(3);
        vals[ACC_ROBUST] = 0.0;
#pragma unroll
        for (int s = ACC_ROBUST + 1; s < ACC_SLOTS; s++) vals[s] = 0.0;
        block_reduce(vals, dst);
    }
};
#undef ACC_D
#undef ACC_F
#endif

template <class T>
static __device__ __forceinline__ void write_record(u64 i, const unsigned char* ord, const cx<T>* R, bool ok,
                                                    unsigned char flags, unsigned char* rec_order, double* rec_R,
                                                    unsigned char* rec_flags)
{
    for (int e = 0; e < FT_E; e++) rec_order[i * FT_E + e] = ord[e];
    for (int j = 0; j < FT_K; j++) {
        rec_R[(i * FT_K + j) * 2] = ok ? (double)R[j].re : 0.0;
        rec_R[(i * FT_K + j) * 2 + 1] = ok ? (double)R[j].im : 0.0;
    }
    rec_flags[i] = flags;
}

#if FT_PREC == 0
// one sample in FP64 from stream state g (advanced past the sample's 2E-1 draws)
static __device__ __forceinline__ void sample64(xo& g, const table_ref& tr, const double* prm, u64 i, accum& A,
                                                unsigned char flags, unsigned char* rec_order, double* rec_X,
                                                double* rec_R, unsigned char* rec_flags)
{
    unsigned char ord[FT_E];
    cx<double> R[FT_K];
#pragma unroll
    for (int j = 0; j < FT_K; j++) R[j] = cmk(0.0, 0.0);
    double X[FT_E];
    double F, Gv;
    draw_sector64(g, tr, prm[P_JRFULL], X, F, Gv, ord);
    if (FT_RECORD)
        for (int e = 0; e < FT_E; e++) rec_X[i * FT_E + e] = X[e];
    bool rob = false;
    const bool ok = integrand64(prm, X, F, Gv * F, R, rob);
    if (rob) {
        A.robust += 1;
        flags |= REC_ROBUST;
    }
    if (!ok) {
        A.dropped += 1;
        flags |= REC_DROPPED;
    } else {
        A.add64(R);
    }
    if (FT_RECORD) write_record(i, ord, R, ok, flags, rec_order, rec_R, rec_flags);
}
#endif

// ------------------------------------------------------------------ one thread's samples
// Samples [first, last) of the stream, g holding the state of sample `first`.  In the
// mixed form, samples whose FP32 evaluation is not trustworthy are queued for the FP64
// pass and left out of the sums here: 5 words, the sample (its index in the
// single-integral kernels; item << BQ_ITEM_SHIFT | lane << BQ_LANE_SHIFT | (i - first)
// naming the block's work item in the batch kernels) and its stream state.
static __device__ __forceinline__ void sample_range(xo& g, const table_ref& tr, const double* __restrict__ prm,
                                                    u64 first, u64 last, u64 chunk, accum& A, u64* __restrict__ queue,
                                                    unsigned int* __restrict__ qcount, unsigned int qcap,
                                                    unsigned char* __restrict__ rec_order, double* __restrict__ rec_X,
                                                    double* __restrict__ rec_R, unsigned char* __restrict__ rec_flags)
{
#if FT_PREC == 1
    const float* pf = (const float*)(prm + P_SIZE);
    const float* pd = (const float*)(prm + P_SIZE + (P_SIZE + 1) / 2);   // two-float pairs
#endif
    (void)chunk;
#if FT_VARIANT & 4
    // Every thread of the block makes `chunk` trips and the block starts each sample
    // together: the warps then run the same stretch of the (long, straight-line)
    // per-sample code at the same time and share its instruction fetches.
    for (u64 k = 0; k < chunk; k++) {
        __syncthreads();
        const u64 i = first + k;
        if (i >= last) continue;
#else
    for (u64 i = first; i < last; i++) {
#endif
#if FT_PREC == 0
        sample64(g, tr, prm, i, A, 0, rec_order, rec_X, rec_R, rec_flags);
#else
        unsigned char ord[FT_E];
        unsigned char flags = 0;
        cx<float> R[FT_K];
#pragma unroll
        for (int j = 0; j < FT_K; j++) R[j] = cmk(0.0f, 0.0f);
        const xo g0 = g;
        f2 lx[FT_E], lF, lG;
        const int ex = draw_sector32(g, tr, pf, lx, lF, lG, ord);
        if (ex) flags |= REC_EXACT;
        if (FT_RECORD)
            for (int e = 0; e < FT_E; e++) rec_X[i * FT_E + e] = exp((double)lx[e].hi + (double)lx[e].lo);
        bool need64 = false;
        const bool ok = integrand32(pd, pf, lx, lF, lG, R, need64);
        if (need64) {
            flags |= REC_QUEUED;
            A.note32(0.0f, 1.0f, (float)ex);
            const unsigned int slot = atomicAdd(qcount, 1u);
            if (slot < qcap) {
                u64* q = queue + (size_t)slot * 5;
#if FT_BATCH
                q[0] = (s_batch_item << BQ_ITEM_SHIFT) | ((u64)threadIdx.x << BQ_LANE_SHIFT) | (i - first);
#else
                q[0] = i;
#endif
                q[1] = g0.a;
                q[2] = g0.b;
                q[3] = g0.c;
                q[4] = g0.d;
            }
            if (FT_RECORD) write_record(i, ord, R, false, flags, rec_order, rec_R, rec_flags);
            continue;
        }
        if (!ok) {
            A.note32(1.0f, 0.0f, (float)ex);
            flags |= REC_DROPPED;
        } else {
            A.note32(0.0f, 0.0f, (float)ex);
            A.add32(R);
        }
        if (FT_RECORD) write_record(i, ord, R, ok, flags, rec_order, rec_R, rec_flags);
#endif
    }
}

#if !FT_BATCH
// ------------------------------------------------------------------ single-integral kernels
// Thread t of the launch owns samples [t*chunk, min(nsamples, (t+1)*chunk)) counted
// from the launch's first sample.  warp_states[4w ..] is the stream state of the first
// sample of warp w's lane 0 (computed by a preparation kernel), so a thread skips only
// over its lane's offset.  Block b writes its partial sums to acc_out[b * ACC_SLOTS ...].
extern "C" __global__ void __launch_bounds__(FT_BLOCK, FT_MINB) ft_sample(
    const double* __restrict__ prm, const unsigned char* __restrict__ tab, const u64* __restrict__ lanepw,
    int lanebits, const u64* __restrict__ warp_states, u64 nsamples, u64 chunk, double* __restrict__ acc_out,
    u64* __restrict__ queue, unsigned int* __restrict__ qcount, unsigned int qcap,
    unsigned char* __restrict__ rec_order, double* __restrict__ rec_X, double* __restrict__ rec_R,
    unsigned char* __restrict__ rec_flags)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const table_ref tr = stage_table(smem, tab);

    const u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    xo g = load_state(warp_states + (size_t)(t >> 5) * 4);
    skip_lanes(g, t & 31u, lanepw, lanebits < 5 ? lanebits : 5);

    u64 first = (u64)t * chunk;
    u64 last = first + chunk;
    if (last > nsamples) last = nsamples;

    accum A;
    A.init(smem + ACC_SMEM_OFFSET);
    sample_range(g, tr, prm, first, last, chunk, A, queue, qcount, qcap, rec_order, rec_X, rec_R, rec_flags);
    A.finish(acc_out + (size_t)blockIdx.x * ACC_SLOTS);
}

#if FT_PREC == 0
// FP64 pass over the samples a mixed launch queued (grid-stride over the entries).
extern "C" __global__ void __launch_bounds__(FT_BLOCK) ft_sample_queue(
    const double* __restrict__ prm, const unsigned char* __restrict__ tab, const u64* __restrict__ queue,
    const unsigned int* __restrict__ qcount, unsigned int qcap, double* __restrict__ acc_out,
    unsigned char* __restrict__ rec_order, double* __restrict__ rec_X, double* __restrict__ rec_R,
    unsigned char* __restrict__ rec_flags)
{
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned int n = *qcount;
    if (n > qcap) n = qcap;
    if ((size_t)blockIdx.x * blockDim.x >= n) {
        // no entry for this block (the whole block leaves together): zero sums
        for (int s = threadIdx.x; s < ACC_SLOTS; s += blockDim.x) acc_out[(size_t)blockIdx.x * ACC_SLOTS + s] = 0.0;
        return;
    }
    const table_ref tr = stage_table(smem, tab);
    accum A;
    A.init(smem + ACC_SMEM_OFFSET);
    for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const u64* q = queue + (size_t)k * 5;
        xo g;
        g.a = q[1];
        g.b = q[2];
        g.c = q[3];
        g.d = q[4];
        sample64(g, tr, prm, q[0], A, REC_QUEUED, rec_order, rec_X, rec_R, rec_flags);
    }
    A.finish(acc_out + (size_t)blockIdx.x * ACC_SLOTS);
}
#endif

#else
// ------------------------------------------------------------------ batch kernels
// Many integrals of this topology (each with its own kinematics, table, seed and N)
// in one persistent launch.  The samples of instance i are cut into work items of
// FT_BLOCK * chunk consecutive samples; items are numbered instance after instance
// (instance i owns items [first_item, first_item + nitems)).  A block takes the next
// item from a device counter, thread t of the block owns samples
// [item_base + t*chunk, item_base + (t+1)*chunk) of the instance, and the block writes
// the item's sums to acc_out[item * ACC_SLOTS ...].  item_state[item] is the stream
// state of the item's first sample (computed by a preparation kernel); thread t
// reaches its own first sample with the lane skip matrices (T^(chunk * (2E-1)))^(2^b).
struct batch_inst {
    const double* prm;          // parameter block of the instance (P_SIZE doubles, floats, two-floats)
    const unsigned char* tab;   // J(gamma) table of the instance (global layout)
    u64 nsamples;
    u64 first_item;
    u64 nitems;
    u64 pad[3];
};

// the instance owning `item`: the last instance whose first_item <= item
static __device__ __forceinline__ int find_instance(const batch_inst* __restrict__ inst, int ninst, u64 item)
{
    int lo = 0, hi = ninst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (inst[mid].first_item <= item)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// parameter block of the current instance, staged beside its table (P_SIZE doubles,
// the same as floats, then as two-float pairs)
#define PRM_WORDS (P_SIZE + (P_SIZE + 1) / 2 + P_SIZE)

extern "C" __global__ void __launch_bounds__(FT_BLOCK, FT_MINB) ft_sample_batch(
    const batch_inst* __restrict__ inst, int ninst, const u64* __restrict__ total_items,
    const u64* __restrict__ item_state, const u64* __restrict__ lanepw, int lanebits, u64 chunk,
    unsigned long long* __restrict__ counter, double* __restrict__ acc_out, u64* __restrict__ queue,
    unsigned int* __restrict__ qcount, unsigned int qcap)
{
    extern __shared__ __align__(16) unsigned char smem[];
    // the instance's table and parameters sit at fixed shared-memory addresses, so the
    // per-sample code holds no pointer to them in registers
    __shared__ __align__(16) double s_prm[PRM_WORDS];
    __shared__ int s_inst;
    int cur = -1;
    for (;;) {
        if (threadIdx.x == 0) {
            const u64 it = atomicAdd(counter, 1ull);
            s_batch_item = it;
            s_inst = it < *total_items ? find_instance(inst, ninst, it) : -1;
        }
        // also orders this item's staging after every thread's previous item
        __syncthreads();
        const int id = s_inst;
        if (id < 0) break;
        if (id != cur) {
            copy_table(smem, inst[id].tab);
            const double* __restrict__ src = inst[id].prm;
            for (int k = threadIdx.x; k < PRM_WORDS; k += FT_BLOCK) s_prm[k] = src[k];
            if (threadIdx.x == 0) s_batch_tab = inst[id].tab;
            __syncthreads();
            cur = id;
        }
#if FT_TABLE_GLOBAL
        const table_ref tr = table_at(smem, s_batch_tab);
#else
        const table_ref tr = table_at(smem, nullptr);
#endif
        const u64 it = s_batch_item;
        const u64 n = inst[id].nsamples;
        const u64 first = (it - inst[id].first_item) * (u64)FT_BLOCK * chunk + (u64)threadIdx.x * chunk;
        u64 last = first + chunk;
        if (last > n) last = n;
        xo g = load_state(item_state + it * 4);
        skip_lanes(g, threadIdx.x, lanepw, lanebits);
        accum A;
        A.init(smem + ACC_SMEM_OFFSET);
        sample_range(g, tr, s_prm, first, last, chunk, A, queue, qcount, qcap, nullptr, nullptr, nullptr, nullptr);
        // read before the reduction's barriers, after which the first thread may take
        // the next item
        double* dst = acc_out + s_batch_item * ACC_SLOTS;
        A.finish(dst);
    }
}

#if FT_PREC == 0
// Exact, order-independent sum of doubles: digit j of an accumulator (a signed 64-bit
// counter) weighs 2^(32 j - 1074); v = m 2^(p - 1074) with its integer significand m
// (53 bits) enters as the three 32-bit digits of m 2^(p mod 32) at digit p / 32, so
// every add is exact and integer addition makes the result independent of the order
// in which the threads' atomics land.  Non-finite values are not added (the FP64 pass
// keeps only finite samples).
static __device__ __forceinline__ void exact_add(u64* __restrict__ dig, double v)
{
    const u64 b = (u64)__double_as_longlong(v);
    const int be = (int)((b >> 52) & 0x7ffull);
    if (be == 0x7ff) return;
    u64 m = b & 0xfffffffffffffull;
    int p = 0;
    if (be) {
        m |= 1ull << 52;
        p = be - 1;
    }
    if (m == 0) return;
    const int j = p >> 5, sh = p & 31;
    const u64 lo = m << sh, hi = sh ? (m >> (64 - sh)) : 0ull;
    const bool neg = (b >> 63) != 0;
    const u64 c0 = lo & 0xffffffffull, c1 = lo >> 32;
    atomicAdd(dig + j, neg ? 0ull - c0 : c0);
    if (c1) atomicAdd(dig + j + 1, neg ? 0ull - c1 : c1);
    if (hi) atomicAdd(dig + j + 2, neg ? 0ull - hi : hi);
}

// FP64 pass over the samples a mixed batch launch queued: each entry names its work
// item (hence the instance) and carries the sample's stream state.  Each kept sample's
// values go exactly into the instance's accumulators in qacc (FT_XA_DIGITS words each):
// per eps order j accumulators 4j + 0..3 = re f, re f^2, im f, im f^2; then the
// counters kept, dropped, robust (integer atomics).
extern "C" __global__ void __launch_bounds__(FT_BLOCK) ft_sample_queue_batch(
    const batch_inst* __restrict__ inst, int ninst, const u64* __restrict__ queue,
    const unsigned int* __restrict__ qcount, unsigned int qcap, u64* __restrict__ qacc)
{
    unsigned int n = *qcount;
    if (n > qcap) n = qcap;
    for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const u64* q = queue + (size_t)k * 5;
        const u64 item = q[0] >> BQ_ITEM_SHIFT;
        xo g;
        g.a = q[1];
        g.b = q[2];
        g.c = q[3];
        g.d = q[4];
        const int id = find_instance(inst, ninst, item);
        const double* prm = inst[id].prm;
        const unsigned char* tab = inst[id].tab;
        table_ref tr;
        tr.w = tab + T_W64;
        tr.Jr = tab + T_JR64;
        tr.ri = tab + T_RI64;
        tr.meta = tab + T_META;
        tr.gm = tab;
        cx<double> R[FT_K];
#pragma unroll
        for (int j = 0; j < FT_K; j++) R[j] = cmk(0.0, 0.0);
        double X[FT_E];
        double F, Gv;
        unsigned char ord[FT_E];
        draw_sector64(g, tr, prm[P_JRFULL], X, F, Gv, ord);
        bool rob = false;
        const bool ok = integrand64(prm, X, F, Gv * F, R, rob);
        u64* qa = qacc + (size_t)id * (4 * FT_K * FT_XA_DIGITS + 4);
        u64* cnt = qa + 4 * FT_K * FT_XA_DIGITS;
        if (rob) atomicAdd(cnt + 2, 1ull);
        if (!ok) {
            atomicAdd(cnt + 1, 1ull);
            continue;
        }
        atomicAdd(cnt, 1ull);
#pragma unroll
        for (int j = 0; j < FT_K; j++) {
            if (FT_ONLY_PSI && j > 0) break;
            exact_add(qa + (4 * j + 0) * FT_XA_DIGITS, R[j].re);
            exact_add(qa + (4 * j + 1) * FT_XA_DIGITS, R[j].re * R[j].re);
            if (ACC_PARTS == 4) {
                exact_add(qa + (4 * j + 2) * FT_XA_DIGITS, R[j].im);
                exact_add(qa + (4 * j + 3) * FT_XA_DIGITS, R[j].im * R[j].im);
            }
        }
    }
}
#endif
#endif  // FT_BATCH
#endif  // FT_HOST_SIM
