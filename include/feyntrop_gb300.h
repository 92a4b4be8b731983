/*
 * feyntrop_gb300 — C ABI of the GB300 tropical sampling + integrand evaluation path.
 *
 * This library replaces the reference's in-process seam
 *
 *   generate_subgraph_table(g, D, P, m2, eps_expansion, bNonEuclidean)
 *       srcs/tropical_sampling.hpp:284-291
 *   feynman_integral_estimate(N, g, D, P, m2, num_eps_terms, lambda, table, gen)
 *       srcs/feynman_integral.hpp:30-41, called from srcs/feyntrop.cpp:251
 *
 * and the decisions the CLI makes around it (srcs/feyntrop.cpp:25-239).  Plain
 * pointers and sizes only; no exception crosses the boundary: every call returns
 * a status code and ft_last_error() holds the reference's message for the last
 * failure on the calling thread.  Caller-owned result buffers.  Distinct plans may
 * be used from different host threads concurrently.
 */
#ifndef FEYNTROP_GB300_H
#define FEYNTROP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes; the reference throws the matching C++ exception type */
#define FT_OK 0
#define FT_ERR_INVALID_ARGUMENT 1 /* std::invalid_argument (input shape, graph checks) */
#define FT_ERR_DOMAIN 2           /* std::domain_error (kinematics, divergences, GP checks) */
#define FT_ERR_RUNTIME 3          /* std::runtime_error */
#define FT_ERR_CUDA 4             /* device, driver or runtime-compiler failure */
#define FT_ERR_NO_DEVICE 5        /* no CUDA device: this library has no CPU path */

/* arithmetic of the sampling kernels */
#define FT_PRECISION_FP64 0  /* every operation in FP64 */
#define FT_PRECISION_MIXED 1 /* FP32 integrand, FP64 sector decisions, FP64 re-evaluation of flagged samples */

typedef struct ft_plan ft_plan;

/* One Feynman integral: the reference's low-level JSON input as arrays
 * (srcs/feyntrop.cpp:39-96). */
typedef struct {
    int32_t num_edges;            /* E */
    const int32_t* edges;         /* 2E vertex numbers, edge e = (edges[2e], edges[2e+1]) */
    const double* nu;             /* E edge weights */
    int32_t num_vertices;         /* V; must equal max vertex + 1, or -1 to derive it */
    const double* scalarproducts; /* V*V, row major */
    const double* masses_sqr;     /* E */
    double dimension;             /* D */
    int32_t num_eps_terms;        /* K >= 1 */
    double lambda;                /* deformation parameter */
} ft_problem;

/* Host preprocessing and upload: input checks, regime decision and the J(gamma)
 * table (replaces srcs/feyntrop.cpp:64-239 and generate_subgraph_table). */
int ft_plan_create(const ft_problem* problem, ft_plan** out);
void ft_plan_destroy(ft_plan* plan);

/* ft_plan_create for many problems at once on all host threads (kinematic scans,
 * batches; the reference prepares one input per process, srcs/feyntrop.cpp:143-158).  out[i] is NULL where problem i failed; status[i] (may be NULL) holds each
 * problem's code.  Returns FT_OK, or the code of the first failure (its message, with
 * the problem's index, in ft_last_error()). */
int ft_plans_create(const ft_problem* problems, int32_t count, ft_plan** out, int32_t* status);

typedef struct {
    double W;                     /* superficial degree of divergence */
    double IGtr;                  /* tropical normalisation I_G^tr */
    int32_t loops;
    int32_t euclidean, pseudo_euclidean, generic, gp_property;
    int32_t deformed;             /* 1 when the contour deformation is used */
    double lambda_used;
    double seconds_preprocessing;
    uint64_t table_bytes;         /* device bytes of the J(gamma) table */
    int32_t num_log_lines;        /* diagnostics the reference prints to stderr */
} ft_plan_info;

int ft_plan_get_info(const ft_plan* plan, ft_plan_info* info);
/* i-th diagnostic line (0-based), NUL-terminated, owned by the plan */
const char* ft_plan_log_line(const ft_plan* plan, int32_t i);

typedef struct {
    uint64_t num_samples;   /* N */
    uint64_t seed;
    uint64_t first_sample;  /* index of the first sample in the seed's stream (sharding) */
    int32_t precision;      /* FT_PRECISION_* */
    void* stream;           /* cudaStream_t, NULL for the library's own stream */
} ft_run_options;

/* Raw sums, mergeable across shards: per eps order j and part p (0 = Re, 1 = Im)
 * the slot [2j+p] holds count, sum f (hi, lo) and sum f^2 (hi, lo). */
typedef struct {
    double n;
    double s1_hi, s1_lo, s2_hi, s2_lo;
} ft_moments;

typedef struct {
    int32_t num_eps_terms;    /* K, entries in the arrays below */
    double* re_avg;           /* caller-owned, K each */
    double* re_acc;
    double* im_avg;
    double* im_acc;
    ft_moments* moments;      /* caller-owned 2K entries, may be NULL */
    uint64_t kept, dropped;   /* samples accumulated / dropped as non-finite */
    uint64_t fp64_fallback;   /* mixed: samples re-evaluated in FP64 */
    uint64_t exact_steps;     /* mixed: sector steps decided by the FP64 re-check */
    uint64_t robust;          /* complex Laplacians that needed complete pivoting */
    double kernel_ms;         /* device time of the sampling kernels (CUDA events) */
    double seconds_sampling;  /* host wall time of the call */
    int32_t kernel_launches;
} ft_result;

/* Samples first_sample .. first_sample+N-1 of the seed's stream (replaces
 * feynman_integral_estimate).  With first_sample = 0 the samples are exactly those
 * of the reference run with OMP_NUM_THREADS=1. */
int ft_integrate(ft_plan* plan, const ft_run_options* opts, ft_result* result);

/* Several integrals in one call: a batch (below) created, run once and destroyed.  Plans
 * with FT_PRECISION_MIXED options form one batch, the others a second.  Each result is
 * that of ft_integrate with the same options, up to the order of the sums.  The
 * reference integrates one graph per process (srcs/feyntrop.cpp:251); this is the
 * in-process counterpart of running it once per kinematic point. */
int ft_integrate_batch(ft_plan* const* plans, int32_t count, const ft_run_options* opts, ft_result* results);

/* A batch: many integrals (any mix of graphs, kinematics, seeds and sample counts) run
 * by one CUDA graph launch (each integral replaces one feynman_integral_estimate call,
 * srcs/feynman_integral.hpp:30-41).  Integrals of one kernel class (same topology, eps orders,
 * regime) share one persistent sampling launch whose blocks take work items of
 * consecutive samples from a device counter; classes run side by side.  The batch
 * copies the plans' parameters and tables at creation; the plans must outlive it (their
 * host data finalises the results).  Reusable: ft_batch_run may be called any number of
 * times with new sample counts, seeds and first samples; the graph is captured on the
 * first run and again only when a run needs more work items or FP64 hand-off entries
 * than the previous ones.  precision applies to every integral of the batch. */
typedef struct ft_batch ft_batch;
int ft_batch_create(ft_plan* const* plans, int32_t count, int32_t precision, ft_batch** out);
void ft_batch_destroy(ft_batch* batch);
/* opts[i] (num_samples, seed, first_sample) for integral i; opts[0].stream (or NULL for
 * the batch's own stream) carries the graph launch; precision fields are ignored.
 * results[i] as from ft_integrate; kernel_ms is the whole graph's device time. */
int ft_batch_run(ft_batch* batch, const ft_run_options* opts, ft_result* results);

typedef struct {
    int32_t num_integrals;
    int32_t num_classes;         /* persistent sampling launches per run */
    int32_t graph_captures;      /* captures so far */
    int32_t kernel_launches;     /* kernel nodes of the graph */
    uint64_t work_items;         /* of the last run */
    uint64_t fp64_queue_capacity;
    double kernel_ms;            /* device time of the last run (CUDA events) */
} ft_batch_info;
int ft_batch_get_info(const ft_batch* batch, ft_batch_info* info);

/* Integration that allocates no memory, for callers that must not allocate device
 * memory while they integrate (an embedding application or serving loop that owns all
 * device memory, or a region where allocation is forbidden).  No counterpart in the
 * reference.  The same samples as ft_integrate, and its launch shape with the number
 * of blocks capped at what the scratch holds, asynchronous on opts->stream (or the
 * plan's stream): the final sums are written to d_slots, a caller-owned DEVICE buffer
 * of 8K+8 doubles: for eps order j and part p (0 Re, 1 Im) [8j+4p .. +3] = sum f
 * (hi, lo), sum f^2 (hi, lo); then kept, dropped, samples handed to the FP64 pass
 * (all of them, also those beyond the queue), exact sector steps, complete-pivoting
 * factorisations.
 * Scratch is one static device array per GPU (about 7 MB, held until exit): at most
 * 2048 blocks, 16 eps orders and 65536 samples handed to the FP64 pass per call; the
 * hand-offs beyond 65536 are not evaluated, which slot 8K+2 > 65536 (equivalently
 * kept + dropped < N) reports.  The plan's kernels must already be
 * loaded by one ft_integrate call with the same precision.  The first call on a device
 * looks up the scratch address (call it once before any stream capture).  Calls share
 * the scratch, so calls that overlap on the GPU race. */
int ft_integrate_noalloc(ft_plan* plan, const ft_run_options* opts, double* d_slots);

/* avg / acc from merged moments, with the reference's formulas (srcs/stats.hpp:86-104);
 * real_only marks integrals whose imaginary part the reference reports as (0, 0). */
int ft_finalize_moments(const ft_moments* moments, int32_t num_eps_terms, int32_t real_only, ft_result* result);

/* Per-sample records of samples first_sample .. +N-1 (parity checks; no counterpart in
 * the reference, whose per-sample values exist only inside its loop,
 * srcs/feynman_integral.hpp:162-362): removal order
 * (N x E bytes), X before rescaling (N x E), integrand per eps order (N x K x 2:
 * re, im) and flags (bit 0 dropped, 1 re-evaluated in FP64, 2 exact sector step,
 * 3 complete-pivoting LU).  Any pointer may be NULL. */
int ft_sample_records(ft_plan* plan, const ft_run_options* opts, uint8_t* order, double* X, double* R,
                      uint8_t* flags);

/* The reference's CLI contract in process: input JSON text in, output JSON text
 * out (srcs/feyntrop.cpp:20-281).  *output is malloc'd; free with ft_free. */
int ft_run_json(const char* input_json, char** output, char** log);
void ft_free(void* p);

/* Host preprocessing only (no device): the J(gamma) table of
 * generate_subgraph_table (srcs/tropical_sampling.hpp:284-458), indexed by the edge
 * bitmask of gamma, 2^E entries each (Jr, r, mass-momentum-spanning flag, loop
 * number), and the plan information.  Any output pointer may be NULL. */
int ft_subgraph_table(const ft_problem* problem, double* Jr, double* r, uint8_t* mm, uint8_t* loops,
                      ft_plan_info* info);

/* No counterpart in the reference (it has no device code).  Host preprocessing plus
 * run-time compilation of the sampling kernels for this problem's topology (FP64 and, if requested, mixed; with FT_PRECOMPILE_BATCH or'ed
 * into precision also the batch kernels), without touching a device: warms the kernel
 * cache.  *seconds receives the compile time (0 when cached). */
#define FT_PRECOMPILE_BATCH 0x100
int ft_precompile(const ft_problem* problem, int32_t precision, double* seconds);

/* Autotuner (no counterpart in the reference): times the sampling kernels of this plan's kernel class (topology, eps
 * orders, regime, precision) under candidate launch shapes (threads per block, blocks
 * per SM given to the register allocator, code-size variants), `samples` samples per
 * trial (at least 256 per thread of a full launch, so that the trials see the steady
 * state), then the batch work-item size (samples per thread: 32 .. 256) under the chosen
 * shape (batches of this integral with at least 1024 samples per thread of the GPU, so
 * that the largest item still leaves every SM several), and records both in the tuning
 * table (in memory and in tuning.json beside the kernel cache), which every later plan
 * and batch of the class uses.  A candidate replaces the default shape or work item
 * only when it is at least 3 % faster in these trials.  The candidates' kernels are compiled concurrently
 * before the timing. */
typedef struct {
    int32_t block, min_blocks_per_sm, variant;   /* the recorded shape */
    double samples_per_second;                   /* its rate */
    double default_samples_per_second;           /* the default shape's rate (-1 if not a candidate) */
    int32_t candidates;
    uint64_t batch_chunk;                        /* recorded batch work item: samples per thread */
    double batch_samples_per_second;             /* its rate in a batch of this integral */
} ft_tune_result;
int ft_autotune(ft_plan* plan, int32_t precision, uint64_t samples, ft_tune_result* out);

/* No counterpart in the reference.  Measured FP32 and FP64 FMA issue rates of the current device in TFLOP/s (an
 * FMA-chain probe kernel; the denominators of the sampling kernels' roofline). */
int ft_device_peaks(double* fp32_tflops, double* fp64_tflops);

const char* ft_last_error(void);
const char* ft_version(void);

#ifdef __cplusplus
}
#endif
#endif
