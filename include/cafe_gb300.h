/* cafe_gb300.h -- C ABI of the GB300 (sm_103a) CAFE5 likelihood path.
 *
 * Drop-in boundary for CAFE5's likelihood hot path: transition-matrix
 * construction (matrix_cache / probability.cpp) and Felsenstein pruning of
 * every gene family (inference_prune) as called by the base and gamma
 * models and, through them, by optimizer_scorer and the Nelder-Mead search;
 * and for the analyses built on the same matrices and walk: Pupko ancestral
 * reconstruction and branch probabilities, p-values, and the simulator.
 * Plain C types only.
 *
 * Every entry point returns a cafe_status. No call throws, and no pointer
 * handed back to the host aliases device memory. A context owns all
 * device-resident state (trees, family counts, prior, error model and the
 * transition-matrix cache); callers own every host buffer they pass.
 *
 * Reference interfaces each entry point replaces are cited per function
 * (paths relative to the CAFE5 project).
 */
#ifndef CAFE_GB300_H
#define CAFE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    CAFE_OK = 0,
    CAFE_ERR_OOM = 1,            /* device allocation refused */
    CAFE_ERR_MISSING_MATRIX = 2, /* matrix_cache::get_matrix on an absent key */
    CAFE_ERR_SATURATED = 3,      /* reported in cafe_result.status only */
    CAFE_ERR_UNDERFLOW = 4,      /* reported in cafe_result.status only */
    CAFE_ERR_TIMEOUT = 5,        /* a bounded wait ran out */
    CAFE_ERR_INVALID = 6,        /* malformed argument */
    CAFE_ERR_CUDA = 7,           /* CUDA runtime error; see cafe_last_error */
    CAFE_ERR_BUSY = 8,           /* request not finished / not admitted yet */
    CAFE_ERR_NOT_FOUND = 9       /* unknown tree / family-set / ticket id */
} cafe_status;

typedef enum { CAFE_MODEL_BASE = 0, CAFE_MODEL_GAMMA = 1 } cafe_model;
typedef enum { CAFE_LAMBDA_SINGLE = 0, CAFE_LAMBDA_MULTIPLE = 1 } cafe_lambda_kind;

/* Arithmetic of the pruning step. Matrices, root weighting and the final
 * log-likelihood sums are FP64 in every mode.
 *   FP64_REF     reference semantics: one global state bound S and root
 *                bound R, unscaled FP64 (underflow behaves as in CAFE5)
 *   FP64_BINNED  per-family S bins, FP64 with per-node power-of-two rescale
 *   MIXED_TF32X3 per-family S bins on the tensor cores (tcgen05, kind::tf32):
 *                each operand is split into two TF32 parts (hi, lo), products
 *                hi*hi + hi*lo + lo*hi accumulate in FP32, node vectors carry
 *                integer power-of-two exponents; bins wider than 512 states,
 *                trees with a node of more than two children, and families
 *                whose factors lose FP32 range (a per-family error bound) are
 *                computed in FP64_BINNED */
typedef enum {
    CAFE_PREC_FP64_REF = 0,
    CAFE_PREC_FP64_BINNED = 1,
    CAFE_PREC_MIXED_TF32X3 = 2
} cafe_precision;

typedef struct cafe_ctx cafe_ctx;

typedef struct {
    int device;                  /* CUDA device ordinal */
    size_t matrix_cache_bytes;   /* cap on the matrices of each of the cache's two generations of
                                    device memory; 0 = the smaller of 4 GB and 1/8 of free HBM. Past the
                                    cap the cache starts over in its other generation, whose builds wait
                                    for that generation's earlier users (no synchronisation) */
    int n_streams;               /* concurrent request streams for cafe_submit; 0 = 4 */
    int max_bins;                /* reserved, 0 */
} cafe_config;

/* One score request: one infer_family_likelihoods call
 * (model::infer_family_likelihoods, src/core.h:174). */
typedef struct {
    int tree_id;
    int set_id;
    int model;                   /* cafe_model */
    int lambda_kind;             /* cafe_lambda_kind */
    int n_lambdas;
    const double* lambdas;       /* host; lambda per lambda index */
    int n_categories;            /* gamma: K; base: ignored (1) */
    const double* multipliers;   /* host; gamma lambda multipliers m_k */
    const double* cat_probs;     /* host; gamma category probabilities */
    int use_error_model;         /* leaves from the context's error model */
    int max_family_size;         /* FP64_REF: global S; binned modes: 0 */
    int max_root_family_size;    /* FP64_REF: global R; binned modes: 0 */
    int precision;               /* cafe_precision */
    int dedupe;                  /* prune identical count rows once (base model) */
} cafe_request;

typedef struct {
    double* family_lnl;          /* host, n_families, or NULL */
    double* category_lnl;        /* host, n_families * K (natural log), or NULL */
    double total_neg_lnl;        /* -sum lnL; +inf on the reference's rejection paths */
    int status;                  /* CAFE_OK / CAFE_ERR_SATURATED / CAFE_ERR_UNDERFLOW */
    int64_t n_failed;            /* gamma: families whose category root vector summed to 0 */
    int64_t n_fallback;          /* mixed: families recomputed in FP64 */
    double device_ms;            /* device time of the request (CUDA events) */
} cafe_result;

/* ---- context --------------------------------------------------------- */
int cafe_ctx_create(const cafe_config* cfg, cafe_ctx** out);
int cafe_ctx_destroy(cafe_ctx* ctx);
const char* cafe_last_error(const cafe_ctx* ctx);
const char* cafe_status_string(int status);
int cafe_version(void);

/* Test hooks (no counterpart in the reference). CAFE_DEBUG_TC_WAIT_LIMIT:
 * value n > 0 makes the tensor-core kernel's wait for a node's GEMMs give
 * up after n - 1 polls (1: at once); 0 restores the default bound of 2^24
 * polls. With 1 a test can check that the kernel drains its own copies and
 * MMAs, frees TMEM, and the call returns CAFE_ERR_TIMEOUT with the context
 * still usable. */
typedef enum { CAFE_DEBUG_TC_WAIT_LIMIT = 1 } cafe_debug_knob;
int cafe_debug_set(cafe_ctx* ctx, int knob, int64_t value);

/* ---- inputs ---------------------------------------------------------- */
/* Species tree (clade, src/clade.h:25-121). Nodes are numbered so that the
 * children of every node appear in increasing index (Newick order), which
 * is the descendant order used for the product over children. parent[i]
 * is -1 for the root. lambda_index[i] (0-based) selects the rate of the
 * branch above node i (multiple_lambda, src/lambda.cpp:32-40); NULL means
 * all 0. Leaves are the nodes without children, in increasing index; that
 * order is the column order of the counts passed to cafe_families_upload. */
int cafe_tree_upload(cafe_ctx* ctx, int n_nodes, const int32_t* parent, const double* branch_length,
                     const int32_t* lambda_index, int* tree_id);

/* Gene families (gene_family, src/gene_family.h) as an int32 matrix
 * counts[n_families][n_leaves], kept resident on the device. */
int cafe_families_upload(cafe_ctx* ctx, int tree_id, const int32_t* counts, int64_t n_families, int n_leaves,
                         int* set_id);
/* Replace the counts of an existing set in place (same shape): always
 * copied to the device; the derived tables (per-family maxima, duplicate
 * rows, S-bins) are rebuilt only when the counts differ from the set's. */
int cafe_families_update(cafe_ctx* ctx, int set_id, const int32_t* counts);
int cafe_families_free(cafe_ctx* ctx, int set_id);

/* Root prior: prior[j] = root_equilibrium_distribution::compute(j)
 * (src/root_equilibrium_distribution.cpp:81-87), already rounded to float
 * by the caller, for root-vector index j; 0 beyond n. */
int cafe_prior_set(cafe_ctx* ctx, const double* prior, int n);

/* Error model (error_model::get_probs, src/error_model.cpp:52-57): rows of
 * n_dev probabilities per observed count; counts past the last row use the
 * last row. n_rows = 0 clears it. */
int cafe_error_model_set(cafe_ctx* ctx, const double* rows, int n_rows, int n_dev);

/* ---- matrix cache (matrix_cache, src/matrix_cache.h:70-96) ------------ */
/* precalculate_matrices (src/matrix_cache.cpp:113-163): build every missing
 * (lambda, t) matrix of the given size, keyed and computed at
 * lambda truncated to 1e-9 and t truncated to 1e-3. */
int cafe_matrices_build(cafe_ctx* ctx, const double* lambdas, int n_lambdas, const double* branch_lengths,
                        int n_branch_lengths, int matrix_size);
/* get_matrix (src/matrix_cache.cpp:88-105): copy one cached matrix
 * (row-major size x size) to host memory; CAFE_ERR_MISSING_MATRIX if the
 * key was never built. */
int cafe_matrix_get(cafe_ctx* ctx, double lambda, double branch_length, int matrix_size, double* out);
int cafe_matrix_cache_size(cafe_ctx* ctx, int64_t* n_matrices);
int cafe_matrix_cache_clear(cafe_ctx* ctx);
/* is_saturated (src/matrix_cache.cpp:107-111). */
int cafe_is_saturated(double branch_length, double lambda);

/* ---- scoring --------------------------------------------------------- */
/* Synchronous infer_family_likelihoods (src/base_model.cpp:53-100,
 * src/gamma_core.cpp:168-237): results copied into the caller's host
 * buffers. Rejections the reference reports as a score (invalid lambda,
 * saturation, gamma underflow) return CAFE_OK with total_neg_lnl = +inf
 * and result->status set. */
int cafe_score(cafe_ctx* ctx, const cafe_request* req, cafe_result* res);

/* Batched candidates (many optimizer steps, or the B candidate vectors of
 * one search round, scored together): n requests that share tree, family
 * set, model, category count, precision, error-model use and (FP64_REF)
 * bounds, each with its own lambdas, multipliers and category
 * probabilities. Every (candidate, category) pair is pruned in the same
 * launches; results[i] is exactly what cafe_score(reqs[i]) reports, within
 * the precision's tolerance (bit-identical for the FP64 modes). A
 * candidate the reference would reject scores +inf without affecting the
 * others. */
int cafe_score_batch(cafe_ctx* ctx, const cafe_request* reqs, int n, cafe_result* results);

/* Autotuner for the tensor-core launch shapes: for every S-bin width of the
 * requests' family set (<= 256 states), times the batch (cafe_score_batch
 * semantics, MIXED_TF32X3) with the default shape and with the candidate
 * shapes (the three largest feasible CTA counts per SM x 1-4 pipeline
 * stages), one bin at a time, and keeps the fastest per width for every
 * later call on this context. `reps` timed runs per candidate (after one
 * untimed run). Results do not depend on the shape. Writes up to max_out
 * (width, CTAs per SM, stages, ms) entries. */
typedef struct {
    int width;
    int ctas_per_sm;
    int stages;
    double ms;                   /* mean device time of the batch with this shape */
} cafe_tune_result;
int cafe_autotune(cafe_ctx* ctx, const cafe_request* reqs, int n, int reps, cafe_tune_result* out, int max_out,
                  int* n_out);

/* Device-resident variant: enqueues the whole evaluation on `stream`
 * (a cudaStream_t; NULL = the context's stream) and writes per-family lnL
 * to d_family_lnl (device, n_families doubles, may be NULL) and the total
 * to d_total (device, one double, may be NULL) without any host sync.
 * res->status and counters are not filled. */
int cafe_score_device(cafe_ctx* ctx, const cafe_request* req, double* d_family_lnl, double* d_total,
                      void* stream);
/* Device-resident batch (the requests of cafe_score_batch): d_family_lnl
 * is [n][n_families], d_total [n]. */
int cafe_score_batch_device(cafe_ctx* ctx, const cafe_request* reqs, int n, double* d_family_lnl, double* d_total,
                            void* stream);

/* Continuous-batching request loop for many concurrent optimizers: submit
 * returns at once with a ticket; the request is admitted when a stream is
 * free and its estimated device footprint fits the loop's budget (a quarter
 * of the device memory free at context creation). Compatible requests
 * queued at that moment (the batching rules of cafe_score_batch) are merged
 * into one batched launch; admitted batches run concurrently on separate
 * streams. `res` is filled when done (host buffers must stay valid).
 * poll returns CAFE_OK when finished, CAFE_ERR_BUSY while pending;
 * wait_ms < 0 waits without limit, otherwise at most wait_ms. */
int cafe_submit(cafe_ctx* ctx, const cafe_request* req, cafe_result* res, uint64_t* ticket);
int cafe_poll(cafe_ctx* ctx, uint64_t ticket, int wait_ms);

/* Per-kernel device timing for measurement. When enabled, the library
 * records CUDA events around each kernel it launches on the synchronous
 * workspace stream (cafe_score / cafe_score_device) and accumulates their
 * durations; cafe_profile_read waits for that stream, returns the sums
 * since the previous read and resets them. `prune_flops` is the
 * algorithmic flop count of the pruning launches (2 x rows x states per
 * internal-child contraction, rows x states per extra child product). */
typedef struct {
    double matrix_ms;            /* K1 transition-matrix builds */
    double prune_ms;             /* pruning + root weighting (FP64 or tensor core) */
    double finish_ms;            /* per-family lnL and the total */
    double other_ms;             /* conversion / fallback launches */
    double prune_flops;
    int64_t launches;            /* kernels launched */
    int64_t prune_launches;
    int64_t matrices_built;
    double host_keys_ms;         /* host: matrix keys, cache builds, pointer tables */
    double host_plan_ms;         /* host: conversion jobs, tiles, launch plans */
    double host_total_ms;        /* host: whole enqueue of the profiled calls */
    double host_build_ms;        /* host: part of host_keys_ms spent enqueueing matrix builds
                                    (job tables, cache memory, the K1 launch) */
} cafe_timings;
int cafe_profile_enable(cafe_ctx* ctx, int enable);
int cafe_profile_read(cafe_ctx* ctx, cafe_timings* out);

/* No-allocation FP64 pruning, for callers that cannot call cudaMalloc (a
 * host framework that owns every device allocation through its own pool, a
 * serving loop that must not allocate per request, a plug-in living inside
 * another allocator). No counterpart in the reference: it is an extra entry
 * point of this library. It runs the same pruning kernel as cafe_score in
 * FP64 for the base model (per-family lnL = max_j log L_root[j] + log
 * prior[j], src/base_model.cpp:77-95) with one global state bound, and takes
 * every input and output as the caller's memory:
 *   parent[n_nodes]         host, tree as in cafe_tree_upload
 *   node_matrix[n_nodes]    host array of device pointers: the FP64
 *                           matrix_size x matrix_size matrix of the branch
 *                           above each node (root entry ignored)
 *   d_counts                device int32 [n_families][n_leaves]
 *   d_prior                 device, n_prior doubles (float-rounded prior)
 *   scaled                  0 = reference arithmetic, 1 = per-node rescale
 *   d_family_lnl            device output, n_families doubles
 *   stream                  cudaStream_t the work is enqueued on
 * It allocates nothing: its working space is one static device array of
 * 40 MiB that the library reserves on every GPU that loads it until the
 * process exits. Limits: n_families <= 262,144, n_nodes <= 512, and
 * (internal-node slots) x max(S+1, R) x 32 doubles must fit in 32 MiB;
 * larger calls return CAFE_ERR_INVALID without launching anything. The
 * first call on each device looks up the array's device address (with that
 * device current), so make it before any stream capture. All calls share
 * the array: calls whose GPU work overlaps race and must be serialised. */
int cafe_prune_fp64_noalloc(int n_nodes, const int32_t* parent, const double* const* node_matrix,
                            int matrix_size, const int32_t* d_counts, int64_t n_families, int n_leaves,
                            int max_family_size, int max_root_family_size, const double* d_prior, int n_prior,
                            int scaled, double* d_family_lnl, void* stream);

/* Serving statistics since context creation: completed requests, p50 and
 * p99 latency (ms, submit -> done), current in-flight count. */
int cafe_serving_stats(cafe_ctx* ctx, int64_t* completed, double* p50_ms, double* p99_ms, int* in_flight);
/* Serving-loop counters since context creation. */
typedef struct {
    int64_t batches;             /* batched launches */
    int64_t merged;              /* requests that shared a launch with others */
    int64_t retried;             /* requests rerun alone after their batch failed */
    double enqueue_ms;           /* host time enqueuing batches (context lock held) */
    double wait_ms;              /* host time waiting for batches to finish */
    double device_ms;            /* device time of the batches (events) */
    double overlap_ms;           /* device time during which batches ran side by side: the summed pairwise
                                    intersections of the batches' event intervals (0 when every batch ran
                                    alone) */
} cafe_serving_info;
int cafe_serving_counters(cafe_ctx* ctx, cafe_serving_info* out);

/* ---- parameter search (src/optimizer.cpp, src/optimizer_scorer.cpp) ---- */
/* Which parameters the search varies (the scorer classes of
 * src/optimizer_scorer.h:28-150):
 *   LAMBDA          lambdas only (lambda_optimizer; base model, or gamma
 *                   with the request's fixed categories)
 *   ALPHA           alpha only, lambdas fixed at the request's (gamma_optimizer)
 *   LAMBDA_ALPHA    lambdas + alpha (gamma_lambda_optimizer); the request's
 *                   multipliers and cat_probs are recomputed from alpha each
 *                   evaluation by cafe_discrete_gamma
 *   LAMBDA_EPSILON  lambdas + the error model's distinct epsilons
 *                   (lambda_epsilon_optimizer); the context's error model
 *                   (3 deviations per row) is rewritten by
 *                   error_model::replace_epsilons each evaluation and left
 *                   at the last evaluated values */
typedef enum {
    CAFE_OPT_LAMBDA = 0,
    CAFE_OPT_LAMBDA_ALPHA = 1,
    CAFE_OPT_LAMBDA_EPSILON = 2,
    CAFE_OPT_ALPHA = 3,
} cafe_opt_kind;

typedef struct {
    int kind;                    /* cafe_opt_kind */
    int n_params;                /* n_lambdas (+1 alpha | + number of epsilons); ALPHA: 1 */
    const double* initial;       /* starting point, n_params (optimizer_scorer::initial_guesses) */
    int max_iterations;          /* <= 0: 300 (optimizer_parameters::neldermead_iterations) */
    double reflection;           /* <= 0: 1 (Nelder-Mead rho) */
    double expansion;            /* <= 0: 2 (Nelder-Mead chi) */
} cafe_opt_config;

typedef struct {
    double* values;              /* host, n_params: best point found */
    double score;                /* -lnL there (+inf if every point was rejected) */
    int iterations;
    int evaluations;             /* objective (= cafe_score) calls */
    int converged;               /* 1 if tolx/tolf were reached before max_iterations */
} cafe_opt_result;

/* optimizer::optimize with the Standard Nelder-Mead strategy
 * (src/optimizer.cpp:60-73, 156-322, 430-487): simplex start 5 % away from
 * `initial` per coordinate (0.00025 for a zero coordinate), tolx = tolf =
 * 1e-6, reflection/expansion/contraction/shrink 1/2/0.5/0.5. Each objective
 * evaluation scores `base` through cafe_score with the candidate
 * parameters substituted; NaN scores count as +inf. As in
 * optimizer::get_initial_guesses (src/optimizer.cpp:343-360) the initial
 * point is scored first; if that is +inf the call returns
 * CAFE_ERR_INVALID without searching. `evaluations` counts that call. */
int cafe_optimize(cafe_ctx* ctx, const cafe_request* base, const cafe_opt_config* cfg, cafe_opt_result* out);

/* fminsearch_min (src/optimizer.cpp:281-322) over a caller-supplied
 * objective, for scorers that are not likelihoods (the reference's
 * optimizer_scorer interface, src/optimizer_scorer.h:13-20): the same
 * simplex rules and defaults as cafe_optimize (`kind` is ignored), without
 * the initial-point check; `evaluations` counts objective calls. */
int cafe_nelder_mead(const cafe_opt_config* cfg, double (*objective)(const double* x, int n, void* user), void* user,
                     cafe_opt_result* out);

/* gamma_model::set_alpha (src/gamma.cpp:15-52, 225-241): K equal-probability
 * rate categories of a mean-1 Gamma(alpha) distribution, each represented
 * by its median, rescaled so the multipliers average 1. */
int cafe_discrete_gamma(int K, double alpha, double* probs, double* multipliers);

/* ---- ancestral reconstruction ------------------------------------------ */

typedef struct {
    int32_t* node_count;         /* host [F][n_nodes] or NULL: reconstructed family size per node
                                    (reconstruction::get_node_count); leaves hold the observed count */
    double* node_mean;           /* host [F][n_nodes] or NULL: gamma sum_k p_k * state_k
                                    (get_weighted_averages); base: the state */
    int32_t* category_state;     /* host [K][F][n_nodes] or NULL: Pupko state per category (K = 1 for base) */
    double* root_max;            /* host [K][F] or NULL: largest root L (reconstructed iff > 0) */
    int exhaustive;              /* in: 1 = exact FP64 scan of every child state (no log2 filter) */
    int64_t n_failed;            /* out: (category, family) pairs whose root L is all 0 */
    double device_ms;            /* out: device time (CUDA events) */
} cafe_reconstruction;

/* Pupko joint ancestral reconstruction of every family of the set
 * (model::reconstruct_ancestral_states, src/base_model.cpp:133-170 and
 * src/gamma_core.cpp:290-339, over pupko_reconstructor::reconstruct_gene_family,
 * src/gene_family_reconstructor.cpp:161-190): one max-product pass per
 * gamma category at lambda * m_k, states 0..max_family_size, root sizes
 * 1..min(max_family_size, max_root_family_size). Uses the request's tree,
 * family set, model, lambdas, gamma categories and both bounds; precision,
 * dedupe and the error model are ignored (the reference reconstructs in
 * plain FP64 from the observed counts). Counts above max_family_size are
 * CAFE_ERR_INVALID. */
int cafe_reconstruct(cafe_ctx* ctx, const cafe_request* req, cafe_reconstruction* out);

/* compute_viterbi_sum (src/gene_family_reconstructor.cpp:390-430) for every
 * family and node: node_count[F][n_nodes] (host, e.g. from cafe_reconstruct)
 * in, out[F][n_nodes] (host) = the probability mass of child sizes below
 * max_family_size that are less likely than the reconstructed one given the
 * parent's (ties count half), under the request's own lambdas; NaN at the
 * root. */
int cafe_branch_probabilities(cafe_ctx* ctx, const cafe_request* req, const int32_t* node_count, double* out);

/* ---- p-values ------------------------------------------------------------ */

typedef struct {
    int n_simulations;           /* in: simulated families per root size (the reference uses 1000) */
    uint32_t seed;               /* in: seed of the std::mt19937 simulation stream (randomizer_engine) */
    double* pvalues;             /* host [F] out */
    double* conditional;         /* host [R][n_simulations] out, or NULL: sorted simulated likelihoods
                                    of root sizes 1..R */
    double* root_likelihood;     /* host [F][R] out, or NULL: observed root vectors (root sizes 1..R) */
    double device_ms;            /* out: device span from the first pruning launch to the last (it
                                    overlaps the host simulation) */
    double host_ms;              /* out: host time (matrix copies, simulation, sorting, p-values) */
    int device_sampling;         /* in: 0 = the reference's std::mt19937 stream drawn on the host (the
                                    reference's families and p-values, bit for bit); 1 = every simulated
                                    family drawn on the GPU from a counter-based generator seeded by
                                    `seed` (the same distributions, not the reference's stream: p-values
                                    agree in distribution only; at most 16,384 simulations per root size) */
} cafe_pvalues_out;

/* compute_pvalues (src/probability.cpp:376-570) at the request's own
 * lambdas (its multipliers are not used, as the estimate action passes the
 * model's base lambda, src/execute.cpp:166-171): for every root size
 * r = 1..max_root_family_size, n_simulations families are simulated down
 * the tree by sampling each child size from the parent's matrix row
 * (std::mt19937 + std::discrete_distribution, the reference's draws in its
 * order), pruned on the GPU with the root fixed at r and states 0..min(S,
 * largest size + max(50, largest / 5)); the observed families are pruned
 * with states 0..S and root sizes 1..R; each family's p-value is the
 * largest, over root sizes up to 1.25 x its largest count, of the share of
 * simulated likelihoods that do not exceed its own. */
int cafe_pvalues(cafe_ctx* ctx, const cafe_request* req, cafe_pvalues_out* out);

/* ---- simulation ------------------------------------------------------------ */

typedef struct {
    int n_families;              /* in */
    const int32_t* root_sizes;   /* in [n_families]: root size of each family
                                    (root_equilibrium_distribution::select_root_size) */
    uint32_t seed;               /* in: seed of the std::mt19937 stream (randomizer_engine) */
    int32_t* sizes;              /* host [n_families][n_nodes] out: every node's simulated size */
    double* lambdas;             /* host [n_families] out, or NULL: the family's (first) lambda */
} cafe_simulation;

/* The simulator action (simulator::simulate_processes / create_trial,
 * src/simulator.cpp:29-91) with LAMBDA_PERTURBATION_STEP_SIZE = 1: per
 * family the gamma model draws a rate category from the category
 * probabilities, then up to 50 attempts fill the tree in prefix order, each
 * child size drawn from its parent's row of the transition matrix (states
 * below max_family_size), leaves passed through the error model when
 * use_error_model is set (deviations -1, 0, +1; a leaf size past the
 * model's rows is CAFE_ERR_INVALID, where the reference throws), until every
 * child of the root has a descendant leaf with a nonzero size. Matrices come
 * from the context cache (built on the GPU); the draws run on the host in
 * the reference's order, so a seed reproduces the reference's families. */
int cafe_simulate(cafe_ctx* ctx, const cafe_request* req, cafe_simulation* io);

#ifdef __cplusplus
}
#endif
#endif
