/* CPU oracle for the CAFE5 likelihood hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, FP64 restatement of the reference algorithm, used by tests/,
 * by __graft_entry__.smoke() and by bench.py's cpu_baseline leg as the
 * checker. The product (cafe5_gb300/, include/) never links or calls it.
 *
 * Parity is pinned two ways (see tests/test_oracle_cpu.py):
 *   - against the known-answer values in the reference's own test.cpp
 *     (committed in tests/golden/reference_kats.json), and
 *   - against hex-float outputs of the reference itself, compiled from its
 *     own sources by oracle/Makefile (committed in tests/golden/ref_*.json,
 *     generated by tests/golden/make_golden.py).
 */
#ifndef CAFE_ORACLE_H
#define CAFE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A rooted tree as flat arrays. Node i has parent parent[i] (-1 for the
 * root). The children of a node are taken in increasing node index, which
 * is the reference's descendant order when nodes are numbered in Newick
 * order. leaf_col[i] is the counts column of leaf i (-1 for internal
 * nodes); lambda_index[i] selects the rate of the branch above node i. */
typedef struct {
    int n_nodes;
    const int* parent;
    const double* branch_length;
    const int* lambda_index;
    const int* leaf_col;
} oracle_tree;

double oracle_chooseln(double n, double r);
double oracle_bd_rate(int s, int c, double log_alpha, double coeff);
double oracle_transition(double lambda, double t, int s, int c);
void oracle_quantize(double lambda, double t, double* lambda_q, double* t_q);
int oracle_is_saturated(double t, double lambda);
void oracle_fill_matrix(double lambda, double t, int size, double* out);
void oracle_multiply(const double* m, int size, const double* v, int s_min, int s_max,
                     int c_min, int c_max, double* result);

/* get_gamma (src/gamma.cpp:225-241 over discrete_gamma, :15-52, with
 * median = 1 and beta = alpha): K category probabilities (1/K each) and the
 * median rate multipliers, through AS 91 (point_chi2), AS 32
 * (incomplete_gamma) and AS 70 (point_normal), step for step so the
 * multipliers carry the reference's bits. Returns 0, or -1 for alpha <= 0
 * or K < 1. */
int oracle_discrete_gamma(int K, double alpha, double* probs, double* multipliers);

/* Prunes one family with matrices given per node (node_matrix[i] is the
 * size x size matrix of the branch above node i; unused for the root).
 * Writes the root vector (R values, index j <-> root size j+1). With
 * scaled != 0, every node vector is renormalised by a power of two and the
 * accumulated natural-log scale is written to *log_scale. */
int oracle_prune(const oracle_tree* tree, const int32_t* counts_row,
                 const double* const* node_matrix, int size,
                 const double* err_rows, int err_nrows, int err_ndev,
                 int S, int R, int scaled, double* root_out, double* log_scale);

/* One infer_family_likelihoods call.
 *   model        0 = base model, 1 = gamma model
 *   lambda_kind  0 = single_lambda (valid iff > 0), 1 = multiple_lambda
 *                (valid iff none < 0)
 *   S, R         global max_family_size / max_root_family_size
 *   fam_S, fam_R optional per-family bounds (binned mode); NULL = global
 *   prior        prior[j] for root index j (already float-rounded), 0 past n_prior
 *   dedupe       prune identical count rows once (base model)
 *   scaled       0 = reference arithmetic, 1 = per-node power-of-two rescale
 * Outputs fam_lnl[F], cat_lh[F*K] (natural log of each category term for
 * the gamma model; NULL allowed) and *total (= -sum lnL, +inf on the
 * reference's rejection paths). Returns 0, or -1 on invalid input. */
int oracle_score(const oracle_tree* tree, const int32_t* counts, int64_t F, int n_leaves,
                 const double* lambdas, int n_lambdas, int lambda_kind,
                 int K, const double* multipliers, const double* cat_probs,
                 const double* prior, int n_prior,
                 const double* err_rows, int err_nrows, int err_ndev,
                 int S, int R, const int* fam_S, const int* fam_R,
                 int model, int dedupe, int scaled, int n_threads,
                 double* fam_lnl, double* cat_lh, double* total);

/* Pupko joint ancestral reconstruction (model::reconstruct_ancestral_states,
 * src/base_model.cpp:133-170 and src/gamma_core.cpp:290-339, over
 * reconstruct_gene_family, src/gene_family_reconstructor.cpp:161-190).
 *   K = 0        base model (one pass at the lambdas themselves)
 *   K >= 1       gamma model: one pass per category at lambda * m_k
 *   S, R         max_family_size / max_root_family_size
 * Outputs state[K'][F][n_nodes] (K' = max(K, 1); leaves hold their observed
 * count), mean[F][n_nodes] (gamma: sum_k p_k * state_k; base: the state),
 * node_count[F][n_nodes] (mean rounded half away from zero) and
 * root_max[K'][F] (largest root L; the reference calls a family
 * reconstructed iff > 0). mean / node_count may be NULL. */
int oracle_reconstruct(const oracle_tree* tree, const int32_t* counts, int64_t F, int n_leaves,
                       const double* lambdas, int n_lambdas, int K, const double* multipliers,
                       const double* cat_probs, const double* prior, int n_prior, int S, int R,
                       int n_threads, int32_t* state, double* mean, int32_t* node_count, double* root_max);

/* compute_viterbi_sum (src/gene_family_reconstructor.cpp:390-430) for every
 * family and node from reconstructed node counts [F][n_nodes]; NaN at the
 * root. */
int oracle_branch_probabilities(const oracle_tree* tree, const double* lambdas, int n_lambdas,
                                const int32_t* node_count, int64_t F, int S, int R, double* out);

/* compute_pvalues (src/probability.cpp:376-570): n_sim families simulated
 * per root size 1..R from a std::mt19937 seeded with `seed` (the
 * reference's randomizer_engine draws, in its order), pruned with the root
 * fixed; observed families pruned with states 0..S and root sizes 1..R.
 * Outputs pvalues[F], and optionally the sorted conditional distributions
 * conditional[R][n_sim] and the observed root vectors root_vectors[F][R]. */
int oracle_pvalues(const oracle_tree* tree, const int32_t* counts, int64_t F, int n_leaves,
                   const double* lambdas, int n_lambdas, int S, int R, int n_sim, uint32_t seed,
                   double* pvalues, double* conditional, double* root_vectors);

/* The simulator action (src/simulator.cpp:29-91) from a std::mt19937 seeded
 * with `seed`: K = 0 base model, K >= 1 gamma (a category drawn per family);
 * root_sizes[n_fam] are the prior's sizes (select_root_size); err_rows
 * [err_nrows][3] or NULL, err_max_count the error model's largest count.
 * Outputs sizes_out[n_fam][n_nodes] and lambda_out[n_fam] (the family's
 * first lambda). Returns 0, -1 on bad input, -2 where the reference throws
 * (a simulated leaf size outside the error model). */
int oracle_simulate(const oracle_tree* tree, const double* lambdas, int n_lambdas, int K,
                    const double* multipliers, const double* cat_probs, const double* err_rows,
                    int err_nrows, int err_ndev, int err_max_count, int S, int R, int n_fam,
                    const int32_t* root_sizes, uint32_t seed, int32_t* sizes_out, double* lambda_out);

#ifdef __cplusplus
}
#endif
#endif
