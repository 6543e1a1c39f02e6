// Shared definitions of the GB300 CAFE5 likelihood kernels.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace cafe {

// Transition-matrix build job: one (lambda, t) matrix of side `size`,
// computed at the quantized values (matrix_cache_key, src/matrix_cache.h:49-62).
struct MatrixJob {
    double lambda;    // quantized lambda
    double t;         // quantized branch length
    double* dst;      // FP64 row-major size x size, M[parent s][child c]
    float* colT;      // optional: FP32 transposed, column-normalised (size x size), or null
    int32_t* colE;    // optional: per-column power-of-two exponent (size), or null
    uint16_t* hi;     // optional: BF16 hi part, row-major (size x ld_bf16), or null
    uint16_t* lo;     // optional: BF16 lo part
    int size;
    int ld_bf16;      // leading dimension of hi/lo in elements (multiple of 8)
};

// Work tile of the pruning kernels: `count` families (indices into the
// request's family permutation starting at `first`) scored in category `k`
// with state bound S (vectors of S + 1 states) and R root rows starting at
// root size `root_lo` (0 means 1: root sizes 1..R).
struct PruneTile {
    int first;
    int count;
    int k;
    int S;
    int R;
    int root_lo;
    int pad[2];
};

// Flattened tree for the kernels, in one device allocation.
//   internal[i]                internal nodes in post-order (root last)
//   cstart[i]..cstart[i+1]     children of internal[i] (indices into child[])
//   child[j]                   child node id
//   leaf_col[node]             counts column of a leaf, -1 for internal
//   slot[node]                 scratch slot of an internal node
struct TreePlan {
    int n_nodes;
    int n_internal;
    int n_leaves;
    int root;
    int n_slots;
    int max_children;
    const int32_t* internal;
    const int32_t* cstart;
    const int32_t* child;
    const int32_t* leaf_col;
    const int32_t* slot;
};

constexpr int kMaxNodes = 512;

}  // namespace cafe

// Launch wrappers implemented in the .cu files (host side).
namespace cafe {

cudaError_t launch_matrix_build(const MatrixJob* d_jobs, int n_jobs, int max_size, cudaStream_t s);

// One-time per-device kernel attributes (shared-memory limits).
cudaError_t tc_kernels_init();

struct Prune64Args {
    TreePlan plan;
    const PruneTile* tiles;
    int n_tiles;
    const int32_t* counts;       // [F][n_leaves]
    const int64_t* perm;         // family index of each tile slot
    const double* const* mats;   // [K][n_nodes] FP64 matrix per (category, node)
    int ld_mat;                  // row stride of every FP64 matrix (= matrix size)
    const double* prior;         // [n_prior]
    int n_prior;
    const double* err;           // [err_rows][err_ndev] or null
    int err_rows;
    int err_ndev;
    const int32_t* fam_R;        // per-family root bound, or null (tile R)
    double* scratch;             // n_ctas * per_cta doubles
    int64_t scratch_per_cta;
    int scaled;                  // per-node power-of-two rescale
    int model;                   // 0 base, 1 gamma
    double* out;                 // [F][K]: base lnl, gamma category value
    int K;                       // categories (all candidates' categories of a batch)
    const double* cat_probs;     // [K]
    int tile_families;           // families per tile (<= 32)
    int W;                       // max vector length over tiles (S + 1 or R)
    const int32_t* n_tiles_dev;  // optional: tile count read from device memory
    const uint8_t* term_mask;    // optional [F][K]: only the terms set here are written
    double* root_out;            // optional (unscaled runs): root vector of every family,
                                 // root_out[f * root_ld + j] = L(root size root_lo + j); no reduction
    int root_ld;
};

cudaError_t launch_prune64(const Prune64Args& a, int n_ctas, cudaStream_t s);

// The same walk with one family per tile (count 1) and a thread-block
// cluster of `cl` CTAs per family (rows split across the cluster); W is the
// vector length of the launch's bin. `n_clusters` clusters loop over the tiles.
size_t prune64_cluster_smem(int n_slots, int W);
size_t prune64_cluster_max_smem();
cudaError_t prune64_cluster_init();
cudaError_t launch_prune64_cluster(const Prune64Args& a, int cl, int n_clusters, cudaStream_t s);

struct FinishArgs {
    int64_t F;
    int K;                       // categories per candidate (1 for the base model)
    int n_cand;                  // candidates scored together (>= 1)
    int model;
    int scaled;
    const double* cat;           // [F][n_cand][K]: gamma terms (linear if !scaled, log if scaled); base: lnl
    const int64_t* ref;          // dedupe reference per family, or null
    double* family_lnl;          // [n_cand][F] out, or null
    double* total;               // [n_cand] out, or null
    int32_t* n_failed;           // [n_cand] out
    double* part_sum;            // [n_cand][2 * finish_parts(F)] workspace
    int32_t* part_cnt;           // [n_cand][2 * finish_parts(F)] workspace
    const int32_t* status;       // optional: nonzero -> total = NaN
};

int finish_parts(int64_t F);
cudaError_t launch_finish(const FinishArgs& a, cudaStream_t s);

// ---- tensor-core (TF32x3) path ----
// Conversion of one cached FP64 matrix into the tensor-core operands.
struct ConvertJob {
    const double* src;   // FP64 row-major, leading dimension `ld`
    int ld;
    int mat;             // index into the request's converted arrays
    int what;            // 1: the TF32 hi/lo operands (an internal child's branch), 2: the
                         // FP32 transpose (a leaf's branch); both where a matrix serves both
};

struct TcBuffers {
    float* hi;           // [n_mat][Wm][Wm] TF32 hi part, row-major M[s][c]
    float* lo;           // [n_mat][Wm][Wm] TF32 lo part
    float* tr;           // [n_mat][Wm][Wm] FP32 transpose: tr[c][s] = M[s][c] (leaf factors); with an
                         // error model, the leaf factor of an observed count c: sum over deviations d of
                         // w_d(c) M[s][c + d] (columns 0 .. Wm - 1, zero weights skipped), summed in FP32
                         // in deviation order
    int Wm;
    const double* err;   // [err_rows][err_ndev] error model, or null
    int err_rows, err_ndev;
};
constexpr int kMaxErrHalf = 8;   // deviations up to +-8 fold into the transposed leaf rows

cudaError_t launch_convert_tc(const ConvertJob* d_jobs, int n_jobs, TcBuffers b, cudaStream_t s);

constexpr int kPhases = 18;   // k_prune_tc phase counters (CAFE_TC_PHASES)

struct PruneTcArgs {
    TreePlan plan;
    const PruneTile* tiles;      // 128-family tiles; S = W - 1 of the tile's bin
    int n_tiles;
    const int32_t* counts;
    const int64_t* perm;
    const int32_t* mat_index;    // [K][n_nodes] converted-matrix index (-1 for the root); bit 30 set
                                 // when the key is saturated
    int Wm;                      // pitch of matrices and node vectors (elements)
    const float* mat_tr;         // [n_mat][Wm][Wm] FP32 transposed matrices (row c = column c of M)
    float* vec;                  // node vectors (FP32), rows = CTA x slot x 128 families
    int n_slots;
    const double* prior;
    int n_prior;
    const double* err;
    int err_rows;
    int err_ndev;
    const int32_t* fam_R;
    double* out;                 // [F][K] natural log of each category term
    int K;
    int model;                   // 0 base (a zero family is -inf), 1 gamma (a zero family is NaN: failed)
    const double* cat_probs;
    int32_t* flags;              // [F] set when a family must be recomputed in FP64
    uint8_t* term_flags;         // [F][K] set with it for the category term that needs the recompute
    float* out_err;              // [F][K] bound on the relative error of each category term from FP32
                                 // range loss (values below 2^-126 flushed), or null
    int32_t* status;             // [1] nonzero when a bounded wait gave up
    int tmem_cols;
    int nsplit;                  // 1: one CTA per tile; 2 or 4: a cluster of nsplit CTAs per tile, CTA h
                                 // computing states [h W/nsplit, (h + 1) W/nsplit) of every node
    int Ws;                      // B rows per stage: the launch's bin width / nsplit
    int stages;                  // pipeline stages (1 to 4)
    int64_t vrow_base;           // first node-vector row of this launch
    unsigned long long* phase_clocks;   // optional [kPhases]: SM clocks of thread 0 in child setup, GEMMs,
                                        // epilogue, root bookkeeping, end-of-node barrier; tile-nodes;
                                        // then the GEMM chain's parts (k_prune_tc.cu)
    int* tile_counter;           // one CTA per tile (nsplit 1): zeroed tile counter the CTAs take
                                 // tiles from; null: a fixed stride
    int debug_wait_limit;        // > 0: the wait for a node's GEMMs gives up after this many polls
                                 // minus one (tests of the time-out path); 0: the default bound
};

// Tensor maps travel by value (__grid_constant__); the host encodes them.
// Operand loads use prune_tc_kchunk()-column boxes (mat, vec; 128-byte
// swizzle for 32 columns, 64-byte for 16); the epilogue stores node vectors
// in 32-column boxes in the 128-byte swizzle (vst). Vector boxes are one
// tile's 128 rows. mat is 3D: the TF32 hi and lo matrices, one buffer
// [2][n_mat Wm][Wm], in boxes of the launch's Ws rows x both halves. tr:
// the FP32 transposed matrices in boxes of 32 columns x the launch's W
// rows (leaf blocks of bins up to 64 states).
struct TcMaps {
    CUtensorMap mat, vec, vst, tr;
};

cudaError_t launch_prune_tc(const TcMaps& maps, const PruneTcArgs& a, int n_ctas, size_t smem, cudaStream_t s);

// ---- device-sampled p-value simulations (k_pvalue.cu) ----
struct SimDrawArgs {
    const double* cdf;           // [n_nodes][n_ps][S] cumulative weights of each (node, parent size) row
    const int32_t* prefix;       // [n_nodes] prefix order
    const int32_t* parent;       // [n_nodes], -1 at the root
    const int32_t* leaf_col;     // [n_nodes] counts column of a leaf, -1 for internal nodes
    int n_nodes, n_leaves, root, n_ps, S, n_sim;
    int64_t n_families;          // R x n_sim; family fi has root size fi / n_sim + 1
    uint64_t key;                // sim_seed_key(seed)
    int32_t* sizes;              // [n_families][n_nodes] scratch
    int32_t* counts;             // [n_families][n_leaves] out: leaf counts
    int32_t* keys;               // [n_families] out: root index x (S + 1) + state bound
    int32_t* hist;               // [R x (S + 1)] zeroed in, families per key out
};
struct SimPlanArgs {
    const int32_t* hist;
    int n_keys;
    int S;
    int32_t* cursor;             // [n_keys] out: first family slot of each key (the scatter's cursor)
    PruneTile* tiles;            // [max_tiles] out: 32-family tiles of equal (root size, bound)
    int64_t max_tiles;
    int32_t* n_tiles;            // [1] out
};
struct PvalueSearchArgs {
    const int32_t* counts;       // [F][n_leaves] observed families
    int64_t F;
    int n_leaves;
    const double* obs;           // [F][R] observed root values (root sizes 1..R)
    const double* sorted;        // [R][n_sim] sorted simulated values
    int R, n_sim;
    double* out;                 // [F] p-values
};
constexpr int kSortRowsMaxP = 16384;   // simulations per root size the device sort takes
uint64_t sim_seed_key(uint32_t seed);
cudaError_t pvalue_kernels_init();
cudaError_t launch_cdf_build(const double* const* mats, int n_nodes, int msize, int S, int n_ps, double* cdf,
                             cudaStream_t s);
cudaError_t launch_sim_draw(const SimDrawArgs& a, cudaStream_t s);
cudaError_t launch_sim_plan(const SimPlanArgs& a, cudaStream_t s);
cudaError_t launch_sim_scatter(const int32_t* keys, int64_t n, int32_t* cursor, int64_t* perm, cudaStream_t s);
cudaError_t launch_sort_rows(double* v, int rows, int n, cudaStream_t s);
cudaError_t launch_pvalue_search(const PvalueSearchArgs& a, cudaStream_t s);

// Families whose tensor-core result may have lost accuracy to FP32's range:
// for every (family, candidate), the category terms' range-error bounds
// weighted by the terms' shares of the family likelihood; over
// tau x |lnL| the family is flagged for the FP64 recompute.
struct RangeFlagArgs {
    const double* cat;           // [F][K] natural log of each category term
    const float* err;            // [F][K] relative bound of each term
    int64_t F;
    int K;                       // combined (candidate, category) indices
    int KC;                      // categories per candidate
    double tau;
    int32_t* flags;              // [F]
    uint8_t* term_flags;         // [F][K]: the terms of a flagged family whose share of the bound is over
                                 // tau / (2 KC), which the FP64 pass recomputes (the rest stay under tau / 2)
    int32_t* any_flag;           // set to 1 when a family is flagged
};
cudaError_t launch_range_flags(const RangeFlagArgs& a, cudaStream_t s);
size_t prune_tc_smem_bytes(int Ws, int n_slots, int stages, int n_internal);
int prune_tc_kchunk();   // K columns per operand box of k_prune_tc (its load maps' box width)
int prune_tc_max_smem(int nsplit = 1);   // dynamic shared memory one k_prune_tc CTA may use (per split)

// Device-side plan of the FP64 recompute of flagged category terms:
// k_fallback_plan compacts the flagged families of each listed bin (in
// permutation order) into fb_perm; k_fallback_tiles then writes a 32-family
// tile for every (chunk of 32 compacted families, listed category) in which
// some family has that term flagged (tile order is immaterial: each tile
// writes its own terms). out_counts[0] = families, out_counts[1] = tiles.
struct FallbackPlanArgs {
    const int32_t* flags;        // [F]
    const uint8_t* term_flags;   // [F][K]
    int K;                       // combined (candidate, category) indices
    const int64_t* perm;         // [F] bin order
    int n_bins;
    int bin_width[16];
    int64_t bin_first[16];
    int64_t bin_count[16];
    const int32_t* cats;         // [n_cats] category indices to recompute
    int n_cats;
    int64_t* fb_perm;            // [F]
    int64_t* fb_bins;            // [2 * 16]: start and count of each bin's families in fb_perm
    PruneTile* fb_tiles;         // [n_cats * (F / 32 + n_bins + 1)]
    int32_t* out_counts;         // [2]
    const int32_t* any_flag;     // optional: zero means no family is flagged
};
cudaError_t launch_fallback_plan(const FallbackPlanArgs& a, cudaStream_t s);

// ---- Pupko joint reconstruction (k_reconstruct.cu) ----
// One CTA walks 32-family tiles of one category up the tree; node L
// vectors (S + 1 states) live in per-CTA scratch, the argmax tables C in
// per-CTA int32 scratch; the backtrack writes every node's state.
struct PupkoArgs {
    TreePlan plan;
    const PruneTile* tiles;      // first family, count (<= 32), category k
    int n_tiles;
    const int32_t* counts;       // [F][n_leaves]
    int64_t F;
    const double* const* mats;   // [K][n_nodes] FP64 matrix per (category, node)
    const float* const* lmats;   // [K][n_nodes] transposed log2 of the internal non-root nodes' matrices,
                                 // (S + 1) x (S + 1) (launch_log2_matrices), null elsewhere
    int ld_mat;                  // matrix side (>= S + 1)
    const double* prior;         // prior[j] = P(root size j)
    int n_prior;
    int S;                       // max_family_size: states 0..S
    int root_len;                // min(S, R) + 1: root sizes 1..root_len - 1
    double* scratch;             // n_ctas * scratch_per_cta doubles
    int64_t scratch_per_cta;     // pupko_scratch_doubles()
    int32_t* cscratch;           // n_ctas * c_per_cta
    int64_t c_per_cta;           // pupko_c_entries()
    int32_t* state;              // [K][F][n_nodes] out
    double* root_max;            // [K][F] out
    int32_t* n_failed;           // [1] out: (category, family) pairs with root max 0
    int exhaustive;              // 1: exact FP64 scan of every child state
};
cudaError_t launch_pupko(const PupkoArgs& a, int n_ctas, cudaStream_t s);
cudaError_t launch_log2_matrices(const double* const* src, float* const* dst, int n_mats, int n, int ld,
                                 cudaStream_t s);
size_t pupko_scratch_doubles(const TreePlan& P, int S);
size_t pupko_c_entries(const TreePlan& P, int S);
cudaError_t launch_recon_counts(const int32_t* state, int64_t F, int n_nodes, int K, const double* cat_probs,
                                int gamma, const int32_t* leaf_col, double* mean, int32_t* node_count,
                                cudaStream_t s);

struct BranchProbArgs {
    const int32_t* parent;       // [n_nodes], -1 at the root
    int n_nodes;
    int64_t F;
    const int32_t* node_count;   // [F][n_nodes]
    const double* const* mats;   // [n_nodes] matrix of the branch above each node
    int ld_mat;
    int S;                       // child sizes 0..S-1 are summed
    double* out;                 // [F][n_nodes], NaN at the root
    int32_t* n_bad;              // [1] counts outside the matrices
};
cudaError_t launch_branch_prob(const BranchProbArgs& a, cudaStream_t s);

}  // namespace cafe
