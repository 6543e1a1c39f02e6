// CPU oracle for the CAFE5 p-values -- TEST INFRASTRUCTURE ONLY.
//
// Restates compute_pvalues (src/probability.cpp:376-570) with the
// reference's random stream: a std::mt19937 seeded by the caller drives
// the same draws in the same order (create_family /
// set_weighted_random_family_size, :351-373 and :449-476, sampling each
// child size with std::discrete_distribution over the parent's matrix row,
// matrix::select_random_y, src/matrix_cache.cpp:60-66), and the simulated
// and observed families are pruned with the reference's bounds
// (compute_family_probabilities, :376-423). Matrices come from
// oracle_fill_matrix (the reference formula, bit-exact).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <random>
#include <vector>

#include "cafe_oracle.h"

namespace {

struct Tree {
    int n;
    std::vector<int> parent, lam, leaf_col;
    std::vector<double> t;
    std::vector<std::vector<int>> kids;   // descendant order = increasing node index
    int root = -1;
    std::vector<int> prefix;              // clade::apply_prefix_order (src/clade.cpp:275-291)
    std::vector<int> post;                // children before parents
};

Tree make_tree(const oracle_tree* o) {
    Tree T;
    T.n = o->n_nodes;
    T.parent.assign(o->parent, o->parent + T.n);
    T.lam.assign(o->lambda_index, o->lambda_index + T.n);
    T.leaf_col.assign(o->leaf_col, o->leaf_col + T.n);
    T.t.assign(o->branch_length, o->branch_length + T.n);
    T.kids.resize(T.n);
    for (int v = 0; v < T.n; ++v) {
        if (T.parent[v] < 0) T.root = v;
        else T.kids[T.parent[v]].push_back(v);
    }
    std::vector<int> st{T.root};
    while (!st.empty()) {
        int v = st.back();
        st.pop_back();
        T.prefix.push_back(v);
        for (auto it = T.kids[v].rbegin(); it != T.kids[v].rend(); ++it) st.push_back(*it);
    }
    T.post.assign(T.prefix.rbegin(), T.prefix.rend());
    return T;
}

// compute_node_probability (src/probability.cpp:175-234) for one family:
// leaves one-hot at their count, internal nodes over states 0..m, the root
// over sizes lo..hi (index s - lo). Sums in child-state order.
std::vector<double> prune(const Tree& T, const std::vector<int>& leaf_size, const std::vector<const double*>& mats,
                          int size, int m, int lo, int hi, int root_len) {
    std::vector<std::vector<double>> L(T.n);
    std::vector<double> res;
    for (int v : T.post) {
        if (T.kids[v].empty()) {
            L[v].assign(m + 1, 0.0);
            L[v][leaf_size[v]] = 1.0;
            continue;
        }
        const bool root = v == T.root;
        const int len = root ? root_len : m + 1;
        L[v].assign(len, 1.0);
        for (int ch : T.kids[v]) {
            const double* M = mats[ch];
            res.assign(std::max(len, hi - lo + 1), 0.0);
            const int s0 = root ? lo : 0, s1 = root ? hi : m;
            for (int s = s0; s <= s1; ++s) {
                double acc = 0;
                for (int c = 0; c <= m; ++c) acc += M[(size_t)s * size + c] * L[ch][c];
                res[s - s0] = acc;
            }
            for (int i = 0; i < len; ++i) L[v][i] *= res[i];
        }
    }
    return L[T.root];
}

}  // namespace

extern "C" int oracle_pvalues(const oracle_tree* tree, const int32_t* counts, int64_t F, int n_leaves,
                              const double* lambdas, int n_lambdas, int S, int R, int n_sim, uint32_t seed,
                              double* pvalues, double* conditional, double* root_vectors) {
    if (!tree || tree->n_nodes < 2 || F < 0 || n_lambdas < 1 || S < 1 || R < 1 || n_sim < 1) return -1;
    Tree T = make_tree(tree);
    const int size = std::max(S, R) + 1;
    // matrix of the branch above every node, at the quantised key values
    std::map<std::pair<long, long>, std::vector<double>> cache;
    std::vector<const double*> mats(T.n, nullptr);
    std::vector<int> saturated(T.n, 0);
    for (int v = 0; v < T.n; ++v) {
        if (T.parent[v] < 0) continue;
        const double lam = lambdas[T.lam[v]];
        const long lq = (long)(lam * 1000000000), tq = (long)(T.t[v] * 1000);
        auto& m = cache[{lq, tq}];
        if (m.empty()) {
            m.resize((size_t)size * size);
            oracle_fill_matrix((double)lq / 1000000000.0, (double)tq / 1000.0, size, m.data());
        }
        mats[v] = m.data();
        saturated[v] = oracle_is_saturated(T.t[v], lam);
    }

    std::mt19937 engine(seed);
    std::vector<std::vector<double>> cd(R);
    std::vector<int> sizes(T.n);
    for (int i = 0; i < R; ++i) {
        const int r = i + 1;
        std::vector<std::vector<int>> fams(n_sim);
        for (int k = 0; k < n_sim; ++k) {
            // create_family: sizes down the tree in prefix order
            sizes[T.root] = r;
            for (int v : T.prefix) {
                if (v == T.root) continue;
                const int ps = sizes[T.parent[v]];
                int c = 0;
                if (ps > 0) {
                    if (saturated[v]) {
                        std::uniform_int_distribution<int> d(0, S - 1);
                        c = d(engine);
                    }
                    const double* row = mats[v] + (size_t)ps * size;
                    std::discrete_distribution<int> d(row, row + S);
                    c = d(engine);
                }
                sizes[v] = c;
            }
            fams[k] = sizes;
        }
        // compute_family_probabilities: each family pruned with the root fixed at r
        std::vector<double>& out = cd[i];
        out.resize(n_sim);
#pragma omp parallel for schedule(dynamic, 4)
        for (int k = 0; k < n_sim; ++k) {
            const std::vector<int>& z = fams[k];
            const int mx = *std::max_element(z.begin(), z.end());
            const int m = std::min(S, mx + std::max(50, mx / 5));
            std::vector<double> root = prune(T, z, mats, size, m, r, r, R + 1);
            out[k] = *std::max_element(root.begin(), root.end());
        }
        std::sort(out.begin(), out.end());
        if (conditional) std::memcpy(conditional + (size_t)i * n_sim, out.data(), sizeof(double) * n_sim);
    }

    // observed families: global bounds, root sizes 1..R; find_best_pvalue
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t f = 0; f < F; ++f) {
        std::vector<int> z(T.n, 0);
        int fmax = 0;
        for (int v = 0; v < T.n; ++v)
            if (T.kids[v].empty()) {
                z[v] = counts[(size_t)f * n_leaves + T.leaf_col[v]];
                fmax = std::max(fmax, z[v]);
            }
        std::vector<double> root = prune(T, z, mats, size, S, 1, R, R);
        if (root_vectors) std::memcpy(root_vectors + (size_t)f * R, root.data(), sizeof(double) * R);
        std::vector<double> pv(R, 0.0);
        const int check = std::min(R, (int)std::rint(fmax * 1.25));
        for (int j = 0; j < check; ++j) {
            const std::vector<double>& d = cd[j];
            size_t idx = d.size() - 1;
            auto b = std::upper_bound(d.begin(), d.end(), root[j]);
            if (b != d.end()) idx = b - d.begin();
            pv[j] = idx / (double)d.size();
        }
        pvalues[f] = *std::max_element(pv.begin(), pv.end());
    }
    return 0;
}

// The simulator action (src/simulator.cpp:29-91): per family, the gamma
// model first picks a rate category (gamma_model::get_simulation_lambda,
// src/gamma_core.cpp:91-95, a std::discrete_distribution over the category
// probabilities); then up to 50 attempts (create_trial) set the root to
// root_sizes[f] and every other node, in prefix order, from its parent's
// matrix row (set_weighted_random_family_size, src/probability.cpp:449-476),
// leaves passed through the error model (adjust_for_error_model, :478-500),
// until the family exists at the root (gene_family::exists_at_root,
// src/gene_family.cpp:62-91).
extern "C" int oracle_simulate(const oracle_tree* tree, const double* lambdas, int n_lambdas, int K,
                               const double* multipliers, const double* cat_probs, const double* err_rows,
                               int err_nrows, int err_ndev, int err_max_count, int S, int R, int n_fam,
                               const int32_t* root_sizes, uint32_t seed, int32_t* sizes_out, double* lambda_out) {
    if (!tree || tree->n_nodes < 2 || n_lambdas < 1 || S < 1 || R < 1 || n_fam < 0) return -1;
    if (err_rows && err_ndev != 3) return -1;
    Tree T = make_tree(tree);
    const int size = std::max(S, R) + 1;
    const bool gamma = K > 0;
    const int KK = gamma ? K : 1;
    std::map<std::pair<long, long>, std::vector<double>> cache;
    std::vector<const double*> mats((size_t)KK * T.n, nullptr);
    std::vector<int> saturated((size_t)KK * T.n, 0);
    for (int k = 0; k < KK; ++k)
        for (int v = 0; v < T.n; ++v) {
            if (T.parent[v] < 0) continue;
            const double lam = lambdas[T.lam[v]] * (gamma ? multipliers[k] : 1.0);
            const long lq = (long)(lam * 1000000000), tq = (long)(T.t[v] * 1000);
            auto& m = cache[{lq, tq}];
            if (m.empty()) {
                m.resize((size_t)size * size);
                oracle_fill_matrix((double)lq / 1000000000.0, (double)tq / 1000.0, size, m.data());
            }
            mats[(size_t)k * T.n + v] = m.data();
            saturated[(size_t)k * T.n + v] = oracle_is_saturated(T.t[v], lam);
        }
    std::mt19937 engine(seed);
    std::vector<int> z(T.n);
    std::vector<char> reg(T.n);
    for (int f = 0; f < n_fam; ++f) {
        int k = 0;
        if (gamma) {
            std::discrete_distribution<int> pick(cat_probs, cat_probs + K);
            k = pick(engine);
        }
        lambda_out[f] = lambdas[0] * (gamma ? multipliers[k] : 1.0);
        for (int attempt = 0; attempt < 50; ++attempt) {
            z[T.root] = root_sizes[f];
            for (int v : T.prefix) {
                if (v == T.root) continue;
                const int ps = z[T.parent[v]];
                int c = 0;
                if (ps > 0) {
                    if (saturated[(size_t)k * T.n + v]) {
                        std::uniform_int_distribution<int> d(0, S - 1);
                        c = d(engine);
                    }
                    const double* row = mats[(size_t)k * T.n + v] + (size_t)ps * size;
                    std::discrete_distribution<int> d(row, row + S);
                    c = d(engine);
                }
                if (T.kids[v].empty() && err_rows) {
                    if (c >= err_max_count) return -2;
                    const double* p = err_rows + (size_t)std::min(c, err_nrows - 1) * 3;
                    std::uniform_real_distribution<double> u(0.0, 1.0);
                    const double rnd = u(engine);
                    if (rnd < p[0]) c--;
                    else if (rnd > (1 - p[2])) c++;
                }
                z[v] = c;
            }
            std::fill(reg.begin(), reg.end(), 0);
            for (int v : T.post)
                if (T.kids[v].empty() && z[v] > 0)
                    for (int p = v; p >= 0 && !reg[p]; p = T.parent[p]) reg[p] = 1;
            bool all = true;
            for (int ch : T.kids[T.root]) all &= reg[ch] != 0;
            if (all) break;
        }
        std::memcpy(sizes_out + (size_t)f * T.n, z.data(), sizeof(int32_t) * T.n);
    }
    return 0;
}
