/* CPU oracle for the CAFE5 likelihood hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C FP64 restatement of the reference algorithm. Each function cites
 * the reference lines it follows (paths relative to the CAFE5 project).
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use
 * this file, and only as the checker / the timed CPU baseline.
 */
#include "cafe_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/probability.cpp:55-91. The reference serves lgamma(n) for integral
 * 0 <= n < 1024 from a table (lgamma2, init_lgamma_cache) and chooseln(n,
 * r) for integral n, r < 100 from a second table built from the first.
 * Both tables hold the values of the direct libm expressions, so caching
 * here changes speed only: the tables are filled once when the library is
 * loaded, and the sum is formed in the same order as the direct form. */
#define G_LGAMMA_N 1024
#define G_CHOOSE_N 100
static double g_lgamma_tab[G_LGAMMA_N];
static double g_choose_tab[G_CHOOSE_N][G_CHOOSE_N];

static double g_lgamma2(double n) {
    if (n >= 0 && n < G_LGAMMA_N && (n - (int)n < 0.00000000001)) return g_lgamma_tab[(int)n];
    return lgamma(n);
}

__attribute__((constructor)) static void g_tables_init(void) {
    for (int i = 0; i < G_LGAMMA_N; i++) g_lgamma_tab[i] = lgamma(i);
    for (int i = 0; i < G_CHOOSE_N; i++)
        for (int j = 0; j < G_CHOOSE_N; j++)
            g_choose_tab[i][j] = g_lgamma2(i + 1) - g_lgamma2(j + 1) - g_lgamma2(i - j + 1);
}

double oracle_chooseln(double n, double r) {
    if (r == 0 || (n == 0 && r == 0)) return 0;
    if (n <= 0 || r <= 0) return log(0.0);
    if (n < G_CHOOSE_N && r < G_CHOOSE_N && (n - (int)n < 0.00000000001) && (r - (int)r < 0.00000000001))
        return g_choose_tab[(int)n][(int)r];
    return g_lgamma2(n + 1) - g_lgamma2(r + 1) - g_lgamma2(n - r + 1);
}

/* src/probability.cpp:104-148: Eqn (1) of Hahn et al. 2005, one exp and
 * one pow per binomial term, summed in j order, clamped to [0, 1]. */
double oracle_bd_rate(int s, int c, double log_alpha, double coeff) {
    int m = c < s ? c : s;
    int s_add_c = s + c;
    double result = 0.0;
    for (int j = 0; j <= m; j++) {
        double t = oracle_chooseln(s, j) + oracle_chooseln(s_add_c - 1 - j, s - 1) +
                   (s_add_c - 2 * j) * log_alpha;
        result += exp(t) * pow(coeff, j);
    }
    if (result > 1.0) result = 1.0;
    if (result < 0.0) result = 0.0;
    return result;
}

/* src/probability.cpp:150-167 and src/matrix_cache.cpp:78-85 (parent size
 * 0 stays 0). */
double oracle_transition(double lambda, double t, int s, int c) {
    if (s == 0) return c == 0 ? 1.0 : 0.0;
    double alpha = lambda * t / (1 + lambda * t);
    double coeff = 1 - 2 * alpha;
    if (coeff > 0 && coeff != 1) return oracle_bd_rate(s, c, log(alpha), coeff);
    return 0.0;
}

/* ---- gamma discretisation (src/gamma.cpp) ----
 * Published algorithms (Applied Statistics AS 70, AS 32, AS 91) in the
 * order of operations the reference evaluates them. */

/* AS 70, src/gamma.cpp:187-203: rational approximation of the standard
 * normal quantile in y = sqrt(ln(1 / p1^2)). */
static double g_normal_quantile(double p) {
    static const double num[5] = {-.322232431088, -1.0, -.342242088547, -.0204231210245, -.453642210148e-4};
    static const double den[5] = {.0993484626060, .588581570495, .531103462366, .103537752850, .0038560700634};
    double p1 = p < 0.5 ? p : 1 - p;
    if (p1 < 1e-20) return -9999;
    double y = sqrt(log(1 / (p1 * p1)));
    double n = num[4], d = den[4];
    for (int i = 3; i >= 0; i--) {
        n = n * y + num[i];
        d = d * y + den[i];
    }
    double z = y + n / d;
    return p < 0.5 ? -z : z;
}

/* AS 32, src/gamma.cpp:66-125: I(x, p) by the series when x <= 1 or x < p,
 * else by the continued fraction (its convergents as the ratio of two
 * recurrences, both scaled down by 1e30 when they grow past it). The
 * continued fraction stops when two successive convergents agree within
 * 1e-8 absolute and relative, and returns with the earlier one. */
static double g_incomplete_gamma(double x, double p, double lng) {
    const double accurate = 1e-8, overflow = 1e30;
    if (x == 0) return 0;
    if (x < 0 || p <= 0) return -1;
    double factor = exp(p * log(x) - x - lng);
    if (!(x > 1 && x >= p)) {
        double gin = 1, term = 1, rn = p;
        for (;;) {
            rn += 1;
            term *= x / rn;
            gin += term;
            if (!(term > accurate)) break;
        }
        return gin * (factor / p);
    }
    double a = 1 - p, b = a + x + 1, term = 0;
    double pn[6] = {1, x, x + 1, x * (a + x + 1), 0, 0};
    double gin = pn[2] / pn[3];
    for (;;) {
        a += 1;
        b += 2;
        term += 1;
        double an = a * term;
        pn[4] = b * pn[2] - an * pn[0];
        pn[5] = b * pn[3] - an * pn[1];
        if (pn[5] != 0) {
            double rn = pn[4] / pn[5];
            double dif = fabs(gin - rn);
            if (dif <= accurate && dif <= accurate * rn) return 1 - factor * gin;
            gin = rn;
        }
        memmove(pn, pn + 2, 4 * sizeof(double));
        if (!(fabs(pn[2]) < overflow))
            for (int i = 0; i < 4; i++) pn[i] /= overflow;
    }
}

/* AS 91, src/gamma.cpp:138-185: chi-square(v) quantile; a starting value
 * (small v against -ln p, v <= 0.32 by Newton steps, else Wilson-Hilferty
 * through AS 70) refined by seventh-order steps on AS 32 until the
 * relative change is at most 5e-7. */
static double g_chi2_quantile(double prob, double v) {
    const double e = .5e-6, aa = .6931471805;
    if (prob < .000002 || prob > .999998 || v <= 0) return -1;
    double g = lgamma(v / 2), xx = v / 2, c = xx - 1, ch;
    if (v < -1.24 * log(prob)) {
        ch = pow((prob * xx * exp(g + xx * aa)), 1 / xx);
        if (ch - e < 0) return ch;
    } else if (v <= .32) {
        double a = log(1 - prob), q;
        ch = 0.4;
        do {
            q = ch;
            double p1 = 1 + ch * (4.67 + ch);
            double p2 = ch * (6.73 + ch * (6.66 + ch));
            double t = -0.5 + (4.67 + 2 * ch) / p1 - (6.73 + ch * (13.32 + 3 * ch)) / p2;
            ch -= (1 - exp(a + g + .5 * ch + c * aa) * p2 / p1) / t;
        } while (fabs(q / ch - 1) - .01 > 0);
    } else {
        double x = g_normal_quantile(prob), p1 = 0.222222 / v;
        ch = v * pow((x * sqrt(p1) + 1 - p1), 3.0);
        if (ch > 2.2 * v + 6) ch = -2 * (log(1 - prob) - c * log(.5 * ch) + g);
    }
    for (;;) {
        double q = ch, p1 = .5 * ch, t = g_incomplete_gamma(p1, xx, g);
        if (t < 0) return -1;
        double p2 = prob - t;
        t = p2 * exp(xx * aa + g + p1 - c * log(ch));
        double b = t / ch, a = 0.5 * t - b * c;
        double s1 = (210 + a * (140 + a * (105 + a * (84 + a * (70 + 60 * a))))) / 420;
        double s2 = (420 + a * (735 + a * (966 + a * (1141 + 1278 * a)))) / 2520;
        double s3 = (210 + a * (462 + a * (707 + 932 * a))) / 2520;
        double s4 = (252 + a * (672 + 1182 * a) + c * (294 + a * (889 + 1740 * a))) / 5040;
        double s5 = (84 + 264 * a + c * (175 + 606 * a)) / 2520;
        double s6 = (120 + c * (346 + 127 * c)) / 5040;
        ch += t * (1 + 0.5 * t * s1 - b * c * (s1 - b * (s2 - b * (s3 - b * (s4 - b * (s5 - b * s6))))));
        if (!(fabs(q / ch - 1) > e)) return ch;
    }
}

/* src/gamma.cpp:15-52 (median = 1) as get_gamma calls it (:225-241):
 * rate k = the Gamma(alpha, alpha) quantile at (2k + 1) / 2K, i.e.
 * point_chi2(., 2 alpha) / (2 alpha), rescaled so the rates sum to K. */
int oracle_discrete_gamma(int K, double alpha, double* probs, double* multipliers) {
    if (K < 1 || !(alpha > 0)) return -1;
    double beta = alpha, gap05 = 1.0 / (2.0 * K), factor = alpha / beta * K, t = 0;
    for (int i = 0; i < K; i++) multipliers[i] = g_chi2_quantile((i * 2.0 + 1) * gap05, 2.0 * alpha) / (2.0 * beta);
    for (int i = 0; i < K; i++) t += multipliers[i];
    for (int i = 0; i < K; i++) {
        multipliers[i] *= factor / t;
        probs[i] = 1.0 / K;
    }
    return 0;
}

/* src/matrix_cache.h:49-62: matrices are computed at lambda truncated to
 * 1e-9 and t truncated to 1e-3. */
void oracle_quantize(double lambda, double t, double* lambda_q, double* t_q) {
    long lq = (long)(lambda * 1000000000);
    long tq = (long)(t * 1000);
    *lambda_q = (double)lq / 1000000000.0;
    *t_q = (double)tq / 1000.0;
}

/* src/matrix_cache.cpp:107-111 */
int oracle_is_saturated(double t, double lambda) {
    double alpha = lambda * t / (1 + lambda * t);
    return (1 - 2 * alpha) < 0;
}

/* src/matrix_cache.cpp:113-163 for one key (lambda, t already quantized):
 * row 0 is delta(c, 0); rows s >= 1 are filled unless saturated. */
void oracle_fill_matrix(double lambda, double t, int size, double* out) {
    memset(out, 0, sizeof(double) * (size_t)size * (size_t)size);
    out[0] = 1.0;
    if (oracle_is_saturated(t, lambda)) return;
    for (int s = 1; s < size; s++)
        for (int c = 0; c < size; c++)
            out[(size_t)s * size + c] = oracle_transition(lambda, t, s, c);
}

/* src/matrix_cache.cpp:32-58 (the scalar branch; the BLAS branch is not
 * compiled in the reference build). */
void oracle_multiply(const double* m, int size, const double* v, int s_min, int s_max,
                     int c_min, int c_max, double* result) {
    for (int s = s_min; s <= s_max; s++) {
        double acc = 0;
        const double* row = m + (size_t)s * size;
        for (int c = c_min; c <= c_max; c++) acc += row[c] * v[c - c_min];
        result[s - s_min] = acc;
    }
}

/* Reverse-level order (src/clade.cpp:69-100): breadth-first from the root,
 * children in descendant order, then reversed. */
static int* reverse_level_order(const oracle_tree* tree, int** child_start_out, int** children_out) {
    int n = tree->n_nodes;
    int* nchild = calloc((size_t)n + 1, sizeof(int));
    int* start = calloc((size_t)n + 1, sizeof(int));
    int* children = malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int* fill = calloc((size_t)n + 1, sizeof(int));
    int root = -1;
    for (int i = 0; i < n; i++) {
        if (tree->parent[i] < 0) root = i;
        else nchild[tree->parent[i]]++;
    }
    for (int i = 0; i < n; i++) start[i + 1] = start[i] + nchild[i];
    for (int i = 0; i < n; i++)
        if (tree->parent[i] >= 0) {
            int p = tree->parent[i];
            children[start[p] + fill[p]++] = i;
        }
    int* queue = malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int head = 0, tail = 0;
    if (root >= 0) queue[tail++] = root;
    while (head < tail) {
        int v = queue[head++];
        for (int k = start[v]; k < start[v + 1]; k++) queue[tail++] = children[k];
    }
    int* order = malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < tail; i++) order[i] = queue[tail - 1 - i];
    free(queue);
    free(nchild);
    free(fill);
    *child_start_out = start;
    *children_out = children;
    return order;
}

static void rescale(double* v, int len, long* expo) {
    double mx = 0;
    for (int i = 0; i < len; i++)
        if (v[i] > mx) mx = v[i];
    if (mx > 0 && isfinite(mx)) {
        int e;
        frexp(mx, &e);
        for (int i = 0; i < len; i++) v[i] = ldexp(v[i], -e);
        *expo += e;
    }
}

typedef struct {
    const oracle_tree* tree;
    const int* order;
    const int* cstart;
    const int* children;
    int root;
} tree_view;

/* inference_prune (src/core.cpp:134-145) over compute_node_probability
 * (src/probability.cpp:175-234). vec is n_nodes * stride scratch, res is
 * stride scratch, expo is n_nodes scratch. */
static int prune_one(const tree_view* tv, const int32_t* counts_row, const double* const* node_matrix,
                     int size, const double* err_rows, int err_nrows, int err_ndev, int S, int R,
                     int scaled, double* vec, int stride, double* res, long* expo, double* root_out,
                     double* log_scale) {
    const oracle_tree* tree = tv->tree;
    int n = tree->n_nodes;
    for (int oi = 0; oi < n; oi++) {
        int v = tv->order[oi];
        double* L = vec + (size_t)v * stride;
        expo[v] = 0;
        if (tv->cstart[v] == tv->cstart[v + 1]) {
            /* leaf: src/probability.cpp:184-203 */
            int cnt = counts_row[tree->leaf_col[v]];
            for (int i = 0; i <= S; i++) L[i] = 0;
            if (cnt < 0 || cnt > S) return -1;
            if (err_rows) {
                const double* p = err_rows + (size_t)(cnt < err_nrows ? cnt : err_nrows - 1) * err_ndev;
                int offset = cnt - (err_ndev - 1) / 2;
                for (int i = 0; i < err_ndev; i++) {
                    if (offset + i < 0 || offset + i > S) continue;
                    L[offset + i] = p[i];
                }
            } else {
                L[cnt] = 1.0;
            }
        } else {
            int is_root = (v == tv->root);
            int len = is_root ? R : S + 1;
            for (int i = 0; i < len; i++) L[i] = 1;
            for (int k = tv->cstart[v]; k < tv->cstart[v + 1]; k++) {
                int ch = tv->children[k];
                const double* m = node_matrix[ch];
                if (!m) return -2;
                if (is_root) oracle_multiply(m, size, vec + (size_t)ch * stride, 1, R, 0, S, res);
                else oracle_multiply(m, size, vec + (size_t)ch * stride, 0, S, 0, S, res);
                for (int i = 0; i < len; i++) L[i] *= res[i];
                expo[v] += expo[ch];
            }
            if (scaled) rescale(L, len, &expo[v]);
        }
    }
    memcpy(root_out, vec + (size_t)tv->root * stride, sizeof(double) * (size_t)R);
    *log_scale = (double)expo[tv->root] * log(2.0);
    return 0;
}

int oracle_prune(const oracle_tree* tree, const int32_t* counts_row, const double* const* node_matrix,
                 int size, const double* err_rows, int err_nrows, int err_ndev, int S, int R,
                 int scaled, double* root_out, double* log_scale) {
    tree_view tv;
    int *cstart, *children;
    tv.tree = tree;
    tv.order = reverse_level_order(tree, &cstart, &children);
    tv.cstart = cstart;
    tv.children = children;
    tv.root = tv.order[tree->n_nodes - 1];
    int stride = (S + 1 > R ? S + 1 : R) + 4;
    double* vec = calloc((size_t)tree->n_nodes * stride, sizeof(double));
    double* res = calloc((size_t)stride + 1024, sizeof(double));
    long* expo = calloc((size_t)tree->n_nodes, sizeof(long));
    int rc = prune_one(&tv, counts_row, node_matrix, size, err_rows, err_nrows, err_ndev, S, R, scaled,
                       vec, stride, res, expo, root_out, log_scale);
    free(vec);
    free(res);
    free(expo);
    free((void*)tv.order);
    free(cstart);
    free(children);
    return rc;
}

/* ---- matrix cache: keys (long(lambda*1e9), long(t*1e3)) ---- */
typedef struct {
    long lq, tq;
    double* m;
} cache_entry;

static int find_key(const cache_entry* e, int n, long lq, long tq) {
    for (int i = 0; i < n; i++)
        if (e[i].lq == lq && e[i].tq == tq) return i;
    return -1;
}

int oracle_score(const oracle_tree* tree, const int32_t* counts, int64_t F, int n_leaves,
                 const double* lambdas, int n_lambdas, int lambda_kind, int K, const double* multipliers,
                 const double* cat_probs, const double* prior, int n_prior, const double* err_rows,
                 int err_nrows, int err_ndev, int S, int R, const int* fam_S, const int* fam_R, int model,
                 int dedupe, int scaled, int n_threads, double* fam_lnl, double* cat_lh, double* total) {
    int n = tree->n_nodes;
    if (n <= 0 || F < 0 || n_lambdas <= 0) return -1;
    double one = 1.0;
    if (model == 0) {
        K = 1;
        multipliers = &one;
    }
    if (K <= 0) return -1;

    /* lambda::is_valid (src/lambda.h:58-60, src/lambda.cpp:172-175) */
    int valid = 1;
    double largest = lambdas[0];
    for (int i = 0; i < n_lambdas; i++) {
        if (lambda_kind == 0 ? !(lambdas[i] > 0) : (lambdas[i] < 0)) valid = 0;
        if (lambdas[i] > largest) largest = lambdas[i];
    }
    /* distinct positive branch lengths, root branch included
     * (src/clade.cpp:236-245) */
    double* bl = malloc(sizeof(double) * (size_t)n);
    int nbl = 0;
    double longest = 0;
    for (int i = 0; i < n; i++) {
        double t = tree->branch_length[i];
        if (!(t > 0)) continue;
        int dup = 0;
        for (int j = 0; j < nbl; j++)
            if (bl[j] == t) dup = 1;
        if (!dup) bl[nbl++] = t;
        if (t > longest) longest = t;
    }
    /* base_model.cpp:56-60; gamma_core.cpp:123-141, 174-178 */
    if (!valid || (model == 1 && nbl > 0 && oracle_is_saturated(longest, largest))) {
        free(bl);
        *total = INFINITY;
        for (int64_t f = 0; f < F; f++) fam_lnl[f] = NAN;
        return 0;
    }

    int Smax = S, Rmax = R;
    if (fam_S) {
        Smax = 0;
        Rmax = 0;
        for (int64_t f = 0; f < F; f++) {
            if (fam_S[f] > Smax) Smax = fam_S[f];
            if (fam_R[f] > Rmax) Rmax = fam_R[f];
        }
    }
    int size = (Rmax > Smax ? Rmax : Smax) + 1; /* base_model.cpp:65 */

    /* precalculate_matrices for every (lambda_i * m_k, t) */
    int cap = K * n_lambdas * (nbl > 0 ? nbl : 1);
    cache_entry* cache = calloc((size_t)cap, sizeof(cache_entry));
    int ncache = 0;
    for (int k = 0; k < K; k++)
        for (int i = 0; i < n_lambdas; i++)
            for (int b = 0; b < nbl; b++) {
                double lam = lambdas[i] * multipliers[k];
                long lq = (long)(lam * 1000000000), tq = (long)(bl[b] * 1000);
                if (find_key(cache, ncache, lq, tq) >= 0) continue;
                cache[ncache].lq = lq;
                cache[ncache].tq = tq;
                cache[ncache].m = malloc(sizeof(double) * (size_t)size * size);
                ncache++;
            }
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < ncache; i++) {
        double lq, tq;
        lq = (double)cache[i].lq / 1000000000.0;
        tq = (double)cache[i].tq / 1000.0;
        oracle_fill_matrix(lq, tq, size, cache[i].m);
    }
    /* node -> matrix per category */
    const double** nm = calloc((size_t)K * n, sizeof(double*));
    for (int k = 0; k < K; k++)
        for (int v = 0; v < n; v++) {
            if (tree->parent[v] < 0) continue;
            double lam = lambdas[tree->lambda_index[v]] * multipliers[k];
            int idx = find_key(cache, ncache, (long)(lam * 1000000000), (long)(tree->branch_length[v] * 1000));
            nm[(size_t)k * n + v] = idx >= 0 ? cache[idx].m : NULL;
        }

    tree_view tv;
    int *cstart, *children;
    tv.tree = tree;
    tv.order = reverse_level_order(tree, &cstart, &children);
    tv.cstart = cstart;
    tv.children = children;
    tv.root = tv.order[n - 1];

    /* base_model.cpp:27-51: identical families are pruned once */
    int64_t* ref = malloc(sizeof(int64_t) * (size_t)(F > 0 ? F : 1));
    for (int64_t f = 0; f < F; f++) ref[f] = f;
    if (dedupe && model == 0 && !fam_S) {
        /* hash rows, then confirm equality */
        int64_t nb = 1;
        while (nb < 2 * F) nb <<= 1;
        int64_t* head = malloc(sizeof(int64_t) * (size_t)nb);
        for (int64_t i = 0; i < nb; i++) head[i] = -1;
        for (int64_t f = 0; f < F; f++) {
            const int32_t* row = counts + (size_t)f * n_leaves;
            uint64_t h = 1469598103934665603ull;
            for (int c = 0; c < n_leaves; c++) h = (h ^ (uint32_t)row[c]) * 1099511628211ull;
            int64_t slot = (int64_t)(h & (uint64_t)(nb - 1));
            for (;;) {
                int64_t g = head[slot];
                if (g < 0) {
                    head[slot] = f;
                    break;
                }
                if (memcmp(counts + (size_t)g * n_leaves, row, sizeof(int32_t) * (size_t)n_leaves) == 0) {
                    ref[f] = g;
                    break;
                }
                slot = (slot + 1) & (nb - 1);
            }
        }
        free(head);
    }

    int fail = 0;
    int stride = (Smax + 1 > Rmax ? Smax + 1 : Rmax) + 4;
#pragma omp parallel
    {
        double* vec = malloc(sizeof(double) * (size_t)n * stride);
        double* res = malloc(sizeof(double) * (size_t)stride);
        double* root = malloc(sizeof(double) * (size_t)stride);
        long* expo = malloc(sizeof(long) * (size_t)n);
#pragma omp for schedule(dynamic, 8)
        for (int64_t f = 0; f < F; f++) {
            if (ref[f] != f) continue;
            int Sf = fam_S ? fam_S[f] : S, Rf = fam_S ? fam_R[f] : R;
            const int32_t* row = counts + (size_t)f * n_leaves;
            if (model == 0) {
                double ls;
                int rc = prune_one(&tv, row, nm, size, err_rows, err_nrows, err_ndev, Sf, Rf, scaled, vec,
                                   stride, res, expo, root, &ls);
                if (rc) {
#pragma omp atomic write
                    fail = rc;
                    continue;
                }
                /* base_model.cpp:80-90: max_j log L[j] + log prior(j) */
                double best = -INFINITY;
                for (int j = 0; j < Rf; j++) {
                    double eq = j < n_prior ? prior[j] : 0.0;
                    double v = log(root[j]) + log(eq);
                    if (j == 0 || v > best) best = v;
                }
                fam_lnl[f] = best + ls;
            } else {
                /* gamma_core.cpp:143-165, 196-207 */
                double fam_lh = 0.0;
                double cmax = -INFINITY;
                double* clog = cat_lh ? cat_lh + (size_t)f * K : NULL;
                double lcat[64];
                int bad = 0;
                for (int k = 0; k < K && !bad; k++) {
                    double ls;
                    int rc = prune_one(&tv, row, nm + (size_t)k * n, size, err_rows, err_nrows, err_ndev, Sf, Rf,
                                       scaled, vec, stride, res, expo, root, &ls);
                    if (rc) {
#pragma omp atomic write
                        fail = rc;
                        bad = 1;
                        break;
                    }
                    double sum = 0.0;
                    for (int j = 0; j < Rf; j++) sum += root[j];
                    if (sum == 0.0) {
                        bad = 1;
                        break;
                    }
                    double mx = 0;
                    for (int j = 0; j < Rf; j++) {
                        double eq = j < n_prior ? prior[j] : 0.0;
                        double v = root[j] * eq;
                        if (j == 0 || v > mx) mx = v;
                    }
                    double cat = mx * cat_probs[k];
                    if (scaled) {
                        lcat[k < 64 ? k : 63] = log(cat) + ls;
                        if (log(cat) + ls > cmax) cmax = log(cat) + ls;
                    } else {
                        fam_lh += cat;
                    }
                    if (clog) clog[k] = log(cat) + ls;
                }
                if (bad) {
                    fam_lnl[f] = NAN;
#pragma omp atomic write
                    fail = fail ? fail : 1;
                    continue;
                }
                if (scaled) {
                    double acc = 0;
                    for (int k = 0; k < K; k++) acc += exp(lcat[k] - cmax);
                    fam_lnl[f] = cmax + log(acc);
                } else {
                    fam_lnl[f] = log(fam_lh);
                }
            }
        }
        free(vec);
        free(res);
        free(root);
        free(expo);
    }
    for (int64_t f = 0; f < F; f++)
        if (ref[f] != f) fam_lnl[f] = fam_lnl[ref[f]];

    if (fail < 0) {
        *total = NAN;
    } else if (fail > 0) {
        *total = INFINITY; /* gamma_core.cpp:216-225 */
    } else {
        double acc = 0.0;
        for (int64_t f = 0; f < F; f++) acc += fam_lnl[f];
        *total = -acc; /* base_model.cpp:95, gamma_core.cpp:233 */
    }

    free(ref);
    free((void*)tv.order);
    free(cstart);
    free(children);
    free(nm);
    for (int i = 0; i < ncache; i++) free(cache[i].m);
    free(cache);
    free(bl);
    return fail < 0 ? -1 : 0;
}

/* ---- Pupko joint reconstruction (src/gene_family_reconstructor.cpp) ---- */

/* Matrices of every (lambda_i * m_k, t) key a tree needs, computed at the
 * quantised key values; nm[k * n + v] is the matrix of the branch above v
 * in category k (NULL at the root). */
typedef struct {
    cache_entry* e;
    int n;
    const double** nm;
} node_mats;

static void node_mats_build(const oracle_tree* tree, const double* lambdas, int K, const double* mult,
                            int size, node_mats* out) {
    int n = tree->n_nodes;
    out->e = calloc((size_t)K * n + 1, sizeof(cache_entry));
    out->n = 0;
    out->nm = calloc((size_t)K * n, sizeof(double*));
    for (int k = 0; k < K; k++)
        for (int v = 0; v < n; v++) {
            if (tree->parent[v] < 0) continue;
            double lam = lambdas[tree->lambda_index[v]] * mult[k];
            long lq = (long)(lam * 1000000000), tq = (long)(tree->branch_length[v] * 1000);
            int idx = find_key(out->e, out->n, lq, tq);
            if (idx < 0) {
                idx = out->n++;
                out->e[idx].lq = lq;
                out->e[idx].tq = tq;
                out->e[idx].m = malloc(sizeof(double) * (size_t)size * size);
                oracle_fill_matrix((double)lq / 1000000000.0, (double)tq / 1000.0, size, out->e[idx].m);
            }
            out->nm[(size_t)k * n + v] = out->e[idx].m;
        }
}

static void node_mats_free(node_mats* m) {
    for (int i = 0; i < m->n; i++) free(m->e[i].m);
    free(m->e);
    free(m->nm);
}

/* reconstruct_gene_family (src/gene_family_reconstructor.cpp:161-190) for
 * one family and one category: leaf (:30-45), root (:47-78) and internal
 * (:80-116) steps in reverse-level order, then the backtrack from the
 * root's single state. L / C hold n_nodes * (S + 1) entries. */
static void pupko_one(const oracle_tree* tree, const int* order, const int* cstart, const int* children,
                      const int32_t* counts_row, const double* const* nm, int size, const double* prior,
                      int n_prior, int S, int R, double* L, int* C, int32_t* state, double* root_max) {
    int n = tree->n_nodes;
    int len = S + 1;
    int root_len = (S < R ? S : R) + 1;
    memset(L, 0, sizeof(double) * (size_t)n * len);
    memset(C, 0, sizeof(int) * (size_t)n * len);
    int root = order[n - 1];
    for (int oi = 0; oi < n; oi++) {
        int v = order[oi];
        double* Lv = L + (size_t)v * len;
        int* Cv = C + (size_t)v * len;
        if (cstart[v] == cstart[v + 1]) {
            int cnt = counts_row[tree->leaf_col[v]];
            const double* m = nm[v];
            for (int i = 0; i < len; i++) {
                Cv[i] = cnt;
                Lv[i] = m[(size_t)i * size + cnt];
            }
        } else if (v == root) {
            for (int i = 1; i < root_len; i++) {
                double max_val = -1;
                for (int j = 1; j < root_len; j++) {
                    double value = 1.0;
                    for (int k = cstart[v]; k < cstart[v + 1]; k++) value *= L[(size_t)children[k] * len + j];
                    double eq = j < n_prior ? prior[j] : 0.0;
                    double val = value * eq;
                    if (val > max_val) {
                        max_val = val;
                        Cv[0] = j;
                    }
                }
                Lv[i] = max_val;
            }
        } else {
            const double* m = nm[v];
            for (int i = 0; i < len; i++) {
                int max_j = 0;
                double max_val = -1;
                for (int j = 0; j < len; j++) {
                    double value = 1.0;
                    for (int k = cstart[v]; k < cstart[v + 1]; k++) value *= L[(size_t)children[k] * len + j];
                    double val = value * m[(size_t)i * size + j];
                    if (val > max_val) {
                        max_j = j;
                        max_val = val;
                    }
                }
                Lv[i] = max_val;
                Cv[i] = max_j;
            }
        }
    }
    /* backtracker: internal nodes take C[parent state]; leaves keep their
     * observed count (get_node_count, src/base_model.cpp:190-199) */
    double mx = L[(size_t)root * len];
    for (int i = 1; i < root_len; i++)
        if (L[(size_t)root * len + i] > mx) mx = L[(size_t)root * len + i];
    *root_max = mx;
    for (int oi = n - 1; oi >= 0; oi--) {
        int v = order[oi];
        if (v == root) state[v] = C[(size_t)root * len];
        else if (cstart[v] == cstart[v + 1]) state[v] = counts_row[tree->leaf_col[v]];
        else state[v] = C[(size_t)v * len + state[tree->parent[v]]];
    }
}

int oracle_reconstruct(const oracle_tree* tree, const int32_t* counts, int64_t F, int n_leaves,
                       const double* lambdas, int n_lambdas, int K, const double* multipliers,
                       const double* cat_probs, const double* prior, int n_prior, int S, int R,
                       int n_threads, int32_t* state, double* mean, int32_t* node_count, double* root_max) {
    int n = tree->n_nodes;
    if (n <= 0 || F < 0 || n_lambdas <= 0 || S < 1 || R < 1) return -1;
    double one = 1.0;
    int gamma = K > 0;
    if (!gamma) {
        K = 1;
        multipliers = &one;
    }
    for (int64_t f = 0; f < F * n_leaves; f++)
        if (counts[f] < 0 || counts[f] > S) return -1;
    int size = (S > R ? S : R) + 1;
    node_mats nm;
    node_mats_build(tree, lambdas, K, multipliers, size, &nm);
    int *cstart, *children;
    int* order = reverse_level_order(tree, &cstart, &children);
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
#pragma omp parallel
    {
        double* L = malloc(sizeof(double) * (size_t)n * (S + 1));
        int* C = malloc(sizeof(int) * (size_t)n * (S + 1));
#pragma omp for schedule(dynamic, 4) collapse(2)
        for (int k = 0; k < K; k++)
            for (int64_t f = 0; f < F; f++)
                pupko_one(tree, order, cstart, children, counts + (size_t)f * n_leaves, nm.nm + (size_t)k * n, size,
                          prior, n_prior, S, R, L, C, state + ((size_t)k * F + f) * n, root_max + (size_t)k * F + f);
        free(L);
        free(C);
    }
    /* gamma: get_weighted_averages (src/gamma_core.cpp:268-287) over the
     * categories in order, rounded by get_node_count (:396-402); the
     * reference's category maps hold internal nodes and the root only */
    for (int64_t f = 0; f < F; f++)
        for (int v = 0; v < n; v++) {
            const int leaf = cstart[v] == cstart[v + 1];
            double val;
            if (leaf) {
                val = (double)counts[(size_t)f * n_leaves + tree->leaf_col[v]];
            } else if (gamma) {
                val = 0.0;
                for (int k = 0; k < K; k++) val += cat_probs[k] * (double)state[((size_t)k * F + f) * n + v];
            } else {
                val = (double)state[(size_t)f * n + v];
            }
            if (mean) mean[(size_t)f * n + v] = val;
            if (node_count) node_count[(size_t)f * n + v] = (int32_t)round(val);
        }
    free(order);
    free(cstart);
    free(children);
    node_mats_free(&nm);
    return 0;
}

/* compute_viterbi_sum (src/gene_family_reconstructor.cpp:390-430): for the
 * branch above each non-root node, the probability mass of child sizes
 * m < S that are less likely than the reconstructed one (ties count half),
 * under the model's own lambdas. NaN at the root (invalid). */
int oracle_branch_probabilities(const oracle_tree* tree, const double* lambdas, int n_lambdas,
                                const int32_t* node_count, int64_t F, int S, int R, double* out) {
    int n = tree->n_nodes;
    if (n <= 0 || F < 0 || n_lambdas <= 0 || S < 1) return -1;
    int size = (S > R ? S : R) + 1;
    double one = 1.0;
    node_mats nm;
    node_mats_build(tree, lambdas, 1, &one, size, &nm);
    int rc = 0;
    for (int64_t f = 0; f < F; f++)
        for (int v = 0; v < n; v++) {
            double* o = out + (size_t)f * n + v;
            int p = tree->parent[v];
            if (p < 0) {
                *o = NAN;
                continue;
            }
            int ps = node_count[(size_t)f * n + p], cs = node_count[(size_t)f * n + v];
            if (ps < 0 || cs < 0 || ps >= size || cs >= size || S > size) {
                rc = -1;
                *o = NAN;
                continue;
            }
            const double* row = nm.nm[v] + (size_t)ps * size;
            double calc = row[cs], result = 0;
            for (int m = 0; m < S; m++) {
                double pm = row[m];
                if (pm == calc) result += pm / 2.0;
                else if (pm < calc) result += pm;
            }
            *o = result;
        }
    node_mats_free(&nm);
    return rc;
}
