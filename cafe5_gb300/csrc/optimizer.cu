// Host-side parameter search over the GPU score.
//
// Restates the reference's Standard Nelder-Mead strategy
// (fminsearch_new, __fminsearch_min_init, fminsearch_min and
// threshold_achieved, src/optimizer.cpp:60-73, 156-322, 603-606; Standard
// strategy tolx = tolf = 1e-6, 300 iterations, reflection 1, expansion 2,
// contraction 0.5, shrink 0.5, initial step 5 % (0.00025 from zero)),
// optimizer::optimize's check of the initial point
// (get_initial_guesses, src/optimizer.cpp:343-360), and the scorer family
// that maps a parameter vector onto the model
// (inference_optimizer_scorer::calculate_score and its lambda, alpha,
// lambda + alpha and lambda + epsilon variants,
// src/optimizer_scorer.cpp:22-180): every objective evaluation is one
// cafe_score call, NaN scores become +inf.
//
// Also provides the median discrete-gamma rate categories of
// gamma_model::set_alpha (src/gamma_core.cpp:61-67 -> get_gamma,
// src/gamma.cpp:15-52, 225-241). The reference computes the medians with
// three published algorithms, restated below so that the multipliers agree
// with it bit for bit (they feed the lambda x multiplier products that key
// the transition-matrix cache):
//   AS 91  Best & Roberts (1975), percentage points of chi-square
//   AS 32  Bhattacharjee (1970), incomplete gamma integral
//   AS 70  Odeh & Evans (1974), percentage points of the normal
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <vector>

#include "runtime.h"

namespace {

// AS 70: normal quantile from a rational approximation in
// y = sqrt(-2 ln p1), p1 = min(p, 1 - p).
double normal_quantile(double p) {
    const double a0 = -0.322232431088, a1 = -1.0, a2 = -0.342242088547, a3 = -0.0204231210245,
                 a4 = -0.453642210148e-4;
    const double b0 = 0.0993484626060, b1 = 0.588581570495, b2 = 0.531103462366, b3 = 0.103537752850,
                 b4 = 0.0038560700634;
    const double p1 = p < 0.5 ? p : 1 - p;
    if (p1 < 1e-20) return -9999;
    const double y = std::sqrt(std::log(1 / (p1 * p1)));
    const double z = y + ((((y * a4 + a3) * y + a2) * y + a1) * y + a0) / ((((y * b4 + b3) * y + b2) * y + b1) * y + b0);
    return p < 0.5 ? -z : z;
}

// AS 32: regularised lower incomplete gamma I(x, a) with ln Gamma(a) given,
// by its power series for x <= 1 or x < a, else by its continued fraction
// (convergents as a ratio of two three-term recurrences, rescaled by 1e30
// when they grow). Returns -1 for invalid arguments.
double incomplete_gamma(double x, double a, double ln_gamma_a) {
    const double accurate = 1e-8, overflow = 1e30;
    if (x == 0) return 0;
    if (x < 0 || a <= 0) return -1;
    const double factor = std::exp(a * std::log(x) - x - ln_gamma_a);
    if (!(x > 1 && x >= a)) {
        double sum = 1, term = 1, rn = a;
        do {
            rn += 1;
            term *= x / rn;
            sum += term;
        } while (term > accurate);
        return sum * (factor / a);
    }
    double u = 1 - a, v = u + x + 1, k = 0;
    double p0 = 1, p1 = x, p2 = x + 1, p3 = x * v;
    double g = p2 / p3;
    for (int it = 0; it < 1000000; ++it) {
        u += 1;
        v += 2;
        k += 1;
        const double an = u * k;
        const double p4 = v * p2 - an * p0;
        const double p5 = v * p3 - an * p1;
        if (p5 != 0) {
            const double r = p4 / p5;
            const double dif = std::fabs(g - r);
            if (dif <= accurate && dif <= accurate * r) return 1 - factor * g;
            g = r;
        }
        p0 = p2;
        p1 = p3;
        p2 = p4;
        p3 = p5;
        if (std::fabs(p4) >= overflow) {
            p0 /= overflow;
            p1 /= overflow;
            p2 /= overflow;
            p3 /= overflow;
        }
    }
    return 1 - factor * g;
}

// AS 91: chi-square quantile with v degrees of freedom. A starting value
// from one of three approximations (small v relative to -ln p, v <= 0.32,
// Wilson-Hilferty otherwise) is refined by a seventh-order Taylor step on
// the incomplete gamma integral until the relative change is below 5e-7.
// Valid for 2e-6 < p < 1 - 2e-6; returns -1 outside.
double chi2_quantile(double p, double v) {
    const double e = 0.5e-6, ln2 = 0.6931471805;
    if (p < 0.000002 || p > 0.999998 || v <= 0) return -1;
    const double g = std::lgamma(v / 2);
    const double xx = v / 2, c = xx - 1;
    double ch;
    if (v < -1.24 * std::log(p)) {
        ch = std::pow(p * xx * std::exp(g + xx * ln2), 1 / xx);
        if (ch - e < 0) return ch;
    } else if (v <= 0.32) {
        ch = 0.4;
        const double a = std::log(1 - p);
        double q;
        do {
            q = ch;
            const double p1 = 1 + ch * (4.67 + ch);
            const double p2 = ch * (6.73 + ch * (6.66 + ch));
            const double t = -0.5 + (4.67 + 2 * ch) / p1 - (6.73 + ch * (13.32 + 3 * ch)) / p2;
            ch -= (1 - std::exp(a + g + 0.5 * ch + c * ln2) * p2 / p1) / t;
        } while (std::fabs(q / ch - 1) - 0.01 > 0);
    } else {
        const double x = normal_quantile(p);
        const double p1 = 0.222222 / v;
        ch = v * std::pow(x * std::sqrt(p1) + 1 - p1, 3.0);
        if (ch > 2.2 * v + 6) ch = -2 * (std::log(1 - p) - c * std::log(0.5 * ch) + g);
    }
    double q;
    do {
        q = ch;
        const double p1 = 0.5 * ch;
        double t = incomplete_gamma(p1, xx, g);
        if (t < 0) return -1;
        const double p2 = p - t;
        t = p2 * std::exp(xx * ln2 + g + p1 - c * std::log(ch));
        const double b = t / ch;
        const double a = 0.5 * t - b * c;
        const double s1 = (210 + a * (140 + a * (105 + a * (84 + a * (70 + 60 * a))))) / 420;
        const double s2 = (420 + a * (735 + a * (966 + a * (1141 + 1278 * a)))) / 2520;
        const double s3 = (210 + a * (462 + a * (707 + 932 * a))) / 2520;
        const double s4 = (252 + a * (672 + 1182 * a) + c * (294 + a * (889 + 1740 * a))) / 5040;
        const double s5 = (84 + 264 * a + c * (175 + 606 * a)) / 2520;
        const double s6 = (120 + c * (346 + 127 * c)) / 5040;
        ch += t * (1 + 0.5 * t * s1 - b * c * (s1 - b * (s2 - b * (s3 - b * (s4 - b * (s5 - b * s6))))));
    } while (std::fabs(q / ch - 1) > e);
    return ch;
}

}  // namespace

namespace cafe {

// Median categories of Gamma(shape alpha, rate alpha): category k's rate is
// the quantile at (2k + 1) / 2K (a Gamma(alpha, rate beta) quantile is a
// chi-square(2 alpha) quantile / 2 beta), scaled so the K rates sum to K.
void discrete_gamma_median(int K, double alpha, double* probs, double* mult) {
    const double beta = alpha;
    const double gap05 = 1.0 / (2.0 * K), factor = alpha / beta * K;
    double t = 0;
    for (int i = 0; i < K; ++i) {
        mult[i] = chi2_quantile((i * 2.0 + 1) * gap05, 2.0 * alpha) / (2.0 * beta);
        t += mult[i];
    }
    for (int i = 0; i < K; ++i) {
        mult[i] *= factor / t;
        probs[i] = 1.0 / K;
    }
}

}  // namespace cafe

namespace {

struct Candidate {
    std::vector<double> v;
    double score = 0;
};

// fminsearch_min with the default threshold (both the simplex extent and
// the score spread within tolerance).
struct NelderMead {
    double rho = 1, chi = 2, psi = 0.5, sigma = 0.5, tolx = 1e-6, tolf = 1e-6, delta = 0.05, zero_delta = 0.00025;
    int maxiters = 300, iters = 0;
    bool bymax = false;
    int n = 0;
    std::vector<Candidate> store;
    std::vector<Candidate*> c;
    std::vector<double> x_mean, x_r, x_tmp;
    std::function<double(const double*)> f;

    void sort() {
        std::sort(c.begin(), c.end(), [](const Candidate* a, const Candidate* b) { return a->score < b->score; });
    }
    bool check_v() const {
        double mx = -std::numeric_limits<double>::max();
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) mx = std::max(mx, std::fabs(c[i + 1]->v[j] - c[i]->v[j]));
        return mx <= tolx;
    }
    bool check_f() const {
        double mx = -std::numeric_limits<double>::max();
        for (int i = 1; i < n + 1; ++i) mx = std::max(mx, std::fabs(c[i]->score - c[0]->score));
        return mx <= tolf;
    }
    // Vertex 0 is X0; vertex i > 0 moves coordinate i - 1 by `delta`
    // (100 x delta when the previous vertex scored +inf).
    void init(const double* X0) {
        for (int i = 0; i < n + 1; ++i) {
            const double step = (i > 1 && std::isinf(c[i - 1]->score)) ? delta * 100 : delta;
            for (int j = 0; j < n; ++j) c[i]->v[j] = ((i - 1) == j) ? (X0[j] ? (1 + step) * X0[j] : zero_delta) : X0[j];
            c[i]->score = f(c[i]->v.data());
        }
        sort();
    }
    void mean() {
        for (int i = 0; i < n; ++i) {
            x_mean[i] = 0;
            for (int j = 0; j < n; ++j) x_mean[i] += c[j]->v[i];
            x_mean[i] /= n;
        }
    }
    void set_last(const std::vector<double>& x, double s) {
        std::copy(x.begin(), x.end(), c.back()->v.begin());
        c.back()->score = s;
        sort();
    }
    void shrink() {
        for (int i = 1; i < n + 1; ++i) {
            for (int j = 0; j < n; ++j) c[i]->v[j] = c[0]->v[j] + sigma * (c[i]->v[j] - c[0]->v[j]);
            c[i]->score = f(c[i]->v.data());
        }
        sort();
    }
    // x = x_mean + coef * (from - to), scored.
    double trial(std::vector<double>& x, const std::vector<double>& from, double coef, const std::vector<double>& to) {
        for (int j = 0; j < n; ++j) x[j] = x_mean[j] + coef * (from[j] - to[j]);
        return f(x.data());
    }
    void run(const double* X0) {
        x_mean.assign(n, 0);
        x_r.assign(n, 0);
        x_tmp.assign(n, 0);
        store.assign(n + 1, Candidate());
        c.clear();
        for (auto& s : store) {
            s.v.assign(n, 0);
            c.push_back(&s);
        }
        init(X0);
        int i;
        for (i = 0; i < maxiters; ++i) {
            if (check_v() && check_f()) break;
            mean();
            const double fr = trial(x_r, x_mean, rho, c[n]->v);               // reflection
            if (fr < c[0]->score) {
                const double fe = trial(x_tmp, x_r, chi, x_mean);             // expansion
                if (fe < fr) set_last(x_tmp, fe);
                else set_last(x_r, fr);
            } else if (fr >= c[n]->score) {
                if (fr > c[n]->score) {
                    const double fc = trial(x_tmp, x_mean, psi, c[n]->v);     // inside contraction
                    if (fc < c[n]->score) set_last(x_tmp, fc);
                    else shrink();
                } else {
                    const double fc = trial(x_tmp, x_r, psi, x_mean);         // outside contraction
                    if (fc <= fr) set_last(x_tmp, fc);
                    else shrink();
                }
            } else {
                set_last(x_r, fr);
            }
        }
        bymax = (i == maxiters);
        iters = i;
    }
};

// error_model::replace_epsilons (src/error_model.cpp:79-109) on a row table
// with deviations {-1, 0, +1}: a row whose last entry is within 1 % of a
// replaced epsilon takes the new value (row 0 keeps its zero first entry).
void replace_epsilons(std::vector<double>& rows, int n_rows, const std::map<double, double>& repl) {
    auto near = [](double x, double y) { return std::fabs(x - y) <= 0.01 * std::fabs(x); };
    for (auto& kv : repl)
        if (near(kv.first, rows[2])) {
            rows[2] = kv.second;
            rows[1] = 1 - kv.second;
        }
    for (int i = 1; i < n_rows; ++i)
        for (auto& kv : repl)
            if (near(kv.first, rows[i * 3 + 2])) {
                rows[i * 3 + 2] = kv.second;
                rows[i * 3 + 0] = kv.second;
                rows[i * 3 + 1] = 1 - (kv.second * 2);
            }
}

int opt_fail(cafe_ctx* C, int code, const char* msg) {
    if (C) C->last_error = msg;
    return code;
}

}  // namespace

extern "C" {

int cafe_discrete_gamma(int K, double alpha, double* probs, double* multipliers) {
    if (K < 1 || !probs || !multipliers || !(alpha > 0)) return CAFE_ERR_INVALID;
    if (K == 1) {
        probs[0] = 1.0;
        multipliers[0] = 1.0;
        return CAFE_OK;
    }
    cafe::discrete_gamma_median(K, alpha, probs, multipliers);
    return CAFE_OK;
}

// Shared setup of both searches from a cafe_opt_config.
static void configure(NelderMead& nm, const cafe_opt_config* cfg) {
    nm.n = cfg->n_params;
    nm.maxiters = cfg->max_iterations > 0 ? cfg->max_iterations : 300;
    if (cfg->expansion > 0) nm.chi = cfg->expansion;
    if (cfg->reflection > 0) nm.rho = cfg->reflection;
}

static void report(const NelderMead& nm, int evaluations, cafe_opt_result* out) {
    std::copy(nm.c[0]->v.begin(), nm.c[0]->v.end(), out->values);
    out->score = nm.c[0]->score;
    out->iterations = nm.iters;
    out->evaluations = evaluations;
    out->converged = nm.bymax ? 0 : 1;
}

int cafe_nelder_mead(const cafe_opt_config* cfg, double (*objective)(const double* x, int n, void* user), void* user,
                     cafe_opt_result* out) {
    if (!cfg || !objective || !out || !out->values || !cfg->initial || cfg->n_params < 1) return CAFE_ERR_INVALID;
    NelderMead nm;
    configure(nm, cfg);
    int evaluations = 0;
    const int n = cfg->n_params;
    nm.f = [&](const double* x) -> double {
        ++evaluations;
        return objective(x, n, user);
    };
    nm.run(cfg->initial);
    report(nm, evaluations, out);
    return CAFE_OK;
}

int cafe_optimize(cafe_ctx* C, const cafe_request* base, const cafe_opt_config* cfg, cafe_opt_result* out) {
    if (!C || !base || !cfg || !out || !cfg->initial || cfg->n_params < 1 || !out->values)
        return opt_fail(C, CAFE_ERR_INVALID, "cafe_optimize: null argument or no parameters");
    const int np = cfg->n_params;
    const int nl = base->n_lambdas;
    const bool gamma = base->model == CAFE_MODEL_GAMMA;
    int n_lam = nl, n_extra = 0;
    switch (cfg->kind) {
        case CAFE_OPT_LAMBDA: break;
        case CAFE_OPT_ALPHA: n_lam = 0; n_extra = 1; break;
        case CAFE_OPT_LAMBDA_ALPHA: n_extra = 1; break;
        case CAFE_OPT_LAMBDA_EPSILON: n_extra = np - nl; break;
        default: return opt_fail(C, CAFE_ERR_INVALID, "cafe_optimize: unknown kind");
    }
    if (nl < 1 || !base->lambdas || np != n_lam + n_extra || n_extra < 0)
        return opt_fail(C, CAFE_ERR_INVALID, "cafe_optimize: n_params does not match the request");
    const bool fit_alpha = cfg->kind == CAFE_OPT_ALPHA || cfg->kind == CAFE_OPT_LAMBDA_ALPHA;
    if (fit_alpha && (!gamma || base->n_categories < 1))
        return opt_fail(C, CAFE_ERR_INVALID, "cafe_optimize: alpha needs the gamma model");

    cafe_request req = *base;
    std::vector<double> lambdas(base->lambdas, base->lambdas + nl), probs, mult;
    if (gamma) {
        probs.assign(base->cat_probs, base->cat_probs + base->n_categories);
        mult.assign(base->multipliers, base->multipliers + base->n_categories);
    }
    std::vector<double> err, current_eps;
    int err_rows = 0;
    if (cfg->kind == CAFE_OPT_LAMBDA_EPSILON) {
        std::lock_guard<std::mutex> lk(C->mu);
        if (C->err_ndev != 3 || C->err_rows < 1)
            return opt_fail(C, CAFE_ERR_INVALID, "cafe_optimize: epsilon search needs a 3-deviation error model");
        err = C->err;
        err_rows = C->err_rows;
        // error_model::get_epsilons: the distinct last entries, ascending
        for (int i = 0; i < err_rows; ++i) current_eps.push_back(err[i * 3 + 2]);
        std::sort(current_eps.begin(), current_eps.end());
        current_eps.erase(std::unique(current_eps.begin(), current_eps.end()), current_eps.end());
        if ((int)current_eps.size() != n_extra)
            return opt_fail(C, CAFE_ERR_INVALID, "cafe_optimize: one parameter per distinct epsilon expected");
    }

    int status = CAFE_OK;
    int evaluations = 0;
    NelderMead nm;
    configure(nm, cfg);
    nm.f = [&](const double* x) -> double {
        ++evaluations;
        if (status != CAFE_OK) return INFINITY;
        for (int i = 0; i < n_lam; ++i) lambdas[i] = x[i];
        req.lambdas = lambdas.data();
        if (fit_alpha) {
            // gamma_model::set_alpha, then can_infer's alpha < 0 rejection
            const double alpha = x[n_lam];
            if (!(alpha > 0)) return INFINITY;
            if (req.n_categories > 1) cafe::discrete_gamma_median(req.n_categories, alpha, probs.data(), mult.data());
            req.multipliers = mult.data();
            req.cat_probs = probs.data();
        }
        if (cfg->kind == CAFE_OPT_LAMBDA_EPSILON) {
            std::map<double, double> repl;
            for (int i = 0; i < n_extra; ++i) {
                repl[current_eps[i]] = x[nl + i];
                current_eps[i] = x[nl + i];
            }
            replace_epsilons(err, err_rows, repl);
            const int rc = cafe_error_model_set(C, err.data(), err_rows, 3);
            if (rc) {
                status = rc;
                return INFINITY;
            }
        }
        cafe_result res{};
        const int rc = cafe_score(C, &req, &res);
        if (rc) {
            status = rc;
            return INFINITY;
        }
        return std::isnan(res.total_neg_lnl) ? INFINITY : res.total_neg_lnl;
    };
    // optimizer::get_initial_guesses scores the starting point first and
    // refuses to search from a point that scores +inf.
    const double first = nm.f(cfg->initial);
    if (status != CAFE_OK) return status;
    if (std::isinf(first)) return opt_fail(C, CAFE_ERR_INVALID, "cafe_optimize: the initial point scores +inf");
    nm.run(cfg->initial);
    if (status != CAFE_OK) return status;
    report(nm, evaluations, out);
    return CAFE_OK;
}

}  // extern "C"
