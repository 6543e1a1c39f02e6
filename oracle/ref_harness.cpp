// Test infrastructure only: a command-line probe that links the CAFE5
// reference objects (compiled from the reference's own sources by
// oracle/Makefile into oracle/_ref/) and calls the reference's likelihood
// hot path exactly as its users do:
//
//   base_model::infer_family_likelihoods   (src/base_model.cpp:53-100)
//   gamma_model::infer_family_likelihoods  (src/gamma_core.cpp:168-237)
//   matrix_cache::precalculate_matrices    (src/matrix_cache.cpp:113-163)
//   inference_prune                        (src/core.cpp:134-145)
//   fminsearch_min over the optimizer scorers (src/optimizer.cpp:281-322,
//                                           src/optimizer_scorer.cpp:22-180)
//   model::reconstruct_ancestral_states     (src/base_model.cpp:133-170,
//                                           src/gamma_core.cpp:290-339)
//   compute_viterbi_sum                     (src/gene_family_reconstructor.cpp:390-430)
//
// It reads the reference's own file formats (Newick tree, CAFE family
// table, error-model file) through the reference's own readers
// (src/clade.cpp:293-419, src/io.cpp:134-217, src/io.cpp:228-274), and
// prints the total -lnL plus every per-family result as C99 hex floats so
// that the parity tests compare bit patterns, not printed decimals.
//
// Nothing in the product links or runs this file.
#include <algorithm>
#include <chrono>
#include <limits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <random>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "easylogging++.h"
#include "base_model.h"
#include "clade.h"
#include "core.h"
#include "error_model.h"
#include "gamma.h"
#include "gamma_core.h"
#include "gene_family.h"
#include "gene_family_reconstructor.h"
#include "io.h"
#include "lambda.h"
#include "matrix_cache.h"
#include "optimizer.h"
#include "optimizer_scorer.h"
#include "probability.h"
#include "root_equilibrium_distribution.h"
#include "simulator.h"
#include "user_data.h"

INITIALIZE_EASYLOGGINGPP

std::mt19937 randomizer_engine(10);

void init_lgamma_cache();

namespace {

// Subclasses only to read the protected per-family results vector.
struct probe_base : public base_model {
    using base_model::base_model;
    const std::vector<family_info_stash>& stash() const { return results; }
};

struct probe_gamma : public gamma_model {
    using gamma_model::gamma_model;
    const std::vector<family_info_stash>& stash() const { return results; }
};

std::string slurp(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

std::vector<double> parse_list(const std::string& s) {
    std::vector<double> v;
    std::stringstream ss(s);
    std::string tok;
    while (std::getline(ss, tok, ',')) v.push_back(std::stod(tok));
    return v;
}

// Analytic objectives for the Nelder-Mead known-answer runs. The parity
// tests evaluate the same expressions in the same order.
struct analytic_scorer : public optimizer_scorer {
    std::string fn;
    int n;
    int evaluations = 0;
    analytic_scorer(std::string f, int n_) : fn(std::move(f)), n(n_) {}
    std::vector<double> initial_guesses() override { return std::vector<double>(n, 1.0); }
    double calculate_score(const double* x) override {
        ++evaluations;
        if (fn == "rosen" || fn == "wall") {
            if (fn == "wall" && x[0] > 1.0) return std::numeric_limits<double>::infinity();
            double s = 0;
            for (int i = 0; i + 1 < n; ++i) {
                const double a = x[i + 1] - x[i] * x[i], b = 1 - x[i];
                s += 100 * a * a + b * b;
            }
            return s;
        }
        if (fn == "bowl") {
            double s = 0;
            for (int i = 0; i < n; ++i) {
                const double d = x[i] - (i + 1);
                s += d * d * (i + 1);
            }
            return s;
        }
        if (fn == "product") {
            double s = 1.0;
            for (int i = 0; i < n; ++i) s *= x[i];
            return s;
        }
        throw std::runtime_error("unknown objective " + fn);
    }
};

// Counts the objective calls of a likelihood scorer.
struct counting_scorer : public optimizer_scorer {
    inference_optimizer_scorer* inner;
    int evaluations = 0;
    explicit counting_scorer(inference_optimizer_scorer* s) : inner(s) {}
    std::vector<double> initial_guesses() override { return inner->initial_guesses(); }
    double calculate_score(const double* x) override {
        ++evaluations;
        return inner->calculate_score(x);
    }
};

void print_search(FMinSearch* pfm, int evaluations) {
    candidate* best = get_best_result(pfm);
    std::printf("best");
    for (double v : best->values) std::printf(" %a", v);
    std::printf("\nscore %a\niters %d\nevals %d\n", best->score, pfm->iters, evaluations);
}

void usage() {
    std::fprintf(stderr,
        "cafe_ref_harness --tree T.nwk --families F.tab --lambdas l1[,l2..]\n"
        "   [--lambda-tree L.nwk] [--error E.txt]\n"
        "   [--gamma-alpha A --gamma-k K] [--gamma-mult m1,.. --gamma-prob p1,..]\n"
        "   [--max-family S --max-root R] [--prior uniform|uniform:N|poisson:X|rootdist:s=n,..]\n"
        "   [--repeat N] [--quiet]\n"
        "   [--optimize lambda|alpha|lambda_alpha|lambda_epsilon --initial x1,..]\n"
        "   [--reconstruct] [--pvalues N_SIMULATIONS --seed S] [--simulate N --seed S]\n"
        "   [--exclude-zero-root] [--estimate-bounds] [--dump-input]\n"
        "cafe_ref_harness nm rosen|wall|bowl|product <maxiters> x1,..\n");
}

}  // namespace

int main(int argc, char** argv) {
    el::Configurations conf;
    conf.setToDefault();
    conf.set(el::Level::Global, el::ConfigurationType::Enabled, "false");
    conf.set(el::Level::Global, el::ConfigurationType::ToFile, "false");
    el::Loggers::reconfigureAllLoggers(conf);

    // "matrix <lambda> <t> <size>": dump one cached transition matrix
    // (matrix_cache::precalculate_matrices + get_matrix) as hex floats.
    if (argc == 5 && std::string(argv[1]) == "matrix") {
        init_lgamma_cache();
        double l = std::stod(argv[2]), t = std::stod(argv[3]);
        int size = std::stoi(argv[4]);
        matrix_cache calc(size);
        calc.precalculate_matrices({l}, std::set<double>{t});
        const matrix* mm = calc.get_matrix(t, l);
        for (int s = 0; s < size; ++s) {
            for (int c = 0; c < size; ++c) std::printf("%a ", mm->get(s, c));
            std::printf("\n");
        }
        return 0;
    }
    // "rate <s> <c> <log_alpha> <coeff>": birthdeath_rate_with_log_alpha.
    if (argc == 6 && std::string(argv[1]) == "rate") {
        init_lgamma_cache();
        double v = birthdeath_rate_with_log_alpha(std::stoi(argv[2]), std::stoi(argv[3]),
                                                  std::stod(argv[4]), std::stod(argv[5]));
        std::printf("%a\n", v);
        return 0;
    }

    // "gamma <K> <alpha>": category probabilities and lambda multipliers
    // from get_gamma (src/gamma.cpp:225-241).
    if (argc == 4 && std::string(argv[1]) == "gamma") {
        int k = std::stoi(argv[2]);
        std::vector<double> freq(k), rate(k);
        get_gamma(freq, rate, std::stod(argv[3]));
        for (int i = 0; i < k; ++i) std::printf("%a %a\n", freq[i], rate[i]);
        return 0;
    }

    // "nm <objective> <maxiters> x1,..": fminsearch_min on an analytic
    // objective with the Standard strategy's tolerances.
    if (argc == 5 && std::string(argv[1]) == "nm") {
        std::vector<double> x0 = parse_list(argv[4]);
        analytic_scorer sc(argv[2], (int)x0.size());
        FMinSearch* pfm = fminsearch_new_with_eq(&sc, (int)x0.size());
        pfm->maxiters = std::stoi(argv[3]);
        pfm->tolx = 1e-6;
        pfm->tolf = 1e-6;
        fminsearch_min(pfm, x0.data());
        print_search(pfm, sc.evaluations);
        fminsearch_free(pfm);
        return 0;
    }

    std::string tree_path, fam_path, lambda_tree_path, err_path, prior_spec = "uniform", opt_kind;
    std::vector<double> opt_initial;
    std::vector<double> lambdas, gmult, gprob;
    double alpha = -1;
    int gk = 0, S = -1, R = -1, repeat = 1;
    bool quiet = false, recon = false, zero_root = false, dump = false, estimate_bounds = false;
    int n_sim = 0, n_simulate = 0;
    unsigned long seed = 10;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        auto next = [&]() -> std::string {
            if (i + 1 >= argc) { usage(); std::exit(2); }
            return argv[++i];
        };
        if (a == "--tree") tree_path = next();
        else if (a == "--families") fam_path = next();
        else if (a == "--lambda-tree") lambda_tree_path = next();
        else if (a == "--lambdas") lambdas = parse_list(next());
        else if (a == "--error") err_path = next();
        else if (a == "--gamma-alpha") alpha = std::stod(next());
        else if (a == "--gamma-k") gk = std::stoi(next());
        else if (a == "--gamma-mult") gmult = parse_list(next());
        else if (a == "--gamma-prob") gprob = parse_list(next());
        else if (a == "--max-family") S = std::stoi(next());
        else if (a == "--max-root") R = std::stoi(next());
        else if (a == "--prior") prior_spec = next();
        else if (a == "--repeat") repeat = std::stoi(next());
        else if (a == "--quiet") quiet = true;
        else if (a == "--optimize") opt_kind = next();
        else if (a == "--initial") opt_initial = parse_list(next());
        else if (a == "--reconstruct") recon = true;
        else if (a == "--pvalues") n_sim = std::stoi(next());
        else if (a == "--seed") seed = std::stoul(next());
        else if (a == "--simulate") n_simulate = std::stoi(next());
        else if (a == "--exclude-zero-root") zero_root = true;
        else if (a == "--dump-input") dump = true;
        else if (a == "--estimate-bounds") estimate_bounds = true;
        else { usage(); return 2; }
    }
    if (tree_path.empty() || fam_path.empty() || lambdas.empty()) { usage(); return 2; }

    try {
        init_lgamma_cache();
        std::string nwk = slurp(tree_path);
        std::unique_ptr<clade> tree(parse_newick(nwk, false));
        std::vector<gene_family> families;
        {
            std::ifstream f(fam_path);
            read_gene_families(f, tree.get(), families);
        }
        // Global bounds exactly as user_data::read_gene_family_data computes
        // them (src/user_data.cpp:39-48) unless overridden: over every family
        // read, before any filter.
        int mx = 0;
        for (auto& gf : families) mx = std::max(mx, gf.get_max_size());
        int est_fam = -1, est_root = -1;
        if (estimate_bounds) {
            // the estimate action's own bounds: user_data::read_gene_family_data
            // on the same file, starting from user_data's defaults
            // (src/user_data.cpp:24-48, src/user_data.h:26-27)
            input_parameters ip;
            ip.input_file_path = fam_path;
            user_data ud;
            std::vector<gene_family> again;
            ud.read_gene_family_data(ip, ud.max_family_size, ud.max_root_family_size, tree.get(), &again);
            est_fam = ud.max_family_size;
            est_root = ud.max_root_family_size;
        }
        // the estimate action's default filter, applied after the bounds
        // (exclude_zero_root_families, src/core.cpp:190-205, over
        // gene_family::exists_at_root; cafexp.cpp reads the data files first)
        if (zero_root)
            families.erase(std::remove_if(families.begin(), families.end(),
                                          [&](const gene_family& gf) { return !gf.exists_at_root(tree.get()); }),
                           families.end());
        int max_root = std::max(30, static_cast<int>(std::rint(mx * 1.25)));
        int max_fam = mx + std::max(50, mx / 5);
        if (estimate_bounds) {
            max_fam = est_fam;
            max_root = est_root;
        }
        if (S >= 0) max_fam = S;
        if (R >= 0) max_root = R;

        std::unique_ptr<clade> ltree;
        std::unique_ptr<lambda> lam;
        if (!lambda_tree_path.empty()) {
            ltree.reset(parse_newick(slurp(lambda_tree_path), true));
            lam.reset(new multiple_lambda(ltree->get_lambda_index_map(), lambdas));
        } else {
            lam.reset(new single_lambda(lambdas[0]));
        }

        std::unique_ptr<error_model> em;
        if (!err_path.empty()) {
            em.reset(new error_model());
            std::ifstream f(err_path);
            read_error_model_file(f, em.get());
        }

        if (dump) {
            // what the reference's readers made of the inputs: the tree in
            // prefix order (name, parent, branch length), every family's
            // counts at the leaves in that order, the lambda index of every
            // node of a lambda tree, and the error model's rows
            std::vector<const clade*> nodes;
            tree->apply_prefix_order([&](const clade* c) { nodes.push_back(c); });
            std::map<const clade*, int> at;
            for (size_t i = 0; i < nodes.size(); ++i) at[nodes[i]] = (int)i;
            for (size_t i = 0; i < nodes.size(); ++i) {
                const clade* c = nodes[i];
                std::printf("node %zu %s %d %a\n", i, c->get_taxon_name().c_str(),
                            c->get_parent() ? at[c->get_parent()] : -1, c->get_branch_length());
            }
            std::printf("families %zu\n", families.size());
            for (auto& gf : families) {
                std::printf("gf %s", gf.id().c_str());
                for (auto* c : nodes)
                    if (c->is_leaf()) std::printf(" %d", gf.get_species_size(c->get_taxon_name()));
                std::printf("\n");
            }
            if (ltree) {
                auto idx = ltree->get_lambda_index_map();
                for (auto* c : nodes) std::printf("lambda_index %s %d\n", c->get_taxon_name().c_str(), idx[c->get_taxon_name()]);
            }
            if (em) {
                for (size_t n = 0; n < em->get_max_family_size(); ++n) {
                    std::printf("erow %zu", n);
                    for (double x : em->get_probs(n)) std::printf(" %a", x);
                    std::printf("\n");
                }
            }
            std::printf("bounds %d %d\n", max_fam, max_root);
            return 0;
        }

        std::unique_ptr<root_equilibrium_distribution> prior;
        if (prior_spec == "uniform") prior.reset(new root_equilibrium_distribution(size_t(max_root)));
        else if (prior_spec.rfind("uniform:", 0) == 0)
            prior.reset(new root_equilibrium_distribution(size_t(std::stoul(prior_spec.substr(8)))));
        else if (prior_spec.rfind("rootdist:", 0) == 0) {
            // rootdist:size=count,size=count,...
            std::map<int, int> rd;
            std::stringstream ss(prior_spec.substr(9));
            std::string tok;
            while (std::getline(ss, tok, ',')) {
                auto eq = tok.find('=');
                rd[std::stoi(tok.substr(0, eq))] = std::stoi(tok.substr(eq + 1));
            }
            prior.reset(new root_equilibrium_distribution(rd));
        }
        else if (prior_spec.rfind("poisson:", 0) == 0)
            prior.reset(new root_equilibrium_distribution(std::stod(prior_spec.substr(8)), size_t(max_root)));
        else throw std::runtime_error("bad prior " + prior_spec);

        bool is_gamma = (alpha > 0 && gk > 1) || !gmult.empty();
        std::unique_ptr<model> m;
        probe_base* pb = nullptr;
        probe_gamma* pg = nullptr;
        if (is_gamma) {
            if (!gmult.empty()) {
                pg = new probe_gamma(lam.get(), tree.get(), &families, max_fam, max_root, gprob, gmult, em.get());
            } else {
                pg = new probe_gamma(lam.get(), tree.get(), &families, max_fam, max_root, gk, alpha, em.get());
            }
            m.reset(pg);
        } else {
            pb = new probe_base(lam.get(), tree.get(), &families, max_fam, max_root, em.get());
            m.reset(pb);
        }

        if (!opt_kind.empty()) {
            // optimizer::optimize with the Standard strategy from a given
            // starting point: the initial-point check of get_initial_guesses,
            // then fminsearch_min (src/optimizer.cpp:343-360, 366-385).
            auto lengths = tree->get_branch_lengths();
            double longest = *std::max_element(lengths.begin(), lengths.end());
            std::unique_ptr<inference_optimizer_scorer> sc;
            if (opt_kind == "lambda") sc.reset(new lambda_optimizer(lam.get(), m.get(), prior.get(), longest));
            else if (opt_kind == "alpha" && pg) sc.reset(new gamma_optimizer(pg, prior.get()));
            else if (opt_kind == "lambda_alpha" && pg)
                sc.reset(new gamma_lambda_optimizer(lam.get(), pg, prior.get(), longest));
            else if (opt_kind == "lambda_epsilon" && em) {
                auto* le = new lambda_epsilon_optimizer(m.get(), em.get(), prior.get(), std::map<int, int>(), lam.get(),
                                                        longest);
                le->initial_guesses();   // records the current epsilons
                sc.reset(le);
            } else throw std::runtime_error("bad --optimize " + opt_kind);
            sc->quiet = true;
            counting_scorer cs(sc.get());
            const double first = cs.calculate_score(opt_initial.data());
            std::printf("first %a\n", first);
            FMinSearch* pfm = fminsearch_new_with_eq(&cs, (int)opt_initial.size());
            pfm->maxiters = 300;
            pfm->tolx = 1e-6;
            pfm->tolf = 1e-6;
            fminsearch_min(pfm, opt_initial.data());
            print_search(pfm, cs.evaluations);
            fminsearch_free(pfm);
            return 0;
        }

        double total = 0;
        double best_ms = 1e300, sum_ms = 0;
        for (int r = 0; r < repeat; ++r) {
            auto t0 = std::chrono::steady_clock::now();
            total = m->infer_family_likelihoods(*prior, lam.get());
            auto t1 = std::chrono::steady_clock::now();
            double ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
            best_ms = std::min(best_ms, ms);
            sum_ms += ms;
        }
        std::printf("bounds %d %d\n", max_fam, max_root);
        std::printf("families %zu\n", families.size());
        std::printf("total %.17g %a\n", total, total);
        std::printf("time_ms best %.6f mean %.6f repeat %d\n", best_ms, sum_ms / repeat, repeat);
        if (!quiet) {
            if (pb) {
                for (auto& s : pb->stash())
                    std::printf("fam %s %a\n", s.family_id.c_str(), s.posterior_probability);
            } else if (pg) {
                for (auto& s : pg->stash())
                    std::printf("cat %s %a %a %a\n", s.family_id.c_str(), s.lambda_multiplier,
                                s.category_likelihood, s.family_likelihood);
            }
        }
        if (n_simulate > 0) {
            // the simulator action (src/simulator.cpp:61-91): the prior is
            // resized to N families first (user_data::create_prior,
            // src/user_data.cpp:204-205, drawing from the engine seeded
            // with seed + 1), then the engine is seeded with `seed` and
            // simulate_processes runs. Prints the root size of every family
            // and every family's simulated sizes in prefix order.
            std::vector<const clade*> nodes;
            tree->apply_prefix_order([&](const clade* c) { nodes.push_back(c); });
            randomizer_engine.seed(seed + 1);
            prior->resize(n_simulate);
            std::printf("roots");
            for (int i = 0; i < n_simulate; ++i) std::printf(" %d", prior->select_root_size(i));
            std::printf("\n");
            user_data ud;
            ud.max_family_size = max_fam;
            ud.max_root_family_size = max_root;
            ud.p_tree = tree.get();
            ud.p_error_model = em.get();
            ud.prior = std::move(*prior);
            input_parameters ui;
            ui.nsims = n_simulate;
            simulator sim(ud, ui);
            randomizer_engine.seed(seed);
            std::vector<simulated_family> results;
            sim.simulate_processes(m.get(), results);
            for (auto& r : results) {
                std::printf("sim %a", r.lambda);
                for (auto* c : nodes) std::printf(" %d", r.values.at(c));
                std::printf("\n");
            }
            return 0;
        }
        if (n_sim > 0) {
            // compute_pvalues as the estimate action runs it
            // (src/execute.cpp:166-171): a cache of side
            // max(max family, max root) + 100 at the model's own lambdas,
            // the simulation stream seeded first. Prints the conditional
            // distribution of every root size and each family's p-value.
            matrix_cache cache(std::max(max_fam, max_root) + 100);
            cache.precalculate_matrices(get_lambda_values(lam.get()), tree->get_branch_lengths());
            randomizer_engine.seed(seed);
            pvalue_parameters pp = {tree.get(), lam.get(), max_fam, max_root, cache};
            std::vector<std::vector<double>> cd(max_root);
            for (int i = 0; i < max_root; ++i) cd[i] = get_random_probabilities(pp, n_sim, i + 1);
            randomizer_engine.seed(seed);
            std::vector<double> pv = compute_pvalues(pp, families, n_sim);
            for (int i = 0; i < max_root; ++i) {
                std::printf("cd %d", i + 1);
                for (double x : cd[i]) std::printf(" %a", x);
                std::printf("\n");
            }
            for (size_t i = 0; i < families.size(); ++i) std::printf("pv %s %a\n", families[i].id().c_str(), pv[i]);
        }
        if (recon) {
            // model::reconstruct_ancestral_states as the estimate action runs
            // it (src/execute.cpp:161-185): a cache of side
            // max(max family, max root) + 100, then compute_viterbi_sum for
            // every node of every family. Nodes are printed in prefix
            // (Newick) order.
            std::vector<const clade*> nodes;
            tree->apply_prefix_order([&](const clade* c) { nodes.push_back(c); });
            user_data ud;
            ud.max_family_size = max_fam;
            ud.max_root_family_size = max_root;
            ud.p_tree = tree.get();
            ud.gene_families.swap(families);   // gene_family is not copy-assignable
            ud.prior = std::move(*prior);
            input_parameters ui;
            matrix_cache cache(std::max(max_fam, max_root) + 100);
            cache.precalculate_matrices(get_lambda_values(lam.get()), tree->get_branch_lengths());
            std::unique_ptr<reconstruction> rec(m->reconstruct_ancestral_states(ud, ui, &cache));
            for (auto& gf : ud.gene_families) {
                std::printf("rec %s", gf.id().c_str());
                for (auto* c : nodes) std::printf(" %d", rec->get_node_count(gf, c));
                std::printf("\n");
                std::printf("bp %s", gf.id().c_str());
                for (auto* c : nodes) {
                    auto bp = compute_viterbi_sum(c, gf, rec.get(), max_fam, cache, lam.get());
                    if (bp._is_valid) std::printf(" %a", bp._value);
                    else std::printf(" NA");
                }
                std::printf("\n");
            }
            if (pg) {
                auto* gr = dynamic_cast<gamma_model_reconstruction*>(rec.get());
                for (auto& gf : ud.gene_families) {
                    auto& r = gr->_reconstructions.at(gf.id());
                    for (size_t k = 0; k < r.category_reconstruction.size(); ++k) {
                        std::printf("rcat %s %zu", gf.id().c_str(), k);
                        for (auto* c : nodes) {
                            auto it = r.category_reconstruction[k].find(c);
                            std::printf(" %d", it == r.category_reconstruction[k].end() ? -1 : it->second);
                        }
                        std::printf("\n");
                    }
                    std::printf("rmean %s", gf.id().c_str());
                    for (auto* c : nodes) {
                        auto it = r.reconstruction.find(c);
                        if (it == r.reconstruction.end()) std::printf(" NA");
                        else std::printf(" %a", it->second);
                    }
                    std::printf("\n");
                }
            }
        }
    } catch (std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
