/* gpu_model.h -- the reference-side binding of the GB300 likelihood path.
 *
 * C++ subclasses of CAFE5's model classes (src/core.h:125-189,
 * src/base_model.h, src/gamma_core.h) that forward
 * infer_family_likelihoods to the C ABI of cafe_gb300.h. A CAFE5 build adds
 * this header next to src/base_model.h, constructs these classes in
 * build_models (src/core.cpp:17-51) in place of base_model / gamma_model,
 * and links -lcafe_gb300 -lcudart; optimizer_scorer and the estimate action
 * keep calling the model as before. Compiled against the reference's own
 * headers by tests/test_binding_cpu.py.
 *
 * Both classes upload the tree and the families once (constructor) and
 * score with CAFE_PREC_FP64_REF at the model's global bounds, which
 * reproduces the reference's -lnL to 1e-10; +inf is returned where the
 * reference returns -log(0). Errors of the library raise
 * std::runtime_error, as the reference's own failures do.
 */
#ifndef CAFE_GB300_GPU_MODEL_H
#define CAFE_GB300_GPU_MODEL_H

#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "base_model.h"
#include "clade.h"
#include "gamma.h"
#include "gamma_core.h"
#include "gene_family.h"
#include "lambda.h"
#include "root_equilibrium_distribution.h"

#include "cafe_gb300.h"

namespace cafe_gpu {

inline void check(cafe_ctx* ctx, int rc) {
    if (rc != CAFE_OK)
        throw std::runtime_error(std::string("cafe_gb300: ") + (ctx ? cafe_last_error(ctx) : cafe_status_string(rc)));
}

// The device-resident inputs shared by both models: the tree (nodes in
// prefix order, so children keep their descendant order), the families'
// leaf counts, and the context.
class device_inputs {
public:
    cafe_ctx* ctx = nullptr;
    int tree_id = 0, set_id = 0;
    std::vector<std::string> ids;

    // lambda_index: the lambda of the branch above each node in prefix
    // order (clade::get_lambda_index_map, 0-based); empty for one lambda.
    device_inputs(const clade* tree, const std::vector<gene_family>* fams, int device = 0,
                  const std::vector<int32_t>& lambda_index = std::vector<int32_t>()) {
        cafe_config cfg{device, 0, 4, 0};
        check(nullptr, cafe_ctx_create(&cfg, &ctx));
        std::vector<const clade*> nodes;
        tree->apply_prefix_order([&](const clade* c) { nodes.push_back(c); });
        std::map<const clade*, int> at;
        for (size_t i = 0; i < nodes.size(); ++i) at[nodes[i]] = (int)i;
        std::vector<int32_t> parent(nodes.size());
        std::vector<double> bl(nodes.size());
        for (size_t i = 0; i < nodes.size(); ++i) {
            parent[i] = nodes[i]->get_parent() ? at[nodes[i]->get_parent()] : -1;
            bl[i] = nodes[i]->get_branch_length();
        }
        std::vector<int32_t> lam = lambda_index;
        lam.resize(nodes.size(), 0);
        check(ctx, cafe_tree_upload(ctx, (int)nodes.size(), parent.data(), bl.data(), lam.data(), &tree_id));
        std::vector<int32_t> counts;
        int leaves = 0;
        for (auto* c : nodes) leaves += c->is_leaf() ? 1 : 0;
        for (auto& gf : *fams) {
            ids.push_back(gf.id());
            for (auto* c : nodes)
                if (c->is_leaf()) counts.push_back(gf.get_species_size(c->get_taxon_name()));
        }
        check(ctx, cafe_families_upload(ctx, tree_id, counts.data(), (int64_t)fams->size(), leaves, &set_id));
    }
    ~device_inputs() {
        if (ctx) cafe_ctx_destroy(ctx);
    }
    device_inputs(const device_inputs&) = delete;
    device_inputs& operator=(const device_inputs&) = delete;

    // prior[j] = compute(j) (float-rounded by the reference) for root index j
    void set_prior(const root_equilibrium_distribution& prior, int max_root_family_size) {
        std::vector<double> pr((size_t)max_root_family_size + 1);
        for (size_t j = 0; j < pr.size(); ++j) pr[j] = prior.compute(j);
        check(ctx, cafe_prior_set(ctx, pr.data(), (int)pr.size()));
    }

    cafe_request request(const lambda* p, int max_family_size, int max_root_family_size, std::vector<double>& lambdas) {
        lambdas = get_lambda_values(p);
        cafe_request rq{};
        rq.tree_id = tree_id;
        rq.set_id = set_id;
        rq.model = CAFE_MODEL_BASE;
        rq.lambda_kind = dynamic_cast<const single_lambda*>(p) ? CAFE_LAMBDA_SINGLE : CAFE_LAMBDA_MULTIPLE;
        rq.n_lambdas = (int)lambdas.size();
        rq.lambdas = lambdas.data();
        rq.n_categories = 1;
        rq.max_family_size = max_family_size;
        rq.max_root_family_size = max_root_family_size;
        rq.precision = CAFE_PREC_FP64_REF;
        rq.dedupe = 1;
        return rq;
    }
};

// base_model::infer_family_likelihoods (src/base_model.cpp:53-100) on the GPU.
class gpu_base_model : public base_model {
    device_inputs _dev;

public:
    gpu_base_model(lambda* l, const clade* tree, const std::vector<gene_family>* fams, int max_family_size,
                   int max_root_family_size, error_model* em, int device = 0,
                   const std::vector<int32_t>& lambda_index = std::vector<int32_t>())
        : base_model(l, tree, fams, max_family_size, max_root_family_size, em), _dev(tree, fams, device, lambda_index) {
        if (em) throw std::runtime_error("gpu_base_model: pass the error model's rows with cafe_error_model_set");
    }

    double infer_family_likelihoods(const root_equilibrium_distribution& prior, const lambda* p) override {
        _dev.set_prior(prior, _max_root_family_size);
        std::vector<double> lambdas;
        cafe_request rq = _dev.request(p, _max_family_size, _max_root_family_size, lambdas);
        std::vector<double> lnl(_dev.ids.size());
        cafe_result res{};
        res.family_lnl = lnl.data();
        check(_dev.ctx, cafe_score(_dev.ctx, &rq, &res));
        results.clear();
        for (size_t i = 0; i < lnl.size(); ++i)
            results.push_back(family_info_stash(_dev.ids[i], 0.0, 0.0, 0.0, lnl[i], false));
        return res.total_neg_lnl;   // +inf where the reference returns -log(0)
    }
};

// gamma_model::infer_family_likelihoods (src/gamma_core.cpp:168-237) on the
// GPU, for the (n_gamma_cats, alpha) form: every category has probability
// 1/K (get_gamma, src/gamma.cpp:225-241) and the multipliers are read from
// the model at each call (set_alpha changes them).
class gpu_gamma_model : public gamma_model {
    device_inputs _dev;
    int _k;

public:
    gpu_gamma_model(lambda* l, clade* tree, std::vector<gene_family>* fams, int max_family_size,
                    int max_root_family_size, int n_gamma_cats, double alpha, error_model* em, int device = 0,
                    const std::vector<int32_t>& lambda_index = std::vector<int32_t>())
        : gamma_model(l, tree, fams, max_family_size, max_root_family_size, n_gamma_cats, alpha, em),
          _dev(tree, fams, device, lambda_index), _k(n_gamma_cats) {
        if (em) throw std::runtime_error("gpu_gamma_model: pass the error model's rows with cafe_error_model_set");
    }

    double infer_family_likelihoods(const root_equilibrium_distribution& prior, const lambda* p) override {
        _dev.set_prior(prior, _max_root_family_size);
        std::vector<double> lambdas;
        cafe_request rq = _dev.request(p, _max_family_size, _max_root_family_size, lambdas);
        std::vector<double> mult = get_lambda_multipliers();
        std::vector<double> probs(mult.size(), 1.0 / (double)mult.size());
        rq.model = CAFE_MODEL_GAMMA;
        rq.n_categories = (int)mult.size();
        rq.multipliers = mult.data();
        rq.cat_probs = probs.data();
        rq.dedupe = 0;
        std::vector<double> lnl(_dev.ids.size());
        cafe_result res{};
        res.family_lnl = lnl.data();
        check(_dev.ctx, cafe_score(_dev.ctx, &rq, &res));
        results.clear();
        for (size_t i = 0; i < lnl.size(); ++i)
            results.push_back(family_info_stash(_dev.ids[i], 0.0, 0.0, 0.0, lnl[i], false));
        return res.total_neg_lnl;
    }
};

}  // namespace cafe_gpu

#endif
