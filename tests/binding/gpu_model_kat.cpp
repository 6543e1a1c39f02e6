// Test driver of the reference-side binding (include/gpu_model.h): the
// reference's infer_processes known-answer case (test.cpp:461-488: tree
// (A:1,B:1), four families, lambda 0.01, max family size 56, root bound 8,
// uniform prior over 100 sizes; -lnL 46.56632) scored by the reference's
// base_model and by gpu_base_model. Built by `make -C oracle binding`
// against the reference's own objects; run by tests/test_binding_cpu.py.
// Prints "reference <value>" and "gpu <value>", or "gpu unavailable" and
// exits 3 where no GPU is present.
#include <cstdio>
#include <memory>
#include <random>
#include <vector>

#include "easylogging++.h"
#include "base_model.h"
#include "clade.h"
#include "gene_family.h"
#include "lambda.h"
#include "root_equilibrium_distribution.h"

#include "gpu_model.h"

INITIALIZE_EASYLOGGINGPP

std::mt19937 randomizer_engine(10);

void init_lgamma_cache();

int main() {
    el::Configurations conf;
    conf.setToDefault();
    conf.set(el::Level::Global, el::ConfigurationType::Enabled, "false");
    el::Loggers::reconfigureAllLoggers(conf);
    init_lgamma_cache();

    std::unique_ptr<clade> tree(parse_newick("(A:1,B:1);", false));
    std::vector<gene_family> families(4);
    const int counts[4][2] = {{1, 2}, {2, 1}, {3, 6}, {6, 3}};
    for (int f = 0; f < 4; ++f) {
        families[f].set_id("f" + std::to_string(f + 1));
        families[f].set_species_size("A", counts[f][0]);
        families[f].set_species_size("B", counts[f][1]);
    }
    single_lambda lambda(0.01);
    root_equilibrium_distribution prior(size_t(100));

    base_model core(&lambda, tree.get(), &families, 56, 8, NULL);
    std::printf("reference %.17g\n", core.infer_family_likelihoods(prior, &lambda));
    try {
        cafe_gpu::gpu_base_model gpu(&lambda, tree.get(), &families, 56, 8, nullptr);
        std::printf("gpu %.17g\n", gpu.infer_family_likelihoods(prior, &lambda));
    } catch (std::exception& e) {
        std::printf("gpu unavailable: %s\n", e.what());
        return 3;
    }
    return 0;
}
