// selector_abi.cpp -- algorithm 14 (deployable AdaptiveOrder) behind the C ABI.
//
// The reference selects one reordering arm for the whole graph
// (GenerateAdaptiveMappingFullGraphStandalone,
// bench/include/graphbrew/reorder/reorder_adaptive.h:517-715): it parses the
// option fields after "14:" (ParseDeployableSelectionPolicy, :166-228),
// computes Tier-0 sampled features and the kernel's modeled property working
// set against the last-level cache, and applies a frozen rule
// (SelectAllKernelLowReuseRule :335-385, SelectBudgetedOneUseRule :259-300).
// Here the features come from the GPU (gbgpu_tier0_features), the cache is the
// GPU's L2 (the kernels run there), and a third model, "learned-mlp", replaces
// the rule with the library's MLP: standardised features -> 64 -> 64 -> 3
// predicted log10 end-to-end times of the arms (algorithm 12, DBG "5", the
// original order "0"), smallest wins, evaluated on the GPU by the same forward
// kernel that trained it.  The frozen rule stays as the fallback where the
// features leave the training range (more than a quarter of the range outside
// it on any feature).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "gbgpu.h"

void gb_ctx_set_error(gbgpu_ctx* ctx, const char* msg);
int gb_ctx_device(gbgpu_ctx* ctx);

struct gbgpu_selector_model_data {
    gbgpu_selector_model view;
    std::vector<float> params;
    std::vector<double> mean, std, lo, hi;
};

namespace {

enum Model {
    kPerceptron = 0,
    kDecisionTree = 1,
    kHybrid = 2,
    kKnn = 3,
    kFamily = 4,
    kTopN = 5,
    kIndividual = 6,
    kBudgeted = 7,
    kAllKernel = 8,
    kLearnedMlp = 9,
};
enum Criterion { kFastestReorder = 0, kFastestExecution = 1, kBestEndToEnd = 2, kBestAmortization = 3 };

struct ParseError : std::invalid_argument {
    using std::invalid_argument::invalid_argument;
};

const char* model_name(int m) {
    switch (m) {
        case kPerceptron: return "perceptron";
        case kDecisionTree: return "decision-tree";
        case kHybrid: return "hybrid";
        case kKnn: return "knn-database";
        case kFamily: return "family";
        case kTopN: return "topn";
        case kIndividual: return "individual";
        case kBudgeted: return "budgeted-rule";
        case kAllKernel: return "allkernel-lowreuse-rule";
        case kLearnedMlp: return "learned-mlp";
        default: return "unknown";
    }
}

const char* criterion_name(int c) {
    switch (c) {
        case kFastestReorder: return "fastest-reorder";
        case kFastestExecution: return "fastest-execution";
        case kBestEndToEnd: return "best-endtoend";
        case kBestAmortization: return "best-amortization";
        default: return "unknown-criterion";
    }
}

// GetSelectionModel (reorder_types.h:1927-1946) plus this library's learned model.
int model_of(const std::string& n) {
    if (n == "perceptron" || n == "perc" || n == "p") return kPerceptron;
    if (n == "decision-tree" || n == "dt" || n == "tree") return kDecisionTree;
    if (n == "hybrid" || n == "model-tree" || n == "hme") return kHybrid;
    if (n == "knn-database" || n == "knn" || n == "database" || n == "db") return kKnn;
    if (n == "family" || n == "fam") return kFamily;
    if (n == "topn" || n == "top-n" || n == "top") return kTopN;
    if (n == "individual" || n == "ind" || n == "all") return kIndividual;
    if (n == "budgeted-rule" || n == "budgeted" || n == "one-use-rule") return kBudgeted;
    if (n == "allkernel-lowreuse-rule" || n == "allkernel-rule" || n == "lowreuse-rule") return kAllKernel;
    if (n == "learned-mlp" || n == "mlp" || n == "learned") return kLearnedMlp;
    throw ParseError("Unknown adaptive selection model: " + n);
}

// GetSelectionCriterion (reorder_types.h:1951-1958).
int criterion_of(const std::string& n) {
    if (n == "fastest-reorder" || n == "reorder" || n == "fr") return kFastestReorder;
    if (n == "fastest-execution" || n == "execution" || n == "fe") return kFastestExecution;
    if (n == "best-endtoend" || n == "endtoend" || n == "e2e") return kBestEndToEnd;
    if (n == "best-amortization" || n == "amortization" || n == "amortize") return kBestAmortization;
    throw ParseError("Unknown adaptive selection criterion: " + n);
}

// The legacy single-field modes (GetSelectionMode + DecomposeSelectionMode,
// reorder_types.h:1992-2023): number or name -> (model, criterion).
bool legacy_mode(const std::string& s, int* m, int* c) {
    struct Row {
        const char* names[5];
        int model, crit;
    };
    static const Row rows[] = {
        {{"0", "fastest-reorder", "reorder", nullptr, nullptr}, kPerceptron, kFastestReorder},
        {{"1", "fastest-execution", "execution", "cache", nullptr}, kPerceptron, kFastestExecution},
        {{"2", "best-endtoend", "endtoend", "e2e", nullptr}, kPerceptron, kBestEndToEnd},
        {{"3", "best-amortization", "amortization", "amortize", nullptr}, kPerceptron, kBestAmortization},
        {{"4", "decision-tree", "dt", "tree", nullptr}, kDecisionTree, kFastestExecution},
        {{"5", "hybrid", "model-tree", "hme", nullptr}, kHybrid, kFastestExecution},
        {{"6", "database", "db", "knn", nullptr}, kKnn, kFastestExecution},
    };
    for (const Row& r : rows)
        for (const char* nm : r.names)
            if (nm && s == nm) {
                *m = r.model;
                *c = r.crit;
                return true;
            }
    return false;
}

std::vector<std::string> split_colon(const std::string& s) {
    std::vector<std::string> out;
    if (s.empty()) return out;
    size_t start = 0;
    while (true) {
        const size_t p = s.find(':', start);
        out.push_back(s.substr(start, p == std::string::npos ? std::string::npos : p - start));
        if (p == std::string::npos) break;
        start = p + 1;
    }
    return out;
}

bool given(const std::string& f) { return !f.empty() && f != "_"; }

// ParseDeployableSelectionPolicy (reorder_adaptive.h:166-228), with the same
// exception texts; "learned-mlp" is deployable and, like the rules, needs an
// explicit reuse count (it is one of its inputs).
gbgpu_selection_policy parse_policy(const std::vector<std::string>& o) {
    gbgpu_selection_policy p{};
    p.model = kPerceptron;
    p.criterion = kFastestExecution;
    p.reuse = 1.0;
    p.reuse_explicit = 0;
    for (size_t i = 0; i < std::min<size_t>(3, o.size()); ++i)
        if (given(o[i])) throw ParseError("AdaptiveOrder reserved fields must be empty");
    const std::string ms = o.size() > 3 ? o[3] : "", cs = o.size() > 4 ? o[4] : "", rs = o.size() > 5 ? o[5] : "";
    if (given(ms)) {
        if (given(cs)) {
            if (ms.find(':') != std::string::npos)
                throw ParseError("AdaptiveOrder model and criterion were specified twice");
            p.model = model_of(ms);
            p.criterion = criterion_of(cs);
        } else {
            const size_t colon = ms.find(':');
            int m = 0, c = 0;
            if (colon != std::string::npos) {
                m = model_of(ms.substr(0, colon));
                c = criterion_of(ms.substr(colon + 1));
            } else if (!legacy_mode(ms, &m, &c)) {
                m = model_of(ms);
                c = kFastestExecution;
            }
            p.model = m;
            p.criterion = c;
        }
    } else if (given(cs)) {
        throw ParseError("AdaptiveOrder criterion requires an explicit model");
    }
    if (given(rs)) {
        size_t used = 0;
        double r = 0.0;
        try {
            r = std::stod(rs, &used);
        } catch (const std::out_of_range&) {
            throw ParseError("stod");
        } catch (const std::invalid_argument&) {
            throw ParseError("stod");
        }
        if (used != rs.size() || !std::isfinite(r) || r <= 0.0)
            throw ParseError("AdaptiveOrder reuse count must be positive");
        p.reuse = r;
        p.reuse_explicit = 1;
    }
    for (size_t i = 6; i < o.size(); ++i)
        if (given(o[i]))
            throw ParseError(
                "AdaptiveOrder no longer accepts graph identity or additional runtime selection fields");
    const bool deployable = p.model == kPerceptron || p.model == kBudgeted || p.model == kAllKernel ||
                            p.model == kLearnedMlp;
    if (!deployable)
        throw ParseError(std::string(model_name(p.model)) + " is offline-only and cannot drive deployable AdaptiveOrder");
    if ((p.model == kBudgeted || p.model == kAllKernel || p.model == kLearnedMlp) && !p.reuse_explicit)
        throw ParseError(std::string(model_name(p.model)) + " requires an explicit reuse count");
    return p;
}

// ModeledPropertyBytes (reorder_types.h:1226-1258).
uint64_t property_bytes(int kernel, uint64_t nodes, uint64_t edges) {
    const uint64_t id = 4, score = 4, count = 8, bitmap = (nodes + 7) / 8;
    switch (kernel) {
        case GBGPU_KERNEL_PR:
        case GBGPU_KERNEL_PR_SPMV: return nodes * 2 * score;
        case GBGPU_KERNEL_BFS: return nodes * 2 * id + 2 * bitmap;
        case GBGPU_KERNEL_CC:
        case GBGPU_KERNEL_CC_SV: return nodes * id + bitmap;
        case GBGPU_KERNEL_SSSP: return nodes * id + edges * id;
        case GBGPU_KERNEL_BC: return nodes * (score + count + 2 * id) + (edges + 7) / 8;
        case GBGPU_KERNEL_TC: return nodes * id;
        default: throw ParseError("Kernel-specific modeled property bytes are unavailable");
    }
}

const char* kRecipe12 = "12:leiden:compose:sg_none:comm_size_desc:intra_gorder:gw8:cd_parallel:sgmb4096:gordf5000:norefine:2:2";
const char* kRecipeBudgeted = "12:leiden:compose:sg_none:comm_identity:intra_gorder:gw32:gordf500:cd_parallel:1:1";

void set_arm(gbgpu_selection* out, int arm, const char* applied, const char* reason) {
    out->arm = arm;
    std::snprintf(out->applied, sizeof(out->applied), "%s", applied);
    std::snprintf(out->reason, sizeof(out->reason), "%s", reason);
}

// ShouldUseAllKernelLowReuseRule (reorder_adaptive.h:302-333): features are
// num_nodes [0], avg_degree [2], degree variation [3], and the working-set
// ratio computed above.
void allkernel_rule(const double* f, int kernel, double reuse, double wsr, gbgpu_selection* out) {
    const bool supported = kernel == GBGPU_KERNEL_PR || kernel == GBGPU_KERNEL_PR_SPMV || kernel == GBGPU_KERNEL_BFS ||
                           kernel == GBGPU_KERNEL_CC || kernel == GBGPU_KERNEL_CC_SV || kernel == GBGPU_KERNEL_BC ||
                           kernel == GBGPU_KERNEL_SSSP;
    const bool use = supported && reuse <= 2.0 && f[0] >= 1000 && wsr <= 3.2 &&
                     ((f[3] <= 2.68 && (f[2] <= 60.0 || wsr <= 0.82)) || f[3] > 8.0);
    if (use) set_arm(out, 12, kRecipe12, "allkernel-lowreuse-match");
    else set_arm(out, 5, "5", "allkernel-lowreuse-fallback");
}

// ShouldUseBudgetedLeidenGorder (reorder_adaptive.h:240-257).
void budgeted_rule(const double* f, int kernel, double reuse, gbgpu_selection* out) {
    const bool pr = kernel == GBGPU_KERNEL_PR || kernel == GBGPU_KERNEL_PR_SPMV;
    const bool use = pr && reuse <= 1.0 && f[0] >= 1000 && f[2] >= 45.0 && f[3] < 3.0 && f[5] >= 0.3;
    if (use) set_arm(out, 12, kRecipeBudgeted, "budgeted-one-use-match");
    else set_arm(out, 5, "5", "budgeted-one-use-fallback");
}

struct Fail {
    int status;
    std::string msg;
};

}  // namespace

extern "C" {

int gbgpu_parse_selection_policy(const char* opts, gbgpu_selection_policy* out, char* err, size_t err_len) {
    if (err && err_len) err[0] = '\0';
    if (!out) return GBGPU_E_INVALID;
    try {
        *out = parse_policy(split_colon(opts ? opts : ""));
        return GBGPU_OK;
    } catch (const std::exception& e) {
        if (err && err_len) std::snprintf(err, err_len, "%s", e.what());
        return GBGPU_E_PARSE;
    }
}

const char* gbgpu_selection_model_name(int32_t model) { return model_name(model); }
const char* gbgpu_selection_criterion_name(int32_t criterion) { return criterion_name(criterion); }

int64_t gbgpu_modeled_property_bytes(int32_t kernel, int64_t nodes, int64_t directed_edges) {
    try {
        return (int64_t)property_bytes(kernel, (uint64_t)nodes, (uint64_t)directed_edges);
    } catch (const std::exception&) {
        return -1;
    }
}

int gbgpu_apply_selection_rule(int32_t model, const double* features, double property_wsr, int32_t kernel,
                               double reuse, gbgpu_selection* out) {
    if (!features || !out) return GBGPU_E_INVALID;
    if (model == kAllKernel) allkernel_rule(features, kernel, reuse, property_wsr, out);
    else if (model == kBudgeted) budgeted_rule(features, kernel, reuse, out);
    else return GBGPU_E_UNSUPPORTED;
    return GBGPU_OK;
}

int gbgpu_selector_model_load(const char* path, gbgpu_selector_model** out) {
    if (!path || !out) return GBGPU_E_INVALID;
    *out = nullptr;
    std::ifstream in(path, std::ios::binary);
    if (!in) return GBGPU_E_INVALID;
    char magic[8];
    int32_t dims[4];
    int64_t cache = 0;
    in.read(magic, 8);
    in.read(reinterpret_cast<char*>(dims), sizeof(dims));
    in.read(reinterpret_cast<char*>(&cache), sizeof(cache));
    if (!in || std::memcmp(magic, "GBSEL01\0", 8) != 0) return GBGPU_E_INVALID;
    const int in_dim = dims[0];
    if (in_dim <= 0 || in_dim > 256 || dims[1] != 64 || dims[2] != 3 || cache <= 0) return GBGPU_E_INVALID;
    const int count = gbgpu_mlp_param_count(in_dim);
    auto* m = new gbgpu_selector_model_data();
    m->params.resize(count);
    m->mean.resize(in_dim);
    m->std.resize(in_dim);
    m->lo.resize(in_dim);
    m->hi.resize(in_dim);
    in.read(reinterpret_cast<char*>(m->params.data()), count * sizeof(float));
    for (std::vector<double>* v : {&m->mean, &m->std, &m->lo, &m->hi})
        in.read(reinterpret_cast<char*>(v->data()), in_dim * sizeof(double));
    if (!in) {
        delete m;
        return GBGPU_E_INVALID;
    }
    m->view.in_dim = in_dim;
    m->view.params = m->params.data();
    m->view.mean = m->mean.data();
    m->view.std = m->std.data();
    m->view.lo = m->lo.data();
    m->view.hi = m->hi.data();
    m->view.cache_bytes = cache;
    *out = &m->view;
    return GBGPU_OK;
}

void gbgpu_selector_model_free(gbgpu_selector_model* m) {
    if (!m) return;
    delete reinterpret_cast<gbgpu_selector_model_data*>(reinterpret_cast<char*>(m) -
                                                        offsetof(gbgpu_selector_model_data, view));
}

int gbgpu_select_arm(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz,
                     const char* opts, int32_t kernel, const gbgpu_selector_model* model, gbgpu_selection* out,
                     uint32_t flags) {
    if (!ctx) return GBGPU_E_INVALID;
    if (!out) {
        gb_ctx_set_error(ctx, "gbgpu_select_arm: null selection");
        return GBGPU_E_INVALID;
    }
    std::memset(out, 0, sizeof(*out));
    try {
        const gbgpu_selection_policy p = parse_policy(split_colon(opts ? opts : ""));
        out->policy = p;
        if (n == 0) {   // an empty graph keeps the identity map (reorder_adaptive.h:536-540)
            set_arm(out, 0, "0", "empty-graph");
            gb_ctx_set_error(ctx, "");
            return GBGPU_OK;
        }
        if (p.model == kPerceptron)
            throw Fail{GBGPU_E_UNSUPPORTED,
                       "perceptron selection needs the reference's trained weight database; use "
                       "allkernel-lowreuse-rule, budgeted-rule or learned-mlp"};
        if ((p.model == kAllKernel || p.model == kBudgeted) && p.criterion != kBestEndToEnd)
            throw ParseError(std::string(model_name(p.model)) + " requires best-endtoend criterion");
        int rc = gbgpu_tier0_features(ctx, row_ptr, col, n, nnz, out->features, flags);
        if (rc != GBGPU_OK) return rc;   // error text set by the features call
        int64_t cache = 0;
        if (p.model == kLearnedMlp) {
            if (!model) throw Fail{GBGPU_E_INVALID, "learned-mlp selection needs a model (gbgpu_selector_model_load)"};
            cache = model->cache_bytes;
        } else {
            int l2 = 0;
            if (cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, gb_ctx_device(ctx)) != cudaSuccess || l2 <= 0)
                throw Fail{GBGPU_E_CUDA, "cannot read the device's L2 size"};
            cache = l2;
        }
        out->cache_bytes = cache;
        out->property_bytes = (int64_t)property_bytes(kernel, (uint64_t)n, (uint64_t)nnz);
        out->property_wsr = (double)out->property_bytes / (double)cache;
        const double* f = out->features;
        if (p.model == kBudgeted) {
            budgeted_rule(f, kernel, p.reuse, out);
        } else if (p.model == kAllKernel) {
            allkernel_rule(f, kernel, p.reuse, out->property_wsr, out);
        } else {
            // learned-mlp: the feature vector of graphbrew_gb300.selector.feature_vector.
            const int in_dim = model->in_dim;
            const bool mlp_kernel = kernel == GBGPU_KERNEL_PR || kernel == GBGPU_KERNEL_BFS || kernel == GBGPU_KERNEL_CC;
            std::vector<double> x = {std::log10(f[0] + 1.0), std::log10(f[1] + 1.0), f[2], f[3], f[5], f[7], f[8],
                                     out->property_wsr, kernel == GBGPU_KERNEL_PR ? 1.0 : 0.0,
                                     kernel == GBGPU_KERNEL_BFS ? 1.0 : 0.0, kernel == GBGPU_KERNEL_CC ? 1.0 : 0.0,
                                     p.reuse};
            if ((int)x.size() != in_dim) throw Fail{GBGPU_E_INVALID, "selector model expects a different feature count"};
            bool in_range = mlp_kernel;
            for (int i = 0; i < in_dim && in_range; ++i) {
                const double span = model->hi[i] - model->lo[i];
                in_range = x[i] >= model->lo[i] - 0.25 * span && x[i] <= model->hi[i] + 0.25 * span;
            }
            if (!in_range) {
                allkernel_rule(f, kernel, p.reuse, out->property_wsr, out);
                std::snprintf(out->reason, sizeof(out->reason), "%s", "frozen-rule-fallback");
            } else {
                std::vector<float> xs(in_dim);
                for (int i = 0; i < in_dim; ++i) xs[i] = (float)((x[i] - model->mean[i]) / model->std[i]);
                rc = gbgpu_mlp_forward(ctx, model->params, xs.data(), 1, in_dim, out->predicted_log10_ms, 0);
                if (rc != GBGPU_OK) return rc;
                int best = 0;
                for (int k = 1; k < 3; ++k)
                    if (out->predicted_log10_ms[k] < out->predicted_log10_ms[best]) best = k;
                static const int arms[3] = {12, 5, 0};
                static const char* specs[3] = {kRecipe12, "5", "0"};
                set_arm(out, arms[best], specs[best], "learned-mlp");
            }
        }
        gb_ctx_set_error(ctx, "");
        return GBGPU_OK;
    } catch (const Fail& e) {
        gb_ctx_set_error(ctx, e.msg.c_str());
        return e.status;
    } catch (const ParseError& e) {
        gb_ctx_set_error(ctx, e.what());
        return GBGPU_E_PARSE;
    } catch (const std::exception& e) {
        gb_ctx_set_error(ctx, e.what());
        return GBGPU_E_INVALID;
    }
}

}  // extern "C"
