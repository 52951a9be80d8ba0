// ref_harness.cc -- C entry points into the GraphBrew reference, compiled from
// the reference's own headers where they lie (see Makefile, target "ref").
//
// TEST INFRASTRUCTURE ONLY.  It is built in the development container, where
// the GraphBrew sources are mounted, and used to pin the plain-C oracle and to
// generate the golden fixtures under tests/golden/.  Nothing here ships, and
// nothing on the GPU path can load it (the sources are absent there).
#include <fcntl.h>
#include <unistd.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_set>
#include <vector>

#include "benchmark.h"
#include "builder.h"
#include "graphbrew/reorder/reorder_graphbrew.h"

namespace {

// Silences the reference's stdout progress lines during a call.
struct QuietStdout {
    int saved = -1;
    explicit QuietStdout(bool on) {
        if (!on) return;
        fflush(stdout);
        saved = dup(1);
        int devnull = open("/dev/null", O_WRONLY);
        dup2(devnull, 1);
        close(devnull);
    }
    ~QuietStdout() {
        if (saved < 0) return;
        fflush(stdout);
        dup2(saved, 1);
        close(saved);
    }
};

Graph MakeGraph(int64_t n, const int64_t* row_ptr, const int32_t* col) {
    const int64_t nnz = row_ptr[n];
    auto* neighs = new NodeID[nnz > 0 ? nnz : 1];
    std::memcpy(neighs, col, sizeof(NodeID) * nnz);
    auto** index = new NodeID*[n + 1];
    for (int64_t u = 0; u <= n; ++u) index[u] = neighs + row_ptr[u];
    return Graph(n, index, neighs);
}

std::vector<std::string> SplitTokens(const char* opts) {
    std::vector<std::string> out;
    std::string s(opts ? opts : "");
    size_t start = 0;
    while (true) {
        size_t colon = s.find(':', start);
        out.push_back(s.substr(start, colon == std::string::npos ? std::string::npos : colon - start));
        if (colon == std::string::npos) break;
        start = colon + 1;
    }
    if (out.size() == 1 && out[0].empty()) out.clear();
    return out;
}

void CopyError(const std::exception& e, char* err, size_t cap) {
    if (err && cap) {
        std::snprintf(err, cap, "%s", e.what());
    }
}

Graph* g_last = nullptr;

}  // namespace

extern "C" {

void ref_set_threads(int threads) {
    if (threads > 0) omp_set_num_threads(threads);
}

double ref_auto_resolution(int64_t n, const int64_t* row_ptr, const int32_t* col) {
    Graph g = MakeGraph(n, row_ptr, col);
    return computeAutoResolution<NodeID, NodeID>(g);
}

// parseGraphBrewCliConfig + graphBrewEffectiveConfigJson.  Returns 0 and the
// JSON, or -1 and the exception text.
int ref_effective_config_json(const char* opts, double auto_resolution, char* out, size_t cap) {
    try {
        auto config = graphbrew::parseGraphBrewCliConfig(SplitTokens(opts), auto_resolution);
        std::string json = graphbrew::graphBrewEffectiveConfigJson(config);
        std::snprintf(out, cap, "%s", json.c_str());
        return 0;
    } catch (const std::exception& e) {
        CopyError(e, out, cap);
        return -1;
    }
}

// runGraphBrew -> membership (and summary counts).
int ref_run_graphbrew(int64_t n, const int64_t* row_ptr, const int32_t* col,
                      const char* opts, double auto_resolution,
                      uint32_t* membership, int64_t* summary /* passes, iters, comms */,
                      int quiet, char* err, size_t cap) {
    try {
        QuietStdout q(quiet != 0);
        Graph g = MakeGraph(n, row_ptr, col);
        auto config = graphbrew::parseGraphBrewCliConfig(SplitTokens(opts), auto_resolution);
        auto result = graphbrew::runGraphBrew<uint32_t>(g, config);
        for (int64_t i = 0; i < n; ++i) membership[i] = result.membership[i];
        if (summary) {
            summary[0] = result.totalPasses;
            summary[1] = result.totalIterations;
            summary[2] = static_cast<int64_t>(result.numCommunities);
        }
        return 0;
    } catch (const std::exception& e) {
        CopyError(e, err, cap);
        return -1;
    }
}

// orderCompose on a given membership.
int ref_order_compose(int64_t n, const int64_t* row_ptr, const int32_t* col,
                      const uint32_t* membership, const char* opts, double auto_resolution,
                      int32_t* new_ids, int64_t* gorder_stats /* 5 entries */,
                      int quiet, char* err, size_t cap) {
    try {
        QuietStdout q(quiet != 0);
        Graph g = MakeGraph(n, row_ptr, col);
        auto config = graphbrew::parseGraphBrewCliConfig(SplitTokens(opts), auto_resolution);
        graphbrew::GraphBrewResult<uint32_t> result;
        result.membership.assign(membership, membership + n);
        std::unordered_set<uint32_t> uniq(result.membership.begin(), result.membership.end());
        result.numCommunities = uniq.size();
        std::vector<uint32_t> degrees(n);
        for (int64_t u = 0; u < n; ++u) degrees[u] = static_cast<uint32_t>(g.out_degree(u));
        pvector<NodeID> ids(n);
        auto realized = graphbrew::makeGraphBrewRealizedConfig(config);
        graphbrew::orderCompose<uint32_t, NodeID, NodeID>(ids, result, degrees, g, n, config, &realized);
        for (int64_t i = 0; i < n; ++i) new_ids[i] = ids[i];
        if (gorder_stats) {
            gorder_stats[0] = realized.gorderCommunities;
            gorder_stats[1] = realized.gorderVertices;
            gorder_stats[2] = realized.gorderMaxCommunity;
            gorder_stats[3] = realized.gorderFallbackCommunities;
            gorder_stats[4] = realized.gorderFallbackVertices;
        }
        return 0;
    } catch (const std::exception& e) {
        CopyError(e, err, cap);
        return -1;
    }
}

// generateGraphBrewMapping end to end (Leiden + ordering).
int ref_generate_mapping(int64_t n, const int64_t* row_ptr, const int32_t* col,
                         const char* opts, double auto_resolution, int32_t* new_ids,
                         int quiet, char* err, size_t cap) {
    try {
        QuietStdout q(quiet != 0);
        Graph g = MakeGraph(n, row_ptr, col);
        auto config = graphbrew::parseGraphBrewCliConfig(SplitTokens(opts), auto_resolution);
        pvector<NodeID> ids(n);
        graphbrew::generateGraphBrewMapping<uint32_t>(g, ids, config);
        for (int64_t i = 0; i < n; ++i) new_ids[i] = ids[i];
        return 0;
    } catch (const std::exception& e) {
        CopyError(e, err, cap);
        return -1;
    }
}

// RelabelByMapping (undirected) -> rebuilt CSR and the composed org ids.
int ref_relabel(int64_t n, const int64_t* row_ptr, const int32_t* col, const int32_t* new_ids,
                int64_t* out_row_ptr, int32_t* out_col, int32_t* org_ids, int quiet) {
    QuietStdout q(quiet != 0);
    Graph g = MakeGraph(n, row_ptr, col);
    pvector<NodeID> ids(n);
    for (int64_t i = 0; i < n; ++i) ids[i] = new_ids[i];
    Graph r = Builder::RelabelByMapping(g, ids);
    out_row_ptr[0] = 0;
    int64_t pos = 0;
    for (int64_t u = 0; u < n; ++u) {
        for (NodeID v : r.out_neigh(u)) out_col[pos++] = v;
        out_row_ptr[u + 1] = pos;
    }
    if (org_ids) {
        const NodeID* org = r.get_org_ids();
        for (int64_t i = 0; i < n; ++i) org_ids[i] = org[i];
    }
    return 0;
}

double ref_modularity(int64_t n, const int64_t* row_ptr, const int32_t* col,
                      const uint32_t* membership, double resolution) {
    Graph g = MakeGraph(n, row_ptr, col);
    std::vector<uint32_t> comm(membership, membership + n);
    return computeModularityCSR<uint32_t, NodeID, NodeID>(g, comm, resolution);
}

// Local Gorder on an explicit directed adjacency (the shape of the
// reference's own known-answer test, test_graphbrew_config.cc:974-1000).
int ref_gorder_kat(int64_t n, const int64_t* row_ptr, const int32_t* col, int window,
                   int32_t* local_ids) {
    std::vector<std::vector<NodeID>> out(n), in(n);
    int64_t ne = 0;
    for (int64_t u = 0; u < n; ++u)
        for (int64_t e = row_ptr[u]; e < row_ptr[u + 1]; ++e) {
            out[u].push_back(col[e]);
            in[col[e]].push_back(static_cast<NodeID>(u));
            ++ne;
        }
    auto build = [&](const std::vector<std::vector<NodeID>>& rows, NodeID*& neigh) {
        neigh = new NodeID[ne > 0 ? ne : 1];
        auto** index = new NodeID*[n + 1];
        int64_t p = 0;
        for (int64_t u = 0; u < n; ++u) {
            index[u] = neigh + p;
            for (NodeID v : rows[u]) neigh[p++] = v;
        }
        index[n] = neigh + p;
        return index;
    };
    NodeID *on = nullptr, *inn = nullptr;
    NodeID** oi = build(out, on);
    NodeID** ii = build(in, inn);
    Graph g(n, oi, on, ii, inn);
    std::vector<NodeID> verts(n), membership(n, 0), degrees(n), lids(n, -1);
    std::vector<size_t> v2l(n);
    for (int64_t i = 0; i < n; ++i) {
        verts[i] = static_cast<NodeID>(i);
        degrees[i] = static_cast<NodeID>(g.out_degree(i));
        v2l[i] = static_cast<size_t>(i);
    }
    std::vector<NodeID> placed;
    std::vector<std::vector<size_t>> scratch;
    graphbrew::intraGorderGreedy<NodeID, NodeID, NodeID>(
        verts, 0, membership, degrees, g, v2l, window, placed, scratch, lids);
    for (int64_t i = 0; i < n; ++i) local_ids[i] = lids[i];
    return 0;
}

// The reference's own graph generator (-g / -u with -k), symmetrized and
// squished as the converter builds it.  Returns n; *nnz receives the entry
// count.  Call ref_last_graph_copy to fetch the CSR.
int64_t ref_gapbs_generate(int scale, int degree, int uniform, int64_t* nnz, int quiet) {
    QuietStdout q(quiet != 0);
    setenv("GRAPHBREW_TOPOLOGY_ANALYSIS", "0", 1);
    std::string s = std::to_string(scale), k = std::to_string(degree);
    static char prog[] = "gen";
    std::vector<std::string> args = {prog, uniform ? "-u" : "-g", s, "-k", k};
    std::vector<char*> argv;
    for (auto& a : args) argv.push_back(const_cast<char*>(a.c_str()));
    argv.push_back(nullptr);
    optind = 1;
    CLBase cli(static_cast<int>(args.size()), argv.data(), "gen");
    if (!cli.ParseArgs()) return -1;
    Builder b(cli);
    delete g_last;
    g_last = new Graph(b.MakeGraph());
    *nnz = g_last->num_edges_directed();
    return g_last->num_nodes();
}

void ref_last_graph_copy(int64_t* row_ptr, int32_t* col) {
    int64_t pos = 0;
    row_ptr[0] = 0;
    for (int64_t u = 0; u < g_last->num_nodes(); ++u) {
        for (NodeID v : g_last->out_neigh(u)) col[pos++] = v;
        row_ptr[u + 1] = pos;
    }
}

// GenerateDBGMapping (reorder_hub.h:267-342) on out-degrees.
void ref_dbg_mapping(int64_t n, const int64_t* row_ptr, const int32_t* col, int32_t* new_ids) {
    QuietStdout q(true);
    Graph g = MakeGraph(n, row_ptr, col);
    pvector<NodeID> ids(n);
    ::GenerateDBGMapping(g, ids, true);
    for (int64_t i = 0; i < n; ++i) new_ids[i] = ids[i];
}

// ComputeTier0SampledGraphFeatures (reorder_types.h:6066-6186), sample seed 0;
// out = num_nodes, num_edges, avg_degree, degree_variance (cv), internal_density,
// hub_concentration, packing_factor, avg_reuse_distance (normalised span),
// window_neighbor_overlap.
void ref_tier0_features(int64_t n, const int64_t* row_ptr, const int32_t* col, double* out) {
    Graph g = MakeGraph(n, row_ptr, col);
    const CommunityFeatures f = ComputeTier0SampledGraphFeatures(g);
    const double v[9] = {(double)f.num_nodes, (double)f.num_edges, f.avg_degree, f.degree_variance,
                         f.internal_density, f.hub_concentration, f.packing_factor, f.avg_reuse_distance,
                         f.window_neighbor_overlap};
    for (int i = 0; i < 9; ++i) out[i] = v[i];
}

// ParseDeployableSelectionPolicy on the fields after "14:" (split on ':'):
// model and criterion ordinals, reuse and whether it was given; or the
// exception text (return 1).
int ref_parse_selection_policy(const char* opts, int* model, int* criterion, double* reuse, int* explicit_reuse,
                               char* err, size_t cap) {
    try {
        auto p = adaptive::ParseDeployableSelectionPolicy(SplitTokens(opts));
        *model = (int)p.model;
        *criterion = (int)p.criterion;
        *reuse = p.reuse_count;
        *explicit_reuse = p.reuse_count_explicit ? 1 : 0;
        return 0;
    } catch (const std::exception& e) {
        std::snprintf(err, cap, "%s", e.what());
        return 1;
    }
}

// The two frozen rules on given features (kernel = BenchmarkType ordinal).
int ref_allkernel_rule(double num_nodes, double avg_degree, double degree_variance, double hub_concentration,
                       double wsr, int kernel, double reuse) {
    CommunityFeatures f;
    f.num_nodes = (size_t)num_nodes;
    f.avg_degree = avg_degree;
    f.degree_variance = degree_variance;
    f.hub_concentration = hub_concentration;
    f.working_set_ratio = wsr;
    return adaptive::ShouldUseAllKernelLowReuseRule(f, (BenchmarkType)kernel, reuse) ? 1 : 0;
}

int ref_budgeted_rule(double num_nodes, double avg_degree, double degree_variance, double hub_concentration,
                      int kernel, double reuse) {
    CommunityFeatures f;
    f.num_nodes = (size_t)num_nodes;
    f.avg_degree = avg_degree;
    f.degree_variance = degree_variance;
    f.hub_concentration = hub_concentration;
    return adaptive::ShouldUseBudgetedLeidenGorder(f, (BenchmarkType)kernel, reuse) ? 1 : 0;
}

// ModeledPropertyBytes; -1 when the reference throws (generic kernel).
long long ref_property_bytes(int kernel, unsigned long long nodes, unsigned long long edges) {
    try {
        return (long long)ModeledPropertyBytes((BenchmarkType)kernel, nodes, edges);
    } catch (const std::exception&) {
        return -1;
    }
}

}  // extern "C"
