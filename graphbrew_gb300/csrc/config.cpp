// config.cpp -- algorithm-12 option grammar (host, C++17).
//
// The grammar is an ordered list of rules; the first rule whose matcher
// accepts a token applies it.  The rule order, the aliases of each rule and
// the validation of numeric suffixes are those of parseGraphBrewConfig
// (bench/include/graphbrew/reorder/reorder_graphbrew_parser.h:13-707); the
// preset / positional layer is parseGraphBrewCliConfig (:714-912).  Numeric
// text is read with std::stoi / std::stod / std::stoull exactly like the
// reference, so edge cases (signs, exponents, hex floats) agree.
#include "gb_config.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <functional>
#include <initializer_list>
#include <limits>
#include <map>
#include <string>
#include <vector>

#include "gb_common.cuh"

namespace gb {

namespace {

bool exact_int(const std::string& text, int& value) {
    try {
        size_t parsed = 0;
        value = std::stoi(text, &parsed);
        return parsed == text.size();
    } catch (...) {
        return false;
    }
}

bool exact_double(const std::string& text, double& value) {
    try {
        size_t parsed = 0;
        value = std::stod(text, &parsed);
        return parsed == text.size() && std::isfinite(value);
    } catch (...) {
        return false;
    }
}

bool exact_size(const std::string& text, size_t& value) {
    if (text.empty()) return false;
    for (unsigned char ch : text)
        if (!std::isdigit(ch)) return false;
    try {
        size_t parsed = 0;
        const unsigned long long v = std::stoull(text, &parsed);
        if (parsed != text.size() || v > (unsigned long long)std::numeric_limits<size_t>::max()) return false;
        value = (size_t)v;
        return true;
    } catch (...) {
        return false;
    }
}

bool starts_with(const std::string& s, const char* p) { return s.rfind(p, 0) == 0; }

bool one_of(const std::string& s, std::initializer_list<const char*> xs) {
    for (const char* x : xs)
        if (s == x) return true;
    return false;
}

enum class Outcome { NoMatch, Applied, Rejected };

using Rule = std::function<Outcome(const std::string&, Config&)>;

// Simple alias rule.
Rule alias(std::initializer_list<const char*> names, std::function<void(Config&)> act) {
    std::vector<std::string> v(names.begin(), names.end());
    return [v, act](const std::string& t, Config& c) {
        for (const auto& n : v)
            if (t == n) { act(c); return Outcome::Applied; }
        return Outcome::NoMatch;
    };
}

void set_ordering(Config& c, Ordering o) {
    c.ordering = o;
    c.hasExplicitOrdering = true;
}

void enter_layer(Config& c) {
    c.ordering = Ordering::Layer;
    c.useSmallCommunityMerging = true;
    if (c.finalAlgoId < 0) c.finalAlgoId = 8;
}

const std::vector<Rule>& rules() {
    static const std::vector<Rule> r = [] {
        std::vector<Rule> v;
        v.push_back(alias({"cd_parallel", "cd:parallel", "community_parallel"},
                          [](Config& c) { c.deterministicCommunityDetection = false; }));
        v.push_back(alias({"cd_serial", "cd:serial", "community_serial"},
                          [](Config& c) { c.deterministicCommunityDetection = true; }));
        v.push_back([](const std::string& t, Config& c) {
            if (!(t.size() > 4 && t.compare(0, 4, "sgmb") == 0)) return Outcome::NoMatch;
            int b = 0;
            if (!exact_int(t.substr(4), b) || b <= 0) return Outcome::Rejected;
            c.superGraphMoveBatch = b;
            return Outcome::Applied;
        });
        v.push_back([](const std::string& t, Config& c) {
            if (!(t.size() > 6 && t.compare(0, 6, "capl2k") == 0)) return Outcome::NoMatch;
            size_t kib = 0;
            if (!exact_size(t.substr(6), kib) || kib == 0 || kib > std::numeric_limits<size_t>::max() / 1024)
                return Outcome::Rejected;
            c.capacityL2Bytes = kib * 1024;
            return Outcome::Applied;
        });
        v.push_back([](const std::string& t, Config& c) {
            if (!(t.size() > 7 && t.compare(0, 7, "capllck") == 0)) return Outcome::NoMatch;
            size_t kib = 0;
            if (!exact_size(t.substr(7), kib) || kib == 0 || kib > std::numeric_limits<size_t>::max() / 1024)
                return Outcome::Rejected;
            c.capacityLLCBytes = kib * 1024;
            return Outcome::Applied;
        });
        v.push_back([](const std::string& t, Config& c) {
            if (!(t.size() > 4 && t.compare(0, 4, "capv") == 0)) return Outcome::NoMatch;
            size_t bytes = 0;
            if (!exact_size(t.substr(4), bytes) || bytes == 0) return Outcome::Rejected;
            c.capacityPropertyBytesPerVertex = bytes;
            return Outcome::Applied;
        });
        v.push_back(alias({"rabbit", "rabbitorder", "cd_rabbit", "cd:rabbit", "cdrabbit"},
                          [](Config& c) { c.algorithm = Algorithm::Rabbit; }));
        v.push_back(alias({"cd_leiden", "cd:leiden", "cdleiden"}, [](Config& c) {
            c.algorithm = Algorithm::Leiden;
            c.communityMode = CommunityMode::FullLeiden;
            c.useRefinement = true;
            c.refinementDepth = -1;
        }));
        // Ordering strategies.
        v.push_back(alias({"hierarchical", "hier"}, [](Config& c) { set_ordering(c, Ordering::Hierarchical); }));
        v.push_back(alias({"connectivity", "conn", "connbfs"},
                          [](Config& c) { set_ordering(c, Ordering::ConnectivityBFS); }));
        v.push_back(alias({"dfs"}, [](Config& c) { set_ordering(c, Ordering::DendrogramDFS); }));
        v.push_back(alias({"bfs"}, [](Config& c) { set_ordering(c, Ordering::DendrogramBFS); }));
        v.push_back(alias({"community", "comm"}, [](Config& c) { set_ordering(c, Ordering::CommunitySort); }));
        v.push_back(alias({"hubcluster", "hub"}, [](Config& c) { set_ordering(c, Ordering::HubCluster); }));
        v.push_back(alias({"dbg"}, [](Config& c) { set_ordering(c, Ordering::DBG); }));
        v.push_back(alias({"corder"}, [](Config& c) { set_ordering(c, Ordering::Corder); }));
        v.push_back(alias({"dbg-global", "dbgglobal"}, [](Config& c) { set_ordering(c, Ordering::DBGGlobal); }));
        v.push_back(alias({"corder-global", "corderglobal"},
                          [](Config& c) { set_ordering(c, Ordering::CorderGlobal); }));
        v.push_back(alias({"hcache", "hiercache", "hierarchical-cache"},
                          [](Config& c) { set_ordering(c, Ordering::HierarchicalCacheAware); }));
        v.push_back(alias({"hrab", "hybrid-rabbit", "leidenrabbit"}, [](Config& c) {
            set_ordering(c, Ordering::HybridLeidenRabbit);
            c.useRCMIntra = true;
        }));
        v.push_back(alias({"tqr", "tile-quantized", "tilequantized", "tilerabbit"},
                          [](Config& c) { set_ordering(c, Ordering::TileQuantizedRabbit); }));
        v.push_back(alias({"hlr", "hier-rabbit", "hierarchical-rabbit", "hierleidenrabbit"},
                          [](Config& c) { set_ordering(c, Ordering::HierarchicalLeidenRabbit); }));
        v.push_back(alias({"compose", "pluggable"}, [](Config& c) { set_ordering(c, Ordering::Compose); }));
        // Community order.
        v.push_back(alias({"s2_size", "s2:size", "s2size", "comm_size", "comm:size", "commsize", "comm_size_desc",
                           "comm:size_desc", "commsizedesc"},
                          [](Config& c) { c.communityOrder = CommunityOrder::SizeDesc; }));
        v.push_back(alias({"s2_size_asc", "s2:size_asc", "s2sizeasc", "comm_size_asc", "comm:size_asc", "commsizeasc"},
                          [](Config& c) { c.communityOrder = CommunityOrder::SizeAsc; }));
        v.push_back(alias({"s2_degree", "s2:degree", "s2degree", "comm_degree", "comm:degree", "commdegree",
                           "comm_degree_desc", "comm:degree_desc", "commdegreedesc"},
                          [](Config& c) { c.communityOrder = CommunityOrder::DegreeDesc; }));
        v.push_back(alias({"s2_degree_asc", "s2:degree_asc", "s2degreeasc", "comm_degree_asc", "comm:degree_asc",
                           "commdegreeasc"},
                          [](Config& c) { c.communityOrder = CommunityOrder::DegreeAsc; }));
        v.push_back(alias({"s2_capacity", "s2:capacity", "comm_capacity_runs", "comm:capacity_runs", "comm_cache_fit",
                           "capacity_runs", "cache_fit"},
                          [](Config& c) { c.communityOrder = CommunityOrder::CapacityRuns; }));
        v.push_back(alias({"s2_cut_min", "s2:cut_min", "s2cutmin", "comm_cut_min", "comm:cut_min", "commcutmin",
                           "cut_min", "cutmin"},
                          [](Config& c) { c.communityOrder = CommunityOrder::CutMin; }));
        // Intra-community order.
        v.push_back(alias({"s3_bfs", "s3:bfs", "s3bfs", "intra_bfs", "intra:bfs", "intrabfs"},
                          [](Config& c) { c.intraCommunityOrder = IntraOrder::BFSFromHub; }));
        v.push_back(alias({"s3_rcm", "s3:rcm", "s3rcm", "intra_rcm", "intra:rcm", "intrarcm"},
                          [](Config& c) { c.intraCommunityOrder = IntraOrder::RCM; }));
        v.push_back(alias({"s3_rcmpp", "s3:rcmpp", "s3rcmpp", "intra_rcmpp", "intra:rcmpp", "intrarcmpp", "rcmpp",
                           "rcm++"},
                          [](Config& c) { c.intraCommunityOrder = IntraOrder::RCMpp; }));
        v.push_back(alias({"s3_dendrogram", "s3:dendrogram", "s3dendrogram", "intra_dendrogram", "intra:dendrogram",
                           "intradendrogram", "s3_dend", "intra_dend"},
                          [](Config& c) { c.intraCommunityOrder = IntraOrder::Dendrogram; }));
        v.push_back(alias({"s3_gorder", "s3:gorder", "s3gorder", "intra_gorder", "intra:gorder", "intragorder",
                           "s3_gord", "intra_gord"},
                          [](Config& c) { c.intraCommunityOrder = IntraOrder::Gorder; }));
        v.push_back(alias({"s3_gorder_faithful", "s3:gorder_faithful", "intra_gorder_faithful",
                           "intra:gorder_faithful", "intra_gorder2"},
                          [](Config& c) { c.intraCommunityOrder = IntraOrder::GorderFaithful; }));
        v.push_back(alias({"s3_hubsort", "s3:hubsort", "s3hubsort", "intra_hubsort", "intra:hubsort", "intrahubsort",
                           "intra_hub", "intra:hub"},
                          [](Config& c) { c.intraCommunityOrder = IntraOrder::HubSort; }));
        v.push_back(alias({"s3_deg_asc", "s3:deg_asc", "s3degasc", "intra_deg_asc", "intra:deg_asc", "intra_degasc",
                           "intra_degree_asc", "deg_asc", "degasc"},
                          [](Config& c) { c.intraCommunityOrder = IntraOrder::DegreeAsc; }));
        v.push_back(alias({"s3_hub2", "s3:hub2", "s3hub2", "intra_hub2", "intra:hub2", "intrahub2", "hub2"},
                          [](Config& c) { c.intraCommunityOrder = IntraOrder::Hub2; }));
        v.push_back(alias({"s3_alternate", "s3:alternate", "s3alt", "intra_alternate", "intra:alternate", "intra_alt",
                           "alternate", "alt"},
                          [](Config& c) { c.intraCommunityOrder = IntraOrder::Alternate; }));
        v.push_back(alias({"s3_random", "s3:random", "s3rand", "intra_random", "intra:random", "intra_rand", "random",
                           "rand"},
                          [](Config& c) { c.intraCommunityOrder = IntraOrder::Random; }));
        v.push_back(alias({"s3_boundary_last", "s3:boundary_last", "s3bndlast", "intra_boundary_last",
                           "intra:boundary_last", "intra_bndlast", "boundary_last", "bndlast", "boundarylast"},
                          [](Config& c) { c.intraCommunityOrder = IntraOrder::BoundaryLast; }));
        v.push_back(alias({"s3_core", "s3:core", "s3core", "intra_core", "intra:core", "intracore", "core_order",
                           "coreorder", "core"},
                          [](Config& c) { c.intraCommunityOrder = IntraOrder::CoreOrder; }));
        // Super-graph order.
        v.push_back(alias({"s1_none", "s1:none", "s1none", "sg_none", "sg:none", "sgnone"},
                          [](Config& c) { c.superGraphOrder = SuperGraphOrder::None; }));
        v.push_back(alias({"s1_super_rabbit", "s1:super_rabbit", "s1srabbit", "sg_super_rabbit", "sg:super_rabbit",
                           "sgsrabbit"},
                          [](Config& c) { c.superGraphOrder = SuperGraphOrder::SuperRabbit; }));
        v.push_back(alias({"s1_super_rcm", "s1:super_rcm", "s1srcm", "sg_super_rcm", "sg:super_rcm", "sgsrcm"},
                          [](Config& c) { c.superGraphOrder = SuperGraphOrder::SuperRCM; }));
        v.push_back(alias({"s1_tile_rabbit", "s1:tile_rabbit", "s1tilerabbit", "sg_tile_rabbit", "sg:tile_rabbit",
                           "sgtilerabbit"},
                          [](Config& c) { c.superGraphOrder = SuperGraphOrder::TileRabbit; }));
        v.push_back(alias({"s1_hilbert", "s1:hilbert", "s1hilbert", "sg_hilbert", "sg:hilbert", "sghilbert",
                           "hilbert"},
                          [](Config& c) { c.superGraphOrder = SuperGraphOrder::Hilbert; }));
        v.push_back(alias({"s2_identity", "s2:identity", "s2identity", "comm_identity", "comm:identity",
                           "commidentity"},
                          [](Config& c) { c.communityOrder = CommunityOrder::Identity; }));
        v.push_back(alias({"refine_2swap", "refine:2swap", "refine2swap", "r2swap", "twoswap", "2swap"},
                          [](Config& c) { c.refinementPass = RefinementPass::TwoSwap; }));
        v.push_back(alias({"refine_none", "refine:none", "refinenone"},
                          [](Config& c) { c.refinementPass = RefinementPass::None; }));
        // LAYER mode (per-community external dispatch).
        v.push_back(alias({"graphbrew", "gb"}, [](Config& c) {
            c.ordering = Ordering::Layer;
            c.hasExplicitOrdering = true;
            c.useSmallCommunityMerging = true;
            if (c.finalAlgoId < 0) c.finalAlgoId = 8;
        }));
        v.push_back([](const std::string& t, Config& c) {
            if (!(t.size() > 5 && t.compare(0, 5, "final") == 0)) return Outcome::NoMatch;
            std::string num = t.substr(5);
            if (!num.empty() && num[0] == ':') num = num.substr(1);
            int id = -1;
            if (!exact_int(num, id) || id < 0 || id > 11) return Outcome::Rejected;
            c.finalAlgoId = id;
            c.ordering = Ordering::Layer;
            c.useSmallCommunityMerging = true;
            return Outcome::Applied;
        });
        v.push_back(alias({"flat", "norecurse"}, [](Config& c) {
            c.recursiveDepth = 0;
            enter_layer(c);
        }));
        v.push_back(alias({"recursive", "recurse"}, [](Config& c) {
            c.recursiveDepth = std::max(c.recursiveDepth, 1);
            enter_layer(c);
        }));
        v.push_back([](const std::string& t, Config& c) {
            if (!(t.size() > 5 && t.compare(0, 5, "depth") == 0)) return Outcome::NoMatch;
            std::string num = t.substr(5);
            if (!num.empty() && num[0] == ':') num = num.substr(1);
            int depth = -1;
            if (!exact_int(num, depth) || depth < 0 || depth > 10) return Outcome::Rejected;
            c.recursiveDepth = depth;
            enter_layer(c);
            return Outcome::Applied;
        });
        v.push_back(alias({"subauto", "sub:auto"}, [](Config& c) { c.subAlgoId = -1; }));
        v.push_back([](const std::string& t, Config& c) {
            if (!(t.size() > 3 && t.compare(0, 3, "sub") == 0)) return Outcome::NoMatch;
            std::string num = t.substr(3);
            if (!num.empty() && num[0] == ':') num = num.substr(1);
            if (num == "auto") {
                c.subAlgoId = -1;
                return Outcome::Applied;
            }
            int id = -1;
            if (!exact_int(num, id) || id < 0 || id > 11) return Outcome::Rejected;
            c.subAlgoId = id;
            return Outcome::Applied;
        });
        // Aggregation strategy.
        v.push_back(alias({"leiden"}, [](Config& c) { c.aggregation = Aggregation::LeidenCSR; }));
        v.push_back(alias({"streaming", "lazy"}, [](Config& c) { c.aggregation = Aggregation::RabbitLazy; }));
        v.push_back(alias({"hybrid"}, [](Config& c) { c.aggregation = Aggregation::Hybrid; }));
        v.push_back(alias({"merge", "coarsen"}, [](Config& c) { c.useCommunityMerging = true; }));
        v.push_back(alias({"hubx", "hub-extract", "hubextract"}, [](Config& c) { c.useHubExtraction = true; }));
        v.push_back([](const std::string& t, Config& c) {
            if (!(t.size() > 4 && t.compare(0, 4, "hubx") == 0)) return Outcome::NoMatch;
            c.useHubExtraction = true;
            double pct = 0.0;
            if (!exact_double(t.substr(4), pct) || pct <= 0 || pct >= 100) return Outcome::Rejected;
            c.hubExtractionPct = pct / 100.0;
            return Outcome::Applied;
        });
        v.push_back(alias({"gord", "gorder"}, [](Config& c) { c.useGorderIntra = true; }));
        v.push_back([](const std::string& t, Config& c) {
            if (!(t.size() > 4 && t.compare(0, 4, "gord") == 0 && std::isdigit((unsigned char)t[4])))
                return Outcome::NoMatch;
            c.useGorderIntra = true;
            int w = 0;
            if (!exact_int(t.substr(4), w) || w <= 0 || w > 100) return Outcome::Rejected;
            c.gorderWindow = w;
            return Outcome::Applied;
        });
        v.push_back([](const std::string& t, Config& c) {
            if (!(t.size() > 5 && t.compare(0, 5, "gordf") == 0)) return Outcome::NoMatch;
            c.useGorderIntra = true;
            int f = 0;
            if (!exact_int(t.substr(5), f) || f <= 0) return Outcome::Rejected;
            c.gorderFallback = f;
            return Outcome::Applied;
        });
        v.push_back([](const std::string& t, Config& c) {
            if (!(t.size() > 2 && t.compare(0, 2, "gw") == 0 && std::isdigit((unsigned char)t[2])))
                return Outcome::NoMatch;
            int w = 0;
            if (!exact_int(t.substr(2), w) || w <= 0 || w > 100) return Outcome::Rejected;
            c.gorderWindow = w;
            return Outcome::Applied;
        });
        v.push_back([](const std::string& t, Config& c) {
            if (!((t.size() > 5 && t.compare(0, 5, "sgres") == 0) || (t.size() > 5 && t.compare(0, 5, "gamma") == 0)))
                return Outcome::NoMatch;
            double r = 0.0;
            if (!exact_double(t.substr(5), r) || r <= 0.0 || r > 10.0) return Outcome::Rejected;
            c.superGraphResolution = r;
            return Outcome::Applied;
        });
        v.push_back(alias({"hsort", "hubsort"}, [](Config& c) { c.useHubSort = true; }));
        v.push_back(alias({"rcm"}, [](Config& c) {
            c.useRCMSuper = true;
            c.useRCMIntra = true;
        }));
        v.push_back(alias({"rcm_super", "rcmsuper"}, [](Config& c) { c.useRCMSuper = true; }));
        v.push_back(alias({"rcm_intra", "rcmintra"}, [](Config& c) { c.useRCMIntra = true; }));
        v.push_back(alias({"bfs_intra", "bfsintra", "no_rcm_intra"}, [](Config& c) { c.useRCMIntra = false; }));
        v.push_back(alias({"norefine"}, [](Config& c) { c.useRefinement = false; }));
        v.push_back(alias({"cd_full", "cd_leiden"}, [](Config& c) {
            c.communityMode = CommunityMode::FullLeiden;
            c.useRefinement = true;
            c.refinementDepth = -1;
        }));
        v.push_back(alias({"cd_louvain"}, [](Config& c) {
            c.communityMode = CommunityMode::FullLeiden;
            c.useRefinement = false;
        }));
        v.push_back(alias({"cd_lp_only", "cd_lp"}, [](Config& c) {
            c.communityMode = CommunityMode::FastLP;
            c.useRefinement = false;
        }));
        v.push_back(alias({"cd_hybrid"}, [](Config& c) {
            c.communityMode = CommunityMode::Hybrid;
            c.useRefinement = true;
            c.refinementDepth = 0;
        }));
        v.push_back(alias({"cd_gve"}, [](Config& c) {
            c.communityMode = CommunityMode::FullLeiden;
            c.useRefinement = true;
            c.refinementDepth = 0;
        }));
        v.push_back([](const std::string& t, Config& c) {
            if (!(t.size() > 6 && t.compare(0, 6, "refine") == 0 && std::isdigit((unsigned char)t[6])))
                return Outcome::NoMatch;
            int depth = -1;
            if (!exact_int(t.substr(6), depth) || depth < 0) return Outcome::Rejected;
            c.refinementDepth = depth;
            return Outcome::Applied;
        });
        v.push_back(alias({"totalm", "gvem"}, [](Config& c) { c.mComputation = MComputation::TotalEdges; }));
        v.push_back(alias({"halfm"}, [](Config& c) { c.mComputation = MComputation::HalfEdges; }));
        v.push_back(alias({"gvecsr", "gve-csr"}, [](Config& c) { c.aggregation = Aggregation::GveCSR; }));
        v.push_back(alias({"quality"}, [](Config& c) {
            c.aggregation = Aggregation::GveCSR;
            c.mComputation = MComputation::TotalEdges;
            c.refinementDepth = 0;
            c.ordering = Ordering::Hierarchical;
        }));
        v.push_back(alias({"lazyupdate", "lazyupdates"}, [](Config& c) { c.useLazyUpdates = true; }));
        v.push_back(alias({"verify"}, [](Config& c) { c.verifyTopology = true; }));
        v.push_back(alias({"auto", "0"}, [](Config& c) { c.resolution = kDefaultResolution; }));
        v.push_back(alias({"dynamic"}, [](Config& c) {
            c.resolution = kDefaultResolution;
            c.useDynamicResolution = true;
        }));
        v.push_back([](const std::string& t, Config& c) {
            if (!starts_with(t, "dynamic_")) return Outcome::NoMatch;
            double init = 0.0;
            if (!exact_double(t.substr(8), init) || init <= 0.0 || init > 3.0) return Outcome::Rejected;
            c.resolution = init;
            c.useDynamicResolution = true;
            return Outcome::Applied;
        });
        // Numeric fallback: resolution, then iterations, then passes.
        v.push_back([](const std::string& t, Config& c) {
            try {
                size_t parsed = 0;
                const double val = std::stod(t, &parsed);
                if (parsed != t.size() || !std::isfinite(val)) return Outcome::Rejected;
                if (val > 0 && val <= 3 && (t.find('.') != std::string::npos || val < 1)) {
                    c.resolution = val;
                } else if (val >= 1 && val <= 100) {
                    const int iv = static_cast<int>(val);
                    if (c.maxIterations == kDefaultMaxIterations) c.maxIterations = iv;
                    else c.maxPasses = iv;
                } else if (val > 0 && val <= 3) {
                    c.resolution = val;
                } else {
                    return Outcome::Rejected;
                }
                return Outcome::Applied;
            } catch (...) {
                return Outcome::Rejected;
            }
        });
        return v;
    }();
    return r;
}

void parse_error(const std::string& msg) { throw Error(GBGPU_E_PARSE, msg); }

const char* algorithm_name(Algorithm a) { return a == Algorithm::Rabbit ? "rabbit" : "leiden"; }

const char* aggregation_name(Aggregation a) {
    switch (a) {
        case Aggregation::LeidenCSR: return "leiden-csr";
        case Aggregation::RabbitLazy: return "streaming";
        case Aggregation::Hybrid: return "hybrid";
        case Aggregation::GveCSR: return "gve-csr";
    }
    return "unknown";
}

const char* ordering_name(Ordering o) {
    static const char* names[] = {"hierarchical", "connectivity-bfs", "dendrogram-dfs", "dendrogram-bfs",
                                  "community-sort", "hubcluster", "dbg", "corder", "dbg-global", "corder-global",
                                  "hcache", "hrab", "hlr", "tqr", "compose", "layer"};
    const int i = static_cast<int>(o);
    return (i >= 0 && i < 16) ? names[i] : "unknown";
}

const char* community_mode_name(CommunityMode m) {
    switch (m) {
        case CommunityMode::FullLeiden: return "full-leiden";
        case CommunityMode::FastLP: return "fast-lp";
        case CommunityMode::Hybrid: return "hybrid";
    }
    return "unknown";
}

const char* super_graph_name(SuperGraphOrder s) {
    static const char* names[] = {"none", "super-rabbit", "super-rcm", "tile-rabbit", "hilbert"};
    const int i = static_cast<int>(s);
    return (i >= 0 && i < 5) ? names[i] : "unknown";
}

const char* community_order_name(CommunityOrder c) {
    static const char* names[] = {"size-desc", "size-asc", "degree-desc", "degree-asc",
                                  "capacity-runs", "cut-min", "identity"};
    const int i = static_cast<int>(c);
    return (i >= 0 && i < 7) ? names[i] : "unknown";
}

const char* intra_name(IntraOrder o) {
    static const char* names[] = {"bfs", "rcm", "rcmpp", "dendrogram", "gorder", "gorder-faithful", "hubsort",
                                  "degree-asc", "hub2", "alternate", "random", "boundary-last", "core"};
    const int i = static_cast<int>(o);
    return (i >= 0 && i < 13) ? names[i] : "unknown";
}

std::string fmt_double(double v) {
    // std::ostream with setprecision(17) and the default float field formats
    // like printf("%.17g").
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.17g", v);
    return buf;
}

const char* tf(bool b) { return b ? "true" : "false"; }

}  // namespace

std::vector<std::string> split_tokens(const std::string& opts) {
    std::vector<std::string> out;
    size_t start = 0;
    while (true) {
        const size_t colon = opts.find(':', start);
        out.push_back(opts.substr(start, colon == std::string::npos ? std::string::npos : colon - start));
        if (colon == std::string::npos) break;
        start = colon + 1;
    }
    if (out.size() == 1 && out[0].empty()) out.clear();
    return out;
}

Config parse_tokens(const std::vector<std::string>& options, bool strict) {
    Config c;
    for (const std::string& t : options) {
        if (t.empty()) continue;
        for (const Rule& rule : rules()) {
            const Outcome o = rule(t, c);
            if (o == Outcome::NoMatch) continue;
            if (o == Outcome::Rejected && strict) parse_error("Unknown or invalid GraphBrew option: " + t);
            break;
        }
    }
    if (strict && c.ordering == Ordering::Compose) {
        bool sg = false, comm = false;
        for (const std::string& t : options) {
            sg = sg || starts_with(t, "sg_") || starts_with(t, "sg:") || starts_with(t, "s1_") ||
                 starts_with(t, "s1:");
            comm = comm || starts_with(t, "comm_") || starts_with(t, "comm:") || starts_with(t, "s2_") ||
                   starts_with(t, "s2:") || t == "capacity_runs" || t == "cache_fit";
        }
        if (sg && !comm) parse_error("COMPOSE super-graph order requires an explicit community-order token");
    }
    const bool geometry = c.capacityL2Bytes > 0 || c.capacityLLCBytes > 0 || c.capacityPropertyBytesPerVertex > 0;
    if (strict && c.communityOrder == CommunityOrder::CapacityRuns) {
        if (c.ordering != Ordering::Compose) parse_error("Capacity-run community ordering requires COMPOSE");
        if (c.superGraphOrder != SuperGraphOrder::None)
            parse_error("Capacity-run community ordering requires sg_none");
        if (c.capacityL2Bytes == 0 || c.capacityLLCBytes == 0 || c.capacityPropertyBytesPerVertex == 0)
            parse_error("Capacity-run community ordering requires pinned capl2k, capllck, and capv tokens");
    } else if (strict && geometry) {
        parse_error("Capacity geometry tokens require capacity-run community ordering");
    }
    if (strict && c.intraCommunityOrder == IntraOrder::GorderFaithful && c.ordering != Ordering::Compose)
        parse_error("Faithful local Gorder requires COMPOSE");
    if (c.capacityL2Bytes > 0 && c.capacityLLCBytes > 0 && c.capacityLLCBytes < c.capacityL2Bytes)
        parse_error("Capacity-run LLC bytes must be at least L2 bytes");
    return c;
}

Config parse_cli(const std::vector<std::string>& options, double auto_resolution) {
    static const std::vector<std::string> kLeiden = {"gvecsr", "totalm", "refine0", "graphbrew"};
    if (options.empty() || options[0].empty()) {
        Config c = parse_tokens(kLeiden, true);
        c.resolution = auto_resolution;
        return c;
    }
    static const std::map<std::string, std::vector<std::string>> presets = {
        {"leiden", kLeiden},
        {"rabbit", {"rabbitorder", "0.5"}},
        {"hubcluster", {"hubcluster"}},
    };
    auto is_numeric = [](const std::string& t) {
        double v;
        try {
            size_t parsed = 0;
            v = std::stod(t, &parsed);
            return parsed == t.size() && std::isfinite(v);
        } catch (...) {
            return false;
        }
    };
    auto is_integer = [](const std::string& t) {
        try {
            size_t parsed = 0;
            (void)std::stoi(t, &parsed);
            return parsed == t.size();
        } catch (...) {
            return false;
        }
    };
    auto dynamic_initial = [&](const std::string& t, double& init) {
        if (t == "dynamic") {
            init = auto_resolution;
            return true;
        }
        if (!starts_with(t, "dynamic_") || !is_numeric(t.substr(8))) return false;
        init = std::stod(t.substr(8));
        return init > 0.0 && init <= 3.0;
    };
    auto finish = [&](Config& c) {
        if (c.algorithm != Algorithm::Rabbit && c.ordering == Ordering::ConnectivityBFS) c.ordering = Ordering::Layer;
        if (c.ordering == Ordering::Layer) {
            c.useSmallCommunityMerging = true;
            if (c.finalAlgoId < 0) c.finalAlgoId = 8;
        }
        if (c.resolution == kDefaultResolution) c.resolution = auto_resolution;
    };

    const auto preset = presets.find(options[0]);
    if (preset == presets.end()) {
        Config c = parse_tokens(options, true);
        finish(c);
        return c;
    }
    std::vector<std::string> tokens = preset->second;
    for (size_t i = 1; i < options.size(); ++i) {
        const std::string& t = options[i];
        if (t.empty()) continue;
        bool positional = false;
        const bool numeric = is_numeric(t);
        double init = 0.0;
        if ((i == 1 || i == 3 || i == 4 || i == 5) && numeric && !is_integer(t))
            parse_error("GraphBrew positional integer is malformed: " + t);
        if (i == 1 && is_integer(t)) positional = true;
        if (i == 2 && (numeric || t == "auto" || dynamic_initial(t, init))) positional = true;
        if ((i == 3 || i == 4) && is_integer(t)) positional = true;
        if (i == 5 && (is_integer(t) || t == "auto" || t == "adaptive")) positional = true;
        if (!positional) tokens.push_back(t);
    }
    Config c = parse_tokens(tokens, true);
    finish(c);
    if (options.size() > 1 && is_integer(options[1])) {
        const int fa = std::stoi(options[1]);
        if (fa < 0 || fa > 11) parse_error("Invalid GraphBrew final algorithm: " + options[1]);
        c.finalAlgoId = fa;
    }
    if (options.size() > 2 && !options[2].empty()) {
        const std::string& r = options[2];
        if (r != "auto" && r != "0") {
            double init = 0.0;
            if (dynamic_initial(r, init)) {
                c.resolution = init;
                c.useDynamicResolution = true;
            } else if (is_numeric(r)) {
                const double v = std::stod(r);
                if (v <= 0.0 || v > 3.0) parse_error("Invalid GraphBrew resolution: " + r);
                c.resolution = v;
            }
        }
    }
    if (options.size() > 3 && is_integer(options[3])) {
        const int passes = std::stoi(options[3]);
        if (passes <= 0 || passes > 50) parse_error("Invalid GraphBrew pass count: " + options[3]);
        c.maxPasses = passes;
    }
    if (options.size() > 4 && !options[4].empty()) {
        const std::string& d = options[4];
        if (d == "recursive" || d == "recurse") {
            c.recursiveDepth = std::max(c.recursiveDepth, 1);
        } else if (is_integer(d)) {
            const int v = std::stoi(d);
            if (v < 0 || v > 10) parse_error("Invalid GraphBrew recursion depth: " + d);
            c.recursiveDepth = v;
        }
    }
    if (options.size() > 5 && !options[5].empty()) {
        const std::string& sa = options[5];
        if (sa == "auto" || sa == "adaptive") {
            c.subAlgoId = -1;
        } else if (is_integer(sa)) {
            const int v = std::stoi(sa);
            if (v < 0 || v > 11) parse_error("Invalid GraphBrew sub-algorithm: " + sa);
            c.subAlgoId = v;
        }
    }
    return c;
}

std::string effective_config_json(const Config& c) {
    const char* ordering = (c.algorithm == Algorithm::Rabbit && !c.hasExplicitOrdering) ? "rabbit-native-dfs"
                                                                                         : ordering_name(c.ordering);
    std::string s = "{\"schema\":\"graphbrew_config/v3\"";
    auto str = [&](const char* k, const char* v) { s += std::string(",\"") + k + "\":\"" + v + "\""; };
    auto raw = [&](const char* k, const std::string& v) { s += std::string(",\"") + k + "\":" + v; };
    str("algorithm", algorithm_name(c.algorithm));
    str("community_mode", community_mode_name(c.communityMode));
    str("aggregation", aggregation_name(c.aggregation));
    str("ordering", ordering);
    str("super_graph", super_graph_name(c.superGraphOrder));
    str("community_order", community_order_name(c.communityOrder));
    str("intra_community_order", intra_name(c.intraCommunityOrder));
    str("refinement_pass", c.refinementPass == RefinementPass::TwoSwap ? "two-swap" : "none");
    raw("resolution", c.algorithm == Algorithm::Rabbit ? std::string("null") : fmt_double(c.resolution));
    raw("super_graph_resolution", fmt_double(c.superGraphResolution));
    raw("max_iterations", std::to_string(c.maxIterations));
    raw("max_passes", std::to_string(c.maxPasses));
    raw("refinement_depth", std::to_string(c.refinementDepth));
    str("m_computation", c.mComputation == MComputation::TotalEdges ? "total-edges" : "half-edges");
    raw("deterministic_community_detection", tf(c.deterministicCommunityDetection));
    raw("supergraph_move_batch", std::to_string(c.superGraphMoveBatch));
    raw("gorder_window", std::to_string(c.gorderWindow));
    raw("gorder_fallback", std::to_string(c.gorderFallback));
    raw("capacity_l2_bytes", std::to_string(c.capacityL2Bytes));
    raw("capacity_llc_bytes", std::to_string(c.capacityLLCBytes));
    raw("capacity_property_bytes_per_vertex", std::to_string(c.capacityPropertyBytesPerVertex));
    raw("final_algo_id", std::to_string(c.finalAlgoId));
    raw("recursive_depth", std::to_string(c.recursiveDepth));
    raw("sub_algo_id", std::to_string(c.subAlgoId));
    raw("rabbit_degree_sort_preprocess", tf(c.rabbitDegreeSortPreprocess));
    raw("use_refinement", tf(c.useRefinement));
    raw("use_lazy_updates", tf(c.useLazyUpdates));
    raw("verify_topology", tf(c.verifyTopology));
    raw("dynamic_resolution", tf(c.useDynamicResolution));
    raw("degree_sorting", tf(c.useDegreeSorting));
    raw("community_merging", tf(c.useCommunityMerging));
    raw("hub_extraction", tf(c.useHubExtraction));
    raw("hub_extraction_pct", fmt_double(c.hubExtractionPct));
    raw("gorder_intra", tf(c.useGorderIntra));
    raw("hub_sort", tf(c.useHubSort));
    raw("rcm_super", tf(c.useRCMSuper));
    raw("rcm_intra", tf(c.useRCMIntra));
    raw("small_community_merging", tf(c.useSmallCommunityMerging));
    raw("has_explicit_ordering", tf(c.hasExplicitOrdering));
    s += "}";
    return s;
}

std::string gpu_unsupported_reason(const Config& c) {
    if (c.algorithm != Algorithm::Leiden) return "community detection 'rabbit' is not on the GPU path";
    if (c.aggregation != Aggregation::GveCSR) return "only gvecsr aggregation is on the GPU path";
    if (c.ordering != Ordering::Compose) return std::string("ordering '") + ordering_name(c.ordering) +
                                                "' is not on the GPU path (use compose)";
    if (c.superGraphOrder == SuperGraphOrder::TileRabbit)
        return "super-graph order sg_tile_rabbit is not on the GPU path";
    switch (c.communityOrder) {
        case CommunityOrder::SizeDesc: case CommunityOrder::SizeAsc: case CommunityOrder::DegreeDesc:
        case CommunityOrder::DegreeAsc: case CommunityOrder::Identity: break;
        default: return std::string("community order '") + community_order_name(c.communityOrder) +
                        "' is not on the GPU path";
    }
    switch (c.intraCommunityOrder) {
        case IntraOrder::BFSFromHub: case IntraOrder::Gorder: case IntraOrder::Dendrogram: case IntraOrder::RCM:
        case IntraOrder::RCMpp: case IntraOrder::HubSort: case IntraOrder::DegreeAsc: case IntraOrder::Hub2: case IntraOrder::Alternate:
        case IntraOrder::Random: case IntraOrder::BoundaryLast: case IntraOrder::CoreOrder: break;
        default: return std::string("intra-community order '") + intra_name(c.intraCommunityOrder) +
                        "' is not on the GPU path";
    }
    if (c.refinementPass != RefinementPass::None) return "refinement pass 2swap is not on the GPU path";
    if (c.useDynamicResolution) return "dynamic resolution is not on the GPU path";
    if (c.useCommunityMerging) return "community merging is not on the GPU path";
    if (c.useLazyUpdates) return "lazy updates are not on the GPU path";
    return "";
}

}  // namespace gb
