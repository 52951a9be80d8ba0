// gb_config.h -- algorithm-12 option grammar (host, C++17).
//
// Mirrors GraphBrewConfig (bench/include/graphbrew/reorder/reorder_graphbrew.h:398-603)
// and the "-o 12:<tok>:<tok>..." grammar of parseGraphBrewConfig /
// parseGraphBrewCliConfig (reorder_graphbrew_parser.h:13-912): same tokens,
// presets, positional overrides, defaults and exception texts, so the
// effective-config JSON (graphbrew_config/v3, reorder_graphbrew.h:693-775) is
// byte-identical.
#pragma once

#include <cstddef>
#include <string>
#include <vector>

namespace gb {

// Defaults shared by the reorder family (reorder_types.h:213-226).
constexpr double kDefaultResolution = 1.0;
constexpr double kDefaultTolerance = 1e-2;
constexpr double kDefaultAggregationTolerance = 0.8;
constexpr double kDefaultToleranceDrop = 10.0;
constexpr int kDefaultMaxIterations = 10;
constexpr int kDefaultMaxPasses = 10;

enum class Algorithm { Leiden = 0, Rabbit = 1 };
enum class CommunityMode { FullLeiden = 0, FastLP = 1, Hybrid = 2 };
enum class Aggregation { LeidenCSR = 0, RabbitLazy = 1, Hybrid = 2, GveCSR = 3 };
enum class MComputation { HalfEdges = 0, TotalEdges = 1 };
enum class Ordering {
    Hierarchical = 0, ConnectivityBFS, DendrogramDFS, DendrogramBFS, CommunitySort, HubCluster, DBG, Corder,
    DBGGlobal, CorderGlobal, HierarchicalCacheAware, HybridLeidenRabbit, HierarchicalLeidenRabbit,
    TileQuantizedRabbit, Compose, Layer
};
enum class CommunityOrder { SizeDesc = 0, SizeAsc, DegreeDesc, DegreeAsc, CapacityRuns, CutMin, Identity };
enum class IntraOrder {
    BFSFromHub = 0, RCM, RCMpp, Dendrogram, Gorder, GorderFaithful, HubSort, DegreeAsc, Hub2, Alternate,
    Random, BoundaryLast, CoreOrder
};
enum class RefinementPass { None = 0, TwoSwap = 1 };
enum class SuperGraphOrder { None = 0, SuperRabbit, SuperRCM, TileRabbit, Hilbert };

struct Config {
    double resolution = kDefaultResolution;
    double tolerance = kDefaultTolerance;
    double aggregationTolerance = kDefaultAggregationTolerance;
    double toleranceDrop = kDefaultToleranceDrop;
    int maxIterations = kDefaultMaxIterations;
    int maxPasses = kDefaultMaxPasses;
    Algorithm algorithm = Algorithm::Leiden;
    CommunityMode communityMode = CommunityMode::FullLeiden;
    Aggregation aggregation = Aggregation::LeidenCSR;
    Ordering ordering = Ordering::ConnectivityBFS;
    bool useRefinement = true;
    int refinementDepth = -1;
    MComputation mComputation = MComputation::HalfEdges;
    bool deterministicCommunityDetection = true;
    int superGraphMoveBatch = 1;
    bool verifyTopology = false;
    bool useDynamicResolution = false;
    bool useDegreeSorting = false;
    bool useCommunityMerging = false;
    bool useHubExtraction = false;
    double hubExtractionPct = 0.001;
    bool useGorderIntra = false;
    int gorderWindow = 5;
    int gorderFallback = 0;
    bool useHubSort = false;
    bool useRCMSuper = false;
    bool useRCMIntra = false;
    SuperGraphOrder superGraphOrder = SuperGraphOrder::None;
    CommunityOrder communityOrder = CommunityOrder::SizeDesc;
    IntraOrder intraCommunityOrder = IntraOrder::BFSFromHub;
    RefinementPass refinementPass = RefinementPass::None;
    int refineMaxPasses = 3;
    size_t capacityL2Bytes = 0;
    size_t capacityLLCBytes = 0;
    size_t capacityPropertyBytesPerVertex = 0;
    double superGraphResolution = 0.10;
    int finalAlgoId = -1;
    bool useSmallCommunityMerging = false;
    int recursiveDepth = -1;
    int subAlgoId = 8;
    bool hasExplicitOrdering = false;
    bool rabbitDegreeSortPreprocess = false;
    bool useLazyUpdates = false;
};

// Token parser (parseGraphBrewConfig).  Throws gb::Error(GBGPU_E_PARSE, text).
Config parse_tokens(const std::vector<std::string>& options, bool strict);
// Public CLI grammar with presets and positional overrides (parseGraphBrewCliConfig).
Config parse_cli(const std::vector<std::string>& options, double auto_resolution);
// "a:b:c" -> {"a","b","c"} as the GAPBS command line splits -o (command_line.h:163-182).
std::vector<std::string> split_tokens(const std::string& opts);
// graphBrewEffectiveConfigJson (with schema).
std::string effective_config_json(const Config& c);
// Why the GPU path cannot run this configuration ("" when it can).
std::string gpu_unsupported_reason(const Config& c);

}  // namespace gb
