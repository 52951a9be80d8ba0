/*
 * gbgpu.h -- C ABI of the GB300 implementation of GraphBrew's algorithm-12
 * mapping path ("-o 12:leiden:compose:...").
 *
 * Every entry point takes plain pointers and sizes and returns a gbgpu_status.
 * Graph inputs are undirected CSR graphs as the GAPBS builder produces them
 * (int64 row offsets, int32 neighbour ids, each undirected edge stored in both
 * rows, rows sorted ascending, no duplicates, no self-loops).  Pointers are
 * host pointers unless GBGPU_DEVICE_POINTERS is set in `flags`, in which case
 * every array argument of that call is a device pointer on the context's
 * device and the call does no host<->device copies.
 *
 * A context owns one CUDA stream and a stream-ordered memory pool.  Calls on
 * one context are not thread-safe; use one context per host thread.
 *
 * Reference interfaces replaced (paths relative to the GraphBrew project root):
 *   gbgpu_generate_mapping  -> graphbrew::generateGraphBrewMapping<uint32_t>
 *                              (bench/include/graphbrew/reorder/reorder_graphbrew.h:7836-8013),
 *                              reached from BuilderBase::GenerateGraphBrewMappingUnified
 *                              (bench/include/external/gapbs/builder.h:3669-3783)
 *   gbgpu_leiden            -> graphbrew::runGraphBrew (reorder_graphbrew.h:7238-7571)
 *   gbgpu_compose           -> graphbrew::orderCompose (reorder_graphbrew.h:6286-7087)
 *   gbgpu_relabel_csr       -> BuilderBase::RelabelByMapping (builder.h:1046-1206)
 *   gbgpu_validate_permutation -> BuilderBase::ValidatePermutationOrThrow (builder.h:2042-2081)
 *   gbgpu_parse_config      -> graphbrew::parseGraphBrewCliConfig + graphBrewEffectiveConfigJson
 *                              (reorder_graphbrew_parser.h:714-912, reorder_graphbrew.h:693-775)
 *   gbgpu_auto_resolution   -> computeAutoResolution (reorder_types.h:2743-2780)
 *   gbgpu_fingerprint       -> BuilderBase::MappingFingerprint (builder.h:1398-1411)
 */
#ifndef GBGPU_H_
#define GBGPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GBGPU_OK = 0,
    GBGPU_E_INVALID = 1,        /* malformed argument or graph (std::invalid_argument) */
    GBGPU_E_UNSUPPORTED = 2,    /* option valid in the grammar but not on this path */
    GBGPU_E_CUDA = 3,           /* CUDA runtime error */
    GBGPU_E_NOMEM = 4,          /* device or host allocation failed */
    GBGPU_E_NOT_PERMUTATION = 5,/* validation failed (std::runtime_error) */
    GBGPU_E_PARSE = 6,          /* option grammar rejected a token (std::invalid_argument) */
    GBGPU_E_OVERFLOW = 7,       /* size beyond a documented limit (std::overflow_error) */
    GBGPU_E_TIMEOUT = 8         /* a bounded device wait gave up */
} gbgpu_status;

/* flags */
#define GBGPU_DEVICE_POINTERS 0x1u   /* all array arguments are device pointers */
#define GBGPU_QUIET 0x2u             /* no stdout progress lines */

typedef struct gbgpu_ctx gbgpu_ctx;

/* Algorithm-12 configuration after option parsing (the fields of
 * GraphBrewConfig that the mapping path reads, reorder_graphbrew.h:398-603). */
typedef struct {
    double resolution;
    double tolerance;
    double aggregation_tolerance;
    double tolerance_drop;
    int32_t max_iterations;
    int32_t max_passes;
    int32_t total_edges_m;          /* totalm */
    int32_t gve_aggregation;        /* gvecsr */
    int32_t use_refinement;
    int32_t refinement_depth;
    int32_t deterministic;          /* cd_serial (1) / cd_parallel (0) */
    int32_t super_move_batch;       /* sgmb<k> */
    int32_t ordering;               /* OrderingStrategy ordinal */
    int32_t super_graph_order;      /* SuperGraphOrder ordinal */
    int32_t community_order;        /* CommunityOrder ordinal */
    int32_t intra_order;            /* IntraCommunityOrder ordinal */
    int32_t refinement_pass;        /* RefinementPass ordinal */
    int32_t gorder_window;
    int32_t gorder_fallback;
    int32_t algorithm;              /* 0 Leiden, 1 Rabbit */
} gbgpu_config;

/* Per-call statistics; times are device (CUDA event) milliseconds. */
typedef struct {
    double total_ms;
    double leiden_ms;
    double local_move_ms;
    double aggregate_ms;
    double compose_ms;
    double intra_ms;
    double validate_ms;
    double relabel_ms;
    double h2d_ms;
    double d2h_ms;
    int32_t passes;
    int32_t iterations;
    int32_t super_move_iterations;
    int32_t super_move_ctas;      // CTAs of the super-move thread-block cluster (0: batched launches)
    int64_t super_moves;
    int64_t pass0_communities;
    int64_t aggregated_communities;
    int64_t communities;            /* distinct ids in the final membership */
    int64_t num_communities;        /* max id + 1 (orderCompose's numComm) */
    int64_t isolated;
    int64_t gorder_communities;
    int64_t gorder_vertices;
    int64_t gorder_max_community;
    int64_t fallback_communities;
    int64_t fallback_vertices;
    int64_t largest_community;
    int64_t bfs_levels;
    int64_t kernel_launches;        /* kernels this call launched */
    double resolution;              /* resolution used */
    int64_t local_move_rounds;      /* speculative rounds of the serial-order engine */
    int64_t local_move_evaluations; /* vertex evaluations in those rounds */
    int64_t local_move_streams;     /* > 0: cd_parallel ran the stream-mode engine with this many streams */
} gbgpu_stats;

/* Context lifetime.  device < 0 selects the current device. */
int gbgpu_ctx_create(gbgpu_ctx** out, int device);
void gbgpu_ctx_destroy(gbgpu_ctx* ctx);
/* Message of the last failing call on this context ("" if none). */
const char* gbgpu_last_error(const gbgpu_ctx* ctx);
/* Use a caller-owned cudaStream_t (NULL restores the context's own stream). */
int gbgpu_set_stream(gbgpu_ctx* ctx, void* cuda_stream);
/* Block until the context's stream is idle. */
int gbgpu_synchronize(gbgpu_ctx* ctx);

/* Parse the tokens after "12:" ("leiden:compose:...:2:2").  On success the
 * effective-config JSON (graphbrew_config/v3, byte-identical to the
 * reference's) is written to json_out when json_cap > 0.  On failure the
 * reference's exception text is written there instead. */
int gbgpu_parse_config(const char* opts, double auto_resolution, gbgpu_config* out,
                       char* json_out, size_t json_cap);

/* Automatic resolution from the degree distribution.  The variance is summed
 * on the device in a fixed order, so the result may differ from a serial sum
 * in the last bits. */
int gbgpu_auto_resolution(gbgpu_ctx* ctx, const int64_t* row_ptr, int64_t n, int64_t nnz,
                          uint32_t flags, double* out);

/* Full algorithm-12 mapping: Leiden, COMPOSE placement, intra-community order.
 * new_ids_out: n entries, forward map old id -> new id.  auto_resolution < 0
 * computes it with gbgpu_auto_resolution.  stats may be NULL. */
int gbgpu_generate_mapping(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col,
                           int64_t n, int64_t nnz, const char* opts, double auto_resolution,
                           int32_t* new_ids_out, gbgpu_stats* stats, uint32_t flags);

/* Community detection stage only (membership_out: n entries).  The final
 * membership is not renumbered after the last local-moving pass, exactly as
 * the reference returns it. */
int gbgpu_leiden(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n,
                 int64_t nnz, const char* opts, double resolution, uint32_t* membership_out,
                 gbgpu_stats* stats, uint32_t flags);

/* COMPOSE stage only, from a given membership (n entries). */
int gbgpu_compose(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n,
                  int64_t nnz, const uint32_t* membership, const char* opts,
                  int32_t* new_ids_out, gbgpu_stats* stats, uint32_t flags);

/* Check that new_ids is a permutation of 0..n-1.  *result: 0 valid,
 * 1 out-of-range id, 2 duplicate id (ValidatePermutationOrThrow's cases). */
int gbgpu_validate_permutation(gbgpu_ctx* ctx, const int32_t* new_ids, int64_t n,
                               uint32_t flags, int32_t* result);

/* Rebuild the CSR under new_ids: out_row_ptr n + 1 entries, out_col nnz
 * entries, every row sorted ascending.  org_ids_out (n entries, may be NULL)
 * receives the inverse map new -> old (the graph's org ids after
 * update_org_ids on a freshly built graph).  new_ids must be a permutation. */
int gbgpu_relabel_csr(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n,
                      int64_t nnz, const int32_t* new_ids, int64_t* out_row_ptr,
                      int32_t* out_col, int32_t* org_ids_out, uint32_t flags);

/* The builder's mapping lifecycle after GenerateMapping (builder.h:829-940):
 * mapping, device-side validation, relabel.  Equivalent to the three calls
 * above on one resident copy of the graph.  out_row_ptr / out_col may be NULL
 * to skip the relabel.  With host buffers, a page-locked out_col (cudaHostAlloc
 * / cudaHostRegister, e.g. torch pin_memory) is written by the relabel kernels
 * directly; pageable memory is filled by a copy afterwards. */
int gbgpu_map_and_relabel(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col,
                          int64_t n, int64_t nnz, const char* opts, double auto_resolution,
                          int32_t* new_ids_out, int64_t* out_row_ptr, int32_t* out_col,
                          gbgpu_stats* stats, uint32_t flags);

/* ---- Batched mode ----
 * No counterpart in the reference (it maps one graph per process).  Many
 * graphs are mapped with one recipe; graphs run concurrently on `streams`
 * worker streams of the context's device (each worker has its own context,
 * created on first use and kept until the parent is destroyed), so the
 * latency-bound stages of small graphs overlap.  Every graph's result equals
 * gbgpu_generate_mapping's on that graph.  Host pointers unless
 * GBGPU_DEVICE_POINTERS. */
typedef struct {
    const int64_t* row_ptr;
    const int32_t* col;
    int64_t n;
    int64_t nnz;
    int32_t* new_ids_out;           /* n entries */
} gbgpu_graph;

typedef struct {
    int32_t streams;                /* concurrent graphs (1..64); 0 = 4 */
    int32_t order;                  /* 0 = as given, 1 = largest graph first */
    int64_t exact_window;           /* serial-order engine window; 0 = library default */
} gbgpu_schedule;

/* stats (may be NULL): one entry per graph, in the given order; *wall_ms
 * (may be NULL): host wall time of the whole batch.  schedule may be NULL
 * (4 streams, largest first, default window).  Stops at the first failing
 * graph and returns its status. */
int gbgpu_generate_mappings_batched(gbgpu_ctx* ctx, const gbgpu_graph* graphs, int32_t count, const char* opts,
                                    const gbgpu_schedule* schedule, gbgpu_stats* stats, double* wall_ms,
                                    uint32_t flags);

/* Largest n accepted by gbgpu_validate_permutation_noalloc. */
#define GBGPU_NOALLOC_MAX_VERTICES (1 << 20)

/* Permutation check that allocates no device memory.  No counterpart in the
 * reference: it serves callers that cannot allocate device memory -- a process
 * whose GPU memory is reserved by another framework's allocator, or a
 * latency-critical loop that cannot take cudaMalloc's implicit
 * synchronisation.  Same *result codes as gbgpu_validate_permutation;
 * new_ids_dev must be device memory; n at most GBGPU_NOALLOC_MAX_VERTICES
 * (larger n returns GBGPU_E_OVERFLOW).  Scratch is a fixed 4 MiB array in the
 * library's device image, held by every GPU that loads the library until exit
 * and shared by all calls: calls whose GPU work overlaps race and must be
 * serialised by the caller.  The first call on each device looks up that
 * array's address (a one-time set-up step).  The call waits for its result on
 * the context's stream and leaves the caller's current device unchanged. */
int gbgpu_validate_permutation_noalloc(gbgpu_ctx* ctx, const int32_t* new_ids_dev, int64_t n,
                                       int32_t* result);

/* Arithmetic self-check, no counterpart in the reference.  The local-moving
 * kernels evaluate deltaModularity (reorder_graphbrew.h:1295-1298) with the
 * two quotients formed from precomputed double-double reciprocals and an
 * exact FMA remainder instead of full double divisions (and the first one,
 * (kuc - kud) / M, read from a table of RN(k / M) for |k| <= 1024).  This call runs both
 * forms on the device over `count` seeded inputs (a graph of total weight M,
 * 1 <= M < 4e15, resolution 0 < R < 1e6; plus bare quotients over a wide
 * exponent range) and writes into *mismatches how many results differ in any
 * bit; 0 is the expected answer. */
int gbgpu_selfcheck_delta(gbgpu_ctx* ctx, double M, double R, int64_t count, uint64_t seed, int64_t* mismatches);

/* FNV-1a-64 fingerprint of a forward map, on the host, as the builder prints
 * it ("Mapping Fingerprint"). */
uint64_t gbgpu_fingerprint(const int32_t* new_ids, int64_t n);

/* ---- Synthetic inputs of the builder lifecycle ----
 * gbgpu_gapbs_edge_list -> Generator::GenerateEL (bench/include/external/gapbs/
 *   generator.h:101-164): the edge list `converter -g <scale> -k <degree>`
 *   (uniform = 0, RMAT with permuted ids) or `-u <scale> -k <degree>`
 *   (uniform = 1) draws, seed kRandSeed (util.h:47), on the HOST with
 *   `threads` threads (0 = all).  src/dst are host arrays of
 *   gbgpu_gapbs_edge_count(scale, degree) entries.  The builder's squish
 *   (vertex count = largest id + 1, symmetrize, sort, de-duplicate, drop
 *   self-loops; builder.h:254-312) is left to the caller.  gbgpu_gapbs_edge_count
 *   returns -1 for a scale outside 0..30 or a negative degree. */
int64_t gbgpu_gapbs_edge_count(int32_t scale, int32_t degree);
int gbgpu_gapbs_edge_list(int32_t scale, int32_t degree, int32_t uniform, int32_t* src, int32_t* dst,
                          int32_t threads);

/* ---- Consumers timed after a mapping, and the selector's other arm ----
 * The reference's "map + kernel" end-to-end time is the mapping plus runs of
 * a benchmark kernel on the relabelled graph.  *ms_out (may be NULL) receives
 * the device time of the kernel itself.
 *   gbgpu_pagerank   -> PageRank pull form (bench/src/pr.cc:40-90): damping 0.85,
 *                       Jacobi sweeps until the L1 change < epsilon or max_iters;
 *                       scores agree with a float64 restatement to float tolerance
 *   gbgpu_bfs        -> BFS depths from `source` (bench/src/bfs.cc), -1 = unreached
 *   gbgpu_connected_components -> component = smallest vertex id in it (bench/src/cc.cc)
 *   gbgpu_dbg_mapping -> GenerateDBGMapping (bench/include/graphbrew/reorder/
 *                       reorder_hub.h:267-342), bit-exact */
int gbgpu_pagerank(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz,
                   int32_t max_iters, double epsilon, float* scores_out, int32_t* iters_out, double* ms_out,
                   uint32_t flags);
int gbgpu_bfs(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz,
              int64_t source, int32_t* depth_out, double* ms_out, uint32_t flags);
int gbgpu_connected_components(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n,
                               int64_t nnz, int32_t* comp_out, double* ms_out, uint32_t flags);
int gbgpu_dbg_mapping(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz,
                      int32_t* new_ids_out, double* ms_out, uint32_t flags);

/* ---- Selector ----
 * gbgpu_tier0_features -> ComputeTier0SampledGraphFeatures
 *   (bench/include/graphbrew/reorder/reorder_types.h:6066-6186).  features_out
 *   is always a HOST array of 9 doubles: num_nodes, num_edges, avg_degree,
 *   degree_cv, internal_density, hub_concentration, packing_factor,
 *   normalized_edge_span, window_neighbor_overlap.
 * The learned selector is a float32 MLP in_dim -> 64 -> 64 -> 3 (ReLU) whose
 * outputs are predicted log end-to-end times of the arms (algorithm 12, DBG,
 * original order).  Parameters are packed W1[in x 64], b1, W2[64 x 64], b2,
 * W3[64 x 3], b3 (row-major, input index first).  Loss is the mean squared
 * error over rows x 3 outputs; gbgpu_mlp_train runs Adam (0.9, 0.999, 1e-8) on
 * minibatches of a seeded shuffle and returns the last epoch's mean loss. */
int gbgpu_tier0_features(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz,
                         double* features_out, uint32_t flags);
int gbgpu_mlp_param_count(int32_t in_dim);
int gbgpu_mlp_forward(gbgpu_ctx* ctx, const float* params, const float* X, int32_t rows, int32_t in_dim,
                      float* Y, uint32_t flags);
int gbgpu_mlp_gradient(gbgpu_ctx* ctx, const float* params, const float* X, const float* T, int32_t rows,
                       int32_t in_dim, float* grad_out, float* loss_out, uint32_t flags);
int gbgpu_mlp_train(gbgpu_ctx* ctx, float* params_inout, const float* X, const float* T, int32_t rows,
                    int32_t in_dim, int32_t epochs, int32_t batch, float lr, uint64_t seed, float* loss_out,
                    uint32_t flags);

/* ---- Algorithm 14: deployable selector ("-o 14:_:_:_:<model>:<criterion>:<reuse>") ----
 * Replaces the full-graph AdaptiveOrder entry
 * (GenerateAdaptiveMappingFullGraphStandalone,
 * bench/include/graphbrew/reorder/reorder_adaptive.h:517-715) for the
 * deployable models:
 *   gbgpu_parse_selection_policy -> ParseDeployableSelectionPolicy
 *       (reorder_adaptive.h:166-228; model names from GetSelectionModel /
 *       GetSelectionCriterion, reorder_types.h:1927-2066), same exception texts
 *       in err (status GBGPU_E_PARSE); opts are the fields after "14:".
 *       Models: 0 perceptron (parses; selecting with it returns
 *       GBGPU_E_UNSUPPORTED: it needs the reference's weight database),
 *       7 budgeted-rule, 8 allkernel-lowreuse-rule (the frozen rule), and
 *       9 learned-mlp (aliases mlp, learned): this library's MLP, which like
 *       the rules needs an explicit reuse count.
 *   gbgpu_select_arm -> the selection itself: Tier-0 features on the GPU,
 *       ModeledPropertyBytes (reorder_types.h:1226-1258) of `kernel` against a
 *       cache (the device's L2 for the rules, the model's cache_bytes for
 *       learned-mlp), then SelectAllKernelLowReuseRule /
 *       SelectBudgetedOneUseRule (reorder_adaptive.h:240-385) or the MLP's
 *       smallest predicted end-to-end time.  The learned model falls back to
 *       the frozen rule (reason "frozen-rule-fallback") where the features lie
 *       more than a quarter of their training range outside it, or for a
 *       kernel it was not trained on.  The chosen arm is out->arm: 12 (the
 *       recipe in out->applied, run with gbgpu_generate_mapping), 5 (DBG,
 *       gbgpu_dbg_mapping) or 0 (original order).  kernel GBGPU_KERNEL_GENERIC
 *       fails like the reference ("Kernel-specific modeled property bytes are
 *       unavailable").
 *   gbgpu_selector_model_load reads a model file written by
 *       graphbrew_gb300.selector (LearnedSelector.save_binary): magic
 *       "GBSEL01\0", int32 in_dim, hidden (64), outputs (3), reserved, int64
 *       cache_bytes, float32 params[gbgpu_mlp_param_count(in_dim)], then
 *       float64 mean, std, lo, hi [in_dim] each. */
enum {
    GBGPU_KERNEL_GENERIC = 0,
    GBGPU_KERNEL_PR = 1,
    GBGPU_KERNEL_BFS = 2,
    GBGPU_KERNEL_CC = 3,
    GBGPU_KERNEL_SSSP = 4,
    GBGPU_KERNEL_BC = 5,
    GBGPU_KERNEL_TC = 6,
    GBGPU_KERNEL_PR_SPMV = 7,
    GBGPU_KERNEL_CC_SV = 8
};

typedef struct {
    int32_t model;          /* 0 perceptron, 7 budgeted-rule, 8 allkernel-lowreuse-rule, 9 learned-mlp */
    int32_t criterion;      /* 0 fastest-reorder, 1 fastest-execution, 2 best-endtoend, 3 best-amortization */
    double reuse;           /* reuse count (1.0 unless given) */
    int32_t reuse_explicit; /* the reuse field was given */
} gbgpu_selection_policy;

typedef struct {
    int32_t in_dim;         /* features per row (12) */
    const float* params;    /* gbgpu_mlp_param_count(in_dim) floats, packed as for gbgpu_mlp_forward */
    const double* mean;     /* standardisation and training range, in_dim each */
    const double* std;
    const double* lo;
    const double* hi;
    int64_t cache_bytes;    /* cache the model's working-set ratio feature is taken against */
} gbgpu_selector_model;

typedef struct {
    gbgpu_selection_policy policy;
    int32_t arm;                  /* 12, 5 or 0 */
    char applied[160];            /* "12:<recipe>", "5" or "0" */
    char reason[48];              /* allkernel-lowreuse-match / -fallback, budgeted-one-use-match /
                                     -fallback, learned-mlp, frozen-rule-fallback, empty-graph */
    double features[9];           /* Tier-0 features (as gbgpu_tier0_features) */
    int64_t property_bytes;       /* ModeledPropertyBytes of the kernel */
    int64_t cache_bytes;          /* cache the working-set ratio is taken against */
    double property_wsr;          /* property_bytes / cache_bytes */
    float predicted_log10_ms[3];  /* learned-mlp: predicted log10 ms of arms 12, 5, 0 */
} gbgpu_selection;

int gbgpu_parse_selection_policy(const char* opts, gbgpu_selection_policy* out, char* err, size_t err_len);
const char* gbgpu_selection_model_name(int32_t model);
const char* gbgpu_selection_criterion_name(int32_t criterion);
/* The rule step alone on features the caller already has (model 7 or 8;
 * features as gbgpu_tier0_features, property_wsr = property bytes / cache
 * bytes): fills out->arm, applied and reason. */
int gbgpu_apply_selection_rule(int32_t model, const double* features, double property_wsr, int32_t kernel,
                               double reuse, gbgpu_selection* out);
/* ModeledPropertyBytes; -1 for GBGPU_KERNEL_GENERIC (the reference throws). */
int64_t gbgpu_modeled_property_bytes(int32_t kernel, int64_t nodes, int64_t directed_edges);
int gbgpu_selector_model_load(const char* path, gbgpu_selector_model** out);
void gbgpu_selector_model_free(gbgpu_selector_model* model);
int gbgpu_select_arm(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz,
                     const char* opts, int32_t kernel, const gbgpu_selector_model* model, gbgpu_selection* out,
                     uint32_t flags);

/* Library version string. */
const char* gbgpu_version(void);

#ifdef __cplusplus
}
#endif

#endif /* GBGPU_H_ */
