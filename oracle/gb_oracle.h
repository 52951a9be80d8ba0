/*
 * gb_oracle.h -- CPU oracle for the algorithm-12 mapping path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of GraphBrew's
 * algorithm-12 pipeline (GVE-style Leiden -> COMPOSE placement -> per-community
 * Gorder / BFS / RCM -> relabel).  It exists to check the CUDA implementation
 * and to serve as the timed CPU baseline.  Only tests, the smoke check and the
 * benchmark's CPU-baseline leg may load it; the product library never links it.
 *
 * Each function cites the reference code it follows (paths relative to the
 * GraphBrew project root).
 */
#ifndef GB_ORACLE_H_
#define GB_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ORC_OK = 0,
    ORC_EINVAL = -1,
    ORC_ENOMEM = -2,
    ORC_EUNSUPPORTED = -3
};

/* Undirected CSR: rows hold every neighbour once per direction. */
typedef struct {
    int64_t n;
    const int64_t *row_ptr; /* n + 1 entries */
    const int32_t *col;     /* row_ptr[n] entries */
} orc_graph;

/* computeAutoResolution (bench/include/graphbrew/reorder/reorder_types.h:2743-2780),
 * with the degree variance summed serially in vertex order. */
double orc_auto_resolution(const orc_graph *g);

typedef struct {
    double resolution;
    double tolerance;             /* DEFAULT_TOLERANCE 1e-2 */
    double aggregation_tolerance; /* DEFAULT_AGGREGATION_TOLERANCE 0.8 */
    double tolerance_drop;        /* DEFAULT_TOLERANCE_DROP 10 */
    int max_iterations;
    int max_passes;
    int total_edges_m;            /* 1: M = max(1, m) (totalm); 0: M = m / 2 */
    int super_move_batch;         /* sgmb<k>; 1 = sequential super-move */
    int parallel;                 /* 0: cd_serial semantics; 1: racy OpenMP (cd_parallel) */
    int threads;                  /* OpenMP threads for parallel=1 (0 = runtime default) */
    int refine;                   /* useRefinement (refine<k> / norefine) */
    int refine_depth;             /* refinementDepth: -1 every pass, k: passes 0..k */
} orc_leiden_cfg;

typedef struct {
    int passes;                   /* GraphBrewResult::totalPasses */
    int iterations;               /* local-moving iterations, all passes */
    int pass_iterations[16];      /* per pass */
    int64_t pass0_communities;    /* communities after pass-0 local moving */
    int64_t aggregated_communities; /* after the GVE super-move merge (0 if none) */
    int super_move_iterations;
    int64_t super_moves;
    int64_t communities;          /* distinct ids in the final membership */
    double local_move_seconds, aggregate_seconds;
} orc_leiden_stats;

/* runGraphBrew in GVE_CSR mode without refinement
 * (bench/include/graphbrew/reorder/reorder_graphbrew.h:7238-7571), with
 * localMovingPhase<false> (:1588-1734), countCommunities/renumberCommunities
 * (:1843-1889), buildCommunityVertices (:1912-1942), aggregateGVEStyle
 * (:2156-2439).  membership: n entries. */
int orc_leiden(const orc_graph *g, const orc_leiden_cfg *cfg,
               uint32_t *membership, orc_leiden_stats *stats);

/* Community-order axis (CommunityOrder, reorder_graphbrew.h:286-297). */
enum {
    ORC_COMM_SIZE_DESC = 0,
    ORC_COMM_SIZE_ASC = 1,
    ORC_COMM_DEGREE_DESC = 2,
    ORC_COMM_DEGREE_ASC = 3,
    ORC_COMM_IDENTITY = 6
};
/* Intra-community axis (IntraCommunityOrder, reorder_graphbrew.h:302-378).
 * The sorted orders (HubSort .. CoreOrder) sort with std::sort, whose tie
 * order is that of the standard library; libstdc++'s (GCC 13) is restated. */
enum {
    ORC_INTRA_BFS = 0,
    ORC_INTRA_RCM = 1,
    ORC_INTRA_RCMPP = 2,
    ORC_INTRA_GORDER = 4,
    ORC_INTRA_HUBSORT = 6,
    ORC_INTRA_DEGREE_ASC = 7,
    ORC_INTRA_HUB2 = 8,
    ORC_INTRA_ALTERNATE = 9,
    ORC_INTRA_RANDOM = 10,
    ORC_INTRA_BOUNDARY_LAST = 11,
    ORC_INTRA_CORE = 12
};

/* libstdc++ (GCC 13) std::sort of `count` element ids by comp(a, b) =
 * key[a] < key[b]: the tie order the sorted intra orders inherit. */
int orc_libstdcxx_sort(uint32_t *elems, int64_t count, const uint64_t *key);
/* intra_random's swap indices (RG:6825-6845): out[j] for j = count - 1 .. 1
 * drawn in that order from std::mt19937(seed) by libstdc++'s
 * uniform_int_distribution (Lemire's method); out[0] = 0. */
int orc_random_draws(uint32_t seed, int64_t count, uint32_t *out);
/* Its depth-limit fallback alone (__partial_sort(first, last, last)). */
int orc_libstdcxx_heap_sort(uint32_t *elems, int64_t count, const uint64_t *key);

typedef struct {
    int community_order;
    int intra_order;
    int gorder_window;    /* gw<k> */
    int gorder_fallback;  /* gordf<k>; 0 = no fallback */
    int threads;          /* 1 = serial; otherwise the OpenMP default */
    int super_order;      /* ORC_SUPER_*: stage1Perm, the community order's tie-break */
    float super_gamma;    /* superGraphResolution (sg_super_rabbit) */
} orc_compose_cfg;

enum {
    ORC_SUPER_NONE = 0,
    ORC_SUPER_RABBIT = 1,   /* sg_super_rabbit, the reference's one-thread result */
    ORC_SUPER_RCM = 2,      /* sg_super_rcm, the reference's one-thread result */
    ORC_SUPER_HILBERT = 4   /* sg_hilbert */
};

/* Iteration order of a libstdc++ std::unordered_map keyed by an unsigned
 * integer after the k distinct keys are inserted in order (k <= 101473717). */
int orc_umap_order(const uint32_t *keys, int64_t k, uint32_t *out);
/* stage1Perm of a super-graph order (ORC_SUPER_*) for the membership; out has
 * max(membership) + 1 entries; gamma: superGraphResolution (Rabbit only). */
int orc_super_stage1(const orc_graph *g, const uint32_t *membership, int super_order, float gamma, uint32_t *out);

typedef struct {
    int64_t num_communities;   /* max(membership) + 1 */
    int64_t isolated;
    int64_t gorder_communities, gorder_vertices, gorder_max_community;
    int64_t fallback_communities, fallback_vertices;
    int64_t largest_community;
} orc_compose_stats;

/* orderCompose (reorder_graphbrew.h:6286-7087) for super-graph order "none".
 * new_ids: n entries, forward map old -> new. */
int orc_compose(const orc_graph *g, const uint32_t *membership,
                const orc_compose_cfg *cfg, int32_t *new_ids,
                orc_compose_stats *stats);

/* ValidatePermutationOrThrow (bench/include/external/gapbs/builder.h:2056-2080):
 * 0 = valid, 1 = out-of-range id, 2 = duplicate id. */
int orc_validate_permutation(const int32_t *new_ids, int64_t n);

/* MappingFingerprint (builder.h:1398-1411): FNV-1a-64 over (old, new) pairs. */
uint64_t orc_fingerprint(const int32_t *new_ids, int64_t n);

/* RelabelByMapping, undirected branch (builder.h:1046-1206, :1168-1201):
 * out_row_ptr n + 1 entries, out_col row_ptr[n] entries, rows sorted. */
int orc_relabel(const orc_graph *g, const int32_t *new_ids,
                int64_t *out_row_ptr, int32_t *out_col, int threads);

/* computeModularityCSR (reorder_types.h:3211-3291), summed in vertex order. */
double orc_modularity(const orc_graph *g, const uint32_t *membership,
                      double resolution);

/* Number of OpenMP threads the library was built to use (1 without OpenMP). */
int orc_max_threads(void);

/* The reference's CPU benchmark kernels (gb_kernels_cpu.c), for timing the
 * selector's arms on the host; each returns its wall time in ms.
 * `threads` <= 0 keeps the OpenMP default. */
double orc_pagerank_gs(const orc_graph *g, int max_iters, double epsilon, float *scores, int threads,
                       int *iters_out);
double orc_bfs_do(const orc_graph *g, int64_t source, int32_t *depth, int threads);
double orc_cc_afforest(const orc_graph *g, int32_t *comp, int threads);
double orc_dbg_cpu(const orc_graph *g, int32_t *new_ids, int threads);

#ifdef __cplusplus
}
#endif

#endif /* GB_ORACLE_H_ */
