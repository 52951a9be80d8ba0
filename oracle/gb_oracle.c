/*
 * gb_oracle.c -- CPU oracle for GraphBrew's algorithm-12 mapping path.
 *
 * TEST INFRASTRUCTURE ONLY: a plain-C restatement of the reference algorithm,
 * used by the tests to check the CUDA path and by the benchmark as the CPU
 * baseline.  The product library never links or loads this file.
 *
 * Reference file paths below are relative to the GraphBrew project root;
 * RG = bench/include/graphbrew/reorder/reorder_graphbrew.h,
 * RT = bench/include/graphbrew/reorder/reorder_types.h,
 * BH = bench/include/external/gapbs/builder.h.
 *
 * Floating point: every Delta-modularity expression keeps the reference's
 * association and is compiled with -ffp-contract=off, so each product, sum and
 * quotient is one IEEE double operation, exactly as in the reference.
 */
#include "gb_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_NONE ((uint32_t)0xFFFFFFFFu)

static double now_seconds(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static inline int64_t degree_of(const orc_graph *g, int64_t u)
{
    return g->row_ptr[u + 1] - g->row_ptr[u];
}

/* ------------------------------------------------------------------------ */
/* Auto resolution: RT:2743-2780.                                            */
/* ------------------------------------------------------------------------ */
double orc_auto_resolution(const orc_graph *g)
{
    const int64_t n = g->n;
    if (n == 0) return 1.0;
    /* num_edges() of an undirected CSRGraph is the directed count / 2. */
    const int64_t m = (g->row_ptr[n] - g->row_ptr[0]) / 2;
    const double avg_degree = (double)m / (double)n;
    double sum_sq = 0.0;
    for (int64_t v = 0; v < n; ++v) {
        const double d = (double)degree_of(g, v);
        const double diff = d - avg_degree;
        sum_sq += diff * diff;
    }
    const double variance = sum_sq / (double)n;
    const double cv = (avg_degree > 0) ? sqrt(variance) / avg_degree : 0.0;
    double resolution = 0.5 + 0.25 * log10(avg_degree + 1);
    resolution = fmax(0.5, fmin(1.2, resolution));
    if (cv > 2.0) {
        const double factor = 2.0 / fmax(2.0, sqrt(cv));
        resolution = fmax(0.5, resolution * factor);
    }
    return resolution;
}

/* ------------------------------------------------------------------------ */
/* Dense accumulator with a touched list.  The reference keeps a sparse     */
/* open-addressing table (RG:1133-1232); the selection below is independent */
/* of key iteration order, so a dense table gives the same answers.         */
/* ------------------------------------------------------------------------ */
typedef struct {
    double *val;       /* capacity entries, all 0 between uses */
    uint32_t *keys;    /* touched keys */
    int64_t nkeys;
} orc_acc;

static int acc_init(orc_acc *a, int64_t capacity, int64_t max_keys)
{
    a->val = (double *)calloc((size_t)(capacity > 0 ? capacity : 1), sizeof(double));
    a->keys = (uint32_t *)malloc((size_t)(max_keys > 0 ? max_keys : 1) * sizeof(uint32_t));
    a->nkeys = 0;
    return (a->val && a->keys) ? ORC_OK : ORC_ENOMEM;
}

static void acc_free(orc_acc *a)
{
    free(a->val);
    free(a->keys);
}

static inline void acc_add(orc_acc *a, uint32_t k, double w)
{
    /* A key is "touched" when first added; weights here are always > 0. */
    if (a->val[k] == 0.0) a->keys[a->nkeys++] = k;
    a->val[k] += w;
}

static inline void acc_clear(orc_acc *a)
{
    for (int64_t i = 0; i < a->nkeys; ++i) a->val[a->keys[i]] = 0.0;
    a->nkeys = 0;
}

/* deltaModularity (RG:1295-1298). */
static inline double delta_modularity(double k_u_c, double k_u_d, double k_u,
                                      double sigma_c, double sigma_d,
                                      double M, double R)
{
    return (k_u_c - k_u_d) / M - R * k_u * (sigma_c - sigma_d + k_u) / (2.0 * M * M);
}

/* chooseCommunityGreedy (RG:1494-1527): the candidate with the largest
 * positive delta; equal deltas go to the smaller community id. */
static inline uint32_t choose_community(const orc_acc *a, uint32_t d, double k_u,
                                        const double *ctot, double M, double R,
                                        double *best_delta_out)
{
    uint32_t best_c = d;
    double best_delta = 0.0;
    int found = 0;
    const double k_u_d = a->val[d];
    const double sigma_d = ctot[d];
    for (int64_t i = 0; i < a->nkeys; ++i) {
        const uint32_t c = a->keys[i];
        if (c == d) continue;
        const double delta = delta_modularity(a->val[c], k_u_d, k_u, ctot[c], sigma_d, M, R);
        if (delta > best_delta || (found && delta == best_delta && c < best_c)) {
            best_delta = delta;
            best_c = c;
            found = 1;
        }
    }
    *best_delta_out = best_delta;
    return best_c;
}

/* localMovingPhase<false> in serial order (RG:1588-1734 with one thread). */
static int local_move_serial(const orc_graph *g, uint32_t *vcom, double *ctot,
                             char *vaff, const double *vtot, double M, double R,
                             double tolerance, int max_iterations, orc_acc *acc)
{
    const int64_t n = g->n;
    int iterations = 0;
    for (int iter = 0; iter < max_iterations; ++iter) {
        double total_delta = 0.0;
        for (int64_t u = 0; u < n; ++u) {
            if (!vaff[u]) continue;
            const uint32_t d = vcom[u];
            acc_clear(acc);
            for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) {
                const int32_t v = g->col[e];
                if (v == u) continue;
                acc_add(acc, vcom[v], 1.0);
            }
            double delta;
            const uint32_t best_c = choose_community(acc, d, vtot[u], ctot, M, R, &delta);
            if (best_c != d) {
                ctot[d] -= vtot[u];
                ctot[best_c] += vtot[u];
                vcom[u] = best_c;
                for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e)
                    vaff[g->col[e]] = 1;
            }
            vaff[u] = 0;
            total_delta += delta;
        }
        ++iterations;
        if (total_delta <= tolerance) break;
    }
    return iterations;
}

/* Refinement (RG:7330-7392): bounds = the local-moving membership, every
 * vertex back to a singleton, then one serial sweep of
 * localMovingPhase<true> (RG:1588-1734): a vertex whose community already
 * holds more than itself (ctot > k_u * 1.001) stays; the others scan only
 * neighbours inside their bound (scanCommunities<true>, RG:1392-1437) and
 * move greedily; changeCommunity<true> (RG:1538-1573) repeats the singleton
 * test, which in serial order always passes here. */
static void refine_serial(const orc_graph *g, uint32_t *vcom, double *ctot, const double *vtot,
                          const uint32_t *vcob, double M, double R, orc_acc *acc)
{
    const int64_t n = g->n;
    for (int64_t u = 0; u < n; ++u) {
        const uint32_t d = vcom[u];
        if (ctot[d] > vtot[u] * 1.001) continue;
        acc_clear(acc);
        for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) {
            const int32_t v = g->col[e];
            if (v == u) continue;
            if (vcob[v] != vcob[u]) continue;
            acc_add(acc, vcom[v], 1.0);
        }
        double delta;
        const uint32_t best_c = choose_community(acc, d, vtot[u], ctot, M, R, &delta);
        if (best_c != d) {
            const double old_ctot = ctot[d];
            ctot[d] -= vtot[u];
            if (old_ctot > vtot[u] * 1.001) {
                ctot[d] += vtot[u];
                continue;
            }
            ctot[best_c] += vtot[u];
            vcom[u] = best_c;
        }
    }
}

#ifdef _OPENMP
/* localMovingPhase<false> as the reference runs it with several threads:
 * dynamic chunks of 4096 vertices (DEFAULT_TILE_SIZE), racy reads of vcom and
 * ctot, atomic ctot updates (RG:1538-1573, :1655-1724). */
static int local_move_parallel(const orc_graph *g, uint32_t *vcom, double *ctot,
                               char *vaff, const double *vtot, double M, double R,
                               double tolerance, int max_iterations,
                               orc_acc *accs)
{
    const int64_t n = g->n;
    int iterations = 0;
    for (int iter = 0; iter < max_iterations; ++iter) {
        double total_delta = 0.0;
#pragma omp parallel reduction(+ : total_delta)
        {
            orc_acc *acc = &accs[omp_get_thread_num()];
#pragma omp for schedule(dynamic, 4096)
            for (int64_t u = 0; u < n; ++u) {
                if (!__atomic_load_n(&vaff[u], __ATOMIC_RELAXED)) continue;
                const uint32_t d = __atomic_load_n(&vcom[u], __ATOMIC_RELAXED);
                acc_clear(acc);
                for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) {
                    const int32_t v = g->col[e];
                    if (v == u) continue;
                    acc_add(acc, __atomic_load_n(&vcom[v], __ATOMIC_RELAXED), 1.0);
                }
                double delta;
                const uint32_t best_c = choose_community(acc, d, vtot[u], ctot, M, R, &delta);
                if (best_c != d) {
#pragma omp atomic
                    ctot[d] -= vtot[u];
#pragma omp atomic
                    ctot[best_c] += vtot[u];
                    __atomic_store_n(&vcom[u], best_c, __ATOMIC_RELAXED);
                    for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e)
                        __atomic_store_n(&vaff[g->col[e]], (char)1, __ATOMIC_RELAXED);
                }
                __atomic_store_n(&vaff[u], (char)0, __ATOMIC_RELAXED);
                total_delta += delta;
            }
        }
        ++iterations;
        if (total_delta <= tolerance) break;
    }
    return iterations;
}
#endif

/* countCommunities (RG:1843-1865). */
static int64_t count_communities(const uint32_t *vcom, int64_t n, uint32_t *exists)
{
    memset(exists, 0, (size_t)n * sizeof(uint32_t));
    int64_t count = 0;
    for (int64_t u = 0; u < n; ++u) {
        if (!exists[vcom[u]]) {
            exists[vcom[u]] = 1;
            ++count;
        }
    }
    return count;
}

/* renumberCommunities (RG:1870-1889): increasing old id. */
static int64_t renumber_communities(uint32_t *vcom, int64_t n, uint32_t *cmap)
{
    uint32_t next = 0;
    for (int64_t i = 0; i < n; ++i)
        if (cmap[i]) cmap[i] = next++;
    for (int64_t u = 0; u < n; ++u) vcom[u] = cmap[vcom[u]];
    return next;
}

/* aggregateGVEStyle (RG:2156-2439).  vcom holds renumbered ids < C on entry;
 * on exit it holds the merged, first-occurrence renumbered ids and ctot their
 * totals.  Returns the merged community count. */
static int64_t aggregate_gve(const orc_graph *g, uint32_t *vcom, double *ctot,
                             const double *vtot, int64_t C, double M, double R,
                             int max_iterations, int batch, int parallel,
                             orc_leiden_stats *stats)
{
    const int64_t n = g->n;
    int64_t result = -1;
    double *super_weight = (double *)calloc((size_t)(C > 0 ? C : 1), sizeof(double));
    int64_t *coff = (int64_t *)calloc((size_t)C + 1, sizeof(int64_t));
    uint32_t *cvtx = (uint32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(uint32_t));
    int64_t *adj_off = (int64_t *)calloc((size_t)C + 1, sizeof(int64_t));
    uint32_t *super_comm = (uint32_t *)malloc((size_t)(C > 0 ? C : 1) * sizeof(uint32_t));
    double *super_ctot = (double *)malloc((size_t)(C > 0 ? C : 1) * sizeof(double));
    uint32_t *proposed = (uint32_t *)malloc((size_t)(C > 0 ? C : 1) * sizeof(uint32_t));
    double *proposed_delta = (double *)malloc((size_t)(C > 0 ? C : 1) * sizeof(double));
    uint32_t *adj_c = NULL;
    double *adj_w = NULL;
    orc_acc acc = {0};
    orc_acc *taccs = NULL;
    int ntacc = 0;
    if (!super_weight || !coff || !cvtx || !adj_off || !super_comm || !super_ctot ||
        !proposed || !proposed_delta || acc_init(&acc, C, C) != ORC_OK)
        goto done;
#ifdef _OPENMP
    if (parallel) {
        ntacc = omp_get_max_threads();
        taccs = (orc_acc *)calloc((size_t)ntacc, sizeof(orc_acc));
        if (!taccs) goto done;
        for (int i = 0; i < ntacc; ++i)
            if (acc_init(&taccs[i], C, C) != ORC_OK) goto done;
    }
#endif

    /* super_weight (RG:2173-2178). */
    for (int64_t v = 0; v < n; ++v) super_weight[vcom[v]] += vtot[v];

    /* buildCommunityVertices (RG:1912-1942): stable counting sort. */
    for (int64_t u = 0; u < n; ++u) coff[vcom[u] + 1]++;
    for (int64_t c = 0; c < C; ++c) coff[c + 1] += coff[c];
    {
        int64_t *pos = (int64_t *)malloc((size_t)(C > 0 ? C : 1) * sizeof(int64_t));
        if (!pos) goto done;
        memcpy(pos, coff, (size_t)C * sizeof(int64_t));
        for (int64_t u = 0; u < n; ++u) cvtx[pos[vcom[u]]++] = (uint32_t)u;
        free(pos);
    }

    /* Super-graph adjacency: inter-community edges only (RG:2184-2224). */
    {
        /* First pass: count distinct neighbour communities per community. */
        for (int64_t c = 0; c < C; ++c) {
            acc_clear(&acc);
            for (int64_t i = coff[c]; i < coff[c + 1]; ++i) {
                const uint32_t u = cvtx[i];
                for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) {
                    const uint32_t cv = vcom[g->col[e]];
                    if (cv != (uint32_t)c) acc_add(&acc, cv, 1.0);
                }
            }
            adj_off[c + 1] = adj_off[c] + acc.nkeys;
        }
        acc_clear(&acc);
        adj_c = (uint32_t *)malloc((size_t)(adj_off[C] > 0 ? adj_off[C] : 1) * sizeof(uint32_t));
        adj_w = (double *)malloc((size_t)(adj_off[C] > 0 ? adj_off[C] : 1) * sizeof(double));
        if (!adj_c || !adj_w) goto done;
        for (int64_t c = 0; c < C; ++c) {
            acc_clear(&acc);
            for (int64_t i = coff[c]; i < coff[c + 1]; ++i) {
                const uint32_t u = cvtx[i];
                for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) {
                    const uint32_t cv = vcom[g->col[e]];
                    if (cv != (uint32_t)c) acc_add(&acc, cv, 1.0);
                }
            }
            for (int64_t k = 0; k < acc.nkeys; ++k) {
                adj_c[adj_off[c] + k] = acc.keys[k];
                adj_w[adj_off[c] + k] = acc.val[acc.keys[k]];
            }
        }
        acc_clear(&acc);
    }

    /* Batched super-move (RG:2226-2380).  A batch of 1 is the sequential
     * variant (RG:2325-2380): both propose from the state before the vertex's
     * own batch and commit moves with a positive delta in id order. */
    for (int64_t c = 0; c < C; ++c) {
        super_comm[c] = (uint32_t)c;
        super_ctot[c] = super_weight[c];
    }
    const int super_max_iter = max_iterations < 3 ? max_iterations : 3;
    const int64_t bs = batch > 1 ? batch : 1;
    int iters_run = 0;
    for (int iter = 0; iter < super_max_iter; ++iter) {
        int64_t moves = 0;
        ++iters_run;
        for (int64_t begin = 0; begin < C; begin += bs) {
            const int64_t end = begin + bs < C ? begin + bs : C;
#ifdef _OPENMP
#pragma omp parallel if (parallel && end - begin > 256)
#endif
            {
                orc_acc *a = &acc;
#ifdef _OPENMP
                if (taccs) a = &taccs[omp_get_thread_num()];
#pragma omp for schedule(static)
#endif
                for (int64_t c = begin; c < end; ++c) {
                    const uint32_t d = super_comm[c];
                    const double kc = super_weight[c];
                    const double sigma_d = super_ctot[d];
                    const double delta_removal = R * kc * (sigma_d - kc) / M;
                    acc_clear(a);
                    for (int64_t k = adj_off[c]; k < adj_off[c + 1]; ++k)
                        acc_add(a, super_comm[adj_c[k]], adj_w[k]);
                    const double kc_to_d = a->val[d];
                    uint32_t best_comm = d;
                    double best_delta = 0.0;
                    for (int64_t k = 0; k < a->nkeys; ++k) {
                        const uint32_t e = a->keys[k];
                        const double kc_to_e = a->val[e];
                        const double delta_addition = e == d
                            ? kc_to_d - delta_removal
                            : kc_to_e - R * kc * super_ctot[e] / M;
                        const double delta = delta_addition - delta_removal + kc_to_d;
                        if (delta > best_delta || (delta == best_delta && e < best_comm)) {
                            best_delta = delta;
                            best_comm = e;
                        }
                    }
                    acc_clear(a);
                    proposed[c] = best_comm;
                    proposed_delta[c] = best_delta;
                }
            }
            for (int64_t c = begin; c < end; ++c) {
                const uint32_t d = super_comm[c];
                const uint32_t best_comm = proposed[c];
                if (best_comm == d || proposed_delta[c] <= 0.0) continue;
                const double kc = super_weight[c];
                super_ctot[d] -= kc;
                super_ctot[best_comm] += kc;
                super_comm[c] = best_comm;
                ++moves;
            }
        }
        stats->super_moves += moves;
        if (moves == 0) break;
    }
    stats->super_move_iterations += iters_run;

    /* Remap and first-occurrence renumber (RG:2389-2419). */
    for (int64_t v = 0; v < n; ++v) vcom[v] = super_comm[vcom[v]];
    {
        uint32_t max_c = 0;
        for (int64_t v = 0; v < n; ++v) if (vcom[v] > max_c) max_c = vcom[v];
        uint32_t *renum = (uint32_t *)malloc(((size_t)max_c + 1) * sizeof(uint32_t));
        if (!renum) goto done;
        for (uint32_t c = 0; c <= max_c; ++c) renum[c] = ORC_NONE;
        uint32_t next = 0;
        for (int64_t v = 0; v < n; ++v)
            if (renum[vcom[v]] == ORC_NONE) renum[vcom[v]] = next++;
        for (int64_t v = 0; v < n; ++v) vcom[v] = renum[vcom[v]];
        free(renum);
        result = next;
    }
    /* ctot of the merged communities (RG:2421-2428); ctot has n entries. */
    for (int64_t v = 0; v < n; ++v) ctot[v] = 0.0;
    for (int64_t v = 0; v < n; ++v) ctot[vcom[v]] += vtot[v];

done:
    free(super_weight);
    free(coff);
    free(cvtx);
    free(adj_off);
    free(adj_c);
    free(adj_w);
    free(super_comm);
    free(super_ctot);
    free(proposed);
    free(proposed_delta);
    acc_free(&acc);
    if (taccs) {
        for (int i = 0; i < ntacc; ++i) acc_free(&taccs[i]);
        free(taccs);
    }
    return result;
}

int orc_leiden(const orc_graph *g, const orc_leiden_cfg *cfg,
               uint32_t *membership, orc_leiden_stats *stats)
{
    if (!g || !cfg || !membership || g->n < 0) return ORC_EINVAL;
    orc_leiden_stats local_stats;
    if (!stats) stats = &local_stats;
    memset(stats, 0, sizeof(*stats));
    const int64_t n = g->n;
    if (n == 0) return ORC_OK;
    const int64_t m = (g->row_ptr[n] - g->row_ptr[0]) / 2;
    /* RG:7246-7248. */
    const double M = cfg->total_edges_m ? fmax(1.0, (double)m) : (double)m / 2.0;
    const double R = cfg->resolution;

    int rc = ORC_ENOMEM;
    double *vtot = (double *)malloc((size_t)n * sizeof(double));
    double *ctot = (double *)malloc((size_t)n * sizeof(double));
    char *vaff = (char *)malloc((size_t)n);
    uint32_t *cmap = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
    uint32_t *vcob = NULL;
    orc_acc *accs = NULL;
    int nacc = 1;
#ifdef _OPENMP
    if (cfg->parallel) {
        if (cfg->threads > 0) omp_set_num_threads(cfg->threads);
        nacc = omp_get_max_threads();
    }
#endif
    accs = (orc_acc *)calloc((size_t)nacc, sizeof(orc_acc));
    if (!vtot || !ctot || !vaff || !cmap || !accs) goto done;
    for (int i = 0; i < nacc; ++i)
        if (acc_init(&accs[i], n, n) != ORC_OK) goto done;

    /* computeVertexWeights / initializeCommunities (RG:1307-1381). */
    for (int64_t u = 0; u < n; ++u) {
        vtot[u] = (double)degree_of(g, u);
        membership[u] = (uint32_t)u;
        ctot[u] = vtot[u];
        vaff[u] = 1;
    }

    double tolerance = cfg->tolerance;
    int64_t prev_communities = n;
    int pass = 0;
    for (; pass < cfg->max_passes && M > 0; ++pass) {
        double t0 = now_seconds();
        int iters;
#ifdef _OPENMP
        if (cfg->parallel)
            iters = local_move_parallel(g, membership, ctot, vaff, vtot, M, R,
                                        tolerance, cfg->max_iterations, accs);
        else
#endif
            iters = local_move_serial(g, membership, ctot, vaff, vtot, M, R,
                                      tolerance, cfg->max_iterations, &accs[0]);
        stats->local_move_seconds += now_seconds() - t0;
        if (pass < 16) stats->pass_iterations[pass] = iters;
        stats->iterations += iters;
        if (cfg->refine && (cfg->refine_depth < 0 || pass <= cfg->refine_depth)) {
            if (cfg->parallel) { rc = ORC_EUNSUPPORTED; goto done; }
            if (!vcob) {
                vcob = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
                if (!vcob) goto done;
            }
            memcpy(vcob, membership, (size_t)n * sizeof(uint32_t));
            for (int64_t u = 0; u < n; ++u) {
                membership[u] = (uint32_t)u;
                ctot[u] = vtot[u];
            }
            refine_serial(g, membership, ctot, vtot, vcob, M, R, &accs[0]);
        }

        const int64_t nc = count_communities(membership, n, cmap);
        if (pass == 0) stats->pass0_communities = nc;
        /* GVE mode checks convergence only after aggregation (RG:7400-7421). */
        if (pass >= cfg->max_passes - 1) break;

        t0 = now_seconds();
        const int64_t C = renumber_communities(membership, n, cmap);
        const int64_t merged = aggregate_gve(g, membership, ctot, vtot, C, M, R,
                                             cfg->max_iterations, cfg->super_move_batch,
                                             cfg->parallel, stats);
        stats->aggregate_seconds += now_seconds() - t0;
        if (merged < 0) goto done;
        stats->aggregated_communities = merged;
        /* RG:7436-7452. */
        if (merged >= prev_communities || merged == 1) break;
        if ((double)merged / (double)prev_communities >= cfg->aggregation_tolerance) break;
        prev_communities = merged;
        for (int64_t v = 0; v < n; ++v) vaff[v] = 1;
        tolerance /= cfg->tolerance_drop;
    }
    stats->passes = pass + 1;
    {
        const int64_t distinct = count_communities(membership, n, cmap);
        stats->communities = distinct;
    }
    rc = ORC_OK;
done:
    free(vtot);
    free(ctot);
    free(vaff);
    free(cmap);
    free(vcob);
    if (accs) {
        for (int i = 0; i < nacc; ++i) acc_free(&accs[i]);
        free(accs);
    }
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Intra-community primitives.                                               */
/* ------------------------------------------------------------------------ */

/* intraBFSFromHub (RG:3929-3984): FIFO BFS from the first max-degree vertex,
 * neighbours in row order restricted to the community, unreached vertices
 * appended in vertex order. */
static void intra_bfs(const orc_graph *g, const uint32_t *verts, int64_t sz, uint32_t c,
                      const uint32_t *memb, const uint32_t *deg, const int64_t *v2l,
                      uint32_t *local_ids, char *visited, uint32_t *queue)
{
    if (sz == 0) return;
    if (sz == 1) { local_ids[verts[0]] = 0; return; }
    memset(visited, 0, (size_t)sz);
    uint32_t start = verts[0];
    uint32_t max_deg = deg[verts[0]];
    for (int64_t i = 0; i < sz; ++i)
        if (deg[verts[i]] > max_deg) { max_deg = deg[verts[i]]; start = verts[i]; }
    uint32_t local_id = 0;
    int64_t head = 0, tail = 0;
    queue[tail++] = start;
    visited[v2l[start]] = 1;
    while (head < tail) {
        const uint32_t u = queue[head++];
        local_ids[u] = local_id++;
        for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) {
            const int32_t v = g->col[e];
            if (memb[v] != c) continue;
            const int64_t li = v2l[v];
            if (li != -1 && !visited[li]) {
                visited[li] = 1;
                queue[tail++] = (uint32_t)v;
            }
        }
    }
    for (int64_t i = 0; i < sz; ++i)
        if (!visited[i]) local_ids[verts[i]] = local_id++;
}

typedef struct { uint32_t deg, v; } orc_pair;

static int pair_cmp(const void *a, const void *b)
{
    const orc_pair *x = (const orc_pair *)a, *y = (const orc_pair *)b;
    if (x->deg != y->deg) return x->deg < y->deg ? -1 : 1;
    if (x->v != y->v) return x->v < y->v ? -1 : 1;
    return 0;
}

typedef struct { uint64_t key; uint32_t v; } orc_rankrec;

static int rankrec_cmp(const void *a, const void *b)
{
    const orc_rankrec *x = (const orc_rankrec *)a, *y = (const orc_rankrec *)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->v < y->v ? -1 : (x->v > y->v);
}

/* RCM++ start (RG:4185-4256): BFS depths from the min-degree seed (seed
 * marked visited; unreached vertices keep depth 0), then the vertex with
 * the least degree rank + depth rank, ranks by (degree, id) ascending and
 * (depth descending, id); ties to the smaller id.  The reference's score
 * 0.5 * degRank + 0.5 * depthRank is exact in double, so the sum of ranks
 * orders the same. */
static int rcmpp_start(const orc_graph *g, const uint32_t *verts, int64_t sz, uint32_t c,
                       const uint32_t *memb, const uint32_t *deg, const int64_t *v2l, uint32_t seed,
                       char *visited, uint32_t *level_a, uint32_t *level_b, uint32_t *out)
{
    uint32_t *depth = (uint32_t *)calloc((size_t)sz, sizeof(uint32_t));
    orc_rankrec *byd = (orc_rankrec *)malloc((size_t)sz * sizeof(orc_rankrec));
    orc_rankrec *byp = (orc_rankrec *)malloc((size_t)sz * sizeof(orc_rankrec));
    int64_t *rank = (int64_t *)calloc((size_t)sz, sizeof(int64_t));
    if (!depth || !byd || !byp || !rank) {
        free(depth); free(byd); free(byp); free(rank);
        return ORC_ENOMEM;
    }
    memset(visited, 0, (size_t)sz);
    uint32_t *cur = level_a, *nxt = level_b;
    int64_t ncur = 1, nnxt;
    cur[0] = seed;
    visited[v2l[seed]] = 1;
    uint32_t d = 0;
    while (ncur > 0) {
        nnxt = 0;
        for (int64_t i = 0; i < ncur; ++i) {
            const uint32_t u = cur[i];
            depth[v2l[u]] = d;
            for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) {
                const int32_t v = g->col[e];
                if (memb[v] != c) continue;
                const int64_t li = v2l[v];
                if (li != -1 && !visited[li]) { visited[li] = 1; nxt[nnxt++] = (uint32_t)v; }
            }
        }
        ++d;
        uint32_t *t = cur; cur = nxt; nxt = t; ncur = nnxt;
    }
    for (int64_t i = 0; i < sz; ++i) {
        const uint32_t v = verts[i];
        byd[i].key = deg[v];
        byd[i].v = v;
        byp[i].key = ~(uint64_t)depth[i];
        byp[i].v = v;
    }
    qsort(byd, (size_t)sz, sizeof(orc_rankrec), rankrec_cmp);
    qsort(byp, (size_t)sz, sizeof(orc_rankrec), rankrec_cmp);
    for (int64_t i = 0; i < sz; ++i) {
        rank[v2l[byd[i].v]] += i;
        rank[v2l[byp[i].v]] += i;
    }
    uint32_t best = seed;
    int64_t best_rank = INT64_MAX;
    for (int64_t i = 0; i < sz; ++i) {
        const uint32_t v = verts[i];
        if (rank[i] < best_rank || (rank[i] == best_rank && v < best)) { best_rank = rank[i]; best = v; }
    }
    *out = best;
    free(depth); free(byd); free(byp); free(rank);
    return ORC_OK;
}

/* intraRCM (RG:4000-4134): min-degree start (ties -> smaller id), up to 3
 * George-Liu steps for sz > 32, Cuthill-McKee BFS with children sorted by
 * (degree, id), reversal of the reached part, unreached tail in input order.
 * pp: intraRCMpp (RG:4154-4342), the same with the RCM++ start for sz > 32
 * and George-Liu ties to the smaller id instead of the first in level order. */
static int intra_rcm(const orc_graph *g, const uint32_t *verts, int64_t sz, uint32_t c,
                     const uint32_t *memb, const uint32_t *deg, const int64_t *v2l,
                     uint32_t *local_ids, char *visited, uint32_t *queue,
                     uint32_t *level_a, uint32_t *level_b, orc_pair *cand, int pp)
{
    if (sz == 0) return ORC_OK;
    if (sz == 1) { local_ids[verts[0]] = 0; return ORC_OK; }
    uint32_t start = verts[0];
    uint32_t min_deg = deg[verts[0]];
    for (int64_t i = 0; i < sz; ++i) {
        const uint32_t v = verts[i];
        if (deg[v] < min_deg || (deg[v] == min_deg && v < start)) { min_deg = deg[v]; start = v; }
    }
    if (pp && sz > 32) {
        const int rc = rcmpp_start(g, verts, sz, c, memb, deg, v2l, start, visited, level_a, level_b, &start);
        if (rc != ORC_OK) return rc;
    }
    const int max_gl = sz <= 32 ? 0 : 3;
    if (max_gl > 0) {
        uint32_t gl_node = start;
        int64_t prev_ecc = 0;
        for (int it = 0; it < max_gl; ++it) {
            memset(visited, 0, (size_t)sz);
            uint32_t *cur = level_a, *nxt = level_b;
            int64_t ncur = 1, nnxt;
            cur[0] = gl_node;
            int64_t ecc = 0;
            /* The George-Liu sweep does not mark its start vertex visited. */
            for (;;) {
                nnxt = 0;
                for (int64_t i = 0; i < ncur; ++i) {
                    const uint32_t u = cur[i];
                    for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) {
                        const int32_t v = g->col[e];
                        if (memb[v] != c) continue;
                        const int64_t li = v2l[v];
                        if (li != -1 && !visited[li]) { visited[li] = 1; nxt[nnxt++] = (uint32_t)v; }
                    }
                }
                if (nnxt == 0) break;
                ++ecc;
                uint32_t *t = cur; cur = nxt; nxt = t; ncur = nnxt;
            }
            if (ecc <= prev_ecc) break;
            prev_ecc = ecc;
            uint32_t best_v = cur[0];
            uint32_t best_deg = deg[cur[0]];
            for (int64_t i = 1; i < ncur; ++i)
                if (deg[cur[i]] < best_deg || (pp && deg[cur[i]] == best_deg && cur[i] < best_v)) {
                    best_deg = deg[cur[i]];
                    best_v = cur[i];
                }
            gl_node = best_v;
        }
        start = gl_node;
    }
    memset(visited, 0, (size_t)sz);
    int64_t head = 0, tail = 0, nord = 0;
    uint32_t *order = level_a; /* cmOrder */
    const int64_t sli = v2l[start];
    if (sli >= 0 && sli < sz) { queue[tail++] = start; visited[sli] = 1; }
    while (head < tail) {
        const uint32_t u = queue[head++];
        order[nord++] = u;
        int64_t nc = 0;
        for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) {
            const int32_t v = g->col[e];
            if (memb[v] != c) continue;
            const int64_t li = v2l[v];
            if (li != -1 && !visited[li]) {
                visited[li] = 1;
                cand[nc].deg = deg[v];
                cand[nc].v = (uint32_t)v;
                ++nc;
            }
        }
        qsort(cand, (size_t)nc, sizeof(orc_pair), pair_cmp);
        for (int64_t i = 0; i < nc; ++i) queue[tail++] = cand[i].v;
    }
    const int64_t main_size = nord;
    for (int64_t i = 0; i < sz; ++i)
        if (!visited[i]) order[nord++] = verts[i];
    for (int64_t i = 0; i < main_size; ++i) local_ids[order[i]] = (uint32_t)(main_size - 1 - i);
    for (int64_t i = main_size; i < nord; ++i) local_ids[order[i]] = (uint32_t)i;
    return ORC_OK;
}

/* intraGorderGreedy (RG:4420-4587): relaxed Gorder with a UnitHeap.  The
 * linked list keeps buckets contiguous in descending key order; each bucket
 * is LIFO (insert at front), extract-max takes the front of the highest
 * non-empty bucket.  The heap's "top" cursor never reaches the output, so it
 * is not kept. */
typedef struct {
    int *key, *prev, *next;   /* per local vertex */
    int *bfirst, *bsecond;    /* per bucket */
    int64_t *ladj_off;        /* local adjacency */
    int64_t *ladj;
    uint32_t *placed;
    int64_t cap_v, cap_e, cap_b;
} orc_gorder_ws;

static int gorder_ws_reserve(orc_gorder_ws *w, int64_t sz, int64_t ne, int64_t nb)
{
    if (sz > w->cap_v) {
        free(w->key); free(w->prev); free(w->next); free(w->ladj_off); free(w->placed);
        w->key = (int *)malloc((size_t)sz * sizeof(int));
        w->prev = (int *)malloc((size_t)sz * sizeof(int));
        w->next = (int *)malloc((size_t)sz * sizeof(int));
        w->ladj_off = (int64_t *)malloc(((size_t)sz + 1) * sizeof(int64_t));
        w->placed = (uint32_t *)malloc((size_t)sz * sizeof(uint32_t));
        w->cap_v = sz;
        if (!w->key || !w->prev || !w->next || !w->ladj_off || !w->placed) return ORC_ENOMEM;
    }
    if (ne > w->cap_e) {
        free(w->ladj);
        w->ladj = (int64_t *)malloc((size_t)(ne > 0 ? ne : 1) * sizeof(int64_t));
        w->cap_e = ne;
        if (!w->ladj) return ORC_ENOMEM;
    }
    if (nb > w->cap_b) {
        free(w->bfirst); free(w->bsecond);
        w->bfirst = (int *)malloc((size_t)nb * sizeof(int));
        w->bsecond = (int *)malloc((size_t)nb * sizeof(int));
        w->cap_b = nb;
        if (!w->bfirst || !w->bsecond) return ORC_ENOMEM;
    }
    return ORC_OK;
}

static void gorder_ws_free(orc_gorder_ws *w)
{
    free(w->key); free(w->prev); free(w->next); free(w->ladj_off); free(w->placed);
    free(w->ladj); free(w->bfirst); free(w->bsecond);
    memset(w, 0, sizeof(*w));
}

typedef struct {
    orc_gorder_ws *w;
    int max_key;
} orc_unitheap;

static void uh_unlink(orc_unitheap *h, int idx)
{
    orc_gorder_ws *w = h->w;
    const int p = w->prev[idx], nx = w->next[idx];
    if (p >= 0) w->next[p] = nx;
    if (nx >= 0) w->prev[nx] = p;
    const int k = w->key[idx];
    if (w->bfirst[k] == idx && w->bsecond[k] == idx) {
        w->bfirst[k] = w->bsecond[k] = -1;
    } else if (w->bfirst[k] == idx) {
        w->bfirst[k] = nx;
    } else if (w->bsecond[k] == idx) {
        w->bsecond[k] = p;
    }
}

static void uh_link_front(orc_unitheap *h, int idx, int k)
{
    orc_gorder_ws *w = h->w;
    w->key[idx] = k;
    if (w->bfirst[k] < 0) {
        int after = -1;
        for (int bk = k - 1; bk >= 0; --bk)
            if (w->bfirst[bk] >= 0) { after = w->bfirst[bk]; break; }
        int before = -1;
        for (int bk = k + 1; bk <= h->max_key; ++bk)
            if (w->bsecond[bk] >= 0) { before = w->bsecond[bk]; break; }
        w->prev[idx] = before;
        w->next[idx] = after;
        if (before >= 0) w->next[before] = idx;
        if (after >= 0) w->prev[after] = idx;
        w->bfirst[k] = w->bsecond[k] = idx;
    } else {
        const int old_first = w->bfirst[k];
        const int before_old = w->prev[old_first];
        w->prev[idx] = before_old;
        w->next[idx] = old_first;
        w->prev[old_first] = idx;
        if (before_old >= 0) w->next[before_old] = idx;
        w->bfirst[k] = idx;
    }
    if (k > h->max_key) h->max_key = k;
}

static void uh_delete(orc_unitheap *h, int idx)
{
    orc_gorder_ws *w = h->w;
    uh_unlink(h, idx);
    w->prev[idx] = w->next[idx] = -1;
    w->key[idx] = -1;
    while (h->max_key > 0 && w->bfirst[h->max_key] < 0) h->max_key--;
}

static int uh_extract_max(orc_unitheap *h)
{
    orc_gorder_ws *w = h->w;
    while (h->max_key > 0 && w->bfirst[h->max_key] < 0) h->max_key--;
    const int idx = w->bfirst[h->max_key];
    if (idx >= 0) uh_delete(h, idx);
    return idx;
}

static int intra_gorder(const orc_graph *g, const uint32_t *verts, int64_t sz, uint32_t c,
                        const uint32_t *memb, const uint32_t *deg, const int64_t *v2l,
                        int window, uint32_t *local_ids, orc_gorder_ws *w)
{
    if (sz == 0) return ORC_OK;
    if (sz == 1) { local_ids[verts[0]] = 0; return ORC_OK; }
    if (sz <= 3) {
        for (int64_t i = 0; i < sz; ++i) local_ids[verts[i]] = (uint32_t)i;
        return ORC_OK;
    }
    int64_t ne = 0;
    for (int64_t i = 0; i < sz; ++i) ne += degree_of(g, verts[i]);
    /* A key never exceeds a vertex's local degree (< sz); 16 mirrors the
     * reference's initial bucket count. */
    const int64_t nb = (sz + 1 > 16 ? sz + 1 : 16);
    if (gorder_ws_reserve(w, sz, ne, nb) != ORC_OK) return ORC_ENOMEM;

    int64_t pos = 0;
    for (int64_t i = 0; i < sz; ++i) {
        w->ladj_off[i] = pos;
        const uint32_t u = verts[i];
        for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) {
            const int32_t v = g->col[e];
            if (memb[v] != c) continue;
            const int64_t li = v2l[v];
            if (li != -1 && li < sz) w->ladj[pos++] = li;
        }
    }
    w->ladj_off[sz] = pos;

    for (int64_t i = 0; i < sz; ++i) {
        w->key[i] = 0;
        w->prev[i] = (int)i - 1;
        w->next[i] = (i + 1 < sz) ? (int)(i + 1) : -1;
    }
    for (int64_t b = 0; b < nb; ++b) w->bfirst[b] = w->bsecond[b] = -1;
    w->bfirst[0] = 0;
    w->bsecond[0] = (int)(sz - 1);
    orc_unitheap h = {w, 0};

    int64_t seed = 0;
    uint32_t seed_deg = deg[verts[0]];
    for (int64_t i = 1; i < sz; ++i)
        if (deg[verts[i]] > seed_deg) { seed_deg = deg[verts[i]]; seed = i; }

    uh_delete(&h, (int)seed);
    int64_t nplaced = 0;
    w->placed[nplaced++] = (uint32_t)seed;
    local_ids[verts[seed]] = 0;
    for (int64_t k = w->ladj_off[seed]; k < w->ladj_off[seed + 1]; ++k) {
        const int64_t nb_i = w->ladj[k];
        if (w->key[nb_i] >= 0) {
            const int old = w->key[nb_i];
            uh_unlink(&h, (int)nb_i);
            uh_link_front(&h, (int)nb_i, old + 1);
        }
    }
    for (uint32_t local_id = 1; local_id < (uint32_t)sz; ++local_id) {
        const int best = uh_extract_max(&h);
        if (best < 0) {
            for (int64_t i = 0; i < sz && local_id < (uint32_t)sz; ++i) {
                if (w->key[i] >= 0) {
                    uh_delete(&h, (int)i);
                    local_ids[verts[i]] = local_id++;
                }
            }
            break;
        }
        w->placed[nplaced++] = (uint32_t)best;
        local_ids[verts[best]] = local_id;
        for (int64_t k = w->ladj_off[best]; k < w->ladj_off[best + 1]; ++k) {
            const int64_t nb_i = w->ladj[k];
            if (w->key[nb_i] >= 0) {
                const int old = w->key[nb_i];
                uh_unlink(&h, (int)nb_i);
                uh_link_front(&h, (int)nb_i, old + 1);
            }
        }
        if (nplaced > window) {
            const uint32_t old_v = w->placed[nplaced - 1 - window];
            for (int64_t k = w->ladj_off[old_v]; k < w->ladj_off[old_v + 1]; ++k) {
                const int64_t nb_i = w->ladj[k];
                if (w->key[nb_i] >= 0) {
                    const int old = w->key[nb_i];
                    if (old <= 0) continue;
                    uh_unlink(&h, (int)nb_i);
                    uh_link_front(&h, (int)nb_i, old - 1);
                }
            }
        }
    }
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Sorted intra orders (RG:6759-6955): HubSort, DegreeAsc, Hub2, Alternate,  */
/* BoundaryLast and CoreOrder each std::sort the community's vertices        */
/* (vertex order to start with) by a per-vertex comparator.  std::sort is    */
/* not stable, so the order of ties is whatever the standard library's       */
/* sort leaves; the reference is built against libstdc++ (GCC 13), whose    */
/* published algorithm is restated here (bits/stl_algo.h: __sort,           */
/* __introsort_loop, __unguarded_partition_pivot, __move_median_to_first,   */
/* __unguarded_partition, __final_insertion_sort, __insertion_sort,         */
/* __unguarded_linear_insert; bits/stl_heap.h: __make_heap, __sort_heap,    */
/* __adjust_heap, __push_heap): an introsort with a depth limit of          */
/* 2 floor(log2 n), median-of-three pivot moved to the front, an unguarded  */
/* Hoare partition, heap sort when the depth limit runs out, and a final    */
/* insertion sort with threshold 16.  Each comparator is encoded as a       */
/* 64-bit key with comp(a, b) = key[a] < key[b].                            */
/* ------------------------------------------------------------------------ */
#define LS_THRESHOLD 16

static inline int ls_less(const uint64_t *key, uint32_t a, uint32_t b) { return key[a] < key[b]; }
static inline void ls_swap(uint32_t *x, uint32_t *y) { const uint32_t t = *x; *x = *y; *y = t; }

static void ls_move_median_to_first(uint32_t *result, uint32_t *a, uint32_t *b, uint32_t *c,
                                    const uint64_t *key)
{
    if (ls_less(key, *a, *b)) {
        if (ls_less(key, *b, *c)) ls_swap(result, b);
        else if (ls_less(key, *a, *c)) ls_swap(result, c);
        else ls_swap(result, a);
    } else if (ls_less(key, *a, *c)) {
        ls_swap(result, a);
    } else if (ls_less(key, *b, *c)) {
        ls_swap(result, c);
    } else {
        ls_swap(result, b);
    }
}

static uint32_t *ls_unguarded_partition(uint32_t *first, uint32_t *last, const uint32_t *pivot,
                                        const uint64_t *key)
{
    for (;;) {
        while (ls_less(key, *first, *pivot)) ++first;
        --last;
        while (ls_less(key, *pivot, *last)) --last;
        if (!(first < last)) return first;
        ls_swap(first, last);
        ++first;
    }
}

static void ls_push_heap(uint32_t *first, int64_t hole, int64_t top, uint32_t value, const uint64_t *key)
{
    int64_t parent = (hole - 1) / 2;
    while (hole > top && ls_less(key, first[parent], value)) {
        first[hole] = first[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    first[hole] = value;
}

static void ls_adjust_heap(uint32_t *first, int64_t hole, int64_t len, uint32_t value, const uint64_t *key)
{
    const int64_t top = hole;
    int64_t child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (ls_less(key, first[child], first[child - 1])) child--;
        first[hole] = first[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        first[hole] = first[child - 1];
        hole = child - 1;
    }
    ls_push_heap(first, hole, top, value, key);
}

/* __partial_sort(first, last, last): make_heap, then sort_heap. */
static void ls_heap_sort(uint32_t *first, uint32_t *last, const uint64_t *key)
{
    const int64_t len = last - first;
    if (len >= 2) {
        int64_t parent = (len - 2) / 2;
        for (;;) {
            ls_adjust_heap(first, parent, len, first[parent], key);
            if (parent == 0) break;
            parent--;
        }
    }
    while (last - first > 1) {
        --last;
        const uint32_t value = *last;
        *last = *first;
        ls_adjust_heap(first, 0, last - first, value, key);
    }
}

static void ls_introsort_loop(uint32_t *first, uint32_t *last, int64_t depth, const uint64_t *key)
{
    while (last - first > LS_THRESHOLD) {
        if (depth == 0) {
            ls_heap_sort(first, last, key);
            return;
        }
        --depth;
        uint32_t *mid = first + (last - first) / 2;
        ls_move_median_to_first(first, first + 1, mid, last - 1, key);
        uint32_t *cut = ls_unguarded_partition(first + 1, last, first, key);
        ls_introsort_loop(cut, last, depth, key);
        last = cut;
    }
}

static void ls_unguarded_linear_insert(uint32_t *last, const uint64_t *key)
{
    const uint32_t val = *last;
    uint32_t *next = last - 1;
    while (ls_less(key, val, *next)) {
        *last = *next;
        last = next;
        --next;
    }
    *last = val;
}

static void ls_insertion_sort(uint32_t *first, uint32_t *last, const uint64_t *key)
{
    if (first == last) return;
    for (uint32_t *i = first + 1; i != last; ++i) {
        if (ls_less(key, *i, *first)) {
            const uint32_t val = *i;
            memmove(first + 1, first, (size_t)(i - first) * sizeof(uint32_t));
            *first = val;
        } else {
            ls_unguarded_linear_insert(i, key);
        }
    }
}

static void ls_sort(uint32_t *first, uint32_t *last, const uint64_t *key)
{
    if (first == last) return;
    const int64_t n = last - first;
    const int64_t lg = 63 - __builtin_clzll((unsigned long long)n);
    ls_introsort_loop(first, last, 2 * lg, key);
    if (last - first > LS_THRESHOLD) {
        ls_insertion_sort(first, first + LS_THRESHOLD, key);
        for (uint32_t *i = first + LS_THRESHOLD; i != last; ++i) ls_unguarded_linear_insert(i, key);
    } else {
        ls_insertion_sort(first, last, key);
    }
}

int orc_libstdcxx_heap_sort(uint32_t *elems, int64_t count, const uint64_t *key)
{
    if (count < 0 || (count > 0 && (!elems || !key))) return ORC_EINVAL;
    ls_heap_sort(elems, elems + count, key);
    return ORC_OK;
}

int orc_libstdcxx_sort(uint32_t *elems, int64_t count, const uint64_t *key)
{
    if (count < 0 || (count > 0 && (!elems || !key))) return ORC_EINVAL;
    ls_sort(elems, elems + count, key);
    return ORC_OK;
}

/* Core numbers of every community's induced subgraph (RG:6881-6955): the
 * internal degree counts neighbours in the same community (a self loop
 * included); peeling in degree order (Batagelj-Zaversnik bins here, the
 * reference's lazy buckets give the same, uniquely defined, numbers). */
static int community_cores(const orc_graph *g, const uint32_t *membership, const uint32_t *cverts,
                           const int64_t *cstart, uint32_t num_comm, const int64_t *v2l, uint32_t *core)
{
    const int64_t n = g->n;
    uint32_t *d = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
    int64_t *pos = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    uint32_t *vert = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
    int64_t *bin = NULL;
    int64_t bin_cap = 0;
    int rc = ORC_ENOMEM;
    if (!d || !pos || !vert) goto out;
    for (uint32_t c = 0; c < num_comm; ++c) {
        const uint32_t *verts = cverts + cstart[c];
        const int64_t sz = cstart[c + 1] - cstart[c];
        if (sz == 0) continue;
        uint32_t md = 0;
        for (int64_t i = 0; i < sz; ++i) {
            const uint32_t v = verts[i];
            uint32_t k = 0;
            for (int64_t e = g->row_ptr[v]; e < g->row_ptr[v + 1]; ++e)
                if (membership[g->col[e]] == c) ++k;
            d[v] = k;
            if (k > md) md = k;
        }
        if ((int64_t)md + 2 > bin_cap) {
            free(bin);
            bin_cap = (int64_t)md + 2;
            bin = (int64_t *)malloc((size_t)bin_cap * sizeof(int64_t));
            if (!bin) goto out;
        }
        memset(bin, 0, (size_t)(md + 2) * sizeof(int64_t));
        for (int64_t i = 0; i < sz; ++i) bin[d[verts[i]]]++;
        int64_t start = 0;
        for (uint32_t k = 0; k <= md; ++k) {
            const int64_t num = bin[k];
            bin[k] = start;
            start += num;
        }
        for (int64_t i = 0; i < sz; ++i) {
            const uint32_t v = verts[i];
            pos[v] = bin[d[v]];
            vert[bin[d[v]]] = v;
            bin[d[v]]++;
        }
        for (uint32_t k = md; k >= 1; --k) bin[k] = bin[k - 1];
        bin[0] = 0;
        for (int64_t i = 0; i < sz; ++i) {
            const uint32_t v = vert[i];
            core[v] = d[v];
            for (int64_t e = g->row_ptr[v]; e < g->row_ptr[v + 1]; ++e) {
                const uint32_t u = (uint32_t)g->col[e];
                if (membership[u] != c || v2l[u] < 0) continue;
                if (d[u] > d[v]) {
                    const uint32_t du = d[u];
                    const int64_t pu = pos[u], pw = bin[du];
                    const uint32_t w = vert[pw];
                    if (u != w) {
                        pos[u] = pw;
                        vert[pu] = w;
                        pos[w] = pu;
                        vert[pw] = u;
                    }
                    bin[du]++;
                    d[u]--;
                }
            }
        }
    }
    rc = ORC_OK;
out:
    free(d); free(pos); free(vert); free(bin);
    return rc;
}

static int is_sorted_intra(int order)
{
    return order == ORC_INTRA_HUBSORT || order == ORC_INTRA_DEGREE_ASC || order == ORC_INTRA_HUB2 ||
           order == ORC_INTRA_ALTERNATE || order == ORC_INTRA_BOUNDARY_LAST || order == ORC_INTRA_CORE;
}

/* Per-vertex sort keys of the sorted intra orders. */
static int sorted_intra_keys(const orc_graph *g, const uint32_t *membership, const uint32_t *deg,
                             const uint32_t *cverts, const int64_t *cstart, uint32_t num_comm,
                             const int64_t *v2l, int order, uint64_t *key)
{
    const int64_t n = g->n;
    const uint64_t m32 = 0xFFFFFFFFull;
    if (order == ORC_INTRA_CORE) {
        uint32_t *core = (uint32_t *)calloc((size_t)n, sizeof(uint32_t));
        if (!core) return ORC_ENOMEM;
        const int rc = community_cores(g, membership, cverts, cstart, num_comm, v2l, core);
        if (rc == ORC_OK)
            for (int64_t v = 0; v < n; ++v) key[v] = ((m32 - core[v]) << 32) | (m32 - deg[v]);
        free(core);
        return rc;
    }
    for (int64_t v = 0; v < n; ++v) {
        switch (order) {
        case ORC_INTRA_HUBSORT:
        case ORC_INTRA_ALTERNATE: key[v] = m32 - deg[v]; break;
        case ORC_INTRA_DEGREE_ASC: key[v] = deg[v]; break;
        case ORC_INTRA_HUB2: {
            uint64_t sc = 0;
            for (int64_t e = g->row_ptr[v]; e < g->row_ptr[v + 1]; ++e) sc += deg[g->col[e]];
            key[v] = ~sc;
            break;
        }
        case ORC_INTRA_BOUNDARY_LAST: {
            uint64_t ext = 0;
            for (int64_t e = g->row_ptr[v]; e < g->row_ptr[v + 1]; ++e)
                if (membership[g->col[e]] != membership[v]) ++ext;
            key[v] = (ext << 32) | (m32 - deg[v]);
            break;
        }
        default: return ORC_EUNSUPPORTED;
        }
    }
    return ORC_OK;
}

/* One community of a sorted intra order; tmp holds sz entries. */
static void intra_sorted(const uint32_t *verts, int64_t sz, int order, const uint64_t *key,
                         uint32_t *local_ids, uint32_t *tmp)
{
    if (sz == 0) return;
    if (sz == 1) {
        local_ids[verts[0]] = 0;
        return;
    }
    memcpy(tmp, verts, (size_t)sz * sizeof(uint32_t));
    ls_sort(tmp, tmp + sz, key);
    if (order == ORC_INTRA_ALTERNATE) {
        /* Hubs and leaves interleaved from both ends (RG:6806-6824). */
        const int64_t mid = (sz + 1) / 2;
        int64_t lo = 0, hi = sz - 1, p = 0;
        for (int64_t i = 0; i < mid; ++i) {
            local_ids[tmp[lo++]] = (uint32_t)p++;
            if (hi >= lo) local_ids[tmp[hi--]] = (uint32_t)p++;
        }
        return;
    }
    for (int64_t j = 0; j < sz; ++j) local_ids[tmp[j]] = (uint32_t)j;
}

/* intra_random (RG:6825-6845): std::mt19937 seeded with 0xDEADBEEF ^ c,
 * Fisher-Yates from the back, each swap index drawn by
 * std::uniform_int_distribution<size_t>(0, j).
 *
 * The engine is MT19937 (Matsumoto and Nishimura 1998) with the parameters
 * and seeding recurrence of the C++ standard's mersenne_twister_engine; the
 * state is twisted all at once when its 624 words are used up, as libstdc++
 * does (the output sequence does not depend on that).  libstdc++ maps a
 * 32-bit engine onto [0, j] by Lemire's nearly divisionless method
 * ("Fast Random Integer Generation in an Interval", 2019): the high half of
 * draw * (j + 1), redrawing while the low half is below 2^32 mod (j + 1). */
typedef struct {
    uint32_t mt[624];
    int idx;
} orc_mt19937;

static void mt_seed(orc_mt19937 *r, uint32_t seed)
{
    r->mt[0] = seed;
    for (int i = 1; i < 624; ++i) r->mt[i] = 1812433253u * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (uint32_t)i;
    r->idx = 624;
}

static uint32_t mt_next(orc_mt19937 *r)
{
    if (r->idx >= 624) {
        for (int i = 0; i < 624; ++i) {
            const uint32_t y = (r->mt[i] & 0x80000000u) | (r->mt[(i + 1) % 624] & 0x7FFFFFFFu);
            r->mt[i] = r->mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908B0DFu : 0u);
        }
        r->idx = 0;
    }
    uint32_t y = r->mt[r->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9D2C5680u;
    y ^= (y << 15) & 0xEFC60000u;
    y ^= y >> 18;
    return y;
}

static uint32_t uniform_below(orc_mt19937 *r, uint32_t range)
{
    uint64_t prod = (uint64_t)mt_next(r) * range;
    uint32_t low = (uint32_t)prod;
    if (low < range) {
        const uint32_t thr = (0u - range) % range;
        while (low < thr) {
            prod = (uint64_t)mt_next(r) * range;
            low = (uint32_t)prod;
        }
    }
    return (uint32_t)(prod >> 32);
}

int orc_random_draws(uint32_t seed, int64_t count, uint32_t *out)
{
    if (count < 0 || count > 0xFFFFFFFFll || (count > 0 && !out)) return ORC_EINVAL;
    orc_mt19937 *rng = (orc_mt19937 *)malloc(sizeof(orc_mt19937));
    if (!rng) return ORC_ENOMEM;
    mt_seed(rng, seed);
    if (count > 0) out[0] = 0;
    for (int64_t j = count - 1; j > 0; --j) out[j] = uniform_below(rng, (uint32_t)j + 1u);
    free(rng);
    return ORC_OK;
}

static void intra_random(const uint32_t *verts, int64_t sz, uint32_t c, uint32_t *local_ids, uint32_t *tmp,
                         orc_mt19937 *rng)
{
    if (sz == 0) return;
    if (sz == 1) {
        local_ids[verts[0]] = 0;
        return;
    }
    memcpy(tmp, verts, (size_t)sz * sizeof(uint32_t));
    mt_seed(rng, 0xDEADBEEFu ^ c);
    for (int64_t j = sz - 1; j > 0; --j) {
        const uint32_t k = uniform_below(rng, (uint32_t)j + 1u);
        const uint32_t t = tmp[j];
        tmp[j] = tmp[k];
        tmp[k] = t;
    }
    for (int64_t j = 0; j < sz; ++j) local_ids[tmp[j]] = (uint32_t)j;
}

/* ------------------------------------------------------------------------ */
/* Super-graph orders of orderCompose, one thread: sg_super_rcm (RG:4990-5090 */
/* buildCommunitySuperGraph, :5726-5871 runRCMOnSuperCSR) and sg_hilbert      */
/* (:6421-6459).  Each gives stage1Perm, the tie-break of the community      */
/* order (:6460-6462).                                                        */
/* ------------------------------------------------------------------------ */

/* Bucket counts a default-constructed libstdc++ std::unordered_map goes
 * through as it grows (maximum load factor 1): the first insertion
 * allocates 13 buckets, and inserting element B + 1 into B buckets rehashes
 * to the next count.  Measured on the toolchain's own container; the tests
 * check it again (pin_umap_bucket_count in stdsort_pin.cc). */
static const int64_t kUmapBuckets[] = {13, 29, 59, 127, 257, 541, 1109, 2357, 5087, 10273, 20753, 42043, 85229,
                                       172933, 351061, 712697, 1447153, 2938679, 5967347, 12117689, 24607243,
                                       49969847, 101473717};
#define ORC_UMAP_MAX 101473717ll

/* Iteration order of a libstdc++ std::unordered_map keyed by an unsigned
 * integer (identity hash) after the k distinct keys are inserted in order
 * into an empty map.  The container keeps one singly linked list of all
 * nodes, and each bucket points at the node before its first node.  A key
 * whose bucket is empty goes to the front of the list (the bucket of the old
 * front then starts after it); otherwise it goes right after its bucket's
 * before-node.  A rehash walks the list in order and puts every node back by
 * the same two rules into the new buckets. */
int orc_umap_order(const uint32_t *keys, int64_t k, uint32_t *out)
{
    const int64_t END = -1, EMPTY = -1, BEFORE = -2;
    if (k < 0 || k > ORC_UMAP_MAX) return ORC_EINVAL;
    if (k == 0) return ORC_OK;
    int64_t bmax = 0;
    for (size_t i = 0; i < sizeof(kUmapBuckets) / sizeof(kUmapBuckets[0]); ++i)
        if (kUmapBuckets[i] >= k) { bmax = kUmapBuckets[i]; break; }
    int64_t *nxt = (int64_t *)malloc((size_t)k * sizeof(int64_t));
    int64_t *bkt = (int64_t *)malloc((size_t)bmax * sizeof(int64_t));
    if (!nxt || !bkt) { free(nxt); free(bkt); return ORC_ENOMEM; }
    int64_t head = END, B = 0;
    int gi = -1;
    for (int64_t i = 0; i < k; ++i) {
        if (i + 1 > B) {
            B = kUmapBuckets[++gi];
            for (int64_t b = 0; b < B; ++b) bkt[b] = EMPTY;
            int64_t p = head, first_bkt = 0;
            head = END;
            while (p != END) {
                const int64_t q = nxt[p];
                const int64_t b = (int64_t)(keys[p] % (uint64_t)B);
                if (bkt[b] == EMPTY) {
                    nxt[p] = head;
                    head = p;
                    bkt[b] = BEFORE;
                    if (nxt[p] != END) bkt[first_bkt] = p;
                    first_bkt = b;
                } else if (bkt[b] == BEFORE) {
                    nxt[p] = head;
                    head = p;
                } else {
                    nxt[p] = nxt[bkt[b]];
                    nxt[bkt[b]] = p;
                }
                p = q;
            }
        }
        const int64_t b = (int64_t)(keys[i] % (uint64_t)B);
        if (bkt[b] == EMPTY) {
            nxt[i] = head;
            head = i;
            if (nxt[i] != END) bkt[(int64_t)(keys[nxt[i]] % (uint64_t)B)] = i;
            bkt[b] = BEFORE;
        } else if (bkt[b] == BEFORE) {
            nxt[i] = head;
            head = i;
        } else {
            nxt[i] = nxt[bkt[b]];
            nxt[bkt[b]] = i;
        }
    }
    int64_t j = 0;
    for (int64_t p = head; p != END; p = nxt[p]) out[j++] = keys[p];
    free(nxt);
    free(bkt);
    return j == k ? ORC_OK : ORC_EINVAL;
}

/* Pair set for first occurrences of (community, neighbour community). */
static int64_t pairset_insert(uint64_t *tab, int64_t mask, uint64_t key)
{
    uint64_t h = key * 0x9E3779B97F4A7C15ull;
    int64_t i = (int64_t)(h >> 20) & mask;
    while (tab[i] != UINT64_MAX) {
        if (tab[i] == key) return 0;
        i = (i + 1) & mask;
    }
    tab[i] = key;
    return 1;
}

/* One FIFO BFS of the super-graph from root over active nodes (the
 * reference's superBFS): returns the number of levels after the root and
 * the widest level; the last level is left in last[0..*nlast). */
static void super_bfs(const int64_t *aoff, const uint32_t *adj, const int64_t *csize, uint32_t C, uint32_t root,
                      char *vis, uint32_t *cur, uint32_t *nxtl, int64_t *ecc, int64_t *maxw, uint32_t **last,
                      int64_t *nlast)
{
    memset(vis, 0, C);
    int64_t nc = 1;
    cur[0] = root;
    vis[root] = 1;
    *ecc = 0;
    *maxw = 1;
    for (;;) {
        int64_t nn = 0;
        for (int64_t i = 0; i < nc; ++i)
            for (int64_t e = aoff[cur[i]]; e < aoff[cur[i] + 1]; ++e) {
                const uint32_t d = adj[e];
                if (!vis[d] && csize[d] > 0) {
                    vis[d] = 1;
                    nxtl[nn++] = d;
                }
            }
        if (nn == 0) break;
        ++*ecc;
        if (nn > *maxw) *maxw = nn;
        uint32_t *t = cur;
        cur = nxtl;
        nxtl = t;
        nc = nn;
    }
    *last = cur;
    *nlast = nc;
}

/* stage1Perm of sg_super_rcm.  The super-graph of every community's
 * non-isolated vertices: edges[c] is the reference's map of neighbour
 * communities d >= c, filled one thread in vertex order and then copied
 * into the merged map in the per-thread map's iteration order; superAdj[c]
 * is edges[c] without c, then every c' < c with c in edges[c'] in c'
 * order.  George-Liu picks the start (up to 20 BFS from the first
 * minimum-degree node, keeping the narrowest), Cuthill-McKee runs from it
 * and then from every seed in degree order (std::sort, unstable), each node's
 * neighbours sorted by degree (std::sort) when it leaves the queue; the order
 * is reversed, and communities it did not reach follow in id order. */
static int super_rcm_perm(const orc_graph *g, const uint32_t *memb, const uint32_t *deg, const int64_t *csize,
                          uint32_t C, uint32_t *perm)
{
    const int64_t n = g->n;
    int rc = ORC_ENOMEM;
    int64_t npairs = 0, cap = 0;
    for (int64_t u = 0; u < n; ++u) if (deg[u]) cap += deg[u];
    int64_t tabsz = 64;
    while (tabsz < 2 * cap) tabsz <<= 1;
    uint64_t *tab = (uint64_t *)malloc((size_t)tabsz * sizeof(uint64_t));
    uint64_t *pairs = (uint64_t *)malloc((size_t)(cap > 0 ? cap : 1) * sizeof(uint64_t));
    int64_t *moff = (int64_t *)calloc((size_t)C + 1, sizeof(int64_t));
    uint32_t *mkeys = NULL, *ord1 = NULL, *ord2 = NULL, *adj = NULL, *cur = NULL, *nxtl = NULL, *seeds = NULL,
             *queue = NULL, *order = NULL;
    int64_t *aoff = NULL, *fill = NULL;
    uint64_t *rdeg = NULL;
    char *vis = NULL;
    if (!tab || !pairs || !moff) goto out;
    memset(tab, 0xFF, (size_t)tabsz * sizeof(uint64_t));
    for (int64_t u = 0; u < n; ++u) {
        if (!deg[u]) continue;
        const uint32_t cu = memb[u];
        for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) {
            const uint32_t cv = memb[g->col[e]];
            if (cu > cv) continue;
            const uint64_t key = ((uint64_t)cu << 32) | cv;
            if (pairset_insert(tab, tabsz - 1, key)) pairs[npairs++] = key;
        }
    }
    /* Per-map insertion sequences (stable by community). */
    mkeys = (uint32_t *)malloc((size_t)(npairs > 0 ? npairs : 1) * sizeof(uint32_t));
    ord1 = (uint32_t *)malloc((size_t)(npairs > 0 ? npairs : 1) * sizeof(uint32_t));
    ord2 = (uint32_t *)malloc((size_t)(npairs > 0 ? npairs : 1) * sizeof(uint32_t));
    fill = (int64_t *)calloc((size_t)C + 1, sizeof(int64_t));
    if (!mkeys || !ord1 || !ord2 || !fill) goto out;
    for (int64_t i = 0; i < npairs; ++i) moff[(pairs[i] >> 32) + 1]++;
    for (uint32_t c = 0; c < C; ++c) moff[c + 1] += moff[c];
    for (int64_t i = 0; i < npairs; ++i) {
        const uint32_t c = (uint32_t)(pairs[i] >> 32);
        mkeys[moff[c] + fill[c]++] = (uint32_t)pairs[i];
    }
    for (uint32_t c = 0; c < C; ++c) {
        const int64_t len = moff[c + 1] - moff[c];
        if (orc_umap_order(mkeys + moff[c], len, ord1 + moff[c]) != ORC_OK ||
            orc_umap_order(ord1 + moff[c], len, ord2 + moff[c]) != ORC_OK) {
            rc = ORC_EINVAL;
            goto out;
        }
    }
    /* superAdj. */
    aoff = (int64_t *)calloc((size_t)C + 1, sizeof(int64_t));
    if (!aoff) goto out;
    for (uint32_t c = 0; c < C; ++c)
        for (int64_t i = moff[c]; i < moff[c + 1]; ++i)
            if (ord2[i] != c) { aoff[c + 1]++; aoff[ord2[i] + 1]++; }
    for (uint32_t c = 0; c < C; ++c) aoff[c + 1] += aoff[c];
    adj = (uint32_t *)malloc((size_t)(aoff[C] > 0 ? aoff[C] : 1) * sizeof(uint32_t));
    if (!adj) goto out;
    memset(fill, 0, ((size_t)C + 1) * sizeof(int64_t));
    for (uint32_t c = 0; c < C; ++c)
        for (int64_t i = moff[c]; i < moff[c + 1]; ++i)
            if (ord2[i] != c) adj[aoff[c] + fill[c]++] = ord2[i];
    for (uint32_t c = 0; c < C; ++c)
        for (int64_t i = moff[c]; i < moff[c + 1]; ++i)
            if (ord2[i] != c) adj[aoff[ord2[i]] + fill[ord2[i]]++] = c;
    rdeg = (uint64_t *)malloc(((size_t)C + 1) * sizeof(uint64_t));
    vis = (char *)malloc((size_t)C + 1);
    cur = (uint32_t *)malloc(((size_t)C + 1) * sizeof(uint32_t));
    nxtl = (uint32_t *)malloc(((size_t)C + 1) * sizeof(uint32_t));
    seeds = (uint32_t *)malloc(((size_t)C + 1) * sizeof(uint32_t));
    queue = (uint32_t *)malloc(((size_t)C + 1) * sizeof(uint32_t));
    order = (uint32_t *)malloc(((size_t)C + 1) * sizeof(uint32_t));
    if (!rdeg || !vis || !cur || !nxtl || !seeds || !queue || !order) goto out;
    for (uint32_t c = 0; c < C; ++c) rdeg[c] = (uint64_t)(aoff[c + 1] - aoff[c]);

    /* George-Liu start. */
    int64_t first_nonempty = -1;
    uint32_t gl = 0;
    uint64_t mind = UINT64_MAX;
    for (uint32_t c = 0; c < C; ++c) {
        if (!(csize[c] > 0 && rdeg[c] > 0)) continue;
        if (first_nonempty < 0) { first_nonempty = c; gl = c; }
        if (rdeg[c] < mind) { mind = rdeg[c]; gl = c; }
    }
    uint32_t best = gl;
    if (first_nonempty >= 0 || C > 0) {
        int64_t prev_ecc = 0, best_w = INT64_MAX;
        for (int it = 0; it < 20; ++it) {
            int64_t ecc, maxw, nlast;
            uint32_t *last;
            super_bfs(aoff, adj, csize, C, gl, vis, cur, nxtl, &ecc, &maxw, &last, &nlast);
            if (maxw < best_w || (maxw == best_w && ecc > prev_ecc)) { best_w = maxw; best = gl; }
            if (ecc <= prev_ecc) break;
            prev_ecc = ecc;
            uint32_t nx = last[0];
            uint64_t nd = rdeg[last[0]];
            for (int64_t i = 1; i < nlast; ++i)
                if (rdeg[last[i]] < nd) { nd = rdeg[last[i]]; nx = last[i]; }
            gl = nx;
        }
    }
    /* Cuthill-McKee from the start, then from every seed in degree order. */
    for (uint32_t c = 0; c < C; ++c) seeds[c] = c;
    if (C > 0) ls_sort(seeds, seeds + C, rdeg);
    memset(vis, 0, C);
    int64_t norder = 0;
    for (int64_t s = -1; s < (int64_t)C; ++s) {
        const uint32_t seed = s < 0 ? best : seeds[s];
        if (C == 0 || vis[seed] || !(csize[seed] > 0)) continue;
        int64_t qh = 0, qt = 0;
        queue[qt++] = seed;
        vis[seed] = 1;
        while (qh < qt) {
            const uint32_t u = queue[qh++];
            order[norder++] = u;
            uint32_t *a = adj + aoff[u], *ae = adj + aoff[u + 1];
            if (ae > a) ls_sort(a, ae, rdeg);
            for (; a != ae; ++a)
                if (!vis[*a] && csize[*a] > 0) {
                    vis[*a] = 1;
                    queue[qt++] = *a;
                }
        }
    }
    for (uint32_t c = 0; c < C; ++c) perm[c] = UINT32_MAX;
    for (int64_t i = 0; i < norder; ++i) perm[order[norder - 1 - i]] = (uint32_t)i;
    {
        uint32_t next = (uint32_t)norder;
        for (uint32_t c = 0; c < C; ++c) if (perm[c] == UINT32_MAX) perm[c] = next++;
    }
    rc = ORC_OK;
out:
    free(tab); free(pairs); free(moff); free(mkeys); free(ord1); free(ord2); free(fill); free(aoff); free(adj);
    free(rdeg); free(vis); free(cur); free(nxtl); free(seeds); free(queue); free(order);
    return rc;
}

/* edges[c] of the super-graph with weights, one thread (RG:5033-5072): moff
 * (C + 1 offsets), the merged map's keys in iteration order (ord2) and
 * their weights.  A weight is the per-thread map's float sum of 1.0f per
 * entry, which stops growing at 2^24 (2^24 + 1 rounds back to 2^24). */
static int super_maps(const orc_graph *g, const uint32_t *memb, const uint32_t *deg, uint32_t C, int64_t **moff_out,
                      uint32_t **ord2_out, float **w_out)
{
    const int64_t n = g->n;
    int rc = ORC_ENOMEM;
    int64_t npairs = 0, cap = 0;
    for (int64_t u = 0; u < n; ++u) cap += deg[u];
    int64_t tabsz = 64;
    while (tabsz < 2 * cap) tabsz <<= 1;
    uint64_t *tab = (uint64_t *)malloc((size_t)tabsz * sizeof(uint64_t));
    int64_t *tix = (int64_t *)malloc((size_t)tabsz * sizeof(int64_t));
    uint64_t *pairs = (uint64_t *)malloc((size_t)(cap > 0 ? cap : 1) * sizeof(uint64_t));
    int64_t *cnt = (int64_t *)calloc((size_t)(cap > 0 ? cap : 1), sizeof(int64_t));
    int64_t *moff = (int64_t *)calloc((size_t)C + 1, sizeof(int64_t));
    int64_t *fill = (int64_t *)calloc((size_t)C + 1, sizeof(int64_t));
    uint32_t *mkeys = NULL, *ord1 = NULL, *ord2 = NULL;
    float *w2 = NULL;
    if (!tab || !tix || !pairs || !cnt || !moff || !fill) goto out;
    memset(tab, 0xFF, (size_t)tabsz * sizeof(uint64_t));
    for (int64_t u = 0; u < n; ++u) {
        if (!deg[u]) continue;
        const uint32_t cu = memb[u];
        for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) {
            const uint32_t cv = memb[g->col[e]];
            if (cu > cv) continue;
            const uint64_t key = ((uint64_t)cu << 32) | cv;
            int64_t i = (int64_t)((key * 0x9E3779B97F4A7C15ull) >> 20) & (tabsz - 1);
            while (tab[i] != UINT64_MAX && tab[i] != key) i = (i + 1) & (tabsz - 1);
            if (tab[i] == UINT64_MAX) {
                tab[i] = key;
                tix[i] = npairs;
                pairs[npairs++] = key;
            }
            cnt[tix[i]]++;
        }
    }
    const int64_t np1 = npairs > 0 ? npairs : 1;
    mkeys = (uint32_t *)malloc((size_t)np1 * sizeof(uint32_t));
    ord1 = (uint32_t *)malloc((size_t)np1 * sizeof(uint32_t));
    ord2 = (uint32_t *)malloc((size_t)np1 * sizeof(uint32_t));
    w2 = (float *)malloc((size_t)np1 * sizeof(float));
    if (!mkeys || !ord1 || !ord2 || !w2) goto out;
    for (int64_t i = 0; i < npairs; ++i) moff[(pairs[i] >> 32) + 1]++;
    for (uint32_t c = 0; c < C; ++c) moff[c + 1] += moff[c];
    for (int64_t i = 0; i < npairs; ++i) {
        const uint32_t c = (uint32_t)(pairs[i] >> 32);
        mkeys[moff[c] + fill[c]++] = (uint32_t)pairs[i];
    }
    for (uint32_t c = 0; c < C; ++c) {
        const int64_t len = moff[c + 1] - moff[c];
        if (orc_umap_order(mkeys + moff[c], len, ord1 + moff[c]) != ORC_OK ||
            orc_umap_order(ord1 + moff[c], len, ord2 + moff[c]) != ORC_OK) {
            rc = ORC_EINVAL;
            goto out;
        }
        for (int64_t i = moff[c]; i < moff[c + 1]; ++i) {
            const uint64_t key = ((uint64_t)c << 32) | ord2[i];
            int64_t j = (int64_t)((key * 0x9E3779B97F4A7C15ull) >> 20) & (tabsz - 1);
            while (tab[j] != key) j = (j + 1) & (tabsz - 1);
            const int64_t k = cnt[tix[j]];
            w2[i] = k >= 16777216 ? 16777216.0f : (float)k;
        }
    }
    *moff_out = moff;
    *ord2_out = ord2;
    *w_out = w2;
    moff = NULL;
    ord2 = NULL;
    w2 = NULL;
    rc = ORC_OK;
out:
    free(tab); free(tix); free(pairs); free(cnt); free(moff); free(fill); free(mkeys); free(ord1); free(ord2);
    free(w2);
    return rc;
}

typedef struct {
    uint32_t d;
    float w;
} orc_sedge;

static int u64_cmp(const void *a, const void *b)
{
    const uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : (x > y);
}

/* stage1Perm of sg_super_rabbit, one thread (RG:5495-5715 runRabbitOnSuperCSR
 * with its OpenMP loops run by one thread): RabbitOrder on the super-graph.
 * vtx[c] lists the (d, w) of every c' < c whose map holds c, by c', then c's
 * own map in iteration order; degrees are those weights summed in the same
 * order.  Communities in ascending (degree, id) unite their own and their
 * not yet aggregated children's edges (a scanner: keys in first-insertion
 * order, float sums in traversal order), then merge into the neighbour
 * root of the largest w - gamma str_u str_d / 2M (ties to the smaller id)
 * when that is > 0.  The dendrogram is walked from the roots (non-empty
 * ones first, each group by id), children chains before siblings. */
static int super_rabbit_perm(const orc_graph *g, const uint32_t *memb, const uint32_t *deg, const int64_t *csize,
                             uint32_t C, float gamma, uint32_t *perm)
{
    const uint32_t INV = UINT32_MAX;
    const float INVALID_STR = -1.0f;
    int rc = ORC_ENOMEM;
    int64_t *moff = NULL, *voff = NULL, *vlen = NULL, *vcur = NULL, *spos = NULL;
    uint32_t *ord2 = NULL, *order = NULL, *dest = NULL, *child = NULL, *sibling = NULL, *united = NULL,
             *keys = NULL, *stack = NULL;
    float *w2 = NULL, *degc = NULL, *str = NULL, *sums = NULL;
    orc_sedge *arena = NULL;
    int64_t arena_len = 0, arena_cap = 0;
    if (super_maps(g, memb, deg, C, &moff, &ord2, &w2) != ORC_OK) goto out;
    const int64_t m = moff[C];
    voff = (int64_t *)calloc((size_t)C + 1, sizeof(int64_t));
    vlen = (int64_t *)calloc((size_t)C + 1, sizeof(int64_t));
    vcur = (int64_t *)calloc((size_t)C + 1, sizeof(int64_t));
    degc = (float *)calloc((size_t)C + 1, sizeof(float));
    if (!voff || !vlen || !vcur || !degc) goto out;
    for (uint32_t c = 0; c < C; ++c)
        for (int64_t i = moff[c]; i < moff[c + 1]; ++i) {
            vlen[c]++;
            if (ord2[i] != c) vlen[ord2[i]]++;
        }
    for (uint32_t c = 0; c < C; ++c) voff[c + 1] = voff[c] + vlen[c];
    arena_cap = 2 * voff[C] + 64;
    arena = (orc_sedge *)malloc((size_t)arena_cap * sizeof(orc_sedge));
    if (!arena) goto out;
    arena_len = voff[C];
    memcpy(vcur, voff, (size_t)C * sizeof(int64_t));
    for (uint32_t c = 0; c < C; ++c)
        for (int64_t i = moff[c]; i < moff[c + 1]; ++i) {
            const uint32_t d = ord2[i];
            const float w = w2[i];
            arena[vcur[c]].d = d;
            arena[vcur[c]++].w = w;
            degc[c] += w;
            if (d != c) {
                arena[vcur[d]].d = c;
                arena[vcur[d]++].w = w;
                degc[d] += w;
            }
        }
    (void)m;
    float M = 0.0f;
    for (uint32_t c = 0; c < C; ++c) M += degc[c];
    M /= 2.0f;
    const float inv2M = M > 0.0f ? 1.0f / (2.0f * M) : 0.0f;

    order = (uint32_t *)malloc(((size_t)C + 1) * sizeof(uint32_t));
    dest = (uint32_t *)malloc(((size_t)C + 1) * sizeof(uint32_t));
    child = (uint32_t *)malloc(((size_t)C + 1) * sizeof(uint32_t));
    sibling = (uint32_t *)malloc(((size_t)C + 1) * sizeof(uint32_t));
    united = (uint32_t *)malloc(((size_t)C + 1) * sizeof(uint32_t));
    keys = (uint32_t *)malloc(((size_t)C + 1) * sizeof(uint32_t));
    const int64_t stack_cap = 2 * (int64_t)C + 2;
    stack = (uint32_t *)malloc((size_t)stack_cap * sizeof(uint32_t));
    str = (float *)malloc(((size_t)C + 1) * sizeof(float));
    sums = (float *)calloc((size_t)C + 1, sizeof(float));
    spos = (int64_t *)malloc(((size_t)C + 1) * sizeof(int64_t));
    if (!order || !dest || !child || !sibling || !united || !keys || !stack || !str || !sums || !spos) goto out;
    for (uint32_t c = 0; c < C; ++c) {
        order[c] = c;
        dest[c] = c;
        child[c] = INV;
        sibling[c] = INV;
        united[c] = INV;
        str[c] = degc[c];
        spos[c] = -1;
    }
    {
        /* ascending (degree, id): the degree's bits order like the float */
        uint64_t *k = (uint64_t *)malloc(((size_t)C + 1) * sizeof(uint64_t));
        if (!k) goto out;
        for (uint32_t c = 0; c < C; ++c) {
            uint32_t b;
            memcpy(&b, &degc[c], sizeof(b));
            k[c] = ((uint64_t)b << 32) | c;
        }
        qsort(k, C, sizeof(uint64_t), u64_cmp);
        for (uint32_t c = 0; c < C; ++c) order[c] = (uint32_t)k[c];
        free(k);
    }
    for (uint32_t i = 0; i < C; ++i) {
        const uint32_t u = order[i];
        if (degc[u] == 0.0f) continue;
        /* unite(u) */
        int64_t nk = 0;
#define ORC_SCAN_ADD(dd, ww)                                                                              \
    do {                                                                                                  \
        uint32_t r_ = (dd);                                                                               \
        while (dest[r_] != r_) r_ = dest[r_];                                                             \
        if (r_ != u) {                                                                                    \
            if (spos[r_] < 0) { spos[r_] = nk; keys[nk++] = r_; }                                         \
            sums[r_] += (ww);                                                                             \
        }                                                                                                 \
    } while (0)
        for (int64_t e = voff[u]; e < voff[u] + vlen[u]; ++e) ORC_SCAN_ADD(arena[e].d, arena[e].w);
        const uint32_t first_child = child[u], uc = united[u];
        int64_t sp = 0;
        if (first_child != uc && first_child != INV) stack[sp++] = first_child;
        while (sp > 0) {
            const uint32_t c = stack[--sp];
            if (c == uc || c == INV) continue;
            for (int64_t e = voff[c]; e < voff[c] + vlen[c]; ++e) ORC_SCAN_ADD(arena[e].d, arena[e].w);
            if (sp + 2 > stack_cap) { rc = ORC_EINVAL; goto out; }
            if (sibling[c] != uc && sibling[c] != INV) stack[sp++] = sibling[c];
            const uint32_t cf = child[c];
            if (cf != united[c] && cf != INV) stack[sp++] = cf;
            united[c] = cf;
        }
#undef ORC_SCAN_ADD
        if (arena_len + nk > arena_cap) {
            arena_cap = 2 * (arena_len + nk) + 64;
            orc_sedge *na = (orc_sedge *)realloc(arena, (size_t)arena_cap * sizeof(orc_sedge));
            if (!na) goto out;
            arena = na;
        }
        voff[u] = arena_len;
        vlen[u] = nk;
        for (int64_t j = 0; j < nk; ++j) {
            arena[arena_len + j].d = keys[j];
            arena[arena_len + j].w = sums[keys[j]];
        }
        arena_len += nk;
        united[u] = first_child;
        const float str_u = str[u];
        str[u] = INVALID_STR;
        uint32_t best = INV;
        float best_dq = 0.0f;
        const float gu = gamma * str_u;
        for (int64_t j = 0; j < nk; ++j) {
            const uint32_t d = keys[j];
            const float str_d = str[d];
            if (str_d == INVALID_STR) continue;
            const float dq = sums[d] - gu * str_d * inv2M;
            if (dq > best_dq || (dq == best_dq && (best == INV || d < best))) {
                best_dq = dq;
                best = d;
            }
        }
        for (int64_t j = 0; j < nk; ++j) {
            spos[keys[j]] = -1;
            sums[keys[j]] = 0.0f;
        }
        if (best == INV || best_dq <= 0.0f) {
            str[u] = str_u;
            continue;
        }
        sibling[u] = child[best];
        str[best] = str[best] + str_u;
        child[best] = u;
        dest[u] = best;
    }
    /* Dendrogram roots: non-empty ones by id, then empty ones by id. */
    {
        int64_t nr = 0, next = 0;
        for (int pass = 0; pass < 2; ++pass)
            for (uint32_t c = 0; c < C; ++c) {
                if (dest[c] != c) continue;
                const int empty = degc[c] == 0.0f && csize[c] == 0;
                if (empty != pass) continue;
                keys[nr++] = c;
            }
        for (uint32_t c = 0; c < C; ++c) perm[c] = INV;
        for (int64_t b = 0; b < nr; ++b) {
            int64_t sp = 0;
            for (uint32_t v = keys[b]; v != INV; v = child[v]) {
                if (sp >= stack_cap) { rc = ORC_EINVAL; goto out; }
                stack[sp++] = v;
            }
            while (sp > 0) {
                const uint32_t c = stack[--sp];
                if (perm[c] != INV) continue;
                perm[c] = (uint32_t)next++;
                if (sibling[c] != INV)
                    for (uint32_t v = sibling[c]; v != INV; v = child[v]) {
                        if (sp >= stack_cap) { rc = ORC_EINVAL; goto out; }
                        stack[sp++] = v;
                    }
            }
        }
        for (uint32_t c = 0; c < C; ++c) if (perm[c] == INV) perm[c] = (uint32_t)next++;
    }
    rc = ORC_OK;
out:
    free(moff); free(voff); free(vlen); free(vcur); free(spos); free(ord2); free(order); free(dest); free(child);
    free(sibling); free(united); free(keys); free(stack); free(w2); free(degc); free(str); free(sums); free(arena);
    return rc;
}

/* The reference's Hilbert index of (x, y) on an n x n grid (xy2d with its
 * own rotation, s - 1 - x, in 32-bit unsigned arithmetic). */
static uint64_t hilbert_xy2d(uint32_t n, uint32_t x, uint32_t y)
{
    uint64_t d = 0;
    for (uint32_t s = n / 2; s > 0; s /= 2) {
        const uint32_t rx = (x & s) > 0, ry = (y & s) > 0;
        d += (uint64_t)s * s * ((3u * rx) ^ ry);
        if (ry == 0) {
            if (rx == 1) {
                x = s - 1 - x;
                y = s - 1 - y;
            }
            const uint32_t t = x;
            x = y;
            y = t;
        }
    }
    return d;
}

typedef struct { uint64_t d; uint32_t c; } orc_hrec;

static int hrec_cmp(const void *a, const void *b)
{
    const orc_hrec *x = (const orc_hrec *)a, *y = (const orc_hrec *)b;
    if (x->d != y->d) return x->d < y->d ? -1 : 1;
    return x->c < y->c ? -1 : (x->c > y->c);
}

/* stage1Perm of sg_hilbert: communities by the Hilbert index of (size,
 * average degree), each axis scaled to [0, 255] by its maximum (at least 1). */
static int hilbert_perm(const uint32_t *deg, const uint32_t *cverts, const int64_t *cstart, const int64_t *csize,
                        uint32_t C, uint32_t *perm)
{
    uint64_t *tot = (uint64_t *)calloc((size_t)C + 1, sizeof(uint64_t));
    orc_hrec *rec = (orc_hrec *)malloc(((size_t)C + 1) * sizeof(orc_hrec));
    if (!tot || !rec) { free(tot); free(rec); return ORC_ENOMEM; }
    uint64_t max_sz = 1, max_avg = 1;
    for (uint32_t c = 0; c < C; ++c) {
        for (int64_t i = cstart[c]; i < cstart[c + 1]; ++i) tot[c] += deg[cverts[i]];
        if ((uint64_t)csize[c] > max_sz) max_sz = (uint64_t)csize[c];
        const uint64_t avg = csize[c] ? tot[c] / (uint64_t)csize[c] : 0;
        if (avg > max_avg) max_avg = avg;
    }
    for (uint32_t c = 0; c < C; ++c) {
        const uint64_t avg = csize[c] ? tot[c] / (uint64_t)csize[c] : 0;
        const uint32_t bx = (uint32_t)(((uint64_t)csize[c] * 255u) / max_sz);
        const uint32_t by = (uint32_t)((avg * 255u) / max_avg);
        rec[c].d = hilbert_xy2d(256, bx, by);
        rec[c].c = c;
    }
    qsort(rec, C, sizeof(orc_hrec), hrec_cmp);
    for (uint32_t i = 0; i < C; ++i) perm[rec[i].c] = i;
    free(tot);
    free(rec);
    return ORC_OK;
}

int orc_super_stage1(const orc_graph *g, const uint32_t *membership, int super_order, float gamma, uint32_t *out)
{
    if (!g || !membership || !out) return ORC_EINVAL;
    const int64_t n = g->n;
    uint32_t C = 0;
    for (int64_t v = 0; v < n; ++v)
        if (membership[v] + 1 > C) C = membership[v] + 1;
    int rc = ORC_ENOMEM;
    uint32_t *deg = (uint32_t *)malloc(((size_t)n + 1) * sizeof(uint32_t));
    int64_t *csize = (int64_t *)calloc((size_t)C + 1, sizeof(int64_t));
    int64_t *cstart = (int64_t *)calloc((size_t)C + 1, sizeof(int64_t));
    int64_t *cur = (int64_t *)calloc((size_t)C + 1, sizeof(int64_t));
    uint32_t *cverts = (uint32_t *)malloc(((size_t)n + 1) * sizeof(uint32_t));
    if (deg && csize && cstart && cur && cverts) {
        for (int64_t v = 0; v < n; ++v) {
            deg[v] = (uint32_t)degree_of(g, v);
            if (deg[v]) csize[membership[v]]++;
        }
        for (uint32_t c = 0; c < C; ++c) cstart[c + 1] = cstart[c] + csize[c];
        memcpy(cur, cstart, (size_t)C * sizeof(int64_t));
        for (int64_t v = 0; v < n; ++v)
            if (deg[v]) cverts[cur[membership[v]]++] = (uint32_t)v;
        if (super_order == ORC_SUPER_RCM) rc = super_rcm_perm(g, membership, deg, csize, C, out);
        else if (super_order == ORC_SUPER_RABBIT) rc = super_rabbit_perm(g, membership, deg, csize, C, gamma, out);
        else if (super_order == ORC_SUPER_HILBERT) rc = hilbert_perm(deg, cverts, cstart, csize, C, out);
        else rc = ORC_EUNSUPPORTED;
    }
    free(deg); free(csize); free(cstart); free(cur); free(cverts);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* orderCompose (RG:6286-7087), super-graph order "none".                    */
/* ------------------------------------------------------------------------ */
typedef struct { int64_t key; uint32_t c, tie; } orc_sortrec;

static int sortrec_cmp(const void *a, const void *b)
{
    /* Ascending key; equal keys keep the order the reference's
     * std::stable_sort starts from: community ids (iota), or stage1Perm's
     * order when a super-graph order is set (:6460-6462). */
    const orc_sortrec *x = (const orc_sortrec *)a, *y = (const orc_sortrec *)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->tie < y->tie ? -1 : (x->tie > y->tie);
}

int orc_compose(const orc_graph *g, const uint32_t *membership,
                const orc_compose_cfg *cfg, int32_t *new_ids,
                orc_compose_stats *stats)
{
    if (!g || !membership || !cfg || !new_ids) return ORC_EINVAL;
    orc_compose_stats local_stats;
    if (!stats) stats = &local_stats;
    memset(stats, 0, sizeof(*stats));
    const int64_t n = g->n;
    if (n == 0) return ORC_OK;
    if (cfg->intra_order == ORC_INTRA_GORDER && cfg->gorder_window <= 0) return ORC_EINVAL;
    if (cfg->intra_order != ORC_INTRA_BFS && cfg->intra_order != ORC_INTRA_RCM &&
        cfg->intra_order != ORC_INTRA_RCMPP && cfg->intra_order != ORC_INTRA_GORDER &&
        cfg->intra_order != ORC_INTRA_RANDOM && !is_sorted_intra(cfg->intra_order))
        return ORC_EUNSUPPORTED;
    if (cfg->super_order != ORC_SUPER_NONE && cfg->super_order != ORC_SUPER_RCM &&
        cfg->super_order != ORC_SUPER_HILBERT && cfg->super_order != ORC_SUPER_RABBIT)
        return ORC_EUNSUPPORTED;

    int rc = ORC_ENOMEM;
    uint32_t num_comm = 0;
    for (int64_t v = 0; v < n; ++v)
        if (membership[v] + 1 > num_comm) num_comm = membership[v] + 1;
    stats->num_communities = num_comm;

    uint32_t *deg = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
    int64_t *csize = (int64_t *)calloc((size_t)num_comm + 1, sizeof(int64_t));
    int64_t *cstart = (int64_t *)calloc((size_t)num_comm + 1, sizeof(int64_t));
    uint32_t *cverts = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
    orc_sortrec *recs = (orc_sortrec *)malloc((size_t)num_comm * sizeof(orc_sortrec));
    int64_t *offsets = (int64_t *)calloc((size_t)num_comm + 1, sizeof(int64_t));
    int64_t *v2l = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    uint32_t *local_ids = (uint32_t *)calloc((size_t)n, sizeof(uint32_t));
    uint64_t *skey = NULL;   /* sort keys of the sorted intra orders */
    uint32_t *stage1 = NULL; /* stage1Perm of a super-graph order */
    if (!deg || !csize || !cstart || !cverts || !recs || !offsets || !v2l || !local_ids)
        goto done;
    for (int64_t v = 0; v < n; ++v) deg[v] = (uint32_t)degree_of(g, v);

    /* Grouping: non-isolated vertices per community in vertex order. */
    int64_t isolated = 0;
    for (int64_t v = 0; v < n; ++v) {
        if (deg[v] == 0) ++isolated;
        else csize[membership[v]]++;
    }
    stats->isolated = isolated;
    for (uint32_t c = 0; c < num_comm; ++c) cstart[c + 1] = cstart[c] + csize[c];
    {
        int64_t *cur = (int64_t *)malloc(((size_t)num_comm + 1) * sizeof(int64_t));
        if (!cur) goto done;
        memcpy(cur, cstart, ((size_t)num_comm + 1) * sizeof(int64_t));
        for (int64_t v = 0; v < n; ++v)
            if (deg[v] != 0) cverts[cur[membership[v]]++] = (uint32_t)v;
        free(cur);
    }

    /* Super-graph order (stage1Perm), then the community order: stable sort
     * of 0..C-1 (RG:6438-6502). */
    if (cfg->super_order != ORC_SUPER_NONE) {
        stage1 = (uint32_t *)malloc(((size_t)num_comm + 1) * sizeof(uint32_t));
        if (!stage1) goto done;
        rc = cfg->super_order == ORC_SUPER_RCM
                 ? super_rcm_perm(g, membership, deg, csize, num_comm, stage1)
                 : cfg->super_order == ORC_SUPER_RABBIT
                       ? super_rabbit_perm(g, membership, deg, csize, num_comm, cfg->super_gamma, stage1)
                       : hilbert_perm(deg, cverts, cstart, csize, num_comm, stage1);
        if (rc != ORC_OK) goto done;
        rc = ORC_ENOMEM;
    }
    for (uint32_t c = 0; c < num_comm; ++c) {
        int64_t key = 0;
        int64_t tdeg = 0;
        if (cfg->community_order == ORC_COMM_DEGREE_DESC || cfg->community_order == ORC_COMM_DEGREE_ASC)
            for (int64_t i = cstart[c]; i < cstart[c + 1]; ++i) tdeg += deg[cverts[i]];
        switch (cfg->community_order) {
        case ORC_COMM_SIZE_DESC: key = -csize[c]; break;
        case ORC_COMM_SIZE_ASC: key = csize[c]; break;
        case ORC_COMM_DEGREE_DESC: key = -tdeg; break;
        case ORC_COMM_DEGREE_ASC: key = tdeg; break;
        case ORC_COMM_IDENTITY: key = 0; break;
        default: rc = ORC_EUNSUPPORTED; goto done;
        }
        recs[c].key = key;
        recs[c].c = c;
        recs[c].tie = stage1 ? stage1[c] : c;
    }
    qsort(recs, num_comm, sizeof(orc_sortrec), sortrec_cmp);
    for (uint32_t i = 0; i < num_comm; ++i) offsets[i + 1] = offsets[i] + csize[recs[i].c];

    for (int64_t v = 0; v < n; ++v) v2l[v] = -1;
    for (uint32_t c = 0; c < num_comm; ++c)
        for (int64_t i = cstart[c]; i < cstart[c + 1]; ++i) v2l[cverts[i]] = i - cstart[c];

    if (cfg->intra_order == ORC_INTRA_GORDER) {
        for (uint32_t i = 0; i < num_comm; ++i) {
            const int64_t sz = csize[recs[i].c];
            if (cfg->gorder_fallback > 0 && sz > cfg->gorder_fallback) {
                stats->fallback_communities++;
                stats->fallback_vertices += sz;
                continue;
            }
            if (sz <= 3) continue;
            stats->gorder_communities++;
            stats->gorder_vertices += sz;
            if (sz > stats->gorder_max_community) stats->gorder_max_community = sz;
        }
    }
    for (uint32_t c = 0; c < num_comm; ++c)
        if (csize[c] > stats->largest_community) stats->largest_community = csize[c];
    if (is_sorted_intra(cfg->intra_order)) {
        skey = (uint64_t *)malloc((size_t)n * sizeof(uint64_t));
        if (!skey) goto done;
        rc = sorted_intra_keys(g, membership, deg, cverts, cstart, num_comm, v2l, cfg->intra_order, skey);
        if (rc != ORC_OK) goto done;
        rc = ORC_ENOMEM;
    }

    /* Per-community intra order, one community per task as in the reference
     * (RG:6680-6962, schedule(dynamic, 1)); every task writes only its own
     * vertices' local ids. */
    {
        int failed = 0;
        const int64_t max_sz = stats->largest_community > 0 ? stats->largest_community : 1;
#ifdef _OPENMP
#pragma omp parallel if (cfg->threads != 1)
#endif
        {
            char *t_visited = (char *)malloc((size_t)max_sz);
            uint32_t *t_queue = (uint32_t *)malloc((size_t)max_sz * sizeof(uint32_t));
            uint32_t *t_la = (uint32_t *)malloc((size_t)max_sz * sizeof(uint32_t));
            uint32_t *t_lb = (uint32_t *)malloc((size_t)max_sz * sizeof(uint32_t));
            orc_pair *t_cand = (orc_pair *)malloc((size_t)max_sz * sizeof(orc_pair));
            orc_gorder_ws t_ws;
            memset(&t_ws, 0, sizeof(t_ws));
            orc_mt19937 *t_rng = (orc_mt19937 *)malloc(sizeof(orc_mt19937));
            const int ok = t_visited && t_queue && t_la && t_lb && t_cand && t_rng;
            if (!ok) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
                failed = 1;
            }
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
            for (int64_t i = 0; i < (int64_t)num_comm; ++i) {
                if (!ok) continue;
                const uint32_t c = recs[i].c;
                const uint32_t *verts = cverts + cstart[c];
                const int64_t sz = csize[c];
                if (skey) {
                    intra_sorted(verts, sz, cfg->intra_order, skey, local_ids, t_la);
                } else if (cfg->intra_order == ORC_INTRA_RANDOM) {
                    intra_random(verts, sz, c, local_ids, t_la, t_rng);
                } else if (cfg->intra_order == ORC_INTRA_RCM || cfg->intra_order == ORC_INTRA_RCMPP) {
                    if (intra_rcm(g, verts, sz, c, membership, deg, v2l, local_ids, t_visited,
                                  t_queue, t_la, t_lb, t_cand, cfg->intra_order == ORC_INTRA_RCMPP) != ORC_OK) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
                        failed = 1;
                    }
                } else if (cfg->intra_order == ORC_INTRA_GORDER &&
                           !(cfg->gorder_fallback > 0 && sz > cfg->gorder_fallback)) {
                    if (intra_gorder(g, verts, sz, c, membership, deg, v2l, cfg->gorder_window,
                                     local_ids, &t_ws) != ORC_OK) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
                        failed = 1;
                    }
                } else {
                    intra_bfs(g, verts, sz, c, membership, deg, v2l, local_ids, t_visited,
                              t_queue);
                }
            }
            free(t_visited); free(t_queue); free(t_la); free(t_lb); free(t_cand); free(t_rng);
            gorder_ws_free(&t_ws);
        }
        if (failed) goto done;
    }

    /* Final assign (RG:7003-7017). */
    for (uint32_t i = 0; i < num_comm; ++i) {
        const uint32_t c = recs[i].c;
        for (int64_t k = cstart[c]; k < cstart[c + 1]; ++k) {
            const uint32_t v = cverts[k];
            new_ids[v] = (int32_t)(offsets[i] + local_ids[v]);
        }
    }
    {
        int64_t tail = offsets[num_comm];
        for (int64_t v = 0; v < n; ++v)
            if (deg[v] == 0) new_ids[v] = (int32_t)(tail++);
    }
    rc = ORC_OK;
done:
    free(deg); free(csize); free(cstart); free(cverts); free(recs); free(offsets);
    free(v2l); free(local_ids); free(skey); free(stage1);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Validation, fingerprint, relabel, modularity.                            */
/* ------------------------------------------------------------------------ */
int orc_validate_permutation(const int32_t *ids, int64_t n)
{
    if (n == 0) return 0;
    unsigned char *seen = (unsigned char *)calloc((size_t)n, 1);
    if (!seen) return ORC_ENOMEM;
    int rc = 0;
    for (int64_t i = 0; i < n; ++i) {
        const int64_t v = ids[i];
        if (v < 0 || v >= n) { rc = 1; break; }
        if (seen[v]) { rc = 2; break; }
        seen[v] = 1;
    }
    free(seen);
    return rc;
}

uint64_t orc_fingerprint(const int32_t *ids, int64_t n)
{
    uint64_t h = UINT64_C(1469598103934665603);
    for (int64_t i = 0; i < n; ++i) {
        h ^= (uint64_t)i;
        h *= UINT64_C(1099511628211);
        h ^= (uint64_t)(int64_t)ids[i];
        h *= UINT64_C(1099511628211);
    }
    return h;
}

/* Ascending in-place sort of a row: insertion sort for short runs,
 * median-of-three quicksort (recursing into the smaller side) above that. */
static void sort_i32(int32_t *a, int64_t n)
{
    while (n > 24) {
        int32_t x = a[0], y = a[n / 2], z = a[n - 1];
        int32_t p = x < y ? (y < z ? y : (x < z ? z : x)) : (x < z ? x : (y < z ? z : y));
        int64_t i = 0, j = n - 1;
        for (;;) {
            while (a[i] < p) ++i;
            while (a[j] > p) --j;
            if (i >= j) break;
            int32_t t = a[i]; a[i] = a[j]; a[j] = t;
            ++i; --j;
        }
        /* [0, j] <= p <= [j + 1, n) */
        if (j + 1 < n - j - 1) { sort_i32(a, j + 1); a += j + 1; n -= j + 1; }
        else { sort_i32(a + j + 1, n - j - 1); n = j + 1; }
    }
    for (int64_t i = 1; i < n; ++i) {
        int32_t v = a[i];
        int64_t k = i - 1;
        while (k >= 0 && a[k] > v) { a[k + 1] = a[k]; --k; }
        a[k + 1] = v;
    }
}

int orc_relabel(const orc_graph *g, const int32_t *new_ids,
                int64_t *out_row_ptr, int32_t *out_col, int threads)
{
    const int64_t n = g->n;
    (void)threads;
    out_row_ptr[0] = 0;
    if (n == 0) return ORC_OK;
    int64_t *deg = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    if (!deg) return ORC_ENOMEM;
    for (int64_t v = 0; v < n; ++v) deg[new_ids[v]] = degree_of(g, v);
    for (int64_t v = 0; v < n; ++v) out_row_ptr[v + 1] = out_row_ptr[v] + deg[v];
    free(deg);
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1024)
#endif
    for (int64_t u = 0; u < n; ++u) {
        const int64_t base = out_row_ptr[new_ids[u]];
        int64_t k = 0;
        for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) out_col[base + k++] = new_ids[g->col[e]];
        sort_i32(out_col + base, k);
    }
    return ORC_OK;
}

double orc_modularity(const orc_graph *g, const uint32_t *membership, double resolution)
{
    const int64_t n = g->n;
    if (n == 0) return 0.0;
    const double M = (double)((g->row_ptr[n] - g->row_ptr[0]) / 2);
    if (M == 0) return 0.0;
    double Q = 0.0;
    for (int64_t u = 0; u < n; ++u) {
        const uint32_t cu = membership[u];
        const double du = (double)degree_of(g, u);
        for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) {
            const int32_t v = g->col[e];
            if (membership[v] == cu)
                Q += 1.0 - resolution * du * (double)degree_of(g, v) / (2.0 * M);
        }
    }
    return Q / (2.0 * M);
}
