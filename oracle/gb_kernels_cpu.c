/*
 * gb_kernels_cpu.c -- the reference's CPU benchmark kernels, restated for
 * timing the CPU side of the selector's arms.
 *
 * TEST INFRASTRUCTURE ONLY (see gb_oracle.h).  Algorithm 14 chooses between
 * arms by map + reuse x kernel time; on the reference's CPU path the kernels
 * are GAPBS's OpenMP programs.  These are OpenMP restatements of the
 * published algorithms those programs implement:
 *   - PageRank, pull direction with Gauss-Seidel updates of the outgoing
 *     contributions (bench/src/pr.cc:40-90: float scores, damping 0.85,
 *     stop when the L1 change < epsilon);
 *   - direction-optimizing BFS (Beamer, Asanovic, Patterson, SC'12; as in
 *     bench/src/bfs.cc:164-250: alpha 15, beta 18, top-down steps over a
 *     queue, bottom-up steps over a bitmap);
 *   - Afforest connected components (Sutton, Ben-Nun, Barak, IPDPS'18; as in
 *     bench/src/cc.cc:153-260: two neighbour-sampling rounds, the most
 *     frequent component of a sample skipped in the final linking);
 *   - DBG degree bucketing (bench/include/graphbrew/reorder/reorder_hub.h:
 *     267-342).
 * Each returns its wall time in milliseconds (omp_get_wtime), so the caller
 * times exactly the kernel.  Graphs are undirected CSRs (in = out neighbours).
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "gb_oracle.h"

static void set_threads(int threads) {
    if (threads > 0) omp_set_num_threads(threads);
}

double orc_pagerank_gs(const orc_graph *g, int max_iters, double epsilon, float *scores, int threads,
                       int *iters_out) {
    set_threads(threads);
    const int64_t n = g->n;
    const float damp = 0.85f;
    float *contrib = (float *)malloc((size_t)(n > 0 ? n : 1) * sizeof(float));
    if (!contrib) return -1.0;
    const double t0 = omp_get_wtime();
    const float init = n ? 1.0f / (float)n : 0.0f, base = n ? (1.0f - damp) / (float)n : 0.0f;
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < n; ++v) {
        const int64_t d = g->row_ptr[v + 1] - g->row_ptr[v];
        scores[v] = init;
        contrib[v] = d ? init / (float)d : 0.0f;
    }
    int it = 0;
    for (; it < max_iters; ++it) {
        double err = 0.0;
#pragma omp parallel for reduction(+ : err) schedule(dynamic, 16384)
        for (int64_t u = 0; u < n; ++u) {
            float in = 0.0f;
            for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) {
                float c;
                __atomic_load(&contrib[g->col[e]], &c, __ATOMIC_RELAXED);
                in += c;
            }
            const float old = scores[u];
            scores[u] = base + damp * in;
            err += fabs((double)(scores[u] - old));
            const int64_t d = g->row_ptr[u + 1] - g->row_ptr[u];
            const float c = d ? scores[u] / (float)d : 0.0f;
            __atomic_store(&contrib[u], &c, __ATOMIC_RELAXED);
        }
        if (err < epsilon) {
            ++it;
            break;
        }
    }
    const double t1 = omp_get_wtime();
    free(contrib);
    if (iters_out) *iters_out = it;
    return (t1 - t0) * 1e3;
}

/* ---- direction-optimizing BFS ---- */
static inline int bit_get(const uint64_t *b, int64_t i) { return (int)((b[i >> 6] >> (i & 63)) & 1u); }

double orc_bfs_do(const orc_graph *g, int64_t source, int32_t *depth, int threads) {
    set_threads(threads);
    const int64_t n = g->n;
    if (n == 0) return 0.0;
    const int64_t words = (n + 63) >> 6;
    uint64_t *front = (uint64_t *)calloc((size_t)words, sizeof(uint64_t));
    uint64_t *next = (uint64_t *)calloc((size_t)words, sizeof(uint64_t));
    int32_t *queue = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int32_t *nq = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    if (!front || !next || !queue || !nq) {
        free(front); free(next); free(queue); free(nq);
        return -1.0;
    }
    const double t0 = omp_get_wtime();
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < n; ++v) depth[v] = -1;
    depth[source] = 0;
    queue[0] = (int32_t)source;
    int64_t qn = 1, level = 0;
    int64_t edges_to_check = g->row_ptr[n];
    int64_t scout = g->row_ptr[source + 1] - g->row_ptr[source];
    const int alpha = 15, beta = 18;
    while (qn > 0) {
        if (scout > edges_to_check / alpha) {
            /* bottom-up steps until the frontier is small and shrinking */
            memset(front, 0, (size_t)words * sizeof(uint64_t));
            for (int64_t i = 0; i < qn; ++i) front[queue[i] >> 6] |= 1ull << (queue[i] & 63);
            int64_t awake = qn, old;
            do {
                old = awake;
                awake = 0;
                memset(next, 0, (size_t)words * sizeof(uint64_t));
#pragma omp parallel for reduction(+ : awake) schedule(dynamic, 1024)
                for (int64_t v = 0; v < n; ++v) {
                    if (depth[v] >= 0) continue;
                    for (int64_t e = g->row_ptr[v]; e < g->row_ptr[v + 1]; ++e) {
                        if (bit_get(front, g->col[e])) {
                            depth[v] = (int32_t)(level + 1);
                            __atomic_fetch_or(&next[v >> 6], 1ull << (v & 63), __ATOMIC_RELAXED);
                            ++awake;
                            break;
                        }
                    }
                }
                uint64_t *t = front;
                front = next;
                next = t;
                ++level;
            } while (awake > 0 && (awake >= old || awake > n / beta));
            /* back to a queue */
            qn = 0;
            for (int64_t v = 0; v < n; ++v)
                if (bit_get(front, v)) queue[qn++] = (int32_t)v;
            scout = 1;
        } else {
            edges_to_check -= scout;
            int64_t nn = 0, sc = 0;
#pragma omp parallel
            {
                int32_t local[256];
                int ln = 0;
                int64_t lsc = 0;
#pragma omp for schedule(dynamic, 64)
                for (int64_t i = 0; i < qn; ++i) {
                    const int32_t u = queue[i];
                    for (int64_t e = g->row_ptr[u]; e < g->row_ptr[u + 1]; ++e) {
                        const int32_t v = g->col[e];
                        int32_t expect = -1;
                        if (depth[v] < 0 &&
                            __atomic_compare_exchange_n(&depth[v], &expect, (int32_t)(level + 1), 0,
                                                        __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
                            local[ln++] = v;
                            lsc += g->row_ptr[v + 1] - g->row_ptr[v];
                            if (ln == 256) {
                                const int64_t at = __atomic_fetch_add(&nn, 256, __ATOMIC_RELAXED);
                                memcpy(nq + at, local, sizeof(local));
                                ln = 0;
                            }
                        }
                    }
                }
                const int64_t at = __atomic_fetch_add(&nn, ln, __ATOMIC_RELAXED);
                memcpy(nq + at, local, (size_t)ln * sizeof(int32_t));
                __atomic_fetch_add(&sc, lsc, __ATOMIC_RELAXED);
            }
            int32_t *t = queue;
            queue = nq;
            nq = t;
            qn = nn;
            scout = sc;
            ++level;
        }
    }
    const double t1 = omp_get_wtime();
    free(front); free(next); free(queue); free(nq);
    return (t1 - t0) * 1e3;
}

/* ---- Afforest connected components ---- */
static void cc_link(int32_t u, int32_t v, int32_t *comp) {
    int32_t p1 = __atomic_load_n(&comp[u], __ATOMIC_RELAXED), p2 = __atomic_load_n(&comp[v], __ATOMIC_RELAXED);
    while (p1 != p2) {
        const int32_t high = p1 > p2 ? p1 : p2, low = p1 + (p2 - high);
        int32_t ph = __atomic_load_n(&comp[high], __ATOMIC_RELAXED);
        if (ph == low) break;
        if (ph == high) {
            int32_t expect = high;
            if (__atomic_compare_exchange_n(&comp[high], &expect, low, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) break;
        }
        p1 = __atomic_load_n(&comp[__atomic_load_n(&comp[high], __ATOMIC_RELAXED)], __ATOMIC_RELAXED);
        p2 = __atomic_load_n(&comp[low], __ATOMIC_RELAXED);
    }
}

static void cc_compress(int64_t n, int32_t *comp) {
#pragma omp parallel for schedule(dynamic, 16384)
    for (int64_t v = 0; v < n; ++v)
        while (comp[v] != comp[comp[v]]) comp[v] = comp[comp[v]];
}

double orc_cc_afforest(const orc_graph *g, int32_t *comp, int threads) {
    set_threads(threads);
    const int64_t n = g->n;
    if (n == 0) return 0.0;
    const int rounds = 2;
    const double t0 = omp_get_wtime();
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < n; ++v) comp[v] = (int32_t)v;
    for (int r = 0; r < rounds; ++r) {
#pragma omp parallel for schedule(dynamic, 16384)
        for (int64_t u = 0; u < n; ++u)
            if (g->row_ptr[u] + r < g->row_ptr[u + 1]) cc_link((int32_t)u, g->col[g->row_ptr[u] + r], comp);
        cc_compress(n, comp);
    }
    /* The most frequent component among 1,024 sampled vertices (a fixed
     * linear congruential sequence of positions). */
    const int samples = 1024;
    int32_t *seen = (int32_t *)malloc(sizeof(int32_t) * samples);
    uint64_t x = 27491095u;
    for (int i = 0; i < samples; ++i) {
        x = x * 6364136223846793005ull + 1442695040888963407ull;
        seen[i] = comp[(x >> 33) % (uint64_t)n];
    }
    int32_t big = seen[0];
    int best = 0;
    for (int i = 0; i < samples; ++i) {
        int c = 0;
        for (int j = 0; j < samples; ++j) c += seen[j] == seen[i];
        if (c > best) { best = c; big = seen[i]; }
    }
    free(seen);
#pragma omp parallel for schedule(dynamic, 16384)
    for (int64_t u = 0; u < n; ++u) {
        if (comp[u] == big) continue;
        for (int64_t e = g->row_ptr[u] + rounds; e < g->row_ptr[u + 1]; ++e) cc_link((int32_t)u, g->col[e], comp);
    }
    cc_compress(n, comp);
    const double t1 = omp_get_wtime();
    return (t1 - t0) * 1e3;
}

/* ---- DBG: 8 degree buckets, highest first, id order inside a bucket ---- */
double orc_dbg_cpu(const orc_graph *g, int32_t *new_ids, int threads) {
    set_threads(threads);
    const int64_t n = g->n;
    if (n == 0) return 0.0;
    const double t0 = omp_get_wtime();
    const uint64_t avg = (uint64_t)g->row_ptr[n] / (uint64_t)n;
    const uint64_t th[7] = {avg / 2, avg, avg * 2, avg * 4, avg * 8, avg * 16, avg * 32};
    const int T = omp_get_max_threads();
    int64_t *cnt = (int64_t *)calloc((size_t)T * 8, sizeof(int64_t));
    uint8_t *bk = (uint8_t *)malloc((size_t)n);
#pragma omp parallel
    {
        const int t = omp_get_thread_num(), nt = omp_get_num_threads();
        const int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
        for (int64_t v = lo; v < hi; ++v) {
            const uint64_t d = (uint64_t)(g->row_ptr[v + 1] - g->row_ptr[v]);
            int b = 7;
            while (b > 0 && d <= th[b - 1]) --b;
            bk[v] = (uint8_t)b;
            cnt[t * 8 + b]++;
        }
#pragma omp barrier
#pragma omp single
        {
            int64_t run = 0;
            for (int b = 7; b >= 0; --b)
                for (int tt = 0; tt < nt; ++tt) {
                    const int64_t c = cnt[tt * 8 + b];
                    cnt[tt * 8 + b] = run;
                    run += c;
                }
        }
        for (int64_t v = lo; v < hi; ++v) new_ids[v] = (int32_t)cnt[t * 8 + bk[v]]++;
    }
    free(cnt);
    free(bk);
    const double t1 = omp_get_wtime();
    return (t1 - t0) * 1e3;
}
