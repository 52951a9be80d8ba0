// gapbs_graph.cc -- TEST INFRASTRUCTURE ONLY: the CPU side's copy of GAPBS's
// synthetic graphs, for the benchmark's CPU legs and the tests, so that they
// need neither the GPU library nor the GraphBrew sources.
//
// Edge list: bench/include/external/gapbs/generator.h:101-164 (blocks of 2^18
// edges, block b drawn by std::mt19937 seeded kRandSeed + b; RMAT quadrant
// rule on 32-bit draws against A/B/C = 0.57/0.19/0.19 of 2^32-1; RMAT ids
// relabelled by std::shuffle of 0..2^scale-1 under std::mt19937(kRandSeed);
// uniform endpoints are draws modulo 2^scale).  Graph: builder.h:160-171
// (vertex count = largest id + 1), :186-200 (degrees, both directions),
// :444-461 (fill), :254-290 (per row: sort, unique, drop self-loop).
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <numeric>
#include <random>
#include <vector>

namespace {
const int64_t kSeed = 27491095;
const int64_t kBlockEdges = int64_t(1) << 18;
std::vector<int64_t> g_rp;
std::vector<int32_t> g_col;
}  // namespace

extern "C" int64_t orc_gapbs_build(int scale, int degree, int uniform) {
    const int64_t nodes = int64_t(1) << scale, m = nodes * degree;
    std::vector<int32_t> eu((size_t)m), ev((size_t)m);
    const int64_t nblocks = (m + kBlockEdges - 1) / kBlockEdges;
    const uint32_t full = 0xFFFFFFFFu;
    const uint32_t qa = (uint32_t)(0.57 * full), qb = (uint32_t)(0.19 * full), qc = (uint32_t)(0.19 * full);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t blk = 0; blk < nblocks; ++blk) {
        std::mt19937 gen((std::mt19937::result_type)(kSeed + blk));
        for (int64_t e = blk * kBlockEdges; e < std::min(m, (blk + 1) * kBlockEdges); ++e) {
            if (uniform) {
                eu[e] = (int32_t)((uint32_t)gen() % (uint32_t)nodes);
                ev[e] = (int32_t)((uint32_t)gen() % (uint32_t)nodes);
                continue;
            }
            int64_t a = 0, b = 0;
            for (int lvl = 0; lvl < scale; ++lvl) {
                const uint32_t r = (uint32_t)gen();
                const bool lower = r >= qa + qb;
                a = 2 * a + (lower ? 1 : 0);
                b = 2 * b + (lower ? (r > qa + qb + qc ? 1 : 0) : (r > qa ? 1 : 0));
            }
            eu[e] = (int32_t)a;
            ev[e] = (int32_t)b;
        }
    }
    if (!uniform) {
        std::vector<int32_t> relabel((size_t)nodes);
        std::iota(relabel.begin(), relabel.end(), 0);
        std::mt19937 pg((std::mt19937::result_type)kSeed);
        std::shuffle(relabel.begin(), relabel.end(), pg);
#pragma omp parallel for
        for (int64_t e = 0; e < m; ++e) {
            eu[e] = relabel[eu[e]];
            ev[e] = relabel[ev[e]];
        }
    }
    int64_t n = 0;
    for (int64_t e = 0; e < m; ++e) n = std::max<int64_t>(n, std::max(eu[e], ev[e]) + 1);
    std::vector<std::atomic<int64_t>> fill((size_t)n + 1);
    for (auto& f : fill) f.store(0, std::memory_order_relaxed);
#pragma omp parallel for
    for (int64_t e = 0; e < m; ++e) {
        fill[eu[e] + 1].fetch_add(1, std::memory_order_relaxed);
        fill[ev[e] + 1].fetch_add(1, std::memory_order_relaxed);
    }
    std::vector<int64_t> start((size_t)n + 1, 0);
    for (int64_t v = 0; v < n; ++v) start[v + 1] = start[v] + fill[v + 1].load();
    for (int64_t v = 0; v <= n; ++v) fill[v].store(start[v]);
    std::vector<int32_t> raw((size_t)start[n]);
#pragma omp parallel for
    for (int64_t e = 0; e < m; ++e) {
        raw[fill[eu[e]].fetch_add(1)] = ev[e];
        raw[fill[ev[e]].fetch_add(1)] = eu[e];
    }
    std::vector<int64_t> kept((size_t)n, 0);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t v = 0; v < n; ++v) {
        int32_t* b = raw.data() + start[v];
        int32_t* e = raw.data() + start[v + 1];
        std::sort(b, e);
        e = std::unique(b, e);
        e = std::remove(b, e, (int32_t)v);
        kept[v] = e - b;
    }
    g_rp.assign((size_t)n + 1, 0);
    for (int64_t v = 0; v < n; ++v) g_rp[v + 1] = g_rp[v] + kept[v];
    g_col.assign((size_t)g_rp[n], 0);
#pragma omp parallel for
    for (int64_t v = 0; v < n; ++v)
        std::copy(raw.data() + start[v], raw.data() + start[v] + kept[v], g_col.data() + g_rp[v]);
    return n;
}

extern "C" int64_t orc_gapbs_nnz(void) { return g_rp.empty() ? 0 : g_rp.back(); }

extern "C" void orc_gapbs_copy(int64_t* rp, int32_t* col) {
    std::copy(g_rp.begin(), g_rp.end(), rp);
    std::copy(g_col.begin(), g_col.end(), col);
    g_rp.clear();
    g_rp.shrink_to_fit();
    g_col.clear();
    g_col.shrink_to_fit();
}
