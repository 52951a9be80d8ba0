// gapbs_gen.cpp -- the edge lists of GAPBS's synthetic graphs (`-g` / `-u`).
//
// The reference's converter and benchmarks build their synthetic inputs with
// GAPBS's generator (bench/include/external/gapbs/generator.h:101-164,
// seed kRandSeed = 27491095 from util.h:47) and then the builder symmetrizes
// and squishes them (builder.h:254-312, :463-500).  A drop-in for `-g 22`
// must hand the mapping the very same graph, or its "Mapping Fingerprint"
// cannot be compared with the reference's.  The generator's published steps:
//
//   * edges are drawn in blocks of 2^18; block b uses a 32-bit Mersenne
//     Twister (std::mt19937) seeded with kRandSeed + b, so the list does not
//     depend on how blocks are spread over threads;
//   * RMAT: for each of `scale` levels one 32-bit draw r picks a quadrant
//     against A/B/C = 0.57/0.19/0.19 of 2^32-1 (truncated to integers):
//     r < A+B keeps the source bit 0 and sets the destination bit iff r > A;
//     otherwise the source bit is 1 and the destination bit is set iff
//     r > A+B+C;
//   * RMAT ids are then relabelled by a permutation of 0..2^scale-1 shuffled
//     with std::shuffle under one std::mt19937 seeded with kRandSeed;
//   * uniform: both endpoints are draws modulo 2^scale (the generator's
//     rejection step never triggers for a power-of-two range).
//
// The Mersenne Twister and the shuffle are the C++ standard library's own, so
// the list is the reference's wherever both are compiled against the same
// standard library.  The builder's part (vertex count = largest id + 1,
// symmetrize, sort rows, drop duplicates and self-loops) is done by the
// caller on the device or on the host.
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <random>
#include <thread>
#include <vector>

#include "gbgpu.h"

namespace {

constexpr int64_t kGapbsSeed = 27491095;
constexpr int64_t kBlock = int64_t(1) << 18;

void rmat_blocks(int scale, int64_t m, int64_t b0, int64_t b1, int32_t* src, int32_t* dst) {
    const uint32_t umax = 0xFFFFFFFFu;
    const uint32_t A = (uint32_t)(0.57 * umax), B = (uint32_t)(0.19 * umax), C = (uint32_t)(0.19 * umax);
    const uint32_t ab = A + B, abc = A + B + C;
    std::mt19937 rng;
    for (int64_t b = b0; b < b1; ++b) {
        rng.seed((std::mt19937::result_type)(kGapbsSeed + b));
        const int64_t end = std::min((b + 1) * kBlock, m);
        for (int64_t e = b * kBlock; e < end; ++e) {
            uint32_t s = 0, d = 0;
            for (int level = 0; level < scale; ++level) {
                const uint32_t r = (uint32_t)rng();
                s <<= 1;
                d <<= 1;
                if (r < ab) {
                    d += r > A;
                } else {
                    s += 1;
                    d += r > abc;
                }
            }
            src[e] = (int32_t)s;
            dst[e] = (int32_t)d;
        }
    }
}

void uniform_blocks(int scale, int64_t m, int64_t b0, int64_t b1, int32_t* src, int32_t* dst) {
    const uint32_t mask = scale >= 32 ? 0xFFFFFFFFu : ((uint32_t(1) << scale) - 1);
    std::mt19937 rng;
    for (int64_t b = b0; b < b1; ++b) {
        rng.seed((std::mt19937::result_type)(kGapbsSeed + b));
        const int64_t end = std::min((b + 1) * kBlock, m);
        for (int64_t e = b * kBlock; e < end; ++e) {
            // Source first, then destination; the builder symmetrizes, so the
            // pair's order within an edge does not change the graph.
            const uint32_t s = (uint32_t)rng() & mask;
            const uint32_t d = (uint32_t)rng() & mask;
            src[e] = (int32_t)s;
            dst[e] = (int32_t)d;
        }
    }
}

template <class F>
void over_blocks(int64_t blocks, int threads, F&& f) {
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    threads = (int)std::min<int64_t>(threads, std::max<int64_t>(blocks, 1));
    std::vector<std::thread> pool;
    const int64_t per = (blocks + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        const int64_t b0 = t * per, b1 = std::min(blocks, b0 + per);
        if (b0 >= b1) break;
        pool.emplace_back([=, &f] { f(b0, b1); });
    }
    for (auto& th : pool) th.join();
}

}  // namespace

extern "C" int64_t gbgpu_gapbs_edge_count(int32_t scale, int32_t degree) {
    if (scale < 0 || scale > 30 || degree < 0) return -1;
    return (int64_t(1) << scale) * degree;
}

extern "C" int gbgpu_gapbs_edge_list(int32_t scale, int32_t degree, int32_t uniform, int32_t* src, int32_t* dst,
                                     int32_t threads) {
    const int64_t m = gbgpu_gapbs_edge_count(scale, degree);
    if (m < 0) return GBGPU_E_INVALID;
    if (m > 0 && (!src || !dst)) return GBGPU_E_INVALID;
    const int64_t blocks = (m + kBlock - 1) / kBlock;
    if (uniform) {
        over_blocks(blocks, threads, [&](int64_t b0, int64_t b1) { uniform_blocks(scale, m, b0, b1, src, dst); });
        return GBGPU_OK;
    }
    over_blocks(blocks, threads, [&](int64_t b0, int64_t b1) { rmat_blocks(scale, m, b0, b1, src, dst); });
    // PermuteIDs (generator.h:89-99): one shuffled permutation of every id.
    const int64_t n = int64_t(1) << scale;
    std::vector<int32_t> perm((size_t)n);
    std::iota(perm.begin(), perm.end(), 0);
    std::mt19937 prng((std::mt19937::result_type)kGapbsSeed);
    std::shuffle(perm.begin(), perm.end(), prng);
    over_blocks(blocks, threads, [&](int64_t b0, int64_t b1) {
        const int64_t e0 = b0 * kBlock, e1 = std::min(b1 * kBlock, m);
        for (int64_t e = e0; e < e1; ++e) {
            src[e] = perm[(size_t)src[e]];
            dst[e] = perm[(size_t)dst[e]];
        }
    });
    return GBGPU_OK;
}
