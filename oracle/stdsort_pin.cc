// stdsort_pin.cc -- TEST INFRASTRUCTURE ONLY: calls the toolchain's own
// std::sort so that the oracle's restatement of libstdc++'s introsort
// (orc_libstdcxx_sort in gb_oracle.c) can be checked element for element,
// ties included, on arbitrary inputs; and the toolchain's std::mt19937 with
// std::uniform_int_distribution<size_t>, which pin the oracle's restatement
// behind intra_random (orc_random_draws).  No GraphBrew source is involved.
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <random>
#include <unordered_map>

extern "C" void pin_std_sort(uint32_t* elems, int64_t count, const uint64_t* key) {
    std::sort(elems, elems + count, [key](uint32_t a, uint32_t b) { return key[a] < key[b]; });
}

// std::partial_sort over the whole range runs libstdc++'s __partial_sort
// (make_heap + sort_heap): the introsort's depth-limit fallback.
extern "C" void pin_std_heap_sort(uint32_t* elems, int64_t count, const uint64_t* key) {
    std::partial_sort(elems, elems + count, elems + count,
                      [key](uint32_t a, uint32_t b) { return key[a] < key[b]; });
}

// The swap indices of a Fisher-Yates shuffle of `count` elements from the
// back: out[j] = uniform_int_distribution<size_t>(0, j)(engine) for
// j = count - 1 .. 1, in that order; out[0] = 0.
extern "C" void pin_std_shuffle_draws(uint32_t seed, int64_t count, uint32_t* out) {
    std::mt19937 rng(seed);
    if (count > 0) out[0] = 0;
    for (int64_t j = count - 1; j > 0; --j) {
        std::uniform_int_distribution<std::size_t> dist(0, (std::size_t)j);
        out[j] = (uint32_t)dist(rng);
    }
}

// Iteration order of std::unordered_map<uint32_t, float> after the keys are
// inserted in order with operator[] (distinct keys: out gets all of them).
extern "C" void pin_umap_order(const uint32_t* keys, int64_t count, uint32_t* out) {
    std::unordered_map<uint32_t, float> m;
    for (int64_t i = 0; i < count; ++i) m[keys[i]] += 1.0f;
    int64_t j = 0;
    for (const auto& kv : m) out[j++] = kv.first;
}

// bucket_count() after `count` distinct insertions into an empty map.
extern "C" int64_t pin_umap_bucket_count(int64_t count) {
    std::unordered_map<uint32_t, float> m;
    for (int64_t i = 0; i < count; ++i) m[(uint32_t)i] += 1.0f;
    return (int64_t)m.bucket_count();
}
