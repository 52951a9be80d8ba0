// stdsort_pin.cc -- TEST INFRASTRUCTURE ONLY: calls the toolchain's own
// std::sort so that the oracle's restatement of libstdc++'s introsort
// (orc_libstdcxx_sort in gb_oracle.c) can be checked element for element,
// ties included, on arbitrary inputs.  No GraphBrew source is involved.
#include <algorithm>
#include <cstdint>

extern "C" void pin_std_sort(uint32_t* elems, int64_t count, const uint64_t* key) {
    std::sort(elems, elems + count, [key](uint32_t a, uint32_t b) { return key[a] < key[b]; });
}

// std::partial_sort over the whole range runs libstdc++'s __partial_sort
// (make_heap + sort_heap): the introsort's depth-limit fallback.
extern "C" void pin_std_heap_sort(uint32_t* elems, int64_t count, const uint64_t* key) {
    std::partial_sort(elems, elems + count, elems + count,
                      [key](uint32_t a, uint32_t b) { return key[a] < key[b]; });
}
