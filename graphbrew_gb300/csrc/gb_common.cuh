// gb_common.cuh -- shared device/host helpers for the GB300 mapping library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "gbgpu.h"

namespace gb {

// Status-carrying exception used inside the library; the C ABI converts it
// back to a gbgpu_status and a message (gbgpu_last_error).
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& msg) : std::runtime_error(msg), status(s) {}
};

#define GB_CUDA(expr)                                                                  \
    do {                                                                               \
        cudaError_t gb_err_ = (expr);                                                  \
        if (gb_err_ != cudaSuccess) {                                                  \
            throw ::gb::Error(GBGPU_E_CUDA, std::string(#expr) + ": " +                \
                                                cudaGetErrorString(gb_err_));          \
        }                                                                              \
    } while (0)

#define GB_LAUNCH_CHECK() GB_CUDA(cudaGetLastError())

#define GB_REQUIRE(cond, status, msg)                                                  \
    do {                                                                               \
        if (!(cond)) throw ::gb::Error((status), (msg));                               \
    } while (0)

constexpr int kNumSMs = 152;        // GB300: 2 dies x 76 SMs
constexpr uint32_t kNone = 0xFFFFFFFFu;

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Grid size for a grid-stride loop over `work` items with `threads` per block.
inline int grid_for(int64_t work, int threads, int blocks_per_sm = 8) {
    int64_t b = ceil_div(work > 0 ? work : 1, threads);
    int64_t cap = (int64_t)kNumSMs * blocks_per_sm * 4;
    return (int)(b < cap ? b : cap);
}

// Stream-ordered device buffer drawn from the context's memory pool
// (cudaMallocAsync).  Freed on the same stream when it goes out of scope.
template <typename T>
struct DevBuf {
    T* ptr = nullptr;
    size_t count = 0;
    cudaStream_t stream = nullptr;
    DevBuf() = default;
    DevBuf(size_t n, cudaStream_t s) { alloc(n, s); }
    void alloc(size_t n, cudaStream_t s) {
        release();
        stream = s;
        count = n;
        if (n) GB_CUDA(cudaMallocAsync((void**)&ptr, n * sizeof(T), s));
    }
    void release() {
        if (ptr) cudaFreeAsync(ptr, stream);
        ptr = nullptr;
        count = 0;
    }
    ~DevBuf() { release(); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : ptr(o.ptr), count(o.count), stream(o.stream) { o.ptr = nullptr; o.count = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) { release(); ptr = o.ptr; count = o.count; stream = o.stream; o.ptr = nullptr; o.count = 0; }
        return *this;
    }
    T* get() const { return ptr; }
    operator T*() const { return ptr; }
};

#ifdef __CUDACC__
// Warp-aggregated atomics on arrays indexed by a key (a community id): lanes
// holding the same key combine their values and the lowest such lane issues
// the one atomic.  All 32 lanes of the warp call; a lane with nothing to add
// passes active = false.
__device__ __forceinline__ unsigned warp_key_peers(uint32_t key, bool active, bool* leader) {
    const unsigned act = __ballot_sync(0xFFFFFFFFu, active);
    if (!active) return 0u;
    const unsigned peers = __match_any_sync(act, key);
    *leader = (int)(threadIdx.x & 31) == __ffs(peers) - 1;
    return peers;
}

__device__ __forceinline__ void warp_add_u32(uint32_t* arr, uint32_t key, uint32_t val, bool active) {
    bool leader = false;
    const unsigned peers = warp_key_peers(key, active, &leader);
    if (!active) return;
    const uint32_t sum = __reduce_add_sync(peers, val);
    if (leader) atomicAdd(&arr[key], sum);
}

// Values below 2^32 each (degrees): summed in 16-bit halves so that 32 of
// them cannot overflow the 32-bit warp reduction.
__device__ __forceinline__ void warp_add_u64(unsigned long long* arr, uint32_t key, unsigned long long val,
                                             bool active) {
    bool leader = false;
    const unsigned peers = warp_key_peers(key, active, &leader);
    if (!active) return;
    const uint32_t lo = __reduce_add_sync(peers, (uint32_t)(val & 0xFFFFull));
    const uint32_t hi = __reduce_add_sync(peers, (uint32_t)(val >> 16));
    if (leader) atomicAdd(&arr[key], ((unsigned long long)hi << 16) + lo);
}

// Minimum of values that increase with the lane (vertex ids of a warp-aligned
// range): the leader's own value.
__device__ __forceinline__ void warp_min_ordered_i32(int32_t* arr, uint32_t key, int32_t val, bool active) {
    bool leader = false;
    warp_key_peers(key, active, &leader);
    if (leader) atomicMin(&arr[key], val);
}
#endif  // __CUDACC__

// Read-only view of an undirected CSR graph resident in HBM.
struct DeviceCSR {
    int64_t n = 0;
    int64_t nnz = 0;
    const int64_t* row_ptr = nullptr;
    const int32_t* col = nullptr;
};

// -------------------------------------------------------------------------
// Primitives (primitives.cu)
// -------------------------------------------------------------------------

// Exclusive prefix sum of n int64 values; out may alias in.  Returns nothing;
// out[n] is NOT written (callers size their own totals).
void exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n, cudaStream_t s);
// Same, also writing the grand total to *total_dev (device pointer).
void exclusive_scan_i64_total(const int64_t* in, int64_t* out, int64_t n, int64_t* total_dev,
                              cudaStream_t s);
// Exclusive prefix sum of n int32 flags/counts into int64 offsets, and the
// total into *total_dev (device pointer, may be null).
void exclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, int64_t n, int64_t* total_dev,
                               cudaStream_t s);
void exclusive_scan_u8_to_i64(const uint8_t* in, int64_t* out, int64_t n, int64_t* total_dev, cudaStream_t s);

// Stable LSD radix sort of (key, value) pairs by the low `key_bits` bits of
// the key.  keys/values are sorted in place (double-buffered through scratch).
void radix_sort_pairs_u32(uint32_t* keys, uint32_t* values, int64_t n, int key_bits, cudaStream_t s);
void radix_sort_pairs_u64(uint64_t* keys, uint32_t* values, int64_t n, int key_bits, cudaStream_t s);
// Stable LSD radix sort of 64-bit keys alone.
void radix_sort_keys_u64(uint64_t* keys, int64_t n, int key_bits, cudaStream_t s);

// Fill helpers.
void fill_u32(uint32_t* p, uint32_t v, int64_t n, cudaStream_t s);
void fill_i64(int64_t* p, int64_t v, int64_t n, cudaStream_t s);
void iota_u32(uint32_t* p, int64_t n, cudaStream_t s);

// Degree of every vertex (int64) from row_ptr.
void degrees_i64(const int64_t* row_ptr, int64_t* deg, int64_t n, cudaStream_t s);

inline int bits_for(uint64_t max_value) {
    int b = 0;
    while (b < 64 && (max_value >> b) != 0) ++b;
    return b;
}

}  // namespace gb
