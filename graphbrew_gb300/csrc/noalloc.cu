// noalloc.cu -- permutation check that allocates no device memory.
//
// Some callers of this library cannot allocate: a serving process whose GPU
// memory is reserved up front by another framework's allocator (a cudaMalloc
// there fails or steals memory the framework has promised elsewhere), or a
// latency-critical loop that cannot afford the implicit device
// synchronisation of cudaMalloc/cudaFree.  gbgpu_validate_permutation_noalloc
// gives them the builder's permutation check (same results as
// gbgpu_validate_permutation) using only the scratch array below, which lives
// in the library's own device image.
//
// The scratch is a file-scope __device__ array: every GPU that loads the
// library holds it (4 MiB) until the process exits.  Host code must not use the
// array's name as a device address; the address is obtained once per device
// with cudaGetSymbolAddress while that device is current, and passed to the
// kernels.  That lookup happens on the first call on each device (a
// one-time set-up step, not an allocation).  Every call shares the
// array and the array keeps the last call's contents: each call re-initialises
// the part it reads.  Calls whose GPU work overlaps (different streams or
// contexts on one device) race on the array and must be serialised by the
// caller.  The call reads its two-word result back and waits for its stream,
// and it leaves the caller's current device as it found it.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "gb_common.cuh"
#include "gbgpu.h"

// [0, max): smallest index holding each id; [max]: first out-of-range index;
// [max + 1]: first index repeating an earlier id.
static __device__ __align__(256) int32_t g_noalloc_scratch[GBGPU_NOALLOC_MAX_VERTICES + 2];

cudaStream_t gb_ctx_stream(gbgpu_ctx* ctx);
int gb_ctx_device(gbgpu_ctx* ctx);
void gb_ctx_set_error(gbgpu_ctx* ctx, const char* msg);

namespace {

constexpr int64_t kMax = GBGPU_NOALLOC_MAX_VERTICES;
constexpr int32_t kIntMax = 0x7FFFFFFF;
constexpr int kMaxDevices = 64;

std::mutex g_setup_mutex;
int32_t* g_scratch_ptr[kMaxDevices] = {};

// Once per device, with that device current: the device address of the scratch.
int scratch_for_current_device(int device, int32_t** out) {
    if (device < 0 || device >= kMaxDevices) return GBGPU_E_INVALID;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return GBGPU_E_CUDA;
        g_scratch_ptr[device] = static_cast<int32_t*>(p);
    }
    *out = g_scratch_ptr[device];
    return GBGPU_OK;
}

__global__ void k_na_init(int32_t* __restrict__ scratch, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        scratch[i] = kIntMax;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        scratch[kMax] = kIntMax;
        scratch[kMax + 1] = kIntMax;
    }
}

__global__ void k_na_first(const int32_t* __restrict__ ids, int64_t n, int32_t* __restrict__ scratch) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = ids[i];
        if (v < 0 || (int64_t)v >= n) atomicMin(&scratch[kMax], (int32_t)i);
        else atomicMin(&scratch[v], (int32_t)i);
    }
}

__global__ void k_na_dup(const int32_t* __restrict__ ids, int64_t n, int32_t* __restrict__ scratch) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = ids[i];
        if (v >= 0 && (int64_t)v < n && scratch[v] != (int32_t)i) atomicMin(&scratch[kMax + 1], (int32_t)i);
    }
}

}  // namespace

extern "C" int gbgpu_validate_permutation_noalloc(gbgpu_ctx* ctx, const int32_t* new_ids_dev, int64_t n,
                                                  int32_t* result) {
    if (!ctx) return GBGPU_E_INVALID;
    if (!result || n < 0 || (n > 0 && !new_ids_dev)) {
        gb_ctx_set_error(ctx, "gbgpu_validate_permutation_noalloc: null result, negative n, or null new_ids_dev");
        return GBGPU_E_INVALID;
    }
    if (n > kMax) {
        gb_ctx_set_error(ctx, ("gbgpu_validate_permutation_noalloc: n = " + std::to_string(n) +
                               " exceeds GBGPU_NOALLOC_MAX_VERTICES = " + std::to_string(kMax))
                                  .c_str());
        return GBGPU_E_OVERFLOW;
    }
    if (n == 0) {
        *result = 0;
        gb_ctx_set_error(ctx, "");
        return GBGPU_OK;
    }
    const int device = gb_ctx_device(ctx);
    if (device < 0 || device >= kMaxDevices) {
        gb_ctx_set_error(ctx, ("gbgpu_validate_permutation_noalloc: device index " + std::to_string(device) +
                               " is beyond the " + std::to_string(kMaxDevices) + " devices it supports")
                                  .c_str());
        return GBGPU_E_INVALID;
    }
    // The context's device becomes current for the launches; the caller's
    // current device is put back before returning, on every path.
    int caller_device = -1;
    cudaError_t e = cudaGetDevice(&caller_device);
    if (e == cudaSuccess && caller_device != device) e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        gb_ctx_set_error(ctx, (std::string("gbgpu_validate_permutation_noalloc: cannot make device ") +
                               std::to_string(device) + " current: " + cudaGetErrorString(e))
                                  .c_str());
        return GBGPU_E_CUDA;
    }
    struct RestoreDevice {
        int caller, own;
        ~RestoreDevice() {
            if (caller >= 0 && caller != own) cudaSetDevice(caller);
        }
    } restore{caller_device, device};
    int32_t* scratch = nullptr;
    const int rc = scratch_for_current_device(device, &scratch);
    if (rc != GBGPU_OK) {
        gb_ctx_set_error(ctx, "cudaGetSymbolAddress failed for the no-allocation scratch array");
        return rc;
    }
    cudaStream_t s = gb_ctx_stream(ctx);
    const int grid = (int)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024);
    k_na_init<<<grid, 256, 0, s>>>(scratch, n);
    k_na_first<<<grid, 256, 0, s>>>(new_ids_dev, n, scratch);
    k_na_dup<<<grid, 256, 0, s>>>(new_ids_dev, n, scratch);
    int32_t mins[2] = {kIntMax, kIntMax};
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(mins, scratch + kMax, sizeof(mins), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        gb_ctx_set_error(ctx, cudaGetErrorString(e));
        return GBGPU_E_CUDA;
    }
    if (mins[0] == kIntMax && mins[1] == kIntMax) *result = 0;
    else *result = mins[0] < mins[1] ? 1 : 2;
    gb_ctx_set_error(ctx, "");
    return GBGPU_OK;
}
