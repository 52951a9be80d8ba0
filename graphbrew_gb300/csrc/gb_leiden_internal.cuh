// gb_leiden_internal.cuh -- device helpers shared by the local-moving engines.
#pragma once

#include <vector>

#include "gb_common.cuh"

namespace gb {

constexpr int kWarpMaxDeg = 512;       // warp path up to this degree
constexpr int kWarpHash = 1024;        // per-warp shared table slots (>= 2 x kWarpMaxDeg)
constexpr int kHubThreads = 512;
constexpr int kHubSmemSlots = 16384;   // hub table in shared memory up to 8192 neighbours

__device__ __forceinline__ uint32_t hash_u32(uint32_t x) {
    return (uint32_t)(((uint64_t)x * 0x9E3779B97F4A7C15ull) >> 32);
}

// deltaModularity (:1295-1298) with the reference's association.
__device__ __forceinline__ double delta_q(double kuc, double kud, double ku, double sc, double sd, double M, double R) {
    const double a = __ddiv_rn(__dsub_rn(kuc, kud), M);
    const double t = __dadd_rn(__dsub_rn(sc, sd), ku);
    const double b = __dmul_rn(__dmul_rn(R, ku), t);
    const double den = __dmul_rn(__dmul_rn(2.0, M), M);
    return __dsub_rn(a, __ddiv_rn(b, den));
}

// (delta, id) ordering: larger delta first, then smaller id.
__device__ __forceinline__ bool better(double da, uint32_t ia, double db, uint32_t ib) {
    return da > db || (da == db && ia < ib);
}

__device__ __forceinline__ void warp_argmax(double& d, uint32_t& c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double od = __shfl_xor_sync(0xFFFFFFFFu, d, o);
        const uint32_t oc = __shfl_xor_sync(0xFFFFFFFFu, c, o);
        if (better(od, oc, d, c)) { d = od; c = oc; }
    }
}

// Shared-memory open-addressing insert (keys kNone = empty).
__device__ __forceinline__ void table_add(uint32_t* keys, uint32_t* vals, uint32_t mask, uint32_t k, uint32_t w) {
    uint32_t h = hash_u32(k) & mask;
    while (true) {
        const uint32_t prev = atomicCAS(&keys[h], kNone, k);
        if (prev == kNone || prev == k) {
            atomicAdd(&vals[h], w);
            return;
        }
        h = (h + 1) & mask;
    }
}

__device__ __forceinline__ uint32_t table_get(const uint32_t* keys, const uint32_t* vals, uint32_t mask, uint32_t k) {
    uint32_t h = hash_u32(k) & mask;
    while (true) {
        const uint32_t s = keys[h];
        if (s == k) return vals[h];
        if (s == kNone) return 0;
        h = (h + 1) & mask;
    }
}


// State shared by the asynchronous and the exact local-moving engines.
struct LocalMoveContext {
    DeviceCSR g;
    uint32_t* vcom = nullptr;
    unsigned long long* ctot = nullptr;   // int64 totals (two's complement adds)
    uint8_t* vaff = nullptr;
    const uint32_t* vcob = nullptr;       // refinement bounds: localMovingPhase<true> when set
    double M = 1.0, R = 1.0;
    std::vector<uint32_t> hubs_h;         // vertices above kWarpMaxDeg, id order
    const uint32_t* hubs = nullptr;
    int hub_grid = 1;
    uint32_t* hub_gk = nullptr;           // per-CTA global tables for very large hubs
    uint32_t* hub_gv = nullptr;
    int64_t hub_gcap = 0;
};

// Serial-order local moving (leiden_exact.cu).  Returns the iterations run.
int local_move_exact(const LocalMoveContext& ctx, double tolerance, int max_iterations, int64_t window,
                     cudaStream_t s, int64_t* launches, int64_t* rounds_out, int64_t* evals_out);

}  // namespace gb
