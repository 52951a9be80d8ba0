// compose_random.cu -- intra_random of orderCompose on the GPU.
//
// The reference (bench/include/graphbrew/reorder/reorder_graphbrew.h:
// 6825-6845) shuffles each community's vertex list (vertex order) by
// Fisher-Yates from the back: for j = size - 1 .. 1 it swaps entries j and
// k_j, k_j = std::uniform_int_distribution<size_t>(0, j) drawn from a
// std::mt19937 seeded with 0xDEADBEEF ^ community id; then the entry at
// position j gets local id j.  libstdc++ maps a 32-bit engine onto [0, j] by
// Lemire's nearly divisionless method ("Fast Random Integer Generation in an
// Interval", 2019): the high half of draw * (j + 1), redrawing while the low
// half is below 2^32 mod (j + 1).  The engine is MT19937 (Matsumoto and
// Nishimura, 1998) with the C++ standard's parameters and seeding recurrence.
//
// Two phases, both exact:
//
// 1. Draws.  A warp per community of two or more vertices runs its engine:
//    one lane seeds the 624 state words (a chain of dependent steps); each
//    block of 624 outputs is twisted in 20 chunks of 32 words -- a chunk
//    reads only words at or after its own, not yet rewritten, or words of
//    earlier chunks, already rewritten, which is what the sequential
//    in-place twist reads -- and then consumed 32 outputs at a time against
//    the next 32 swap positions.  A ballot finds the first rejected output:
//    the positions before it are settled, the rejected output is dropped and
//    the next chunk starts at the same position.  k_j goes to target[j] as
//    an absolute position of the skeleton.
// 2. Swaps.  A shuffle whose swap indices are known is applied in rounds of
//    deterministic reservations (Shun, Gu, Blelloch, Fineman and Gibbons,
//    "Sequential Random Permutation, List Contraction and Tree Contraction
//    are Highly Parallel", SODA 2015).  Every pending step reserves its two
//    positions with its priority, the larger position first (the loop runs
//    j downwards; positions of different communities never meet).  A step
//    that holds both reservations swaps; the others wait for the next round.
//    So a step swaps only after every earlier step on its positions has
//    swapped, and before any later one does: the result is the sequential
//    shuffle's.  Each round settles at least the first pending step of every
//    community; for random swap indices the number of rounds grows
//    logarithmically with the community size.
#include <algorithm>
#include <utility>

#include "gb_common.cuh"
#include "gb_stages.h"

namespace gb {

namespace {

constexpr int kT = 256;
constexpr int kMtN = 624;                  // MT19937 state words
constexpr int kMtM = 397;                  // middle word offset
constexpr uint32_t kMtMatrix = 0x9908B0DFu;
constexpr uint32_t kMtInit = 1812433253u;  // seeding multiplier
constexpr uint32_t kSeedBase = 0xDEADBEEFu;
constexpr int kDrawWarps = 8;

template <typename T>
T read_dev(const T* p, cudaStream_t s) {
    T h;
    GB_CUDA(cudaMemcpyAsync(&h, p, sizeof(T), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    return h;
}

__device__ __forceinline__ uint32_t mt_temper(uint32_t y) {
    y ^= y >> 11;
    y ^= (y << 7) & 0x9D2C5680u;
    y ^= (y << 15) & 0xEFC60000u;
    y ^= y >> 18;
    return y;
}

// The next 624 state words, in place, by one warp.
__device__ __forceinline__ void mt_twist(uint32_t* mt, int lane) {
    for (int b = 0; b < kMtN; b += 32) {
        const int i = b + lane;
        uint32_t nv = 0;
        if (i < kMtN) {
            const uint32_t y = (mt[i] & 0x80000000u) | (mt[i + 1 < kMtN ? i + 1 : 0] & 0x7FFFFFFFu);
            nv = mt[i + kMtM < kMtN ? i + kMtM : i + kMtM - kMtN] ^ (y >> 1) ^ ((y & 1u) ? kMtMatrix : 0u);
        }
        __syncwarp();
        if (i < kMtN) mt[i] = nv;
        __syncwarp();
    }
}

// Swap targets of every community listed (size >= 2): target[base + j] =
// base + k_j for j = size - 1 .. 1.
__global__ void __launch_bounds__(kDrawWarps * 32)
k_random_draws(const int32_t* __restrict__ list, const int32_t* __restrict__ count_p,
               const uint32_t* __restrict__ order_v, const uint32_t* __restrict__ memb,
               const int64_t* __restrict__ offs, const int64_t* __restrict__ ssize, uint32_t* __restrict__ target) {
    __shared__ uint32_t state[kDrawWarps][kMtN];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t* mt = state[w];
    const int32_t cnt = *count_p;
    for (int64_t q = (int64_t)blockIdx.x * kDrawWarps + w; q < cnt; q += (int64_t)gridDim.x * kDrawWarps) {
        const int32_t r = list[q];
        const int64_t base = offs[r];
        const int64_t sz = ssize[r];
        const uint32_t c = memb[order_v[base]];
        if (lane == 0) {
            uint32_t x = kSeedBase ^ c;
            mt[0] = x;
            for (int i = 1; i < kMtN; ++i) {
                x = kMtInit * (x ^ (x >> 30)) + (uint32_t)i;
                mt[i] = x;
            }
        }
        __syncwarp();
        int idx = kMtN;       // outputs of the current block consumed
        int64_t j = sz - 1;   // next swap position, relative to base
        while (j > 0) {
            if (idx == kMtN) {
                mt_twist(mt, lane);
                idx = 0;
            }
            const int64_t jl = j - lane;
            const bool valid = lane < kMtN - idx && jl > 0;   // a prefix of the lanes
            bool rej = false;
            uint32_t k = 0;
            if (valid) {
                const uint32_t range = (uint32_t)jl + 1u;
                const uint64_t prod = (uint64_t)mt_temper(mt[idx + lane]) * range;
                const uint32_t low = (uint32_t)prod;
                rej = low < range && low < (0u - range) % range;
                k = (uint32_t)(prod >> 32);
            }
            const unsigned vm = __ballot_sync(0xFFFFFFFFu, valid);
            const unsigned rm = __ballot_sync(0xFFFFFFFFu, rej);
            const int first = rm ? __ffs(rm) - 1 : __popc(vm);
            if (lane < first) target[base + jl] = (uint32_t)(base + k);
            idx += first + (rm ? 1 : 0);
            j -= first;
        }
        __syncwarp();   // the next community reseeds the state
    }
}

// perm = the skeleton's vertex lists; every position but a community's
// first is a pending step.
__global__ void k_random_init(const uint32_t* __restrict__ order_v, const uint32_t* __restrict__ ranks,
                              const int64_t* __restrict__ offs, int64_t nn, uint32_t* __restrict__ perm,
                              uint32_t* __restrict__ resv, uint32_t* __restrict__ pend, int* __restrict__ pend_count) {
    const int lane = threadIdx.x & 31;
    for (int64_t p0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane; p0 < nn;
         p0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = p0 + lane;
        bool step = false;
        if (p < nn) {
            perm[p] = order_v[p];
            resv[p] = 0;
            step = p != offs[ranks[p]];
        }
        const unsigned m = __ballot_sync(0xFFFFFFFFu, step);
        int at = 0;
        if (lane == 0 && m) at = atomicAdd(pend_count, __popc(m));
        at = __shfl_sync(0xFFFFFFFFu, at, 0);
        if (step) pend[at + __popc(m & ((1u << lane) - 1u))] = (uint32_t)p;
    }
}

__global__ void k_random_reserve(const uint32_t* __restrict__ pend, int64_t np, const uint32_t* __restrict__ target,
                                 uint32_t* __restrict__ resv) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t p = pend[i];
        atomicMax(&resv[p], p + 1u);
        atomicMax(&resv[target[p]], p + 1u);
    }
}

__global__ void k_random_commit(const uint32_t* __restrict__ pend, int64_t np, const uint32_t* __restrict__ target,
                                const uint32_t* __restrict__ resv, uint32_t* __restrict__ perm,
                                uint32_t* __restrict__ next, int* __restrict__ next_count) {
    const int lane = threadIdx.x & 31;
    for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane; i0 < np;
         i0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = i0 + lane;
        bool wait = false;
        uint32_t p = 0;
        if (i < np) {
            p = pend[i];
            const uint32_t t = target[p];
            if (resv[p] == p + 1u && resv[t] == p + 1u) {
                const uint32_t a = perm[p];
                perm[p] = perm[t];
                perm[t] = a;
            } else {
                wait = true;
            }
        }
        const unsigned m = __ballot_sync(0xFFFFFFFFu, wait);
        int at = 0;
        if (lane == 0 && m) at = atomicAdd(next_count, __popc(m));
        at = __shfl_sync(0xFFFFFFFFu, at, 0);
        if (wait) next[at + __popc(m & ((1u << lane) - 1u))] = p;
    }
}

__global__ void k_random_reset(const uint32_t* __restrict__ pend, int64_t np, const uint32_t* __restrict__ target,
                               uint32_t* __restrict__ resv) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t p = pend[i];
        resv[p] = 0;
        resv[target[p]] = 0;
    }
}

__global__ void k_random_local(const uint32_t* __restrict__ perm, const uint32_t* __restrict__ ranks,
                               const int64_t* __restrict__ offs, int64_t nn, uint32_t* __restrict__ local) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nn; p += (int64_t)gridDim.x * blockDim.x)
        local[perm[p]] = (uint32_t)(p - offs[ranks[p]]);
}

}  // namespace

int64_t random_communities(const uint32_t* memb, const uint32_t* order_v, const uint32_t* ranks, const int64_t* offs,
                           const int64_t* ssize, const int32_t* list, const int32_t* count_dev, int32_t count,
                           int64_t nn, uint32_t* local, cudaStream_t s, int64_t* launches) {
    if (nn == 0) return 0;
    GB_REQUIRE(nn < (int64_t)0xFFFFFFFFll, GBGPU_E_INVALID, "intra_random: too many vertices");
    DevBuf<uint32_t> target(nn, s), perm(nn, s), resv(nn, s), pend(nn, s), next(nn, s);
    DevBuf<int> counts(2, s);
    GB_CUDA(cudaMemsetAsync(counts, 0, 2 * sizeof(int), s));
    // Every step's target is written by the draws; zero keeps any position
    // in bounds all the same.
    GB_CUDA(cudaMemsetAsync(target, 0, nn * sizeof(uint32_t), s));
    int64_t nl = 0;
    if (count > 0) {
        const int grid = (int)std::min<int64_t>(ceil_div(count, kDrawWarps), (int64_t)kNumSMs * 8);
        k_random_draws<<<grid, kDrawWarps * 32, 0, s>>>(list, count_dev, order_v, memb, offs, ssize, target);
        GB_LAUNCH_CHECK();
        ++nl;
    }
    k_random_init<<<grid_for(nn, kT), kT, 0, s>>>(order_v, ranks, offs, nn, perm, resv, pend, counts.get());
    GB_LAUNCH_CHECK();
    ++nl;
    int64_t np = read_dev(counts.get(), s);
    int64_t rounds = 0;
    while (np > 0) {
        // Every round settles at least one step per community.
        GB_REQUIRE(++rounds <= nn, GBGPU_E_CUDA, "intra_random: swap rounds made no progress");
        GB_CUDA(cudaMemsetAsync(counts.get() + 1, 0, sizeof(int), s));
        const int grid = grid_for(np, kT);
        k_random_reserve<<<grid, kT, 0, s>>>(pend, np, target, resv);
        GB_LAUNCH_CHECK();
        k_random_commit<<<grid, kT, 0, s>>>(pend, np, target, resv, perm, next, counts.get() + 1);
        GB_LAUNCH_CHECK();
        k_random_reset<<<grid, kT, 0, s>>>(pend, np, target, resv);
        GB_LAUNCH_CHECK();
        nl += 3;
        np = read_dev(counts.get() + 1, s);
        std::swap(pend.ptr, next.ptr);
    }
    k_random_local<<<grid_for(nn, kT), kT, 0, s>>>(perm, ranks, offs, nn, local);
    GB_LAUNCH_CHECK();
    ++nl;
    if (launches) *launches += nl;
    return rounds;
}

}  // namespace gb
