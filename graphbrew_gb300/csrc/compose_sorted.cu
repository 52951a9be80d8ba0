// compose_sorted.cu -- the sorted intra-community orders of orderCompose on the GPU.
//
// HubSort, DegreeAsc, Hub2, Alternate, BoundaryLast and CoreOrder
// (bench/include/graphbrew/reorder/reorder_graphbrew.h:6759-6955) each
// std::sort a community's vertices (vertex order to start with) by a
// per-vertex comparator.  std::sort is not stable: ties end where the
// standard library's introsort leaves them, and the reference is built
// against libstdc++.  So that the permutation is the reference's bit for
// bit, this file runs libstdc++'s introsort itself (bits/stl_algo.h
// __introsort_loop / __unguarded_partition_pivot / __final_insertion_sort,
// bits/stl_heap.h for the depth-limit fallback), restated for the GPU:
//
// * every community is one segment of the placement skeleton; all segments
//   of all communities advance one partition level per step;
// * a partition step is the unguarded Hoare partition around the
//   median-of-three pivot moved to the segment's front.  Its swaps pair the
//   k-th element >= pivot from the left with the k-th element <= pivot from
//   the right while the former lies left of the latter, so two prefix sums
//   (one from each side) give every swap and the cut without a sequential
//   scan;
// * both halves continue with the depth limit less one; segments of at most
//   16 elements stop and get libstdc++'s final insertion sort (stable inside
//   each segment, since no element crosses a partition boundary); a segment
//   whose depth limit runs out is heap-sorted by one thread with libstdc++'s
//   make_heap / sort_heap, exactly (rare: adversarial key patterns only).
//
// Each comparator is one 64-bit key, comp(a, b) = key(a) < key(b):
//   HubSort, Alternate   ~deg (32 bits)            DegreeAsc   deg
//   Hub2                 ~(sum of neighbour degrees)
//   BoundaryLast         external degree, then ~deg
//   CoreOrder            ~core number (community-induced), then ~deg
// Core numbers come from a level-synchronous peel of every community at
// once; they are unique, so they equal the reference's bucket peel.
#include <algorithm>
#include <climits>

#include "gb_chunks.cuh"
#include "gb_common.cuh"
#include "gb_stages.h"

namespace gb {

namespace {

constexpr int kT = 256;
constexpr int kFinalMax = 16;          // libstdc++ _S_threshold
constexpr uint32_t kCoreUnset = 0xFFFFFFFFu;

enum SortedOrder { kHubSort = 6, kDegreeAsc = 7, kHub2 = 8, kAlternate = 9, kBoundaryLast = 11, kCore = 12 };

__device__ __forceinline__ uint32_t degree(const int64_t* rp, uint32_t v) { return (uint32_t)(rp[v + 1] - rp[v]); }

template <typename T>
T read_dev(const T* p, cudaStream_t s) {
    T h;
    GB_CUDA(cudaMemcpyAsync(&h, p, sizeof(T), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    return h;
}

// Per-vertex neighbour sums, entry-parallel: mode 0 sum of neighbour degrees
// (u64), 1 neighbours in another community, 2 neighbours in the same
// community (u32, self loops included).
constexpr int kSumThreads = 256;

__global__ void __launch_bounds__(kSumThreads)
k_neighbour_sums(const int64_t* __restrict__ rp, const int32_t* __restrict__ col, const uint32_t* __restrict__ memb,
                 int64_t n, int64_t nnz, const int32_t* __restrict__ chunk_row, int mode,
                 unsigned long long* __restrict__ out64, uint32_t* __restrict__ out32) {
    constexpr int kPer = kEdgeChunk / kSumThreads;
    __shared__ int32_t srow[kEdgeChunkPadded];
    __shared__ int32_t wmax[kSumThreads / 32];
    const int64_t chunks = (nnz + kEdgeChunk - 1) / kEdgeChunk;
    for (int64_t c = blockIdx.x; c < chunks; c += gridDim.x) {
        const int64_t e0 = c * kEdgeChunk, e1 = min(nnz, e0 + kEdgeChunk);
        chunk_entry_rows<kSumThreads>(rp, n, chunk_row[c], e0, e1, srow, wmax);
#pragma unroll 4
        for (int k = 0; k < kPer; ++k) {
            const int i = k * kSumThreads + threadIdx.x;
            const bool in = e0 + i < e1;
            const uint32_t u = in ? (uint32_t)srow[chunk_pad(i)] : 0u;
            const uint32_t v = in ? (uint32_t)col[e0 + i] : 0u;
            if (mode == 0) {
                warp_add_u64(out64, u, in ? (unsigned long long)degree(rp, v) : 0ull, in);
            } else {
                const bool same = in && memb[v] == memb[u];
                const bool hit = in && (mode == 1 ? !same : same);
                warp_add_u32(out32, u, 1u, hit);
            }
        }
        __syncthreads();
    }
}

// ---- core numbers: level-synchronous peel of all communities ----
__global__ void k_core_init(const uint32_t* __restrict__ order_v, int64_t nn, const uint32_t* __restrict__ intdeg,
                            uint32_t* __restrict__ cd, uint32_t* __restrict__ core) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nn; p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t v = order_v[p];
        cd[v] = intdeg[v];
        core[v] = kCoreUnset;
    }
}

// The peel's control block.  A level k starts with a scan for the unpeeled
// vertices whose remaining degree is <= k (the first frontier); peeling a
// frontier appends every neighbour whose remaining degree falls from k + 1 to
// k to the next frontier, so a level scans the vertices once and then touches
// only its frontiers.  When a level's frontiers run out, level k + 1 starts
// with a scan; a scan that finds nothing moves to the smallest remaining
// degree, which the same scan found.  A scan reads only the vertices that
// were unpeeled at the previous scan and writes out those it leaves.  A step
// is two kernels (scan, apply); the apply's last CTA ends the step.
//
// A frontier is three lists by row length, so that no row holds one warp for
// long: rows up to kCoreWarpMax entries get a warp, rows up to kCoreCtaMax a
// CTA, longer rows every warp of the grid.
constexpr int64_t kCoreWarpMax = 512;
constexpr int64_t kCoreCtaMax = 8192;

struct CoreCtl {
    uint32_t k;        // level
    uint32_t next;     // smallest remaining degree above k (an empty scan's next level)
    uint32_t cnt[3];   // vertices in the current frontier, per tier
    uint32_t ncnt[3];  // vertices appended to the next frontier, per tier
    long long left;    // vertices not yet peeled
    long long steps;   // steps run
    long long max_steps;  // bound on steps (each one peels a vertex or raises the level)
    int scan;          // this step starts level k with a scan
    int par;           // the current frontier's buffers
    int done;
    int error;
    unsigned arrive;   // apply CTAs finished in this step
    unsigned rcount;   // vertices in the current remaining list
    unsigned rnext;    // vertices the scan wrote to the next remaining list
    int rpar;          // the current remaining list's buffer
};

// Frontier buffers: f[buffer][tier], each n entries.
struct CoreFronts {
    uint32_t* f[2][3];
};

__device__ __forceinline__ int core_tier(const int64_t* __restrict__ rp, uint32_t v) {
    const int64_t d = rp[v + 1] - rp[v];
    return d <= kCoreWarpMax ? 0 : (d <= kCoreCtaMax ? 1 : 2);
}

// Scan of level k: unpeeled vertices whose remaining degree is <= k form the
// first frontier; the others go to the next remaining list (one atomic per
// CTA for warp-tier rows and survivors, one per vertex for longer rows), and
// their smallest remaining degree is the next level if no vertex is taken
// (one atomicMin per CTA).
__global__ void __launch_bounds__(kT)
k_core_scan(uint32_t* rem0, uint32_t* rem1, const int64_t* __restrict__ rp, const uint32_t* __restrict__ cd,
            const uint32_t* __restrict__ core, CoreFronts fr, CoreCtl* __restrict__ ctl) {
    __shared__ unsigned wsum[kT / 32], wkeep[kT / 32];
    __shared__ unsigned wmin[kT / 32];
    __shared__ unsigned base, kbase;
    if (ctl->done || !ctl->scan) return;
    const uint32_t k = ctl->k;
    const int64_t nr = ctl->rcount;
    const int par = ctl->par;
    const uint32_t* rem = ctl->rpar ? rem1 : rem0;
    uint32_t* rnext = ctl->rpar ? rem0 : rem1;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned m = 0xFFFFFFFFu;
    for (int64_t p0 = (int64_t)blockIdx.x * kT; p0 < nr; p0 += (int64_t)gridDim.x * kT) {
        const int64_t p = p0 + threadIdx.x;
        uint32_t v = 0;
        bool take = false, keep = false;
        if (p < nr) {
            v = rem[p];
            if (core[v] == kCoreUnset) {
                const uint32_t d = cd[v];
                take = d <= k;
                keep = !take;
                if (keep) m = min(m, d);
            }
        }
        if (take) {
            const int t = core_tier(rp, v);
            if (t > 0) {
                fr.f[par][t][atomicAdd(&ctl->cnt[t], 1u)] = v;   // long rows: few, one atomic each
                take = false;
            }
        }
        const unsigned b = __ballot_sync(0xFFFFFFFFu, take);
        const unsigned kb = __ballot_sync(0xFFFFFFFFu, keep);
        if (lane == 0) {
            wsum[w] = (unsigned)__popc(b);
            wkeep[w] = (unsigned)__popc(kb);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned t = 0, tk = 0;
            for (int q = 0; q < kT / 32; ++q) {
                t += wsum[q];
                tk += wkeep[q];
            }
            base = t ? atomicAdd(&ctl->cnt[0], t) : 0u;
            kbase = tk ? atomicAdd(&ctl->rnext, tk) : 0u;
        }
        __syncthreads();
        unsigned o = base, ok = kbase;
        for (int q = 0; q < w; ++q) {
            o += wsum[q];
            ok += wkeep[q];
        }
        if (take) fr.f[par][0][o + __popc(b & ((1u << lane) - 1u))] = v;
        if (keep) rnext[ok + __popc(kb & ((1u << lane) - 1u))] = v;
        __syncthreads();
    }
    m = __reduce_min_sync(0xFFFFFFFFu, m);
    if (lane == 0) wmin[w] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 0; q < kT / 32; ++q) m = min(m, wmin[q]);
        if (m != 0xFFFFFFFFu) atomicMin(&ctl->next, m);
    }
}

// End of a step (the last apply CTA, after every other CTA's updates).
__device__ void core_step_end(volatile CoreCtl* c) {
    const unsigned peeled = c->cnt[0] + c->cnt[1] + c->cnt[2];
    const unsigned appended = c->ncnt[0] + c->ncnt[1] + c->ncnt[2];
    if (c->scan) {
        c->rcount = c->rnext;   // the scan's survivors are the remaining list
        c->rnext = 0;
        c->rpar = c->rpar ^ 1;
    }
    bool clear = true;
    if (c->scan && peeled == 0) {
        // Nothing at level k: go to the smallest remaining degree.
        if (c->next == 0xFFFFFFFFu || c->next <= c->k) {
            c->error = 1;   // unpeeled vertices but no level to go to
            c->done = 1;
        } else {
            c->k = c->next;
        }
    } else {
        c->left = c->left - peeled;
        if (c->left <= 0) {
            c->done = 1;
        } else if (appended > 0) {
            c->par = c->par ^ 1;    // the appended vertices are the next frontier
            for (int t = 0; t < 3; ++t) c->cnt[t] = c->ncnt[t];
            c->scan = 0;
            clear = false;
        } else {
            c->k = c->k + 1;        // level k is peeled: scan level k + 1
            c->scan = 1;
        }
    }
    for (int t = 0; t < 3; ++t) {
        if (clear) c->cnt[t] = 0;
        c->ncnt[t] = 0;
    }
    c->next = 0xFFFFFFFFu;
    c->steps = c->steps + 1;
    if (c->steps >= c->max_steps && !c->done) {
        c->error = 1;   // the bound only guards against a broken invariant
        c->done = 1;
    }
}

// Removing peeled vertex v at level k: its unpeeled neighbours in the
// community lose one (a neighbour in the same frontier may lose one too; it
// is peeled at k all the same).  The one decrement that takes a neighbour
// from k + 1 to k appends it to the next frontier.  Edges [e_begin, e_end)
// of v's row, e_begin warp-uniform, in steps of `stride` per warp.
__device__ __forceinline__ void core_remove(uint32_t v, int64_t e_begin, int64_t e_end, int64_t stride, uint32_t k,
                                            const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                            const uint32_t* __restrict__ memb, const uint32_t* core,
                                            uint32_t* __restrict__ cd, const CoreFronts& fr, int npar,
                                            CoreCtl* __restrict__ ctl) {
    const int lane = threadIdx.x & 31;
    const uint32_t c = memb[v];
    for (int64_t e0 = e_begin; e0 < e_end; e0 += stride) {
        const int64_t e = e0 + lane;
        uint32_t u = 0;
        bool push = false;
        if (e < e_end) {
            u = (uint32_t)col[e];
            if (u != v && memb[u] == c && core[u] == kCoreUnset) push = atomicSub(&cd[u], 1u) == k + 1u;
        }
        if (push) {
            const int t = core_tier(rp, u);
            if (t > 0) {
                fr.f[npar][t][atomicAdd(&ctl->ncnt[t], 1u)] = u;   // long rows: few, one atomic each
                push = false;
            }
        }
        const unsigned b = __ballot_sync(0xFFFFFFFFu, push);
        if (b) {
            unsigned base = 0;
            if (lane == 0) base = atomicAdd(&ctl->ncnt[0], (unsigned)__popc(b));
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (push) fr.f[npar][0][base + __popc(b & ((1u << lane) - 1u))] = u;
        }
    }
}

// Peels the frontier: a warp per warp-tier vertex, a CTA per CTA-tier
// vertex, every warp of the grid on each longer row.  The last CTA to
// finish ends the step and sets the peel loop's condition (the graph's while
// node); no CTA waits for another.
__global__ void __launch_bounds__(kT)
k_core_apply(CoreFronts fr, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
             const uint32_t* __restrict__ memb, uint32_t* __restrict__ core, uint32_t* __restrict__ cd,
             CoreCtl* __restrict__ ctl, cudaGraphConditionalHandle cond) {
    __shared__ bool s_last;
    const uint32_t c0 = ctl->cnt[0], c1 = ctl->cnt[1], c2 = ctl->cnt[2];
    const bool active = !ctl->done && !(ctl->scan && c0 + c1 + c2 == 0);
    if (active) {
        const uint32_t k = ctl->k;
        const int par = ctl->par, npar = par ^ 1;
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
        const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
        for (int64_t i = gw; i < (int64_t)c0; i += nw) {
            const uint32_t v = fr.f[par][0][i];
            if (lane == 0) core[v] = k;
            core_remove(v, rp[v], rp[v + 1], 32, k, rp, col, memb, core, cd, fr, npar, ctl);
        }
        for (int64_t i = blockIdx.x; i < (int64_t)c1; i += gridDim.x) {
            const uint32_t v = fr.f[par][1][i];
            if (threadIdx.x == 0) core[v] = k;
            core_remove(v, rp[v] + w * 32, rp[v + 1], kT, k, rp, col, memb, core, cd, fr, npar, ctl);
        }
        for (uint32_t j = 0; j < c2; ++j) {
            const uint32_t v = fr.f[par][2][j];
            if (gw == 0 && lane == 0) core[v] = k;
            core_remove(v, rp[v] + gw * 32, rp[v + 1], nw * 32, k, rp, col, memb, core, cd, fr, npar, ctl);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&ctl->arrive, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        __threadfence();
        volatile CoreCtl* c = ctl;
        if (!c->done) core_step_end(c);
        c->arrive = 0;
        cudaGraphSetConditional(cond, c->done ? 0u : 1u);
    }
}


// ---- keys and segments ----
__global__ void k_sorted_keys(const uint32_t* __restrict__ order_v, int64_t nn, const int64_t* __restrict__ rp,
                              int order, const unsigned long long* __restrict__ score,
                              const uint32_t* __restrict__ aux, uint32_t* __restrict__ E, uint64_t* __restrict__ Kv) {
    const uint64_t m32 = 0xFFFFFFFFull;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nn; p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t v = order_v[p];
        const uint64_t d = degree(rp, v);
        uint64_t key;
        switch (order) {
            case kDegreeAsc: key = d; break;
            case kHub2: key = ~(uint64_t)score[v]; break;
            case kBoundaryLast: key = ((uint64_t)aux[v] << 32) | (m32 - d); break;
            case kCore: key = ((m32 - aux[v]) << 32) | (m32 - d); break;
            default: key = m32 - d; break;   // HubSort, Alternate
        }
        E[p] = v;
        Kv[p] = key;
    }
}

struct Segs {
    uint32_t* E;          // element (vertex) at each position
    uint64_t* K;          // its key
    int32_t* S;           // start of the segment holding each position
    int32_t* end;         // per head: one past the segment's last position
    int32_t* depth;       // per head: remaining depth limit
    uint8_t* act;         // per head: 1 partition this level, 2 heap sort, 0 final
    uint64_t* piv;        // per head: pivot key of this level
    int32_t* kcnt;        // per head: swaps of this level
    int32_t* cut;         // per head: cut of this level
    int32_t* ge;          // per position: >= pivot (left stops)
    int32_t* le;          // per position: <= pivot (right stops)
    int64_t* PG;          // exclusive prefix of ge (nn + 1)
    int64_t* PL;          // exclusive prefix of le (nn + 1)
    int32_t* L;           // per segment: left stops in order
    int32_t* R;           // per segment: right stops, right to left
    int64_t nn;
};

__device__ __forceinline__ void swap_at(const Segs& s, int64_t a, int64_t b) {
    const uint32_t e = s.E[a];
    s.E[a] = s.E[b];
    s.E[b] = e;
    const uint64_t k = s.K[a];
    s.K[a] = s.K[b];
    s.K[b] = k;
}

__global__ void k_seg_init(const uint32_t* __restrict__ ranks, const int64_t* __restrict__ offs,
                           const int64_t* __restrict__ ssize, Segs s) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < s.nn; p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t r = ranks[p];
        const int64_t h = offs[r];
        s.S[p] = (int32_t)h;
        if (p == h) {
            const int64_t sz = ssize[r];
            s.end[p] = (int32_t)(h + sz);
            s.depth[p] = 2 * (63 - __clzll((long long)sz));   // 2 floor(log2 size)
        }
    }
}

// Heads: classify, and for a partition the median of three moves to the front
// (__move_median_to_first(first, first + 1, mid, last - 1)).
__global__ void k_seg_heads(Segs s, int* __restrict__ any) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < s.nn; p += (int64_t)gridDim.x * blockDim.x) {
        if (s.S[p] != (int32_t)p) continue;
        const int64_t e = s.end[p], sz = e - p;
        uint8_t a = 0;
        if (sz > kFinalMax) a = s.depth[p] > 0 ? 1 : 2;
        s.act[p] = a;
        if (a != 1) continue;
        const int64_t x = p + 1, y = p + sz / 2, z = e - 1;
        const uint64_t kx = s.K[x], ky = s.K[y], kz = s.K[z];
        int64_t pick;
        if (kx < ky) pick = ky < kz ? y : (kx < kz ? z : x);
        else pick = kx < kz ? x : (ky < kz ? z : y);
        swap_at(s, p, pick);
        s.piv[p] = s.K[p];
        *any = 1;
    }
}

__global__ void k_seg_flags(Segs s) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < s.nn; p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t h = s.S[p];
        int32_t g = 0, l = 0;
        if (s.act[h] == 1 && p > h) {
            const uint64_t pv = s.piv[h], k = s.K[p];
            g = !(k < pv);
            l = !(pv < k);
        }
        s.ge[p] = g;
        s.le[p] = l;
    }
}

__global__ void k_seg_lists(Segs s) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < s.nn; p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t h = s.S[p];
        if (s.act[h] != 1 || p <= h) continue;
        if (s.ge[p]) s.L[h + (s.PG[p] - s.PG[h + 1])] = (int32_t)p;
        if (s.le[p]) {
            const int32_t e = s.end[h];
            s.R[h + (s.PL[e] - s.PL[p + 1])] = (int32_t)p;
        }
    }
}

// Swaps of the unguarded partition: pairs k = 0, 1, ... while L[k] < R[k];
// the cut is min(L[K], R[K - 1]).
__global__ void k_seg_cut(Segs s) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < s.nn; p += (int64_t)gridDim.x * blockDim.x) {
        if (s.S[p] != (int32_t)p || s.act[p] != 1) continue;
        const int32_t e = s.end[p];
        const int64_t nL = s.PG[e] - s.PG[p + 1], nR = s.PL[e] - s.PL[p + 1];
        int64_t lo = 0, hi = min(nL, nR);   // first k with L[k] >= R[k], else min(nL, nR)
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (s.L[p + mid] < s.R[p + mid]) lo = mid + 1; else hi = mid;
        }
        const int64_t K = lo;
        int64_t c = INT64_MAX;
        if (K < nL) c = s.L[p + K];
        if (K >= 1) c = min(c, (int64_t)s.R[p + K - 1]);
        s.kcnt[p] = (int32_t)K;
        s.cut[p] = (int32_t)c;
    }
}

__global__ void k_seg_swap(Segs s) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < s.nn; p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t h = s.S[p];
        if (s.act[h] != 1 || p <= h || !s.ge[p]) continue;
        const int64_t k = s.PG[p] - s.PG[h + 1];
        if (k < s.kcnt[h]) swap_at(s, p, s.R[h + k]);
    }
}

__global__ void k_seg_split(Segs s) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < s.nn; p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t h = s.S[p];
        if (s.act[h] != 1) continue;
        const int32_t c = s.cut[h];
        if (p == h) {
            const int32_t e = s.end[h], d = s.depth[h] - 1;
            s.end[h] = c;
            s.depth[h] = d;
            s.end[c] = e;
            s.depth[c] = d;
        }
        if (p >= c) s.S[p] = c;
    }
}

// libstdc++ __adjust_heap / __push_heap over positions [f, f + len).
__device__ void heap_adjust(const Segs& s, int64_t f, int64_t hole, int64_t len, uint32_t ve, uint64_t vk) {
    const int64_t top = hole;
    int64_t child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (s.K[f + child] < s.K[f + child - 1]) child--;
        s.E[f + hole] = s.E[f + child];
        s.K[f + hole] = s.K[f + child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        s.E[f + hole] = s.E[f + child - 1];
        s.K[f + hole] = s.K[f + child - 1];
        hole = child - 1;
    }
    int64_t parent = (hole - 1) / 2;
    while (hole > top && s.K[f + parent] < vk) {
        s.E[f + hole] = s.E[f + parent];
        s.K[f + hole] = s.K[f + parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    s.E[f + hole] = ve;
    s.K[f + hole] = vk;
}

// Depth limit reached: __partial_sort(first, last, last) = make_heap + sort_heap.
__global__ void k_seg_heap(Segs s) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < s.nn; p += (int64_t)gridDim.x * blockDim.x) {
        if (s.S[p] != (int32_t)p || s.act[p] != 2) continue;
        const int64_t len = s.end[p] - p;
        for (int64_t parent = (len - 2) / 2;; --parent) {
            heap_adjust(s, p, parent, len, s.E[p + parent], s.K[p + parent]);
            if (parent == 0) break;
        }
        for (int64_t last = len - 1; last > 0; --last) {
            const uint32_t ve = s.E[p + last];
            const uint64_t vk = s.K[p + last];
            s.E[p + last] = s.E[p];
            s.K[p + last] = s.K[p];
            heap_adjust(s, p, 0, last, ve, vk);
        }
    }
}

// libstdc++'s final insertion sort, segment by segment (<= 16 elements).
__global__ void k_seg_final(Segs s) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < s.nn; p += (int64_t)gridDim.x * blockDim.x) {
        if (s.S[p] != (int32_t)p) continue;
        const int64_t e = s.end[p];
        if (e - p > kFinalMax) continue;
        for (int64_t i = p + 1; i < e; ++i) {
            const uint32_t ve = s.E[i];
            const uint64_t vk = s.K[i];
            int64_t j = i;
            while (j > p && vk < s.K[j - 1]) {
                s.E[j] = s.E[j - 1];
                s.K[j] = s.K[j - 1];
                --j;
            }
            s.E[j] = ve;
            s.K[j] = vk;
        }
    }
}

// Local ids: position inside the community, or Alternate's interleave of
// both ends (RG:6806-6824).
__global__ void k_sorted_local(const uint32_t* __restrict__ E, int64_t nn, const uint32_t* __restrict__ ranks,
                               const int64_t* __restrict__ offs, const int64_t* __restrict__ ssize, bool alternate,
                               uint32_t* __restrict__ local) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nn; p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t r = ranks[p];
        const int64_t j = p - offs[r];
        int64_t id = j;
        if (alternate) {
            const int64_t sz = ssize[r], mid = (sz + 1) / 2;
            id = j < mid ? 2 * j : 2 * (sz - 1 - j) + 1;
        }
        local[E[p]] = (uint32_t)id;
    }
}

}  // namespace

bool is_sorted_intra_order(int intra) {
    return intra == kHubSort || intra == kDegreeAsc || intra == kHub2 || intra == kAlternate ||
           intra == kBoundaryLast || intra == kCore;
}

int64_t sorted_communities(const DeviceCSR& g, const uint32_t* memb, int intra, const uint32_t* order_v,
                           const uint32_t* ranks, const int64_t* offs, const int64_t* ssize, int64_t nn,
                           uint32_t* local, cudaStream_t s, int64_t* launches) {
    if (nn == 0) return 0;
    const int64_t n = g.n;
    int64_t nl = 0;
    // Per-vertex inputs of the key.
    DevBuf<unsigned long long> score(intra == kHub2 ? n : 0, s);
    DevBuf<uint32_t> aux((intra == kBoundaryLast || intra == kCore) ? n : 0, s);
    if ((intra == kHub2 || intra == kBoundaryLast || intra == kCore) && g.nnz > 0) {
        DevBuf<int32_t> crow(edge_chunks(g.nnz), s);
        chunk_rows_device(g.row_ptr, n, g.nnz, crow, s);
        const int mode = intra == kHub2 ? 0 : (intra == kBoundaryLast ? 1 : 2);
        if (mode == 0) GB_CUDA(cudaMemsetAsync(score, 0, n * sizeof(unsigned long long), s));
        else GB_CUDA(cudaMemsetAsync(aux, 0, n * sizeof(uint32_t), s));
        k_neighbour_sums<<<grid_for(edge_chunks(g.nnz), 1), kSumThreads, 0, s>>>(
            g.row_ptr, g.col, memb, n, g.nnz, crow, mode, score.get(), aux.get());
        GB_LAUNCH_CHECK();
        nl += 2;
    } else if (intra == kBoundaryLast || intra == kCore) {
        GB_CUDA(cudaMemsetAsync(aux, 0, n * sizeof(uint32_t), s));
    }
    if (intra == kCore) {
        // aux holds the internal degree; peel it into core numbers, in place.
        // The whole peel is one graph launch: a while node over steps
        // (scan, apply) whose condition the apply's last CTA sets.
        // Every step peels at least one vertex or raises the level, so at
        // most 2 nn steps run.
        DevBuf<uint32_t> cd(n, s), core(n, s), rem0(nn, s), rem1(nn, s);
        DevBuf<uint32_t> fbuf[2][3];
        CoreFronts fr{};
        for (int b = 0; b < 2; ++b)
            for (int t = 0; t < 3; ++t) {
                fbuf[b][t].alloc(nn, s);
                fr.f[b][t] = fbuf[b][t].get();
            }
        DevBuf<CoreCtl> ctl(1, s);
        CoreCtl init{};
        init.next = 0xFFFFFFFFu;
        init.left = (long long)nn;
        init.max_steps = 2 * (long long)nn + 2;
        init.scan = 1;
        init.rcount = (unsigned)nn;
        GB_CUDA(cudaMemcpyAsync(ctl, &init, sizeof(init), cudaMemcpyHostToDevice, s));
        GB_CUDA(cudaMemcpyAsync(rem0, order_v, nn * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
        k_core_init<<<grid_for(nn, kT), kT, 0, s>>>(order_v, nn, aux, cd, core);
        GB_LAUNCH_CHECK();
        // Grid-stride scans with one resident wave: most steps skip them.
        const int g_all = std::min(grid_for(nn, kT), kNumSMs * 8);
        const int g_apply = kNumSMs * 8;
        struct PeelGraph {
            cudaGraph_t g = nullptr;
            cudaGraphExec_t e = nullptr;
            cudaStream_t cs = nullptr;
            ~PeelGraph() {
                if (e) cudaGraphExecDestroy(e);
                if (g) cudaGraphDestroy(g);
                if (cs) cudaStreamDestroy(cs);
            }
        } pg;
        GB_CUDA(cudaStreamCreateWithFlags(&pg.cs, cudaStreamNonBlocking));
        GB_CUDA(cudaGraphCreate(&pg.g, 0));
        cudaGraphConditionalHandle cond;
        GB_CUDA(cudaGraphConditionalHandleCreate(&cond, pg.g, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = cond;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t loop_node;
        GB_CUDA(cudaGraphAddNode(&loop_node, pg.g, nullptr, nullptr, 0, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        GB_CUDA(cudaStreamBeginCaptureToGraph(pg.cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        k_core_scan<<<g_all, kT, 0, pg.cs>>>(rem0, rem1, g.row_ptr, cd, core, fr, ctl);
        k_core_apply<<<g_apply, kT, 0, pg.cs>>>(fr, g.row_ptr, g.col, memb, core, cd, ctl, cond);
        GB_LAUNCH_CHECK();
        GB_CUDA(cudaStreamEndCapture(pg.cs, &body));
        GB_CUDA(cudaGraphInstantiate(&pg.e, pg.g, 0));
        GB_CUDA(cudaGraphLaunch(pg.e, s));
        const CoreCtl h = read_dev(ctl.get(), s);
        nl += 2 * h.steps;
        GB_REQUIRE(h.done && !h.error, GBGPU_E_CUDA, "core peel made no progress");
        GB_CUDA(cudaMemcpyAsync(aux, core, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    }

    DevBuf<uint32_t> E(nn, s);
    DevBuf<uint64_t> K(nn, s);
    const int grid = grid_for(nn, kT);
    k_sorted_keys<<<grid, kT, 0, s>>>(order_v, nn, g.row_ptr, intra, score.get(), aux.get(), E, K);
    GB_LAUNCH_CHECK();
    nl += 1;
    libstdcxx_sort_segments(E, K, ranks, offs, ssize, nn, s, &nl);
    k_sorted_local<<<grid, kT, 0, s>>>(E, nn, ranks, offs, ssize, intra == kAlternate, local);
    GB_LAUNCH_CHECK();
    nl += 1;
    if (launches) *launches += nl;
    return 0;
}

void libstdcxx_sort_segments(uint32_t* E, uint64_t* K, const uint32_t* ranks, const int64_t* offs,
                             const int64_t* ssize, int64_t nn, cudaStream_t s, int64_t* launches) {
    if (nn == 0) return;
    GB_REQUIRE(nn < (int64_t)INT32_MAX, GBGPU_E_INVALID, "segmented sort: too many elements");
    int64_t nl = 0;
    Segs sg{};
    DevBuf<uint64_t> piv(nn, s);
    DevBuf<int32_t> S(nn, s), end(nn, s), depth(nn, s), kcnt(nn, s), cut(nn, s), ge(nn, s), le(nn, s), L(nn, s),
        R(nn, s);
    DevBuf<uint8_t> act(nn, s);
    DevBuf<int64_t> PG(nn + 1, s), PL(nn + 1, s);
    sg.E = E;
    sg.K = K;
    sg.S = S;
    sg.end = end;
    sg.depth = depth;
    sg.act = act;
    sg.piv = piv;
    sg.kcnt = kcnt;
    sg.cut = cut;
    sg.ge = ge;
    sg.le = le;
    sg.PG = PG;
    sg.PL = PL;
    sg.L = L;
    sg.R = R;
    sg.nn = nn;
    const int grid = grid_for(nn, kT);
    k_seg_init<<<grid, kT, 0, s>>>(ranks, offs, ssize, sg);
    GB_LAUNCH_CHECK();
    nl += 1;
    DevBuf<int> any(1, s);
    // Each level halves the largest active segment or spends one unit of its
    // depth limit (<= 2 log2 nn + 2 levels).
    const int max_levels = 2 * 64;
    bool settled = false;
    for (int level = 0; level <= max_levels && !settled; ++level) {
        GB_CUDA(cudaMemsetAsync(any, 0, sizeof(int), s));
        k_seg_heads<<<grid, kT, 0, s>>>(sg, any);
        GB_LAUNCH_CHECK();
        nl += 1;
        settled = read_dev(any.get(), s) == 0;
        if (settled) break;
        k_seg_flags<<<grid, kT, 0, s>>>(sg);
        GB_LAUNCH_CHECK();
        exclusive_scan_i32_to_i64(ge, PG, nn, PG.get() + nn, s);
        exclusive_scan_i32_to_i64(le, PL, nn, PL.get() + nn, s);
        k_seg_lists<<<grid, kT, 0, s>>>(sg);
        GB_LAUNCH_CHECK();
        k_seg_cut<<<grid, kT, 0, s>>>(sg);
        GB_LAUNCH_CHECK();
        k_seg_swap<<<grid, kT, 0, s>>>(sg);
        GB_LAUNCH_CHECK();
        k_seg_split<<<grid, kT, 0, s>>>(sg);
        GB_LAUNCH_CHECK();
        nl += 11;
    }
    GB_REQUIRE(settled, GBGPU_E_CUDA, "sorted intra order: partition levels did not settle");
    k_seg_heap<<<grid, kT, 0, s>>>(sg);
    GB_LAUNCH_CHECK();
    k_seg_final<<<grid, kT, 0, s>>>(sg);
    GB_LAUNCH_CHECK();
    nl += 2;
    if (launches) *launches += nl;
}

}  // namespace gb
