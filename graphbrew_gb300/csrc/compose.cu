// compose.cu -- COMPOSE placement and intra-community ordering on the device.
//
// Follows graphbrew::orderCompose (bench/include/graphbrew/reorder/reorder_graphbrew.h:6286-7087)
// with super-graph order "none":
//   * vertices of degree 0 go to the global tail in id order (:6336-6386);
//   * communities are stable-sorted by the community-order key (:6438-6502);
//   * each community's vertices keep vertex-id order (commVertices, :6373-6386);
//   * intra order: Gorder with window w for 4..fallback vertices
//     (intraGorderGreedy, :4420-4587), BFS from the hub above the fallback
//     (intraBFSFromHub, :3929-3984), identity for <= 3 vertices; or reverse
//     Cuthill-McKee for every community (intraRCM, :4000-4134);
//   * newIds[v] = offset(community) + localId[v] (:7003-7017).
//
// Layout in HBM (n vertices): one stable radix sort of (rank(community), v)
// gives the whole placement skeleton: position p in [0, n) holds the vertex
// placed p-th before intra ordering, isolated vertices last.  Every later
// kernel indexes communities by their contiguous position range.
#include <algorithm>
#include <type_traits>

#include "gb_common.cuh"
#include "gb_stages.h"

namespace gb {

namespace {

enum CommunityOrderOrd { kSizeDesc = 0, kSizeAsc = 1, kDegreeDesc = 2, kDegreeAsc = 3, kIdentity = 6 };
enum IntraOrd { kIntraBFS = 0, kIntraRCM = 1, kIntraRCMpp = 2, kIntraDendrogram = 3, kIntraGorder = 4, kIntraRandom = 10 };

constexpr int kT = 256;

__global__ void k_max_u32(const uint32_t* __restrict__ a, int64_t n, uint32_t* __restrict__ out) {
    uint32_t m = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = max(m, a[i]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// Community sizes over non-isolated vertices, optional degree totals.
__global__ void k_comm_sizes(const int64_t* __restrict__ rp, const uint32_t* __restrict__ memb, int64_t n,
                             uint32_t* __restrict__ csize, unsigned long long* __restrict__ cdeg) {
    const int lane = threadIdx.x & 31;
    for (int64_t v0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane; v0 < n;
         v0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = v0 + lane;
        const int64_t d = v < n ? rp[v + 1] - rp[v] : 0;
        const uint32_t c = d ? memb[v] : 0u;
        warp_add_u32(csize, c, 1u, d != 0);
        if (cdeg) warp_add_u64(cdeg, c, (unsigned long long)d, d != 0);
    }
}

__global__ void k_max_u32_u64(const uint32_t* __restrict__ a, const unsigned long long* __restrict__ b, int64_t n,
                              uint32_t* __restrict__ out_a, unsigned long long* __restrict__ out_b) {
    uint32_t ma = 0;
    unsigned long long mb = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        ma = max(ma, a[i]);
        if (b) mb = max(mb, b[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        ma = max(ma, __shfl_xor_sync(0xFFFFFFFFu, ma, o));
        mb = max(mb, __shfl_xor_sync(0xFFFFFFFFu, mb, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out_a, ma);
        if (b) atomicMax(out_b, mb);
    }
}

// stage1, when given (a super-graph order), places community c at position
// stage1[c] before the stable sort, so equal keys keep stage1's order.
__global__ void k_comm_keys(int order, const uint32_t* __restrict__ csize, const unsigned long long* __restrict__ cdeg,
                            int64_t C, uint32_t max_size, unsigned long long max_deg,
                            const uint32_t* __restrict__ stage1, uint64_t* __restrict__ keys,
                            uint32_t* __restrict__ ids) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C; c += (int64_t)gridDim.x * blockDim.x) {
        uint64_t k = 0;
        switch (order) {
            case kSizeDesc: k = (uint64_t)(max_size - csize[c]); break;
            case kSizeAsc: k = csize[c]; break;
            case kDegreeDesc: k = max_deg - cdeg[c]; break;
            case kDegreeAsc: k = cdeg[c]; break;
            default: k = 0; break;
        }
        const int64_t at = stage1 ? (int64_t)stage1[c] : c;
        keys[at] = k;
        ids[at] = (uint32_t)c;
    }
}

// rank[c] and sorted sizes.
__global__ void k_rank(const uint32_t* __restrict__ order, const uint32_t* __restrict__ csize, int64_t C,
                       uint32_t* __restrict__ rank, int64_t* __restrict__ ssize) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < C; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t c = order[i];
        rank[c] = (uint32_t)i;
        ssize[i] = csize[c];
    }
}

// Sort keys for the placement skeleton: rank of the vertex's community, or C
// for isolated vertices (they sort last, in id order).
__global__ void k_vertex_keys(const int64_t* __restrict__ rp, const uint32_t* __restrict__ memb,
                              const uint32_t* __restrict__ rank, int64_t n, uint32_t C,
                              uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        keys[v] = (rp[v + 1] == rp[v]) ? C : rank[memb[v]];
        vals[v] = (uint32_t)v;
    }
}

// pos_of[v], local index (identity intra order) per vertex.
__global__ void k_positions(const uint32_t* __restrict__ order_v, const uint32_t* __restrict__ keys_sorted,
                            const int64_t* __restrict__ offs, int64_t n, uint32_t C,
                            int64_t* __restrict__ pos_of, uint32_t* __restrict__ local) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t v = order_v[p];
        const uint32_t r = keys_sorted[p];
        pos_of[v] = p;
        local[v] = (r < C) ? (uint32_t)(p - offs[r]) : 0u;
    }
}

// Community classes: 1 = Gorder (thread), 2 = Gorder (warp, shared memory),
// 3 = Gorder (warp, global workspace), 4 = BFS.  Lists hold ranks.
struct ClassCounts {
    int32_t n[5];
    unsigned long long gorder_communities, gorder_vertices, fallback_communities, fallback_vertices;
    uint32_t gorder_max, largest;
};

constexpr int kThreadGorderMax = 32;
constexpr int kSmemGorderMax = 4096;
constexpr int kMaxGorderWindow = 100;   // the thread variant's bound (kMaxB) too

__global__ void k_classify(const int64_t* __restrict__ ssize, int64_t C, int intra, int fallback,
                           int32_t* __restrict__ lists, ClassCounts* __restrict__ cc) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < C; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t sz = ssize[i];
        if (sz == 0) continue;
        atomicMax(&cc->largest, (uint32_t)sz);
        int cls = 0;
        if (intra == kIntraGorder) {
            if (fallback > 0 && sz > fallback) {
                atomicAdd(&cc->fallback_communities, 1ull);
                atomicAdd(&cc->fallback_vertices, (unsigned long long)sz);
                cls = 4;
            } else if (sz > 3) {
                atomicAdd(&cc->gorder_communities, 1ull);
                atomicAdd(&cc->gorder_vertices, (unsigned long long)sz);
                atomicMax(&cc->gorder_max, (uint32_t)sz);
                cls = sz <= kThreadGorderMax ? 1 : (sz <= kSmemGorderMax ? 2 : 3);
            }
        } else {
            cls = sz >= 2 ? 4 : 0;
        }
        if (cls) {
            const int32_t slot = atomicAdd(&cc->n[cls], 1);
            lists[(int64_t)cls * C + slot] = (int32_t)i;
        }
    }
}

// ---------------------------------------------------------------------------
// Local adjacency for Gorder communities: for each position p, the local
// indices of in-community neighbours in row order.
// ---------------------------------------------------------------------------
__global__ void k_mark_gorder_positions(const int32_t* __restrict__ list, const int32_t* __restrict__ count_p,
                                        const int64_t* __restrict__ offs, const int64_t* __restrict__ ssize,
                                        uint8_t* __restrict__ mark) {
    const int32_t count = *count_p;
    for (int32_t j = blockIdx.x; j < count; j += gridDim.x) {
        const int32_t r = list[j];
        const int64_t b = offs[r], sz = ssize[r];
        for (int64_t k = threadIdx.x; k < sz; k += blockDim.x) mark[b + k] = 1;
    }
}

__global__ void k_local_count(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                              const uint32_t* __restrict__ memb, const uint32_t* __restrict__ order_v,
                              const uint8_t* __restrict__ mark, int64_t nn, int64_t* __restrict__ cnt) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nn; p += (int64_t)gridDim.x * blockDim.x) {
        int64_t c = 0;
        if (mark[p]) {
            const uint32_t u = order_v[p];
            const uint32_t cu = memb[u];
            for (int64_t e = rp[u]; e < rp[u + 1]; ++e) c += (memb[col[e]] == cu);
        }
        cnt[p] = c;
    }
}

__global__ void k_local_fill(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                             const uint32_t* __restrict__ memb, const uint32_t* __restrict__ order_v,
                             const uint8_t* __restrict__ mark, const uint32_t* __restrict__ local,
                             const int64_t* __restrict__ loff, int64_t nn, uint16_t* __restrict__ ladj16,
                             uint32_t* __restrict__ ladj32) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nn; p += (int64_t)gridDim.x * blockDim.x) {
        if (!mark[p]) continue;
        const uint32_t u = order_v[p];
        const uint32_t cu = memb[u];
        int64_t o = loff[p];
        for (int64_t e = rp[u]; e < rp[u + 1]; ++e) {
            const int32_t w = col[e];
            if (memb[w] == cu) {
                if (ladj32) ladj32[o++] = local[w];
                else ladj16[o++] = (uint16_t)local[w];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// UnitHeap replica (intraGorderGreedy).  The list keeps buckets contiguous in
// descending key order; insertion is at the bucket front; extract-max takes
// the front of the highest non-empty bucket.  Storage is abstracted so one
// body serves thread-private arrays, shared memory and global workspaces.
// ---------------------------------------------------------------------------
struct HeapView {
    int* key;
    int* prev;
    int* next;
    int* bfirst;
    int* bsecond;
    int max_key;

    __device__ __forceinline__ void unlink(int idx) {
        const int p = prev[idx], nx = next[idx];
        if (p >= 0) next[p] = nx;
        if (nx >= 0) prev[nx] = p;
        const int k = key[idx];
        if (bfirst[k] == idx && bsecond[k] == idx) {
            bfirst[k] = bsecond[k] = -1;
        } else if (bfirst[k] == idx) {
            bfirst[k] = nx;
        } else if (bsecond[k] == idx) {
            bsecond[k] = p;
        }
    }
    __device__ __forceinline__ void link_front(int idx, int k) {
        key[idx] = k;
        if (bfirst[k] < 0) {
            int after = -1;
            for (int bk = k - 1; bk >= 0; --bk)
                if (bfirst[bk] >= 0) { after = bfirst[bk]; break; }
            int before = -1;
            for (int bk = k + 1; bk <= max_key; ++bk)
                if (bsecond[bk] >= 0) { before = bsecond[bk]; break; }
            prev[idx] = before;
            next[idx] = after;
            if (before >= 0) next[before] = idx;
            if (after >= 0) prev[after] = idx;
            bfirst[k] = bsecond[k] = idx;
        } else {
            const int old_first = bfirst[k];
            const int before_old = prev[old_first];
            prev[idx] = before_old;
            next[idx] = old_first;
            prev[old_first] = idx;
            if (before_old >= 0) next[before_old] = idx;
            bfirst[k] = idx;
        }
        if (k > max_key) max_key = k;
    }
    __device__ __forceinline__ void remove(int idx) {
        unlink(idx);
        prev[idx] = next[idx] = -1;
        key[idx] = -1;
        while (max_key > 0 && bfirst[max_key] < 0) --max_key;
    }
    __device__ __forceinline__ int extract_max() {
        while (max_key > 0 && bfirst[max_key] < 0) --max_key;
        const int idx = bfirst[max_key];
        if (idx >= 0) remove(idx);
        return idx;
    }
    __device__ __forceinline__ void bump(int idx, int delta) {
        const int old = key[idx];
        if (old < 0) return;
        if (delta < 0 && old <= 0) return;
        unlink(idx);
        link_front(idx, old + delta);
    }
};

// Runs the greedy placement of one community of sz vertices (local indices
// 0..sz-1 in vertex-id order).  ladj/loff give local adjacency; seed_deg the
// degrees for seeding; out_local receives local ids by local index.
template <typename LAdj>
__device__ void gorder_run(HeapView& h, int sz, int nbuckets, int window, const LAdj* __restrict__ ladj,
                           const int64_t* __restrict__ loff, const uint32_t* __restrict__ degs,
                           int* __restrict__ placed, uint32_t* __restrict__ out_local) {
    for (int i = 0; i < sz; ++i) {
        h.key[i] = 0;
        h.prev[i] = i - 1;
        h.next[i] = (i + 1 < sz) ? i + 1 : -1;
    }
    for (int b = 0; b < nbuckets; ++b) h.bfirst[b] = h.bsecond[b] = -1;
    h.bfirst[0] = 0;
    h.bsecond[0] = sz - 1;
    h.max_key = 0;
    int seed = 0;
    uint32_t seed_deg = degs[0];
    for (int i = 1; i < sz; ++i)
        if (degs[i] > seed_deg) { seed_deg = degs[i]; seed = i; }
    h.remove(seed);
    int nplaced = 0;
    placed[nplaced++] = seed;
    out_local[seed] = 0;
    for (int64_t k = loff[seed]; k < loff[seed + 1]; ++k) h.bump((int)ladj[k], +1);
    for (int lid = 1; lid < sz; ++lid) {
        const int best = h.extract_max();
        if (best < 0) {
            for (int i = 0; i < sz && lid < sz; ++i) {
                if (h.key[i] >= 0) {
                    h.remove(i);
                    out_local[i] = (uint32_t)lid++;
                }
            }
            break;
        }
        placed[nplaced++] = best;
        out_local[best] = (uint32_t)lid;
        for (int64_t k = loff[best]; k < loff[best + 1]; ++k) h.bump((int)ladj[k], +1);
        if (nplaced > window) {
            const int old_v = placed[nplaced - 1 - window];
            for (int64_t k = loff[old_v]; k < loff[old_v + 1]; ++k) h.bump((int)ladj[k], -1);
        }
    }
}

// One thread per community of 4..32 vertices; state in thread-private arrays.
template <typename LAdj>
__global__ void k_gorder_thread(const int32_t* __restrict__ list, const int32_t* __restrict__ count_p,
                                const int64_t* __restrict__ offs, const int64_t* __restrict__ ssize,
                                const uint32_t* __restrict__ order_v, const int64_t* __restrict__ rp,
                                const LAdj* __restrict__ ladj, const int64_t* __restrict__ loff,
                                int window, uint32_t* __restrict__ local_by_pos) {
    constexpr int kMaxB = 102 + 8;  // window <= 100
    const int32_t count = *count_p;
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x) {
        const int32_t r = list[j];
        const int64_t base = offs[r];
        const int sz = (int)ssize[r];
        int key[kThreadGorderMax], prev[kThreadGorderMax], next[kThreadGorderMax], placed[kThreadGorderMax];
        int bf[kMaxB], bs[kMaxB];
        uint32_t degs[kThreadGorderMax];
        for (int i = 0; i < sz; ++i) {
            const uint32_t u = order_v[base + i];
            degs[i] = (uint32_t)(rp[u + 1] - rp[u]);
        }
        HeapView h{key, prev, next, bf, bs, 0};
        const int nb = min(window + 2, kMaxB);
        gorder_run<LAdj>(h, sz, nb, window, ladj, loff + base, degs, placed, local_by_pos + base);
    }
}

// ---------------------------------------------------------------------------
// The same UnitHeap, held so that a warp can apply a placed vertex's bumps
// together.  Each bucket is a stack in a push log: a bump pushes the vertex
// onto its new bucket's stack; an entry is live while it is its vertex's
// latest push and the vertex is unplaced; a bucket's front (extract-max,
// bucket-front insertion) is its newest live entry.  That is the linked
// list's order exactly: a bucket lists the vertices moved into it, newest
// first, then -- bucket 0 only -- the untouched vertices in local order (the
// initial pushes, vertex 0 last).  A batch of bumps by one placed vertex
// touches distinct vertices, so it is applied a warp at a time, pushes
// ordered as the reference processes the adjacency: entries are allocated in
// that order and each links to the previous push onto the same bucket (a
// __match_any_sync group).  Stale entries are skipped when a front is taken;
// when the log is full, a compaction keeps each live vertex's latest entry in
// push order and relinks the stacks.
// ---------------------------------------------------------------------------
struct LazyHeap {
    int* key;        // [S] bucket of each local vertex, -1 once placed
    int* lastpush;   // [S] log entry of its latest push
    int* log_v;      // [L] pushed vertex
    int* log_next;   // [L] entry below it in the same bucket (-1: bottom)
    int* top;        // [nb] newest entry of each bucket (-1: empty)
    int* last;       // [nb] compaction scratch
    int* ring;       // [window + 1] the last placed vertices
    uint32_t* degs;  // [S] degrees (seed choice)
    int L;
};

__host__ __device__ constexpr int lazy_log_cap(int S) { return 2 * S + 64; }
__host__ __device__ constexpr int64_t lazy_ws_ints(int64_t S, int nb, int window) {
    return 3 * S + 2 * (int64_t)lazy_log_cap((int)S) + 2 * nb + window + 1;
}

__device__ __forceinline__ LazyHeap lazy_view(int* ws, int64_t S, int nb, int window) {
    LazyHeap h;
    h.L = lazy_log_cap((int)S);
    h.key = ws;
    h.lastpush = h.key + S;
    h.log_v = h.lastpush + S;
    h.log_next = h.log_v + h.L;
    h.top = h.log_next + h.L;
    h.last = h.top + nb;
    h.ring = h.last + nb;
    h.degs = reinterpret_cast<uint32_t*>(h.ring + window + 1);
    return h;
}

template <typename LAdj>
__device__ void gorder_lazy_warp(const LazyHeap& h, int sz, int nb, int window, const LAdj* __restrict__ ladj,
                                 const int64_t* __restrict__ loff, uint32_t* __restrict__ out_local) {
    const int lane = threadIdx.x & 31;
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const unsigned lower_lanes = (1u << lane) - 1u;
    // Bucket 0 lists 0..sz-1 with 0 in front: pushed sz-1 first, 0 last.
    for (int e = lane; e < sz; e += 32) {
        const int v = sz - 1 - e;
        h.log_v[e] = v;
        h.log_next[e] = e - 1;
        h.key[v] = 0;
        h.lastpush[v] = e;
    }
    for (int b = lane; b < nb; b += 32) h.top[b] = b == 0 ? sz - 1 : -1;
    // Seed: largest degree, first in local order.
    uint32_t bd = 0;
    int bi = -1;
    for (int i = lane; i < sz; i += 32)
        if (bi < 0 || h.degs[i] > bd) {
            bd = h.degs[i];
            bi = i;
        }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint32_t od = __shfl_xor_sync(kFull, bd, o);
        const int oi = __shfl_xor_sync(kFull, bi, o);
        if (oi >= 0 && (bi < 0 || od > bd || (od == bd && oi < bi))) {
            bd = od;
            bi = oi;
        }
    }
    const int seed = bi;
    int len = sz, max_key = 0;
    __syncwarp();
    if (lane == 0) {
        h.key[seed] = -1;
        out_local[seed] = 0;
        h.ring[0] = seed;
    }
    __syncwarp();

    auto compact = [&]() {
        for (int b = lane; b < nb; b += 32) h.last[b] = -1;
        __syncwarp();
        int nl = 0;
        for (int c0 = 0; c0 < len; c0 += 32) {
            const int e = c0 + lane;
            int v = -1, b = -1;
            bool keep = false;
            if (e < len) {
                v = h.log_v[e];
                b = h.key[v];
                keep = b >= 0 && h.lastpush[v] == e;
            }
            const unsigned kb = __ballot_sync(kFull, keep);
            const int ne = nl + __popc(kb & lower_lanes);
            const unsigned peers = __match_any_sync(kFull, keep ? b : -1 - lane);
            const unsigned below = peers & lower_lanes;
            const int ne_below = __shfl_sync(kFull, ne, below ? 31 - __clz(below) : lane);
            const int prev = keep ? (below ? ne_below : h.last[b]) : -1;
            __syncwarp();
            if (keep) {
                h.log_v[ne] = v;
                h.log_next[ne] = prev;
                h.lastpush[v] = ne;
                if ((peers >> lane) == 1u) h.last[b] = ne;
            }
            nl += __popc(kb);
            __syncwarp();
        }
        for (int b = lane; b < nb; b += 32) h.top[b] = h.last[b];
        len = nl;
        __syncwarp();
    };

    // bump(n, delta) for every neighbour n of v, in adjacency order.
    auto bump_all = [&](int v, int delta) {
        const int64_t e0 = loff[v], e1 = loff[v + 1];
        if (len + (e1 - e0) > h.L) compact();
        for (int64_t base = e0; base < e1; base += 32) {
            const int64_t idx = base + lane;
            int n = -1, k = -1;
            if (idx < e1) {
                n = (int)ladj[idx];
                k = h.key[n];
            }
            const bool app = k >= 0 && !(delta < 0 && k <= 0);
            const int t = k + delta;
            const unsigned ab = __ballot_sync(kFull, app);
            const int e = len + __popc(ab & lower_lanes);
            const unsigned peers = __match_any_sync(kFull, app ? t : -1 - lane);
            const unsigned below = peers & lower_lanes;
            const int e_below = __shfl_sync(kFull, e, below ? 31 - __clz(below) : lane);
            const int prev = app ? (below ? e_below : h.top[t]) : -1;
            __syncwarp();
            if (app) {
                h.log_v[e] = n;
                h.log_next[e] = prev;
                h.key[n] = t;
                h.lastpush[n] = e;
                if ((peers >> lane) == 1u) h.top[t] = e;
            }
            len += __popc(ab);
            int tm = app ? t : 0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) tm = max(tm, __shfl_xor_sync(kFull, tm, o));
            max_key = max(max_key, tm);
            __syncwarp();
        }
    };

    bump_all(seed, +1);
    int nplaced = 1;
    for (int lid = 1; lid < sz; ++lid) {
        // extract-max: newest live entry of the highest non-empty bucket.
        int best = -1, b = max_key;
        if (lane == 0) {
            while (true) {
                int e = h.top[b];
                while (e >= 0) {
                    const int v = h.log_v[e];
                    if (h.key[v] == b && h.lastpush[v] == e) break;
                    e = h.log_next[e];
                }
                if (e >= 0) {
                    best = h.log_v[e];
                    h.top[b] = h.log_next[e];
                    h.key[best] = -1;
                    break;
                }
                h.top[b] = -1;
                if (b == 0) break;
                --b;
            }
        }
        best = __shfl_sync(kFull, best, 0);
        max_key = __shfl_sync(kFull, b, 0);
        if (best < 0) {   // no live vertex left: the rest in local order
            if (lane == 0)
                for (int i = 0; i < sz && lid < sz; ++i)
                    if (h.key[i] >= 0) {
                        h.key[i] = -1;
                        out_local[i] = (uint32_t)lid++;
                    }
            break;
        }
        if (lane == 0) {
            out_local[best] = (uint32_t)lid;
            h.ring[nplaced % (window + 1)] = best;
        }
        ++nplaced;
        __syncwarp();
        bump_all(best, +1);
        if (nplaced > window) {
            int old_v = 0;
            if (lane == 0) old_v = h.ring[(nplaced - 1 - window) % (window + 1)];
            old_v = __shfl_sync(kFull, old_v, 0);
            bump_all(old_v, -1);
        }
    }
    __syncwarp();
}

// One warp per community of 33..gordf vertices; its workspace in shared
// memory (capacity S of the launch) or, for the largest class, in global
// memory (one slice per CTA).
template <typename LAdj, bool kShared>
__global__ void k_gorder_warp(const int32_t* __restrict__ list, const int32_t* __restrict__ count_p,
                              const int64_t* __restrict__ offs, const int64_t* __restrict__ ssize,
                              const uint32_t* __restrict__ order_v, const int64_t* __restrict__ rp,
                              const LAdj* __restrict__ ladj, const int64_t* __restrict__ loff, int window,
                              uint32_t* __restrict__ local_by_pos, int* __restrict__ gws, int64_t cap) {
    extern __shared__ int smem[];
    const int32_t count = *count_p;
    const int lane = threadIdx.x & 31;
    const int nb = window + 2;
    int* ws = kShared ? smem : gws + (int64_t)blockIdx.x * lazy_ws_ints(cap, nb, window);
    const LazyHeap h = lazy_view(ws, cap, nb, window);
    for (int32_t j = blockIdx.x; j < count; j += gridDim.x) {
        const int32_t r = list[j];
        const int64_t base = offs[r];
        const int sz = (int)ssize[r];
        for (int i = lane; i < sz; i += 32) {
            const uint32_t u = order_v[base + i];
            h.degs[i] = (uint32_t)(rp[u + 1] - rp[u]);
        }
        __syncwarp();
        gorder_lazy_warp<LAdj>(h, sz, nb, window, ladj, loff + base, local_by_pos + base);
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Exact-order BFS from the hub (intraBFSFromHub), level-synchronous over all
// BFS communities at once.  Within one community the reference's FIFO order
// is reproduced: a vertex is discovered by the earliest frontier vertex (queue
// position) that reaches it and, within that parent, in row order.  Claims are
// atomicMin of (frontier index << 32 | row offset); the children of a level
// are then written in (frontier index, row offset) order by an exclusive scan
// over per-edge flags.
// ---------------------------------------------------------------------------
__global__ void k_bfs_slots(const int32_t* __restrict__ list, const int32_t* __restrict__ count_p,
                            const uint32_t* __restrict__ order_v, const int64_t* __restrict__ offs,
                            const uint32_t* __restrict__ memb, int32_t* __restrict__ slot_of_comm,
                            int64_t* __restrict__ slot_base, int64_t* __restrict__ slot_size,
                            const int64_t* __restrict__ ssize) {
    const int32_t count = *count_p;
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x) {
        const int32_t r = list[j];
        const uint32_t c = memb[order_v[offs[r]]];
        slot_of_comm[c] = j;
        slot_base[j] = offs[r];
        slot_size[j] = ssize[r];
    }
}

// Hub = max degree, first in vertex-id (= position) order.
__global__ void k_bfs_hubs(const int64_t* __restrict__ slot_base, const int64_t* __restrict__ slot_size, int32_t nslots,
                           const uint32_t* __restrict__ order_v, const int64_t* __restrict__ rp,
                           unsigned long long* __restrict__ hubkey) {
    // grid-stride over (slot, position) flattened per slot: one block per slot chunk
    for (int32_t j = blockIdx.y; j < nslots; j += gridDim.y) {
        const int64_t b = slot_base[j], sz = slot_size[j];
        unsigned long long best = 0;
        for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < sz; k += (int64_t)gridDim.x * blockDim.x) {
            const uint32_t u = order_v[b + k];
            const uint64_t d = (uint64_t)(rp[u + 1] - rp[u]);
            const unsigned long long key = (d << 32) | (0xFFFFFFFFull - (uint64_t)k);
            best = key > best ? key : best;
        }
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long t = __shfl_xor_sync(0xFFFFFFFFu, best, o);
            best = t > best ? t : best;
        }
        if ((threadIdx.x & 31) == 0) atomicMax(&hubkey[j], best);
    }
}

__global__ void k_bfs_init(const unsigned long long* __restrict__ hubkey, const int64_t* __restrict__ slot_base,
                           int32_t nslots, const uint32_t* __restrict__ order_v, int32_t* __restrict__ frontier,
                           uint8_t* __restrict__ visited, uint32_t* __restrict__ local, int64_t* __restrict__ qlen,
                           int64_t* __restrict__ fs, int64_t* __restrict__ fe) {
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nslots; j += gridDim.x * blockDim.x) {
        const int64_t k = (int64_t)(0xFFFFFFFFull - (hubkey[j] & 0xFFFFFFFFull));
        const uint32_t hub = order_v[slot_base[j] + k];
        frontier[j] = (int32_t)hub;
        visited[hub] = 1;
        local[hub] = 0;
        qlen[j] = 1;
        fs[j] = j;
        fe[j] = j + 1;
    }
}

__global__ void k_frontier_degrees(const int32_t* __restrict__ F, int64_t nf, const int64_t* __restrict__ rp,
                                   int64_t* __restrict__ fdeg) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nf; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = F[i];
        fdeg[i] = rp[u + 1] - rp[u];
    }
}

__device__ __forceinline__ int64_t upper_index(const int64_t* __restrict__ D, int64_t nf, int64_t e) {
    // largest i in [0, nf) with D[i] <= e
    int64_t lo = 0, hi = nf - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (D[mid] <= e) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Frontier edges in runs of kEdgeRun consecutive edge indices per thread:
// one binary search for the run's first edge, then the owning frontier
// vertex advances with the edge index.
constexpr int kEdgeRun = 8;

template <typename Fn>
__device__ __forceinline__ void for_frontier_edges(const int64_t* __restrict__ D, int64_t nf, int64_t T, Fn&& fn) {
    for (int64_t e0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) * kEdgeRun; e0 < T;
         e0 += (int64_t)gridDim.x * blockDim.x * kEdgeRun) {
        int64_t i = upper_index(D, nf, e0);
        int64_t next = D[i + 1];
        const int64_t e1 = min(T, e0 + kEdgeRun);
        for (int64_t e = e0; e < e1; ++e) {
            while (e >= next) {
                ++i;
                next = D[i + 1];
            }
            fn(i, e - D[i], e);
        }
    }
}

inline int edge_grid(int64_t T) { return grid_for(ceil_div(T, kEdgeRun), 256); }

__global__ void k_bfs_claim(const int32_t* __restrict__ F, int64_t nf, const int64_t* __restrict__ D, int64_t T,
                            const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                            const uint32_t* __restrict__ memb, const uint8_t* __restrict__ visited,
                            unsigned long long* __restrict__ claim) {
    for_frontier_edges(D, nf, T, [&](int64_t i, int64_t k, int64_t) {
        const int32_t u = F[i];
        const int32_t w = col[rp[u] + k];
        if (memb[w] == memb[u] && !visited[w])
            atomicMin(&claim[w], ((unsigned long long)i << 32) | (unsigned long long)k);
    });
}

__global__ void k_bfs_flag(const int32_t* __restrict__ F, int64_t nf, const int64_t* __restrict__ D, int64_t T,
                           const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                           const uint32_t* __restrict__ memb, const uint8_t* __restrict__ visited,
                           const unsigned long long* __restrict__ claim, uint8_t* __restrict__ flag) {
    for_frontier_edges(D, nf, T, [&](int64_t i, int64_t k, int64_t e) {
        const int32_t u = F[i];
        const int32_t w = col[rp[u] + k];
        flag[e] = (memb[w] == memb[u] && !visited[w] &&
                   claim[w] == (((unsigned long long)i << 32) | (unsigned long long)k)) ? 1 : 0;
    });
}

// Per community: where its children start in the next frontier this level.
__global__ void k_bfs_bases(int32_t nslots, const int64_t* __restrict__ fs, const int64_t* __restrict__ fe,
                            const int64_t* __restrict__ D, const int64_t* __restrict__ P,
                            int64_t* __restrict__ base, int64_t* __restrict__ end) {
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nslots; j += gridDim.x * blockDim.x) {
        base[j] = P[D[fs[j]]];
        end[j] = P[D[fe[j]]];
    }
}

__global__ void k_bfs_write(const int32_t* __restrict__ F, int64_t nf, const int64_t* __restrict__ D, int64_t T,
                            const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                            const uint32_t* __restrict__ memb, const uint8_t* __restrict__ flag,
                            const int64_t* __restrict__ P, const int32_t* __restrict__ slot_of_comm,
                            const int64_t* __restrict__ qlen, const int64_t* __restrict__ base,
                            int32_t* __restrict__ nextF, uint8_t* __restrict__ visited, uint32_t* __restrict__ local) {
    for_frontier_edges(D, nf, T, [&](int64_t i, int64_t k, int64_t e) {
        if (!flag[e]) return;
        const int32_t u = F[i];
        const int32_t w = col[rp[u] + k];
        const int64_t p = P[e];
        const int32_t j = slot_of_comm[memb[u]];
        nextF[p] = w;
        visited[w] = 1;
        local[w] = (uint32_t)(qlen[j] + (p - base[j]));
    });
}

__global__ void k_bfs_advance(int32_t nslots, int64_t* __restrict__ qlen, int64_t* __restrict__ fs,
                              int64_t* __restrict__ fe, const int64_t* __restrict__ base,
                              const int64_t* __restrict__ end) {
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nslots; j += gridDim.x * blockDim.x) {
        qlen[j] += end[j] - base[j];
        fs[j] = base[j];
        fe[j] = end[j];
    }
}

// Unreached vertices of BFS communities, in vertex order after the BFS order.
__global__ void k_bfs_left_flags(const uint32_t* __restrict__ order_v, int64_t nn, const uint32_t* __restrict__ memb,
                                 const int32_t* __restrict__ slot_of_comm, const uint8_t* __restrict__ visited,
                                 int32_t* __restrict__ flag) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nn; p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t v = order_v[p];
        flag[p] = (slot_of_comm[memb[v]] >= 0 && !visited[v]) ? 1 : 0;
    }
}

__global__ void k_bfs_left_assign(const uint32_t* __restrict__ order_v, int64_t nn, const uint32_t* __restrict__ memb,
                                  const int32_t* __restrict__ slot_of_comm, const int32_t* __restrict__ flag,
                                  const int64_t* __restrict__ R, const int64_t* __restrict__ slot_base,
                                  const int64_t* __restrict__ qlen, uint32_t* __restrict__ local) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nn; p += (int64_t)gridDim.x * blockDim.x) {
        if (!flag[p]) continue;
        const uint32_t v = order_v[p];
        const int32_t j = slot_of_comm[memb[v]];
        local[v] = (uint32_t)(qlen[j] + (R[p] - R[slot_base[j]]));
    }
}

// ---------------------------------------------------------------------------
// Reverse Cuthill-McKee (intraRCM, :4000-4134) over all communities at once,
// level-synchronous like the BFS above:
//   * start: minimum degree, ties to the smaller id;
//   * communities above 32 vertices: up to three George-Liu sweeps, each a
//     BFS from the current node whose start is *not* marked visited (so it
//     reappears on level 2, as in the reference); while the eccentricity
//     grows, the next node is the minimum-degree vertex of the last level,
//     first in level order;
//   * Cuthill-McKee BFS: a level's children are ordered by (parent position,
//     degree, id) -- claims give (parent, row offset) order, a stable sort by
//     (parent, degree) finishes it;
//   * the reached part is reversed, unreached vertices follow in id order.
// ---------------------------------------------------------------------------
__global__ void k_rcm_start(const int64_t* __restrict__ slot_base, const int64_t* __restrict__ slot_size,
                            int32_t nslots, const uint32_t* __restrict__ order_v, const int64_t* __restrict__ rp,
                            unsigned long long* __restrict__ key) {
    for (int32_t j = blockIdx.y; j < nslots; j += gridDim.y) {
        const int64_t b = slot_base[j], sz = slot_size[j];
        unsigned long long best = ~0ull;
        for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < sz; k += (int64_t)gridDim.x * blockDim.x) {
            const uint32_t u = order_v[b + k];
            const unsigned long long kk = ((unsigned long long)(rp[u + 1] - rp[u]) << 32) | u;
            best = kk < best ? kk : best;
        }
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long t = __shfl_xor_sync(0xFFFFFFFFu, best, o);
            best = t < best ? t : best;
        }
        if ((threadIdx.x & 31) == 0) atomicMin(&key[j], best);
    }
}

// Frontier of a sweep: one start per participating slot, in slot order.
__global__ void k_rcm_frontier(int32_t nslots, const int32_t* __restrict__ part, const int64_t* __restrict__ pos,
                               const uint32_t* __restrict__ start, int mark, int32_t* __restrict__ F,
                               uint8_t* __restrict__ visited, int64_t* __restrict__ fs, int64_t* __restrict__ fe,
                               int64_t* __restrict__ qlen, int32_t* __restrict__ ecc,
                               unsigned long long* __restrict__ cand) {
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nslots; j += gridDim.x * blockDim.x) {
        fs[j] = pos[j];
        fe[j] = pos[j] + part[j];
        qlen[j] = part[j];
        ecc[j] = 0;
        cand[j] = ~0ull;
        if (part[j]) {
            F[pos[j]] = (int32_t)start[j];
            if (mark) visited[start[j]] = 1;
        }
    }
}

// Children in (parent, row offset) order with their parent's frontier index.
__global__ void k_rcm_write(const int32_t* __restrict__ F, int64_t nf, const int64_t* __restrict__ D, int64_t T,
                            const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                            const uint8_t* __restrict__ flag, const int64_t* __restrict__ P,
                            int32_t* __restrict__ nextF, int64_t* __restrict__ parent, uint8_t* __restrict__ visited) {
    for_frontier_edges(D, nf, T, [&](int64_t i, int64_t k, int64_t e) {
        if (!flag[e]) return;
        const int32_t w = col[rp[F[i]] + k];
        const int64_t p = P[e];
        nextF[p] = w;
        parent[p] = i;
        visited[w] = 1;
    });
}

// Last level of a slot whose next level is empty: minimum degree, first in
// level order (RCM) or smallest id (RCM++).
__global__ void k_rcm_last_level(const int32_t* __restrict__ F, int64_t nf, const int64_t* __restrict__ rp,
                                 const uint32_t* __restrict__ memb, const int32_t* __restrict__ slot_of_comm,
                                 const int64_t* __restrict__ bbase, const int64_t* __restrict__ bend, int by_id,
                                 unsigned long long* __restrict__ cand) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nf; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = F[i];
        const int32_t j = slot_of_comm[memb[u]];
        if (bend[j] != bbase[j]) continue;
        const unsigned long long tie = by_id ? (unsigned long long)(uint32_t)u : (unsigned long long)i;
        atomicMin(&cand[j], ((unsigned long long)(rp[u + 1] - rp[u]) << 32) | tie);
    }
}

__global__ void k_rcm_level_done(int32_t nslots, const int64_t* __restrict__ fs, const int64_t* __restrict__ fe,
                                 const int64_t* __restrict__ bbase, const int64_t* __restrict__ bend,
                                 const int32_t* __restrict__ F, int by_id, unsigned long long* __restrict__ cand,
                                 uint32_t* __restrict__ last_node, int32_t* __restrict__ ecc) {
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nslots; j += gridDim.x * blockDim.x) {
        if (fe[j] == fs[j]) continue;
        if (bend[j] > bbase[j]) {
            ++ecc[j];
        } else if (cand[j] != ~0ull) {
            const uint32_t lo = (uint32_t)(cand[j] & 0xFFFFFFFFull);
            last_node[j] = by_id ? lo : (uint32_t)F[lo];
            cand[j] = ~0ull;
        }
    }
}

// RCM++ start (RG:4185-4256): depth of each reached vertex from the seed.
__global__ void k_rcm_depth(const int32_t* __restrict__ F, int64_t nf, uint32_t level, uint32_t* __restrict__ depth) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nf; i += (int64_t)gridDim.x * blockDim.x)
        depth[F[i]] = level;
}

// Rank keys over the placement skeleton: (community rank, degree) or
// (community rank, ~depth); a stable sort keeps vertex order for ties.
__global__ void k_rcmpp_keys(const uint32_t* __restrict__ order_v, const uint32_t* __restrict__ ranks, int64_t nn,
                             const int64_t* __restrict__ rp, const uint32_t* __restrict__ depth, int low_bits,
                             uint32_t max_depth, int by_depth, uint64_t* __restrict__ keys,
                             uint32_t* __restrict__ pos) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nn; p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t v = order_v[p];
        const uint64_t low = by_depth ? (uint64_t)(max_depth - depth[v]) : (uint64_t)(rp[v + 1] - rp[v]);
        keys[p] = ((uint64_t)ranks[p] << low_bits) | low;
        pos[p] = (uint32_t)p;
    }
}

__global__ void k_rcmpp_rank(const uint32_t* __restrict__ sorted_pos, const uint32_t* __restrict__ ranks,
                             const int64_t* __restrict__ offs, int64_t nn, int64_t* __restrict__ score) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t p = sorted_pos[i];
        score[p] += i - offs[ranks[p]];
    }
}

// Least degree rank + depth rank per participating slot, ties to the smaller id.
__global__ void k_rcmpp_pick(const uint32_t* __restrict__ order_v, int64_t nn, const uint32_t* __restrict__ memb,
                             const int32_t* __restrict__ slot_of_comm, const int32_t* __restrict__ part,
                             const int64_t* __restrict__ score, unsigned long long* __restrict__ best) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nn; p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t v = order_v[p];
        const int32_t j = slot_of_comm[memb[v]];
        if (j < 0 || !part[j]) continue;
        atomicMin(&best[j], ((unsigned long long)score[p] << 32) | v);
    }
}

__global__ void k_rcmpp_start(int32_t nslots, const int32_t* __restrict__ part,
                              const unsigned long long* __restrict__ best, uint32_t* __restrict__ start) {
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nslots; j += gridDim.x * blockDim.x)
        if (part[j] && best[j] != ~0ull) start[j] = (uint32_t)(best[j] & 0xFFFFFFFFull);
}

// George-Liu step: keep sweeping while the eccentricity grows.
__global__ void k_rcm_gl_step(int32_t nslots, int32_t* __restrict__ part, const int32_t* __restrict__ ecc,
                              int32_t* __restrict__ prev_ecc, const uint32_t* __restrict__ last_node,
                              uint32_t* __restrict__ start, int32_t* __restrict__ still) {
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nslots; j += gridDim.x * blockDim.x) {
        if (!part[j]) continue;
        if (ecc[j] <= prev_ecc[j]) {
            part[j] = 0;
            continue;
        }
        prev_ecc[j] = ecc[j];
        start[j] = last_node[j];
        atomicAdd(still, 1);
    }
}

__global__ void k_rcm_keys(const int32_t* __restrict__ NF, const int64_t* __restrict__ parent, int64_t cnt,
                           const int64_t* __restrict__ rp, int degbits, uint64_t* __restrict__ keys,
                           uint32_t* __restrict__ vals) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < cnt; p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t w = NF[p];
        keys[p] = ((uint64_t)parent[p] << degbits) | (uint64_t)(rp[w + 1] - rp[w]);
        vals[p] = (uint32_t)w;
    }
}

__global__ void k_rcm_assign(const uint32_t* __restrict__ sorted, int64_t cnt, const uint32_t* __restrict__ memb,
                             const int32_t* __restrict__ slot_of_comm, const int64_t* __restrict__ qlen,
                             const int64_t* __restrict__ bbase, int32_t* __restrict__ NF,
                             uint32_t* __restrict__ local) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < cnt; p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t w = sorted[p];
        const int32_t j = slot_of_comm[memb[w]];
        NF[p] = (int32_t)w;
        local[w] = (uint32_t)(qlen[j] + (p - bbase[j]));
    }
}

// Reverse the reached part: local = reached - 1 - Cuthill-McKee position.
__global__ void k_rcm_reverse(const uint32_t* __restrict__ order_v, int64_t nn, const uint32_t* __restrict__ memb,
                              const int32_t* __restrict__ slot_of_comm, const uint8_t* __restrict__ visited,
                              const int64_t* __restrict__ qlen, uint32_t* __restrict__ local) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nn; p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t v = order_v[p];
        const int32_t j = slot_of_comm[memb[v]];
        if (j >= 0 && visited[v]) local[v] = (uint32_t)(qlen[j] - 1 - local[v]);
    }
}

__global__ void k_rcm_init_slots(int32_t nslots, const int64_t* __restrict__ slot_size,
                                 const unsigned long long* __restrict__ key, uint32_t* __restrict__ start,
                                 int32_t* __restrict__ part, int32_t* __restrict__ prev_ecc) {
    for (int32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nslots; j += gridDim.x * blockDim.x) {
        start[j] = (uint32_t)(key[j] & 0xFFFFFFFFull);
        part[j] = slot_size[j] > 32 ? 1 : 0;
        prev_ecc[j] = 0;
    }
}

__global__ void k_max_degree_of(const int32_t* __restrict__ list, int64_t cnt, const int64_t* __restrict__ rp,
                                unsigned long long* __restrict__ out) {
    unsigned long long m = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < cnt; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = list[i];
        const unsigned long long d = (unsigned long long)(rp[u + 1] - rp[u]);
        m = d > m ? d : m;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xFFFFFFFFu, m, o);
        m = t > m ? t : m;
    }
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

__global__ void k_fill_i32(int32_t* p, int64_t n, int32_t v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

__global__ void k_gather_local(const uint32_t* __restrict__ order_v, const uint32_t* __restrict__ local_by_pos,
                               const uint8_t* __restrict__ mark, int64_t nn, uint32_t* __restrict__ local) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nn; p += (int64_t)gridDim.x * blockDim.x)
        if (mark[p]) local[order_v[p]] = local_by_pos[p];
}

__global__ void k_final_assign(const uint32_t* __restrict__ order_v, const uint32_t* __restrict__ keys_sorted,
                               const int64_t* __restrict__ offs, const uint32_t* __restrict__ local, int64_t n,
                               uint32_t C, int32_t* __restrict__ new_ids) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t v = order_v[p];
        const uint32_t r = keys_sorted[p];
        new_ids[v] = (r < C) ? (int32_t)(offs[r] + local[v]) : (int32_t)p;
    }
}

template <typename T>
T read_dev(const T* p, cudaStream_t s) {
    T h;
    GB_CUDA(cudaMemcpyAsync(&h, p, sizeof(T), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    return h;
}

}  // namespace

// Reverse Cuthill-McKee for the listed communities (see the kernels above).
// Returns the number of BFS levels run.
int64_t rcm_communities(const DeviceCSR& g, const uint32_t* memb, const int32_t* blist, const int32_t* count_p,
                        int32_t nslots, const uint32_t* order_v, const uint32_t* ranks, const int64_t* offs,
                        const int64_t* ssize, int64_t C, int64_t nn, uint32_t largest, bool pp, uint32_t* local,
                        cudaStream_t s, int64_t* launches) {
    const int64_t n = g.n;
    DevBuf<int32_t> slot_of_comm(C, s);
    GB_CUDA(cudaMemsetAsync(slot_of_comm, 0xFF, C * sizeof(int32_t), s));
    DevBuf<int64_t> slot_base(nslots, s), slot_size(nslots, s), qlen(nslots, s), fs(nslots, s), fe(nslots, s),
        bbase(nslots, s), bend(nslots, s), pos(nslots + 1, s);
    k_bfs_slots<<<grid_for(nslots, kT), kT, 0, s>>>(blist, count_p, order_v, offs, memb, slot_of_comm, slot_base,
                                                    slot_size, ssize);
    GB_LAUNCH_CHECK();
    DevBuf<unsigned long long> key(nslots, s), cand(nslots, s);
    GB_CUDA(cudaMemsetAsync(key, 0xFF, nslots * sizeof(unsigned long long), s));
    {
        dim3 grid((unsigned)std::min<int64_t>(ceil_div(largest, kT), 64), (unsigned)std::min(nslots, 65535));
        k_rcm_start<<<grid, kT, 0, s>>>(slot_base, slot_size, nslots, order_v, g.row_ptr, key);
        GB_LAUNCH_CHECK();
    }
    DevBuf<uint32_t> start(nslots, s), last_node(nslots, s);
    DevBuf<int32_t> part(nslots, s), prev_ecc(nslots, s), ecc(nslots, s), still(1, s);
    k_rcm_init_slots<<<grid_for(nslots, kT), kT, 0, s>>>(nslots, slot_size, key, start, part, prev_ecc);
    GB_LAUNCH_CHECK();
    *launches += 4;
    DevBuf<uint8_t> visited(n, s);
    DevBuf<unsigned long long> claim(n, s);
    DevBuf<int32_t> F(nn + 1, s), NF(nn + 1, s);
    DevBuf<int64_t> D(nn + 1, s), parent(nn + 1, s);
    int64_t levels = 0;
    DevBuf<uint32_t> depth(pp ? n : 0, s);
    // One BFS over the participating slots: a George-Liu sweep, the
    // Cuthill-McKee order (cm), or the RCM++ depths from the seed (dep).
    auto sweep = [&](bool cm, bool dep = false) -> void {
        exclusive_scan_i32_to_i64(part, pos, nslots, pos.get() + nslots, s);
        const int64_t np = read_dev(pos.get() + nslots, s);
        GB_CUDA(cudaMemsetAsync(visited, 0, n, s));
        GB_CUDA(cudaMemsetAsync(claim, 0xFF, n * sizeof(unsigned long long), s));
        k_rcm_frontier<<<grid_for(nslots, kT), kT, 0, s>>>(nslots, part, pos, start, (cm || dep) ? 1 : 0, F,
                                                           visited, fs, fe, qlen, ecc, cand);
        GB_LAUNCH_CHECK();
        *launches += 4;
        if (cm) {
            // the start is Cuthill-McKee position 0 of its community
            DevBuf<uint32_t> sorted(np > 0 ? np : 1, s);
            GB_CUDA(cudaMemsetAsync(bbase, 0, nslots * sizeof(int64_t), s));
            GB_CUDA(cudaMemcpyAsync(sorted, F.get(), np * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
            DevBuf<int64_t> zero(nslots, s);
            GB_CUDA(cudaMemsetAsync(zero, 0, nslots * sizeof(int64_t), s));
            k_rcm_assign<<<grid_for(np, kT), kT, 0, s>>>(sorted, np, memb, slot_of_comm, zero, pos, F, local);
            GB_LAUNCH_CHECK();
            *launches += 1;
        }
        int64_t nf = np;
        uint32_t level = 0;
        while (nf > 0) {
            ++levels;
            if (dep) {
                k_rcm_depth<<<grid_for(nf, kT), kT, 0, s>>>(F, nf, level, depth);
                GB_LAUNCH_CHECK();
                ++*launches;
            }
            ++level;
            k_frontier_degrees<<<grid_for(nf, kT), kT, 0, s>>>(F, nf, g.row_ptr, D);
            GB_LAUNCH_CHECK();
            exclusive_scan_i64_total(D, D, nf, D.get() + nf, s);
            const int64_t T = read_dev(D.get() + nf, s);
            DevBuf<uint8_t> flag(T > 0 ? T : 1, s);
            DevBuf<int64_t> P(T + 1, s);
            if (T > 0) {
                k_bfs_claim<<<edge_grid(T), 256, 0, s>>>(F, nf, D, T, g.row_ptr, g.col, memb, visited, claim);
                GB_LAUNCH_CHECK();
                k_bfs_flag<<<edge_grid(T), 256, 0, s>>>(F, nf, D, T, g.row_ptr, g.col, memb, visited, claim, flag);
                GB_LAUNCH_CHECK();
                exclusive_scan_u8_to_i64(flag, P, T, P.get() + T, s);
            } else {
                GB_CUDA(cudaMemsetAsync(P, 0, sizeof(int64_t), s));
            }
            k_bfs_bases<<<grid_for(nslots, kT), kT, 0, s>>>(nslots, fs, fe, D, P, bbase, bend);
            GB_LAUNCH_CHECK();
            if (T > 0) {
                k_rcm_write<<<edge_grid(T), 256, 0, s>>>(F, nf, D, T, g.row_ptr, g.col, flag, P, NF, parent,
                                                           visited);
                GB_LAUNCH_CHECK();
            }
            const int64_t next = T > 0 ? read_dev(P.get() + T, s) : 0;
            if (!cm && !dep) {
                k_rcm_last_level<<<grid_for(nf, kT), kT, 0, s>>>(F, nf, g.row_ptr, memb, slot_of_comm, bbase, bend,
                                                                 pp ? 1 : 0, cand);
                GB_LAUNCH_CHECK();
                k_rcm_level_done<<<grid_for(nslots, kT), kT, 0, s>>>(nslots, fs, fe, bbase, bend, F, pp ? 1 : 0, cand,
                                                                     last_node, ecc);
                GB_LAUNCH_CHECK();
            } else if (cm && next > 0) {
                // Children of one parent by (degree, id): stable sort by (parent, degree).
                unsigned long long md = 0;
                {
                    DevBuf<unsigned long long> mdd(1, s);
                    GB_CUDA(cudaMemsetAsync(mdd, 0, sizeof(unsigned long long), s));
                    k_max_degree_of<<<grid_for(next, kT), kT, 0, s>>>(NF, next, g.row_ptr, mdd);
                    GB_LAUNCH_CHECK();
                    md = read_dev(mdd.get(), s);
                }
                const int degbits = bits_for(md);
                const int pbits = bits_for((uint64_t)(nf > 1 ? nf - 1 : 1));
                DevBuf<uint64_t> keys(next, s);
                DevBuf<uint32_t> vals(next, s);
                k_rcm_keys<<<grid_for(next, kT), kT, 0, s>>>(NF, parent, next, g.row_ptr, degbits, keys, vals);
                GB_LAUNCH_CHECK();
                radix_sort_pairs_u64(keys, vals, next, degbits + pbits, s);
                k_rcm_assign<<<grid_for(next, kT), kT, 0, s>>>(vals, next, memb, slot_of_comm, qlen, bbase, NF,
                                                               local);
                GB_LAUNCH_CHECK();
                *launches += 4 + 3 * ((degbits + pbits + 7) / 8);
            }
            k_bfs_advance<<<grid_for(nslots, kT), kT, 0, s>>>(nslots, qlen, fs, fe, bbase, bend);
            GB_LAUNCH_CHECK();
            *launches += 8;
            std::swap(F.ptr, NF.ptr);
            nf = next;
        }
    };
    if (pp) {
        // RCM++ start for the communities above 32 vertices: BFS depths from
        // the seed, ranks by (degree, id) and (depth descending, id), least sum.
        int32_t np_host = 0;
        {
            DevBuf<int64_t> tot(1, s);
            exclusive_scan_i32_to_i64(part, pos, nslots, tot, s);
            np_host = (int32_t)read_dev(tot.get(), s);
        }
        if (np_host > 0) {
            GB_CUDA(cudaMemsetAsync(depth, 0, n * sizeof(uint32_t), s));
            sweep(false, true);
            DevBuf<unsigned long long> mx(1, s);
            GB_CUDA(cudaMemsetAsync(mx, 0, sizeof(unsigned long long), s));
            k_max_degree_of<<<grid_for(nn, kT), kT, 0, s>>>(reinterpret_cast<const int32_t*>(order_v), nn, g.row_ptr,
                                                            mx);
            GB_LAUNCH_CHECK();
            const int degbits = bits_for(read_dev(mx.get(), s));
            const uint32_t max_depth = (uint32_t)std::max<int64_t>(0, levels);   // depth < levels run so far
            const int dbits = bits_for(max_depth);
            const int rbits = bits_for((uint64_t)(C > 1 ? C - 1 : 1));
            DevBuf<int64_t> score(nn, s);
            GB_CUDA(cudaMemsetAsync(score, 0, nn * sizeof(int64_t), s));
            DevBuf<uint64_t> keys(nn, s);
            DevBuf<uint32_t> sp(nn, s);
            for (int by_depth = 0; by_depth < 2; ++by_depth) {
                const int low = by_depth ? dbits : degbits;
                k_rcmpp_keys<<<grid_for(nn, kT), kT, 0, s>>>(order_v, ranks, nn, g.row_ptr, depth.get(), low, max_depth,
                                                            by_depth, keys, sp);
                GB_LAUNCH_CHECK();
                radix_sort_pairs_u64(keys, sp, nn, low + rbits, s);
                k_rcmpp_rank<<<grid_for(nn, kT), kT, 0, s>>>(sp, ranks, offs, nn, score);
                GB_LAUNCH_CHECK();
                *launches += 2 + 3 * ((low + rbits + 7) / 8);
            }
            DevBuf<unsigned long long> best(nslots, s);
            GB_CUDA(cudaMemsetAsync(best, 0xFF, nslots * sizeof(unsigned long long), s));
            k_rcmpp_pick<<<grid_for(nn, kT), kT, 0, s>>>(order_v, nn, memb, slot_of_comm, part, score, best);
            GB_LAUNCH_CHECK();
            k_rcmpp_start<<<grid_for(nslots, kT), kT, 0, s>>>(nslots, part, best, start);
            GB_LAUNCH_CHECK();
            *launches += 3;
        }
    }
    // George-Liu sweeps (communities above 32 vertices), at most three.
    for (int it = 0; it < 3; ++it) {
        int32_t np_host = 0;
        {
            DevBuf<int64_t> tot(1, s);
            exclusive_scan_i32_to_i64(part, pos, nslots, tot, s);
            np_host = (int32_t)read_dev(tot.get(), s);
        }
        if (np_host == 0) break;
        sweep(false);
        GB_CUDA(cudaMemsetAsync(still, 0, sizeof(int32_t), s));
        k_rcm_gl_step<<<grid_for(nslots, kT), kT, 0, s>>>(nslots, part, ecc, prev_ecc, last_node, start, still);
        GB_LAUNCH_CHECK();
        *launches += 2;
        if (read_dev(still.get(), s) == 0) break;
    }
    // Cuthill-McKee BFS from the final starts, all communities.
    k_fill_i32<<<grid_for(nslots, kT), kT, 0, s>>>(part, nslots, 1);
    GB_LAUNCH_CHECK();
    sweep(true);
    // Reverse the reached part; unreached vertices follow in vertex order.
    k_rcm_reverse<<<grid_for(nn, kT), kT, 0, s>>>(order_v, nn, memb, slot_of_comm, visited, qlen, local);
    GB_LAUNCH_CHECK();
    DevBuf<int32_t> lflag(nn, s);
    DevBuf<int64_t> R(nn + 1, s);
    k_bfs_left_flags<<<grid_for(nn, kT), kT, 0, s>>>(order_v, nn, memb, slot_of_comm, visited, lflag);
    GB_LAUNCH_CHECK();
    exclusive_scan_i32_to_i64(lflag, R, nn, R.get() + nn, s);
    k_bfs_left_assign<<<grid_for(nn, kT), kT, 0, s>>>(order_v, nn, memb, slot_of_comm, lflag, R, slot_base, qlen,
                                                      local);
    GB_LAUNCH_CHECK();
    *launches += 7;
    return levels;
}

void compose_device(const DeviceCSR& g, const uint32_t* memb, const ComposeParams& p, int32_t* new_ids,
                    gbgpu_stats* st, cudaStream_t s) {
    const int64_t n = g.n;
    if (n == 0) return;
    int intra = p.intra_order;
    if (intra == kIntraDendrogram) intra = kIntraBFS;  // Leiden has no Rabbit dendrogram (:6668-6677)
    const bool sorted_intra = is_sorted_intra_order(intra);
    const bool random_intra = intra == kIntraRandom;
    GB_REQUIRE(intra == kIntraBFS || intra == kIntraGorder || intra == kIntraRCM || intra == kIntraRCMpp ||
                   sorted_intra || random_intra,
               GBGPU_E_UNSUPPORTED, "intra-community order not available on the GPU path");
    const int co = p.community_order;
    GB_REQUIRE(co == kSizeDesc || co == kSizeAsc || co == kDegreeDesc || co == kDegreeAsc || co == kIdentity,
               GBGPU_E_UNSUPPORTED, "community order not available on the GPU path");
    GB_REQUIRE(intra != kIntraGorder || p.gorder_window > 0, GBGPU_E_INVALID,
               "Local Gorder requires a positive window");
    GB_REQUIRE(p.gorder_window <= 100, GBGPU_E_INVALID, "Gorder window above 100");
    int64_t launches = 0;
    cudaEvent_t ev0, ev1;
    GB_CUDA(cudaEventCreate(&ev0));
    GB_CUDA(cudaEventCreate(&ev1));
    GB_CUDA(cudaEventRecord(ev0, s));

    // numComm = max(membership) + 1 (:6338-6343).
    DevBuf<uint32_t> scal(4, s);
    GB_CUDA(cudaMemsetAsync(scal, 0, 4 * sizeof(uint32_t), s));
    k_max_u32<<<grid_for(n, kT), kT, 0, s>>>(memb, n, scal.get());
    GB_LAUNCH_CHECK();
    const int64_t C = (int64_t)read_dev(scal.get(), s) + 1;
    GB_REQUIRE(C <= n, GBGPU_E_INVALID, "membership ids must be < n");

    DevBuf<uint32_t> csize(C, s);
    GB_CUDA(cudaMemsetAsync(csize, 0, C * sizeof(uint32_t), s));
    const bool need_deg = (co == kDegreeDesc || co == kDegreeAsc);
    DevBuf<unsigned long long> cdeg(need_deg ? C : 0, s);
    if (need_deg) GB_CUDA(cudaMemsetAsync(cdeg, 0, C * sizeof(unsigned long long), s));
    k_comm_sizes<<<grid_for(n, kT), kT, 0, s>>>(g.row_ptr, memb, n, csize, need_deg ? cdeg.get() : nullptr);
    GB_LAUNCH_CHECK();

    // Community order: stable sort of 0..C-1 by the order key.
    DevBuf<uint32_t> comm_order(C, s);
    {
        DevBuf<unsigned long long> maxdeg(1, s);
        GB_CUDA(cudaMemsetAsync(scal, 0, sizeof(uint32_t), s));
        GB_CUDA(cudaMemsetAsync(maxdeg, 0, sizeof(unsigned long long), s));
        k_max_u32_u64<<<grid_for(C, kT), kT, 0, s>>>(csize, need_deg ? cdeg.get() : nullptr, C, scal.get(), maxdeg.get());
        GB_LAUNCH_CHECK();
        const uint32_t max_size = read_dev(scal.get(), s);
        const unsigned long long max_deg = read_dev(maxdeg.get(), s);
        DevBuf<uint32_t> stage1;
        if (p.super_order != 0) {
            stage1.alloc(C, s);
            super_order_device(g, memb, csize, C, p.super_order, p.super_gamma, stage1, s, &launches);
        }
        DevBuf<uint64_t> keys(C, s);
        k_comm_keys<<<grid_for(C, kT), kT, 0, s>>>(co, csize, need_deg ? cdeg.get() : nullptr, C, max_size, max_deg,
                                                   stage1.get(), keys, comm_order);
        GB_LAUNCH_CHECK();
        int kbits = 0;
        if (co == kSizeDesc || co == kSizeAsc) kbits = bits_for(max_size);
        else if (co == kDegreeDesc || co == kDegreeAsc) kbits = bits_for(max_deg);
        radix_sort_pairs_u64(keys, comm_order, C, kbits, s);
        launches += 4 + 3 * ((kbits + 7) / 8);
    }
    DevBuf<uint32_t> rank(C, s);
    DevBuf<int64_t> ssize(C, s);
    DevBuf<int64_t> offs(C + 1, s);
    k_rank<<<grid_for(C, kT), kT, 0, s>>>(comm_order, csize, C, rank, ssize);
    GB_LAUNCH_CHECK();
    exclusive_scan_i64_total(ssize, offs, C, offs.get() + C, s);
    const int64_t nn = read_dev(offs.get() + C, s);  // non-isolated vertices

    // Placement skeleton: stable sort of (rank(community) | C for isolated, v).
    DevBuf<uint32_t> vkeys(n, s), order_v(n, s);
    k_vertex_keys<<<grid_for(n, kT), kT, 0, s>>>(g.row_ptr, memb, rank, n, (uint32_t)C, vkeys, order_v);
    GB_LAUNCH_CHECK();
    const int vbits = bits_for((uint64_t)C);
    radix_sort_pairs_u32(vkeys, order_v, n, vbits, s);
    DevBuf<int64_t> pos_of(n, s);
    DevBuf<uint32_t> local(n, s);
    k_positions<<<grid_for(n, kT), kT, 0, s>>>(order_v, vkeys, offs, n, (uint32_t)C, pos_of, local);
    GB_LAUNCH_CHECK();
    launches += 6 + 3 * ((vbits + 7) / 8);

    // Classify communities.
    DevBuf<int32_t> lists(5 * C, s);
    DevBuf<ClassCounts> cc(1, s);
    GB_CUDA(cudaMemsetAsync(cc, 0, sizeof(ClassCounts), s));
    k_classify<<<grid_for(C, kT), kT, 0, s>>>(ssize, C, intra, p.gorder_fallback, lists, cc);
    GB_LAUNCH_CHECK();
    ClassCounts hc = read_dev(cc.get(), s);
    launches += 1;

    cudaEvent_t ev_intra0, ev_intra1;
    GB_CUDA(cudaEventCreate(&ev_intra0));
    GB_CUDA(cudaEventCreate(&ev_intra1));
    GB_CUDA(cudaEventRecord(ev_intra0, s));

    // ---- Gorder communities ----
    const int32_t ng = hc.n[1] + hc.n[2] + hc.n[3];
    if (ng > 0) {
        DevBuf<uint8_t> mark(nn, s);
        GB_CUDA(cudaMemsetAsync(mark, 0, nn, s));
        for (int cls = 1; cls <= 3; ++cls) {
            if (hc.n[cls] == 0) continue;
            k_mark_gorder_positions<<<kNumSMs * 8, kT, 0, s>>>(lists.get() + cls * C, cc.get()->n + cls, offs, ssize, mark);
            GB_LAUNCH_CHECK();
            ++launches;
        }
        DevBuf<int64_t> loff(nn + 1, s);
        k_local_count<<<grid_for(nn, kT), kT, 0, s>>>(g.row_ptr, g.col, memb, order_v, mark, nn, loff);
        GB_LAUNCH_CHECK();
        exclusive_scan_i64_total(loff, loff, nn, loff.get() + nn, s);
        const int64_t ltot = read_dev(loff.get() + nn, s);
        const bool wide = hc.gorder_max > 65535;
        DevBuf<uint16_t> l16(wide ? 0 : (ltot > 0 ? ltot : 1), s);
        DevBuf<uint32_t> l32(wide ? (ltot > 0 ? ltot : 1) : 0, s);
        k_local_fill<<<grid_for(nn, kT), kT, 0, s>>>(g.row_ptr, g.col, memb, order_v, mark, local, loff, nn,
                                                     l16.get(), wide ? l32.get() : nullptr);
        GB_LAUNCH_CHECK();
        DevBuf<uint32_t> local_by_pos(nn, s);
        GB_CUDA(cudaMemsetAsync(local_by_pos, 0, nn * sizeof(uint32_t), s));
        launches += 5;
        auto run = [&](auto* ladj) {
            using LT = std::remove_pointer_t<decltype(ladj)>;
            if (hc.n[1] > 0) {
                k_gorder_thread<LT><<<grid_for(hc.n[1], 64), 64, 0, s>>>(lists.get() + 1 * C, cc.get()->n + 1, offs,
                                                                          ssize, order_v, g.row_ptr, ladj, loff,
                                                                          p.gorder_window, local_by_pos);
                GB_LAUNCH_CHECK();
                ++launches;
            }
            if (hc.n[2] > 0) {
                // Workspace sized by this call's largest community of the class
                // (occupancy follows it); the attribute is the one constant
                // maximum, so concurrent callers never race on it.
                const int nb = p.gorder_window + 2;
                const int64_t cap = std::min<int64_t>(kSmemGorderMax, std::max<int64_t>(hc.gorder_max, 33));
                const int smem = (int)(sizeof(int) * lazy_ws_ints(cap, nb, p.gorder_window));
                GB_CUDA(cudaFuncSetAttribute(k_gorder_warp<LT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(sizeof(int) * lazy_ws_ints(kSmemGorderMax, kMaxGorderWindow + 2,
                                                                              kMaxGorderWindow))));
                int per_sm = 1;
                GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gorder_warp<LT, true>, 32, smem));
                const int grid = std::min<int>(hc.n[2], kNumSMs * std::max(1, per_sm));
                k_gorder_warp<LT, true><<<grid, 32, smem, s>>>(lists.get() + 2 * C, cc.get()->n + 2, offs, ssize,
                                                               order_v, g.row_ptr, ladj, loff, p.gorder_window,
                                                               local_by_pos, nullptr, cap);
                GB_LAUNCH_CHECK();
                ++launches;
            }
            if (hc.n[3] > 0) {
                const int grid = std::min<int>(hc.n[3], kNumSMs * 4);
                const int64_t cap = hc.gorder_max;
                const int nb = p.gorder_window + 2;
                DevBuf<int> gws((int64_t)grid * lazy_ws_ints(cap, nb, p.gorder_window), s);
                k_gorder_warp<LT, false><<<grid, 32, 0, s>>>(lists.get() + 3 * C, cc.get()->n + 3, offs, ssize,
                                                             order_v, g.row_ptr, ladj, loff, p.gorder_window,
                                                             local_by_pos, gws, cap);
                GB_LAUNCH_CHECK();
                ++launches;
            }
        };
        if (wide) run(l32.get()); else run(l16.get());
        k_gather_local<<<grid_for(nn, kT), kT, 0, s>>>(order_v, local_by_pos, mark, nn, local);
        GB_LAUNCH_CHECK();
        ++launches;
    }

    // ---- RCM: every community of two or more vertices ----
    const int32_t nbfs = hc.n[4];
    int64_t levels = 0;
    if (nbfs > 0 && (intra == kIntraRCM || intra == kIntraRCMpp)) {
        levels = rcm_communities(g, memb, lists.get() + 4 * C, cc.get()->n + 4, nbfs, order_v, vkeys, offs, ssize, C,
                                 nn, hc.largest, intra == kIntraRCMpp, local, s, &launches);
    }
    // ---- sorted orders: every community ----
    if (sorted_intra) sorted_communities(g, memb, intra, order_v, vkeys, offs, ssize, nn, local, s, &launches);
    // ---- intra_random: every community of two or more vertices ----
    if (random_intra)
        random_communities(memb, order_v, vkeys, offs, ssize, lists.get() + 4 * C, cc.get()->n + 4, nbfs, nn, local, s,
                           &launches);
    // ---- BFS communities ----
    if (nbfs > 0 && intra != kIntraRCM && intra != kIntraRCMpp && !sorted_intra && !random_intra) {
        const int32_t* blist = lists.get() + 4 * C;
        DevBuf<int32_t> slot_of_comm(C, s);
        GB_CUDA(cudaMemsetAsync(slot_of_comm, 0xFF, C * sizeof(int32_t), s));
        DevBuf<int64_t> slot_base(nbfs, s), slot_size(nbfs, s), qlen(nbfs, s), fs(nbfs, s), fe(nbfs, s),
            bbase(nbfs, s), bend(nbfs, s);
        k_bfs_slots<<<grid_for(nbfs, kT), kT, 0, s>>>(blist, cc.get()->n + 4, order_v, offs, memb, slot_of_comm,
                                                      slot_base, slot_size, ssize);
        GB_LAUNCH_CHECK();
        DevBuf<unsigned long long> hubkey(nbfs, s);
        GB_CUDA(cudaMemsetAsync(hubkey, 0, nbfs * sizeof(unsigned long long), s));
        {
            dim3 grid((unsigned)std::min<int64_t>(ceil_div(hc.largest, kT), 64), (unsigned)std::min(nbfs, 65535));
            k_bfs_hubs<<<grid, kT, 0, s>>>(slot_base, slot_size, nbfs, order_v, g.row_ptr, hubkey);
            GB_LAUNCH_CHECK();
        }
        DevBuf<uint8_t> visited(n, s);
        GB_CUDA(cudaMemsetAsync(visited, 0, n, s));
        DevBuf<unsigned long long> claim(n, s);
        GB_CUDA(cudaMemsetAsync(claim, 0xFF, n * sizeof(unsigned long long), s));
        DevBuf<int32_t> F(nn + 1, s), NF(nn + 1, s);
        k_bfs_init<<<grid_for(nbfs, kT), kT, 0, s>>>(hubkey, slot_base, nbfs, order_v, F, visited, local, qlen, fs, fe);
        GB_LAUNCH_CHECK();
        launches += 3;
        int64_t nf = nbfs;
        DevBuf<int64_t> D(nn + 1, s);
        while (nf > 0) {
            ++levels;
            k_frontier_degrees<<<grid_for(nf, kT), kT, 0, s>>>(F, nf, g.row_ptr, D);
            GB_LAUNCH_CHECK();
            exclusive_scan_i64_total(D, D, nf, D.get() + nf, s);
            const int64_t T = read_dev(D.get() + nf, s);
            if (T == 0) break;
            DevBuf<uint8_t> flag(T, s);
            DevBuf<int64_t> P(T + 1, s);
            k_bfs_claim<<<edge_grid(T), 256, 0, s>>>(F, nf, D, T, g.row_ptr, g.col, memb, visited, claim);
            GB_LAUNCH_CHECK();
            k_bfs_flag<<<edge_grid(T), 256, 0, s>>>(F, nf, D, T, g.row_ptr, g.col, memb, visited, claim, flag);
            GB_LAUNCH_CHECK();
            exclusive_scan_u8_to_i64(flag, P, T, P.get() + T, s);
            k_bfs_bases<<<grid_for(nbfs, kT), kT, 0, s>>>(nbfs, fs, fe, D, P, bbase, bend);
            GB_LAUNCH_CHECK();
            k_bfs_write<<<edge_grid(T), 256, 0, s>>>(F, nf, D, T, g.row_ptr, g.col, memb, flag, P, slot_of_comm,
                                                       qlen, bbase, NF, visited, local);
            GB_LAUNCH_CHECK();
            k_bfs_advance<<<grid_for(nbfs, kT), kT, 0, s>>>(nbfs, qlen, fs, fe, bbase, bend);
            GB_LAUNCH_CHECK();
            const int64_t next = read_dev(P.get() + T, s);
            launches += 10;
            std::swap(F.ptr, NF.ptr);
            nf = next;
        }
        // Unreached vertices keep vertex order after the BFS order (:3978-3983).
        DevBuf<int32_t> lflag(nn, s);
        DevBuf<int64_t> R(nn + 1, s);
        k_bfs_left_flags<<<grid_for(nn, kT), kT, 0, s>>>(order_v, nn, memb, slot_of_comm, visited, lflag);
        GB_LAUNCH_CHECK();
        exclusive_scan_i32_to_i64(lflag, R, nn, R.get() + nn, s);
        k_bfs_left_assign<<<grid_for(nn, kT), kT, 0, s>>>(order_v, nn, memb, slot_of_comm, lflag, R, slot_base, qlen,
                                                          local);
        GB_LAUNCH_CHECK();
        launches += 5;
    }
    GB_CUDA(cudaEventRecord(ev_intra1, s));

    k_final_assign<<<grid_for(n, kT), kT, 0, s>>>(order_v, vkeys, offs, local, n, (uint32_t)C, new_ids);
    GB_LAUNCH_CHECK();
    launches += 1;
    GB_CUDA(cudaEventRecord(ev1, s));
    GB_CUDA(cudaEventSynchronize(ev1));
    if (st) {
        float ms = 0, ims = 0;
        cudaEventElapsedTime(&ms, ev0, ev1);
        cudaEventElapsedTime(&ims, ev_intra0, ev_intra1);
        st->compose_ms += ms;
        st->intra_ms += ims;
        st->num_communities = C;
        st->isolated = n - nn;
        st->gorder_communities = (int64_t)hc.gorder_communities;
        st->gorder_vertices = (int64_t)hc.gorder_vertices;
        st->gorder_max_community = hc.gorder_max;
        st->fallback_communities = (int64_t)hc.fallback_communities;
        st->fallback_vertices = (int64_t)hc.fallback_vertices;
        st->largest_community = hc.largest;
        st->bfs_levels = levels;
        st->kernel_launches += launches;
    }
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    cudaEventDestroy(ev_intra0);
    cudaEventDestroy(ev_intra1);
}

}  // namespace gb
