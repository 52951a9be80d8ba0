// leiden.cu -- GVE-style Leiden community detection on the device.
//
// Follows graphbrew::runGraphBrew in GVE_CSR mode without refinement
// (bench/include/graphbrew/reorder/reorder_graphbrew.h:7238-7571):
//   pass loop: local moving on the original graph (localMovingPhase<false>,
//   :1588-1734), community count and renumber (:1843-1889), GVE aggregation
//   with the batched super-graph move (aggregateGVEStyle, :2156-2439),
//   convergence checks (:7436-7452), tolerance drop per pass.
//
// Numerics: all edge weights are 1, so every community total and neighbour
// weight is an exact integer; they are kept as int64 / uint32 and converted to
// double only inside Delta-modularity, which is evaluated with explicitly
// rounded IEEE operations in the reference's association (no FMA contraction),
// so every delta equals the reference's bit for bit.
//
// Local moving (cd_parallel): asynchronous like the reference's OpenMP loop --
// vertices are processed in id order in launches of `chunk_vertices`; a warp
// per vertex accumulates neighbour communities (registers + __match_any_sync
// up to 32 neighbours, a shared-memory hash table up to 1024), a CTA per hub
// (a shared-memory or global hash table), community totals are updated with
// integer atomics, and later launches see every earlier move.
//
// Super-graph move (sgmb<k>): batches of k communities in id order; proposals
// read only the state before their batch and commits are commutative integer
// adds, so the result is independent of thread scheduling.  The whole move
// runs in one persistent CTA when the super-graph is small, otherwise one
// launch pair per batch.
#include <algorithm>
#include <cmath>
#include <vector>

#include "gb_chunks.cuh"
#include "gb_common.cuh"
#include "gb_leiden_internal.cuh"
#include "gb_stages.h"

namespace gb {

namespace {

constexpr int kT = 256;
constexpr int kLmWarpsPerBlock = 4;
struct LmArgs {
    const int64_t* rp;
    const int32_t* col;
    uint32_t* vcom;
    unsigned long long* ctot;   // int64 totals, two's complement adds
    uint8_t* vaff;
    double M, R;
    DqConst dq;
    double* total_delta;
    unsigned long long* moves;
};

// Vertex state read by the asynchronous engine: through L2 in stream mode,
// where a warp reads right after its own (atomic) updates.
template <bool kStream, typename T>
__device__ __forceinline__ T lm_load(const T* p) {
    if constexpr (kStream) return __ldcg(p);
    else return *p;
}

// Warp per vertex, degree <= kWarpMaxDeg.  Chunk mode: the warps of a launch
// take the vertices of [begin, end) round-robin.  Stream mode: warp w sweeps
// its own contiguous block of stream_len vertices in order, as one thread of
// the reference's parallel mode sweeps its block (racy across warps).
template <bool kStream>
__global__ void __launch_bounds__(kLmWarpsPerBlock * 32)
k_local_move_warp(LmArgs a, int64_t begin, int64_t end, int64_t stream_len) {
    extern __shared__ uint32_t lm_smem[];  // kLmWarpsPerBlock x (keys, vals) x kWarpHash
    __shared__ double sdelta[kLmWarpsPerBlock];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t* tk = lm_smem + (size_t)w * 2 * kWarpHash;
    uint32_t* tv = tk + kWarpHash;
    double acc_delta = 0.0;
    unsigned long long acc_moves = 0;
    const int64_t warps_total = (int64_t)gridDim.x * kLmWarpsPerBlock;
    const int64_t gw = (int64_t)blockIdx.x * kLmWarpsPerBlock + w;
    const int64_t u0 = kStream ? begin + gw * stream_len : begin + gw;
    const int64_t u1 = kStream ? min(end, u0 + stream_len) : end;
    const int64_t step = kStream ? 1 : warps_total;
    for (int64_t u = u0; u < u1; u += step) {
        const int64_t rb = a.rp[u];
        const int deg = (int)(a.rp[u + 1] - rb);
        if (deg > kWarpMaxDeg) continue;  // hub kernel
        if (!lm_load<kStream>(&a.vaff[u])) continue;
        const uint32_t d = lm_load<kStream>(&a.vcom[u]);
        double best_d = 0.0;
        uint32_t best_c = kNone;
        if (deg <= 32) {
            uint32_t c = kNone;
            if (lane < deg) {
                const int32_t v = a.col[rb + lane];
                if (v != (int32_t)u) c = lm_load<kStream>(&a.vcom[v]);
            }
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, c);
            const unsigned dmask = __ballot_sync(0xFFFFFFFFu, c == d);
            const int kud = __popc(dmask);
            const bool leader = (c != kNone) && (lane == __ffs(peers) - 1) && c != d;
            if (leader) {
                const long long sd = (long long)lm_load<kStream>(&a.ctot[d]);
                const long long sc = (long long)lm_load<kStream>(&a.ctot[c]);
                const double dl = delta_qi(a.dq, __popc(peers), kud, deg, sc, sd);
                if (dpos(dl)) { best_d = dl; best_c = c; }
            }
        } else {
            uint32_t H = 64;
            while (H < 2u * (uint32_t)deg) H <<= 1;
            const uint32_t mask = H - 1;
            for (uint32_t i = lane; i < H; i += 32) { tk[i] = kNone; tv[i] = 0; }
            __syncwarp();
            for (int base = 0; base < deg; base += 32) {
                uint32_t c = kNone;
                if (base + lane < deg) {
                    const int32_t v = a.col[rb + base + lane];
                    if (v != (int32_t)u) c = lm_load<kStream>(&a.vcom[v]);
                }
                const unsigned peers = __match_any_sync(0xFFFFFFFFu, c);
                if (c != kNone && lane == __ffs(peers) - 1) table_add(tk, tv, mask, c, (uint32_t)__popc(peers));
            }
            __syncwarp();
            const uint32_t kud = table_get(tk, tv, mask, d);
            const long long sd = (long long)lm_load<kStream>(&a.ctot[d]);
            for (uint32_t i = lane; i < H; i += 32) {
                const uint32_t c = tk[i];
                if (c == kNone || c == d) continue;
                const long long sc = (long long)lm_load<kStream>(&a.ctot[c]);
                const double dl = delta_qi(a.dq, tv[i], kud, deg, sc, sd);
                if (dpos(dl) && better_pos(dl, c, best_d, best_c)) { best_d = dl; best_c = c; }
            }
            __syncwarp();
        }
        warp_argmax_pos(best_d, best_c);
        if (best_d > 0.0 && best_c != d && best_c != kNone) {
            if (lane == 0) {
                atomicAdd(&a.ctot[d], (unsigned long long)(-(long long)deg));
                atomicAdd(&a.ctot[best_c], (unsigned long long)(long long)deg);
                a.vcom[u] = best_c;
                acc_moves += 1;
            }
            for (int i = lane; i < deg; i += 32) a.vaff[a.col[rb + i]] = 1;
            __syncwarp();
        } else {
            best_d = 0.0;
        }
        if (lane == 0) {
            a.vaff[u] = 0;
            acc_delta += best_d;
        }
    }
    if (lane == 0) sdelta[w] = acc_delta;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < kLmWarpsPerBlock; ++i) s += sdelta[i];
        if (s != 0.0) atomicAdd(a.total_delta, s);
    }
    if (lane == 0 && acc_moves) atomicAdd(a.moves, acc_moves);
}

// Id locality of a graph, sampled: for every 64th vertex u, the first 32
// entries of its row; counts entries v with |u - v| <= 64 (near) and all
// sampled entries.  A warp takes 32 sampled vertices, one coalesced row
// prefix at a time.
__global__ void __launch_bounds__(256)
k_near_sample(const int64_t* __restrict__ rp, const int32_t* __restrict__ col, int64_t n,
              unsigned long long* __restrict__ near_total) {
    const int lane = threadIdx.x & 31;
    const int64_t samples = (n + 63) / 64;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long near = 0, total = 0;
    for (int64_t s0 = gw * 32; s0 < samples; s0 += nw * 32) {
        const int64_t s1 = min(samples, s0 + 32);
        for (int64_t si = s0; si < s1; ++si) {
            const int64_t u = si * 64;
            const int64_t rb = rp[u];
            const int64_t len = rp[u + 1] - rb;
            const int64_t d = len < 32 ? len : 32;
            if (lane < d) {
                const int64_t v = col[rb + lane];
                near += (v - u <= 64 && u - v <= 64);
                ++total;
            }
        }
    }
    near = __reduce_add_sync(0xFFFFFFFFu, (unsigned)near);
    total = __reduce_add_sync(0xFFFFFFFFu, (unsigned)total);
    if (lane == 0 && total) {
        atomicAdd(&near_total[0], near);
        atomicAdd(&near_total[1], total);
    }
}

// CTA per hub vertex (degree > kWarpMaxDeg).  Table in shared memory when it
// fits, otherwise in this CTA's slice of a global workspace.
__global__ void __launch_bounds__(kHubThreads)
k_local_move_hub(LmArgs a, const uint32_t* __restrict__ hubs, int64_t hub_begin, int64_t hub_end,
                 uint32_t* __restrict__ gkeys, uint32_t* __restrict__ gvals, int64_t gcap) {
    extern __shared__ uint32_t sm[];
    __shared__ double red_d[kHubThreads / 32];
    __shared__ uint32_t red_c[kHubThreads / 32];
    __shared__ uint32_t s_kud;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int64_t hi = hub_begin + blockIdx.x; hi < hub_end; hi += gridDim.x) {
        const uint32_t u = hubs[hi];
        if (!a.vaff[u]) continue;
        const int64_t rb = a.rp[u];
        const int64_t deg = a.rp[u + 1] - rb;
        uint32_t H = 1024;
        while ((int64_t)H < 2 * deg) H <<= 1;
        uint32_t *tk, *tv;
        if (H <= (uint32_t)kHubSmemSlots) { tk = sm; tv = sm + kHubSmemSlots; }
        else { tk = gkeys + (int64_t)blockIdx.x * gcap; tv = gvals + (int64_t)blockIdx.x * gcap; }
        const uint32_t mask = H - 1;
        for (uint32_t i = threadIdx.x; i < H; i += blockDim.x) { tk[i] = kNone; tv[i] = 0; }
        __syncthreads();
        const uint32_t d = a.vcom[u];
        for (int64_t base = 0; base < deg; base += blockDim.x) {
            uint32_t c = kNone;
            if (base + threadIdx.x < deg) {
                const int32_t v = a.col[rb + base + threadIdx.x];
                if (v != (int32_t)u) c = a.vcom[v];
            }
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, c);
            if (c != kNone && lane == __ffs(peers) - 1) table_add(tk, tv, mask, c, (uint32_t)__popc(peers));
        }
        __syncthreads();
        if (threadIdx.x == 0) s_kud = table_get(tk, tv, mask, d);
        __syncthreads();
        const uint32_t kud = s_kud;
        const long long sd = (long long)a.ctot[d];
        double best_d = 0.0;
        uint32_t best_c = kNone;
        for (uint32_t i = threadIdx.x; i < H; i += blockDim.x) {
            const uint32_t c = tk[i];
            if (c == kNone || c == d) continue;
            const long long sc = (long long)a.ctot[c];
            const double dl = delta_qi(a.dq, tv[i], kud, deg, sc, sd);
            if (dpos(dl) && better_pos(dl, c, best_d, best_c)) { best_d = dl; best_c = c; }
        }
        warp_argmax_pos(best_d, best_c);
        if (lane == 0) { red_d[w] = best_d; red_c[w] = best_c; }
        __syncthreads();
        if (w == 0) {
            best_d = lane < (int)(blockDim.x / 32) ? red_d[lane] : 0.0;
            best_c = lane < (int)(blockDim.x / 32) ? red_c[lane] : kNone;
            warp_argmax_pos(best_d, best_c);
            if (lane == 0) { red_d[0] = best_d; red_c[0] = best_c; }
        }
        __syncthreads();
        best_d = red_d[0];
        best_c = red_c[0];
        const bool move = best_d > 0.0 && best_c != d && best_c != kNone;
        if (move) {
            if (threadIdx.x == 0) {
                atomicAdd(&a.ctot[d], (unsigned long long)(-(long long)deg));
                atomicAdd(&a.ctot[best_c], (unsigned long long)(long long)deg);
                a.vcom[u] = best_c;
                atomicAdd(a.moves, 1ull);
            }
            for (int64_t i = threadIdx.x; i < deg; i += blockDim.x) a.vaff[a.col[rb + i]] = 1;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            a.vaff[u] = 0;
            if (move) atomicAdd(a.total_delta, best_d);
        }
        __syncthreads();
    }
}

// ---- counting / renumbering ----
__global__ void k_mark_exists(const uint32_t* __restrict__ vcom, int64_t n, int32_t* __restrict__ exists) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        exists[vcom[v]] = 1;
}

// cmap (exclusive scan of exists) -> renumbered vcom; super weights.
__global__ void k_apply_renumber(uint32_t* __restrict__ vcom, int64_t n, const int64_t* __restrict__ cmap) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        vcom[v] = (uint32_t)cmap[vcom[v]];
}

__global__ void k_super_weights(const int32_t* __restrict__ exists, const int64_t* __restrict__ cmap,
                                const unsigned long long* __restrict__ ctot, int64_t n,
                                long long* __restrict__ sweight) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        if (exists[c]) sweight[cmap[c]] = (long long)ctot[c];
}

// Inter-community edges as keys (community(u) << 32 | community(v)), one
// entry-parallel pass: each CTA compacts its chunk's hits warp by warp and
// reserves their slots with one atomic on the cursor.  The keys are sorted
// next, so the order in which CTAs reserve does not reach the result.
constexpr int kInterThreads = 256;

__global__ void __launch_bounds__(kInterThreads)
k_inter_edges(const int64_t* __restrict__ rp, const int32_t* __restrict__ col, const uint32_t* __restrict__ vcom,
              int64_t n, int64_t nnz, const int32_t* __restrict__ chunk_row, uint64_t* __restrict__ keys,
              unsigned long long* __restrict__ cursor) {
    constexpr int kPer = kEdgeChunk / kInterThreads;
    __shared__ int32_t srow[kEdgeChunkPadded];
    __shared__ int32_t wmax[kInterThreads / 32];
    __shared__ uint32_t wcnt[kInterThreads / 32];
    __shared__ unsigned long long base;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const int64_t chunks = (nnz + kEdgeChunk - 1) / kEdgeChunk;
    for (int64_t c = blockIdx.x; c < chunks; c += gridDim.x) {
        const int64_t e0 = c * kEdgeChunk, e1 = min(nnz, e0 + kEdgeChunk);
        chunk_entry_rows<kInterThreads>(rp, n, chunk_row[c], e0, e1, srow, wmax);
        uint64_t key[kPer];
        unsigned hits[kPer];
        uint32_t cnt = 0;
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const int i = k * kInterThreads + t;
            bool hit = false;
            key[k] = 0;
            if (e0 + i < e1) {
                const uint32_t cu = vcom[srow[chunk_pad(i)]];
                const uint32_t cv = vcom[col[e0 + i]];
                hit = cu != cv;
                key[k] = ((uint64_t)cu << 32) | cv;
            }
            hits[k] = __ballot_sync(0xFFFFFFFFu, hit);
            cnt += __popc(hits[k]);
        }
        if (lane == 0) wcnt[warp] = cnt;
        __syncthreads();
        if (t == 0) {
            unsigned long long tot = 0;
            for (int w = 0; w < kInterThreads / 32; ++w) tot += wcnt[w];
            base = tot ? atomicAdd(cursor, tot) : 0ull;
        }
        __syncthreads();
        unsigned long long o = base;
        for (int w = 0; w < warp; ++w) o += wcnt[w];
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            if ((hits[k] >> lane) & 1u) keys[o + __popc(hits[k] & lt)] = key[k];
            o += __popc(hits[k]);
        }
        __syncthreads();  // srow, wcnt and base are reused by the next chunk
    }
}

// Run-length encode sorted keys: unique flags.
__global__ void k_rle_flags(const uint64_t* __restrict__ keys, int64_t m, int32_t* __restrict__ flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void k_rle_emit(const uint64_t* __restrict__ keys, int64_t m, const int32_t* __restrict__ flag,
                           const int64_t* __restrict__ pos, int64_t nuniq, uint32_t* __restrict__ snbr,
                           uint32_t* __restrict__ sw, int32_t* __restrict__ sdeg, int64_t* __restrict__ start) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        if (!flag[i]) continue;
        const int64_t p = pos[i];
        snbr[p] = (uint32_t)(keys[i] & 0xFFFFFFFFull);
        start[p] = i;
        atomicAdd(&sdeg[keys[i] >> 32], 1);
    }
}

__global__ void k_rle_weights(const int64_t* __restrict__ start, int64_t nuniq, int64_t m, uint32_t* __restrict__ sw) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nuniq; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = (p + 1 < nuniq) ? start[p + 1] : m;
        sw[p] = (uint32_t)(e - start[p]);
    }
}

// Active communities (super-degree > 0), in id order.
__global__ void k_active_flags(const int32_t* __restrict__ sdeg, int64_t C, int32_t* __restrict__ flag) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C; c += (int64_t)gridDim.x * blockDim.x)
        flag[c] = sdeg[c] > 0 ? 1 : 0;
}

__global__ void k_active_emit(const int32_t* __restrict__ flag, const int64_t* __restrict__ pos, int64_t C,
                              uint32_t* __restrict__ active) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C; c += (int64_t)gridDim.x * blockDim.x)
        if (flag[c]) active[pos[c]] = (uint32_t)c;
}

// Start index in `active` of every batch of `batch` communities.
__global__ void k_batch_starts(const uint32_t* __restrict__ active, int64_t na, int64_t nbatch, int64_t batch,
                               int64_t* __restrict__ bstart) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b <= nbatch; b += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t lo_c = (uint64_t)(b * batch);
        int64_t lo = 0, hi = na;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if ((uint64_t)active[mid] < lo_c) lo = mid + 1; else hi = mid;
        }
        bstart[b] = lo;
    }
}

__global__ void k_big_super_flags(const uint32_t* __restrict__ active, int64_t na, const int64_t* __restrict__ soff,
                                  int64_t limit, int32_t* __restrict__ flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < na; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t c = active[i];
        flag[i] = soff[c + 1] - soff[c] > limit;
    }
}

__global__ void k_big_super_emit(const uint32_t* __restrict__ active, int64_t na, const int32_t* __restrict__ flag,
                                 const int64_t* __restrict__ pos, uint32_t* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < na; i += (int64_t)gridDim.x * blockDim.x)
        if (flag[i]) out[pos[i]] = active[i];
}

// light[b] = 1 when batch b has at most kLightNodes super-nodes, each of
// degree <= kLightDeg (constants defined with the cluster kernel).
__global__ void k_batch_light(const uint32_t* __restrict__ active, const int64_t* __restrict__ bstart,
                              const int64_t* __restrict__ soff, int64_t nbatch, int max_nodes, int max_deg,
                              uint8_t* __restrict__ light) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nbatch; b += (int64_t)gridDim.x * blockDim.x) {
        const int64_t lo = bstart[b], hi = bstart[b + 1];
        bool ok = hi - lo <= max_nodes;
        for (int64_t i = lo; ok && i < hi; ++i) {
            const uint32_t c = active[i];
            ok = soff[c + 1] - soff[c] <= max_deg;
        }
        light[b] = ok ? 1 : 0;
    }
}

struct SmArgs {
    const int64_t* soff;
    const uint32_t* snbr;
    const uint32_t* sw;
    const long long* sweight;     // kc per community
    uint32_t* scomm;
    unsigned long long* sctot;    // int64 totals
    const uint32_t* active;
    const int64_t* bstart;
    int64_t nbatch;
    uint32_t* proposed;
    double* pdelta;
    double M, R;
    uint32_t* gkeys;              // per-warp global tables for big super-nodes
    uint32_t* gvals;
    int64_t gcap;
    // Super-nodes above kBigSuper (cluster kernel) or kBigSuperBatched
    // (batched launches) neighbours: one CTA each.
    const uint32_t* big_active;   // ascending
    const int64_t* bigstart;      // per batch
    uint32_t* bkeys;              // per-CTA global tables
    uint32_t* bvals;
    int64_t bcap;
    // Batches of at most kLightNodes super-nodes of degree <= kLightDeg: one
    // thread per super-node on the cluster's first CTA.
    const uint8_t* light;
    int64_t warp_max;             // batched launches: warps take super-nodes up to this degree
    // Batched launches: super-nodes above huge_min neighbours are split over
    // several CTAs (edge segments accumulate into one table per node, table
    // segments select, the last CTA of a node reduces).  huge_min 0: none.
    int64_t huge_min;
    const uint32_t* huge_c;       // huge super-nodes, id order
    const int64_t* huge_toff;     // table offset in the pool
    const uint32_t* huge_tcap;    // table capacity (pow2 >= 2 x degree)
    const int32_t* huge_tfirst;   // first table segment of each node
    const int32_t* huge_tcount;   // table segments of each node
    int32_t* huge_done;           // table segments finished, per node
    const int2* huge_eseg;        // (node, part) of every edge segment
    const int2* huge_tseg;        // (node, part) of every table segment
    uint32_t* hkeys;              // table pool
    uint32_t* hvals;
    double* part_d;               // best of each table segment
    uint32_t* part_c;
    // 1/M as a double-double (make_dq): quotients by M are formed by
    // div_rn_by, bit-identical to full divisions at a fraction of the FP64 work.
    double yMh = 0.0, yMl = 0.0;
};

constexpr int kSmSmall = 256;     // per-warp shared table slots

__device__ __forceinline__ void super_commit(const SmArgs& a, uint32_t c, int* moves) {
    const uint32_t d = a.scomm[c];
    const uint32_t best = a.proposed[c];
    if (best == d || !(a.pdelta[c] > 0.0)) return;
    const long long kc = a.sweight[c];
    atomicAdd(&a.sctot[d], (unsigned long long)(-kc));
    atomicAdd(&a.sctot[best], (unsigned long long)kc);
    a.scomm[c] = best;
    atomicAdd(moves, 1);
}

// Whole super-move in one thread-block cluster: batches in order, propose /
// cluster barrier / commit / cluster barrier; iterations stop early when a
// full iteration moves nothing.  The cluster barrier is the hardware
// barrier.cluster (release / acquire), so the CTAs' global writes of one
// phase are visible to the next.  A warp keeps its proposals in shared
// memory and its lanes commit them after the barrier; small super-nodes use
// a shared table that also caches each candidate's total at insertion.
constexpr int kSmCluster = 8;     // portable cluster size
constexpr int kSmClusterMax = 16; // non-portable size, used where the GPU can place it
constexpr int kSmPerWarp = 16;    // proposals a warp keeps per batch (4096 / (8 x 32))
constexpr int kBigSuper = 1024;   // super-nodes with more neighbours: one CTA each
constexpr int kBigSuperBatched = kSmSmall / 2;   // batched launches: warps only with shared tables

__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

struct SmProposal {
    uint32_t c, d, best, pad;
    long long kc;
    double delta;
};

// Candidate (dl, ek) into a running best that starts at (+0.0, own
// community): a proposal commits only when its delta is > 0, so candidates at
// or below +0.0 change no outcome and are skipped; among the others the order
// is better()'s, compared on the integer pipe.
__device__ __forceinline__ void take_pos(double dl, uint32_t ek, double& best_d, uint32_t& best_c) {
    if (dpos(dl) && better_pos(dl, ek, best_d, best_c)) {
        best_d = dl;
        best_c = ek;
    }
}

// Proposal for super-node c by one warp (the GVE super-move proposals of
// RG:2264-2302): neighbour communities into a shared table (a per-warp
// global one above kSmSmall / 2 neighbours) whose third array caches each
// candidate's total, loaded by the inserting lane; best Delta-modularity,
// ties to the smaller community.
__device__ void super_propose_cached(const SmArgs& a, uint32_t c, uint32_t* tk, uint32_t* tv,
                                     unsigned long long* tt, uint32_t* gk, uint32_t* gv, SmProposal& out) {
    const int lane = threadIdx.x & 31;
    const int64_t b = a.soff[c], e = a.soff[c + 1];
    const int64_t deg = e - b;
    uint32_t H = 64;
    while ((int64_t)H < 2 * deg) H <<= 1;
    const bool shared = H <= (uint32_t)kSmSmall;
    uint32_t *k = shared ? tk : gk, *v = shared ? tv : gv;
    const uint32_t mask = H - 1;
    for (uint32_t i = lane; i < H; i += 32) { k[i] = kNone; v[i] = 0; }
    __syncwarp();
    const uint32_t d = a.scomm[c];
    const long long kcl = a.sweight[c];
    const unsigned long long sd_raw = a.sctot[d];
    for (int64_t i0 = b; i0 < e; i0 += 32) {
        uint32_t key = kNone, wgt = 0;
        if (i0 + lane < e) {
            key = a.scomm[a.snbr[i0 + lane]];
            wgt = a.sw[i0 + lane];
        }
        if (key != kNone) {
            uint32_t h = hash_u32(key) & mask;
            while (true) {
                const uint32_t prev = atomicCAS(&k[h], kNone, key);
                if (prev == kNone && shared) tt[h] = a.sctot[key];
                if (prev == kNone || prev == key) {
                    atomicAdd(&v[h], wgt);
                    break;
                }
                h = (h + 1) & mask;
            }
        }
    }
    __syncwarp();
    const double kc_to_d = (double)table_get(k, v, mask, d);
    // Occupied slots to the front, in slot order: the scoring loop then takes
    // ceil(occupied / 32) full-warp steps instead of H / 32 mostly idle ones
    // (an FP64 instruction costs the same with one lane active or 32).
    uint32_t occ = 0;
    for (uint32_t i0 = 0; i0 < H; i0 += 32) {
        const uint32_t i = i0 + lane;
        const uint32_t ek = k[i], ev = v[i];
        const unsigned long long et = shared ? tt[i] : 0ull;
        const unsigned m = __ballot_sync(0xFFFFFFFFu, ek != kNone);
        __syncwarp();
        if (ek != kNone) {
            const uint32_t j = occ + (uint32_t)__popc(m & ((1u << lane) - 1u));
            k[j] = ek;
            v[j] = ev;
            if (shared) tt[j] = et;
        }
        __syncwarp();
        occ += (uint32_t)__popc(m);
    }
    const double kc = (double)kcl;
    const double sigma_d = (double)(long long)sd_raw;
    const double removal = div_rn_by(__dmul_rn(__dmul_rn(a.R, kc), __dsub_rn(sigma_d, kc)), a.M, a.yMh, a.yMl);
    double best_d = 0.0;
    uint32_t best_c = d;
    for (uint32_t i = lane; i < occ; i += 32) {
        const uint32_t ek = k[i];
        const double kce = (double)v[i];
        double add;
        if (ek == d) {
            add = __dsub_rn(kc_to_d, removal);
        } else {
            const double se = (double)(long long)(shared ? tt[i] : a.sctot[ek]);
            add = __dsub_rn(kce, div_rn_by(__dmul_rn(__dmul_rn(a.R, kc), se), a.M, a.yMh, a.yMl));
        }
        const double dl = __dadd_rn(__dsub_rn(add, removal), kc_to_d);
        take_pos(dl, ek, best_d, best_c);
    }
    warp_argmax_pos(best_d, best_c);
    out.c = c;
    out.d = d;
    out.best = best_c;
    out.kc = kcl;
    out.delta = best_d;
    __syncwarp();
}

// Proposal for a big super-node by the whole CTA (global table of the CTA).
__device__ void super_propose_block(const SmArgs& a, uint32_t c, SmProposal* out, double* red_d, uint32_t* red_c) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int64_t b = a.soff[c], e = a.soff[c + 1];
    const int64_t deg = e - b;
    uint32_t H = 64;
    while ((int64_t)H < 2 * deg) H <<= 1;
    uint32_t* k = a.bkeys + (int64_t)blockIdx.x * a.bcap;
    uint32_t* v = a.bvals + (int64_t)blockIdx.x * a.bcap;
    const uint32_t mask = H - 1;
    for (uint32_t i = tid; i < H; i += blockDim.x) { k[i] = kNone; v[i] = 0; }
    const uint32_t d = a.scomm[c];
    const long long kcl = a.sweight[c];
    const double kc = (double)kcl;
    const double sigma_d = (double)(long long)a.sctot[d];
    __syncthreads();
#pragma unroll 4
    for (int64_t idx = b + tid; idx < e; idx += blockDim.x) table_add(k, v, mask, a.scomm[a.snbr[idx]], a.sw[idx]);
    __syncthreads();
    const double removal = div_rn_by(__dmul_rn(__dmul_rn(a.R, kc), __dsub_rn(sigma_d, kc)), a.M, a.yMh, a.yMl);
    const double kc_to_d = (double)table_get(k, v, mask, d);
    double best_d = 0.0;
    uint32_t best_c = d;
#pragma unroll 8
    for (uint32_t i = tid; i < H; i += blockDim.x) {
        const uint32_t ek = k[i];
        if (ek == kNone) continue;
        const double kce = (double)v[i];
        double add;
        if (ek == d) {
            add = __dsub_rn(kc_to_d, removal);
        } else {
            const double se = (double)(long long)a.sctot[ek];
            add = __dsub_rn(kce, div_rn_by(__dmul_rn(__dmul_rn(a.R, kc), se), a.M, a.yMh, a.yMl));
        }
        const double dl = __dadd_rn(__dsub_rn(add, removal), kc_to_d);
        take_pos(dl, ek, best_d, best_c);
    }
    warp_argmax_pos(best_d, best_c);
    if (lane == 0) { red_d[w] = best_d; red_c[w] = best_c; }
    __syncthreads();
    if (tid == 0) {
        double bd = red_d[0];
        uint32_t bc = red_c[0];
        for (int q = 1; q < (int)(blockDim.x >> 5); ++q)
            if (better_pos(red_d[q], red_c[q], bd, bc)) { bd = red_d[q]; bc = red_c[q]; }
        out->c = c;
        out->d = d;
        out->best = bc;
        out->kc = kcl;
        out->delta = bd;
    }
    __syncthreads();
}

constexpr int kLightDeg = 8;
constexpr int kLightNodes = 1024;

// Proposal for a super-node of degree <= kLightDeg by one thread: the same
// candidates, weights, totals and arithmetic as super_propose_cached, with
// the table replaced by a first-occurrence merge in registers.  scomm and
// sctot are read through L2 (they change between batches of one CTA).
__device__ void super_propose_light(const SmArgs& a, uint32_t c, SmProposal& out) {
    const int64_t b = a.soff[c];
    const int deg = (int)(a.soff[c + 1] - b);
    const uint32_t d = __ldcg(&a.scomm[c]);
    const long long kcl = a.sweight[c];
    const unsigned long long sd_raw = __ldcg(&a.sctot[d]);
    uint32_t key[kLightDeg], wsum[kLightDeg];
#pragma unroll
    for (int k = 0; k < kLightDeg; ++k) {
        key[k] = kNone;
        wsum[k] = 0;
        if (k < deg) {
            key[k] = __ldcg(&a.scomm[a.snbr[b + k]]);
            wsum[k] = a.sw[b + k];
        }
    }
    // Weights onto first occurrences; later duplicates become empty.
#pragma unroll
    for (int k = 1; k < kLightDeg; ++k) {
#pragma unroll
        for (int j = 0; j < k; ++j) {
            if (key[k] != kNone && key[j] == key[k]) {
                wsum[j] += wsum[k];
                key[k] = kNone;
            }
        }
    }
    unsigned long long se_raw[kLightDeg];
#pragma unroll
    for (int k = 0; k < kLightDeg; ++k) se_raw[k] = key[k] != kNone && key[k] != d ? __ldcg(&a.sctot[key[k]]) : 0ull;
    uint32_t kc_to_d_w = 0;
#pragma unroll
    for (int k = 0; k < kLightDeg; ++k)
        if (key[k] == d) kc_to_d_w = wsum[k];
    const double kc = (double)kcl;
    const double sigma_d = (double)(long long)sd_raw;
    const double removal = div_rn_by(__dmul_rn(__dmul_rn(a.R, kc), __dsub_rn(sigma_d, kc)), a.M, a.yMh, a.yMl);
    const double kc_to_d = (double)kc_to_d_w;
    double best_d = 0.0;
    uint32_t best_c = d;
#pragma unroll
    for (int k = 0; k < kLightDeg; ++k) {
        const uint32_t ek = key[k];
        if (ek == kNone) continue;
        double add;
        if (ek == d) {
            add = __dsub_rn(kc_to_d, removal);
        } else {
            const double se = (double)(long long)se_raw[k];
            add = __dsub_rn((double)wsum[k], div_rn_by(__dmul_rn(__dmul_rn(a.R, kc), se), a.M, a.yMh, a.yMl));
        }
        const double dl = __dadd_rn(__dsub_rn(add, removal), kc_to_d);
        take_pos(dl, ek, best_d, best_c);
    }
    out.c = c;
    out.d = d;
    out.best = best_c;
    out.kc = kcl;
    out.delta = best_d;
}

__global__ void __launch_bounds__(1024)
k_super_move_cluster(SmArgs a, int max_iter, int* iters_out, long long* moves_out, int* gmoves) {
    extern __shared__ uint32_t sm_smem[];   // 32 warps x (keys, vals, totals) x kSmSmall
    __shared__ SmProposal props[32][kSmPerWarp];
    __shared__ SmProposal bprop;
    __shared__ double red_d[32];
    __shared__ uint32_t red_c[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int64_t gw = (int64_t)blockIdx.x * nw + w, gnw = (int64_t)gridDim.x * nw;
    uint32_t* tk = sm_smem + (size_t)w * 4 * kSmSmall;
    uint32_t* tv = tk + kSmSmall;
    unsigned long long* tt = reinterpret_cast<unsigned long long*>(tv + kSmSmall);
    long long total_moves = 0;
    int it = 0;
    for (; it < max_iter; ++it) {
        // Runs of light batches are done by CTA 0 alone, CTA barriers between
        // propose and commit; the cluster barrier before the next heavy batch
        // (or the iteration's move count) publishes them to the other CTAs.
        bool light_pending = false;
        for (int64_t bt = 0; bt < a.nbatch; ++bt) {
            const int64_t lo = a.bstart[bt], hi = a.bstart[bt + 1];
            if (lo == hi) continue;
            if (a.light[bt]) {
                light_pending = true;
                if (blockIdx.x != 0) continue;
                SmProposal pr;
                const int64_t i = lo + threadIdx.x;
                if (i < hi) super_propose_light(a, a.active[i], pr);
                __syncthreads();
                if (i < hi && pr.best != pr.d && pr.delta > 0.0) {
                    atomicAdd(&a.sctot[pr.d], (unsigned long long)(-pr.kc));
                    atomicAdd(&a.sctot[pr.best], (unsigned long long)pr.kc);
                    a.scomm[pr.c] = pr.best;
                    atomicAdd(&gmoves[it], 1);
                }
                __syncthreads();
                continue;
            }
            if (light_pending) {
                cluster_sync_all();
                light_pending = false;
            }
            // Warps: super-nodes up to kBigSuper neighbours.
            int kept = 0;
            for (int64_t i = lo + gw; i < hi; i += gnw) {
                const uint32_t c = a.active[i];
                if (a.soff[c + 1] - a.soff[c] > kBigSuper) continue;
                SmProposal pr;
                super_propose_cached(a, c, tk, tv, tt, a.gkeys + gw * a.gcap, a.gvals + gw * a.gcap, pr);
                if (kept < kSmPerWarp) {
                    if (lane == 0) props[w][kept] = pr;
                } else if (lane == 0) {   // more than the warp keeps: through global memory
                    a.proposed[pr.c] = pr.best;
                    a.pdelta[pr.c] = pr.delta;
                }
                ++kept;
            }
            __syncwarp();
            // CTAs: the batch's big super-nodes (proposals through global memory).
            const int64_t blo = a.bigstart[bt], bhi = a.bigstart[bt + 1];
            __syncthreads();
            for (int64_t j = blo + blockIdx.x; j < bhi; j += gridDim.x) {
                super_propose_block(a, a.big_active[j], &bprop, red_d, red_c);
                if (threadIdx.x == 0) {
                    a.proposed[bprop.c] = bprop.best;
                    a.pdelta[bprop.c] = bprop.delta;
                }
            }
            cluster_sync_all();
            if (lane < min(kept, kSmPerWarp)) {
                const SmProposal pr = props[w][lane];
                if (pr.best != pr.d && pr.delta > 0.0) {
                    atomicAdd(&a.sctot[pr.d], (unsigned long long)(-pr.kc));
                    atomicAdd(&a.sctot[pr.best], (unsigned long long)pr.kc);
                    a.scomm[pr.c] = pr.best;
                    atomicAdd(&gmoves[it], 1);
                }
            }
            if (kept > kSmPerWarp) {
                // The warp's nodes past kSmPerWarp, in the same order as proposed.
                int seen = 0;
                for (int64_t i = lo + gw; i < hi; i += gnw) {
                    const uint32_t c = a.active[i];
                    if (a.soff[c + 1] - a.soff[c] > kBigSuper) continue;
                    if (seen++ < kSmPerWarp) continue;
                    if (lane == 0) super_commit(a, c, &gmoves[it]);
                }
            }
            if (threadIdx.x == 0)
                for (int64_t j = blo + blockIdx.x; j < bhi; j += gridDim.x) super_commit(a, a.big_active[j], &gmoves[it]);
            cluster_sync_all();
        }
        if (light_pending) cluster_sync_all();
        const int m = atomicAdd(&gmoves[it], 0);
        total_moves += m;
        if (m == 0) { ++it; break; }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *iters_out = it;
        *moves_out = total_moves;
    }
}

// Batched launches for super-graphs above one cluster's size: per batch,
// lanes propose the super-nodes up to kLightDeg neighbours, warps those up to
// kBigSuperBatched (shared tables), CTAs the bigger ones, then the commit.
__global__ void __launch_bounds__(256, 4) k_super_propose_batch(SmArgs a, int64_t bt) {
    __shared__ uint32_t tk[8][kSmSmall];
    __shared__ uint32_t tv[8][kSmSmall];
    __shared__ unsigned long long tt[8][kSmSmall];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t lo = a.bstart[bt], hi = a.bstart[bt + 1];
    const int64_t gw = (int64_t)blockIdx.x * 8 + w;
    const int64_t nwt = (int64_t)gridDim.x * 8;
    // Light super-nodes, a lane each: warp w of every CTA takes 32 of them
    // before warp w + 1 of any, so a batch's FP64 work spreads over the SMs.
    const int64_t lw = (int64_t)w * gridDim.x + blockIdx.x;
    for (int64_t i = lo + lw * 32 + lane; i < hi; i += nwt * 32) {
        const uint32_t c = a.active[i];
        if (a.soff[c + 1] - a.soff[c] > kLightDeg) continue;
        SmProposal pr;
        super_propose_light(a, c, pr);
        a.proposed[c] = pr.best;
        a.pdelta[c] = pr.delta;
    }
    for (int64_t i = lo + gw; i < hi; i += nwt) {
        const uint32_t c = a.active[i];
        const int64_t deg = a.soff[c + 1] - a.soff[c];
        if (deg <= kLightDeg || deg > a.warp_max) continue;
        SmProposal pr;
        super_propose_cached(a, c, tk[w], tv[w], tt[w], a.gkeys + gw * a.gcap, a.gvals + gw * a.gcap, pr);
        if (lane == 0) {
            a.proposed[pr.c] = pr.best;
            a.pdelta[pr.c] = pr.delta;
        }
    }
}

// CTA per super-node of the batch's big list (a quarter of an SM each, so
// four run per SM); the table is the CTA's global slice.
constexpr int kBigBatchThreads = 256;

__global__ void __launch_bounds__(kBigBatchThreads) k_super_propose_big_batch(SmArgs a, int64_t bt) {
    __shared__ SmProposal bprop;
    __shared__ double red_d[32];
    __shared__ uint32_t red_c[32];
    for (int64_t j = a.bigstart[bt] + blockIdx.x; j < a.bigstart[bt + 1]; j += gridDim.x) {
        const uint32_t c = a.big_active[j];
        if (a.huge_min > 0 && a.soff[c + 1] - a.soff[c] > a.huge_min) continue;   // split over CTAs
        super_propose_block(a, c, &bprop, red_d, red_c);
        if (threadIdx.x == 0) {
            a.proposed[bprop.c] = bprop.best;
            a.pdelta[bprop.c] = bprop.delta;
        }
    }
}

// Huge super-nodes, first half: each CTA inserts one segment of kHugeSeg
// neighbour entries into the node's table (the pool is cleared before every
// iteration of the super-move).
constexpr int kHugeSeg = 4096;    // entries (edges or table slots) per CTA: 4 per thread

__global__ void __launch_bounds__(1024) k_super_huge_accum(SmArgs a, int64_t seg0) {
    const int2 sg = a.huge_eseg[seg0 + blockIdx.x];
    const uint32_t c = a.huge_c[sg.x];
    const int64_t e = a.soff[c + 1];
    const int64_t e0 = a.soff[c] + (int64_t)sg.y * kHugeSeg, e1 = min(e, e0 + kHugeSeg);
    uint32_t* k = a.hkeys + a.huge_toff[sg.x];
    uint32_t* v = a.hvals + a.huge_toff[sg.x];
    const uint32_t mask = a.huge_tcap[sg.x] - 1;
    uint32_t key[4], w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int64_t i = e0 + q * (int64_t)blockDim.x + threadIdx.x;
        key[q] = i < e1 ? a.scomm[a.snbr[i]] : kNone;
        w[q] = i < e1 ? a.sw[i] : 0u;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
        if (key[q] != kNone) table_add(k, v, mask, key[q], w[q]);
}

// Second half: each CTA scores one segment of the node's table slots with
// super_propose_block's arithmetic; the last CTA of the node takes the best
// of the segments' bests (the selection is a total order, so the split does
// not change it) and records the proposal.
__global__ void __launch_bounds__(1024) k_super_huge_select(SmArgs a, int64_t seg0) {
    __shared__ double red_d[32];
    __shared__ uint32_t red_c[32];
    __shared__ int s_last;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int64_t q = seg0 + blockIdx.x;
    const int2 sg = a.huge_tseg[q];
    const int j = sg.x;
    const uint32_t c = a.huge_c[j];
    const uint32_t* k = a.hkeys + a.huge_toff[j];
    const uint32_t* v = a.hvals + a.huge_toff[j];
    const uint32_t H = a.huge_tcap[j], mask = H - 1;
    const uint32_t d = a.scomm[c];
    const long long kcl = a.sweight[c];
    const double kc = (double)kcl;
    const double sigma_d = (double)(long long)a.sctot[d];
    const double removal = div_rn_by(__dmul_rn(__dmul_rn(a.R, kc), __dsub_rn(sigma_d, kc)), a.M, a.yMh, a.yMl);
    const double kc_to_d = (double)table_get(k, v, mask, d);
    double best_d = 0.0;
    uint32_t best_c = d;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const uint32_t i = (uint32_t)sg.y * kHugeSeg + r * blockDim.x + tid;
        if (i >= H) continue;
        const uint32_t ek = k[i];
        if (ek == kNone) continue;
        const double kce = (double)v[i];
        double add;
        if (ek == d) {
            add = __dsub_rn(kc_to_d, removal);
        } else {
            const double se = (double)(long long)a.sctot[ek];
            add = __dsub_rn(kce, div_rn_by(__dmul_rn(__dmul_rn(a.R, kc), se), a.M, a.yMh, a.yMl));
        }
        const double dl = __dadd_rn(__dsub_rn(add, removal), kc_to_d);
        take_pos(dl, ek, best_d, best_c);
    }
    warp_argmax_pos(best_d, best_c);
    if (lane == 0) { red_d[w] = best_d; red_c[w] = best_c; }
    __syncthreads();
    if (tid == 0) {
        double bd = red_d[0];
        uint32_t bc = red_c[0];
        for (int r = 1; r < (int)(blockDim.x >> 5); ++r)
            if (better_pos(red_d[r], red_c[r], bd, bc)) { bd = red_d[r]; bc = red_c[r]; }
        a.part_d[q] = bd;
        a.part_c[q] = bc;
        __threadfence();
        s_last = atomicAdd(&a.huge_done[j], 1) == a.huge_tcount[j] - 1;
        if (s_last) {
            __threadfence();
            const int f = a.huge_tfirst[j], nt = a.huge_tcount[j];
            bd = ((volatile double*)a.part_d)[f];
            bc = ((volatile uint32_t*)a.part_c)[f];
            for (int r = 1; r < nt; ++r) {
                const double pd = ((volatile double*)a.part_d)[f + r];
                const uint32_t pc = ((volatile uint32_t*)a.part_c)[f + r];
                if (better_pos(pd, pc, bd, bc)) { bd = pd; bc = pc; }
            }
            a.proposed[c] = bc;
            a.pdelta[c] = bd;
            a.huge_done[j] = 0;
        }
    }
}

__global__ void k_super_commit_batch(SmArgs a, int64_t bt, int* moves) {
    const int64_t lo = a.bstart[bt], hi = a.bstart[bt + 1];
    for (int64_t i = lo + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < hi; i += (int64_t)gridDim.x * blockDim.x)
        super_commit(a, a.active[i], moves);
}

// Map back and first-occurrence renumber (:2389-2419).
__global__ void k_remap(uint32_t* __restrict__ vcom, int64_t n, const uint32_t* __restrict__ scomm,
                        int32_t* __restrict__ firstpos) {
    const int lane = threadIdx.x & 31;
    for (int64_t v0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane; v0 < n;
         v0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = v0 + lane;
        uint32_t c = 0;
        if (v < n) {
            c = scomm[vcom[v]];
            vcom[v] = c;
        }
        warp_min_ordered_i32(firstpos, c, (int32_t)v, v < n);
    }
}

__global__ void k_first_flags(const uint32_t* __restrict__ vcom, int64_t n, const int32_t* __restrict__ firstpos,
                              int32_t* __restrict__ flag) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        flag[v] = firstpos[vcom[v]] == (int32_t)v ? 1 : 0;
}

__global__ void k_first_apply(uint32_t* __restrict__ vcom, int64_t n, const int32_t* __restrict__ firstpos,
                              const int64_t* __restrict__ rk) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        vcom[v] = (uint32_t)rk[firstpos[vcom[v]]];
}

__global__ void k_ctot_from_members(const int64_t* __restrict__ rp, const uint32_t* __restrict__ vcom, int64_t n,
                                    unsigned long long* __restrict__ ctot) {
    const int lane = threadIdx.x & 31;
    for (int64_t v0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane; v0 < n;
         v0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = v0 + lane;
        const int64_t d = v < n ? rp[v + 1] - rp[v] : 0;
        warp_add_u64(ctot, d ? vcom[v] : 0u, (unsigned long long)d, d != 0);
    }
}

__global__ void k_init_state(const int64_t* __restrict__ rp, int64_t n, uint32_t* __restrict__ vcom,
                             unsigned long long* __restrict__ ctot, uint8_t* __restrict__ vaff) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        vcom[v] = (uint32_t)v;
        ctot[v] = (unsigned long long)(rp[v + 1] - rp[v]);
        vaff[v] = 1;
    }
}

__global__ void k_max_degree(const int64_t* __restrict__ rp, int64_t n, unsigned long long* __restrict__ out) {
    unsigned long long m = 0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long d = (unsigned long long)(rp[v + 1] - rp[v]);
        m = d > m ? d : m;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xFFFFFFFFu, m, o);
        m = t > m ? t : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void k_hub_flags(const int64_t* __restrict__ rp, int64_t n, int32_t* __restrict__ flag) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        flag[v] = (rp[v + 1] - rp[v]) > kWarpMaxDeg ? 1 : 0;
}

__global__ void k_hub_emit(const int32_t* __restrict__ flag, const int64_t* __restrict__ pos, int64_t n,
                           uint32_t* __restrict__ hubs) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        if (flag[v]) hubs[pos[v]] = (uint32_t)v;
}

// ---- Local moving over the vertices that have neighbours ----
// A vertex without neighbours never moves and is never a candidate, so its
// community is a singleton that no other vertex can reach.  Local moving
// runs on the graph without those vertices, renumbered in id order (the
// rows keep their offsets: removed rows are empty), and on the communities
// of the remaining vertices renumbered in id order: both maps are monotone,
// so the serial order and every id tie-break are the same.
__global__ void k_nonisolated_flags(const int64_t* __restrict__ rp, int64_t n, int32_t* __restrict__ flag) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        flag[v] = rp[v + 1] > rp[v] ? 1 : 0;
}

__global__ void k_compact_rows(const int64_t* __restrict__ rp, const int32_t* __restrict__ flag,
                               const int64_t* __restrict__ pos, int64_t n, int64_t* __restrict__ rp_c,
                               uint32_t* __restrict__ orig) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        if (flag[v]) {
            rp_c[pos[v]] = rp[v];
            orig[pos[v]] = (uint32_t)v;
        }
}

__global__ void k_compact_cols(const int32_t* __restrict__ col, int64_t nnz, const int64_t* __restrict__ pos,
                               int32_t* __restrict__ col_c) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x)
        col_c[e] = (int32_t)pos[col[e]];
}

__global__ void k_map_u32(const uint32_t* __restrict__ in, int64_t m, const int64_t* __restrict__ pos,
                          uint32_t* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (uint32_t)pos[in[i]];
}

// cflag[c] = 1 for every community of a kept vertex.
__global__ void k_comm_flags(const uint32_t* __restrict__ vcom, const uint32_t* __restrict__ orig, int64_t nc,
                             int32_t* __restrict__ cflag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nc; i += (int64_t)gridDim.x * blockDim.x)
        cflag[vcom[orig[i]]] = 1;
}

__global__ void k_comm_inverse(const int32_t* __restrict__ cflag, const int64_t* __restrict__ cpos, int64_t n,
                               uint32_t* __restrict__ cinv) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
        if (cflag[c]) cinv[cpos[c]] = (uint32_t)c;
}

__global__ void k_gather_state(const uint32_t* __restrict__ orig, int64_t nc, const uint32_t* __restrict__ vcom,
                               const uint8_t* __restrict__ vaff, const uint32_t* __restrict__ vcob,
                               const int64_t* __restrict__ cpos, uint32_t* __restrict__ vcom_c,
                               uint8_t* __restrict__ vaff_c, uint32_t* __restrict__ vcob_c) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nc; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t v = orig[i];
        vcom_c[i] = (uint32_t)cpos[vcom[v]];
        vaff_c[i] = vaff[v];
        if (vcob) vcob_c[i] = vcob[v];
    }
}

__global__ void k_gather_totals(const uint32_t* __restrict__ cinv, int64_t cc, const unsigned long long* __restrict__ ctot,
                                unsigned long long* __restrict__ ctot_c) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < cc; i += (int64_t)gridDim.x * blockDim.x)
        ctot_c[i] = ctot[cinv[i]];
}

__global__ void k_scatter_state(const uint32_t* __restrict__ orig, int64_t nc, const uint32_t* __restrict__ vcom_c,
                                const uint32_t* __restrict__ cinv, uint32_t* __restrict__ vcom) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nc; i += (int64_t)gridDim.x * blockDim.x)
        vcom[orig[i]] = cinv[vcom_c[i]];
}

__global__ void k_scatter_totals(const uint32_t* __restrict__ cinv, int64_t cc,
                                 const unsigned long long* __restrict__ ctot_c, unsigned long long* __restrict__ ctot) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < cc; i += (int64_t)gridDim.x * blockDim.x)
        ctot[cinv[i]] = ctot_c[i];
}

template <typename T>
T read_dev(const T* p, cudaStream_t s) {
    T h;
    GB_CUDA(cudaMemcpyAsync(&h, p, sizeof(T), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    return h;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

}  // namespace

double auto_resolution_device(const int64_t* row_ptr, int64_t n, int64_t nnz, cudaStream_t s);

// Cluster size of the super-move: 16 CTAs where the GPU can place such a
// cluster of 1,024-thread CTAs with this much shared memory, else 8.
// The result does not depend on it (proposals read the batch's frozen state;
// commits are integer atomics on distinct super-nodes).
int probe_super_cluster_size(int smem) {
    int size = kSmCluster;
    if (cudaFuncSetAttribute(k_super_move_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
        cudaSuccess) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(kSmClusterMax);
        cfg.blockDim = dim3(1024);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = kSmClusterMax;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int clusters = 0;
        if (cudaOccupancyMaxActiveClusters(&clusters, k_super_move_cluster, &cfg) == cudaSuccess && clusters > 0)
            size = kSmClusterMax;
    }
    cudaGetLastError();
    return size;
}

int super_cluster_size(int smem) {
    static const int size = probe_super_cluster_size(smem);   // smem is the same constant on every call
    return size;
}

void leiden_device(const DeviceCSR& g, const LeidenParams& p, uint32_t* vcom, gbgpu_stats* st, cudaStream_t s) {
    const int64_t n = g.n;
    if (n == 0) return;
    GB_REQUIRE(n < (int64_t)0x7FFFFFFF, GBGPU_E_OVERFLOW, "graph has more vertices than int32 ids can name");
    int64_t launches = 0;
    const int64_t m = g.nnz / 2;
    const double M = p.total_edges_m ? std::max(1.0, (double)m) : (double)m / 2.0;
    const double R = p.resolution;

    cudaEvent_t e0, e1, ea, eb;
    GB_CUDA(cudaEventCreate(&e0));
    GB_CUDA(cudaEventCreate(&e1));
    GB_CUDA(cudaEventCreate(&ea));
    GB_CUDA(cudaEventCreate(&eb));
    GB_CUDA(cudaEventRecord(e0, s));
    double lm_ms = 0.0, agg_ms = 0.0;

    DevBuf<unsigned long long> ctot(n, s);
    DevBuf<uint8_t> vaff(n, s);
    DevBuf<double> dacc(1, s);
    DevBuf<unsigned long long> macc(1, s);
    k_init_state<<<grid_for(n, kT), kT, 0, s>>>(g.row_ptr, n, vcom, ctot, vaff);
    GB_LAUNCH_CHECK();
    ++launches;

    // Hub list (degree > kWarpMaxDeg), id order; host copy for chunk ranges.
    std::vector<uint32_t> hubs_h;
    DevBuf<uint32_t> hubs;
    int64_t max_hub_deg = 0;
    {
        DevBuf<int32_t> flag(n, s);
        DevBuf<int64_t> pos(n + 1, s);
        k_hub_flags<<<grid_for(n, kT), kT, 0, s>>>(g.row_ptr, n, flag);
        GB_LAUNCH_CHECK();
        exclusive_scan_i32_to_i64(flag, pos, n, pos.get() + n, s);
        const int64_t nh = read_dev(pos.get() + n, s);
        launches += 4;
        if (nh > 0) {
            hubs.alloc(nh, s);
            k_hub_emit<<<grid_for(n, kT), kT, 0, s>>>(flag, pos, n, hubs);
            GB_LAUNCH_CHECK();
            ++launches;
            hubs_h.resize(nh);
            GB_CUDA(cudaMemcpyAsync(hubs_h.data(), hubs.get(), nh * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
            DevBuf<unsigned long long> md(1, s);
            GB_CUDA(cudaMemsetAsync(md, 0, sizeof(unsigned long long), s));
            k_max_degree<<<grid_for(n, kT), kT, 0, s>>>(g.row_ptr, n, md);
            GB_LAUNCH_CHECK();
            max_hub_deg = (int64_t)read_dev(md.get(), s);
            launches += 1;
        }
    }
    int64_t hub_gcap = 0;
    if (max_hub_deg * 2 > kHubSmemSlots) {
        hub_gcap = 1024;
        while (hub_gcap < 2 * max_hub_deg) hub_gcap <<= 1;
    }
    const int hub_grid = (int)std::min<int64_t>(std::max<int64_t>(1, (int64_t)hubs_h.size()), kNumSMs);
    DevBuf<uint32_t> hub_gk(hub_gcap ? hub_grid * hub_gcap : 0, s), hub_gv(hub_gcap ? hub_grid * hub_gcap : 0, s);
    const int hub_smem = 2 * kHubSmemSlots * (int)sizeof(uint32_t);
    GB_CUDA(cudaFuncSetAttribute(k_local_move_hub, cudaFuncAttributeMaxDynamicSharedMemorySize, hub_smem));
    const int lm_smem = kLmWarpsPerBlock * 2 * kWarpHash * (int)sizeof(uint32_t);
    GB_CUDA(cudaFuncSetAttribute(k_local_move_warp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lm_smem));
    GB_CUDA(cudaFuncSetAttribute(k_local_move_warp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lm_smem));
    const int sm_smem = 32 * 4 * kSmSmall * (int)sizeof(uint32_t);
    GB_CUDA(cudaFuncSetAttribute(k_super_move_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_smem));

    DevBuf<double> atab(kAtabMax + 1, s);
    fill_atab(atab.get(), M, s);
    LmArgs la{g.row_ptr, g.col, vcom, ctot, vaff, M, R, make_dq(M, R), dacc, macc};
    la.dq.atab = atab.get();
    const int64_t chunk = p.chunk_vertices > 0 ? p.chunk_vertices : n;

    // Serial-order engine: cd_serial always; cd_parallel too, except on large
    // graphs whose neighbours sit at nearby ids (meshes, grids, road networks
    // in traversal order): there a decision changes every few thousand
    // vertices, the serial order's rounds commit little, and the stream mode
    // (each warp sweeping its own block in order, as one thread of the
    // reference's parallel mode does) keeps the serial order's modularity at
    // a fraction of its time.
    // 4,864 streams (32 warps on each of the 152 SMs): on a 4096 x 4096 grid
    // this keeps modularity 0.509 (serial order 0.536, the reference's
    // parallel mode ~0.50); 152 streams keep 0.530 at four times the time.
    constexpr int64_t kAutoStreams = 4864;
    bool exact = p.deterministic || n <= p.exact_max_vertices;
    int64_t streams = p.async_streams;
    if (exact && !p.deterministic && p.auto_streams && streams == 0 && n >= p.auto_streams_min_vertices) {
        DevBuf<unsigned long long> nt(2, s);
        GB_CUDA(cudaMemsetAsync(nt, 0, 2 * sizeof(unsigned long long), s));
        k_near_sample<<<kNumSMs * 8, 256, 0, s>>>(g.row_ptr, g.col, n, nt);
        GB_LAUNCH_CHECK();
        ++launches;
        unsigned long long h[2] = {0, 0};
        GB_CUDA(cudaMemcpyAsync(h, nt.get(), sizeof(h), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaStreamSynchronize(s));
        if (h[1] > 0 && 4 * h[0] >= h[1]) {   // a quarter of the sampled entries near
            exact = false;
            streams = kAutoStreams;
        }
    }
    LocalMoveContext lmc;
    lmc.g = g;
    lmc.vcom = vcom;
    lmc.ctot = ctot;
    lmc.vaff = vaff;
    lmc.M = M;
    lmc.R = R;
    lmc.dq = la.dq;
    lmc.hubs_h = hubs_h;
    lmc.hubs = hubs.get();
    lmc.hub_grid = hub_grid;
    lmc.hub_gk = hub_gk.get();
    lmc.hub_gv = hub_gv.get();
    lmc.hub_gcap = hub_gcap;
    int64_t exact_rounds = 0, exact_evals = 0;

    // The serial-order engine runs without the vertices that have no
    // neighbours when they are at least a sixteenth of the graph (RMAT
    // graphs: ~40 %): they would take window slots and rounds while never
    // moving (see k_nonisolated_flags).
    struct Compacted {
        int64_t nc = 0;
        DevBuf<int64_t> pos, rp, cpos;
        DevBuf<int32_t> col, cflag;
        DevBuf<uint32_t> orig, hubs, vcom, vcob, cinv;
        DevBuf<unsigned long long> ctot;
        DevBuf<uint8_t> vaff;
        LocalMoveContext lmc;
    } cp;
    bool compact = false;
    if (exact && n > 0) {
        DevBuf<int32_t> flag(n, s);
        cp.pos.alloc(n + 1, s);
        k_nonisolated_flags<<<grid_for(n, kT), kT, 0, s>>>(g.row_ptr, n, flag);
        GB_LAUNCH_CHECK();
        exclusive_scan_i32_to_i64(flag, cp.pos, n, cp.pos.get() + n, s);
        cp.nc = read_dev(cp.pos.get() + n, s);
        launches += 3;
        if (cp.nc > 0 && (n - cp.nc) * 16 >= n) {
            compact = true;
            const int64_t nc = cp.nc;
            cp.rp.alloc(nc + 1, s);
            cp.orig.alloc(nc, s);
            k_compact_rows<<<grid_for(n, kT), kT, 0, s>>>(g.row_ptr, flag, cp.pos, n, cp.rp, cp.orig);
            GB_LAUNCH_CHECK();
            GB_CUDA(cudaMemcpyAsync(cp.rp.get() + nc, g.row_ptr + n, sizeof(int64_t), cudaMemcpyDeviceToDevice, s));
            cp.col.alloc(g.nnz > 0 ? g.nnz : 1, s);
            if (g.nnz > 0) {
                k_compact_cols<<<grid_for(g.nnz, kT), kT, 0, s>>>(g.col, g.nnz, cp.pos, cp.col);
                GB_LAUNCH_CHECK();
            }
            cp.lmc = lmc;
            cp.lmc.g = DeviceCSR{nc, g.nnz, cp.rp.get(), cp.col.get()};
            if (!hubs_h.empty()) {
                const int64_t nh = (int64_t)hubs_h.size();
                cp.hubs.alloc(nh, s);
                k_map_u32<<<grid_for(nh, kT), kT, 0, s>>>(hubs, nh, cp.pos, cp.hubs);
                GB_LAUNCH_CHECK();
                GB_CUDA(cudaMemcpyAsync(cp.lmc.hubs_h.data(), cp.hubs.get(), nh * sizeof(uint32_t),
                                        cudaMemcpyDeviceToHost, s));
                GB_CUDA(cudaStreamSynchronize(s));
                cp.lmc.hubs = cp.hubs.get();
            }
            cp.vcom.alloc(nc, s);
            cp.vaff.alloc(nc, s);
            cp.ctot.alloc(nc, s);
            cp.cinv.alloc(nc, s);
            cp.cflag.alloc(n, s);
            cp.cpos.alloc(n + 1, s);
            cp.lmc.vcom = cp.vcom.get();
            cp.lmc.vaff = cp.vaff.get();
            cp.lmc.ctot = cp.ctot.get();
            launches += 3 + (hubs_h.empty() ? 0 : 1);
        }
    }
    // One call of the serial-order engine on the current membership (vcob:
    // refinement bounds or null), through the compacted graph when there is one.
    auto run_exact = [&](double tolerance, int max_iterations, const uint32_t* vcob) -> int {
        if (!compact) {
            lmc.vcob = vcob;
            const int it = local_move_exact(lmc, tolerance, max_iterations, p.exact_window, s, &launches,
                                            &exact_rounds, &exact_evals);
            lmc.vcob = nullptr;
            return it;
        }
        const int64_t nc = cp.nc;
        GB_CUDA(cudaMemsetAsync(cp.cflag, 0, n * sizeof(int32_t), s));
        k_comm_flags<<<grid_for(nc, kT), kT, 0, s>>>(vcom, cp.orig, nc, cp.cflag);
        GB_LAUNCH_CHECK();
        exclusive_scan_i32_to_i64(cp.cflag, cp.cpos, n, cp.cpos.get() + n, s);
        const int64_t cc = read_dev(cp.cpos.get() + n, s);
        k_comm_inverse<<<grid_for(n, kT), kT, 0, s>>>(cp.cflag, cp.cpos, n, cp.cinv);
        GB_LAUNCH_CHECK();
        if (vcob && !cp.vcob) cp.vcob.alloc(nc, s);
        k_gather_state<<<grid_for(nc, kT), kT, 0, s>>>(cp.orig, nc, vcom, vaff, vcob, cp.cpos, cp.vcom, cp.vaff,
                                                       vcob ? cp.vcob.get() : nullptr);
        GB_LAUNCH_CHECK();
        GB_CUDA(cudaMemsetAsync(cp.ctot, 0, nc * sizeof(unsigned long long), s));
        k_gather_totals<<<grid_for(cc, kT), kT, 0, s>>>(cp.cinv, cc, ctot, cp.ctot);
        GB_LAUNCH_CHECK();
        cp.lmc.vcob = vcob ? cp.vcob.get() : nullptr;
        const int it = local_move_exact(cp.lmc, tolerance, max_iterations, p.exact_window, s, &launches,
                                        &exact_rounds, &exact_evals);
        cp.lmc.vcob = nullptr;
        k_scatter_state<<<grid_for(nc, kT), kT, 0, s>>>(cp.orig, nc, cp.vcom, cp.cinv, vcom);
        GB_LAUNCH_CHECK();
        k_scatter_totals<<<grid_for(cc, kT), kT, 0, s>>>(cp.cinv, cc, cp.ctot, ctot);
        GB_LAUNCH_CHECK();
        launches += 9;
        return it;
    };

    auto local_move = [&](double tolerance) -> int {
        if (exact) return run_exact(tolerance, p.max_iterations, nullptr);
        int iters = 0;
        for (int it = 0; it < p.max_iterations; ++it) {
            GB_CUDA(cudaMemsetAsync(dacc, 0, sizeof(double), s));
            GB_CUDA(cudaMemsetAsync(macc, 0, sizeof(unsigned long long), s));
            if (streams > 0) {
                // Stream mode: every warp sweeps one contiguous block in order.
                const int64_t warps = std::min<int64_t>(streams, std::max<int64_t>(1, n));
                const int grid = (int)ceil_div(warps, kLmWarpsPerBlock);
                // Warps past the last block (gw >= warps) start at or past n.
                const int64_t len = ceil_div(n, warps);
                k_local_move_warp<true><<<grid, kLmWarpsPerBlock * 32, lm_smem, s>>>(la, 0, n, len);
                GB_LAUNCH_CHECK();
                ++launches;
            } else {
                for (int64_t b = 0; b < n; b += chunk) {
                    const int64_t e = std::min(n, b + chunk);
                    const int64_t warps = e - b;
                    const int grid = (int)std::min<int64_t>(ceil_div(warps, kLmWarpsPerBlock), (int64_t)kNumSMs * 16);
                    k_local_move_warp<false><<<grid, kLmWarpsPerBlock * 32, lm_smem, s>>>(la, b, e, 0);
                    GB_LAUNCH_CHECK();
                    ++launches;
                }
            }
            // Hubs in one launch per iteration, one CTA each: they see the
            // moves of every lower-degree vertex of this iteration.
            if (!hubs_h.empty()) {
                k_local_move_hub<<<hub_grid, kHubThreads, hub_smem, s>>>(la, hubs, 0, (int64_t)hubs_h.size(),
                                                                         hub_gk, hub_gv, hub_gcap);
                GB_LAUNCH_CHECK();
                ++launches;
            }
            ++iters;
            const double total = read_dev(dacc.get(), s);
            if (total <= tolerance) break;
        }
        return iters;
    };

    double tolerance = p.tolerance;
    int64_t prev = n;
    int pass = 0;
    int total_iters = 0;
    int64_t pass0_comms = 0, aggregated = 0, super_moves = 0;
    int super_iters = 0;
    int super_ctas = 0;
    DevBuf<int32_t> exists(n, s);
    DevBuf<int64_t> cmap(n + 1, s);
    DevBuf<int32_t> chunk_row(std::max<int64_t>(1, edge_chunks(g.nnz)), s);
    DevBuf<unsigned long long> inter_cursor(1, s);
    chunk_rows_device(g.row_ptr, n, g.nnz, chunk_row, s);
    ++launches;
    for (; pass < p.max_passes && M > 0; ++pass) {
        GB_CUDA(cudaEventRecord(ea, s));
        const int iters = local_move(tolerance);
        if (p.refine && (p.refine_depth < 0 || pass <= p.refine_depth)) {
            // Refinement (RG:7330-7392): bounds = this membership, every vertex
            // back to a singleton, one sweep of localMovingPhase<true>.
            GB_REQUIRE(exact, GBGPU_E_UNSUPPORTED, "Leiden refinement needs the serial-order engine");
            DevBuf<uint32_t> vcob(n, s);
            GB_CUDA(cudaMemcpyAsync(vcob, vcom, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
            k_init_state<<<grid_for(n, kT), kT, 0, s>>>(g.row_ptr, n, vcom, ctot, vaff);
            GB_LAUNCH_CHECK();
            ++launches;
            run_exact(tolerance, 1, vcob.get());
        }
        GB_CUDA(cudaEventRecord(eb, s));
        GB_CUDA(cudaEventSynchronize(eb));
        lm_ms += elapsed(ea, eb);
        total_iters += iters;

        // countCommunities + renumber.
        GB_CUDA(cudaMemsetAsync(exists, 0, n * sizeof(int32_t), s));
        k_mark_exists<<<grid_for(n, kT), kT, 0, s>>>(vcom, n, exists);
        GB_LAUNCH_CHECK();
        exclusive_scan_i32_to_i64(exists, cmap, n, cmap.get() + n, s);
        const int64_t C = read_dev(cmap.get() + n, s);
        launches += 4;
        if (pass == 0) pass0_comms = C;
        if (pass >= p.max_passes - 1) break;

        GB_CUDA(cudaEventRecord(ea, s));
        DevBuf<long long> sweight(C, s);
        k_super_weights<<<grid_for(n, kT), kT, 0, s>>>(exists, cmap, ctot, n, sweight);
        GB_LAUNCH_CHECK();
        k_apply_renumber<<<grid_for(n, kT), kT, 0, s>>>(vcom, n, cmap);
        GB_LAUNCH_CHECK();
        launches += 2;

        // Super-graph adjacency (inter-community edges only, :2184-2224).
        DevBuf<uint64_t> ikeys(g.nnz > 0 ? g.nnz : 1, s);
        int64_t ninter = 0;
        if (g.nnz > 0) {
            GB_CUDA(cudaMemsetAsync(inter_cursor, 0, sizeof(unsigned long long), s));
            k_inter_edges<<<grid_for(edge_chunks(g.nnz), 1), kInterThreads, 0, s>>>(
                g.row_ptr, g.col, vcom, n, g.nnz, chunk_row, ikeys, inter_cursor);
            GB_LAUNCH_CHECK();
            ninter = (int64_t)read_dev(inter_cursor.get(), s);
            launches += 1;
        }
        DevBuf<int32_t> sdeg(C, s);
        DevBuf<int64_t> soff(C + 1, s);
        GB_CUDA(cudaMemsetAsync(sdeg, 0, C * sizeof(int32_t), s));
        DevBuf<uint32_t> snbr, sw;
        int64_t nuniq = 0;
        if (ninter > 0) {
            const int cb = bits_for((uint64_t)(C > 0 ? C - 1 : 0));
            radix_sort_keys_u64(ikeys, ninter, 32 + cb, s);
            DevBuf<int32_t> uflag(ninter, s);
            DevBuf<int64_t> upos(ninter + 1, s);
            k_rle_flags<<<grid_for(ninter, kT), kT, 0, s>>>(ikeys, ninter, uflag);
            GB_LAUNCH_CHECK();
            exclusive_scan_i32_to_i64(uflag, upos, ninter, upos.get() + ninter, s);
            nuniq = read_dev(upos.get() + ninter, s);
            snbr.alloc(nuniq, s);
            sw.alloc(nuniq, s);
            DevBuf<int64_t> ustart(nuniq, s);
            k_rle_emit<<<grid_for(ninter, kT), kT, 0, s>>>(ikeys, ninter, uflag, upos, nuniq, snbr, sw, sdeg, ustart);
            GB_LAUNCH_CHECK();
            k_rle_weights<<<grid_for(nuniq, kT), kT, 0, s>>>(ustart, nuniq, ninter, sw);
            GB_LAUNCH_CHECK();
            launches += 7 + 3 * ((32 + cb + 7) / 8);
        }
        {
            // soff = exclusive scan of sdeg (int32 -> int64)
            exclusive_scan_i32_to_i64(sdeg, soff, C, soff.get() + C, s);
            launches += 3;
        }

        // Batched super-move.
        DevBuf<uint32_t> scomm(C, s);
        DevBuf<unsigned long long> sctot(C, s);
        iota_u32(scomm, C, s);
        GB_CUDA(cudaMemcpyAsync(sctot, sweight, C * sizeof(long long), cudaMemcpyDeviceToDevice, s));
        DevBuf<int32_t> aflag(C, s);
        DevBuf<int64_t> apos(C + 1, s);
        k_active_flags<<<grid_for(C, kT), kT, 0, s>>>(sdeg, C, aflag);
        GB_LAUNCH_CHECK();
        exclusive_scan_i32_to_i64(aflag, apos, C, apos.get() + C, s);
        const int64_t na = read_dev(apos.get() + C, s);
        launches += 5;
        const int super_max_iter = std::min(3, p.max_iterations);
        if (na > 0 && super_max_iter > 0) {
            DevBuf<uint32_t> active(na, s);
            k_active_emit<<<grid_for(C, kT), kT, 0, s>>>(aflag, apos, C, active);
            GB_LAUNCH_CHECK();
            const int64_t batch = std::max(1, p.super_move_batch);
            const int64_t nbatch = ceil_div(C, batch);
            DevBuf<int64_t> bstart(nbatch + 1, s);
            k_batch_starts<<<grid_for(nbatch + 1, kT), kT, 0, s>>>(active, na, nbatch, batch, bstart);
            GB_LAUNCH_CHECK();
            DevBuf<uint32_t> proposed(C, s);
            DevBuf<double> pdelta(C, s);
            // Largest super-degree decides the per-warp global table size.
            int64_t max_sdeg = 0;
            {
                DevBuf<unsigned long long> md(1, s);
                GB_CUDA(cudaMemsetAsync(md, 0, sizeof(unsigned long long), s));
                k_max_degree<<<grid_for(C, kT), kT, 0, s>>>(soff, C, md);
                GB_LAUNCH_CHECK();
                max_sdeg = (int64_t)read_dev(md.get(), s);
                ++launches;
            }
            const bool single = nuniq <= p.super_single_cta_max_edges;
            // Super-nodes above big_min neighbours get a CTA each (the cluster
            // kernel: kBigSuper; batched launches: kBigSuperBatched); warps then
            // need tables for at most big_min.
            const int64_t big_min = single ? kBigSuper : kBigSuperBatched;   // degree above: a CTA each
            const int64_t warp_max = std::min<int64_t>(max_sdeg, big_min);
            int64_t gcap = 64;
            while (gcap < 2 * warp_max) gcap <<= 1;
            // Batched launches split super-nodes above kHugeSeg over CTAs; the
            // per-CTA tables then only hold the ones below.
            const int64_t split_min = std::max<int64_t>(big_min, p.super_split_min);
            const bool split_huge = !single && max_sdeg > split_min;
            int64_t bcap = 64;
            while (bcap < 2 * (split_huge ? split_min : max_sdeg)) bcap <<= 1;
            int64_t nbig = 0;
            DevBuf<uint32_t> big_active;
            DevBuf<int64_t> bigstart(nbatch + 1, s);
            {
                DevBuf<int32_t> bflag(na, s);
                DevBuf<int64_t> bpos(na + 1, s);
                k_big_super_flags<<<grid_for(na, kT), kT, 0, s>>>(active, na, soff, big_min, bflag);
                GB_LAUNCH_CHECK();
                exclusive_scan_i32_to_i64(bflag, bpos, na, bpos.get() + na, s);
                nbig = read_dev(bpos.get() + na, s);
                big_active.alloc(nbig > 0 ? nbig : 1, s);
                if (nbig) {
                    k_big_super_emit<<<grid_for(na, kT), kT, 0, s>>>(active, na, bflag, bpos, big_active);
                    GB_LAUNCH_CHECK();
                }
                k_batch_starts<<<grid_for(nbatch + 1, kT), kT, 0, s>>>(big_active, nbig, nbatch, batch, bigstart);
                GB_LAUNCH_CHECK();
                launches += 6;
            }
            const int cluster = super_cluster_size(sm_smem);
            // Batched launches: the big super-nodes of a batch get one CTA each.
            std::vector<int64_t> bs, bgs;
            int64_t max_big_in_batch = 0;
            if (!single) {
                bs.resize(nbatch + 1);
                bgs.resize(nbatch + 1);
                GB_CUDA(cudaMemcpyAsync(bs.data(), bstart.get(), (nbatch + 1) * sizeof(int64_t),
                                        cudaMemcpyDeviceToHost, s));
                GB_CUDA(cudaMemcpyAsync(bgs.data(), bigstart.get(), (nbatch + 1) * sizeof(int64_t),
                                        cudaMemcpyDeviceToHost, s));
                GB_CUDA(cudaStreamSynchronize(s));
                for (int64_t bt = 0; bt < nbatch; ++bt) max_big_in_batch = std::max(max_big_in_batch, bgs[bt + 1] - bgs[bt]);
            }
            const int big_grid = (int)std::min<int64_t>(std::max<int64_t>(1, max_big_in_batch), 4 * kNumSMs);
            const int64_t big_tables = nbig ? (single ? (int64_t)cluster : (int64_t)big_grid) * bcap : 1;
            DevBuf<uint32_t> bk(big_tables, s);
            DevBuf<uint32_t> bv(big_tables, s);
            // Per-warp global tables for super-nodes of kSmSmall / 2 .. big_min neighbours.
            const int64_t nwarps_total = single ? (int64_t)cluster * 32 : (int64_t)kNumSMs * 4 * 8;
            DevBuf<uint32_t> gk(gcap > kSmSmall ? nwarps_total * gcap : 1, s);
            DevBuf<uint32_t> gv(gcap > kSmSmall ? nwarps_total * gcap : 1, s);
            DevBuf<uint8_t> light(nbatch, s);
            if (single) {
                k_batch_light<<<grid_for(nbatch, kT), kT, 0, s>>>(active, bstart, soff, nbatch, kLightNodes, kLightDeg,
                                                                 light);
                GB_LAUNCH_CHECK();
                ++launches;
            }
            SmArgs sa{soff, snbr, sw, sweight, scomm, sctot, active, bstart, nbatch, proposed, pdelta, M, R,
                      gk, gv, gcap > kSmSmall ? gcap : 0, big_active.get(), bigstart.get(), bk.get(), bv.get(),
                      bcap, light.get(), big_min};
            sa.yMh = la.dq.yMh;
            sa.yMl = la.dq.yMl;
            // Batched launches: super-nodes above kHugeSeg neighbours, split over CTAs.
            struct HugeBatch { int64_t e0 = 0, ne = 0, t0 = 0, nt = 0; };
            std::vector<HugeBatch> hb;
            DevBuf<uint32_t> huge_c, hkeys, hvals, part_c;
            DevBuf<int64_t> huge_toff;
            DevBuf<uint32_t> huge_tcap;
            DevBuf<int32_t> huge_tfirst, huge_tcount, huge_done;
            DevBuf<int2> huge_eseg, huge_tseg;
            DevBuf<double> part_d;
            int64_t hpool = 0;
            if (split_huge && nbig > 0) {
                std::vector<uint32_t> big_h(nbig);
                std::vector<int64_t> soff_h(C + 1);
                GB_CUDA(cudaMemcpyAsync(big_h.data(), big_active.get(), nbig * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                        s));
                GB_CUDA(cudaMemcpyAsync(soff_h.data(), soff, (C + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
                GB_CUDA(cudaStreamSynchronize(s));
                std::vector<uint32_t> hc, htcap;
                std::vector<int64_t> htoff;
                std::vector<int32_t> htfirst, htcount;
                std::vector<int2> he, ht;
                hb.assign(nbatch, HugeBatch{});
                for (const uint32_t c : big_h) {   // ascending ids: batches in order
                    const int64_t deg = soff_h[c + 1] - soff_h[c];
                    if (deg <= split_min) continue;
                    const int j = (int)hc.size();
                    const int64_t bt = (int64_t)c / batch;
                    int64_t H = 64;
                    while (H < 2 * deg) H <<= 1;
                    hc.push_back(c);
                    htoff.push_back(hpool);
                    htcap.push_back((uint32_t)H);
                    hpool += H;
                    HugeBatch& b = hb[bt];
                    if (b.ne == 0 && b.nt == 0) { b.e0 = (int64_t)he.size(); b.t0 = (int64_t)ht.size(); }
                    for (int64_t q = 0; q < ceil_div(deg, kHugeSeg); ++q) he.push_back(make_int2(j, (int)q));
                    htfirst.push_back((int32_t)ht.size());
                    const int64_t ntseg = ceil_div(H, kHugeSeg);
                    htcount.push_back((int32_t)ntseg);
                    for (int64_t q = 0; q < ntseg; ++q) ht.push_back(make_int2(j, (int)q));
                    b.ne = (int64_t)he.size() - b.e0;
                    b.nt = (int64_t)ht.size() - b.t0;
                }
                const int64_t nh = (int64_t)hc.size();
                if (nh > 0) {
                    auto up = [&](auto& buf, const auto& vec) {
                        buf.alloc(vec.size(), s);
                        GB_CUDA(cudaMemcpyAsync(buf.get(), vec.data(), vec.size() * sizeof(vec[0]),
                                                cudaMemcpyHostToDevice, s));
                    };
                    up(huge_c, hc);
                    up(huge_toff, htoff);
                    up(huge_tcap, htcap);
                    up(huge_tfirst, htfirst);
                    up(huge_tcount, htcount);
                    up(huge_eseg, he);
                    up(huge_tseg, ht);
                    huge_done.alloc(nh, s);
                    GB_CUDA(cudaMemsetAsync(huge_done, 0, nh * sizeof(int32_t), s));
                    hkeys.alloc(hpool, s);
                    hvals.alloc(hpool, s);
                    part_d.alloc(ht.size(), s);
                    part_c.alloc(ht.size(), s);
                    sa.huge_min = split_min;
                    sa.huge_c = huge_c.get();
                    sa.huge_toff = huge_toff.get();
                    sa.huge_tcap = huge_tcap.get();
                    sa.huge_tfirst = huge_tfirst.get();
                    sa.huge_tcount = huge_tcount.get();
                    sa.huge_done = huge_done.get();
                    sa.huge_eseg = huge_eseg.get();
                    sa.huge_tseg = huge_tseg.get();
                    sa.hkeys = hkeys.get();
                    sa.hvals = hvals.get();
                    sa.part_d = part_d.get();
                    sa.part_c = part_c.get();
                    launches += 1;
                }
            }
            GB_REQUIRE(!split_huge || hpool > 0, GBGPU_E_CUDA, "super-move: no huge super-node to split");
            DevBuf<int> iters_d(1, s), gmoves(super_max_iter, s);
            DevBuf<long long> moves_d(1, s);
            launches += 2;
            if (single) {
                GB_CUDA(cudaMemsetAsync(gmoves, 0, super_max_iter * sizeof(int), s));
                cudaLaunchConfig_t cfg = {};
                cfg.gridDim = dim3(cluster);
                cfg.blockDim = dim3(1024);
                cfg.dynamicSmemBytes = sm_smem;
                cfg.stream = s;
                cudaLaunchAttribute attr[1];
                attr[0].id = cudaLaunchAttributeClusterDimension;
                attr[0].val.clusterDim.x = cluster;
                attr[0].val.clusterDim.y = 1;
                attr[0].val.clusterDim.z = 1;
                cfg.attrs = attr;
                cfg.numAttrs = 1;
                int* gm = gmoves.get();
                int* itp = iters_d.get();
                long long* mvp = moves_d.get();
                GB_CUDA(cudaLaunchKernelEx(&cfg, k_super_move_cluster, sa, super_max_iter, itp, mvp, gm));
                GB_LAUNCH_CHECK();
                super_ctas = cluster;
                ++launches;
                super_iters += read_dev(iters_d.get(), s);
                super_moves += read_dev(moves_d.get(), s);
            } else {
                DevBuf<int> mv(1, s);
                // A batch's three proposal paths read the state before the
                // batch and write disjoint super-nodes' proposals: the
                // CTA-per-super-node and split paths run on side streams
                // beside the warp path, joined before the commit.
                struct BatchFork {
                    cudaStream_t sb = nullptr, sh = nullptr;
                    cudaEvent_t fork = nullptr, jb = nullptr, jh = nullptr;
                    ~BatchFork() {
                        if (fork) cudaEventDestroy(fork);
                        if (jb) cudaEventDestroy(jb);
                        if (jh) cudaEventDestroy(jh);
                        if (sb) cudaStreamDestroy(sb);
                        if (sh) cudaStreamDestroy(sh);
                    }
                } bf;
                GB_CUDA(cudaStreamCreateWithFlags(&bf.sb, cudaStreamNonBlocking));
                GB_CUDA(cudaStreamCreateWithFlags(&bf.sh, cudaStreamNonBlocking));
                GB_CUDA(cudaEventCreateWithFlags(&bf.fork, cudaEventDisableTiming));
                GB_CUDA(cudaEventCreateWithFlags(&bf.jb, cudaEventDisableTiming));
                GB_CUDA(cudaEventCreateWithFlags(&bf.jh, cudaEventDisableTiming));
                for (int it = 0; it < super_max_iter; ++it) {
                    GB_CUDA(cudaMemsetAsync(mv, 0, sizeof(int), s));
                    if (hpool > 0) {
                        GB_CUDA(cudaMemsetAsync(hkeys, 0xFF, hpool * sizeof(uint32_t), s));
                        GB_CUDA(cudaMemsetAsync(hvals, 0, hpool * sizeof(uint32_t), s));
                    }
                    for (int64_t bt = 0; bt < nbatch; ++bt) {
                        const int64_t cnt = bs[bt + 1] - bs[bt];
                        if (cnt == 0) continue;
                        const int64_t nb = bgs[bt + 1] - bgs[bt];
                        const bool huge = hpool > 0 && hb[bt].ne > 0;
                        if (huge || nb > 0) GB_CUDA(cudaEventRecord(bf.fork, s));
                        if (huge) {
                            GB_CUDA(cudaStreamWaitEvent(bf.sh, bf.fork, 0));
                            k_super_huge_accum<<<(int)hb[bt].ne, 1024, 0, bf.sh>>>(sa, hb[bt].e0);
                            GB_LAUNCH_CHECK();
                            k_super_huge_select<<<(int)hb[bt].nt, 1024, 0, bf.sh>>>(sa, hb[bt].t0);
                            GB_LAUNCH_CHECK();
                            GB_CUDA(cudaEventRecord(bf.jh, bf.sh));
                            launches += 2;
                        }
                        if (nb > 0) {
                            GB_CUDA(cudaStreamWaitEvent(bf.sb, bf.fork, 0));
                            const int bgrid = (int)std::min<int64_t>(nb, big_grid);
                            k_super_propose_big_batch<<<bgrid, kBigBatchThreads, 0, bf.sb>>>(sa, bt);
                            GB_LAUNCH_CHECK();
                            GB_CUDA(cudaEventRecord(bf.jb, bf.sb));
                            ++launches;
                        }
                        if (cnt > nb) {
                            const int grid = (int)std::min<int64_t>(ceil_div(cnt - nb, 8), nwarps_total / 8);
                            k_super_propose_batch<<<grid, 256, 0, s>>>(sa, bt);
                            GB_LAUNCH_CHECK();
                            ++launches;
                        }
                        if (huge) GB_CUDA(cudaStreamWaitEvent(s, bf.jh, 0));
                        if (nb > 0) GB_CUDA(cudaStreamWaitEvent(s, bf.jb, 0));
                        k_super_commit_batch<<<(int)std::min<int64_t>(ceil_div(cnt, 256), 1024), 256, 0, s>>>(sa, bt, mv);
                        GB_LAUNCH_CHECK();
                        ++launches;
                    }
                    ++super_iters;
                    const int moved = read_dev(mv.get(), s);
                    super_moves += moved;
                    if (moved == 0) break;
                }
            }
        }

        // Remap, first-occurrence renumber, community totals.
        DevBuf<int32_t> firstpos(C, s);
        fill_u32(reinterpret_cast<uint32_t*>(firstpos.get()), 0x7FFFFFFFu, C, s);
        k_remap<<<grid_for(n, kT), kT, 0, s>>>(vcom, n, scomm, firstpos);
        GB_LAUNCH_CHECK();
        DevBuf<int32_t> fflag(n, s);
        DevBuf<int64_t> rk(n + 1, s);
        k_first_flags<<<grid_for(n, kT), kT, 0, s>>>(vcom, n, firstpos, fflag);
        GB_LAUNCH_CHECK();
        exclusive_scan_i32_to_i64(fflag, rk, n, rk.get() + n, s);
        const int64_t merged = read_dev(rk.get() + n, s);
        k_first_apply<<<grid_for(n, kT), kT, 0, s>>>(vcom, n, firstpos, rk);
        GB_LAUNCH_CHECK();
        GB_CUDA(cudaMemsetAsync(ctot, 0, n * sizeof(unsigned long long), s));
        k_ctot_from_members<<<grid_for(n, kT), kT, 0, s>>>(g.row_ptr, vcom, n, ctot);
        GB_LAUNCH_CHECK();
        launches += 8;
        GB_CUDA(cudaEventRecord(eb, s));
        GB_CUDA(cudaEventSynchronize(eb));
        agg_ms += elapsed(ea, eb);
        aggregated = merged;
        if (merged >= prev || merged == 1) break;
        if ((double)merged / (double)prev >= p.aggregation_tolerance) break;
        prev = merged;
        GB_CUDA(cudaMemsetAsync(vaff, 1, n, s));
        tolerance /= p.tolerance_drop;
    }
    // distinct final communities
    GB_CUDA(cudaMemsetAsync(exists, 0, n * sizeof(int32_t), s));
    k_mark_exists<<<grid_for(n, kT), kT, 0, s>>>(vcom, n, exists);
    GB_LAUNCH_CHECK();
    exclusive_scan_i32_to_i64(exists, cmap, n, cmap.get() + n, s);
    const int64_t distinct = read_dev(cmap.get() + n, s);
    launches += 4;
    GB_CUDA(cudaEventRecord(e1, s));
    GB_CUDA(cudaEventSynchronize(e1));
    if (st) {
        st->leiden_ms += elapsed(e0, e1);
        st->local_move_ms += lm_ms;
        st->aggregate_ms += agg_ms;
        st->passes = pass + 1;
        st->iterations = total_iters;
        st->super_move_iterations = super_iters;
        st->super_move_ctas = super_ctas;
        st->super_moves = super_moves;
        st->pass0_communities = pass0_comms;
        st->aggregated_communities = aggregated;
        st->communities = distinct;
        st->resolution = R;
        st->kernel_launches += launches;
        st->local_move_rounds = exact_rounds;
        st->local_move_evaluations = exact_evals;
        st->local_move_streams = exact ? 0 : streams;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(ea);
    cudaEventDestroy(eb);
}

// ---- auto resolution ----
namespace {
__global__ void k_degree_moments(const int64_t* __restrict__ rp, int64_t n, double avg, double* __restrict__ partial) {
    double s = 0.0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const double diff = (double)(rp[v + 1] - rp[v]) - avg;
        s += diff * diff;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
    __shared__ double ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += ws[i];
        partial[blockIdx.x] = t;
    }
}
}  // namespace

double auto_resolution_device(const int64_t* row_ptr, int64_t n, int64_t nnz, cudaStream_t s) {
    if (n == 0) return 1.0;
    const int64_t m = nnz / 2;
    const double avg = (double)m / (double)n;
    const int grid = 1024;
    DevBuf<double> partial(grid, s);
    k_degree_moments<<<grid, kT, 0, s>>>(row_ptr, n, avg, partial);
    GB_LAUNCH_CHECK();
    std::vector<double> h(grid);
    GB_CUDA(cudaMemcpyAsync(h.data(), partial.get(), grid * sizeof(double), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    double sum_sq = 0.0;
    for (double x : h) sum_sq += x;
    const double variance = sum_sq / (double)n;
    const double cv = (avg > 0) ? std::sqrt(variance) / avg : 0.0;
    double resolution = 0.5 + 0.25 * std::log10(avg + 1);
    resolution = std::max(0.5, std::min(1.2, resolution));
    if (cv > 2.0) {
        const double factor = 2.0 / std::max(2.0, std::sqrt(cv));
        resolution = std::max(0.5, resolution * factor);
    }
    return resolution;
}

}  // namespace gb

namespace gb {

namespace {

__device__ __forceinline__ uint64_t sc_mix(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Two checks per index i, both against full double divisions:
//  (a) deltaModularity of a graph with total weight M and resolution R, on
//      counts and totals drawn from that graph's ranges (ku up to 2^24,
//      totals up to 2M), delta_qi against delta_q;
//  (b) a bare quotient x / m over random 53-bit significands with exponents
//      in [-200, 200], div_rn_by against __ddiv_rn, with the reciprocal
//      pair formed on the device the way make_dq forms it on the host.
__global__ void k_selfcheck_delta(DqConst q, int64_t count, uint64_t seed, unsigned long long* bad) {
    unsigned long long local = 0;
    const double twoM = 2.0 * q.M;
    const long long tmax = twoM < 9.0e15 ? (long long)twoM : (1ll << 53);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t h0 = sc_mix(seed ^ (uint64_t)i), h1 = sc_mix(h0), h2 = sc_mix(h1), h3 = sc_mix(h2);
        // ku log-uniform in [1, 2^24], capped by the graph's total weight
        const int lg = (int)(h0 & 31) % 25;
        long long ku = 1 + (long long)((h0 >> 8) & ((1ull << lg) - 1));
        if (ku > tmax && tmax > 0) ku = tmax;
        const long long kuc = 1 + (long long)((h1 & 0xFFFFFFFFull) % (uint64_t)ku);
        const long long kud = (long long)((h1 >> 32) % (uint64_t)(ku + 1));
        // totals: half uniform over [0, 2M], half small
        const long long span = (h2 & 1) ? tmax : (long long)(ku * 4 + 16);
        const long long sc = (long long)((h2 >> 1) % (uint64_t)(span + 1));
        const long long sd = (long long)((h3 >> 1) % (uint64_t)(span + 1));
        const double ref = delta_q((double)kuc, (double)kud, (double)ku, (double)sc, (double)sd, q.M, q.R);
        const double got = delta_qi(q, kuc, kud, ku, sc, sd);
        local += __double_as_longlong(ref) != __double_as_longlong(got);
        // bare quotient
        const uint64_t h4 = sc_mix(h3), h5 = sc_mix(h4);
        const int ex = (int)((h4 >> 52) % 401) - 200, em = (int)((h5 >> 52) % 401) - 200;
        const double x = __longlong_as_double((long long)(((uint64_t)(1023 + ex) << 52) | (h4 & 0xFFFFFFFFFFFFFull))) *
                         (h3 & 1 ? -1.0 : 1.0);
        const double m = __longlong_as_double((long long)(((uint64_t)(1023 + em) << 52) | (h5 & 0xFFFFFFFFFFFFFull)));
        const double yh = __drcp_rn(m);
        const double yl = __dmul_rn(__fma_rn(-yh, m, 1.0), yh);
        local += __double_as_longlong(__ddiv_rn(x, m)) != __double_as_longlong(div_rn_by(x, m, yh, yl));
    }
    if (local) atomicAdd(bad, local);
}

}  // namespace

namespace {
__global__ void k_fill_atab(double* tab, double M) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= kAtabMax; k += gridDim.x * blockDim.x)
        tab[k] = __ddiv_rn((double)k, M);
}
}  // namespace

void fill_atab(double* tab, double M, cudaStream_t s) {
    k_fill_atab<<<(kAtabMax + 256) / 256, 256, 0, s>>>(tab, M);
    GB_CUDA(cudaGetLastError());
}

int64_t selfcheck_delta_device(double M, double R, int64_t count, uint64_t seed, cudaStream_t s) {
    GB_REQUIRE(M >= 1.0 && M < 4.0e15 && R > 0.0 && R < 1.0e6 && count >= 0, GBGPU_E_INVALID,
               "selfcheck_delta: M must be in [1, 4e15), R in (0, 1e6), count >= 0");
    DevBuf<unsigned long long> bad(1, s);
    DevBuf<double> atab(kAtabMax + 1, s);
    fill_atab(atab.get(), M, s);
    GB_CUDA(cudaMemsetAsync(bad.get(), 0, sizeof(unsigned long long), s));
    if (count > 0) {
        const int64_t blocks = std::min<int64_t>((count + 255) / 256, 152 * 16);
        DqConst q = make_dq(M, R);
        q.atab = atab.get();
        k_selfcheck_delta<<<(int)blocks, 256, 0, s>>>(q, count, seed, bad.get());
        GB_CUDA(cudaGetLastError());
    }
    unsigned long long h = 0;
    GB_CUDA(cudaMemcpyAsync(&h, bad.get(), sizeof(h), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    return (int64_t)h;
}

}  // namespace gb
