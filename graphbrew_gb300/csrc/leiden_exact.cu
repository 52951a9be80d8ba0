// leiden_exact.cu -- local moving with the reference's serial semantics.
//
// localMovingPhase<false> (bench/include/graphbrew/reorder/reorder_graphbrew.h:1588-1734)
// with one thread is a Gauss-Seidel sweep in vertex-id order: vertex u sees
// every move of the vertices before it.  This engine reproduces that sweep
// exactly with a sliding window of speculative decisions:
//
//   * the window [P, E) holds decisions D_prev from the previous round
//     (unknown for vertices that just entered);
//   * each round re-evaluates every window vertex u against the committed
//     state plus the D_prev moves of window vertices before u (neighbour
//     communities, affected flags and community totals at "time u");
//   * the first vertex x whose new decision differs from D_prev bounds the
//     exact prefix: all of [P, x] was evaluated from exact inputs (induction
//     from P), so it is committed; the rest carries its new decisions forward.
//
// Community totals at time u come from an event table rebuilt every round by
// one CTA: each speculative move contributes (old, -k) and (new, +k) at its
// time; events are stably radix-sorted by community slot in shared memory and
// prefix-summed, and a lookup binary-searches the community's events for the
// last time before u.  All totals are exact integers, so every
// Delta-modularity equals the serial one.
//
// Vertices above kWarpMaxDeg ("hubs") are split into 4096-edge segments, each
// accumulated by its own CTA into the hub's global table, then scanned in
// 4096-slot segments; the last CTA of a hub reduces the partial maxima.  The
// whole round reads its window bounds from a device control block, so the host
// enqueues rounds without waiting and checks completion every few rounds.
//
// The iteration's totalDelta decides the tolerance break; it is summed in a
// fixed tree order with a rigorous error bound and re-summed serially in
// vertex order only when the bound cannot settle the comparison.
#include <algorithm>
#include <cmath>
#include <vector>

#include "gb_common.cuh"
#include "gb_leiden_internal.cuh"

namespace gb {

namespace {

constexpr int kT = 256;
constexpr uint8_t kUnknown = 2;
constexpr int kWindowMax = 8192;              // window vertices (events <= 2 x window)
constexpr int kEventsMax = 2 * kWindowMax;    // 16384 -> 14-bit event index
constexpr int kTableSlots = 4 * kWindowMax;   // 32768 hash slots -> 15 bits (+1 for padding)
constexpr int kEvThreads = 1024;
constexpr int kHubSeg = 4096;                 // edges per hub-accumulation CTA
constexpr int kTabSeg = 4096;                 // table slots per hub-selection CTA
constexpr unsigned long long kNoChange = ~0ull;

struct Ctl {
    long long P, E, n, B;
    unsigned long long first_change;
    long long es0, es1;       // hub edge-segment range of the window
    long long ts0, ts1;       // hub table-segment range of the window
    long long round;
};

struct HubSeg {
    int32_t hub;      // index into the hub arrays
    int32_t part;     // segment number within the hub
};

struct ExactState {
    const int64_t* rp;
    const int32_t* col;
    uint32_t* vcom;
    unsigned long long* ctot;
    uint8_t* vaff;
    Ctl* ctl;
    // decisions, double-buffered by round parity
    uint32_t* best[2];
    uint8_t* act[2];
    double* delta[2];
    double* final_delta;
    // event table
    uint32_t* hkey;       // kTableSlots
    int32_t* sstart;      // kTableSlots
    int32_t* send;
    uint32_t* etime_raw;  // kEventsMax (by event index)
    long long* eval_raw;
    uint32_t* stime;      // sorted
    long long* epre;      // inclusive prefix within slot
    long long* gscan;     // scratch: inclusive scan over all sorted events
    // hubs
    const uint32_t* hub_v;        // hub vertex ids (ascending)
    const int64_t* hub_toff;      // table offset
    const uint32_t* hub_tcap;     // table capacity (pow2)
    const int32_t* hub_tfirst;    // first table segment index of each hub
    const int32_t* hub_tcount;    // table segments of each hub
    const HubSeg* eseg;           // edge segments (hub id order)
    const uint32_t* eseg_v;       // hub vertex of each edge segment
    long long n_eseg;
    const HubSeg* tseg;           // table segments
    const uint32_t* tseg_v;
    long long n_tseg;
    uint32_t* tkeys;              // hub tables (pool)
    uint32_t* tvals;
    int32_t* hub_any;
    int32_t* hub_done;
    double* part_d;               // per table segment
    uint32_t* part_c;
    double M, R;
};

__device__ __forceinline__ uint32_t slot_hash(uint32_t c) {
    return (uint32_t)(((uint64_t)c * 0x9E3779B97F4A7C15ull) >> 40);
}

__device__ __forceinline__ int find_slot(const uint32_t* hkey, uint32_t c) {
    uint32_t h = slot_hash(c) & (kTableSlots - 1);
    while (true) {
        const uint32_t k = hkey[h];
        if (k == c) return (int)h;
        if (k == kNone) return -1;
        h = (h + 1) & (kTableSlots - 1);
    }
}

// Community total at time u.
__device__ __forceinline__ long long sigma_at(const ExactState& a, uint32_t c, uint32_t u) {
    long long s = (long long)a.ctot[c];
    const int slot = find_slot(a.hkey, c);
    if (slot < 0) return s;
    int lo = a.sstart[slot], hi = a.send[slot];
    int l = lo, r = hi;
    while (l < r) {
        const int mid = (l + r) >> 1;
        if (a.stime[mid] < u) l = mid + 1; else r = mid;
    }
    if (l > lo) s += a.epre[l - 1];
    return s;
}

struct Round {
    long long P, E;
    const uint32_t* pbest;
    const uint8_t* pact;
    uint32_t* nbest;
    uint8_t* nact;
    double* ndelta;
};

__device__ __forceinline__ Round round_view(const ExactState& a) {
    Round r;
    r.P = a.ctl->P;
    r.E = a.ctl->E;
    const int par = (int)(a.ctl->round & 1);
    r.pbest = a.best[par];
    r.pact = a.act[par];
    r.nbest = a.best[par ^ 1];
    r.nact = a.act[par ^ 1];
    r.ndelta = a.delta[par ^ 1];
    return r;
}

__device__ __forceinline__ bool prev_mover(const ExactState& a, const Round& r, int64_t v) {
    return r.pact[v] == 1 && r.pbest[v] != a.vcom[v];
}

__device__ __forceinline__ uint32_t comm_at(const ExactState& a, const Round& r, int64_t v, int64_t u) {
    if (v >= r.P && v < u && prev_mover(a, r, v)) return r.pbest[v];
    return a.vcom[v];
}

__device__ __forceinline__ void record(const ExactState& a, const Round& r, int64_t u, uint8_t act, uint32_t best,
                                       double delta) {
    r.nact[u] = act;
    r.nbest[u] = best;
    r.ndelta[u] = delta;
    // Only the move itself is visible to later vertices: "inactive" and
    // "evaluated, stays" are the same decision.
    const uint32_t cur = a.vcom[u];
    const uint8_t pa = r.pact[u];
    const bool moves = act == 1 && best != cur;
    const bool pmoves = pa == 1 && r.pbest[u] != cur;
    if (pa == kUnknown || moves != pmoves || (moves && best != r.pbest[u]))
        atomicMin(&a.ctl->first_change, (unsigned long long)u);
}

__device__ __forceinline__ long long lower_bound_u32(const uint32_t* a, long long n, uint32_t key) {
    long long lo = 0, hi = n;
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// Event table (one CTA): hash slots, stable sort by slot, prefix sums.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kEvThreads) k_ex_table(ExactState a) {
    extern __shared__ uint32_t sm[];
    uint32_t* bufA = sm;                               // kEventsMax
    uint32_t* bufB = sm + kEventsMax;                  // kEventsMax
    int32_t* wcnt = reinterpret_cast<int32_t*>(sm + 2 * kEventsMax);  // 32 x 257
    __shared__ int32_t digit_off[256];
    __shared__ long long warp_tot[32];
    const long long P = a.ctl->P, E = a.ctl->E;
    if (P >= a.ctl->n) return;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int W = (int)(E - P);
    const int m = 2 * W;
    const Round r = round_view(a);
    for (int i = tid; i < kTableSlots; i += blockDim.x) a.hkey[i] = kNone;
    if (tid == 0) {
        a.ctl->first_change = kNoChange;
        a.ctl->es0 = lower_bound_u32(a.eseg_v, a.n_eseg, (uint32_t)P);
        a.ctl->es1 = lower_bound_u32(a.eseg_v, a.n_eseg, (uint32_t)E);
        a.ctl->ts0 = lower_bound_u32(a.tseg_v, a.n_tseg, (uint32_t)P);
        a.ctl->ts1 = lower_bound_u32(a.tseg_v, a.n_tseg, (uint32_t)E);
    }
    __syncthreads();
    // Events of D_prev movers, packed as (slot << 14 | event index).
    constexpr uint32_t kPad = (uint32_t)kTableSlots << 14;
    for (int i = tid; i < W; i += blockDim.x) {
        const int64_t wv = P + i;
        uint32_t p0 = kPad | (uint32_t)(2 * i), p1 = kPad | (uint32_t)(2 * i + 1);
        if (r.pact[wv] == 1 && r.pbest[wv] != a.vcom[wv]) {
            const long long deg = (long long)(a.rp[wv + 1] - a.rp[wv]);
            const uint32_t cs[2] = {a.vcom[wv], r.pbest[wv]};
            uint32_t ks[2];
            for (int j = 0; j < 2; ++j) {
                uint32_t h = slot_hash(cs[j]) & (kTableSlots - 1);
                while (true) {
                    const uint32_t prev = atomicCAS(&a.hkey[h], kNone, cs[j]);
                    if (prev == kNone || prev == cs[j]) break;
                    h = (h + 1) & (kTableSlots - 1);
                }
                ks[j] = h;
            }
            p0 = (ks[0] << 14) | (uint32_t)(2 * i);
            p1 = (ks[1] << 14) | (uint32_t)(2 * i + 1);
            a.eval_raw[2 * i] = -deg;
            a.eval_raw[2 * i + 1] = deg;
        } else {
            a.eval_raw[2 * i] = 0;
            a.eval_raw[2 * i + 1] = 0;
        }
        a.etime_raw[2 * i] = (uint32_t)wv;
        a.etime_raw[2 * i + 1] = (uint32_t)wv;
        bufA[2 * i] = p0;
        bufA[2 * i + 1] = p1;
    }
    __syncthreads();
    // Stable LSD radix sort on the slot bits (14..29): two 8-bit passes.
    // Warp w owns a contiguous chunk; inside it 32-element steps keep order.
    const int chunk = (m + 31) / 32;
    uint32_t* src = bufA;
    uint32_t* dst = bufB;
    for (int pass = 0; pass < 2; ++pass) {
        const int shift = 14 + 8 * pass;
        for (int i = tid; i < 32 * 257; i += blockDim.x) wcnt[i] = 0;
        __syncthreads();
        const int c0 = w * chunk, c1 = min(m, c0 + chunk);
        for (int base = c0; base < c1; base += 32) {
            const int idx = base + lane;
            const int d = idx < c1 ? (int)((src[idx] >> shift) & 0xFF) : 256;
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
            if (d < 256 && lane == __ffs(peers) - 1) wcnt[w * 257 + d] += __popc(peers);
            __syncwarp();
        }
        __syncthreads();
        if (tid < 256) {
            int acc = 0;
            for (int ww = 0; ww < 32; ++ww) {
                const int t = wcnt[ww * 257 + tid];
                wcnt[ww * 257 + tid] = acc;
                acc += t;
            }
            digit_off[tid] = acc;  // digit total for now
        }
        __syncthreads();
        if (tid == 0) {
            int acc = 0;
            for (int d = 0; d < 256; ++d) {
                const int t = digit_off[d];
                digit_off[d] = acc;
                acc += t;
            }
        }
        __syncthreads();
        for (int base = c0; base < c1; base += 32) {
            const int idx = base + lane;
            const int d = idx < c1 ? (int)((src[idx] >> shift) & 0xFF) : 256;
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
            const unsigned lt = (1u << lane) - 1u;
            int before = 0;
            if (d < 256) before = wcnt[w * 257 + d];
            __syncwarp();
            if (d < 256) dst[digit_off[d] + before + __popc(peers & lt)] = src[idx];
            if (d < 256 && lane == __ffs(peers) - 1) wcnt[w * 257 + d] = before + __popc(peers);
            __syncwarp();
        }
        __syncthreads();
        uint32_t* t = src;
        src = dst;
        dst = t;
    }
    // src holds the sorted events.  Times, deltas and slot bounds.
    for (int i = tid; i < m; i += blockDim.x) {
        const uint32_t pk = src[i];
        const uint32_t s = pk >> 14, e = pk & 0x3FFF;
        a.stime[i] = a.etime_raw[e];
        if (s < (uint32_t)kTableSlots) {
            if (i == 0 || (src[i - 1] >> 14) != s) a.sstart[s] = i;
            if (i == m - 1 || (src[i + 1] >> 14) != s) a.send[s] = i + 1;
        }
    }
    // Inclusive scan of the deltas in sorted order (global G in epre), then
    // per-slot prefix = G[i] - G[start] + val[start].
    const int per = (m + blockDim.x - 1) / blockDim.x;
    const int b0 = tid * per, b1 = min(m, b0 + per);
    long long run = 0;
    for (int i = b0; i < b1; ++i) run += a.eval_raw[src[i] & 0x3FFF];
    long long incl = run;
    for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (w == 0) {
        long long v = warp_tot[lane];
        long long vi = v;
        for (int o = 1; o < 32; o <<= 1) {
            const long long t = __shfl_up_sync(0xFFFFFFFFu, vi, o);
            if (lane >= o) vi += t;
        }
        warp_tot[lane] = vi - v;
    }
    __syncthreads();
    long long acc = warp_tot[w] + incl - run;
    for (int i = b0; i < b1; ++i) {
        acc += a.eval_raw[src[i] & 0x3FFF];
        a.gscan[i] = acc;
    }
    __syncthreads();
    for (int i = tid; i < m; i += blockDim.x) {
        const uint32_t s = src[i] >> 14;
        if (s >= (uint32_t)kTableSlots) continue;
        const int st = a.sstart[s];
        a.epre[i] = a.gscan[i] - (a.gscan[st] - a.eval_raw[src[st] & 0x3FFF]);
    }
}

constexpr int kExWarpsPerBlock = 4;

// Warp per window vertex (degree <= kWarpMaxDeg).
__global__ void __launch_bounds__(kExWarpsPerBlock * 32) k_ex_eval_warp(ExactState a) {
    extern __shared__ uint32_t ex_smem[];
    if (a.ctl->P >= a.ctl->n) return;
    const Round r = round_view(a);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t* tk = ex_smem + (size_t)w * 2 * kWarpHash;
    uint32_t* tv = tk + kWarpHash;
    const int64_t nw = (int64_t)gridDim.x * kExWarpsPerBlock;
    for (int64_t u = r.P + (int64_t)blockIdx.x * kExWarpsPerBlock + w; u < r.E; u += nw) {
        const int64_t rb = a.rp[u];
        const int deg = (int)(a.rp[u + 1] - rb);
        if (deg > kWarpMaxDeg) continue;
        bool act = a.vaff[u] != 0;
        if (!act) {
            bool any = false;
            for (int i = lane; i < deg && !any; i += 32) {
                const int32_t v = a.col[rb + i];
                any = (v >= r.P && v < u && prev_mover(a, r, v));
            }
            act = __any_sync(0xFFFFFFFFu, any);
        }
        const uint32_t d = a.vcom[u];
        if (!act) {
            if (lane == 0) record(a, r, u, 0, d, 0.0);
            continue;
        }
        const double ku = (double)deg;
        double best_d = 0.0;
        uint32_t best_c = kNone;
        if (deg <= 32) {
            uint32_t c = kNone;
            if (lane < deg) {
                const int32_t v = a.col[rb + lane];
                if (v != (int32_t)u) c = comm_at(a, r, v, u);
            }
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, c);
            const double kud = (double)__popc(__ballot_sync(0xFFFFFFFFu, c == d));
            if (c != kNone && c != d && lane == __ffs(peers) - 1) {
                const double sd = (double)sigma_at(a, d, (uint32_t)u);
                const double sc = (double)sigma_at(a, c, (uint32_t)u);
                const double dl = delta_q((double)__popc(peers), kud, ku, sc, sd, a.M, a.R);
                if (dl > 0.0) { best_d = dl; best_c = c; }
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
                    if (v != (int32_t)u) c = comm_at(a, r, v, u);
                }
                const unsigned peers = __match_any_sync(0xFFFFFFFFu, c);
                if (c != kNone && lane == __ffs(peers) - 1) table_add(tk, tv, mask, c, (uint32_t)__popc(peers));
            }
            __syncwarp();
            const double kud = (double)table_get(tk, tv, mask, d);
            const double sd = (double)sigma_at(a, d, (uint32_t)u);
            for (uint32_t i = lane; i < H; i += 32) {
                const uint32_t c = tk[i];
                if (c == kNone || c == d) continue;
                const double sc = (double)sigma_at(a, c, (uint32_t)u);
                const double dl = delta_q((double)tv[i], kud, ku, sc, sd, a.M, a.R);
                if (dl > 0.0 && better(dl, c, best_d, best_c)) { best_d = dl; best_c = c; }
            }
            __syncwarp();
        }
        warp_argmax(best_d, best_c);
        if (lane == 0) {
            if (best_d > 0.0 && best_c != kNone && best_c != d) record(a, r, u, 1, best_c, best_d);
            else record(a, r, u, 1, d, 0.0);
        }
    }
}

// Hub accumulation: one CTA per 4096-edge segment of a window hub.
__global__ void __launch_bounds__(256) k_ex_hub_accum(ExactState a) {
    if (a.ctl->P >= a.ctl->n) return;
    const Round r = round_view(a);
    const long long q0 = a.ctl->es0, q1 = a.ctl->es1;
    const int lane = threadIdx.x & 31;
    __shared__ int s_any;
    for (long long q = q0 + blockIdx.x; q < q1; q += gridDim.x) {
        const HubSeg sg = a.eseg[q];
        const uint32_t h = a.hub_v[sg.hub];
        const int64_t rb = a.rp[h], re = a.rp[h + 1];
        const int64_t e0 = rb + (int64_t)sg.part * kHubSeg, e1 = min(re, e0 + kHubSeg);
        uint32_t* tk = a.tkeys + a.hub_toff[sg.hub];
        uint32_t* tv = a.tvals + a.hub_toff[sg.hub];
        const uint32_t mask = a.hub_tcap[sg.hub] - 1;
        if (threadIdx.x == 0) s_any = 0;
        __syncthreads();
        bool any = false;
        for (int64_t b = e0; b < e1; b += blockDim.x) {
            uint32_t c = kNone;
            const int64_t e = b + threadIdx.x;
            if (e < e1) {
                const int32_t v = a.col[e];
                any = any || (v >= r.P && v < (int64_t)h && prev_mover(a, r, v));
                if (v != (int32_t)h) c = comm_at(a, r, v, h);
            }
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, c);
            if (c != kNone && lane == __ffs(peers) - 1) table_add(tk, tv, mask, c, (uint32_t)__popc(peers));
        }
        if (any) s_any = 1;
        __syncthreads();
        if (threadIdx.x == 0 && s_any) atomicOr(&a.hub_any[sg.hub], 1);
        __syncthreads();
    }
}

// Hub selection: one CTA per 4096-slot segment of a window hub's table; the
// last CTA of a hub reduces the partial maxima and records the decision.
__global__ void __launch_bounds__(256) k_ex_hub_select(ExactState a) {
    if (a.ctl->P >= a.ctl->n) return;
    const Round r = round_view(a);
    const long long q0 = a.ctl->ts0, q1 = a.ctl->ts1;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __shared__ double red_d[8];
    __shared__ uint32_t red_c[8];
    __shared__ int s_last;
    for (long long q = q0 + blockIdx.x; q < q1; q += gridDim.x) {
        const HubSeg sg = a.tseg[q];
        const int j = sg.hub;
        const uint32_t h = a.hub_v[j];
        const uint32_t* tk = a.tkeys + a.hub_toff[j];
        const uint32_t* tv = a.tvals + a.hub_toff[j];
        const uint32_t cap = a.hub_tcap[j];
        const uint32_t d = a.vcom[h];
        const double ku = (double)(a.rp[h + 1] - a.rp[h]);
        const double kud = (double)table_get(tk, tv, cap - 1, d);
        const double sd = (double)sigma_at(a, d, h);
        double best_d = 0.0;
        uint32_t best_c = kNone;
        const uint32_t s0 = (uint32_t)sg.part * kTabSeg, s1 = min(cap, s0 + kTabSeg);
        for (uint32_t i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
            const uint32_t c = tk[i];
            if (c == kNone || c == d) continue;
            const double sc = (double)sigma_at(a, c, h);
            const double dl = delta_q((double)tv[i], kud, ku, sc, sd, a.M, a.R);
            if (dl > 0.0 && better(dl, c, best_d, best_c)) { best_d = dl; best_c = c; }
        }
        warp_argmax(best_d, best_c);
        if (lane == 0) { red_d[w] = best_d; red_c[w] = best_c; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double bd = red_d[0];
            uint32_t bc = red_c[0];
            for (int k = 1; k < (int)(blockDim.x / 32); ++k)
                if (better(red_d[k], red_c[k], bd, bc)) { bd = red_d[k]; bc = red_c[k]; }
            a.part_d[q] = bd;
            a.part_c[q] = bc;
            __threadfence();
            s_last = atomicAdd(&a.hub_done[j], 1) == a.hub_tcount[j] - 1;
        }
        __syncthreads();
        if (s_last && threadIdx.x == 0) {
            __threadfence();
            double bd = 0.0;
            uint32_t bc = kNone;
            const int f = a.hub_tfirst[j];
            for (int k = 0; k < a.hub_tcount[j]; ++k) {
                const double pd = ((volatile double*)a.part_d)[f + k];
                const uint32_t pc = ((volatile uint32_t*)a.part_c)[f + k];
                if (better(pd, pc, bd, bc)) { bd = pd; bc = pc; }
            }
            const bool act = a.vaff[h] != 0 || ((volatile int32_t*)a.hub_any)[j] != 0;
            if (!act) record(a, r, h, 0, d, 0.0);
            else if (bd > 0.0 && bc != kNone && bc != d) record(a, r, h, 1, bc, bd);
            else record(a, r, h, 1, d, 0.0);
            a.hub_done[j] = 0;
            a.hub_any[j] = 0;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_ex_hub_clear(ExactState a) {
    if (a.ctl->P >= a.ctl->n) return;
    const long long q0 = a.ctl->ts0, q1 = a.ctl->ts1;
    for (long long q = q0 + blockIdx.x; q < q1; q += gridDim.x) {
        const HubSeg sg = a.tseg[q];
        uint32_t* tk = a.tkeys + a.hub_toff[sg.hub];
        uint32_t* tv = a.tvals + a.hub_toff[sg.hub];
        const uint32_t s0 = (uint32_t)sg.part * kTabSeg, s1 = min(a.hub_tcap[sg.hub], s0 + kTabSeg);
        for (uint32_t i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
            tk[i] = kNone;
            tv[i] = 0;
        }
    }
}

__device__ __forceinline__ long long commit_end(const ExactState& a) {
    const unsigned long long f = a.ctl->first_change;
    const long long E = a.ctl->E;
    return f == kNoChange ? E - 1 : min((long long)f, E - 1);
}

// Commit [P, x]: totals of movers, final deltas, processed flags cleared.
__global__ void k_ex_commit_a(ExactState a) {
    if (a.ctl->P >= a.ctl->n) return;
    const Round r = round_view(a);
    const long long x = commit_end(a);
    for (long long u = r.P + blockIdx.x * (long long)blockDim.x + threadIdx.x; u <= x;
         u += (long long)gridDim.x * blockDim.x) {
        double dl = 0.0;
        if (r.nact[u] == 1 && r.nbest[u] != a.vcom[u]) {
            const long long deg = (long long)(a.rp[u + 1] - a.rp[u]);
            atomicAdd(&a.ctot[a.vcom[u]], (unsigned long long)(-deg));
            atomicAdd(&a.ctot[r.nbest[u]], (unsigned long long)deg);
            dl = r.ndelta[u];
        }
        a.final_delta[u] = dl;
        a.vaff[u] = 0;
    }
}

// Affected flags from committed movers: every neighbour outside [P, x] and
// every neighbour in [P, x] processed before the mover.  Non-hub movers here,
// hub movers in k_ex_commit_hub.
__global__ void k_ex_commit_b(ExactState a) {
    if (a.ctl->P >= a.ctl->n) return;
    const Round r = round_view(a);
    const long long x = commit_end(a);
    const int lane = threadIdx.x & 31;
    const long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long w = r.P + wid; w <= x; w += nw) {
        if (!(r.nact[w] == 1 && r.nbest[w] != a.vcom[w])) continue;
        const int64_t rb = a.rp[w], re = a.rp[w + 1];
        if (re - rb > kWarpMaxDeg) continue;
        for (int64_t e = rb + lane; e < re; e += 32) {
            const int32_t v = a.col[e];
            if (v < r.P || v > x || v < w) a.vaff[v] = 1;
        }
    }
}

__global__ void __launch_bounds__(256) k_ex_commit_hub(ExactState a) {
    if (a.ctl->P >= a.ctl->n) return;
    const Round r = round_view(a);
    const long long x = commit_end(a);
    const long long q0 = a.ctl->es0;
    const long long q1 = lower_bound_u32(a.eseg_v, a.n_eseg, (uint32_t)(x + 1));
    for (long long q = q0 + blockIdx.x; q < q1; q += gridDim.x) {
        const HubSeg sg = a.eseg[q];
        const uint32_t h = a.hub_v[sg.hub];
        if (!(r.nact[h] == 1 && r.nbest[h] != a.vcom[h])) continue;
        const int64_t rb = a.rp[h], re = a.rp[h + 1];
        const int64_t e0 = rb + (int64_t)sg.part * kHubSeg, e1 = min(re, e0 + kHubSeg);
        for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
            const int32_t v = a.col[e];
            if (v < r.P || v > x || v < (int64_t)h) a.vaff[v] = 1;
        }
    }
}

__global__ void k_ex_commit_c(ExactState a) {
    if (a.ctl->P >= a.ctl->n) return;
    const Round r = round_view(a);
    const long long x = commit_end(a);
    for (long long u = r.P + blockIdx.x * (long long)blockDim.x + threadIdx.x; u <= x;
         u += (long long)gridDim.x * blockDim.x)
        if (r.nact[u] == 1) a.vcom[u] = r.nbest[u];
}

// Slide the window: the new decisions become D_prev; entering vertices are unknown.
__global__ void __launch_bounds__(1024) k_ex_advance(ExactState a) {
    const long long P = a.ctl->P, E = a.ctl->E, n = a.ctl->n, B = a.ctl->B;
    if (P >= n) return;
    const long long x = commit_end(a);
    const long long nP = x + 1, nE = min(n, nP + B);
    const int par = (int)(a.ctl->round & 1);
    uint8_t* next_prev_act = a.act[par ^ 1];
    for (long long u = E + threadIdx.x; u < nE; u += blockDim.x) next_prev_act[u] = kUnknown;
    __syncthreads();
    if (threadIdx.x == 0) {
        a.ctl->P = nP;
        a.ctl->E = nE;
        a.ctl->round = a.ctl->round + 1;
    }
}

__global__ void __launch_bounds__(1024) k_ex_init_iter(ExactState a) {
    const long long n = a.ctl->n, B = a.ctl->B;
    const long long E = min(n, B);
    for (long long u = threadIdx.x; u < E; u += blockDim.x) a.act[0][u] = kUnknown;
    __syncthreads();
    if (threadIdx.x == 0) {
        a.ctl->P = 0;
        a.ctl->E = E;
        a.ctl->round = 0;
    }
}

// Deterministic tree sum of the iteration's committed deltas (and count).
__global__ void k_sum_deltas(const double* __restrict__ d, int64_t n, double* __restrict__ partial,
                             unsigned long long* __restrict__ cnt) {
    double s = 0.0;
    unsigned long long c = 0;
    const int64_t per = (n + gridDim.x - 1) / gridDim.x;
    const int64_t b = blockIdx.x * per, e = min(n, b + per);
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        s += d[i];
        c += d[i] != 0.0;
    }
    __shared__ double sh[kT];
    __shared__ unsigned long long shc[kT];
    sh[threadIdx.x] = s;
    shc[threadIdx.x] = c;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            sh[threadIdx.x] += sh[threadIdx.x + o];
            shc[threadIdx.x] += shc[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = sh[0];
        atomicAdd(cnt, shc[0]);
    }
}

// Exact left-to-right sum in vertex order (only when the bound is inconclusive).
__global__ void k_sum_serial(const double* __restrict__ d, int64_t n, double* __restrict__ out) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double s = 0.0;
        for (int64_t i = 0; i < n; ++i) s += d[i];
        *out = s;
    }
}

__global__ void k_hub_degrees(const int64_t* __restrict__ rp, const uint32_t* __restrict__ hubs, int64_t nh,
                              int64_t* __restrict__ deg) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nh; j += (int64_t)gridDim.x * blockDim.x)
        deg[j] = rp[hubs[j] + 1] - rp[hubs[j]];
}

template <typename T>
T read_dev(const T* p, cudaStream_t s) {
    T h;
    GB_CUDA(cudaMemcpyAsync(&h, p, sizeof(T), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    return h;
}

template <typename T>
DevBuf<T> upload(const std::vector<T>& v, cudaStream_t s) {
    DevBuf<T> d(v.empty() ? 1 : v.size(), s);
    if (!v.empty()) GB_CUDA(cudaMemcpyAsync(d.get(), v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return d;
}

}  // namespace

int local_move_exact(const LocalMoveContext& ctx, double tolerance, int max_iterations, int64_t window,
                     cudaStream_t s, int64_t* launches, int64_t* rounds_out) {
    const int64_t n = ctx.g.n;
    const int64_t B = std::max<int64_t>(32, std::min<int64_t>(std::min<int64_t>(window, kWindowMax), n));

    // ---- hub segment tables (once per call) ----
    const int64_t nh = (int64_t)ctx.hubs_h.size();
    std::vector<int64_t> hdeg(nh);
    if (nh) {
        DevBuf<int64_t> dd(nh, s);
        k_hub_degrees<<<grid_for(nh, kT), kT, 0, s>>>(ctx.g.row_ptr, ctx.hubs, nh, dd);
        GB_LAUNCH_CHECK();
        GB_CUDA(cudaMemcpyAsync(hdeg.data(), dd.get(), nh * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaStreamSynchronize(s));
    }
    std::vector<int64_t> toff(nh);
    std::vector<uint32_t> tcap(nh);
    std::vector<int32_t> tfirst(nh), tcount(nh);
    std::vector<HubSeg> eseg, tseg;
    std::vector<uint32_t> eseg_v, tseg_v;
    int64_t pool = 0;
    for (int64_t j = 0; j < nh; ++j) {
        uint32_t cap = 64;
        while ((int64_t)cap < 2 * hdeg[j]) cap <<= 1;
        tcap[j] = cap;
        toff[j] = pool;
        pool += cap;
        const int ne = (int)ceil_div(hdeg[j], kHubSeg);
        for (int k = 0; k < ne; ++k) {
            eseg.push_back({(int32_t)j, k});
            eseg_v.push_back(ctx.hubs_h[j]);
        }
        const int nt = (int)ceil_div(cap, kTabSeg);
        tfirst[j] = (int32_t)tseg.size();
        tcount[j] = nt;
        for (int k = 0; k < nt; ++k) {
            tseg.push_back({(int32_t)j, k});
            tseg_v.push_back(ctx.hubs_h[j]);
        }
    }
    DevBuf<int64_t> d_toff = upload(toff, s);
    DevBuf<uint32_t> d_tcap = upload(tcap, s);
    DevBuf<int32_t> d_tfirst = upload(tfirst, s), d_tcount = upload(tcount, s);
    DevBuf<HubSeg> d_eseg = upload(eseg, s), d_tseg = upload(tseg, s);
    DevBuf<uint32_t> d_eseg_v = upload(eseg_v, s), d_tseg_v = upload(tseg_v, s);
    DevBuf<uint32_t> tkeys(pool > 0 ? pool : 1, s), tvals(pool > 0 ? pool : 1, s);
    GB_CUDA(cudaMemsetAsync(tkeys, 0xFF, (pool > 0 ? pool : 1) * sizeof(uint32_t), s));
    GB_CUDA(cudaMemsetAsync(tvals, 0, (pool > 0 ? pool : 1) * sizeof(uint32_t), s));
    DevBuf<int32_t> hub_any(nh > 0 ? nh : 1, s), hub_done(nh > 0 ? nh : 1, s);
    GB_CUDA(cudaMemsetAsync(hub_any, 0, (nh > 0 ? nh : 1) * sizeof(int32_t), s));
    GB_CUDA(cudaMemsetAsync(hub_done, 0, (nh > 0 ? nh : 1) * sizeof(int32_t), s));
    DevBuf<double> part_d(tseg.empty() ? 1 : tseg.size(), s);
    DevBuf<uint32_t> part_c(tseg.empty() ? 1 : tseg.size(), s);

    // ---- round state ----
    DevBuf<uint32_t> best0(n, s), best1(n, s);
    DevBuf<uint8_t> act0(n, s), act1(n, s);
    DevBuf<double> delta0(n, s), delta1(n, s), final_delta(n, s);
    DevBuf<uint32_t> hkey(kTableSlots, s), etime_raw(kEventsMax, s), stime(kEventsMax, s);
    DevBuf<int32_t> sstart(kTableSlots, s), send(kTableSlots, s);
    DevBuf<long long> eval_raw(kEventsMax, s), epre(kEventsMax, s), gscan(kEventsMax, s);
    DevBuf<Ctl> ctl(1, s);
    Ctl* hctl = nullptr;
    GB_CUDA(cudaMallocHost(&hctl, sizeof(Ctl)));
    *hctl = Ctl{};
    hctl->n = n;
    hctl->B = B;
    GB_CUDA(cudaMemcpyAsync(ctl.get(), hctl, sizeof(Ctl), cudaMemcpyHostToDevice, s));
    DevBuf<double> partial(1024, s), dsum(1, s);
    DevBuf<unsigned long long> nmov(1, s);

    ExactState a{};
    a.rp = ctx.g.row_ptr;
    a.col = ctx.g.col;
    a.vcom = ctx.vcom;
    a.ctot = ctx.ctot;
    a.vaff = ctx.vaff;
    a.ctl = ctl.get();
    a.best[0] = best0.get();
    a.best[1] = best1.get();
    a.act[0] = act0.get();
    a.act[1] = act1.get();
    a.delta[0] = delta0.get();
    a.delta[1] = delta1.get();
    a.final_delta = final_delta.get();
    a.hkey = hkey.get();
    a.sstart = sstart.get();
    a.send = send.get();
    a.etime_raw = etime_raw.get();
    a.eval_raw = eval_raw.get();
    a.stime = stime.get();
    a.epre = epre.get();
    a.gscan = gscan.get();
    a.hub_v = ctx.hubs;
    a.hub_toff = d_toff.get();
    a.hub_tcap = d_tcap.get();
    a.hub_tfirst = d_tfirst.get();
    a.hub_tcount = d_tcount.get();
    a.eseg = d_eseg.get();
    a.eseg_v = d_eseg_v.get();
    a.n_eseg = (long long)eseg.size();
    a.tseg = d_tseg.get();
    a.tseg_v = d_tseg_v.get();
    a.n_tseg = (long long)tseg.size();
    a.tkeys = tkeys.get();
    a.tvals = tvals.get();
    a.hub_any = hub_any.get();
    a.hub_done = hub_done.get();
    a.part_d = part_d.get();
    a.part_c = part_c.get();
    a.M = ctx.M;
    a.R = ctx.R;

    const int table_smem = (2 * kEventsMax + 32 * 257) * (int)sizeof(uint32_t);
    GB_CUDA(cudaFuncSetAttribute(k_ex_table, cudaFuncAttributeMaxDynamicSharedMemorySize, table_smem));
    const int eval_smem = kExWarpsPerBlock * 2 * kWarpHash * (int)sizeof(uint32_t);
    GB_CUDA(cudaFuncSetAttribute(k_ex_eval_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, eval_smem));
    const int eval_grid = (int)std::min<int64_t>(ceil_div(B, kExWarpsPerBlock), (int64_t)kNumSMs * 16);
    const int hub_grid = kNumSMs * 4;
    const int commit_grid = (int)std::max<int64_t>(1, ceil_div(B, kT));
    const int commit_b_grid = (int)std::max<int64_t>(1, ceil_div(B * 32, kT));
    const int kBatch = 8;

    int iterations = 0;
    int64_t rounds = 0, nl = 0;
    for (int it = 0; it < max_iterations; ++it) {
        k_ex_init_iter<<<1, 1024, 0, s>>>(a);
        GB_LAUNCH_CHECK();
        ++nl;
        while (true) {
            for (int b = 0; b < kBatch; ++b) {
                k_ex_table<<<1, kEvThreads, table_smem, s>>>(a);
                k_ex_eval_warp<<<eval_grid, kExWarpsPerBlock * 32, eval_smem, s>>>(a);
                if (nh) {
                    k_ex_hub_accum<<<hub_grid, 256, 0, s>>>(a);
                    k_ex_hub_select<<<hub_grid, 256, 0, s>>>(a);
                    k_ex_hub_clear<<<hub_grid, 256, 0, s>>>(a);
                }
                k_ex_commit_a<<<commit_grid, kT, 0, s>>>(a);
                k_ex_commit_b<<<commit_b_grid, kT, 0, s>>>(a);
                if (nh) k_ex_commit_hub<<<hub_grid, 256, 0, s>>>(a);
                k_ex_commit_c<<<commit_grid, kT, 0, s>>>(a);
                k_ex_advance<<<1, 1024, 0, s>>>(a);
                GB_LAUNCH_CHECK();
                nl += nh ? 10 : 6;
            }
            GB_CUDA(cudaMemcpyAsync(hctl, ctl.get(), sizeof(Ctl), cudaMemcpyDeviceToHost, s));
            GB_CUDA(cudaStreamSynchronize(s));
            if (hctl->P >= n) break;
        }
        rounds += hctl->round;
        ++iterations;
        // totalDelta <= tolerance, decided exactly.
        const int sb = 1024;
        GB_CUDA(cudaMemsetAsync(nmov, 0, sizeof(unsigned long long), s));
        k_sum_deltas<<<sb, kT, 0, s>>>(final_delta, n, partial, nmov);
        GB_LAUNCH_CHECK();
        std::vector<double> hp(sb);
        GB_CUDA(cudaMemcpyAsync(hp.data(), partial.get(), sb * sizeof(double), cudaMemcpyDeviceToHost, s));
        const unsigned long long movers = read_dev(nmov.get(), s);
        double total = 0.0;
        for (double v : hp) total += v;
        // All terms are >= 0: any summation order is within (k-1) u sum of the exact value.
        const double bound = (double)(movers + 1) * 2.220446049250313e-16 * total;
        bool stop;
        if (std::fabs(total - tolerance) > 2.0 * bound) {
            stop = total <= tolerance;
        } else {
            k_sum_serial<<<1, 1, 0, s>>>(final_delta, n, dsum);
            GB_LAUNCH_CHECK();
            stop = read_dev(dsum.get(), s) <= tolerance;
            ++nl;
        }
        nl += 2;
        if (stop) break;
    }
    cudaFreeHost(hctl);
    if (launches) *launches += nl;
    if (rounds_out) *rounds_out += rounds;
    return iterations;
}

}  // namespace gb
