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
#include <cstdlib>
#include <cmath>
#include <vector>

#include "gb_common.cuh"
#include "gb_leiden_internal.cuh"

namespace gb {

namespace {

constexpr int kT = 256;
constexpr uint8_t kUnknown = 2;
constexpr int kWindowMax = 65536;             // window vertices (events <= 2 x window)
constexpr int kEventsMax = 2 * kWindowMax;    // event index = 2 x window offset (+1)
constexpr int kSlotBits = 18;
constexpr int kTableSlots = 1 << kSlotBits;   // hash slots, >= 2 x events
constexpr int kCoarseBits = 9;                // event grouping: 512 coarse buckets of slots
constexpr int kCoarse = 1 << kCoarseBits;
constexpr int kFineBits = kSlotBits - kCoarseBits;
constexpr int kTbThreads = 1024;              // table insert / group: one window vertex per thread
constexpr int kTbMinChunk = 512;            // smallest insert chunk (CTA size) the table kernels accept
constexpr int kTbChunks = kWindowMax / kTbMinChunk;   // stride of the per-chunk histograms
constexpr int kTbFinishThreads = 512;         // table finish: one CTA per coarse bucket, a thread per fine digit
constexpr uint32_t kPadSlot = 0xFFFFFFFFu;
static_assert(kTableSlots >= 2 * kEventsMax, "hash load factor <= 1/2");
static_assert(kCoarse <= kTbMinChunk, "one coarse bucket per grouping thread");
// Slots with many events ("hot": a community that many window vertices join
// or leave) get a time-bucket index: bidx[b] = first event at time >= P + 16 b,
// so a lookup searches at most 16 events instead of the whole slot.
constexpr int kHotMin = 128;                  // events that make a slot hot
constexpr int kBucketV = 16;                  // window vertices per time bucket
constexpr int kHotStride = kWindowMax / kBucketV + 1;
constexpr int kHotMax = 2 * kEventsMax / kHotMin;
constexpr int kEndBits = 18;                  // SlotMeta.endh: end | (hot id + 1) << kEndBits
// Designated communities: the few communities with the most events (on RMAT
// the one most vertices join) leave the sorted table.  Each gets a dense row
// over the window (the signed degree of every window offset's move into or
// out of it) and the prefix of its 16-offset bucket sums, so a lookup is one
// prefix load plus one 64-byte read, and no bucket of the sorted table holds
// a giant community.  Chosen each round from the previous table's counts.
constexpr int kZMax = 8;                      // designated communities at most
constexpr int kZKeep = 64;                    // events a designated community needs to stay / be chosen
constexpr int kZCand = 128;                   // hot slots of the sorted table considered
static_assert(kEventsMax < (1 << kEndBits), "event positions fit the end field");
constexpr int kHubThreads2 = 256;             // threads of the hub kernels
constexpr int kBigMaxDeg = 2048;              // rows above kWarpMaxDeg up to this: one CTA each
constexpr int kBigThreads = 256;
constexpr int kBigSlots = 2 * kBigMaxDeg;     // shared table of a big row
constexpr int kHubSeg = 4 * kHubThreads2;     // edges per hub-accumulation CTA (4 per thread)
constexpr int kTabSeg = 4 * kHubThreads2;     // table slots per hub-selection CTA (4 per thread)
constexpr unsigned long long kNoChange = ~0ull;

struct Ctl {
    long long P, E, n, B;
    unsigned long long first_change;
    long long es0, es1;       // hub edge-segment range of the window
    long long ts0, ts1;       // hub table-segment range of the window
    long long ms0, ms1;       // mid-degree list range of the window
    long long bs0, bs1;       // big-row list range of the window
    long long c_bs0, c_bs1;   // big-row range of the last decided window
    long long round;
    long long evals;          // window vertices evaluated in this iteration
    long long cP, cX;         // committed range of the last decided window
    long long c_es0, c_es1;   // its hub edge-segment range
    long long c_ts0, c_ts1;   // its hub table-segment range
    long long max_rounds;     // bound on rounds per iteration (n + 1 always suffices)
    long long error;          // nonzero: the round loop stopped without finishing
    unsigned long long tag;   // generation of the event table (slots of older tags are empty)
    unsigned int nhot;        // hot slots of the current table
    unsigned long long tb_big; // largest coarse bucket: size << 32 | bucket (its CTA starts first)
    unsigned int tb_ticket;    // insert CTAs done this round (the last one scans the histogram)
    unsigned int nz;                 // designated communities of the current table
    unsigned int zc[kZMax];          // their ids
    unsigned int zcount[kZMax];      // events each received in the current table
};

struct __align__(16) SlotMeta {
    unsigned long long tkey;  // table generation << 32 | community id
    int32_t start;            // first sorted event of the slot
    uint32_t endh;            // one past its last event | (hot index + 1) << kEndBits
};

struct HubSeg {
    int32_t hub;      // index into the hub arrays
    int32_t part;     // segment number within the hub
};

struct ExactState {
    const int64_t* rp;
    const int32_t* col;
    const uint32_t* vcob;  // refinement bounds (localMovingPhase<true>), null otherwise
    uint32_t* vcom;
    unsigned long long* ctot;
    uint8_t* vaff;
    uint8_t* mv;          // committed vertex moved (read by the affected-flag kernels)
    Ctl* ctl;
    // decisions, double-buffered by round parity
    uint32_t* best[2];
    uint8_t* act[2];
    double* delta[2];
    double* final_delta;
    // event table
    SlotMeta* slots;      // kTableSlots: community key and its sorted-event range
    uint32_t* stime;      // event times (vertex ids), sorted by slot then time
    long long* epre;      // inclusive prefix of the signed degrees within the slot
    uint32_t* tb_s0;      // per window offset: slot of the departure event (kPadSlot: none)
    uint32_t* tb_s1;      // slot of the arrival event
    int32_t* wdeg;        // degree of a window mover, 0 otherwise
    int32_t* tb_hist;     // coarse bucket x insert chunk counts
    int32_t* tb_base;     // their exclusive prefix in bucket-major order: where a chunk's events of a bucket go
    int32_t* tb_bstart;   // coarse bucket starts (kCoarse + 1)
    unsigned long long* ev1;  // events grouped by coarse bucket: slot << 32 | event index
    unsigned long long* ev2;  // events sorted by slot
    int32_t* hot_bidx;        // kHotMax x kHotStride time-bucket starts of hot slots
    uint8_t* zof;             // per community: designated index + 1, 0 = in the sorted table
    int32_t* zcontrib;        // [2 parities][kZMax][kWindowMax] signed degree per window offset
    long long* zbsum;         // [2][kZMax][kHotStride] 16-offset bucket sums
    long long* zpre;          // [2][kZMax][kHotStride] exclusive prefix of the bucket sums
    unsigned long long* zcand;  // hot slots of the sorted table: events << 32 | community
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
    uint32_t* hub_kud;            // edges of the hub into its own community (accumulated)
    uint32_t* hub_occ;            // per hub (pool offsets): slots of its table in insertion order
    uint32_t* hub_occn;           // per hub: occupied slots
    int32_t* hub_clr;             // per hub: table segments cleared this round
    double* part_d;               // per table segment
    uint32_t* part_c;
    const uint32_t* mid_v;        // vertices with 32 < degree <= kWarpMaxDeg (ascending)
    long long n_mid;
    const uint32_t* big_v;        // vertices with kWarpMaxDeg < degree <= kBigMaxDeg (ascending)
    long long n_big;
    cudaGraphConditionalHandle cond;  // while-node condition (graph-driven rounds)
    int use_cond;
    double M, R;
    DqConst dq;
};

__device__ __forceinline__ uint32_t slot_hash(uint32_t c) {
    return (uint32_t)(((uint64_t)c * 0x9E3779B97F4A7C15ull) >> 40);
}

// Community totals at time u for K communities: the committed total plus the
// speculative events of c before u -- a 16-byte probe per hash step, then a
// binary search over the slot's time-sorted events.  The K probe chains and
// searches advance in lockstep so their loads are in flight together.
// Designated communities read their dense row instead (their probe, issued
// alongside, finds no slot: they are not in the table).
// valid[k] = false entries return 0.
template <int K>
__device__ __forceinline__ void sigma_at_k(const ExactState& a, unsigned long long tag, long long P, int par,
                                           const uint32_t (&c)[K], const bool (&valid)[K], uint32_t u,
                                           long long (&out)[K]) {
    uint32_t h[K], hot[K];
    int lo[K], l[K], r[K];
    bool pending[K];
    uint32_t zd[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        out[k] = valid[k] ? (long long)a.ctot[c[k]] : 0;
        zd[k] = valid[k] ? a.zof[c[k]] : 0u;
        h[k] = slot_hash(c[k]) & (kTableSlots - 1);
        pending[k] = valid[k];
        lo[k] = l[k] = r[k] = 0;
        hot[k] = 0;
    }
    bool any = true;
    while (any) {
        SlotMeta sm[K];
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (pending[k]) sm[k] = a.slots[h[k]];
        any = false;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (!pending[k]) continue;
            if (sm[k].tkey == (tag << 32 | c[k])) {
                lo[k] = l[k] = sm[k].start;
                r[k] = (int)(sm[k].endh & ((1u << kEndBits) - 1u));
                hot[k] = sm[k].endh >> kEndBits;
                if (hot[k] > (uint32_t)kHotMax) {   // never written by a finished table
                    a.ctl->error = 2;
                    hot[k] = 0;
                }
                pending[k] = false;
            } else if ((sm[k].tkey >> 32) != tag) {   // a slot of an older table: empty
                pending[k] = false;
            } else {
                h[k] = (h[k] + 1) & (kTableSlots - 1);
                any = true;
            }
        }
    }
    // Hot slots: narrow [l, r) to u's time bucket.
    {
        int bl[K], br[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (hot[k]) {
                const int32_t* bx = a.hot_bidx + (size_t)(hot[k] - 1) * kHotStride + (int)((u - P) / kBucketV);
                bl[k] = bx[0];
                br[k] = bx[1];
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (hot[k]) { l[k] = bl[k]; r[k] = br[k]; }
    }
    any = true;
    while (any) {
        uint32_t t[K];
        int mid[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            mid[k] = (l[k] + r[k]) >> 1;
            if (l[k] < r[k]) t[k] = a.stime[mid[k]];
        }
        any = false;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (l[k] < r[k]) {
                if (t[k] < u) l[k] = mid[k] + 1; else r[k] = mid[k];
                any = any || l[k] < r[k];
            }
        }
    }
#pragma unroll
    for (int k = 0; k < K; ++k)
        if (l[k] > lo[k]) out[k] += a.epre[l[k] - 1];
    // Designated communities: bucket prefix + the bucket's offsets before u.
    const int off = (int)((long long)u - P), bk = off >> 4, rem = off & 15;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if (!zd[k]) continue;
        const size_t row = (size_t)(par * kZMax + (int)zd[k] - 1);
        const int4* q = reinterpret_cast<const int4*>(a.zcontrib + row * kWindowMax + ((size_t)bk << 4));
        long long sum = a.zpre[row * kHotStride + bk];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const int4 v = q[m];
            if (4 * m + 0 < rem) sum += v.x;
            if (4 * m + 1 < rem) sum += v.y;
            if (4 * m + 2 < rem) sum += v.z;
            if (4 * m + 3 < rem) sum += v.w;
        }
        out[k] += sum;
    }
}

struct Round {
    long long P, E;
    unsigned long long tag;
    int par;              // parity of the round (decision buffers and dense rows)
    const uint32_t* pbest;
    const uint8_t* pact;
    uint32_t* nbest;
    uint8_t* nact;
    double* ndelta;
};

__device__ __forceinline__ Round round_view(const ExactState& a, const Ctl* c) {
    Round r;
    r.P = c->P;
    r.E = c->E;
    r.tag = c->tag;
    const int par = (int)(c->round & 1);
    r.par = par;
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

// Refinement (scanCommunities<true>, RG:1392-1437): only neighbours inside
// u's bound count; ub = vcob[u] (0 when not refining).
__device__ __forceinline__ uint32_t bound_of(const ExactState& a, uint32_t u) { return a.vcob ? a.vcob[u] : 0u; }
__device__ __forceinline__ bool counts(const ExactState& a, int32_t v, uint32_t u, uint32_t ub) {
    return v != (int32_t)u && (a.vcob == nullptr || a.vcob[v] == ub);
}
// localMovingPhase<true> (RG:1663-1666): a vertex whose community already
// holds more than itself stays.
__device__ __forceinline__ bool refine_stays(const ExactState& a, double sigma_d, double ku) {
    return a.vcob != nullptr && sigma_d > __dmul_rn(ku, 1.001);
}

__device__ __forceinline__ void record(const ExactState& a, const Round& r, int64_t u, uint8_t act, uint32_t best,
                                       double delta) {
    r.nact[u] = act;
    r.nbest[u] = best;
    r.ndelta[u] = delta;
    // Only the move itself is visible to later vertices: "inactive",
    // "evaluated, stays" and "not yet evaluated" (kUnknown) are the same
    // input to them, so only a different move is a change.
    const uint32_t cur = a.vcom[u];
    const bool moves = act == 1 && best != cur;
    const bool pmoves = r.pact[u] == 1 && r.pbest[u] != cur;
    if (moves != pmoves || (moves && best != r.pbest[u]))
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

// First index i in the ascending array a[0, n) with a[i] >= key, searched by
// one warp: 32 samples per step narrow the range 32-fold (4 steps for 2^20).
__device__ __forceinline__ long long warp_lower_bound_u32(const uint32_t* a, long long n, uint32_t key,
                                                         int lane) {
    long long lo = 0, hi = n;   // a[0, lo) < key; a[hi] >= key or hi == n
    while (hi - lo > 32) {
        const long long step = (hi - lo + 31) / 32;
        const long long p = lo + (long long)lane * step;
        const bool ge = p < hi ? a[p] >= key : true;
        const unsigned b = __ballot_sync(0xFFFFFFFFu, ge);   // lanes at or past hi vote true
        if (b == 0) {   // every sample < key: the bound lies past the last sample
            lo = lo + 31 * step + 1;
            continue;
        }
        const int f = __ffs(b) - 1;
        if (f == 0) return lo;
        const long long pf = lo + (long long)f * step;
        lo = lo + (long long)(f - 1) * step + 1;
        hi = min(hi, pf);
    }
    const long long p = lo + lane;
    const bool ge = p < hi ? a[p] >= key : true;
    const unsigned b = __ballot_sync(0xFFFFFFFFu, ge);
    return b ? lo + (__ffs(b) - 1) : hi;
}

// Window ranges of the hub segment lists, the mid-degree list and the
// big-row list for the window [P, E): eight searches on warps 0-7.
__device__ __forceinline__ void window_ranges(const ExactState& a, Ctl* c, long long P, long long E) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (w >= 8) return;
    const uint32_t* arr = w < 2 ? a.eseg_v : (w < 4 ? a.tseg_v : (w < 6 ? a.mid_v : a.big_v));
    const long long len = w < 2 ? a.n_eseg : (w < 4 ? a.n_tseg : (w < 6 ? a.n_mid : a.n_big));
    const long long pos = warp_lower_bound_u32(arr, len, (uint32_t)((w & 1) ? E : P), lane);
    if (lane == 0) {
        switch (w) {
            case 0: c->es0 = pos; break;
            case 1: c->es1 = pos; break;
            case 2: c->ts0 = pos; break;
            case 3: c->ts1 = pos; break;
            case 4: c->ms0 = pos; break;
            case 5: c->ms1 = pos; break;
            case 6: c->bs0 = pos; break;
            default: c->bs1 = pos; break;
        }
    }
}

// ---------------------------------------------------------------------------
// Event table.  Each D_prev mover w of the window contributes two events at
// time w: (old community, -deg w) and (new community, +deg w).  A lookup needs,
// per community, its events in time order with inclusive prefix sums.  Built
// in three kernels:
//   insert: one thread per window vertex; movers insert both communities into
//           the generation-tagged hash (no clearing between rounds) and count
//           their events per coarse bucket (high slot bits) per chunk;
//   group:  each chunk scatters its events, in time order, to its coarse
//           buckets' ranges (a stable counting pass);
//   finish: one CTA per coarse bucket sorts its events by the low slot bits
//           (stable, so time order holds inside a slot) and runs the
//           segmented prefix sum, filling each slot's event range.
// ---------------------------------------------------------------------------
struct SegSum {
    long long v;
    int cnt;    // elements since the last segment start
    int head;   // a segment starts inside this range
};

__device__ __forceinline__ SegSum seg_combine(SegSum a, SegSum b) {
    return b.head ? b : SegSum{a.v + b.v, a.cnt + b.cnt, a.head};
}

__device__ __forceinline__ SegSum seg_shfl_up(SegSum x, int o) {
    return SegSum{__shfl_up_sync(0xFFFFFFFFu, x.v, o), __shfl_up_sync(0xFFFFFFFFu, x.cnt, o),
                  __shfl_up_sync(0xFFFFFFFFu, x.head, o)};
}

// Slot of community c in the generation-`tag` table, inserting it if absent.
__device__ __forceinline__ uint32_t table_insert(SlotMeta* slots, unsigned long long tag, uint32_t c) {
    const unsigned long long want = tag << 32 | c;
    uint32_t h = slot_hash(c) & (kTableSlots - 1);
    while (true) {
        unsigned long long cur = ((volatile unsigned long long*)&slots[h].tkey)[0];
        if (cur == want) return h;
        if ((cur >> 32) != tag) {
            const unsigned long long prev = atomicCAS(&slots[h].tkey, cur, want);
            if (prev == cur || prev == want) return h;
            continue;   // another community took the slot: look at it again
        }
        h = (h + 1) & (kTableSlots - 1);
    }
}

// Window chunk `chunk` (blockDim.x consecutive window vertices).
__device__ __forceinline__ void tb_insert_chunk(const ExactState& a, const Ctl* c, int chunk) {
    __shared__ int32_t hist[kCoarse];
    const long long P = c->P, E = c->E;
    const Round r = round_view(a, c);
    const int tid = threadIdx.x;
    for (int b = tid; b < kCoarse; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    const int W = (int)(E - P);
    const int i = chunk * blockDim.x + tid;
    const int nz = (int)c->nz;
    uint32_t z0 = 0, z1 = 0;   // designated index + 1 of the departure / arrival community
    int dg = 0;
    if (i < W) {
        const int64_t wv = P + i;
        const uint8_t pa = r.pact[wv];
        const uint32_t pb = r.pbest[wv], vc = a.vcom[wv];
        const int64_t r0 = a.rp[wv], r1 = a.rp[wv + 1];
        uint32_t s0 = kPadSlot, s1 = kPadSlot;
        if (pa == 1 && pb != vc) {
            dg = (int)(r1 - r0);
            if (nz) {
                z0 = a.zof[vc];
                z1 = a.zof[pb];
            }
            if (!z0) {
                s0 = table_insert(a.slots, r.tag, vc);
                atomicAdd(&hist[s0 >> kFineBits], 1);
            }
            if (!z1) {
                s1 = table_insert(a.slots, r.tag, pb);
                atomicAdd(&hist[s1 >> kFineBits], 1);
            }
        }
        a.tb_s0[i] = s0;
        a.tb_s1[i] = s1;
        a.wdeg[i] = dg;
    }
    // Dense rows: every window offset writes its signed degree for each
    // designated community (zero when it does not move into or out of it), and
    // each 16-offset bucket (a half-warp) its sum; warp-aggregated event counts.
    for (int j = 0; j < nz; ++j) {
        const int v = (z1 == (uint32_t)j + 1 ? dg : 0) - (z0 == (uint32_t)j + 1 ? dg : 0);
        const size_t row = (size_t)(r.par * kZMax + j);
        if (i < W) a.zcontrib[row * kWindowMax + i] = v;
        long long sum = v;
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) sum += __shfl_xor_sync(0xFFFFFFFFu, sum, o);
        if ((i & 15) == 0 && i < W) a.zbsum[row * kHotStride + (i >> 4)] = sum;
        const int evs = __popc(__ballot_sync(0xFFFFFFFFu, z0 == (uint32_t)j + 1)) +
                        __popc(__ballot_sync(0xFFFFFFFFu, z1 == (uint32_t)j + 1));
        if ((tid & 31) == 0 && evs) atomicAdd(&a.ctl->zcount[j], (unsigned)evs);
    }
    __syncthreads();
    for (int b = tid; b < kCoarse; b += blockDim.x) a.tb_hist[b * kTbChunks + chunk] = hist[b];
    __syncthreads();   // hist is reused by the CTA's next chunk
}

// Run by the last insert CTA of a round (chunks = the insert grid): exclusive
// prefix of the (bucket, chunk) counts in bucket-major order -- the offset of
// each chunk's events inside the grouped array -- plus the bucket starts and
// the largest bucket.  Once per round instead of once per grouping CTA.  Warp
// w owns buckets [w * kPerWarp, (w + 1) * kPerWarp); lane l holds chunks l and
// l + 32 of each; all loads are issued before the scans.
constexpr int kScanPerWarp = kCoarse / (kTbThreads / 32);
static_assert(kCoarse % (kTbThreads / 32) == 0, "buckets split evenly over the insert CTA's warps");
static_assert(kWindowMax / kTbThreads <= 64, "two insert chunks per lane");

__device__ __forceinline__ void tb_scan_hist(const ExactState& a, int chunks) {
    __shared__ int32_t bstart[kCoarse];
    __shared__ int32_t wsum[32];
    __shared__ unsigned long long wbig[32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    int v0[kScanPerWarp], v1[kScanPerWarp];
#pragma unroll
    for (int k = 0; k < kScanPerWarp; ++k) {
        const int32_t* h = a.tb_hist + (size_t)(w * kScanPerWarp + k) * kTbChunks;
        v0[k] = lane < chunks ? h[lane] : 0;
        v1[k] = lane + 32 < chunks ? h[lane + 32] : 0;
    }
#pragma unroll
    for (int k = 0; k < kScanPerWarp; ++k) {
        int x0 = v0[k], x1 = v1[k];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y0 = __shfl_up_sync(0xFFFFFFFFu, x0, o), y1 = __shfl_up_sync(0xFFFFFFFFu, x1, o);
            if (lane >= o) { x0 += y0; x1 += y1; }
        }
        const int t0 = __shfl_sync(0xFFFFFFFFu, x0, 31), t1 = __shfl_sync(0xFFFFFFFFu, x1, 31);
        v0[k] = x0 - v0[k];          // exclusive, inside the bucket
        v1[k] = t0 + x1 - v1[k];
        if (lane == 0) bstart[w * kScanPerWarp + k] = t0 + t1;   // bucket total for now
    }
    __syncthreads();
    // Exclusive scan of the bucket totals (kCoarse <= threads) and the largest bucket.
    int tot = tid < kCoarse ? bstart[tid] : 0;
    int incl = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += y;
    }
    unsigned long long big = tot ? ((unsigned long long)tot << 32) | (unsigned long long)tid : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) big = max(big, __shfl_xor_sync(0xFFFFFFFFu, big, o));
    if (lane == 31) wsum[w] = incl;
    if (lane == 0) wbig[w] = big;
    __syncthreads();
    if (w == 0) {
        const int v = wsum[lane];
        int vi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xFFFFFFFFu, vi, o);
            if (lane >= o) vi += y;
        }
        wsum[lane] = vi - v;
        unsigned long long bb = wbig[lane];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) bb = max(bb, __shfl_xor_sync(0xFFFFFFFFu, bb, o));
        if (lane == 0) {
            a.ctl->tb_big = bb;
            a.ctl->tb_ticket = 0;
        }
    }
    __syncthreads();
    if (tid < kCoarse) {
        const int excl = wsum[w] + incl - tot;
        bstart[tid] = excl;
        a.tb_bstart[tid] = excl;
        if (tid == kCoarse - 1) a.tb_bstart[kCoarse] = excl + tot;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kScanPerWarp; ++k) {
        const int b = w * kScanPerWarp + k;
        int32_t* o = a.tb_base + (size_t)b * kTbChunks;
        if (lane < chunks) o[lane] = bstart[b] + v0[k];
        if (lane + 32 < chunks) o[lane + 32] = bstart[b] + v1[k];
    }
}

__global__ void __launch_bounds__(kTbThreads) k_tb_insert(ExactState a) {
    if (a.ctl->P >= a.ctl->n) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.ctl->first_change = kNoChange;
        a.ctl->nhot = 0;
    }
    tb_insert_chunk(a, a.ctl, blockIdx.x);
    // The last CTA to finish scans every CTA's histogram.
    __shared__ bool s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&a.ctl->tb_ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (s_last) {
        __threadfence();
        tb_scan_hist(a, (int)gridDim.x);
    }
}

// Stable scatter of each chunk's events to their coarse buckets.  Warp w of a
// chunk owns its 32 consecutive vertices, i.e. 64 consecutive events.
__device__ __forceinline__ void tb_group_chunk(const ExactState& a, const Ctl* c, int chunk, int chunks) {
    __shared__ int32_t base[kCoarse];
    extern __shared__ int32_t wcnt[];   // warps x kCoarse
    const long long P = c->P, E = c->E;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int nwarps = blockDim.x >> 5;
    const int W = (int)(E - P);
    (void)chunks;
    // This chunk's offset inside each bucket (scanned by the last insert CTA).
    for (int b = tid; b < kCoarse; b += blockDim.x) base[b] = a.tb_base[b * kTbChunks + chunk];
    for (int k = tid; k < nwarps * kCoarse; k += blockDim.x) wcnt[k] = 0;
    __syncthreads();
    // Count per warp, then turn counts into per-warp offsets (exclusive over warps).
    const int v0 = chunk * (int)blockDim.x + w * 32;   // first window offset of this warp
    uint32_t sl[2];
#pragma unroll
    for (int st = 0; st < 2; ++st) {
        const int e = 2 * v0 + st * 32 + lane;    // event index (time order)
        const int i = e >> 1;
        sl[st] = i < W ? ((e & 1) ? a.tb_s1[i] : a.tb_s0[i]) : kPadSlot;
        const int b = sl[st] == kPadSlot ? kCoarse : (int)(sl[st] >> kFineBits);
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, b);
        if (b < kCoarse && lane == __ffs(peers) - 1) wcnt[w * kCoarse + b] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    for (int b = tid; b < kCoarse; b += blockDim.x) {
        int acc = base[b];
        for (int ww = 0; ww < nwarps; ++ww) {
            const int t = wcnt[ww * kCoarse + b];
            wcnt[ww * kCoarse + b] = acc;
            acc += t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int st = 0; st < 2; ++st) {
        const int e = 2 * v0 + st * 32 + lane;
        const int b = sl[st] == kPadSlot ? kCoarse : (int)(sl[st] >> kFineBits);
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, b);
        int pos = 0;
        if (b < kCoarse) pos = wcnt[w * kCoarse + b] + __popc(peers & ((1u << lane) - 1u));
        __syncwarp();
        if (b < kCoarse) {
            a.ev1[pos] = (unsigned long long)sl[st] << 32 | (unsigned)e;
            if (lane == __ffs(peers) - 1) wcnt[w * kCoarse + b] += __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();   // shared arrays are reused by the CTA's next chunk
}

__global__ void __launch_bounds__(kTbThreads) k_tb_group(ExactState a) {
    if (a.ctl->P >= a.ctl->n) return;
    tb_group_chunk(a, a.ctl, blockIdx.x, gridDim.x);
}

// One CTA per coarse bucket: stable pass on the fine slot bits, then the
// segmented inclusive scan of signed degrees; writes times, prefixes and the
// slots' event ranges.
// Coarse bucket number `vb` (after swapping the largest bucket to 0); the
// CTA has at least kFine threads.
__device__ __forceinline__ void tb_finish_bucket(const ExactState& a, const Ctl* c, int vb) {
    constexpr int kFine = 1 << kFineBits;
    constexpr int kRow = kFine + 1;          // padded row of per-warp digit counts
    extern __shared__ int32_t wcnt[];   // warps x kRow per-warp digit counts (dynamic: > 48 KB)
    __shared__ int32_t digit[kFine];
    __shared__ long long warp_v[32];
    __shared__ int warp_h[32];
    const long long P = c->P;
    if (vb >= kCoarse) {
        // Designated community j = vb - kCoarse: exclusive prefix of its
        // bucket sums (one extra entry holds the total).
        const int j = vb - kCoarse;
        if (j >= (int)c->nz) return;
        const int nbk = (int)((c->E - P + kBucketV - 1) / kBucketV);
        const size_t row = ((size_t)(c->round & 1) * kZMax + j) * kHotStride;
        const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nwarps = blockDim.x >> 5;
        const int per = (nbk + blockDim.x - 1) / blockDim.x;
        const int b0 = min(nbk, tid * per), b1 = min(nbk, b0 + per);
        long long own = 0;
        for (int b = b0; b < b1; ++b) own += a.zbsum[row + b];
        long long inc = own;
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) warp_v[w] = inc;
        __syncthreads();
        if (w == 0) {
            const long long x = lane < nwarps ? warp_v[lane] : 0;
            long long xi = x;
            for (int o = 1; o < 32; o <<= 1) {
                const long long y = __shfl_up_sync(0xFFFFFFFFu, xi, o);
                if (lane >= o) xi += y;
            }
            if (lane < nwarps) warp_v[lane] = xi - x;
        }
        __syncthreads();
        long long run = warp_v[w] + inc - own;
        for (int b = b0; b < b1; ++b) {
            a.zpre[row + b] = run;
            run += a.zbsum[row + b];
        }
        if (tid == (int)blockDim.x - 1) a.zpre[row + nbk] = run;
        __syncthreads();
        return;
    }
    // The largest bucket (the one holding a community many window vertices
    // join) goes first (CTA 0 / virtual bucket 0).
    const int big = (int)(a.ctl->tb_big & 0xFFFFFFFFull);
    const int bucket = vb == 0 ? big : (vb == big ? 0 : vb);
    const int bs = a.tb_bstart[bucket], be = a.tb_bstart[bucket + 1];
    const int cnt = be - bs;
    if (cnt == 0) return;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int nwarps = blockDim.x >> 5;
    static_assert(kFine % 32 == 0 && kFine <= kTbMinChunk && kFine <= kTbFinishThreads,
                  "digit scan layout: one thread per fine digit");
    for (int k = tid; k < nwarps * kRow; k += blockDim.x) wcnt[k] = 0;
    __syncthreads();
    // Stable pass on the fine slot bits: warp w owns a contiguous range; the
    // next 32 keys are loaded while the current ones are ranked.
    const int chunk = (cnt + nwarps - 1) / nwarps;
    const int c0 = bs + min(cnt, w * chunk), c1 = bs + min(cnt, (w + 1) * chunk);
    {
        unsigned long long nxt = c0 + lane < c1 ? a.ev1[c0 + lane] : 0ull;
        for (int base = c0; base < c1; base += 32) {
            const int idx = base + lane;
            const unsigned long long key = nxt;
            if (base + 32 + lane < c1) nxt = a.ev1[base + 32 + lane];
            const int d = idx < c1 ? (int)((key >> 32) & (kFine - 1)) : kFine;
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
            if (d < kFine && lane == __ffs(peers) - 1) wcnt[w * kRow + d] += __popc(peers);
            __syncwarp();
        }
    }
    __syncthreads();
    if (tid < kFine) {
        int acc = 0;
        for (int ww = 0; ww < nwarps; ++ww) {
            const int t = wcnt[ww * kRow + tid];
            wcnt[ww * kRow + tid] = acc;
            acc += t;
        }
        digit[tid] = acc;
    }
    __syncthreads();
    if (w == 0) {
        constexpr int kPer = kFine / 32;
        int v[kPer], t = 0;
#pragma unroll
        for (int k = 0; k < kPer; ++k) { v[k] = digit[lane * kPer + k]; t += v[k]; }
        int incl = t;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += y;
        }
        int run = incl - t;
#pragma unroll
        for (int k = 0; k < kPer; ++k) { digit[lane * kPer + k] = run; run += v[k]; }
    }
    __syncthreads();
    {
        unsigned long long nxt = c0 + lane < c1 ? a.ev1[c0 + lane] : 0ull;
        for (int base = c0; base < c1; base += 32) {
            const int idx = base + lane;
            const unsigned long long key = nxt;
            if (base + 32 + lane < c1) nxt = a.ev1[base + 32 + lane];
            const int d = idx < c1 ? (int)((key >> 32) & (kFine - 1)) : kFine;
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
            int before = 0;
            if (d < kFine) before = wcnt[w * kRow + d];
            __syncwarp();
            if (d < kFine) a.ev2[bs + digit[d] + before + __popc(peers & ((1u << lane) - 1u))] = key;
            if (d < kFine && lane == __ffs(peers) - 1) wcnt[w * kRow + d] = before + __popc(peers);
            __syncwarp();
        }
    }
    __syncthreads();
    // Segmented inclusive scan over ev2[bs, be), each thread a contiguous
    // range read eight events at a time (keys, then degrees, in flight
    // together).  The tail of each slot knows the slot's length from the scan
    // and marks it hot.
    __shared__ int s_cnt_w[32];
    const int per = (cnt + blockDim.x - 1) / blockDim.x;
    const int b0 = bs + min(cnt, tid * per), b1 = bs + min(cnt, tid * per + per);
    SegSum own{0, 0, 0};
    {
        uint32_t psl = b0 > bs ? (uint32_t)(a.ev2[b0 - 1] >> 32) : kPadSlot;
        for (int k0 = b0; k0 < b1; k0 += 8) {
            unsigned long long key[8];
            int32_t dg[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) key[j] = k0 + j < b1 ? a.ev2[k0 + j] : 0ull;
#pragma unroll
            for (int j = 0; j < 8; ++j) dg[j] = k0 + j < b1 ? a.wdeg[(uint32_t)key[j] >> 1] : 0;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (k0 + j >= b1) break;
                const uint32_t sl = (uint32_t)(key[j] >> 32), e = (uint32_t)key[j];
                const long long v = (e & 1) ? dg[j] : -(long long)dg[j];
                own = seg_combine(own, SegSum{v, 1, sl != psl});
                psl = sl;
            }
        }
    }
    SegSum inc = own;
    for (int o = 1; o < 32; o <<= 1) {
        const SegSum y = seg_shfl_up(inc, o);
        if (lane >= o) inc = seg_combine(y, inc);
    }
    if (lane == 31) { warp_v[w] = inc.v; s_cnt_w[w] = inc.cnt; warp_h[w] = inc.head; }
    __syncthreads();
    if (w == 0) {
        const SegSum x = lane < nwarps ? SegSum{warp_v[lane], s_cnt_w[lane], warp_h[lane]} : SegSum{0, 0, 0};
        SegSum xi = x;
        for (int o = 1; o < 32; o <<= 1) {
            const SegSum y = seg_shfl_up(xi, o);
            if (lane >= o) xi = seg_combine(y, xi);
        }
        SegSum ex = seg_shfl_up(xi, 1);
        if (lane == 0) ex = SegSum{0, 0, 0};
        if (lane < nwarps) { warp_v[lane] = ex.v; s_cnt_w[lane] = ex.cnt; warp_h[lane] = ex.head; }
    }
    __syncthreads();
    SegSum ex_thread = seg_shfl_up(inc, 1);
    if (lane == 0) ex_thread = SegSum{0, 0, 0};
    const SegSum carry = seg_combine(SegSum{warp_v[w], s_cnt_w[w], warp_h[w]}, ex_thread);
    {
        long long run = carry.v;
        int runc = carry.cnt;
        uint32_t psl = b0 > bs ? (uint32_t)(a.ev2[b0 - 1] >> 32) : kPadSlot;
        for (int k0 = b0; k0 < b1; k0 += 8) {
            unsigned long long key[9];
            int32_t dg[8];
#pragma unroll
            for (int j = 0; j < 9; ++j) key[j] = k0 + j < be ? a.ev2[k0 + j] : ~0ull;   // one past for the tail test
#pragma unroll
            for (int j = 0; j < 8; ++j) dg[j] = k0 + j < b1 ? a.wdeg[(uint32_t)key[j] >> 1] : 0;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int k = k0 + j;
                if (k >= b1) break;
                const uint32_t sl = (uint32_t)(key[j] >> 32), e = (uint32_t)key[j];
                const long long v = (e & 1) ? dg[j] : -(long long)dg[j];
                const bool head = sl != psl;
                run = head ? v : run + v;
                runc = head ? 1 : runc + 1;
                psl = sl;
                a.stime[k] = (uint32_t)(P + (e >> 1));
                a.epre[k] = run;
                if (head) a.slots[sl].start = k;
                if (k == be - 1 || (uint32_t)(key[j + 1] >> 32) != sl) {
                    uint32_t endh = (uint32_t)(k + 1);
                    if (runc >= kHotMin) {
                        const unsigned id = atomicAdd(&a.ctl->nhot, 1u);
                        if (id < (unsigned)kHotMax) endh |= (id + 1) << kEndBits;
                        if (id < (unsigned)kZCand)
                            a.zcand[id] = (unsigned long long)runc << 32 | (uint32_t)a.slots[sl].tkey;
                    }
                    a.slots[sl].endh = endh;
                }
            }
        }
    }
    __syncthreads();
    // Hot slots: their time-bucket starts (bidx[b] = first event at a time
    // >= P + kBucketV * b).
    const int nb = (int)((c->E - P + kBucketV - 1) / kBucketV);
    for (int k0 = b0; k0 < b1; k0 += 8) {
        unsigned long long key[8];
        uint32_t eh[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) key[j] = k0 + j < b1 ? a.ev2[k0 + j] : 0ull;
#pragma unroll
        for (int j = 0; j < 8; ++j) eh[j] = k0 + j < b1 ? a.slots[(uint32_t)(key[j] >> 32)].endh : 0u;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int k = k0 + j;
            const uint32_t hid = eh[j] >> kEndBits;
            if (k >= b1 || !hid) continue;
            if (hid > (uint32_t)kHotMax) {   // never written by a finished table
                a.ctl->error = 2;
                continue;
            }
            const uint32_t sl = (uint32_t)(key[j] >> 32), e = (uint32_t)key[j];
            const int end = (int)(eh[j] & ((1u << kEndBits) - 1u));
            int32_t* bx = a.hot_bidx + (size_t)(hid - 1) * kHotStride;
            const int bk = (int)(e >> 1) / kBucketV;
            const int bprev = k == a.slots[sl].start ? -1 : (int)((uint32_t)a.ev2[k - 1] >> 1) / kBucketV;
            for (int b = bprev + 1; b <= bk; ++b) bx[b] = k;
            if (k == end - 1)
                for (int b = bk + 1; b <= nb; ++b) bx[b] = end;
        }
    }
    __syncthreads();   // shared arrays are reused by the CTA's next bucket
}

// Grid: kCoarse buckets + kZMax designated-community prefixes.
__global__ void __launch_bounds__(kTbFinishThreads) k_tb_finish(ExactState a) {
    if (a.ctl->P >= a.ctl->n) return;
    tb_finish_bucket(a, a.ctl, blockIdx.x);
}

constexpr int kMidWarpsPerBlock = 4;
constexpr int kSmallWarpsPerBlock = 8;
constexpr int kSmallMaxDeg = 32;

// One window vertex by one warp.  Small rows (deg <= 32) hold one neighbour
// per lane and rank communities with __match_any_sync; mid rows
// (32 < deg <= kWarpMaxDeg) accumulate into the warp's shared-memory table.
template <bool kMid>
__device__ __forceinline__ void eval_vertex(const ExactState& a, const Round& r, int64_t u, int lane, uint32_t* tk,
                                            uint32_t* tv) {
    const int64_t rb = a.rp[u];
    const int deg = (int)(a.rp[u + 1] - rb);
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
        return;
    }
    const double ku = (double)deg;
    const uint32_t ub = bound_of(a, (uint32_t)u);
    double best_d = 0.0;
    uint32_t best_c = kNone;
    if (!kMid) {
        if (a.vcob) {
            long long sg1 = 0;
            if (lane == 0) {
                const uint32_t cc[1] = {d};
                const bool vv[1] = {true};
                long long o[1];
                sigma_at_k<1>(a, r.tag, r.P, r.par, cc, vv, (uint32_t)u, o);
                sg1 = o[0];
            }
            sg1 = __shfl_sync(0xFFFFFFFFu, sg1, 0);
            if (refine_stays(a, (double)sg1, ku)) {
                if (lane == 0) record(a, r, u, 1, d, 0.0);
                return;
            }
        }
        uint32_t c = kNone;
        if (lane < deg) {
            const int32_t v = a.col[rb + lane];
            if (counts(a, v, (uint32_t)u, ub)) c = comm_at(a, r, v, u);
        }
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, c);
        const int kud = __popc(__ballot_sync(0xFFFFFFFFu, c == d));
        if (c != kNone && c != d && lane == __ffs(peers) - 1) {
            const uint32_t cc[2] = {c, d};
            const bool vv[2] = {true, true};
            long long sg[2];
            sigma_at_k<2>(a, r.tag, r.P, r.par, cc, vv, (uint32_t)u, sg);
            const double dl = delta_qi(a.dq, __popc(peers), kud, deg, sg[0], sg[1]);
            if (dpos(dl)) { best_d = dl; best_c = c; }
        }
    } else {
        uint32_t H = 64;
        while (H < 2u * (uint32_t)deg) H <<= 1;
        const uint32_t mask = H - 1;
        for (uint32_t i = lane; i < H; i += 32) { tk[i] = kNone; tv[i] = 0; }
        __syncwarp();
        // Neighbour communities, four 32-edge batches in flight per step.
        for (int base = 0; base < deg; base += 128) {
            uint32_t c[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int e = base + 32 * k + lane;
                c[k] = kNone;
                if (e < deg) {
                    const int32_t v = a.col[rb + e];
                    if (counts(a, v, (uint32_t)u, ub)) c[k] = comm_at(a, r, v, u);
                }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const unsigned peers = __match_any_sync(0xFFFFFFFFu, c[k]);
                if (c[k] != kNone && lane == __ffs(peers) - 1)
                    table_add(tk, tv, mask, c[k], (uint32_t)__popc(peers));
            }
        }
        __syncwarp();
        const uint32_t kud = table_get(tk, tv, mask, d);
        // Compact the candidate communities (c != d) to the front of the
        // table, so the selection runs ceil(candidates / 32) lookup rounds.
        uint32_t cnt = 0;
        for (uint32_t i0 = 0; i0 < H; i0 += 32) {
            const uint32_t c = tk[i0 + lane], v = tv[i0 + lane];
            const bool occ = c != kNone && c != d;
            const unsigned bal = __ballot_sync(0xFFFFFFFFu, occ);
            __syncwarp();
            if (occ) {
                const uint32_t pos = cnt + __popc(bal & ((1u << lane) - 1u));
                tk[pos] = c;
                tv[pos] = v;
            }
            cnt += __popc(bal);
            __syncwarp();
        }
        // One candidate per lane per step, its lookup interleaved with d's in
        // the first step (wider interleaving costs registers, and occupancy
        // matters more here: 64 registers, 28 warps per SM).
        long long sd = 0;
        for (uint32_t i0 = 0;; i0 += 32) {
            const uint32_t i = i0 + lane;
            const uint32_t cc[2] = {i < cnt ? tk[i] : kNone, d};
            const bool vv[2] = {i < cnt, i0 == 0};
            long long sg[2];
            sigma_at_k<2>(a, r.tag, r.P, r.par, cc, vv, (uint32_t)u, sg);
            if (i0 == 0) sd = sg[1];
            if (vv[0]) {
                const double dl = delta_qi(a.dq, tv[i], kud, deg, sg[0], sd);
                if (dpos(dl) && better_pos(dl, cc[0], best_d, best_c)) { best_d = dl; best_c = cc[0]; }
            }
            if (i0 + 32 >= cnt) break;
        }
        __syncwarp();
        if (refine_stays(a, (double)sd, ku)) best_c = kNone;   // every lane holds the same sd
    }
    warp_argmax_pos(best_d, best_c);
    if (lane == 0) {
        if (best_d > 0.0 && best_c != kNone && best_c != d) record(a, r, u, 1, best_c, best_d);
        else record(a, r, u, 1, d, 0.0);
    }
}

// Small rows, no shared memory.  A warp takes four consecutive window
// vertices: rows of degree <= 8 are evaluated together by four 8-lane groups
// (one neighbour per lane), rows of degree 9..32 then one at a time by the
// whole warp.
constexpr int kTinyDeg = 8;

__device__ __forceinline__ void eval_small_body(const ExactState& a, const Ctl* c) {
    const Round r = round_view(a, c);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int g = lane >> 3, j = lane & 7;
    const unsigned gmask = 0xFFu << (g * 8);
    const int wpb = (int)(blockDim.x >> 5);
    const int64_t nw = (int64_t)gridDim.x * wpb;
    for (int64_t u0 = r.P + 4 * ((int64_t)blockIdx.x * wpb + w); u0 < r.E; u0 += 4 * nw) {
        const int64_t u = u0 + g;
        const bool inwin = u < r.E;
        int64_t rb = 0;
        int deg = 0;
        if (inwin) {
            rb = a.rp[u];
            deg = (int)(a.rp[u + 1] - rb);
        }
        const bool tiny = inwin && deg <= kTinyDeg;
        // One load round for the row, its vertex state and its neighbours' states.
        int32_t v = -1;
        uint32_t d = kNone;
        bool aff = false;
        uint32_t ub = 0;
        if (tiny) {
            if (j < deg) v = a.col[rb + j];
            d = a.vcom[u];
            aff = a.vaff[u] != 0;
            ub = bound_of(a, (uint32_t)u);
        }
        bool pm = false;
        uint32_t cv = kNone;
        if (v >= 0) {
            const uint32_t vc = a.vcom[v];
            cv = vc;
            if (v >= r.P && v < u) {
                pm = r.pact[v] == 1 && r.pbest[v] != vc;
                if (pm) cv = r.pbest[v];
            }
            if (!counts(a, v, (uint32_t)u, ub)) cv = kNone;   // self loops (and, refining, other bounds)
        }
        // Refinement: the group's vertex stays when its community already holds more.
        bool stays = false;
        if (a.vcob) {
            long long sg1 = 0;
            if (tiny && j == 0) {
                const uint32_t cc[1] = {d};
                const bool vv[1] = {true};
                long long o[1];
                sigma_at_k<1>(a, r.tag, r.P, r.par, cc, vv, (uint32_t)u, o);
                sg1 = o[0];
            }
            sg1 = __shfl_sync(0xFFFFFFFFu, sg1, lane & ~7);
            stays = tiny && refine_stays(a, (double)sg1, (double)deg);
        }
        const unsigned pmb = __ballot_sync(0xFFFFFFFFu, pm);
        const bool act = tiny && (aff || (pmb & gmask) != 0);
        const uint32_t c = act ? cv : kNone;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, ((unsigned long long)g << 32) | c);
        const unsigned eqd = __ballot_sync(0xFFFFFFFFu, act && c != kNone && c == d) & gmask;
        double best_d = 0.0;
        uint32_t best_c = kNone;
        if (act && c != kNone && c != d && lane == __ffs(peers) - 1) {
            const uint32_t cc[2] = {c, d};
            const bool vv[2] = {true, true};
            long long sg[2];
            sigma_at_k<2>(a, r.tag, r.P, r.par, cc, vv, (uint32_t)u, sg);
            const double dl = delta_qi(a.dq, __popc(peers), __popc(eqd), deg, sg[0], sg[1]);
            if (dpos(dl)) { best_d = dl; best_c = c; }
        }
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) {   // argmax inside each 8-lane group
            const double od = __shfl_xor_sync(0xFFFFFFFFu, best_d, o);
            const uint32_t oc = __shfl_xor_sync(0xFFFFFFFFu, best_c, o);
            if (better_pos(od, oc, best_d, best_c)) { best_d = od; best_c = oc; }
        }
        if (tiny && j == 0) {
            if (!act) record(a, r, u, 0, d, 0.0);
            else if (!stays && best_d > 0.0 && best_c != kNone && best_c != d) record(a, r, u, 1, best_c, best_d);
            else record(a, r, u, 1, d, 0.0);
        }
        // Rows of degree 9..32: the whole warp, one row at a time.
#pragma unroll 1
        for (int k = 0; k < 4; ++k) {
            const int dk = __shfl_sync(0xFFFFFFFFu, deg, k * 8);
            const int ik = __shfl_sync(0xFFFFFFFFu, (int)inwin, k * 8);
            if (ik && dk > kTinyDeg && dk <= kSmallMaxDeg) eval_vertex<false>(a, r, u0 + k, lane, nullptr, nullptr);
        }
    }
}

// Four CTAs per SM (registers capped at 64; a few bytes spill): measured
// faster than three CTAs at 68 registers.
__global__ void __launch_bounds__(kSmallWarpsPerBlock * 32, 4) k_ex_eval_small(ExactState a) {
    if (a.ctl->P >= a.ctl->n) return;
    eval_small_body(a, a.ctl);
}

// Big rows (kWarpMaxDeg < degree <= kBigMaxDeg): one CTA per row, table in
// shared memory, candidates compacted, one candidate per thread per step (its
// lookup interleaved with d's in the first step; wider interleaving spilled
// under the register cap).  Three CTAs per SM (registers capped near 80).
__device__ __forceinline__ void eval_big_body(const ExactState& a, const Ctl* c) {
    extern __shared__ uint32_t big_smem[];
    uint32_t* tk = big_smem;                      // kBigSlots keys
    uint32_t* tv = tk + kBigSlots;                // kBigSlots counts
    uint32_t* cand_c = tv + kBigSlots;            // kBigMaxDeg compacted candidates
    uint32_t* cand_w = cand_c + kBigMaxDeg;
    __shared__ int s_any;
    __shared__ uint32_t s_cnt;
    __shared__ double red_d[32];
    __shared__ uint32_t red_c[32];
    const Round r = round_view(a, c);
    const long long b0 = c->bs0, b1 = c->bs1;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    for (long long bi = b0 + blockIdx.x; bi < b1; bi += gridDim.x) {
        const uint32_t u = a.big_v[bi];
        const int64_t rb = a.rp[u], re = a.rp[u + 1];
        const int deg = (int)(re - rb);
        const uint32_t d = a.vcom[u];
        const uint32_t ub = bound_of(a, u);
        uint32_t H = 64;
        while (H < 2u * (uint32_t)deg) H <<= 1;
        const uint32_t mask = H - 1;
        for (uint32_t i = tid; i < H; i += blockDim.x) { tk[i] = kNone; tv[i] = 0; }
        if (tid == 0) {
            s_any = a.vaff[u] != 0;
            s_cnt = 0;
        }
        __syncthreads();
        bool any = false;
        for (int64_t base = rb; base < re; base += 4 * (int64_t)blockDim.x) {
            uint32_t c[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int64_t e = base + k * (int64_t)blockDim.x + tid;
                c[k] = kNone;
                if (e < re) {
                    const int32_t v = a.col[e];
                    any = any || (v >= r.P && v < (int64_t)u && prev_mover(a, r, v));
                    if (counts(a, v, u, ub)) c[k] = comm_at(a, r, v, u);
                }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const unsigned peers = __match_any_sync(0xFFFFFFFFu, c[k]);
                if (c[k] != kNone && lane == __ffs(peers) - 1) table_add(tk, tv, mask, c[k], (uint32_t)__popc(peers));
            }
        }
        if (any) s_any = 1;
        __syncthreads();
        if (!s_any) {
            if (tid == 0) record(a, r, u, 0, d, 0.0);
            __syncthreads();
            continue;
        }
        const double ku = (double)deg;
        const uint32_t kud = table_get(tk, tv, mask, d);
        // Compact the candidates (c != d); their order does not matter, the
        // selection is a total order.
        for (uint32_t i0 = 0; i0 < H; i0 += blockDim.x) {
            const uint32_t i = i0 + tid;
            const uint32_t c = i < H ? tk[i] : kNone;
            const bool occ = c != kNone && c != d;
            const unsigned bal = __ballot_sync(0xFFFFFFFFu, occ);
            uint32_t base = 0;
            if (lane == 0 && bal) base = atomicAdd(&s_cnt, (uint32_t)__popc(bal));
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (occ) {
                const uint32_t pos = base + __popc(bal & ((1u << lane) - 1u));
                cand_c[pos] = c;
                cand_w[pos] = tv[i];
            }
        }
        __syncthreads();
        const uint32_t cnt = s_cnt;
        double best_d = 0.0;
        uint32_t best_c = kNone;
        long long sd = 0;
        for (uint32_t i0 = 0;; i0 += blockDim.x) {
            const uint32_t i = i0 + tid;
            const uint32_t cc[2] = {i < cnt ? cand_c[i] : kNone, d};
            const bool vv[2] = {i < cnt, i0 == 0};
            long long sg[2];
            sigma_at_k<2>(a, r.tag, r.P, r.par, cc, vv, u, sg);
            if (i0 == 0) sd = sg[1];
            if (vv[0]) {
                const double dl = delta_qi(a.dq, cand_w[i], kud, deg, sg[0], sd);
                if (dpos(dl) && better_pos(dl, cc[0], best_d, best_c)) { best_d = dl; best_c = cc[0]; }
            }
            if (i0 + blockDim.x >= cnt) break;
        }
        warp_argmax_pos(best_d, best_c);
        if (lane == 0) { red_d[w] = best_d; red_c[w] = best_c; }
        __syncthreads();
        if (tid == 0) {
            double bd = red_d[0];
            uint32_t bc = red_c[0];
            for (int k = 1; k < (int)(blockDim.x / 32); ++k)
                if (better_pos(red_d[k], red_c[k], bd, bc)) { bd = red_d[k]; bc = red_c[k]; }
            if (!refine_stays(a, (double)sd, ku) && bd > 0.0 && bc != kNone && bc != d) record(a, r, u, 1, bc, bd);
            else record(a, r, u, 1, d, 0.0);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kBigThreads, 3) k_ex_eval_big(ExactState a) {
    if (a.ctl->P >= a.ctl->n) return;
    eval_big_body(a, a.ctl);
}

// Mid rows of the window (from the ascending list of mid-degree vertices).
__device__ __forceinline__ void eval_mid_body(const ExactState& a, const Ctl* c) {
    extern __shared__ uint32_t ex_smem[];
    const Round r = round_view(a, c);
    const long long m0 = c->ms0, m1 = c->ms1;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int wpb = (int)(blockDim.x >> 5);
    uint32_t* tk = ex_smem + (size_t)w * 2 * kWarpHash;
    uint32_t* tv = tk + kWarpHash;
    const long long nw = (long long)gridDim.x * wpb;
    for (long long i = m0 + (long long)blockIdx.x * wpb + w; i < m1; i += nw)
        eval_vertex<true>(a, r, a.mid_v[i], lane, tk, tv);
}

__global__ void __launch_bounds__(kMidWarpsPerBlock * 32) k_ex_eval_mid(ExactState a) {
    if (a.ctl->P >= a.ctl->n) return;
    eval_mid_body(a, a.ctl);
}

__global__ void k_mid_flags(const int64_t* __restrict__ rp, int64_t n, int32_t* __restrict__ flag) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t d = rp[v + 1] - rp[v];
        flag[v] = d > kSmallMaxDeg && d <= kWarpMaxDeg;
    }
}

__global__ void k_mid_scatter(const int32_t* __restrict__ flag, const int64_t* __restrict__ pos, int64_t n,
                              uint32_t* __restrict__ out) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        if (flag[v]) out[pos[v]] = (uint32_t)v;
}

// Hub accumulation: one CTA per kHubSeg-edge segment of a window hub, four
// edges per thread in flight.  Needs no event table: it runs while the
// previous window commits its affected flags and the event table is built.
__device__ __forceinline__ void hub_accum_body(const ExactState& a, const Ctl* c) {
    const Round r = round_view(a, c);
    const long long q0 = c->es0, q1 = c->es1;
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
        uint32_t* occ = a.hub_occ + a.hub_toff[sg.hub];
        uint32_t* occn = a.hub_occn + sg.hub;
        const uint32_t d = a.vcom[h];
        const uint32_t ub = bound_of(a, h);
        if (threadIdx.x == 0) s_any = 0;
        __syncthreads();
        bool any = false;
        uint32_t c[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int64_t e = e0 + k * (int64_t)blockDim.x + threadIdx.x;
            c[k] = kNone;
            if (e < e1) {
                const int32_t v = a.col[e];
                any = any || (v >= r.P && v < (int64_t)h && prev_mover(a, r, v));
                if (counts(a, v, h, ub)) c[k] = comm_at(a, r, v, h);
            }
        }
        uint32_t own = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, c[k]);
            if (c[k] != kNone && lane == __ffs(peers) - 1) {
                // insert-or-add; a new key also goes on the hub's occupied list
                uint32_t hh = hash_u32(c[k]) & mask;
                while (true) {
                    const uint32_t prev = atomicCAS(&tk[hh], kNone, c[k]);
                    if (prev == kNone) occ[atomicAdd(occn, 1u)] = hh;
                    if (prev == kNone || prev == c[k]) {
                        atomicAdd(&tv[hh], (uint32_t)__popc(peers));
                        break;
                    }
                    hh = (hh + 1) & mask;
                }
            }
            own += __popc(__ballot_sync(0xFFFFFFFFu, c[k] == d));
        }
        if (lane == 0 && own) atomicAdd(&a.hub_kud[sg.hub], own);
        if (any) s_any = 1;
        __syncthreads();
        if (threadIdx.x == 0 && s_any) atomicOr(&a.hub_any[sg.hub], 1);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kHubThreads2) k_ex_hub_accum(ExactState a) {
    if (a.ctl->P >= a.ctl->n) return;
    hub_accum_body(a, a.ctl);
}

// Hub selection: one CTA per kTabSeg-slot segment of a window hub's table,
// one slot per thread; the last CTA of a hub reduces the partial maxima and
// records the decision.  Three CTAs per SM, as for the big rows.
__device__ __forceinline__ void hub_select_body(const ExactState& a, const Ctl* c) {
    const Round r = round_view(a, c);
    const long long q0 = c->ts0, q1 = c->ts1;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __shared__ double red_d[32];
    __shared__ uint32_t red_c[32];
    __shared__ int s_last;
    for (long long q = q0 + blockIdx.x; q < q1; q += gridDim.x) {
        const HubSeg sg = a.tseg[q];
        const int j = sg.hub;
        const uint32_t h = a.hub_v[j];
        const uint32_t* tk = a.tkeys + a.hub_toff[j];
        const uint32_t* tv = a.tvals + a.hub_toff[j];
        const uint32_t* occ = a.hub_occ + a.hub_toff[j];
        const uint32_t nocc = a.hub_occn[j];
        const uint32_t d = a.vcom[h];
        const long long ku = a.rp[h + 1] - a.rp[h];
        const uint32_t kud = a.hub_kud[j];
        double best_d = 0.0;
        uint32_t best_c = kNone;
        // Segment `part` covers occupied-list positions [s0, s0 + kTabSeg):
        // one per thread per step, the first step's lookup interleaved with
        // the one for d.
        const uint32_t s0 = (uint32_t)sg.part * kTabSeg, s1 = min(nocc, s0 + kTabSeg);
        if (s0 < s1) {
            long long sd = 0;
            for (uint32_t i0 = s0; i0 < s1; i0 += blockDim.x) {
                const uint32_t i = i0 + threadIdx.x;
                const uint32_t slot = i < s1 ? occ[i] : 0u;
                const uint32_t c0 = i < s1 ? tk[slot] : kNone, w0 = i < s1 ? tv[slot] : 0;
                const uint32_t cc[2] = {c0, d};
                const bool vv[2] = {c0 != kNone && c0 != d, i0 == s0};
                long long sgm[2];
                sigma_at_k<2>(a, r.tag, r.P, r.par, cc, vv, h, sgm);
                if (i0 == s0) sd = sgm[1];
                if (vv[0]) {
                    const double dl = delta_qi(a.dq, w0, kud, ku, sgm[0], sd);
                    if (dpos(dl) && better_pos(dl, c0, best_d, best_c)) { best_d = dl; best_c = c0; }
                }
            }
        }
        warp_argmax_pos(best_d, best_c);
        if (lane == 0) { red_d[w] = best_d; red_c[w] = best_c; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double bd = red_d[0];
            uint32_t bc = red_c[0];
            for (int k = 1; k < (int)(blockDim.x / 32); ++k)
                if (better_pos(red_d[k], red_c[k], bd, bc)) { bd = red_d[k]; bc = red_c[k]; }
            a.part_d[q] = bd;
            a.part_c[q] = bc;
            __threadfence();
            s_last = atomicAdd(&a.hub_done[j], 1) == a.hub_tcount[j] - 1;
        }
        __syncthreads();
        if (s_last) {
            // The whole CTA reduces the hub's partial maxima.
            __threadfence();
            double bd = 0.0;
            uint32_t bc = kNone;
            const int f = a.hub_tfirst[j], nt = a.hub_tcount[j];
            for (int k = threadIdx.x; k < nt; k += blockDim.x) {
                const double pd = ((volatile double*)a.part_d)[f + k];
                const uint32_t pc = ((volatile uint32_t*)a.part_c)[f + k];
                if (better_pos(pd, pc, bd, bc)) { bd = pd; bc = pc; }
            }
            warp_argmax_pos(bd, bc);
            __syncthreads();
            if (lane == 0) { red_d[w] = bd; red_c[w] = bc; }
            __syncthreads();
            if (threadIdx.x == 0) {
                bd = red_d[0];
                bc = red_c[0];
                for (int k = 1; k < (int)(blockDim.x / 32); ++k)
                    if (better_pos(red_d[k], red_c[k], bd, bc)) { bd = red_d[k]; bc = red_c[k]; }
                const bool act = a.vaff[h] != 0 || ((volatile int32_t*)a.hub_any)[j] != 0;
                bool stays = false;
                if (a.vcob) {
                    const uint32_t cc[1] = {d};
                    const bool vv[1] = {true};
                    long long o[1];
                    sigma_at_k<1>(a, r.tag, r.P, r.par, cc, vv, h, o);
                    stays = refine_stays(a, (double)o[0], ku);
                }
                if (!act) record(a, r, h, 0, d, 0.0);
                else if (!stays && bd > 0.0 && bc != kNone && bc != d) record(a, r, h, 1, bc, bd);
                else record(a, r, h, 1, d, 0.0);
                a.hub_done[j] = 0;
                a.hub_any[j] = 0;
                a.hub_kud[j] = 0;
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kHubThreads2, 3) k_ex_hub_select(ExactState a) {
    if (a.ctl->P >= a.ctl->n) return;
    hub_select_body(a, a.ctl);
}

// First change of the decided window (global, written by record()).
__device__ __forceinline__ unsigned long long first_change_of(const ExactState& a) {
    return *(volatile unsigned long long*)&a.ctl->first_change;
}

__device__ __forceinline__ long long commit_end(const ExactState& a, const Ctl* c) {
    const unsigned long long f = first_change_of(a);
    const long long E = c->E;
    return f == kNoChange ? E - 1 : min((long long)f, E - 1);
}

// The window just decided, as the commit kernels see it after the advance:
// [cP, cX] is committed (empty when cX < cP); the decisions are the new
// round's "previous" buffers.
struct CommitView {
    long long P, x;
    const uint8_t* act;
    const uint32_t* best;
    const double* delta;
};

__device__ __forceinline__ CommitView commit_view(const ExactState& a, const Ctl* ct) {
    CommitView c;
    c.P = ct->cP;
    c.x = ct->cX;
    const int par = (int)(ct->round & 1);
    c.act = a.act[par];
    c.best = a.best[par];
    c.delta = a.delta[par];
    return c;
}

// Commit [cP, cX]: totals and memberships of movers, final deltas, processed
// flags cleared, move flags for the affected-flag kernels; and the decided
// window's hub tables cleared for the next round.
// Adds (or, with neg, subtracts) v to total[key] once per distinct key of the
// warp (kNone = no update); every lane of the warp calls it.  Degrees are
// below 2^31, so the 16-bit halves of 32 of them sum without overflow.
__device__ __forceinline__ void warp_add_total(unsigned long long* total, uint32_t key, uint32_t v, bool neg) {
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, key);
    const unsigned lo = __reduce_add_sync(peers, v & 0xFFFFu), hi = __reduce_add_sync(peers, v >> 16);
    if (key != kNone && (threadIdx.x & 31) == __ffs(peers) - 1) {
        const long long sum = ((long long)hi << 16) + (long long)lo;
        if (sum) atomicAdd(&total[key], (unsigned long long)(neg ? -sum : sum));
    }
}

__device__ __forceinline__ void commit_a_body(const ExactState& a, const Ctl* ct) {
    const CommitView c = commit_view(a, ct);
    if (c.x < c.P) return;
    // Warp-uniform loop: the total updates are summed per community inside
    // the warp first (many movers of a window join the same few communities,
    // and their atomics on one total would serialise).
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = c.P + ((blockIdx.x * (long long)blockDim.x + threadIdx.x) & ~31ll); base <= c.x;
         base += stride) {
        const long long u = base + lane;
        bool moves = false;
        uint32_t cur = kNone, nb = kNone;
        uint32_t deg = 0;
        if (u <= c.x) {
            double dl = 0.0;
            cur = a.vcom[u];
            nb = c.best[u];
            moves = c.act[u] == 1 && nb != cur;
            if (moves) {
                deg = (uint32_t)(a.rp[u + 1] - a.rp[u]);
                dl = c.delta[u];
                a.vcom[u] = nb;
            }
            a.mv[u] = moves;
            a.final_delta[u] = dl;
            a.vaff[u] = 0;
        }
        warp_add_total(a.ctot, moves ? cur : kNone, deg, true);
        warp_add_total(a.ctot, moves ? nb : kNone, deg, false);
    }
    const long long q0 = ct->c_ts0, q1 = ct->c_ts1;
    __shared__ int s_last;
    for (long long q = q0 + blockIdx.x; q < q1; q += gridDim.x) {
        const HubSeg sg = a.tseg[q];
        const int j = sg.hub;
        uint32_t* tk = a.tkeys + a.hub_toff[j];
        uint32_t* tv = a.tvals + a.hub_toff[j];
        const uint32_t* occ = a.hub_occ + a.hub_toff[j];
        const uint32_t s0 = (uint32_t)sg.part * kTabSeg, s1 = min(a.hub_occn[j], s0 + kTabSeg);
        for (uint32_t i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
            const uint32_t slot = occ[i];
            tk[slot] = kNone;
            tv[slot] = 0;
        }
        __syncthreads();
        // The hub's last clearing CTA empties its occupied list (every CTA has
        // read the count before it arrives here).
        if (threadIdx.x == 0) s_last = atomicAdd(&a.hub_clr[j], 1) == a.hub_tcount[j] - 1;
        __syncthreads();
        if (s_last && threadIdx.x == 0) {
            a.hub_occn[j] = 0;
            a.hub_clr[j] = 0;
        }
    }
}

__global__ void k_ex_commit_a(ExactState a) { commit_a_body(a, a.ctl); }

// Affected flags from committed movers: every neighbour outside [cP, cX] and
// every neighbour in [cP, cX] processed before the mover.  Non-hub movers
// here, hub movers in k_ex_commit_hub.
__device__ __forceinline__ void commit_b_body(const ExactState& a, const Ctl* ct) {
    const CommitView c = commit_view(a, ct);
    if (c.x < c.P) return;
    // A thread per window vertex: rows of up to kOwnRow entries are flagged
    // by their own thread (four entries in flight), longer ones by the whole
    // warp, one row after another.
    constexpr int kOwnRow = 16;
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = c.P + ((blockIdx.x * (long long)blockDim.x + threadIdx.x) & ~31ll); base <= c.x;
         base += stride) {
        const long long w = base + lane;
        int64_t rb = 0, re = 0;
        if (w <= c.x && a.mv[w]) {
            rb = a.rp[w];
            re = a.rp[w + 1];
            if (re - rb > kWarpMaxDeg) re = rb;   // hubs and big rows: k_ex_commit_hub
        }
        if (re - rb <= kOwnRow) {
            for (int64_t e0 = rb; e0 < re; e0 += 4) {
                int32_t v[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) v[k] = e0 + k < re ? a.col[e0 + k] : -1;
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (v[k] >= 0 && (v[k] < c.P || v[k] > c.x || v[k] < w)) a.vaff[v[k]] = 1;
            }
        }
        unsigned longer = __ballot_sync(0xFFFFFFFFu, re - rb > kOwnRow);
        while (longer) {
            const int src = __ffs(longer) - 1;
            longer &= longer - 1;
            const long long ws = __shfl_sync(0xFFFFFFFFu, w, src);
            const int64_t rbs = __shfl_sync(0xFFFFFFFFu, rb, src), res = __shfl_sync(0xFFFFFFFFu, re, src);
            for (int64_t e = rbs + lane; e < res; e += 32) {
                const int32_t v = a.col[e];
                if (v < c.P || v > c.x || v < ws) a.vaff[v] = 1;
            }
        }
    }
}

__global__ void k_ex_commit_b(ExactState a) { commit_b_body(a, a.ctl); }

__device__ __forceinline__ void commit_hub_body(const ExactState& a, const Ctl* ct) {
    const CommitView c = commit_view(a, ct);
    if (c.x < c.P) return;
    // Work items: the decided window's hub edge segments, then its big rows.
    const long long q0 = ct->c_es0, q1 = ct->c_es1;
    const long long g0 = ct->c_bs0, g1 = ct->c_bs1;
    const long long nseg = q1 - q0, items = nseg + (g1 - g0);
    for (long long q = blockIdx.x; q < items; q += gridDim.x) {
        uint32_t h;
        int64_t e0, e1;
        if (q < nseg) {
            const HubSeg sg = a.eseg[q0 + q];
            h = a.hub_v[sg.hub];
            e0 = a.rp[h] + (int64_t)sg.part * kHubSeg;
            e1 = min(a.rp[h + 1], e0 + kHubSeg);
        } else {
            h = a.big_v[g0 + (q - nseg)];
            e0 = a.rp[h];
            e1 = a.rp[h + 1];
        }
        if ((long long)h > c.x || !a.mv[h]) continue;   // block-uniform
        for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
            const int32_t v = a.col[e];
            if (v < c.P || v > c.x || v < (int64_t)h) a.vaff[v] = 1;
        }
    }
}

__global__ void __launch_bounds__(kHubThreads2) k_ex_commit_hub(ExactState a) { commit_hub_body(a, a.ctl); }

// Re-choose the designated communities of the next table from the counts of
// the table just used: the designated ones' event counts and the sorted
// table's hot slots, largest first, at least kZKeep events each.  Keeps the
// set when nothing in the sorted table was hot and every member kept its
// events.  Called by every thread of one CTA.
__device__ __forceinline__ void designate(const ExactState& a, Ctl* c) {
    __shared__ unsigned long long cand[kZMax + kZCand];
    __shared__ int s_change;
    const int tid = threadIdx.x;
    const int nz = (int)c->nz;
    const int nh = min((int)a.ctl->nhot, kZCand);
    if (tid == 0) {
        int change = nh > 0;
        for (int j = 0; j < nz; ++j) change |= c->zcount[j] < (unsigned)kZKeep;
        s_change = change;
    }
    __syncthreads();
    if (!s_change) {
        if (tid < kZMax) c->zcount[tid] = 0;
        __syncthreads();
        return;
    }
    if (tid < nz) cand[tid] = (unsigned long long)c->zcount[tid] << 32 | c->zc[tid];
    if (tid < nh) cand[nz + tid] = a.zcand[tid];
    __syncthreads();
    if (tid < 32) {
        const int total = nz + nh;
        uint32_t chosen[kZMax];
        int nc = 0;
#pragma unroll 1
        for (int pick = 0; pick < kZMax; ++pick) {
            unsigned long long best = 0;
            int bi = -1;
            for (int t = tid; t < total; t += 32) {
                const unsigned long long v = cand[t];
                if ((v >> 32) >= (unsigned long long)kZKeep && v > best) {
                    best = v;
                    bi = t;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long ob = __shfl_xor_sync(0xFFFFFFFFu, best, o);
                const int oi = __shfl_xor_sync(0xFFFFFFFFu, bi, o);
                if (ob > best) {
                    best = ob;
                    bi = oi;
                }
            }
            if (best == 0) break;
            if (tid == 0) {
                chosen[nc] = (uint32_t)best;
                cand[bi] = 0;
            }
            ++nc;
            __syncwarp();
        }
        if (tid == 0) {
            for (int j = 0; j < nz; ++j) a.zof[c->zc[j]] = 0;
            for (int j = 0; j < nc; ++j) {
                a.zof[chosen[j]] = (uint8_t)(j + 1);
                c->zc[j] = chosen[j];
            }
            c->nz = (unsigned)nc;
            for (int j = 0; j < kZMax; ++j) c->zcount[j] = 0;
        }
    }
    __syncthreads();
}

// After the window's decisions: fix the committed prefix [P, x] for the commit
// kernels, slide the window (the new decisions become D_prev; entering
// vertices are unknown) and tell the graph's loop whether to go on.  The next
// window's event table and this window's commits then run concurrently: they
// touch disjoint vertices.  `c` is the control block this CTA works on; the
// entering vertices' marks are written by threads (tid0, tid0 + tstride, ...).
// Ends with a CTA barrier, so every thread sees the updated block.
__device__ __forceinline__ void advance_ctl(const ExactState& a, Ctl* c, long long tid0, long long tstride,
                                            bool set_cond) {
    const long long P = c->P, E = c->E, n = c->n, B = c->B;
    if (P >= n) {
        __syncthreads();
        if (threadIdx.x == 0) {
            c->cP = 1;   // nothing to commit
            c->cX = 0;
            if (set_cond) cudaGraphSetConditional(a.cond, 0u);
        }
        __syncthreads();
        return;
    }
    const long long x = commit_end(a, c);
    const long long nP = x + 1, nE = min(n, nP + B);
    const int par = (int)(c->round & 1);
    uint8_t* next_prev_act = a.act[par ^ 1];
    for (long long u = E + tid0; u < nE; u += tstride) next_prev_act[u] = kUnknown;
    if (threadIdx.x == 0) {
        c->c_es0 = c->es0;
        c->c_es1 = c->es1;
        c->c_ts0 = c->ts0;
        c->c_ts1 = c->ts1;
        c->c_bs0 = c->bs0;
        c->c_bs1 = c->bs1;
    }
    __syncthreads();
    window_ranges(a, c, nP, nE);
    designate(a, c);
    if (threadIdx.x == 0) {
        const long long rnd = c->round + 1;
        c->cP = P;
        c->cX = x;
        c->evals = c->evals + (E - P);
        c->P = nP;
        c->E = nE;
        c->round = rnd;
        c->tag = c->tag + 1;
        // Every round commits at least vertex P, so the loop ends within n
        // rounds; the bound only guards against a broken invariant.
        bool more = nP < n;
        if (nP <= P || (more && rnd >= c->max_rounds)) {
            c->error = 1;
            c->P = n;
            more = false;
        }
        if (set_cond) cudaGraphSetConditional(a.cond, more ? 1u : 0u);
    }
    __syncthreads();
}

__global__ void __launch_bounds__(1024) k_ex_advance(ExactState a) {
    advance_ctl(a, a.ctl, threadIdx.x, blockDim.x, a.use_cond != 0);
}

// The first window of an iteration; same split of the marks as advance_ctl.
__device__ __forceinline__ void init_ctl(const ExactState& a, Ctl* c, long long tid0, long long tstride) {
    const long long n = c->n, B = c->B;
    const long long E = min(n, B);
    for (long long u = tid0; u < E; u += tstride) a.act[0][u] = kUnknown;
    window_ranges(a, c, 0, E);
    __syncthreads();
    if (threadIdx.x == 0) {
        c->P = 0;
        c->E = E;
        c->round = 0;
        c->evals = 0;
        c->cP = 1;
        c->cX = 0;
        c->tag = c->tag + 1;
        for (int j = 0; j < kZMax; ++j) c->zcount[j] = 0;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(1024) k_ex_init_iter(ExactState a) {
    init_ctl(a, a.ctl, threadIdx.x, blockDim.x);
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
                     cudaStream_t s, int64_t* launches, int64_t* rounds_out, int64_t* evals_out) {
    const int64_t n = ctx.g.n;
    const int64_t B = std::max<int64_t>(32, std::min<int64_t>(std::min<int64_t>(window, kWindowMax), n));

    // ---- hub segment tables (once per call) ----
    // Rows above kWarpMaxDeg: up to kBigMaxDeg one CTA each ("big"), above
    // that segmented over CTAs ("hubs").
    const int64_t nh_all = (int64_t)ctx.hubs_h.size();
    std::vector<int64_t> hdeg_all(nh_all);
    if (nh_all) {
        DevBuf<int64_t> dd(nh_all, s);
        k_hub_degrees<<<grid_for(nh_all, kT), kT, 0, s>>>(ctx.g.row_ptr, ctx.hubs, nh_all, dd);
        GB_LAUNCH_CHECK();
        GB_CUDA(cudaMemcpyAsync(hdeg_all.data(), dd.get(), nh_all * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaStreamSynchronize(s));
    }
    std::vector<uint32_t> big_h, hub_h;
    std::vector<int64_t> hdeg;
    for (int64_t j = 0; j < nh_all; ++j) {
        if (hdeg_all[j] <= kBigMaxDeg) {
            big_h.push_back(ctx.hubs_h[j]);
        } else {
            hub_h.push_back(ctx.hubs_h[j]);
            hdeg.push_back(hdeg_all[j]);
        }
    }
    const int64_t nh = (int64_t)hub_h.size(), n_big = (int64_t)big_h.size();
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
            eseg_v.push_back(hub_h[j]);
        }
        const int nt = (int)std::max<int64_t>(1, ceil_div(hdeg[j], kTabSeg));   // occupied slots <= degree
        tfirst[j] = (int32_t)tseg.size();
        tcount[j] = nt;
        for (int k = 0; k < nt; ++k) {
            tseg.push_back({(int32_t)j, k});
            tseg_v.push_back(hub_h[j]);
        }
    }
    DevBuf<int64_t> d_toff = upload(toff, s);
    DevBuf<uint32_t> d_tcap = upload(tcap, s);
    DevBuf<int32_t> d_tfirst = upload(tfirst, s), d_tcount = upload(tcount, s);
    DevBuf<HubSeg> d_eseg = upload(eseg, s), d_tseg = upload(tseg, s);
    DevBuf<uint32_t> d_eseg_v = upload(eseg_v, s), d_tseg_v = upload(tseg_v, s);
    DevBuf<uint32_t> d_hub_v = upload(hub_h, s), d_big_v = upload(big_h, s);
    DevBuf<uint32_t> tkeys(pool > 0 ? pool : 1, s), tvals(pool > 0 ? pool : 1, s);
    GB_CUDA(cudaMemsetAsync(tkeys, 0xFF, (pool > 0 ? pool : 1) * sizeof(uint32_t), s));
    GB_CUDA(cudaMemsetAsync(tvals, 0, (pool > 0 ? pool : 1) * sizeof(uint32_t), s));
    DevBuf<int32_t> hub_any(nh > 0 ? nh : 1, s), hub_done(nh > 0 ? nh : 1, s);
    GB_CUDA(cudaMemsetAsync(hub_any, 0, (nh > 0 ? nh : 1) * sizeof(int32_t), s));
    GB_CUDA(cudaMemsetAsync(hub_done, 0, (nh > 0 ? nh : 1) * sizeof(int32_t), s));
    DevBuf<uint32_t> hub_kud(nh > 0 ? nh : 1, s), hub_occn(nh > 0 ? nh : 1, s);
    DevBuf<int32_t> hub_clr(nh > 0 ? nh : 1, s);
    DevBuf<uint32_t> hub_occ(pool > 0 ? pool : 1, s);
    GB_CUDA(cudaMemsetAsync(hub_occn, 0, (nh > 0 ? nh : 1) * sizeof(uint32_t), s));
    GB_CUDA(cudaMemsetAsync(hub_clr, 0, (nh > 0 ? nh : 1) * sizeof(int32_t), s));
    GB_CUDA(cudaMemsetAsync(hub_kud, 0, (nh > 0 ? nh : 1) * sizeof(uint32_t), s));
    DevBuf<double> part_d(tseg.empty() ? 1 : tseg.size(), s);
    DevBuf<uint32_t> part_c(tseg.empty() ? 1 : tseg.size(), s);

    // ---- mid-degree list (ascending vertex ids) ----
    int64_t n_mid = 0;
    DevBuf<uint32_t> mid_v;
    {
        DevBuf<int32_t> flag(n, s);
        DevBuf<int64_t> pos(n, s), tot(1, s);
        k_mid_flags<<<grid_for(n, kT), kT, 0, s>>>(ctx.g.row_ptr, n, flag);
        GB_LAUNCH_CHECK();
        exclusive_scan_i32_to_i64(flag, pos, n, tot, s);
        n_mid = read_dev(tot.get(), s);
        mid_v.alloc(n_mid > 0 ? n_mid : 1, s);
        if (n_mid) {
            k_mid_scatter<<<grid_for(n, kT), kT, 0, s>>>(flag, pos, n, mid_v);
            GB_LAUNCH_CHECK();
        }
    }

    // ---- round state ----
    DevBuf<uint32_t> best0(n, s), best1(n, s);
    DevBuf<uint8_t> act0(n, s), act1(n, s);
    DevBuf<double> delta0(n, s), delta1(n, s), final_delta(n, s);
    DevBuf<uint8_t> mv(n, s);
    DevBuf<SlotMeta> slots(kTableSlots, s);
    GB_CUDA(cudaMemsetAsync(slots, 0xFF, kTableSlots * sizeof(SlotMeta), s));   // no generation yet
    DevBuf<uint32_t> stime(kEventsMax, s), tb_s0(kWindowMax, s), tb_s1(kWindowMax, s);
    DevBuf<long long> epre(kEventsMax, s);
    DevBuf<int32_t> wdeg(kWindowMax, s), tb_hist(kCoarse * kTbChunks, s), tb_base(kCoarse * kTbChunks, s),
        tb_bstart(kCoarse + 1, s);
    DevBuf<unsigned long long> ev1(kEventsMax, s), ev2(kEventsMax, s);
    DevBuf<int32_t> hot_bidx((size_t)kHotMax * kHotStride, s);
    DevBuf<uint8_t> zof(n > 0 ? n : 1, s);
    GB_CUDA(cudaMemsetAsync(zof, 0, (n > 0 ? n : 1), s));
    DevBuf<int32_t> zcontrib((size_t)2 * kZMax * kWindowMax, s);
    DevBuf<long long> zbsum((size_t)2 * kZMax * kHotStride, s), zpre((size_t)2 * kZMax * kHotStride, s);
    DevBuf<unsigned long long> zcand(kZCand, s);
    DevBuf<Ctl> ctl(1, s);
    Ctl* hctl = nullptr;
    GB_CUDA(cudaMallocHost(&hctl, sizeof(Ctl)));
    *hctl = Ctl{};
    hctl->n = n;
    hctl->B = B;
    hctl->max_rounds = n + 2;
    GB_CUDA(cudaMemcpyAsync(ctl.get(), hctl, sizeof(Ctl), cudaMemcpyHostToDevice, s));
    DevBuf<double> partial(1024, s), dsum(1, s);
    DevBuf<unsigned long long> nmov(1, s);

    ExactState a{};
    a.rp = ctx.g.row_ptr;
    a.col = ctx.g.col;
    a.vcom = ctx.vcom;
    a.ctot = ctx.ctot;
    a.vaff = ctx.vaff;
    a.vcob = ctx.vcob;
    a.mv = mv.get();
    a.ctl = ctl.get();
    a.best[0] = best0.get();
    a.best[1] = best1.get();
    a.act[0] = act0.get();
    a.act[1] = act1.get();
    a.delta[0] = delta0.get();
    a.delta[1] = delta1.get();
    a.final_delta = final_delta.get();
    a.slots = slots.get();
    a.tb_s0 = tb_s0.get();
    a.tb_s1 = tb_s1.get();
    a.wdeg = wdeg.get();
    a.tb_hist = tb_hist.get();
    a.tb_base = tb_base.get();
    a.tb_bstart = tb_bstart.get();
    a.ev1 = ev1.get();
    a.ev2 = ev2.get();
    a.hot_bidx = hot_bidx.get();
    a.zof = zof.get();
    a.zcontrib = zcontrib.get();
    a.zbsum = zbsum.get();
    a.zpre = zpre.get();
    a.zcand = zcand.get();
    a.stime = stime.get();
    a.epre = epre.get();
    a.hub_v = d_hub_v.get();
    a.big_v = d_big_v.get();
    a.n_big = n_big;
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
    a.hub_kud = hub_kud.get();
    a.hub_occ = hub_occ.get();
    a.hub_occn = hub_occn.get();
    a.hub_clr = hub_clr.get();
    a.hub_done = hub_done.get();
    a.part_d = part_d.get();
    a.part_c = part_c.get();
    a.mid_v = mid_v.get();
    a.n_mid = n_mid;
    a.M = ctx.M;
    a.R = ctx.R;
    a.dq = ctx.dq;

    static_assert(kEventsMax + 32 * 257 <= kTableSlots + kEventsMax, "sort scratch fits the hash area");
    const int group_smem = 32 * kCoarse * (int)sizeof(int32_t);
    GB_CUDA(cudaFuncSetAttribute(k_tb_group, cudaFuncAttributeMaxDynamicSharedMemorySize, group_smem));
    const int tb_grid = (int)ceil_div(B, kTbThreads);
    const int finish_smem = (kTbFinishThreads / 32) * ((1 << kFineBits) + 1) * (int)sizeof(int32_t);
    GB_CUDA(cudaFuncSetAttribute(k_tb_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, finish_smem));
    auto enqueue_table = [&](cudaStream_t st) {
        k_tb_insert<<<tb_grid, kTbThreads, 0, st>>>(a);
        k_tb_group<<<tb_grid, kTbThreads, group_smem, st>>>(a);
        k_tb_finish<<<kCoarse + kZMax, kTbFinishThreads, finish_smem, st>>>(a);
    };
    const int mid_smem = kMidWarpsPerBlock * 2 * kWarpHash * (int)sizeof(uint32_t);
    GB_CUDA(cudaFuncSetAttribute(k_ex_eval_mid, cudaFuncAttributeMaxDynamicSharedMemorySize, mid_smem));
    const int small_grid = (int)std::max<int64_t>(1, ceil_div(B, 4 * kSmallWarpsPerBlock));
    // Grid-stride kernels: one resident wave (blocks per SM from the occupancy
    // of the compiled kernel x the SM count).
    auto resident = [&](const void* fn, int threads, int smem) {
        int per_sm = 0;
        GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
        int dev = 0, sms = kNumSMs;
        GB_CUDA(cudaGetDevice(&dev));
        GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        return std::max(1, per_sm) * sms;
    };
    const int mid_grid = resident((const void*)k_ex_eval_mid, kMidWarpsPerBlock * 32, mid_smem);
    const int select_grid = resident((const void*)k_ex_hub_select, kHubThreads2, 0);
    const int big_smem = (2 * kBigSlots + 2 * kBigMaxDeg) * (int)sizeof(uint32_t);
    GB_CUDA(cudaFuncSetAttribute(k_ex_eval_big, cudaFuncAttributeMaxDynamicSharedMemorySize, big_smem));
    const int big_grid = resident((const void*)k_ex_eval_big, kBigThreads, big_smem);
    const int hub_grid = resident((const void*)k_ex_hub_accum, kHubThreads2, 0);
    const int commit_grid = (int)std::max<int64_t>(1, ceil_div(B, kT));
    const int commit_b_grid = (int)std::max<int64_t>(1, ceil_div(B, kT));
    // eval_small, advance, 3 table kernels, commit_a, commit_b; eval_mid;
    // eval_big; hub_select + hub_accum; commit_hub (hubs or big rows).
    const int per_round = 7 + (n_mid ? 1 : 0) + (n_big ? 1 : 0) + (nh ? 2 : 0) + ((nh || n_big) ? 1 : 0);
    const int commit_a_grid = std::max(commit_grid, nh ? hub_grid : 0);
    // Side streams and events for the fork/join shape of a captured round:
    struct Fork {
        cudaStream_t s1 = nullptr, s2 = nullptr, s3 = nullptr;
        cudaEvent_t ev[9] = {};
        ~Fork() {
            for (cudaEvent_t e : ev)
                if (e) cudaEventDestroy(e);
            if (s1) cudaStreamDestroy(s1);
            if (s2) cudaStreamDestroy(s2);
            if (s3) cudaStreamDestroy(s3);
        }
    } fk;
    // One round: decide the window, advance, then prepare the next window
    // while this one commits.  Forked shape (graph capture):
    //   { eval_small | eval_mid | hub_select } -> advance
    //   -> { table(next) | commit_a -> { commit_b | commit_hub | hub_accum(next) } }
    // hub_accum needs the committed memberships but no event table; the
    // round before the first needs the first window's table and accumulation.
    auto enqueue_round = [&](cudaStream_t st, bool fork) {
        cudaStream_t sm = fork ? fk.s1 : st, sh = fork ? fk.s2 : st, sa = fork ? fk.s3 : st;
        if (fork) {
            GB_CUDA(cudaEventRecord(fk.ev[0], st));
            GB_CUDA(cudaStreamWaitEvent(sm, fk.ev[0], 0));
            GB_CUDA(cudaStreamWaitEvent(sh, fk.ev[0], 0));
        }
        if (fork) GB_CUDA(cudaStreamWaitEvent(sa, fk.ev[0], 0));
        k_ex_eval_small<<<small_grid, kSmallWarpsPerBlock * 32, 0, st>>>(a);
        if (n_mid) k_ex_eval_mid<<<mid_grid, kMidWarpsPerBlock * 32, mid_smem, sm>>>(a);
        if (nh) k_ex_hub_select<<<select_grid, kHubThreads2, 0, sh>>>(a);
        if (n_big) k_ex_eval_big<<<big_grid, kBigThreads, big_smem, sa>>>(a);
        if (fork) {
            GB_CUDA(cudaEventRecord(fk.ev[1], sm));
            GB_CUDA(cudaEventRecord(fk.ev[2], sh));
            GB_CUDA(cudaEventRecord(fk.ev[8], sa));
            GB_CUDA(cudaStreamWaitEvent(st, fk.ev[1], 0));
            GB_CUDA(cudaStreamWaitEvent(st, fk.ev[2], 0));
            GB_CUDA(cudaStreamWaitEvent(st, fk.ev[8], 0));
        }
        k_ex_advance<<<1, 1024, 0, st>>>(a);
        if (fork) {
            GB_CUDA(cudaEventRecord(fk.ev[3], st));
            GB_CUDA(cudaStreamWaitEvent(sm, fk.ev[3], 0));
        }
        enqueue_table(sm);
        k_ex_commit_a<<<commit_a_grid, kT, 0, st>>>(a);
        if (fork) {
            GB_CUDA(cudaEventRecord(fk.ev[4], st));
            GB_CUDA(cudaStreamWaitEvent(sh, fk.ev[4], 0));
            GB_CUDA(cudaStreamWaitEvent(sa, fk.ev[4], 0));
        }
        k_ex_commit_b<<<commit_b_grid, kT, 0, st>>>(a);
        if (nh || n_big) k_ex_commit_hub<<<hub_grid, kHubThreads2, 0, sh>>>(a);
        if (nh) k_ex_hub_accum<<<hub_grid, kHubThreads2, 0, sa>>>(a);
        if (fork) {
            GB_CUDA(cudaEventRecord(fk.ev[5], sm));
            GB_CUDA(cudaEventRecord(fk.ev[6], sh));
            GB_CUDA(cudaEventRecord(fk.ev[7], sa));
            GB_CUDA(cudaStreamWaitEvent(st, fk.ev[5], 0));
            GB_CUDA(cudaStreamWaitEvent(st, fk.ev[6], 0));
            GB_CUDA(cudaStreamWaitEvent(st, fk.ev[7], 0));
        }
        GB_LAUNCH_CHECK();
    };
    auto enqueue_first = [&](cudaStream_t st) {
        k_ex_init_iter<<<1, 1024, 0, st>>>(a);
        enqueue_table(st);
        if (nh) k_ex_hub_accum<<<hub_grid, kHubThreads2, 0, st>>>(a);
    };

    // One local-moving iteration as one graph: the init kernel, then a
    // device-side while loop over rounds whose condition the advance kernel
    // sets.  GBGPU_EXACT_GRAPH=0 enqueues rounds from the host instead.
    const char* genv = std::getenv("GBGPU_EXACT_GRAPH");
    const bool use_graph = !(genv && genv[0] == '0');
    struct GraphGuard {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t e = nullptr;
        cudaStream_t cs = nullptr;
        ~GraphGuard() {
            if (e) cudaGraphExecDestroy(e);
            if (g) cudaGraphDestroy(g);
            if (cs) cudaStreamDestroy(cs);
        }
    } gg;
    if (use_graph) {
        GB_CUDA(cudaStreamCreateWithFlags(&gg.cs, cudaStreamNonBlocking));
        GB_CUDA(cudaGraphCreate(&gg.g, 0));
        cudaGraphConditionalHandle cond;
        GB_CUDA(cudaGraphConditionalHandleCreate(&cond, gg.g, 1, cudaGraphCondAssignDefault));
        a.cond = cond;
        a.use_cond = 1;
        // init -> first window's table (captured) -> while(rounds)
        GB_CUDA(cudaStreamBeginCaptureToGraph(gg.cs, gg.g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        enqueue_first(gg.cs);
        GB_LAUNCH_CHECK();
        GB_CUDA(cudaStreamEndCapture(gg.cs, &gg.g));
        // The captured chain's last node (the one no other node depends on).
        cudaGraphNode_t init_node = nullptr;
        {
            size_t nn = 0;
            GB_CUDA(cudaGraphGetNodes(gg.g, nullptr, &nn));
            std::vector<cudaGraphNode_t> nodes(nn);
            GB_CUDA(cudaGraphGetNodes(gg.g, nodes.data(), &nn));
            for (cudaGraphNode_t nd : nodes) {
                size_t nd_out = 0;
                GB_CUDA(cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &nd_out));
                if (nd_out == 0) init_node = nd;
            }
            if (!init_node) throw Error(GBGPU_E_CUDA, "serial-order local moving: empty init graph");
        }
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = cond;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t loop_node;
        GB_CUDA(cudaGraphAddNode(&loop_node, gg.g, &init_node, nullptr, 1, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        GB_CUDA(cudaStreamCreateWithFlags(&fk.s1, cudaStreamNonBlocking));
        GB_CUDA(cudaStreamCreateWithFlags(&fk.s2, cudaStreamNonBlocking));
        GB_CUDA(cudaStreamCreateWithFlags(&fk.s3, cudaStreamNonBlocking));
        for (cudaEvent_t& e : fk.ev) GB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        GB_CUDA(cudaStreamBeginCaptureToGraph(gg.cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        enqueue_round(gg.cs, true);
        GB_CUDA(cudaStreamEndCapture(gg.cs, &body));
        // Node priorities: the event-table chain that every round waits for
        // (and the advance before it) first; the affected-flag branch, which
        // runs beside the table with time to spare, last; the evaluations in
        // between.  Honoured through cudaGraphInstantiateFlagUseNodePriority
        // (RMAT-22 local moving 105 -> 100 ms: the table's CTAs no longer wait
        // behind the commit branch's).
        {
            int least = 0, greatest = 0;
            GB_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
            const int mid = (least + greatest) / 2;
            size_t nn = 0;
            GB_CUDA(cudaGraphGetNodes(body, nullptr, &nn));
            std::vector<cudaGraphNode_t> nodes(nn);
            GB_CUDA(cudaGraphGetNodes(body, nodes.data(), &nn));
            for (cudaGraphNode_t nd : nodes) {
                cudaGraphNodeType ty;
                GB_CUDA(cudaGraphNodeGetType(nd, &ty));
                if (ty != cudaGraphNodeTypeKernel) continue;
                cudaKernelNodeParams kp;
                GB_CUDA(cudaGraphKernelNodeGetParams(nd, &kp));
                const void* f = kp.func;
                int pr = mid;
                if (f == (const void*)k_tb_insert || f == (const void*)k_tb_group || f == (const void*)k_tb_finish ||
                    f == (const void*)k_ex_advance)
                    pr = greatest;
                else if (f == (const void*)k_ex_commit_b || f == (const void*)k_ex_commit_hub ||
                         f == (const void*)k_ex_hub_accum)
                    pr = least;
                cudaKernelNodeAttrValue v = {};
                v.priority = pr;
                GB_CUDA(cudaGraphKernelNodeSetAttribute(nd, cudaKernelNodeAttributePriority, &v));
            }
        }
        GB_CUDA(cudaGraphInstantiate(&gg.e, gg.g, cudaGraphInstantiateFlagUseNodePriority));
    }
    const int kBatch = 8;

    int iterations = 0;
    int64_t rounds = 0, nl = 0, evals = 0;
    for (int it = 0; it < max_iterations; ++it) {
        if (use_graph) {
            GB_CUDA(cudaGraphLaunch(gg.e, s));
            GB_CUDA(cudaMemcpyAsync(hctl, ctl.get(), sizeof(Ctl), cudaMemcpyDeviceToHost, s));
            GB_CUDA(cudaStreamSynchronize(s));
        } else {
            enqueue_first(s);
            GB_LAUNCH_CHECK();
            while (true) {
                for (int b = 0; b < kBatch; ++b) enqueue_round(s, false);
                GB_CUDA(cudaMemcpyAsync(hctl, ctl.get(), sizeof(Ctl), cudaMemcpyDeviceToHost, s));
                GB_CUDA(cudaStreamSynchronize(s));
                if (hctl->P >= n) break;
            }
        }
        if (hctl->error == 2)
            throw Error(GBGPU_E_CUDA, "serial-order local moving: event table slot with an invalid hot index");
        if (hctl->error)
            throw Error(GBGPU_E_CUDA, "serial-order local moving: round loop stopped without progress");
        nl += 4 + (nh ? 1 : 0) + hctl->round * per_round;
        rounds += hctl->round;
        evals += hctl->evals;
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
    if (evals_out) *evals_out += evals;
    return iterations;
}

}  // namespace gb
