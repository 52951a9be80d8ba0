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
//     exact prefix: all of [P, x] was evaluated from exact inputs, so it is
//     committed; the rest of the window carries its new decisions forward.
//
// Community totals at time u come from an event table rebuilt every round:
// each speculative move contributes (old, -k) and (new, +k) at its time; the
// events are stably sorted by community slot and prefix-summed, and a lookup
// binary-searches the community's events for the last time before u.  All
// totals are exact integers, so every Delta-modularity equals the serial one.
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

struct ExactArgs {
    const int64_t* rp;
    const int32_t* col;
    const uint32_t* vcom;           // committed communities
    const unsigned long long* ctot; // committed totals
    const uint8_t* vaff;            // committed affected flags
    const uint32_t* pbest;          // D_prev
    const uint8_t* pact;
    uint32_t* nbest;                // D_new
    uint8_t* nact;
    double* ndelta;
    // event table
    const uint32_t* hkey;           // hash slot -> community (kNone empty)
    uint32_t hmask;
    const int32_t* sstart;          // slot -> [start, end) in sorted events
    const int32_t* send;
    const uint32_t* etime;          // sorted event times
    const long long* epre;          // inclusive prefix within the slot
    int64_t P, E;
    double M, R;
    unsigned long long* first_change;
};

__device__ __forceinline__ uint32_t slot_hash(uint32_t c) {
    return (uint32_t)(((uint64_t)c * 0x9E3779B97F4A7C15ull) >> 40);
}

__device__ __forceinline__ int find_slot(const uint32_t* hkey, uint32_t mask, uint32_t c) {
    uint32_t h = slot_hash(c) & mask;
    while (true) {
        const uint32_t k = hkey[h];
        if (k == c) return (int)h;
        if (k == kNone) return -1;
        h = (h + 1) & mask;
    }
}

// Community total at time u: committed total plus the speculative moves of
// window vertices before u.
__device__ __forceinline__ long long sigma_at(const ExactArgs& a, uint32_t c, uint32_t u) {
    long long s = (long long)a.ctot[c];
    const int slot = find_slot(a.hkey, a.hmask, c);
    if (slot < 0) return s;
    int lo = a.sstart[slot], hi = a.send[slot];  // events sorted by time
    // last index with time < u
    int l = lo, r = hi;
    while (l < r) {
        const int mid = (l + r) >> 1;
        if (a.etime[mid] < u) l = mid + 1; else r = mid;
    }
    if (l > lo) s += a.epre[l - 1];
    return s;
}

__device__ __forceinline__ bool prev_mover(const ExactArgs& a, int64_t v) {
    return a.pact[v] == 1 && a.pbest[v] != a.vcom[v];
}

// Community of neighbour v as seen at time u.
__device__ __forceinline__ uint32_t comm_at(const ExactArgs& a, int64_t v, int64_t u) {
    if (v >= a.P && v < u && prev_mover(a, v)) return a.pbest[v];
    return a.vcom[v];
}

__device__ __forceinline__ void record(const ExactArgs& a, int64_t u, uint8_t act, uint32_t best, double delta) {
    a.nact[u] = act;
    a.nbest[u] = best;
    a.ndelta[u] = delta;
    if (act != a.pact[u] || (act == 1 && best != a.pbest[u])) atomicMin(a.first_change, (unsigned long long)u);
}

constexpr int kExWarpsPerBlock = 4;

// Warp per window vertex (degree <= kWarpMaxDeg).
__global__ void __launch_bounds__(kExWarpsPerBlock * 32)
k_exact_eval_warp(ExactArgs a) {
    extern __shared__ uint32_t ex_smem[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t* tk = ex_smem + (size_t)w * 2 * kWarpHash;
    uint32_t* tv = tk + kWarpHash;
    const int64_t nw = (int64_t)gridDim.x * kExWarpsPerBlock;
    for (int64_t u = a.P + (int64_t)blockIdx.x * kExWarpsPerBlock + w; u < a.E; u += nw) {
        const int64_t rb = a.rp[u];
        const int deg = (int)(a.rp[u + 1] - rb);
        if (deg > kWarpMaxDeg) continue;
        // Affected at time u: committed flag, or a neighbour before u moved.
        bool act = a.vaff[u] != 0;
        if (!act) {
            bool any = false;
            for (int i = lane; i < deg && !any; i += 32) {
                const int32_t v = a.col[rb + i];
                any = (v >= a.P && v < u && prev_mover(a, v));
            }
            act = __any_sync(0xFFFFFFFFu, any);
        }
        const uint32_t d = a.vcom[u];
        if (!act) {
            if (lane == 0) record(a, u, 0, d, 0.0);
            continue;
        }
        const double ku = (double)deg;
        double best_d = 0.0;
        uint32_t best_c = kNone;
        if (deg <= 32) {
            uint32_t c = kNone;
            if (lane < deg) {
                const int32_t v = a.col[rb + lane];
                if (v != (int32_t)u) c = comm_at(a, v, u);
            }
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, c);
            const double kud = (double)__popc(__ballot_sync(0xFFFFFFFFu, c == d));
            const double sd = (double)sigma_at(a, d, (uint32_t)u);
            if (c != kNone && c != d && lane == __ffs(peers) - 1) {
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
                    if (v != (int32_t)u) c = comm_at(a, v, u);
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
            if (best_d > 0.0 && best_c != kNone && best_c != d) record(a, u, 1, best_c, best_d);
            else record(a, u, 1, d, 0.0);
        }
    }
}

// CTA per window hub (degree > kWarpMaxDeg).
__global__ void __launch_bounds__(kHubThreads)
k_exact_eval_hub(ExactArgs a, const uint32_t* __restrict__ hubs, int64_t h0, int64_t h1,
                 uint32_t* __restrict__ gkeys, uint32_t* __restrict__ gvals, int64_t gcap) {
    extern __shared__ uint32_t sm[];
    __shared__ double red_d[kHubThreads / 32];
    __shared__ uint32_t red_c[kHubThreads / 32];
    __shared__ uint32_t s_kud;
    __shared__ int s_any;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int64_t hi = h0 + blockIdx.x; hi < h1; hi += gridDim.x) {
        const uint32_t u = hubs[hi];
        const int64_t rb = a.rp[u];
        const int64_t deg = a.rp[u + 1] - rb;
        const uint32_t d = a.vcom[u];
        if (threadIdx.x == 0) s_any = a.vaff[u] != 0;
        __syncthreads();
        if (!s_any) {
            bool any = false;
            for (int64_t i = threadIdx.x; i < deg; i += blockDim.x) {
                const int32_t v = a.col[rb + i];
                any = any || (v >= a.P && v < (int64_t)u && prev_mover(a, v));
            }
            if (any) atomicOr(&s_any, 1);
        }
        __syncthreads();
        if (!s_any) {
            if (threadIdx.x == 0) record(a, u, 0, d, 0.0);
            __syncthreads();
            continue;
        }
        uint32_t H = 1024;
        while ((int64_t)H < 2 * deg) H <<= 1;
        uint32_t *tk, *tv;
        if (H <= (uint32_t)kHubSmemSlots) { tk = sm; tv = sm + kHubSmemSlots; }
        else { tk = gkeys + (int64_t)blockIdx.x * gcap; tv = gvals + (int64_t)blockIdx.x * gcap; }
        const uint32_t mask = H - 1;
        for (uint32_t i = threadIdx.x; i < H; i += blockDim.x) { tk[i] = kNone; tv[i] = 0; }
        __syncthreads();
        for (int64_t base = 0; base < deg; base += blockDim.x) {
            uint32_t c = kNone;
            if (base + threadIdx.x < deg) {
                const int32_t v = a.col[rb + base + threadIdx.x];
                if (v != (int32_t)u) c = comm_at(a, v, u);
            }
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, c);
            if (c != kNone && lane == __ffs(peers) - 1) table_add(tk, tv, mask, c, (uint32_t)__popc(peers));
        }
        __syncthreads();
        if (threadIdx.x == 0) s_kud = table_get(tk, tv, mask, d);
        __syncthreads();
        const double kud = (double)s_kud, ku = (double)deg;
        const double sd = (double)sigma_at(a, d, u);
        double best_d = 0.0;
        uint32_t best_c = kNone;
        for (uint32_t i = threadIdx.x; i < H; i += blockDim.x) {
            const uint32_t c = tk[i];
            if (c == kNone || c == d) continue;
            const double sc = (double)sigma_at(a, c, u);
            const double dl = delta_q((double)tv[i], kud, ku, sc, sd, a.M, a.R);
            if (dl > 0.0 && better(dl, c, best_d, best_c)) { best_d = dl; best_c = c; }
        }
        warp_argmax(best_d, best_c);
        if (lane == 0) { red_d[w] = best_d; red_c[w] = best_c; }
        __syncthreads();
        if (w == 0) {
            best_d = lane < (int)(blockDim.x / 32) ? red_d[lane] : 0.0;
            best_c = lane < (int)(blockDim.x / 32) ? red_c[lane] : kNone;
            warp_argmax(best_d, best_c);
            if (lane == 0) {
                if (best_d > 0.0 && best_c != kNone && best_c != d) record(a, u, 1, best_c, best_d);
                else record(a, u, 1, d, 0.0);
            }
        }
        __syncthreads();
    }
}

// Event emission: two slots per window vertex (old, new), padding key = TS.
__global__ void k_exact_events(const int64_t* __restrict__ rp, const uint32_t* __restrict__ vcom,
                               const uint32_t* __restrict__ pbest, const uint8_t* __restrict__ pact, int64_t P,
                               int64_t E, int64_t B, uint32_t* __restrict__ hkey, uint32_t hmask,
                               uint32_t* __restrict__ ekey, uint32_t* __restrict__ eidx, uint32_t* __restrict__ etime,
                               long long* __restrict__ eval) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < B; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t w = P + i;
        uint32_t k0 = hmask + 1, k1 = hmask + 1;
        if (w < E && pact[w] == 1 && pbest[w] != vcom[w]) {
            const long long deg = (long long)(rp[w + 1] - rp[w]);
            const uint32_t cs[2] = {vcom[w], pbest[w]};
            uint32_t ks[2];
            for (int j = 0; j < 2; ++j) {
                uint32_t h = slot_hash(cs[j]) & hmask;
                while (true) {
                    const uint32_t prev = atomicCAS(&hkey[h], kNone, cs[j]);
                    if (prev == kNone || prev == cs[j]) break;
                    h = (h + 1) & hmask;
                }
                ks[j] = h;
            }
            k0 = ks[0];
            k1 = ks[1];
            eval[2 * i] = -deg;
            eval[2 * i + 1] = deg;
        } else {
            eval[2 * i] = 0;
            eval[2 * i + 1] = 0;
        }
        ekey[2 * i] = k0;
        ekey[2 * i + 1] = k1;
        eidx[2 * i] = (uint32_t)(2 * i);
        eidx[2 * i + 1] = (uint32_t)(2 * i + 1);
        etime[2 * i] = (uint32_t)w;
        etime[2 * i + 1] = (uint32_t)w;
    }
}

// After the stable sort by slot: gather times/deltas, segment bounds.
__global__ void k_exact_segments(const uint32_t* __restrict__ skey, const uint32_t* __restrict__ sidx,
                                 const uint32_t* __restrict__ etime, const long long* __restrict__ eval, int64_t m,
                                 uint32_t TS, uint32_t* __restrict__ stime, long long* __restrict__ sval,
                                 int32_t* __restrict__ sstart, int32_t* __restrict__ send) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t s = skey[i];
        stime[i] = etime[sidx[i]];
        sval[i] = eval[sidx[i]];
        if (s >= TS) continue;
        if (i == 0 || skey[i - 1] != s) sstart[s] = (int32_t)i;
        if (i == m - 1 || skey[i + 1] != s) send[s] = (int32_t)(i + 1);
    }
}

// Inclusive prefix within each slot from a global exclusive scan X of sval.
__global__ void k_exact_prefix(const uint32_t* __restrict__ skey, const long long* __restrict__ sval,
                               const int64_t* __restrict__ X, const int32_t* __restrict__ sstart, int64_t m,
                               uint32_t TS, long long* __restrict__ epre) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t s = skey[i];
        if (s >= TS) continue;
        epre[i] = X[i] + sval[i] - X[sstart[s]];
    }
}

// Commit [P, x]: totals and communities of movers; processed flags cleared.
__global__ void k_exact_commit_a(const int64_t* __restrict__ rp, uint32_t* __restrict__ vcom,
                                 unsigned long long* __restrict__ ctot, uint8_t* __restrict__ vaff,
                                 const uint32_t* __restrict__ nbest, const uint8_t* __restrict__ nact,
                                 const double* __restrict__ ndelta, double* __restrict__ final_delta, int64_t P,
                                 int64_t x) {
    for (int64_t u = P + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u <= x; u += (int64_t)gridDim.x * blockDim.x) {
        double dl = 0.0;
        if (nact[u] == 1 && nbest[u] != vcom[u]) {
            const long long deg = (long long)(rp[u + 1] - rp[u]);
            atomicAdd(&ctot[vcom[u]], (unsigned long long)(-deg));
            atomicAdd(&ctot[nbest[u]], (unsigned long long)deg);
            dl = ndelta[u];
        }
        final_delta[u] = dl;
        vaff[u] = 0;
    }
}

// Affected flags set by the committed movers: every neighbour outside [P, x]
// and every neighbour in [P, x] processed before the mover.
__global__ void k_exact_commit_b(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                 uint32_t* __restrict__ vcom, uint8_t* __restrict__ vaff,
                                 const uint32_t* __restrict__ nbest, const uint8_t* __restrict__ nact, int64_t P,
                                 int64_t x) {
    const int lane = threadIdx.x & 31;
    const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = P + wid; w <= x; w += nw) {
        if (!(nact[w] == 1 && nbest[w] != vcom[w])) continue;
        for (int64_t e = rp[w] + lane; e < rp[w + 1]; e += 32) {
            const int32_t v = col[e];
            if (v < P || v > x || v < w) vaff[v] = 1;
        }
    }
}

__global__ void k_exact_commit_c(uint32_t* __restrict__ vcom, const uint32_t* __restrict__ nbest,
                                 const uint8_t* __restrict__ nact, int64_t P, int64_t x) {
    for (int64_t u = P + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u <= x; u += (int64_t)gridDim.x * blockDim.x)
        if (nact[u] == 1) vcom[u] = nbest[u];
}

__global__ void k_exact_mark_unknown(uint8_t* __restrict__ pact, int64_t a, int64_t b) {
    for (int64_t u = a + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < b; u += (int64_t)gridDim.x * blockDim.x)
        pact[u] = kUnknown;
}

// Deterministic tree sum of the iteration's committed deltas (and count).
__global__ void k_sum_deltas(const double* __restrict__ d, int64_t n, double* __restrict__ partial,
                             unsigned long long* __restrict__ cnt) {
    double s = 0.0;
    unsigned long long c = 0;
    const int64_t per = (n + gridDim.x - 1) / gridDim.x;
    const int64_t b = blockIdx.x * per, e = min(n, b + per);
    // fixed per-thread strided order inside the block's fixed range
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

template <typename T>
T read_dev(const T* p, cudaStream_t s) {
    T h;
    GB_CUDA(cudaMemcpyAsync(&h, p, sizeof(T), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    return h;
}

}  // namespace

int local_move_exact(const LocalMoveContext& ctx, double tolerance, int max_iterations, int64_t window,
                     cudaStream_t s, int64_t* launches, int64_t* rounds_out) {
    const int64_t n = ctx.g.n;
    const int64_t B = std::max<int64_t>(32, std::min<int64_t>(window, n));
    const int64_t m = 2 * B;
    uint32_t TS = 1024;
    while ((int64_t)TS < 2 * m) TS <<= 1;
    const int sort_bits = bits_for(TS);

    DevBuf<uint32_t> pbest(n, s), nbest(n, s);
    DevBuf<uint8_t> pact(n, s), nact(n, s);
    DevBuf<double> ndelta(n, s), final_delta(n, s);
    DevBuf<uint32_t> hkey(TS, s), ekey(m, s), eidx(m, s), etime(m, s), stime(m, s);
    DevBuf<long long> eval(m, s), sval(m, s), epre(m, s);
    DevBuf<int64_t> X(m, s);
    DevBuf<int32_t> sstart(TS, s), send(TS, s);
    DevBuf<unsigned long long> fc(1, s);
    DevBuf<double> partial(1024, s), dsum(1, s);
    DevBuf<unsigned long long> nmov(1, s);

    const int eval_smem = kExWarpsPerBlock * 2 * kWarpHash * (int)sizeof(uint32_t);
    GB_CUDA(cudaFuncSetAttribute(k_exact_eval_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, eval_smem));
    const int hub_smem = 2 * kHubSmemSlots * (int)sizeof(uint32_t);
    GB_CUDA(cudaFuncSetAttribute(k_exact_eval_hub, cudaFuncAttributeMaxDynamicSharedMemorySize, hub_smem));

    int iterations = 0;
    int64_t rounds = 0, nl = 0;
    uint32_t* pb = pbest.get();
    uint32_t* nb = nbest.get();
    uint8_t* pa = pact.get();
    uint8_t* na = nact.get();
    for (int it = 0; it < max_iterations; ++it) {
        int64_t P = 0;
        int64_t E = std::min(n, P + B);
        k_exact_mark_unknown<<<grid_for(E, kT), kT, 0, s>>>(pa, 0, E);
        GB_LAUNCH_CHECK();
        ++nl;
        size_t hcur = 0;
        while (P < n) {
            ++rounds;
            // Event table from D_prev.
            GB_CUDA(cudaMemsetAsync(hkey, 0xFF, TS * sizeof(uint32_t), s));
            k_exact_events<<<grid_for(B, kT), kT, 0, s>>>(ctx.g.row_ptr, ctx.vcom, pb, pa, P, E, B, hkey, TS - 1,
                                                         ekey, eidx, etime, eval);
            GB_LAUNCH_CHECK();
            radix_sort_pairs_u32(ekey, eidx, m, sort_bits, s);
            k_exact_segments<<<grid_for(m, kT), kT, 0, s>>>(ekey, eidx, etime, eval, m, TS, stime, sval, sstart,
                                                           send);
            GB_LAUNCH_CHECK();
            exclusive_scan_i64(reinterpret_cast<const int64_t*>(sval.get()), X, m, s);
            k_exact_prefix<<<grid_for(m, kT), kT, 0, s>>>(ekey, sval, X, sstart, m, TS, epre);
            GB_LAUNCH_CHECK();
            // Evaluate the window.
            GB_CUDA(cudaMemsetAsync(fc, 0xFF, sizeof(unsigned long long), s));
            ExactArgs a{ctx.g.row_ptr, ctx.g.col, ctx.vcom, ctx.ctot, ctx.vaff, pb, pa, nb, na, ndelta,
                        hkey, TS - 1, sstart, send, stime, epre, P, E, ctx.M, ctx.R, fc};
            const int grid = (int)std::min<int64_t>(ceil_div(E - P, kExWarpsPerBlock), (int64_t)kNumSMs * 16);
            k_exact_eval_warp<<<grid, kExWarpsPerBlock * 32, eval_smem, s>>>(a);
            GB_LAUNCH_CHECK();
            while (hcur < ctx.hubs_h.size() && (int64_t)ctx.hubs_h[hcur] < P) ++hcur;
            size_t hend = hcur;
            while (hend < ctx.hubs_h.size() && (int64_t)ctx.hubs_h[hend] < E) ++hend;
            if (hend > hcur) {
                const int hg = (int)std::min<size_t>(hend - hcur, (size_t)ctx.hub_grid);
                k_exact_eval_hub<<<hg, kHubThreads, hub_smem, s>>>(a, ctx.hubs, (int64_t)hcur, (int64_t)hend,
                                                                   ctx.hub_gk, ctx.hub_gv, ctx.hub_gcap);
                GB_LAUNCH_CHECK();
                ++nl;
            }
            const unsigned long long first = read_dev(fc.get(), s);
            const int64_t x = (first == ~0ull) ? E - 1 : (int64_t)first;
            // Commit [P, x].
            k_exact_commit_a<<<grid_for(x - P + 1, kT), kT, 0, s>>>(ctx.g.row_ptr, ctx.vcom, ctx.ctot, ctx.vaff,
                                                                   nb, na, ndelta, final_delta, P, x);
            GB_LAUNCH_CHECK();
            k_exact_commit_b<<<grid_for((x - P + 1) * 32, kT), kT, 0, s>>>(ctx.g.row_ptr, ctx.g.col, ctx.vcom,
                                                                           ctx.vaff, nb, na, P, x);
            GB_LAUNCH_CHECK();
            k_exact_commit_c<<<grid_for(x - P + 1, kT), kT, 0, s>>>(ctx.vcom, nb, na, P, x);
            GB_LAUNCH_CHECK();
            nl += 9 + 3 * ((sort_bits + 7) / 8) + 3;
            // Slide: new decisions become D_prev; vertices entering are unknown.
            std::swap(pb, nb);
            std::swap(pa, na);
            const int64_t newP = x + 1;
            const int64_t newE = std::min(n, newP + B);
            if (newE > E) {
                k_exact_mark_unknown<<<grid_for(newE - E, kT), kT, 0, s>>>(pa, E, newE);
                GB_LAUNCH_CHECK();
                ++nl;
            }
            P = newP;
            E = newE;
        }
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
    if (launches) *launches += nl;
    if (rounds_out) *rounds_out += rounds;
    return iterations;
}

}  // namespace gb
