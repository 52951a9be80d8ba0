// relabel.cu -- permutation validation and CSR relabel on the device.
//
// Validation follows BuilderBase::ValidatePermutationOrThrow
// (bench/include/external/gapbs/builder.h:2056-2080): the reported failure is
// the one the reference's in-order scan would meet first (an out-of-range id
// or the second occurrence of a repeated id).  The same pass produces the
// inverse permutation, which the relabel uses.
//
// Relabel follows RelabelByMapping's undirected branch (builder.h:1168-1206):
// new row x = sorted { new_ids[v] : v in N(old(x)) }.  Remap and sort are
// fused per row; rows are bucketed by length: one thread (<= 16 entries),
// one warp with a shared-memory bitonic sort (<= 256), one 256-thread CTA
// (<= 2048) or one 1024-thread CTA (<= 16384) with a shared-memory LSD radix
// sort, and a global radix sort of (row, new id) keys for the few longer
// rows.  The three middle classes run concurrently on forked streams.
#include "gb_common.cuh"
#include "gb_stages.h"

namespace gb {

namespace {

constexpr int32_t kIntMax = 0x7FFFFFFF;

__global__ void k_first_index(const int32_t* __restrict__ ids, int64_t n, int32_t* __restrict__ first,
                              int64_t* __restrict__ oor_min) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = ids[i];
        if (v < 0 || (int64_t)v >= n) {
            atomicMin((unsigned long long*)oor_min, (unsigned long long)i);
        } else {
            atomicMin(&first[v], (int32_t)i);
        }
    }
}

__global__ void k_dup_index(const int32_t* __restrict__ ids, int64_t n, const int32_t* __restrict__ first,
                            int64_t* __restrict__ dup_min) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = ids[i];
        if (v >= 0 && (int64_t)v < n && first[v] != (int32_t)i)
            atomicMin((unsigned long long*)dup_min, (unsigned long long)i);
    }
}

__global__ void k_new_degrees(const int64_t* __restrict__ rp, const int32_t* __restrict__ inv, int64_t n,
                              int64_t* __restrict__ deg_new) {
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = inv[x];
        deg_new[x] = rp[u + 1] - rp[u];
    }
}

constexpr int kThreadRowMax = 16;
constexpr int kWarpRowMax = 256;
constexpr int kMidRowMax = 2048;      // 256-thread CTA, 24 KB shared memory
constexpr int kBlockRowMax = 16384;   // 1024-thread CTA, 160 KB shared memory
constexpr int kRowLists = 4;          // warp, mid-CTA, CTA, huge

__global__ void k_relabel_rows_small(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                     const int32_t* __restrict__ new_ids, const int32_t* __restrict__ inv,
                                     const int64_t* __restrict__ out_rp, int32_t* __restrict__ out_col,
                                     int64_t n, int32_t* __restrict__ lists, int32_t* __restrict__ counts) {
    // counts[0..3]: warp, mid-CTA, CTA, huge list sizes; lists: 4 x n entries.
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = inv[x];
        const int64_t b = rp[u], d = rp[u + 1] - b;
        if (d <= kThreadRowMax) {
            int32_t a[kThreadRowMax];
            for (int i = 0; i < d; ++i) {
                const int32_t v = new_ids[col[b + i]];
                int j = i - 1;
                while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; --j; }
                a[j + 1] = v;
            }
            const int64_t o = out_rp[x];
            for (int i = 0; i < d; ++i) out_col[o + i] = a[i];
        } else {
            const int which = d <= kWarpRowMax ? 0 : (d <= kMidRowMax ? 1 : (d <= kBlockRowMax ? 2 : 3));
            const int32_t slot = atomicAdd(&counts[which], 1);
            lists[(int64_t)which * n + slot] = (int32_t)x;
        }
    }
}

__global__ void k_relabel_rows_warp(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                    const int32_t* __restrict__ new_ids, const int32_t* __restrict__ inv,
                                    const int64_t* __restrict__ out_rp, int32_t* __restrict__ out_col,
                                    const int32_t* __restrict__ list, const int32_t* __restrict__ count) {
    constexpr int kWarps = 8;
    __shared__ int32_t sh[kWarps][kWarpRowMax];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int32_t* s = sh[w];
    const int32_t total = *count;
    for (int64_t r = (int64_t)blockIdx.x * kWarps + w; r < total; r += (int64_t)gridDim.x * kWarps) {
        const int32_t x = list[r];
        const int32_t u = inv[x];
        const int64_t b = rp[u];
        const int d = (int)(rp[u + 1] - b);
        int p = 32;
        while (p < d) p <<= 1;
        for (int i = lane; i < p; i += 32) s[i] = i < d ? new_ids[col[b + i]] : kIntMax;
        __syncwarp();
        for (int k = 2; k <= p; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = lane; i < p; i += 32) {
                    const int ixj = i ^ j;
                    if (ixj > i) {
                        const int32_t a = s[i], c = s[ixj];
                        const bool asc = (i & k) == 0;
                        if ((a > c) == asc) { s[i] = c; s[ixj] = a; }
                    }
                }
                __syncwarp();
            }
        }
        const int64_t o = out_rp[x];
        for (int i = lane; i < d; i += 32) out_col[o + i] = s[i];
        __syncwarp();
    }
}

// One CTA per row: remap into shared memory, then a stable LSD radix sort of
// the new ids in shared memory, 8 bits per pass.  Warp w owns the w-th
// contiguous segment of the row; a pass counts each warp's digits
// (no atomics), scans the digit-major / warp-minor counts, and
// scatters every warp's segment in order, so equal digits keep their order.
// Ranks among a warp's 32 lanes come from a ballot multisplit.
// kThreads = 256 for rows up to kMidRowMax, 1024 up to kBlockRowMax.
constexpr int kRadixBins = 256;

template <int kThreads, int kMaxRow>
constexpr int radix_row_smem() {
    return (2 * kMaxRow + kRadixBins * (kThreads / 32) * 33 / 32) * (int)sizeof(int32_t);
}

// Lanes of the warp holding the same 8-bit digit as this lane, by eight
// ballots (a multisplit; cheaper than __match_any_sync here).
__device__ __forceinline__ unsigned digit_peers8(int dig, unsigned valid) {
    unsigned p = valid;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const bool bit = (dig >> b) & 1;
        const unsigned bal = __ballot_sync(0xFFFFFFFFu, bit);
        p &= bit ? bal : ~bal;
    }
    return p;
}

// Counts are padded one word per 32 so that the scan's per-thread runs of
// consecutive entries fall on distinct banks.
__device__ __forceinline__ int hpad(int i) { return i + (i >> 5); }

template <int kThreads, int kMaxRow>
__global__ void __launch_bounds__(kThreads)
k_relabel_rows_block(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                     const int32_t* __restrict__ new_ids, const int32_t* __restrict__ inv,
                     const int64_t* __restrict__ out_rp, int32_t* __restrict__ out_col,
                     const int32_t* __restrict__ list, const int32_t* __restrict__ count, int vbits) {
    constexpr int kW = kThreads / 32;
    constexpr int kHist = kRadixBins * kW;          // H[digit * kW + warp]
    constexpr int kPer = kHist / kThreads;           // scan entries per thread
    static_assert(kHist % kThreads == 0, "scan shape");
    extern __shared__ int32_t sm[];
    int32_t* A = sm;
    int32_t* B = A + kMaxRow;
    int32_t* H = B + kMaxRow;
    __shared__ int32_t wtot[kW];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const int32_t total = *count;
    for (int64_t r = blockIdx.x; r < total; r += gridDim.x) {
        const int32_t x = list[r];
        const int32_t u = inv[x];
        const int64_t b = rp[u];
        const int d = (int)(rp[u + 1] - b);
        for (int i = t; i < d; i += kThreads) A[i] = new_ids[col[b + i]];
        const int seg = (((d + kW - 1) / kW) + 31) & ~31;
        const int lo = min(d, w * seg), hi = min(d, lo + seg);
        int32_t* src = A;
        int32_t* dst = B;
        for (int shift = 0; shift < vbits; shift += 8) {
            for (int i = t; i < kHist; i += kThreads) H[hpad(i)] = 0;
            __syncthreads();
            for (int i0 = lo; i0 < hi; i0 += 32) {
                const int i = i0 + lane;
                const int dig = i < hi ? (src[i] >> shift) & (kRadixBins - 1) : -1;
                const unsigned peers = digit_peers8(dig, __ballot_sync(0xFFFFFFFFu, dig >= 0));
                if (dig >= 0 && lane == __ffs(peers) - 1) H[hpad(dig * kW + w)] += __popc(peers);
                __syncwarp();
            }
            __syncthreads();
            // Exclusive scan of H: kPer consecutive entries per thread.
            int loc[kPer];
            int sum = 0;
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                loc[k] = H[hpad(t * kPer + k)];
                sum += loc[k];
            }
            int incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= o) incl += y;
            }
            if (lane == 31) wtot[w] = incl;
            __syncthreads();
            int run = incl - sum;
            for (int q = 0; q < w; ++q) run += wtot[q];
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                H[hpad(t * kPer + k)] = run;
                run += loc[k];
            }
            __syncthreads();
            for (int i0 = lo; i0 < hi; i0 += 32) {
                const int i = i0 + lane;
                const int32_t v = i < hi ? src[i] : 0;
                const int dig = i < hi ? (v >> shift) & (kRadixBins - 1) : -1;
                const unsigned peers = digit_peers8(dig, __ballot_sync(0xFFFFFFFFu, dig >= 0));
                if (dig >= 0) dst[H[hpad(dig * kW + w)] + __popc(peers & lt)] = v;
                __syncwarp();
                if (dig >= 0 && lane == __ffs(peers) - 1) H[hpad(dig * kW + w)] += __popc(peers);
                __syncwarp();
            }
            __syncthreads();
            int32_t* tmp = src;
            src = dst;
            dst = tmp;
        }
        const int64_t o = out_rp[x];
        for (int i = t; i < d; i += kThreads) out_col[o + i] = src[i];
        __syncthreads();
    }
}

// Long rows: keys (list index << vbits | new id) in one buffer, sorted by a
// global radix sort, then written back per row.  Both passes are
// entry-parallel (the row of an entry by binary search over the few long
// rows' offsets), so one very long row does not serialise a CTA.
__device__ __forceinline__ int32_t huge_row_of(const int64_t* __restrict__ hoff, int32_t count, int64_t i) {
    int32_t lo = 0, hi = count;   // largest r with hoff[r] <= i
    while (hi - lo > 1) {
        const int32_t mid = (lo + hi) >> 1;
        if (hoff[mid] <= i) lo = mid; else hi = mid;
    }
    return lo;
}

__global__ void k_huge_gather(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                              const int32_t* __restrict__ new_ids, const int32_t* __restrict__ inv,
                              const int32_t* __restrict__ list, const int64_t* __restrict__ hoff,
                              int32_t count, int vbits, uint64_t* __restrict__ keys) {
    const int64_t total = hoff[count];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = huge_row_of(hoff, count, i);
        const int64_t b = rp[inv[list[r]]];
        keys[i] = ((uint64_t)r << vbits) | (uint32_t)new_ids[col[b + (i - hoff[r])]];
    }
}

__global__ void k_huge_scatter(const int32_t* __restrict__ list, const int64_t* __restrict__ hoff,
                               const int64_t* __restrict__ out_rp, int32_t count, int vbits,
                               const uint64_t* __restrict__ keys, int32_t* __restrict__ out_col) {
    const uint64_t mask = (vbits >= 64) ? ~0ull : ((1ull << vbits) - 1ull);
    const int64_t total = hoff[count];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = huge_row_of(hoff, count, i);
        out_col[out_rp[list[r]] + (i - hoff[r])] = (int32_t)(keys[i] & mask);
    }
}

__global__ void k_huge_degrees(const int64_t* __restrict__ rp, const int32_t* __restrict__ inv,
                               const int32_t* __restrict__ list, int32_t count, int64_t* __restrict__ hdeg) {
    for (int32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < count; r += gridDim.x * blockDim.x) {
        const int32_t u = inv[list[r]];
        hdeg[r] = rp[u + 1] - rp[u];
    }
}

__global__ void k_set_last(int64_t* p, int64_t n, int64_t v) { p[n] = v; }

// Squished-CSR check: offsets non-decreasing from 0, neighbour ids in range,
// rows strictly increasing (sorted, no duplicates).  bad[0]: offsets,
// bad[1]: ids out of range, bad[2]: unsorted or duplicate.
// Row offsets: rp[0] == 0, non-decreasing, rp[n] == nnz.
__global__ void k_check_rows(const int64_t* __restrict__ rp, int64_t n, int64_t nnz, int32_t* __restrict__ bad) {
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u <= n; u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = rp[u];
        const bool ok = b >= 0 && b <= nnz && (u == 0 ? b == 0 : rp[u - 1] <= b) && (u != n || b == nnz);
        if (!ok) atomicOr(&bad[0], 1);
    }
}

// Neighbour ids, edge-parallel over chunks of kCheckChunk entries: the row
// starts that fall inside a chunk are marked in a shared bitmap, and every
// entry that is not a row start must exceed its predecessor.  Runs only on
// valid row offsets (bad[0] clear), so every entry lies in exactly one row.
constexpr int kCheckChunk = 4096;
constexpr int kCheckThreads = 256;

__global__ void __launch_bounds__(kCheckThreads)
k_check_cols(const int64_t* __restrict__ rp, const int32_t* __restrict__ col, int64_t n, int64_t nnz,
             int32_t* __restrict__ bad) {
    if (*(volatile int32_t*)&bad[0]) return;
    __shared__ uint32_t starts[kCheckChunk / 32];
    __shared__ int64_t s_u0;
    const int64_t chunks = (nnz + kCheckChunk - 1) / kCheckChunk;
    int range_bad = 0, order_bad = 0;
    for (int64_t c = blockIdx.x; c < chunks; c += gridDim.x) {
        const int64_t e0 = c * kCheckChunk;
        const int64_t e1 = min(nnz, e0 + kCheckChunk);
        for (int w = threadIdx.x; w < kCheckChunk / 32; w += blockDim.x) starts[w] = 0;
        if (threadIdx.x == 0) {
            // Largest u with rp[u] <= e0: the row holding entry e0.
            int64_t lo = 0, hi = n;
            while (hi - lo > 1) {
                const int64_t mid = (lo + hi) >> 1;
                if (rp[mid] <= e0) lo = mid; else hi = mid;
            }
            s_u0 = lo;
        }
        __syncthreads();
        for (int64_t u = s_u0 + threadIdx.x; u <= n; u += blockDim.x) {
            const int64_t r = rp[u];
            if (r >= e1) break;
            if (r >= e0) atomicOr(&starts[(r - e0) >> 5], 1u << ((r - e0) & 31));
        }
        __syncthreads();
        for (int64_t i = e0 + threadIdx.x; i < e1; i += blockDim.x) {
            const int32_t v = col[i];
            range_bad |= (v < 0 || (int64_t)v >= n);
            const int64_t off = i - e0;
            if (i > 0 && !((starts[off >> 5] >> (off & 31)) & 1u)) order_bad |= (col[i - 1] >= v);
        }
        __syncthreads();
    }
    if (range_bad) atomicOr(&bad[1], 1);
    if (order_bad) atomicOr(&bad[2], 1);
}

}  // namespace

void check_graph_device(const DeviceCSR& g, cudaStream_t s) {
    if (g.n == 0) return;
    DevBuf<int32_t> bad(3, s);
    GB_CUDA(cudaMemsetAsync(bad, 0, 3 * sizeof(int32_t), s));
    k_check_rows<<<grid_for(g.n + 1, 256), 256, 0, s>>>(g.row_ptr, g.n, g.nnz, bad);
    GB_LAUNCH_CHECK();
    if (g.nnz > 0) {
        k_check_cols<<<grid_for(ceil_div(g.nnz, kCheckChunk), 1), kCheckThreads, 0, s>>>(g.row_ptr, g.col, g.n,
                                                                                       g.nnz, bad);
        GB_LAUNCH_CHECK();
    }
    int32_t h[3];
    GB_CUDA(cudaMemcpyAsync(h, bad.get(), sizeof(h), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    GB_REQUIRE(!h[0], GBGPU_E_INVALID, "row offsets are not a non-decreasing sequence from 0 to nnz");
    GB_REQUIRE(!h[1], GBGPU_E_INVALID, "neighbour id out of range");
    GB_REQUIRE(!h[2], GBGPU_E_INVALID, "rows must be sorted ascending without duplicates (squished CSR)");
}

int validate_permutation_device(const int32_t* ids, int64_t n, int32_t* inv_out, cudaStream_t s,
                                int64_t* bad_index) {
    if (n == 0) return 0;
    GB_REQUIRE(n <= (int64_t)kIntMax, GBGPU_E_OVERFLOW, "graph has more vertices than int32 ids can name");
    DevBuf<int32_t> first_local;
    int32_t* first = inv_out;
    if (!first) {
        first_local.alloc(n, s);
        first = first_local.get();
    }
    DevBuf<int64_t> mins(2, s);
    fill_u32(reinterpret_cast<uint32_t*>(first), (uint32_t)kIntMax, n, s);
    fill_i64(mins, INT64_MAX, 2, s);
    k_first_index<<<grid_for(n, 256), 256, 0, s>>>(ids, n, first, mins.get());
    GB_LAUNCH_CHECK();
    k_dup_index<<<grid_for(n, 256), 256, 0, s>>>(ids, n, first, mins.get() + 1);
    GB_LAUNCH_CHECK();
    int64_t h[2];
    GB_CUDA(cudaMemcpyAsync(h, mins.get(), sizeof(h), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    if (h[0] == INT64_MAX && h[1] == INT64_MAX) return 0;
    if (h[0] < h[1]) {
        if (bad_index) *bad_index = h[0];
        return 1;
    }
    if (bad_index) *bad_index = h[1];
    return 2;
}

void relabel_csr_device(const DeviceCSR& g, const int32_t* new_ids, const int32_t* inv,
                        int64_t* out_rp, int32_t* out_col, cudaStream_t s, int64_t* launches) {
    const int64_t n = g.n;
    if (n == 0) {
        GB_CUDA(cudaMemsetAsync(out_rp, 0, sizeof(int64_t), s));
        return;
    }
    int64_t nl = 0;
    {
        DevBuf<int64_t> deg_new(n, s);
        k_new_degrees<<<grid_for(n, 256), 256, 0, s>>>(g.row_ptr, inv, n, deg_new);
        GB_LAUNCH_CHECK();
        exclusive_scan_i64(deg_new, out_rp, n, s);
        k_set_last<<<1, 1, 0, s>>>(out_rp, n, g.nnz);
        GB_LAUNCH_CHECK();
        nl += 3;
    }
    DevBuf<int32_t> lists(kRowLists * n, s);
    DevBuf<int32_t> counts(kRowLists, s);
    GB_CUDA(cudaMemsetAsync(counts, 0, kRowLists * sizeof(int32_t), s));
    k_relabel_rows_small<<<grid_for(n, 256), 256, 0, s>>>(g.row_ptr, g.col, new_ids, inv, out_rp, out_col, n,
                                                          lists, counts);
    GB_LAUNCH_CHECK();
    // The warp, 256-thread and 1,024-thread classes write disjoint rows: they
    // run concurrently on two forked streams beside s.
    struct Fork {
        cudaStream_t s1 = nullptr, s2 = nullptr;
        cudaEvent_t ev[3] = {};
        ~Fork() {
            for (cudaEvent_t e : ev)
                if (e) cudaEventDestroy(e);
            if (s1) cudaStreamDestroy(s1);
            if (s2) cudaStreamDestroy(s2);
        }
    } fk;
    GB_CUDA(cudaStreamCreateWithFlags(&fk.s1, cudaStreamNonBlocking));
    GB_CUDA(cudaStreamCreateWithFlags(&fk.s2, cudaStreamNonBlocking));
    for (cudaEvent_t& e : fk.ev) GB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    GB_CUDA(cudaEventRecord(fk.ev[0], s));
    GB_CUDA(cudaStreamWaitEvent(fk.s1, fk.ev[0], 0));
    GB_CUDA(cudaStreamWaitEvent(fk.s2, fk.ev[0], 0));
    const int vbits = bits_for((uint64_t)(n > 1 ? n - 1 : 1));
    constexpr int mid_smem = radix_row_smem<256, kMidRowMax>();
    constexpr int block_smem = radix_row_smem<1024, kBlockRowMax>();
    GB_CUDA(cudaFuncSetAttribute(k_relabel_rows_block<1024, kBlockRowMax>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, block_smem));
    k_relabel_rows_block<1024, kBlockRowMax><<<kNumSMs, 1024, block_smem, fk.s2>>>(
        g.row_ptr, g.col, new_ids, inv, out_rp, out_col, lists.get() + 2 * n, counts.get() + 2, vbits);
    GB_LAUNCH_CHECK();
    k_relabel_rows_block<256, kMidRowMax><<<kNumSMs * 8, 256, mid_smem, fk.s1>>>(
        g.row_ptr, g.col, new_ids, inv, out_rp, out_col, lists.get() + n, counts.get() + 1, vbits);
    GB_LAUNCH_CHECK();
    k_relabel_rows_warp<<<kNumSMs * 8, 256, 0, s>>>(g.row_ptr, g.col, new_ids, inv, out_rp, out_col, lists.get(),
                                                    counts.get());
    GB_LAUNCH_CHECK();
    GB_CUDA(cudaEventRecord(fk.ev[1], fk.s1));
    GB_CUDA(cudaEventRecord(fk.ev[2], fk.s2));
    GB_CUDA(cudaStreamWaitEvent(s, fk.ev[1], 0));
    GB_CUDA(cudaStreamWaitEvent(s, fk.ev[2], 0));
    nl += 4;
    int32_t huge = 0;
    GB_CUDA(cudaMemcpyAsync(&huge, counts.get() + 3, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    if (huge > 0) {
        const int32_t* hlist = lists.get() + 3 * n;
        DevBuf<int64_t> hoff(huge + 1, s);
        k_huge_degrees<<<grid_for(huge, 256), 256, 0, s>>>(g.row_ptr, inv, hlist, huge, hoff);
        GB_LAUNCH_CHECK();
        exclusive_scan_i64_total(hoff, hoff, huge, hoff.get() + huge, s);
        int64_t total = 0;
        GB_CUDA(cudaMemcpyAsync(&total, hoff.get() + huge, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaStreamSynchronize(s));
        const int kbits = vbits + bits_for((uint64_t)huge);
        DevBuf<uint64_t> keys(total, s);
        k_huge_gather<<<grid_for(total, 256), 256, 0, s>>>(g.row_ptr, g.col, new_ids, inv, hlist, hoff, huge, vbits,
                                                           keys);
        GB_LAUNCH_CHECK();
        radix_sort_keys_u64(keys, total, kbits, s);
        k_huge_scatter<<<grid_for(total, 256), 256, 0, s>>>(hlist, hoff, out_rp, huge, vbits, keys, out_col);
        GB_LAUNCH_CHECK();
        nl += 6 + 3 * ((kbits + 7) / 8);
    }
    if (launches) *launches += nl;
}

}  // namespace gb
