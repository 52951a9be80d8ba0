// gb_chunks.cuh -- entry-parallel sweeps over a CSR graph.
//
// A sweep splits the nnz adjacency entries into chunks of kEdgeChunk
// consecutive entries, one chunk per CTA iteration.  chunk_rows_device fills
// chunk_row[c] = the row holding entry c * kEdgeChunk (one thread per row,
// no search).  Inside the CTA, chunk_entry_rows expands that into the row of
// every entry of the chunk: the rows that start inside the chunk are
// scattered to their start offsets in shared memory and a prefix maximum
// fills the gaps.  Entries are then read in coalesced order with their row
// known, whatever the degree distribution: no warp idles on a short row and
// no long row serialises one warp.
#pragma once

#include "gb_common.cuh"

namespace gb {

constexpr int kEdgeChunk = 4096;
// One padding word per 32 entries keeps the per-thread runs of the prefix
// scan off a single bank.
constexpr int kEdgeChunkPadded = kEdgeChunk + kEdgeChunk / 32;

__device__ __forceinline__ int chunk_pad(int i) { return i + (i >> 5); }

// chunk_row has ceil(nnz / kEdgeChunk) entries.  The CSR must be valid
// (row_ptr non-decreasing from 0 to nnz).
void chunk_rows_device(const int64_t* row_ptr, int64_t n, int64_t nnz, int32_t* chunk_row, cudaStream_t s);

inline int64_t edge_chunks(int64_t nnz) { return ceil_div(nnz, kEdgeChunk); }

// srow (kEdgeChunkPadded ints of shared memory) receives, at chunk_pad(i),
// the row of entry e0 + i for i < e1 - e0.  warp_max: kThreads / 32 ints of
// shared memory.  Every thread of the CTA calls it; it ends with a barrier.
template <int kThreads>
__device__ __forceinline__ void chunk_entry_rows(const int64_t* __restrict__ rp, int64_t n, int32_t u0,
                                                 int64_t e0, int64_t e1, int32_t* srow, int32_t* warp_max) {
    static_assert(kEdgeChunk % kThreads == 0 && kThreads % 32 == 0, "chunk / CTA shape");
    constexpr int kPer = kEdgeChunk / kThreads;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    for (int i = t; i < kEdgeChunk; i += kThreads) srow[chunk_pad(i)] = -1;
    __syncthreads();
    if (t == 0) srow[0] = u0;
    // Rows after u0 begin strictly after e0; empty rows share their start
    // with the next non-empty row, which has the larger id.
    for (int64_t u = (int64_t)u0 + 1 + t; u < n; u += kThreads) {
        const int64_t r = rp[u];
        if (r >= e1) break;
        atomicMax(&srow[chunk_pad((int)(r - e0))], (int32_t)u);
    }
    __syncthreads();
    int m = -1;
#pragma unroll
    for (int k = 0; k < kPer; ++k) m = max(m, srow[chunk_pad(t * kPer + k)]);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int x = __shfl_up_sync(0xFFFFFFFFu, m, o);
        if (lane >= o) m = max(m, x);
    }
    if (lane == 31) warp_max[warp] = m;
    __syncthreads();
    int run = __shfl_up_sync(0xFFFFFFFFu, m, 1);
    if (lane == 0) run = -1;
    for (int w = 0; w < warp; ++w) run = max(run, warp_max[w]);
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        const int p = chunk_pad(t * kPer + k);
        run = max(run, srow[p]);
        srow[p] = run;
    }
    __syncthreads();
}

}  // namespace gb
