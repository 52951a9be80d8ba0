// kernels.cu -- the graph kernels timed after a mapping, and the DBG arm.
//
// "Map + kernel" end-to-end time (README.md:127-129 of the reference) is the
// mapping plus r runs of a benchmark kernel on the relabelled graph.  These are
// the GPU counterparts of the reference's timed consumers:
//   PageRank, pull form with damping 0.85 (bench/src/pr.cc:40-90), Jacobi
//     sweeps until the L1 change falls below epsilon or max_iters;
//   BFS depths from a source, direction-optimising (bench/src/bfs.cc);
//   connected components as minimum vertex id per component (bench/src/cc.cc);
// and the selector's fallback arm, DBG (algorithm 5,
// bench/include/graphbrew/reorder/reorder_hub.h:267-342): vertices grouped
// into 8 degree buckets (avg/2, avg, 2avg .. 32avg, inf), highest bucket
// first, vertex-id order inside a bucket -- the order the reference's static
// OpenMP schedule produces for any thread count.
#include <algorithm>
#include <vector>

#include "gb_common.cuh"
#include "gb_stages.h"

namespace gb {

namespace {

constexpr int kT = 256;

__global__ void k_pr_init(const int64_t* __restrict__ rp, int64_t n, float init, float* __restrict__ score,
                          float* __restrict__ contrib) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t d = rp[v + 1] - rp[v];
        score[v] = init;
        contrib[v] = d ? init / (float)d : 0.f;
    }
}

// One Jacobi sweep, warp per vertex: score[u] = base + damp * sum contrib_in[v].
__global__ void k_pr_sweep(const int64_t* __restrict__ rp, const int32_t* __restrict__ col, int64_t n, float base,
                           float damp, const float* __restrict__ cin, float* __restrict__ cout,
                           float* __restrict__ score, double* __restrict__ err) {
    const int lane = threadIdx.x & 31;
    const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double e = 0.0;
    for (int64_t u = wid; u < n; u += nw) {
        float s = 0.f;
        const int64_t b = rp[u], end = rp[u + 1];
        for (int64_t i = b + lane; i < end; i += 32) s += cin[col[i]];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
        if (lane == 0) {
            const float ns = base + damp * s;
            e += fabsf(ns - score[u]);
            score[u] = ns;
            const int64_t d = end - b;
            cout[u] = d ? ns / (float)d : 0.f;
        }
    }
    if (lane == 0 && e != 0.0) atomicAdd(err, e);
}

// ---- BFS ----
__global__ void k_bfs_td(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                         const int32_t* __restrict__ frontier, int64_t nf, int32_t* __restrict__ depth, int32_t level,
                         int32_t* __restrict__ next, int32_t* __restrict__ nnext, unsigned long long* __restrict__ scout) {
    const int lane = threadIdx.x & 31;
    const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = wid; i < nf; i += nw) {
        const int32_t u = frontier[i];
        for (int64_t e = rp[u] + lane; e < rp[u + 1]; e += 32) {
            const int32_t v = col[e];
            if (depth[v] < 0 && atomicCAS(&depth[v], -1, level + 1) == -1) {
                next[atomicAdd(nnext, 1)] = v;
                atomicAdd(scout, (unsigned long long)(rp[v + 1] - rp[v]));
            }
        }
    }
}

__global__ void k_bfs_bu(const int64_t* __restrict__ rp, const int32_t* __restrict__ col, int64_t n,
                         int32_t* __restrict__ depth, int32_t level, int32_t* __restrict__ nnext,
                         unsigned long long* __restrict__ scout) {
    const int lane = threadIdx.x & 31;
    const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = wid; v < n; v += nw) {
        if (depth[v] >= 0) continue;
        bool hit = false;
        for (int64_t e = rp[v] + lane; e < rp[v + 1] && !hit; e += 32) hit = depth[col[e]] == level;
        if (__any_sync(0xFFFFFFFFu, hit) && lane == 0) {
            depth[v] = level + 1;
            atomicAdd(nnext, 1);
            atomicAdd(scout, (unsigned long long)(rp[v + 1] - rp[v]));
        }
    }
}

__global__ void k_bfs_collect(const int32_t* __restrict__ depth, int64_t n, int32_t level, int32_t* __restrict__ q,
                              int32_t* __restrict__ nq) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        if (depth[v] == level) q[atomicAdd(nq, 1)] = (int32_t)v;
}

// ---- connected components: hooking on minimum labels + pointer jumping ----
__global__ void k_cc_hook(const int64_t* __restrict__ rp, const int32_t* __restrict__ col, int64_t n,
                          int32_t* __restrict__ comp, int32_t* __restrict__ changed) {
    const int lane = threadIdx.x & 31;
    const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = wid; u < n; u += nw) {
        const int32_t cu = comp[u];
        for (int64_t e = rp[u] + lane; e < rp[u + 1]; e += 32) {
            const int32_t cv = comp[col[e]];
            if (cv < cu) {
                atomicMin(&comp[cu], cv);
                *changed = 1;
            } else if (cu < cv) {
                atomicMin(&comp[cv], cu);
                *changed = 1;
            }
        }
    }
}

__global__ void k_cc_jump(int64_t n, int32_t* __restrict__ comp) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        int32_t c = comp[v];
        while (comp[c] != c) c = comp[c];
        comp[v] = c;
    }
}

__global__ void k_iota_i32(int32_t* p, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = (int32_t)i;
}

// ---- DBG ----
__global__ void k_dbg_keys(const int64_t* __restrict__ rp, int64_t n, uint64_t avg, uint32_t* __restrict__ keys,
                           uint32_t* __restrict__ vals) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t d = (uint64_t)(rp[v + 1] - rp[v]);
        const uint64_t th[7] = {avg / 2, avg, avg * 2, avg * 4, avg * 8, avg * 16, avg * 32};
        int b = 7;
        for (int j = 0; j < 7; ++j)
            if (d <= th[j]) { b = j; break; }
        keys[v] = (uint32_t)(7 - b);  // highest bucket first
        vals[v] = (uint32_t)v;
    }
}

__global__ void k_scatter_rank(const uint32_t* __restrict__ order, int64_t n, int32_t* __restrict__ new_ids) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        new_ids[order[i]] = (int32_t)i;
}

float ev_ms(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

}  // namespace

double pagerank_device(const DeviceCSR& g, int max_iters, double epsilon, float* score, int* iters_out,
                       cudaStream_t s) {
    const int64_t n = g.n;
    if (n == 0) return 0.0;
    DevBuf<float> ca(n, s), cb(n, s);
    DevBuf<double> err(1, s);
    cudaEvent_t e0, e1;
    GB_CUDA(cudaEventCreate(&e0));
    GB_CUDA(cudaEventCreate(&e1));
    GB_CUDA(cudaEventRecord(e0, s));
    const float init = 1.0f / (float)n, damp = 0.85f, base = (1.0f - damp) / (float)n;
    k_pr_init<<<grid_for(n, kT), kT, 0, s>>>(g.row_ptr, n, init, score, ca);
    GB_LAUNCH_CHECK();
    float* cin = ca.get();
    float* cout = cb.get();
    int it = 0;
    for (; it < max_iters;) {
        GB_CUDA(cudaMemsetAsync(err, 0, sizeof(double), s));
        k_pr_sweep<<<grid_for(n * 32, kT), kT, 0, s>>>(g.row_ptr, g.col, n, base, damp, cin, cout, score, err);
        GB_LAUNCH_CHECK();
        std::swap(cin, cout);
        ++it;
        double h = 0.0;
        GB_CUDA(cudaMemcpyAsync(&h, err.get(), sizeof(double), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaStreamSynchronize(s));
        if (h < epsilon) break;
    }
    GB_CUDA(cudaEventRecord(e1, s));
    GB_CUDA(cudaEventSynchronize(e1));
    if (iters_out) *iters_out = it;
    const double ms = ev_ms(e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}

double bfs_device(const DeviceCSR& g, int64_t source, int32_t* depth, cudaStream_t s) {
    const int64_t n = g.n;
    if (n == 0) return 0.0;
    GB_REQUIRE(source >= 0 && source < n, GBGPU_E_INVALID, "BFS source out of range");
    DevBuf<int32_t> qa(n, s), qb(n, s), cnt(1, s);
    DevBuf<unsigned long long> scout(1, s);
    cudaEvent_t e0, e1;
    GB_CUDA(cudaEventCreate(&e0));
    GB_CUDA(cudaEventCreate(&e1));
    GB_CUDA(cudaEventRecord(e0, s));
    GB_CUDA(cudaMemsetAsync(depth, 0xFF, n * sizeof(int32_t), s));
    const int32_t zero = 0, src = (int32_t)source;
    GB_CUDA(cudaMemcpyAsync(depth + source, &zero, sizeof(int32_t), cudaMemcpyHostToDevice, s));
    GB_CUDA(cudaMemcpyAsync(qa.get(), &src, sizeof(int32_t), cudaMemcpyHostToDevice, s));
    int64_t nf = 1;
    bool bottom_up = false;
    int32_t level = 0;
    // Beamer's heuristic: go bottom-up when the frontier's edges exceed
    // nnz / 14, back to top-down when the frontier is below n / 24.
    uint64_t frontier_edges = 0;
    {
        int64_t h[2];
        GB_CUDA(cudaMemcpyAsync(h, g.row_ptr + source, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaStreamSynchronize(s));
        frontier_edges = (uint64_t)(h[1] - h[0]);
    }
    while (nf > 0) {
        GB_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t), s));
        GB_CUDA(cudaMemsetAsync(scout, 0, sizeof(unsigned long long), s));
        if (!bottom_up && frontier_edges > (uint64_t)g.nnz / 14) bottom_up = true;
        else if (bottom_up && nf < n / 24) {
            bottom_up = false;
            // rebuild the queue of the current level
            k_bfs_collect<<<grid_for(n, kT), kT, 0, s>>>(depth, n, level, qa, cnt);
            GB_LAUNCH_CHECK();
            GB_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t), s));
        }
        if (bottom_up) {
            k_bfs_bu<<<grid_for(n * 32, kT), kT, 0, s>>>(g.row_ptr, g.col, n, depth, level, cnt, scout);
        } else {
            k_bfs_td<<<grid_for(nf * 32, kT), kT, 0, s>>>(g.row_ptr, g.col, qa, nf, depth, level, qb, cnt, scout);
        }
        GB_LAUNCH_CHECK();
        int32_t hn = 0;
        unsigned long long hs = 0;
        GB_CUDA(cudaMemcpyAsync(&hn, cnt.get(), sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaMemcpyAsync(&hs, scout.get(), sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaStreamSynchronize(s));
        nf = hn;
        frontier_edges = hs;
        if (!bottom_up) std::swap(qa.ptr, qb.ptr);
        ++level;
    }
    GB_CUDA(cudaEventRecord(e1, s));
    GB_CUDA(cudaEventSynchronize(e1));
    const double ms = ev_ms(e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}

double cc_device(const DeviceCSR& g, int32_t* comp, cudaStream_t s) {
    const int64_t n = g.n;
    if (n == 0) return 0.0;
    DevBuf<int32_t> changed(1, s);
    cudaEvent_t e0, e1;
    GB_CUDA(cudaEventCreate(&e0));
    GB_CUDA(cudaEventCreate(&e1));
    GB_CUDA(cudaEventRecord(e0, s));
    k_iota_i32<<<grid_for(n, kT), kT, 0, s>>>(comp, n);
    GB_LAUNCH_CHECK();
    for (int round = 0; round < 10000; ++round) {
        GB_CUDA(cudaMemsetAsync(changed, 0, sizeof(int32_t), s));
        k_cc_hook<<<grid_for(n * 32, kT), kT, 0, s>>>(g.row_ptr, g.col, n, comp, changed);
        GB_LAUNCH_CHECK();
        k_cc_jump<<<grid_for(n, kT), kT, 0, s>>>(n, comp);
        GB_LAUNCH_CHECK();
        int32_t h = 0;
        GB_CUDA(cudaMemcpyAsync(&h, changed.get(), sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaStreamSynchronize(s));
        if (!h) break;
    }
    GB_CUDA(cudaEventRecord(e1, s));
    GB_CUDA(cudaEventSynchronize(e1));
    const double ms = ev_ms(e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}

double dbg_mapping_device(const DeviceCSR& g, int32_t* new_ids, cudaStream_t s) {
    const int64_t n = g.n;
    if (n == 0) return 0.0;
    cudaEvent_t e0, e1;
    GB_CUDA(cudaEventCreate(&e0));
    GB_CUDA(cudaEventCreate(&e1));
    GB_CUDA(cudaEventRecord(e0, s));
    DevBuf<uint32_t> keys(n, s), vals(n, s);
    k_dbg_keys<<<grid_for(n, kT), kT, 0, s>>>(g.row_ptr, n, (uint64_t)(g.nnz / n), keys, vals);
    GB_LAUNCH_CHECK();
    radix_sort_pairs_u32(keys, vals, n, 3, s);
    k_scatter_rank<<<grid_for(n, kT), kT, 0, s>>>(vals, n, new_ids);
    GB_LAUNCH_CHECK();
    GB_CUDA(cudaEventRecord(e1, s));
    GB_CUDA(cudaEventSynchronize(e1));
    const double ms = ev_ms(e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}

}  // namespace gb
