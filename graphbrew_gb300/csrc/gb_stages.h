// gb_stages.h -- internal stage entry points shared by the C ABI (api.cu).
#pragma once

#include "gb_common.cuh"

namespace gb {

// ---- relabel.cu ----
// 0 valid, 1 out-of-range, 2 duplicate.  inv_out (n entries, may be null)
// receives the inverse permutation when valid.  *bad_index: first failing index.
int validate_permutation_device(const int32_t* ids, int64_t n, int32_t* inv_out, cudaStream_t s,
                                int64_t* bad_index);
void relabel_csr_device(const DeviceCSR& g, const int32_t* new_ids, const int32_t* inv,
                        int64_t* out_rp, int32_t* out_col, cudaStream_t s, int64_t* launches);
// Rejects graphs that are not squished CSR (every kernel relies on in-range
// ids; the Gorder heap relies on duplicate-free rows).
void check_graph_device(const DeviceCSR& g, cudaStream_t s);

// ---- compose.cu ----
struct ComposeParams {
    int community_order = 0;   // CommunityOrder ordinal
    int intra_order = 4;       // IntraCommunityOrder ordinal
    int gorder_window = 8;
    int gorder_fallback = 5000;
    int super_order = 0;       // SuperGraphOrder ordinal (stage1Perm); 0 = none
    float super_gamma = 0.1f;  // superGraphResolution (sg_super_rabbit)
};
void compose_device(const DeviceCSR& g, const uint32_t* membership, const ComposeParams& p,
                    int32_t* new_ids, gbgpu_stats* st, cudaStream_t s);

// ---- compose_sorted.cu: HubSort, DegreeAsc, Hub2, Alternate, BoundaryLast, CoreOrder ----
bool is_sorted_intra_order(int intra);
// Local ids of every non-isolated vertex for a sorted intra order.  order_v /
// ranks: the placement skeleton (vertex and community rank per position, nn
// positions); offs / ssize: start and size of each ranked community.
int64_t sorted_communities(const DeviceCSR& g, const uint32_t* memb, int intra, const uint32_t* order_v,
                           const uint32_t* ranks, const int64_t* offs, const int64_t* ssize, int64_t nn,
                           uint32_t* local, cudaStream_t s, int64_t* launches);

// libstdc++'s std::sort (introsort: ties end where it leaves them) of every
// segment of (E, K) by K ascending, E moving with its key.  ranks: segment
// of each of the nn positions; offs / ssize: start and size of a segment.
void libstdcxx_sort_segments(uint32_t* E, uint64_t* K, const uint32_t* ranks, const int64_t* offs,
                             const int64_t* ssize, int64_t nn, cudaStream_t s, int64_t* launches);

// ---- compose_super.cu: sg_super_rabbit, sg_super_rcm, sg_hilbert ----
// stage1Perm of a super-graph order (SuperGraphOrder ordinal: 1 super_rabbit,
// 2 super_rcm, 4 hilbert) into stage1[C]; csize: non-isolated vertices per
// community; gamma: superGraphResolution (Rabbit).
void super_order_device(const DeviceCSR& g, const uint32_t* memb, const uint32_t* csize, int64_t C, int order,
                        float gamma, uint32_t* stage1, cudaStream_t s, int64_t* launches);

// ---- compose_random.cu: intra_random ----
// Local ids of every non-isolated vertex for intra_random: list / count_dev
// (count on the host too) are the ranks of the communities of two or more
// vertices.  Returns the number of swap rounds.
int64_t random_communities(const uint32_t* memb, const uint32_t* order_v, const uint32_t* ranks, const int64_t* offs,
                           const int64_t* ssize, const int32_t* list, const int32_t* count_dev, int32_t count,
                           int64_t nn, uint32_t* local, cudaStream_t s, int64_t* launches);

// ---- leiden.cu ----
struct LeidenParams {
    double resolution = 1.0;
    double tolerance = 1e-2;
    double aggregation_tolerance = 0.8;
    double tolerance_drop = 10.0;
    int max_iterations = 10;
    int max_passes = 10;
    bool total_edges_m = true;
    int super_move_batch = 1;
    bool deterministic = false;
    bool refine = false;            // Leiden refinement phase (RG:7330-7392)
    int refine_depth = -1;          // refinement in passes 0..refine_depth (-1: every pass)
    int chunk_vertices = 2048;      // asynchronous engine: vertices per launch
    int64_t async_streams = 0;      // asynchronous engine: > 0 = this many in-order streams (one warp each)
    bool auto_streams = true;       // cd_parallel: stream mode on large graphs whose neighbours sit at nearby ids
    int64_t auto_streams_min_vertices = 1 << 20;
    int64_t super_single_cta_max_edges = 1 << 24;  // super-move in one thread-block cluster up to this size
    int64_t super_split_min = 4096;         // batched super-move: split super-nodes above this degree over CTAs
    int64_t exact_max_vertices = INT64_MAX; // cd_parallel uses the serial-order engine up to this size
    int64_t exact_window = 65536;           // speculative window of the serial-order engine
};
void leiden_device(const DeviceCSR& g, const LeidenParams& p, uint32_t* membership, gbgpu_stats* st,
                   cudaStream_t s);

// Degree-distribution auto resolution (reorder_types.h:2743-2780).
double auto_resolution_device(const int64_t* row_ptr, int64_t n, int64_t nnz, cudaStream_t s);

// ---- kernels.cu: timed consumers and the DBG arm; each returns device ms ----
// deltaModularity with reciprocal-based exact quotients against full double
// divisions on `count` seeded inputs; returns the number of differing results.
int64_t selfcheck_delta_device(double M, double R, int64_t count, uint64_t seed, cudaStream_t s);

double pagerank_device(const DeviceCSR& g, int max_iters, double epsilon, float* score, int* iters_out,
                       cudaStream_t s);
double bfs_device(const DeviceCSR& g, int64_t source, int32_t* depth, cudaStream_t s);
double cc_device(const DeviceCSR& g, int32_t* comp, cudaStream_t s);
double dbg_mapping_device(const DeviceCSR& g, int32_t* new_ids, cudaStream_t s);

}  // namespace gb
