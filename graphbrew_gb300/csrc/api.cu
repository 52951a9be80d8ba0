// api.cu -- the C ABI (include/gbgpu.h).
//
// Every entry point converts library exceptions into a gbgpu_status and keeps
// the message for gbgpu_last_error(); nothing here falls back to a CPU path.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "gb_common.cuh"
#include "gb_config.h"
#include "gb_stages.h"
#include "gbgpu.h"

struct gbgpu_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string last_error;
    int64_t exact_window = 0;               // serial-order engine window (0: default)
    std::vector<gbgpu_ctx*> workers;        // batched calls: one context per worker stream
};

namespace {

using gb::DevBuf;
using gb::Error;

// Schedule of the call running on this host thread (set from its context).
thread_local int64_t tl_exact_window = 0;

template <typename F>
int guarded(gbgpu_ctx* ctx, F&& f) {
    try {
        tl_exact_window = ctx ? ctx->exact_window : 0;
        if (ctx) GB_CUDA(cudaSetDevice(ctx->device));
        f();
        if (ctx) ctx->last_error.clear();
        return GBGPU_OK;
    } catch (const Error& e) {
        if (ctx) ctx->last_error = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        if (ctx) ctx->last_error = "host allocation failed";
        return GBGPU_E_NOMEM;
    } catch (const std::exception& e) {
        if (ctx) ctx->last_error = e.what();
        return GBGPU_E_INVALID;
    }
}

bool on_device(uint32_t flags) { return (flags & GBGPU_DEVICE_POINTERS) != 0; }

// A graph made resident for one call: device pointers as given, or copies of
// host arrays.
struct ResidentGraph {
    gb::DeviceCSR csr;
    DevBuf<int64_t> rp_copy;
    DevBuf<int32_t> col_copy;
};

void make_resident(ResidentGraph& rg, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz,
                   uint32_t flags, cudaStream_t s, gbgpu_stats* st) {
    GB_REQUIRE(n >= 0 && nnz >= 0, GBGPU_E_INVALID, "negative graph size");
    GB_REQUIRE(n < (int64_t)std::numeric_limits<int32_t>::max(), GBGPU_E_OVERFLOW,
               "graph has more vertices than int32 ids can name");
    GB_REQUIRE(row_ptr != nullptr && (nnz == 0 || col != nullptr), GBGPU_E_INVALID, "graph arrays are missing");
    rg.csr.n = n;
    rg.csr.nnz = nnz;
    int64_t last = 0;
    if (on_device(flags)) {
        rg.csr.row_ptr = row_ptr;
        rg.csr.col = col;
        GB_CUDA(cudaMemcpyAsync(&last, row_ptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaStreamSynchronize(s));
    } else {
        last = row_ptr[n];
        cudaEvent_t a, b;
        GB_CUDA(cudaEventCreate(&a));
        GB_CUDA(cudaEventCreate(&b));
        GB_CUDA(cudaEventRecord(a, s));
        rg.rp_copy.alloc(n + 1, s);
        rg.col_copy.alloc(nnz > 0 ? nnz : 1, s);
        GB_CUDA(cudaMemcpyAsync(rg.rp_copy.get(), row_ptr, (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s));
        if (nnz) GB_CUDA(cudaMemcpyAsync(rg.col_copy.get(), col, nnz * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        GB_CUDA(cudaEventRecord(b, s));
        GB_CUDA(cudaEventSynchronize(b));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (st) st->h2d_ms += ms;
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        rg.csr.row_ptr = rg.rp_copy.get();
        rg.csr.col = rg.col_copy.get();
    }
    GB_REQUIRE(last == nnz, GBGPU_E_INVALID, "row_ptr[n] does not equal nnz");
    gb::check_graph_device(rg.csr, s);
    if (st) st->kernel_launches += 1;
}

template <typename T>
void copy_out(T* dst_host_or_dev, const T* src_dev, int64_t count, uint32_t flags, cudaStream_t s,
              gbgpu_stats* st) {
    if (count <= 0) return;
    if (on_device(flags)) {
        if (dst_host_or_dev != src_dev)
            GB_CUDA(cudaMemcpyAsync(dst_host_or_dev, src_dev, count * sizeof(T), cudaMemcpyDeviceToDevice, s));
        return;
    }
    cudaEvent_t a, b;
    GB_CUDA(cudaEventCreate(&a));
    GB_CUDA(cudaEventCreate(&b));
    GB_CUDA(cudaEventRecord(a, s));
    GB_CUDA(cudaMemcpyAsync(dst_host_or_dev, src_dev, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaEventRecord(b, s));
    GB_CUDA(cudaEventSynchronize(b));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (st) st->d2h_ms += ms;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
}

gb::Config parse_checked(const char* opts, double auto_resolution) {
    gb::Config c = gb::parse_cli(gb::split_tokens(opts ? opts : ""), auto_resolution);
    return c;
}

void require_gpu_path(const gb::Config& c) {
    const std::string why = gb::gpu_unsupported_reason(c);
    GB_REQUIRE(why.empty(), GBGPU_E_UNSUPPORTED, why);
}

gb::LeidenParams leiden_params(const gb::Config& c) {
    gb::LeidenParams p;
    p.resolution = c.resolution;
    p.tolerance = c.tolerance;
    p.aggregation_tolerance = c.aggregationTolerance;
    p.tolerance_drop = c.toleranceDrop;
    p.max_iterations = c.maxIterations;
    p.max_passes = c.maxPasses;
    p.total_edges_m = c.mComputation == gb::MComputation::TotalEdges;
    p.super_move_batch = c.superGraphMoveBatch;
    p.deterministic = c.deterministicCommunityDetection;
    p.refine = c.useRefinement;
    p.refine_depth = c.refinementDepth;
    // Schedule knobs (the autotuner's choices; defaults otherwise).
    if (const char* v = std::getenv("GBGPU_EXACT_MAX_VERTICES")) p.exact_max_vertices = std::atoll(v);
    if (const char* v = std::getenv("GBGPU_EXACT_WINDOW")) p.exact_window = std::max(32LL, std::atoll(v));
    if (tl_exact_window > 0) p.exact_window = std::max<int64_t>(32, tl_exact_window);
    if (const char* v = std::getenv("GBGPU_ASYNC_CHUNK")) p.chunk_vertices = std::max(32, std::atoi(v));
    if (const char* v = std::getenv("GBGPU_ASYNC_STREAMS")) p.async_streams = std::max(0LL, std::atoll(v));
    if (const char* v = std::getenv("GBGPU_ASYNC_AUTO")) p.auto_streams = v[0] != '0';
    if (const char* v = std::getenv("GBGPU_SUPER_CLUSTER_MAX_EDGES")) p.super_single_cta_max_edges = std::atoll(v);
    if (const char* v = std::getenv("GBGPU_SUPER_SPLIT_MIN")) p.super_split_min = std::atoll(v);
    return p;
}

gb::ComposeParams compose_params(const gb::Config& c) {
    gb::ComposeParams p;
    p.community_order = static_cast<int>(c.communityOrder);
    p.intra_order = static_cast<int>(c.intraCommunityOrder);
    p.super_order = static_cast<int>(c.superGraphOrder);
    p.super_gamma = static_cast<float>(c.superGraphResolution);
    p.gorder_window = c.gorderWindow;
    p.gorder_fallback = c.gorderFallback;
    return p;
}

void fill_config(const gb::Config& c, gbgpu_config* out) {
    if (!out) return;
    out->resolution = c.resolution;
    out->tolerance = c.tolerance;
    out->aggregation_tolerance = c.aggregationTolerance;
    out->tolerance_drop = c.toleranceDrop;
    out->max_iterations = c.maxIterations;
    out->max_passes = c.maxPasses;
    out->total_edges_m = c.mComputation == gb::MComputation::TotalEdges;
    out->gve_aggregation = c.aggregation == gb::Aggregation::GveCSR;
    out->use_refinement = c.useRefinement;
    out->refinement_depth = c.refinementDepth;
    out->deterministic = c.deterministicCommunityDetection;
    out->super_move_batch = c.superGraphMoveBatch;
    out->ordering = static_cast<int>(c.ordering);
    out->super_graph_order = static_cast<int>(c.superGraphOrder);
    out->community_order = static_cast<int>(c.communityOrder);
    out->intra_order = static_cast<int>(c.intraCommunityOrder);
    out->refinement_pass = static_cast<int>(c.refinementPass);
    out->gorder_window = c.gorderWindow;
    out->gorder_fallback = c.gorderFallback;
    out->algorithm = static_cast<int>(c.algorithm);
}

float ev_ms(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

// Mapping on a resident graph; new_ids_dev is device memory.
void mapping_on_device(const gb::DeviceCSR& g, const gb::Config& c, int32_t* new_ids_dev, gbgpu_stats* st,
                       cudaStream_t s) {
    DevBuf<uint32_t> memb(g.n > 0 ? g.n : 1, s);
    gb::leiden_device(g, leiden_params(c), memb, st, s);
    gb::compose_device(g, memb, compose_params(c), new_ids_dev, st, s);
}

double resolve_auto(const gb::DeviceCSR& g, double auto_resolution, cudaStream_t s) {
    if (auto_resolution >= 0) return auto_resolution;
    return gb::auto_resolution_device(g.row_ptr, g.n, g.nnz, s);
}

}  // namespace

extern "C" {

int gbgpu_ctx_create(gbgpu_ctx** out, int device) {
    if (!out) return GBGPU_E_INVALID;
    *out = nullptr;
    gbgpu_ctx* ctx = new (std::nothrow) gbgpu_ctx();
    if (!ctx) return GBGPU_E_NOMEM;
    int rc = guarded(nullptr, [&] {
        if (device < 0) GB_CUDA(cudaGetDevice(&device));
        ctx->device = device;
        GB_CUDA(cudaSetDevice(device));
        GB_CUDA(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
        ctx->stream = ctx->own_stream;
        cudaMemPool_t pool;
        GB_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
        uint64_t threshold = std::numeric_limits<uint64_t>::max();
        GB_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold));
    });
    if (rc != GBGPU_OK) {
        delete ctx;
        return rc;
    }
    *out = ctx;
    return GBGPU_OK;
}

void gbgpu_ctx_destroy(gbgpu_ctx* ctx) {
    if (!ctx) return;
    for (gbgpu_ctx* w : ctx->workers) gbgpu_ctx_destroy(w);
    cudaSetDevice(ctx->device);
    if (ctx->own_stream) {
        cudaStreamSynchronize(ctx->own_stream);
        cudaStreamDestroy(ctx->own_stream);
    }
    delete ctx;
}

const char* gbgpu_last_error(const gbgpu_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

int gbgpu_set_stream(gbgpu_ctx* ctx, void* cuda_stream) {
    if (!ctx) return GBGPU_E_INVALID;
    ctx->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : ctx->own_stream;
    return GBGPU_OK;
}

int gbgpu_synchronize(gbgpu_ctx* ctx) {
    if (!ctx) return GBGPU_E_INVALID;
    return guarded(ctx, [&] { GB_CUDA(cudaStreamSynchronize(ctx->stream)); });
}

int gbgpu_parse_config(const char* opts, double auto_resolution, gbgpu_config* out, char* json_out,
                       size_t json_cap) {
    try {
        gb::Config c = parse_checked(opts, auto_resolution);
        fill_config(c, out);
        if (json_out && json_cap) std::snprintf(json_out, json_cap, "%s", gb::effective_config_json(c).c_str());
        return GBGPU_OK;
    } catch (const Error& e) {
        if (json_out && json_cap) std::snprintf(json_out, json_cap, "%s", e.what());
        return e.status;
    } catch (const std::exception& e) {
        if (json_out && json_cap) std::snprintf(json_out, json_cap, "%s", e.what());
        return GBGPU_E_INVALID;
    }
}

int gbgpu_auto_resolution(gbgpu_ctx* ctx, const int64_t* row_ptr, int64_t n, int64_t nnz, uint32_t flags,
                          double* out) {
    if (!ctx || !out) return GBGPU_E_INVALID;
    return guarded(ctx, [&] {
        cudaStream_t s = ctx->stream;
        DevBuf<int64_t> rp;
        const int64_t* d = row_ptr;
        if (!on_device(flags)) {
            rp.alloc(n + 1, s);
            GB_CUDA(cudaMemcpyAsync(rp.get(), row_ptr, (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s));
            d = rp.get();
        }
        *out = gb::auto_resolution_device(d, n, nnz, s);
    });
}

int gbgpu_generate_mapping(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz,
                           const char* opts, double auto_resolution, int32_t* new_ids_out, gbgpu_stats* stats,
                           uint32_t flags) {
    if (!ctx) return GBGPU_E_INVALID;
    gbgpu_stats local{};
    gbgpu_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    return guarded(ctx, [&] {
        cudaStream_t s = ctx->stream;
        GB_REQUIRE(new_ids_out != nullptr || n == 0, GBGPU_E_INVALID, "new_ids_out is missing");
        cudaEvent_t t0, t1;
        GB_CUDA(cudaEventCreate(&t0));
        GB_CUDA(cudaEventCreate(&t1));
        GB_CUDA(cudaEventRecord(t0, s));
        ResidentGraph rg;
        make_resident(rg, row_ptr, col, n, nnz, flags, s, st);
        const double ar = resolve_auto(rg.csr, auto_resolution, s);
        gb::Config c = parse_checked(opts, ar);
        require_gpu_path(c);
        if (n > 0) {
            DevBuf<int32_t> ids;
            int32_t* ids_dev = new_ids_out;
            if (!on_device(flags)) {
                ids.alloc(n, s);
                ids_dev = ids.get();
            }
            mapping_on_device(rg.csr, c, ids_dev, st, s);
            copy_out(new_ids_out, ids_dev, n, flags, s, st);
        }
        GB_CUDA(cudaEventRecord(t1, s));
        GB_CUDA(cudaEventSynchronize(t1));
        st->total_ms = ev_ms(t0, t1);
        st->resolution = c.resolution;
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
    });
}

int gbgpu_generate_mappings_batched(gbgpu_ctx* ctx, const gbgpu_graph* graphs, int32_t count, const char* opts,
                                    const gbgpu_schedule* schedule, gbgpu_stats* stats, double* wall_ms,
                                    uint32_t flags) {
    if (!ctx || count < 0 || (count > 0 && !graphs)) return GBGPU_E_INVALID;
    const int streams = schedule && schedule->streams > 0 ? std::min(schedule->streams, 64) : 4;
    const int order = schedule ? schedule->order : 1;
    const int64_t window = schedule ? schedule->exact_window : 0;
    // Worker contexts (one stream each), created once and kept by the context.
    int rc = guarded(ctx, [&] {
        while ((int)ctx->workers.size() < streams) {
            gbgpu_ctx* w = nullptr;
            const int wrc = gbgpu_ctx_create(&w, ctx->device);
            if (wrc != GBGPU_OK) throw Error(wrc, "worker context creation failed");
            ctx->workers.push_back(w);
        }
        GB_CUDA(cudaStreamSynchronize(ctx->stream));
    });
    if (rc != GBGPU_OK) return rc;
    // Order: as given, or largest graph first (longest-processing-time first
    // over the worker streams).
    std::vector<int32_t> idx(count);
    for (int32_t i = 0; i < count; ++i) idx[i] = i;
    if (order == 1)
        std::stable_sort(idx.begin(), idx.end(),
                         [&](int32_t x, int32_t y) { return graphs[x].nnz + graphs[x].n > graphs[y].nnz + graphs[y].n; });
    std::atomic<int32_t> next{0};
    std::atomic<int> first_rc{GBGPU_OK};
    std::vector<std::string> errs(streams);
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    for (int wi = 0; wi < streams; ++wi) {
        pool.emplace_back([&, wi] {
            gbgpu_ctx* w = ctx->workers[wi];
            w->exact_window = window;
            while (first_rc.load() == GBGPU_OK) {
                const int32_t k = next.fetch_add(1);
                if (k >= count) break;
                const gbgpu_graph& g = graphs[idx[k]];
                const int r = gbgpu_generate_mapping(w, g.row_ptr, g.col, g.n, g.nnz, opts, -1.0, g.new_ids_out,
                                                     stats ? &stats[idx[k]] : nullptr, flags);
                if (r != GBGPU_OK) {
                    int expect = GBGPU_OK;
                    if (first_rc.compare_exchange_strong(expect, r)) errs[wi] = w->last_error;
                }
            }
        });
    }
    for (std::thread& t : pool) t.join();
    const auto t1 = std::chrono::steady_clock::now();
    if (wall_ms) *wall_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    const int r = first_rc.load();
    if (r != GBGPU_OK) {
        for (const std::string& e : errs)
            if (!e.empty()) ctx->last_error = e;
        return r;
    }
    ctx->last_error.clear();
    return GBGPU_OK;
}

int gbgpu_leiden(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz,
                 const char* opts, double resolution, uint32_t* membership_out, gbgpu_stats* stats,
                 uint32_t flags) {
    if (!ctx) return GBGPU_E_INVALID;
    gbgpu_stats local{};
    gbgpu_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    return guarded(ctx, [&] {
        cudaStream_t s = ctx->stream;
        ResidentGraph rg;
        make_resident(rg, row_ptr, col, n, nnz, flags, s, st);
        const double ar = resolve_auto(rg.csr, resolution, s);
        gb::Config c = parse_checked(opts, ar);
        const std::string why = gb::gpu_unsupported_reason(c);
        GB_REQUIRE(why.empty(), GBGPU_E_UNSUPPORTED, why);
        if (n == 0) return;
        DevBuf<uint32_t> memb;
        uint32_t* md = membership_out;
        if (!on_device(flags)) {
            memb.alloc(n, s);
            md = memb.get();
        }
        gb::leiden_device(rg.csr, leiden_params(c), md, st, s);
        copy_out(membership_out, md, n, flags, s, st);
        GB_CUDA(cudaStreamSynchronize(s));
    });
}

int gbgpu_compose(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz,
                  const uint32_t* membership, const char* opts, int32_t* new_ids_out, gbgpu_stats* stats,
                  uint32_t flags) {
    if (!ctx) return GBGPU_E_INVALID;
    gbgpu_stats local{};
    gbgpu_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    return guarded(ctx, [&] {
        cudaStream_t s = ctx->stream;
        ResidentGraph rg;
        make_resident(rg, row_ptr, col, n, nnz, flags, s, st);
        gb::Config c = parse_checked(opts, 1.0);
        const std::string why = gb::gpu_unsupported_reason(c);
        GB_REQUIRE(why.empty(), GBGPU_E_UNSUPPORTED, why);
        if (n == 0) return;
        GB_REQUIRE(membership != nullptr && new_ids_out != nullptr, GBGPU_E_INVALID, "missing arrays");
        DevBuf<uint32_t> memb;
        const uint32_t* md = membership;
        if (!on_device(flags)) {
            memb.alloc(n, s);
            GB_CUDA(cudaMemcpyAsync(memb.get(), membership, n * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
            md = memb.get();
        }
        DevBuf<int32_t> ids;
        int32_t* ids_dev = new_ids_out;
        if (!on_device(flags)) {
            ids.alloc(n, s);
            ids_dev = ids.get();
        }
        gb::compose_device(rg.csr, md, compose_params(c), ids_dev, st, s);
        copy_out(new_ids_out, ids_dev, n, flags, s, st);
        GB_CUDA(cudaStreamSynchronize(s));
    });
}

int gbgpu_validate_permutation(gbgpu_ctx* ctx, const int32_t* new_ids, int64_t n, uint32_t flags, int32_t* result) {
    if (!ctx || !result) return GBGPU_E_INVALID;
    return guarded(ctx, [&] {
        cudaStream_t s = ctx->stream;
        DevBuf<int32_t> ids;
        const int32_t* d = new_ids;
        if (!on_device(flags) && n > 0) {
            ids.alloc(n, s);
            GB_CUDA(cudaMemcpyAsync(ids.get(), new_ids, n * sizeof(int32_t), cudaMemcpyHostToDevice, s));
            d = ids.get();
        }
        *result = gb::validate_permutation_device(d, n, nullptr, s, nullptr);
    });
}

int gbgpu_relabel_csr(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz,
                      const int32_t* new_ids, int64_t* out_row_ptr, int32_t* out_col, int32_t* org_ids_out,
                      uint32_t flags) {
    if (!ctx) return GBGPU_E_INVALID;
    return guarded(ctx, [&] {
        cudaStream_t s = ctx->stream;
        ResidentGraph rg;
        make_resident(rg, row_ptr, col, n, nnz, flags, s, nullptr);
        GB_REQUIRE(out_row_ptr != nullptr && (nnz == 0 || out_col != nullptr), GBGPU_E_INVALID, "missing outputs");
        DevBuf<int32_t> ids;
        const int32_t* idd = new_ids;
        if (!on_device(flags) && n > 0) {
            ids.alloc(n, s);
            GB_CUDA(cudaMemcpyAsync(ids.get(), new_ids, n * sizeof(int32_t), cudaMemcpyHostToDevice, s));
            idd = ids.get();
        }
        DevBuf<int32_t> inv(n > 0 ? n : 1, s);
        int64_t bad = -1;
        const int v = gb::validate_permutation_device(idd, n, inv, s, &bad);
        GB_REQUIRE(v == 0, GBGPU_E_NOT_PERMUTATION,
                   v == 1 ? "generated mapping contains an out-of-range ID"
                          : "generated mapping contains a duplicate ID");
        DevBuf<int64_t> orp;
        DevBuf<int32_t> ocol;
        int64_t* rpd = out_row_ptr;
        int32_t* cold = out_col;
        if (!on_device(flags)) {
            orp.alloc(n + 1, s);
            ocol.alloc(nnz > 0 ? nnz : 1, s);
            rpd = orp.get();
            cold = ocol.get();
        }
        gb::relabel_csr_device(rg.csr, idd, inv, rpd, cold, s, nullptr);
        copy_out(out_row_ptr, rpd, n + 1, flags, s, nullptr);
        copy_out(out_col, cold, nnz, flags, s, nullptr);
        if (org_ids_out) copy_out(org_ids_out, inv.get(), n, flags, s, nullptr);
        GB_CUDA(cudaStreamSynchronize(s));
    });
}

int gbgpu_map_and_relabel(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz,
                          const char* opts, double auto_resolution, int32_t* new_ids_out, int64_t* out_row_ptr,
                          int32_t* out_col, gbgpu_stats* stats, uint32_t flags) {
    if (!ctx) return GBGPU_E_INVALID;
    gbgpu_stats local{};
    gbgpu_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    return guarded(ctx, [&] {
        cudaStream_t s = ctx->stream;
        cudaEvent_t t0, t1, ta, tb;
        GB_CUDA(cudaEventCreate(&t0));
        GB_CUDA(cudaEventCreate(&t1));
        GB_CUDA(cudaEventCreate(&ta));
        GB_CUDA(cudaEventCreate(&tb));
        GB_CUDA(cudaEventRecord(t0, s));
        ResidentGraph rg;
        make_resident(rg, row_ptr, col, n, nnz, flags, s, st);
        const double ar = resolve_auto(rg.csr, auto_resolution, s);
        gb::Config c = parse_checked(opts, ar);
        require_gpu_path(c);
        if (n > 0) {
            DevBuf<int32_t> ids;
            int32_t* ids_dev = new_ids_out;
            if (!on_device(flags) || !new_ids_out) {
                ids.alloc(n, s);
                ids_dev = ids.get();
            }
            mapping_on_device(rg.csr, c, ids_dev, st, s);
            GB_CUDA(cudaEventRecord(ta, s));
            DevBuf<int32_t> inv(n, s);
            const int v = gb::validate_permutation_device(ids_dev, n, inv, s, nullptr);
            GB_CUDA(cudaEventRecord(tb, s));
            GB_CUDA(cudaEventSynchronize(tb));
            st->validate_ms = ev_ms(ta, tb);
            GB_REQUIRE(v == 0, GBGPU_E_NOT_PERMUTATION,
                       v == 1 ? "generated mapping contains an out-of-range ID"
                              : "generated mapping contains a duplicate ID");
            if (out_row_ptr) {
                GB_CUDA(cudaEventRecord(ta, s));
                DevBuf<int64_t> orp;
                DevBuf<int32_t> ocol;
                int64_t* rpd = out_row_ptr;
                int32_t* cold = out_col;
                bool direct = false;
                if (!on_device(flags)) {
                    orp.alloc(n + 1, s);
                    rpd = orp.get();
                    // A pinned (page-locked, device-mapped) host array takes the
                    // relabelled columns straight from the kernels over the
                    // C2C link, overlapping what would be a separate copy;
                    // pageable memory goes through a device buffer and a copy.
                    cudaPointerAttributes pa{};
                    if (nnz > 0 && cudaPointerGetAttributes(&pa, out_col) == cudaSuccess &&
                        pa.type == cudaMemoryTypeHost && pa.devicePointer) {
                        cold = static_cast<int32_t*>(pa.devicePointer);
                        direct = true;
                    } else {
                        cudaGetLastError();
                        ocol.alloc(nnz > 0 ? nnz : 1, s);
                        cold = ocol.get();
                    }
                }
                gb::relabel_csr_device(rg.csr, ids_dev, inv, rpd, cold, s, &st->kernel_launches);
                GB_CUDA(cudaEventRecord(tb, s));
                GB_CUDA(cudaEventSynchronize(tb));
                st->relabel_ms = ev_ms(ta, tb);
                copy_out(out_row_ptr, rpd, n + 1, flags, s, st);
                if (!direct) copy_out(out_col, cold, nnz, flags, s, st);
            }
            if (new_ids_out) copy_out(new_ids_out, ids_dev, n, flags, s, st);
        }
        GB_CUDA(cudaEventRecord(t1, s));
        GB_CUDA(cudaEventSynchronize(t1));
        st->total_ms = ev_ms(t0, t1);
        st->resolution = c.resolution;
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        cudaEventDestroy(ta);
        cudaEventDestroy(tb);
    });
}

}  // extern "C"

// Internal accessors for entry points defined in other translation units.
cudaStream_t gb_ctx_stream(gbgpu_ctx* ctx) { return ctx->stream; }
int gb_ctx_device(gbgpu_ctx* ctx) { return ctx->device; }
void gb_ctx_set_error(gbgpu_ctx* ctx, const char* msg) { ctx->last_error = msg ? msg : ""; }

extern "C" {

uint64_t gbgpu_fingerprint(const int32_t* new_ids, int64_t n) {
    uint64_t h = UINT64_C(1469598103934665603);
    for (int64_t i = 0; i < n; ++i) {
        h ^= (uint64_t)i;
        h *= UINT64_C(1099511628211);
        h ^= (uint64_t)(int64_t)new_ids[i];
        h *= UINT64_C(1099511628211);
    }
    return h;
}

const char* gbgpu_version(void) { return "gbgpu 0.1 (sm_103a)"; }

}  // extern "C"
