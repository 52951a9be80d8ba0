// api_ext.cu -- C ABI of the timed graph kernels, the DBG arm, Tier-0 features
// and the selector MLP (include/gbgpu.h).
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "gb_common.cuh"
#include "gb_selector.h"
#include "gb_stages.h"
#include "gbgpu.h"

cudaStream_t gb_ctx_stream(gbgpu_ctx* ctx);
int gb_ctx_device(gbgpu_ctx* ctx);
void gb_ctx_set_error(gbgpu_ctx* ctx, const char* msg);

namespace {

using gb::DevBuf;

template <typename F>
int guarded_ext(gbgpu_ctx* ctx, F&& f) {
    try {
        GB_CUDA(cudaSetDevice(gb_ctx_device(ctx)));
        f(gb_ctx_stream(ctx));
        gb_ctx_set_error(ctx, "");
        return GBGPU_OK;
    } catch (const gb::Error& e) {
        gb_ctx_set_error(ctx, e.what());
        return e.status;
    } catch (const std::exception& e) {
        gb_ctx_set_error(ctx, e.what());
        return GBGPU_E_INVALID;
    }
}

bool dev(uint32_t flags) { return (flags & GBGPU_DEVICE_POINTERS) != 0; }

// Device view of a graph (copies host arrays).
struct Resident {
    gb::DeviceCSR g;
    DevBuf<int64_t> rp;
    DevBuf<int32_t> col;
    Resident(const int64_t* row_ptr, const int32_t* c, int64_t n, int64_t nnz, uint32_t flags, cudaStream_t s) {
        GB_REQUIRE(n >= 0 && nnz >= 0 && row_ptr, GBGPU_E_INVALID, "bad graph arguments");
        g.n = n;
        g.nnz = nnz;
        if (dev(flags)) {
            g.row_ptr = row_ptr;
            g.col = c;
        } else {
            rp.alloc(n + 1, s);
            col.alloc(nnz > 0 ? nnz : 1, s);
            GB_CUDA(cudaMemcpyAsync(rp.get(), row_ptr, (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s));
            if (nnz) GB_CUDA(cudaMemcpyAsync(col.get(), c, nnz * sizeof(int32_t), cudaMemcpyHostToDevice, s));
            g.row_ptr = rp.get();
            g.col = col.get();
        }
        gb::check_graph_device(g, s);
    }
};

template <typename T>
struct OutBuf {
    T* user;
    T* d;
    int64_t count;
    bool host;
    DevBuf<T> buf;
    OutBuf(T* u, int64_t cnt, uint32_t flags, cudaStream_t s) : user(u), d(u), count(cnt), host(!dev(flags)) {
        if (host) {
            buf.alloc(cnt > 0 ? cnt : 1, s);
            d = buf.get();
        }
    }
    void finish(cudaStream_t s) {
        if (host && count > 0 && user)
            GB_CUDA(cudaMemcpyAsync(user, d, count * sizeof(T), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaStreamSynchronize(s));
    }
};

template <typename T>
const T* in_dev(const T* p, int64_t count, uint32_t flags, DevBuf<T>& tmp, cudaStream_t s) {
    if (dev(flags)) return p;
    tmp.alloc(count > 0 ? count : 1, s);
    if (count) GB_CUDA(cudaMemcpyAsync(tmp.get(), p, count * sizeof(T), cudaMemcpyHostToDevice, s));
    return tmp.get();
}

}  // namespace

extern "C" {

int gbgpu_selfcheck_delta(gbgpu_ctx* ctx, double M, double R, int64_t count, uint64_t seed, int64_t* mismatches) {
    if (!ctx || !mismatches) return GBGPU_E_INVALID;
    return guarded_ext(ctx, [&](cudaStream_t s) { *mismatches = gb::selfcheck_delta_device(M, R, count, seed, s); });
}

int gbgpu_pagerank(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz,
                   int32_t max_iters, double epsilon, float* scores_out, int32_t* iters_out, double* ms_out,
                   uint32_t flags) {
    if (!ctx) return GBGPU_E_INVALID;
    return guarded_ext(ctx, [&](cudaStream_t s) {
        Resident r(row_ptr, col, n, nnz, flags, s);
        OutBuf<float> out(scores_out, n, flags, s);
        int it = 0;
        const double ms = gb::pagerank_device(r.g, max_iters, epsilon, out.d, &it, s);
        out.finish(s);
        if (iters_out) *iters_out = it;
        if (ms_out) *ms_out = ms;
    });
}

int gbgpu_bfs(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz, int64_t source,
              int32_t* depth_out, double* ms_out, uint32_t flags) {
    if (!ctx) return GBGPU_E_INVALID;
    return guarded_ext(ctx, [&](cudaStream_t s) {
        Resident r(row_ptr, col, n, nnz, flags, s);
        OutBuf<int32_t> out(depth_out, n, flags, s);
        const double ms = gb::bfs_device(r.g, source, out.d, s);
        out.finish(s);
        if (ms_out) *ms_out = ms;
    });
}

int gbgpu_connected_components(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n,
                               int64_t nnz, int32_t* comp_out, double* ms_out, uint32_t flags) {
    if (!ctx) return GBGPU_E_INVALID;
    return guarded_ext(ctx, [&](cudaStream_t s) {
        Resident r(row_ptr, col, n, nnz, flags, s);
        OutBuf<int32_t> out(comp_out, n, flags, s);
        const double ms = gb::cc_device(r.g, out.d, s);
        out.finish(s);
        if (ms_out) *ms_out = ms;
    });
}

int gbgpu_dbg_mapping(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz,
                      int32_t* new_ids_out, double* ms_out, uint32_t flags) {
    if (!ctx) return GBGPU_E_INVALID;
    return guarded_ext(ctx, [&](cudaStream_t s) {
        Resident r(row_ptr, col, n, nnz, flags, s);
        OutBuf<int32_t> out(new_ids_out, n, flags, s);
        const double ms = gb::dbg_mapping_device(r.g, out.d, s);
        out.finish(s);
        if (ms_out) *ms_out = ms;
    });
}

int gbgpu_tier0_features(gbgpu_ctx* ctx, const int64_t* row_ptr, const int32_t* col, int64_t n, int64_t nnz,
                         double* features_out, uint32_t flags) {
    if (!ctx || !features_out) return GBGPU_E_INVALID;
    return guarded_ext(ctx, [&](cudaStream_t s) {
        Resident r(row_ptr, col, n, nnz, flags, s);
        gb::tier0_features_device(r.g, features_out, s);
    });
}

int gbgpu_mlp_param_count(int32_t in_dim) { return in_dim > 0 ? gb::mlp_param_count(in_dim) : 0; }

int gbgpu_mlp_forward(gbgpu_ctx* ctx, const float* params, const float* X, int32_t rows, int32_t in_dim, float* Y,
                      uint32_t flags) {
    if (!ctx || rows < 0 || in_dim <= 0) return GBGPU_E_INVALID;
    return guarded_ext(ctx, [&](cudaStream_t s) {
        if (rows == 0) return;
        DevBuf<float> tp, tx, h1((int64_t)rows * gb::kMlpHidden, s), h2((int64_t)rows * gb::kMlpHidden, s);
        const float* p = in_dev(params, gb::mlp_param_count(in_dim), flags, tp, s);
        const float* x = in_dev(X, (int64_t)rows * in_dim, flags, tx, s);
        OutBuf<float> y(Y, (int64_t)rows * gb::kMlpOut, flags, s);
        gb::mlp_forward_device(p, x, rows, in_dim, y.d, h1, h2, s);
        y.finish(s);
    });
}

int gbgpu_mlp_gradient(gbgpu_ctx* ctx, const float* params, const float* X, const float* T, int32_t rows,
                       int32_t in_dim, float* grad_out, float* loss_out, uint32_t flags) {
    if (!ctx || rows <= 0 || in_dim <= 0) return GBGPU_E_INVALID;
    return guarded_ext(ctx, [&](cudaStream_t s) {
        DevBuf<float> tp, tx, tt;
        const int P = gb::mlp_param_count(in_dim);
        const float* p = in_dev(params, P, flags, tp, s);
        const float* x = in_dev(X, (int64_t)rows * in_dim, flags, tx, s);
        const float* t = in_dev(T, (int64_t)rows * gb::kMlpOut, flags, tt, s);
        OutBuf<float> g(grad_out, P, flags, s);
        const float loss = gb::mlp_grad_device(p, x, t, rows, in_dim, g.d, s);
        g.finish(s);
        if (loss_out) *loss_out = loss;
    });
}

int gbgpu_mlp_train(gbgpu_ctx* ctx, float* params_inout, const float* X, const float* T, int32_t rows,
                    int32_t in_dim, int32_t epochs, int32_t batch, float lr, uint64_t seed, float* loss_out,
                    uint32_t flags) {
    if (!ctx || rows <= 0 || in_dim <= 0 || epochs < 0 || batch <= 0) return GBGPU_E_INVALID;
    return guarded_ext(ctx, [&](cudaStream_t s) {
        const int P = gb::mlp_param_count(in_dim);
        DevBuf<float> tx, tt, tp;
        const float* x = in_dev(X, (int64_t)rows * in_dim, flags, tx, s);
        const float* t = in_dev(T, (int64_t)rows * gb::kMlpOut, flags, tt, s);
        float* p = params_inout;
        if (!dev(flags)) {
            tp.alloc(P, s);
            GB_CUDA(cudaMemcpyAsync(tp.get(), params_inout, P * sizeof(float), cudaMemcpyHostToDevice, s));
            p = tp.get();
        }
        const float loss = gb::mlp_train_device(p, x, t, rows, in_dim, epochs, batch, lr, seed, s);
        if (!dev(flags)) GB_CUDA(cudaMemcpyAsync(params_inout, p, P * sizeof(float), cudaMemcpyDeviceToHost, s));
        GB_CUDA(cudaStreamSynchronize(s));
        if (loss_out) *loss_out = loss;
    });
}

}  // extern "C"
