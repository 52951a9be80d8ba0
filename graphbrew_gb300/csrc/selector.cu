// selector.cu -- Tier-0 graph features on the device and the learned selector's MLP.
//
// Tier-0 features follow ComputeTier0SampledGraphFeatures
// (bench/include/graphbrew/reorder/reorder_types.h:6066-6186): a strided
// sample of s = clamp(sqrt(n), 1024, 8192) vertices (vertex (2i+1)n/(2s)),
// sample mean degree and coefficient of variation (n-1 denominator, summed in
// sample order like the reference), hub concentration of the top 10% of the
// sample, packing factor of the hubs over 8-vertex property lines, normalised
// edge span and window-neighbour overlap over the sampled rows.  The degree
// statistics and hub terms are summed in the reference's order, so the inputs
// of the frozen rule are exact; the span sums use a tree order.
//
// The learned selector is a float32 MLP in -> 64 -> 64 -> 3 (ReLU) predicting
// log end-to-end times of the three arms (GraphBrew algorithm 12, DBG, original
// order).  Forward, backward (mean squared error) and Adam are hand-written
// kernels with a fixed summation order per output element.
#include <algorithm>
#include <cmath>
#include <vector>

#include "gb_common.cuh"
#include "gb_selector.h"

namespace gb {

namespace {

constexpr int kSampleMax = 8192;
constexpr int kSortThreads = 1024;

struct SampleEntry {
    long long deg;
    long long node;
};

__device__ __forceinline__ bool entry_before(const SampleEntry& a, const SampleEntry& b) {
    // degree descending, vertex id ascending; padding (deg < 0) last
    if (a.deg != b.deg) return a.deg > b.deg;
    return a.node < b.node;
}

__global__ void __launch_bounds__(kSortThreads)
k_tier0(const int64_t* __restrict__ rp, const int32_t* __restrict__ col, int64_t n, int64_t nnz, int s,
        double* __restrict__ out) {
    extern __shared__ unsigned char smem_raw[];
    SampleEntry* e = reinterpret_cast<SampleEntry*>(smem_raw);
    __shared__ double s_span[kSortThreads / 32];
    __shared__ unsigned long long s_edges[kSortThreads / 32], s_window[kSortThreads / 32];
    __shared__ double s_degsum, s_avg;
    int P = 1;
    while (P < s) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        if (i < s) {
            const uint64_t node = ((2ull * (uint64_t)i + 1ull) * (uint64_t)n) / (2ull * (uint64_t)s);
            e[i].node = (long long)node;
            e[i].deg = (long long)(rp[node + 1] - rp[node]);
        } else {
            e[i].node = 0x7FFFFFFFFFFFFFFFll;
            e[i].deg = -1;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int i = 0; i < s; ++i) sum += (double)e[i].deg;
        const double avg = sum / s;
        double var = 0.0;
        for (int i = 0; i < s; ++i) {
            // explicit rounding: no fused multiply-add, as in the reference's sum
            const double d = __dsub_rn((double)e[i].deg, avg);
            var = __dadd_rn(var, __dmul_rn(d, d));
        }
        const double variance = s > 1 ? var / (s - 1) : 0.0;
        out[0] = (double)n;
        out[1] = (double)nnz;
        out[2] = avg;
        out[3] = avg > 0.0 ? sqrt(variance) / avg : 0.0;
        out[4] = n > 1 ? avg / (double)(n - 1) : 0.0;
        s_degsum = sum;
        s_avg = avg;
    }
    __syncthreads();
    // Bitonic sort of the padded sample.
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const bool asc = (i & k) == 0;
                    const SampleEntry a = e[i], b = e[ixj];
                    const bool swap = asc ? entry_before(b, a) : entry_before(a, b);
                    if (swap) { e[i] = b; e[ixj] = a; }
                }
            }
            __syncthreads();
        }
    }
    const int hub_count = max(1, s / 10);
    if (threadIdx.x == 0) {
        double hub_sum = 0.0;
        for (int i = 0; i < hub_count; ++i) hub_sum += (double)e[i].deg;
        out[5] = s_degsum > 0.0 ? hub_sum / s_degsum : 0.0;
        // Hubs on distinct 8-vertex property lines (sizeof(double) = 8 bytes per vertex).
        int distinct = 0;
        for (int i = 0; i < hub_count; ++i) {
            const long long line = e[i].node / 8;
            bool seen = false;
            for (int j = 0; j < i && !seen; ++j) seen = (e[j].node / 8) == line;
            distinct += !seen;
        }
        out[6] = distinct ? (double)hub_count / distinct : 0.0;
    }
    // Span and window overlap over the sampled rows (warp per sampled vertex).
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const double denom = (double)(n - 1 > 1 ? n - 1 : 1);
    double span = 0.0;
    unsigned long long edges = 0, window = 0;
    for (int i = w; i < s; i += blockDim.x / 32) {
        const long long node = e[i].node;
        const long long nline = node / 8;
        for (int64_t q = rp[node] + lane; q < rp[node + 1]; q += 32) {
            const long long dst = col[q];
            span += (double)llabs(dst - node) / denom;
            ++edges;
            window += llabs(dst / 8 - nline) <= 1;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        span += __shfl_xor_sync(0xFFFFFFFFu, span, o);
        edges += __shfl_xor_sync(0xFFFFFFFFu, edges, o);
        window += __shfl_xor_sync(0xFFFFFFFFu, window, o);
    }
    if (lane == 0) { s_span[w] = span; s_edges[w] = edges; s_window[w] = window; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sp = 0.0;
        unsigned long long ed = 0, wi = 0;
        for (int i = 0; i < (int)(blockDim.x / 32); ++i) { sp += s_span[i]; ed += s_edges[i]; wi += s_window[i]; }
        out[7] = ed ? sp / (double)ed : 0.0;
        out[8] = ed ? (double)wi / (double)ed : 0.0;
    }
}

// ---- MLP ----
__global__ void k_dense_fwd(const float* __restrict__ X, const float* __restrict__ W, const float* __restrict__ b,
                            float* __restrict__ Y, int B, int I, int O, int relu) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= B * O) return;
    const int r = idx / O, o = idx % O;
    float acc = b[o];
    for (int i = 0; i < I; ++i) acc += X[r * I + i] * W[i * O + o];
    Y[idx] = relu ? fmaxf(acc, 0.f) : acc;
}

// dX[r,i] = sum_o dY[r,o] W[i,o], masked by the ReLU of the forward output X.
__global__ void k_dense_bwd_x(const float* __restrict__ dY, const float* __restrict__ W,
                              const float* __restrict__ Xfwd, float* __restrict__ dX, int B, int I, int O) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= B * I) return;
    const int r = idx / I, i = idx % I;
    float acc = 0.f;
    for (int o = 0; o < O; ++o) acc += dY[r * O + o] * W[i * O + o];
    dX[idx] = Xfwd[idx] > 0.f ? acc : 0.f;
}

// dW[i,o] = sum_r X[r,i] dY[r,o]; db[o] = sum_r dY[r,o].
__global__ void k_dense_bwd_w(const float* __restrict__ X, const float* __restrict__ dY, float* __restrict__ dW,
                              float* __restrict__ db, int B, int I, int O) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < I * O) {
        const int i = idx / O, o = idx % O;
        float acc = 0.f;
        for (int r = 0; r < B; ++r) acc += X[r * I + i] * dY[r * O + o];
        dW[idx] = acc;
    } else if (idx < I * O + O) {
        const int o = idx - I * O;
        float acc = 0.f;
        for (int r = 0; r < B; ++r) acc += dY[r * O + o];
        db[o] = acc;
    }
}

// Mean squared error over B x O outputs: dY = 2 (Y - T) / (B O); loss summed per row.
__global__ void k_mse(const float* __restrict__ Y, const float* __restrict__ T, float* __restrict__ dY,
                      float* __restrict__ row_loss, int B, int O) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= B) return;
    float l = 0.f;
    for (int o = 0; o < O; ++o) {
        const float d = Y[r * O + o] - T[r * O + o];
        dY[r * O + o] = 2.f * d / (float)(B * O);
        l += d * d;
    }
    row_loss[r] = l;
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    m[i] = b1 * m[i] + (1.f - b1) * g[i];
    v[i] = b2 * v[i] + (1.f - b2) * g[i] * g[i];
    p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
}

__global__ void k_gather_rows(const float* __restrict__ src, const int32_t* __restrict__ idx, int rows, int cols,
                              float* __restrict__ dst) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rows * cols) return;
    dst[t] = src[(int64_t)idx[t / cols] * cols + t % cols];
}

inline int blocks(int64_t work) { return (int)((work + 255) / 256); }

}  // namespace

void tier0_features_device(const DeviceCSR& g, double* out9_host, cudaStream_t s) {
    const int64_t n = g.n;
    if (n == 0) {
        for (int i = 0; i < 9; ++i) out9_host[i] = 0.0;
        return;
    }
    int sample = (int)std::max<int64_t>(1024, std::min<int64_t>((int64_t)std::sqrt((double)n), kSampleMax));
    sample = (int)std::min<int64_t>(sample, n);
    int P = 1;
    while (P < sample) P <<= 1;
    const int smem = P * (int)sizeof(SampleEntry);
    GB_CUDA(cudaFuncSetAttribute(k_tier0, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    DevBuf<double> out(9, s);
    k_tier0<<<1, kSortThreads, smem, s>>>(g.row_ptr, g.col, n, g.nnz, sample, out);
    GB_LAUNCH_CHECK();
    GB_CUDA(cudaMemcpyAsync(out9_host, out.get(), 9 * sizeof(double), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
}

int mlp_param_count(int in_dim) {
    return in_dim * kMlpHidden + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden + kMlpHidden * kMlpOut + kMlpOut;
}

namespace {
struct MlpView {
    const float *W1, *b1, *W2, *b2, *W3, *b3;
};
MlpView view(const float* p, int in) {
    MlpView v;
    v.W1 = p;
    v.b1 = v.W1 + in * kMlpHidden;
    v.W2 = v.b1 + kMlpHidden;
    v.b2 = v.W2 + kMlpHidden * kMlpHidden;
    v.W3 = v.b2 + kMlpHidden;
    v.b3 = v.W3 + kMlpHidden * kMlpOut;
    return v;
}
}  // namespace

void mlp_forward_device(const float* params, const float* X, int B, int in, float* Y, float* H1, float* H2,
                        cudaStream_t s) {
    const MlpView v = view(params, in);
    k_dense_fwd<<<blocks((int64_t)B * kMlpHidden), 256, 0, s>>>(X, v.W1, v.b1, H1, B, in, kMlpHidden, 1);
    k_dense_fwd<<<blocks((int64_t)B * kMlpHidden), 256, 0, s>>>(H1, v.W2, v.b2, H2, B, kMlpHidden, kMlpHidden, 1);
    k_dense_fwd<<<blocks((int64_t)B * kMlpOut), 256, 0, s>>>(H2, v.W3, v.b3, Y, B, kMlpHidden, kMlpOut, 0);
    GB_LAUNCH_CHECK();
}

float mlp_grad_device(const float* params, const float* X, const float* T, int B, int in, float* grad,
                      cudaStream_t s) {
    DevBuf<float> H1((int64_t)B * kMlpHidden, s), H2((int64_t)B * kMlpHidden, s), Y((int64_t)B * kMlpOut, s),
        dY((int64_t)B * kMlpOut, s), dH2((int64_t)B * kMlpHidden, s), dH1((int64_t)B * kMlpHidden, s),
        row_loss(B, s);
    mlp_forward_device(params, X, B, in, Y, H1, H2, s);
    k_mse<<<blocks(B), 256, 0, s>>>(Y, T, dY, row_loss, B, kMlpOut);
    const MlpView v = view(params, in);
    float* gW1 = grad;
    float* gb1 = gW1 + in * kMlpHidden;
    float* gW2 = gb1 + kMlpHidden;
    float* gb2 = gW2 + kMlpHidden * kMlpHidden;
    float* gW3 = gb2 + kMlpHidden;
    float* gb3 = gW3 + kMlpHidden * kMlpOut;
    k_dense_bwd_w<<<blocks((int64_t)kMlpHidden * kMlpOut + kMlpOut), 256, 0, s>>>(H2, dY, gW3, gb3, B, kMlpHidden,
                                                                                  kMlpOut);
    k_dense_bwd_x<<<blocks((int64_t)B * kMlpHidden), 256, 0, s>>>(dY, v.W3, H2, dH2, B, kMlpHidden, kMlpOut);
    k_dense_bwd_w<<<blocks((int64_t)kMlpHidden * kMlpHidden + kMlpHidden), 256, 0, s>>>(H1, dH2, gW2, gb2, B,
                                                                                        kMlpHidden, kMlpHidden);
    k_dense_bwd_x<<<blocks((int64_t)B * kMlpHidden), 256, 0, s>>>(dH2, v.W2, H1, dH1, B, kMlpHidden, kMlpHidden);
    k_dense_bwd_w<<<blocks((int64_t)in * kMlpHidden + kMlpHidden), 256, 0, s>>>(X, dH1, gW1, gb1, B, in,
                                                                                kMlpHidden);
    GB_LAUNCH_CHECK();
    std::vector<float> rl(B);
    GB_CUDA(cudaMemcpyAsync(rl.data(), row_loss.get(), B * sizeof(float), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    double tot = 0.0;
    for (float x : rl) tot += x;
    return (float)(tot / ((double)B * kMlpOut));
}

float mlp_train_device(float* params, const float* X, const float* T, int n, int in, int epochs, int batch,
                       float lr, uint64_t seed, cudaStream_t s) {
    const int P = mlp_param_count(in);
    DevBuf<float> grad(P, s), m(P, s), v(P, s), Xb((int64_t)batch * in, s), Tb((int64_t)batch * kMlpOut, s);
    DevBuf<int32_t> idx(batch, s);
    GB_CUDA(cudaMemsetAsync(m, 0, P * sizeof(float), s));
    GB_CUDA(cudaMemsetAsync(v, 0, P * sizeof(float), s));
    std::vector<int32_t> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    uint64_t state = seed ^ 0x9E3779B97F4A7C15ull;
    auto next = [&]() {
        state += 0x9E3779B97F4A7C15ull;
        uint64_t z = state;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    int t = 0;
    float last = 0.f;
    for (int ep = 0; ep < epochs; ++ep) {
        for (int i = n - 1; i > 0; --i) std::swap(order[i], order[next() % (uint64_t)(i + 1)]);
        double ep_loss = 0.0;
        int nb = 0;
        for (int b0 = 0; b0 < n; b0 += batch) {
            const int B = std::min(batch, n - b0);
            GB_CUDA(cudaMemcpyAsync(idx.get(), order.data() + b0, B * sizeof(int32_t), cudaMemcpyHostToDevice, s));
            k_gather_rows<<<blocks((int64_t)B * in), 256, 0, s>>>(X, idx, B, in, Xb);
            k_gather_rows<<<blocks((int64_t)B * kMlpOut), 256, 0, s>>>(T, idx, B, kMlpOut, Tb);
            ep_loss += mlp_grad_device(params, Xb, Tb, B, in, grad, s);
            ++nb;
            ++t;
            const float c1 = 1.f - std::pow(b1, (float)t), c2 = 1.f - std::pow(b2, (float)t);
            k_adam<<<blocks(P), 256, 0, s>>>(params, grad, m, v, P, lr, b1, b2, eps, c1, c2);
            GB_LAUNCH_CHECK();
        }
        last = (float)(ep_loss / std::max(1, nb));
    }
    GB_CUDA(cudaStreamSynchronize(s));
    return last;
}

}  // namespace gb
