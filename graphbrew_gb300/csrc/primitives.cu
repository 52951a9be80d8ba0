// primitives.cu -- scan, stable radix sort and fill kernels used by every stage.
//
// All of these are bandwidth-bound integer passes: tiles of 2048 elements per
// 256-thread CTA, coalesced loads, shared-memory staging, grid sizes set by
// the element count.
#include "gb_chunks.cuh"
#include "gb_common.cuh"

namespace gb {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int64_t warp_incl_scan(int64_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t t = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Exclusive scan across the CTA; returns this thread's exclusive prefix and
// writes the CTA total to *total.
__device__ __forceinline__ int64_t block_excl_scan(int64_t v, int64_t* total) {
    __shared__ int64_t warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    int64_t incl = warp_incl_scan(v);
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int64_t w = lane < nwarps ? warp_sums[lane] : 0;
        int64_t wi = warp_incl_scan(w);
        if (lane < nwarps) warp_sums[lane] = wi - w;
        if (lane == nwarps - 1) warp_sums[31] = wi;
    }
    __syncthreads();
    int64_t res = warp_sums[warp] + incl - v;
    if (total) *total = warp_sums[31];
    __syncthreads();
    return res;
}

template <typename Tin>
__global__ void k_tile_reduce(const Tin* __restrict__ in, int64_t n, int64_t* __restrict__ partial) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    int64_t sum = 0;
    for (int i = threadIdx.x; i < kScanTile; i += kScanThreads) {
        const int64_t idx = base + i;
        if (idx < n) sum += (int64_t)in[idx];
    }
    int64_t total;
    block_excl_scan(sum, &total);
    if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

template <typename Tin>
__global__ void k_tile_scan(const Tin* __restrict__ in, int64_t* __restrict__ out, int64_t n,
                            const int64_t* __restrict__ tile_offset, int64_t* __restrict__ total_out) {
    __shared__ int64_t s[kScanTile];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    for (int i = threadIdx.x; i < kScanTile; i += kScanThreads) {
        const int64_t idx = base + i;
        s[i] = idx < n ? (int64_t)in[idx] : 0;
    }
    __syncthreads();
    int64_t local[kScanItems];
    int64_t tsum = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        local[j] = s[threadIdx.x * kScanItems + j];
        tsum += local[j];
    }
    int64_t total;
    int64_t run = block_excl_scan(tsum, &total) + (tile_offset ? tile_offset[blockIdx.x] : 0);
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        s[threadIdx.x * kScanItems + j] = run;
        run += local[j];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kScanTile; i += kScanThreads) {
        const int64_t idx = base + i;
        if (idx < n) out[idx] = s[i];
    }
    if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == kScanThreads - 1) {
        *total_out = run;  // prefix of the last tile's end = grand total
    }
}

template <typename Tin>
void exclusive_scan_impl(const Tin* in, int64_t* out, int64_t n, int64_t* total_dev, cudaStream_t s) {
    if (n <= 0) {
        if (total_dev) GB_CUDA(cudaMemsetAsync(total_dev, 0, sizeof(int64_t), s));
        return;
    }
    const int64_t tiles = ceil_div(n, kScanTile);
    if (tiles == 1) {
        k_tile_scan<Tin><<<1, kScanThreads, 0, s>>>(in, out, n, nullptr, total_dev);
        GB_LAUNCH_CHECK();
        return;
    }
    DevBuf<int64_t> partial(tiles, s);
    k_tile_reduce<Tin><<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, partial);
    GB_LAUNCH_CHECK();
    exclusive_scan_impl<int64_t>(partial, partial, tiles, nullptr, s);
    k_tile_scan<Tin><<<(unsigned)tiles, kScanThreads, 0, s>>>(in, out, n, partial, total_dev);
    GB_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits.
// Tile = 8 warps x 256 consecutive keys; each warp walks its 256 keys in 8
// steps of 32, ranking equal digits with __match_any_sync, so ranks follow
// input order (stable).
// ---------------------------------------------------------------------------
constexpr int kRadixThreads = 256;
constexpr int kRadixWarps = kRadixThreads / 32;
constexpr int kRadixPerWarp = 256;
constexpr int kRadixTile = kRadixWarps * kRadixPerWarp;  // 2048
constexpr int kRadixSteps = kRadixPerWarp / 32;           // 8

template <typename K>
__global__ void k_radix_hist(const K* __restrict__ keys, int64_t n, int shift, int64_t num_tiles,
                             int32_t* __restrict__ hist) {
    __shared__ int32_t counts[256];
    counts[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kRadixTile;
    for (int i = threadIdx.x; i < kRadixTile; i += kRadixThreads) {
        const int64_t idx = base + i;
        if (idx < n) atomicAdd(&counts[(unsigned)((keys[idx] >> shift) & 0xFF)], 1);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * num_tiles + blockIdx.x] = counts[threadIdx.x];
}

template <typename K, bool kHasValues>
__global__ void k_radix_scatter(const K* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                                K* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int64_t n,
                                int shift, int64_t num_tiles, const int64_t* __restrict__ offsets) {
    __shared__ int32_t wrun[kRadixWarps][257];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kRadixWarps * 257; i += kRadixThreads) (&wrun[0][0])[i] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kRadixTile + (int64_t)warp * kRadixPerWarp;
    K k_reg[kRadixSteps];
    uint32_t v_reg[kRadixSteps];
    int d_reg[kRadixSteps];
    int r_reg[kRadixSteps];
    const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int st = 0; st < kRadixSteps; ++st) {
        const int64_t idx = base + st * 32 + lane;
        int d = 256;
        K k = 0;
        uint32_t v = 0;
        if (idx < n) {
            k = keys_in[idx];
            if (kHasValues) v = vals_in[idx];
            d = (int)((k >> shift) & 0xFF);
        }
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
        const int before = wrun[warp][d];
        __syncwarp();
        const int leader = __ffs(peers) - 1;
        if (lane == leader) wrun[warp][d] = before + __popc(peers);
        __syncwarp();
        k_reg[st] = k;
        v_reg[st] = v;
        d_reg[st] = d;
        r_reg[st] = before + __popc(peers & lt_mask);
    }
    __syncthreads();
    // Per digit: exclusive prefix over warps (warps cover consecutive keys).
    {
        const int d = threadIdx.x;  // 256 threads == 256 digits
        int acc = 0;
#pragma unroll
        for (int w = 0; w < kRadixWarps; ++w) {
            const int t = wrun[w][d];
            wrun[w][d] = acc;
            acc += t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int st = 0; st < kRadixSteps; ++st) {
        const int d = d_reg[st];
        if (d < 256) {
            const int64_t pos = offsets[(int64_t)d * num_tiles + blockIdx.x] + wrun[warp][d] + r_reg[st];
            keys_out[pos] = k_reg[st];
            if (kHasValues) vals_out[pos] = v_reg[st];
        }
    }
}

template <typename K, bool kHasValues>
void radix_sort_impl(K* keys, uint32_t* values, int64_t n, int key_bits, cudaStream_t s) {
    if (n <= 1 || key_bits <= 0) return;
    const int passes = (key_bits + 7) / 8;
    const int64_t tiles = ceil_div(n, kRadixTile);
    DevBuf<K> kbuf(n, s);
    DevBuf<uint32_t> vbuf(kHasValues ? n : 0, s);
    DevBuf<int32_t> hist(256 * tiles, s);
    DevBuf<int64_t> offs(256 * tiles, s);
    K* kin = keys;
    K* kout = kbuf.get();
    uint32_t* vin = values;
    uint32_t* vout = vbuf.get();
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        k_radix_hist<K><<<(unsigned)tiles, kRadixThreads, 0, s>>>(kin, n, shift, tiles, hist);
        GB_LAUNCH_CHECK();
        exclusive_scan_impl<int32_t>(hist, offs, 256 * tiles, nullptr, s);
        k_radix_scatter<K, kHasValues><<<(unsigned)tiles, kRadixThreads, 0, s>>>(
            kin, vin, kout, vout, n, shift, tiles, offs);
        GB_LAUNCH_CHECK();
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    if (kin != keys) {
        GB_CUDA(cudaMemcpyAsync(keys, kin, n * sizeof(K), cudaMemcpyDeviceToDevice, s));
        if (kHasValues)
            GB_CUDA(cudaMemcpyAsync(values, vin, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    }
}

__global__ void k_fill_u32(uint32_t* p, uint32_t v, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}
__global__ void k_fill_i64(int64_t* p, int64_t v, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}
__global__ void k_iota_u32(uint32_t* p, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = (uint32_t)i;
}
__global__ void k_degrees(const int64_t* __restrict__ rp, int64_t* __restrict__ deg, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        deg[i] = rp[i + 1] - rp[i];
}

__global__ void k_chunk_rows(const int64_t* __restrict__ rp, int64_t n, int32_t* __restrict__ chunk_row) {
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = rp[u], e = rp[u + 1];
        for (int64_t c = (b + kEdgeChunk - 1) / kEdgeChunk; c * kEdgeChunk < e; ++c) chunk_row[c] = (int32_t)u;
    }
}

}  // namespace

void chunk_rows_device(const int64_t* row_ptr, int64_t n, int64_t nnz, int32_t* chunk_row, cudaStream_t s) {
    if (n <= 0 || nnz <= 0) return;
    k_chunk_rows<<<grid_for(n, 256), 256, 0, s>>>(row_ptr, n, chunk_row);
    GB_LAUNCH_CHECK();
}

void exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n, cudaStream_t s) {
    exclusive_scan_impl<int64_t>(in, out, n, nullptr, s);
}

void exclusive_scan_i64_total(const int64_t* in, int64_t* out, int64_t n, int64_t* total_dev,
                              cudaStream_t s) {
    exclusive_scan_impl<int64_t>(in, out, n, total_dev, s);
}

void exclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, int64_t n, int64_t* total_dev,
                               cudaStream_t s) {
    exclusive_scan_impl<int32_t>(in, out, n, total_dev, s);
}

void exclusive_scan_u8_to_i64(const uint8_t* in, int64_t* out, int64_t n, int64_t* total_dev, cudaStream_t s) {
    exclusive_scan_impl<uint8_t>(in, out, n, total_dev, s);
}

void radix_sort_pairs_u32(uint32_t* keys, uint32_t* values, int64_t n, int key_bits, cudaStream_t s) {
    radix_sort_impl<uint32_t, true>(keys, values, n, key_bits, s);
}
void radix_sort_pairs_u64(uint64_t* keys, uint32_t* values, int64_t n, int key_bits, cudaStream_t s) {
    radix_sort_impl<uint64_t, true>(keys, values, n, key_bits, s);
}
void radix_sort_keys_u64(uint64_t* keys, int64_t n, int key_bits, cudaStream_t s) {
    radix_sort_impl<uint64_t, false>(keys, nullptr, n, key_bits, s);
}

void fill_u32(uint32_t* p, uint32_t v, int64_t n, cudaStream_t s) {
    if (n <= 0) return;
    k_fill_u32<<<grid_for(n, 256), 256, 0, s>>>(p, v, n);
    GB_LAUNCH_CHECK();
}
void fill_i64(int64_t* p, int64_t v, int64_t n, cudaStream_t s) {
    if (n <= 0) return;
    k_fill_i64<<<grid_for(n, 256), 256, 0, s>>>(p, v, n);
    GB_LAUNCH_CHECK();
}
void iota_u32(uint32_t* p, int64_t n, cudaStream_t s) {
    if (n <= 0) return;
    k_iota_u32<<<grid_for(n, 256), 256, 0, s>>>(p, n);
    GB_LAUNCH_CHECK();
}
void degrees_i64(const int64_t* row_ptr, int64_t* deg, int64_t n, cudaStream_t s) {
    if (n <= 0) return;
    k_degrees<<<grid_for(n, 256), 256, 0, s>>>(row_ptr, deg, n);
    GB_LAUNCH_CHECK();
}

}  // namespace gb
