// sort.cu — stable LSD radix sort and exclusive scan (see sort.cuh).
//
// One 8-bit pass = three launches:
//   k_digit_hist   per-tile digit counts, written digit-major
//                  (counts[d * tiles + tile]);
//   exclusive scan of that array: the global start of (digit d, tile t);
//   k_scatter      each tile ranks its keys stably (warp match_any + a
//                  per-round prefix over warps), stages them in shared memory
//                  in digit order and writes digit runs out contiguously.
// A tile is 256 threads x 16 keys.  Stability comes from ranking the tile's
// keys in input order: round r holds keys r*256 .. r*256+255, lanes in order.
#include "sort.cuh"

#include <algorithm>

namespace cpq {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kTile = kSortThreads * kSortItems;
constexpr int kWarps = kSortThreads / 32;
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanChunk = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <typename KeyT>
__global__ void __launch_bounds__(kSortThreads) k_digit_hist(const KeyT* __restrict__ keys,
                                                              int64_t n, int shift,
                                                              uint32_t* __restrict__ counts,
                                                              int tiles) {
    __shared__ uint32_t hist[256];
    hist[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kTile;
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        int64_t i = base + r * kSortThreads + threadIdx.x;
        bool valid = i < n;
        uint32_t d = valid ? (uint32_t)((keys[i] >> shift) & 255u) : 256u + (threadIdx.x & 31);
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        if (valid && (peers & lanemask_lt()) == 0) atomicAdd(&hist[d], (uint32_t)__popc(peers));
    }
    __syncthreads();
    counts[(int64_t)threadIdx.x * tiles + blockIdx.x] = hist[threadIdx.x];
}

// Exclusive scan of one value per thread over a block of 256 threads.
__device__ __forceinline__ uint32_t block_scan_256(uint32_t v, uint32_t* warp_tot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    uint32_t off = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) off += (w < warp) ? warp_tot[w] : 0u;
    __syncthreads();
    return off + x - v;
}

template <typename KeyT>
__global__ void __launch_bounds__(kSortThreads) k_scatter(const KeyT* __restrict__ keys_in,
                                                           const int32_t* __restrict__ vals_in,
                                                           KeyT* __restrict__ keys_out,
                                                           int32_t* __restrict__ vals_out,
                                                           int64_t n, int shift,
                                                           const uint32_t* __restrict__ offsets,
                                                           int tiles) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    KeyT* skeys = reinterpret_cast<KeyT*>(smem_raw);
    int32_t* svals = reinterpret_cast<int32_t*>(skeys + kTile);
    uint32_t* tile_base = reinterpret_cast<uint32_t*>(svals + kTile);  // 256
    uint32_t* run = tile_base + 256;                                   // 256
    uint32_t* warp_cnt = run + 256;                                    // kWarps * 256
    uint32_t* warp_tot = warp_cnt + kWarps * 256;                      // kWarps
    uint32_t* global_base = warp_tot + kWarps;                         // 256

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t base = (int64_t)blockIdx.x * kTile;
    const int tile_n = (int)((n - base) < (int64_t)kTile ? (n - base) : (int64_t)kTile);

    KeyT k[kSortItems];
    int32_t v[kSortItems];
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        int64_t i = base + r * kSortThreads + tid;
        if (i < n) {
            k[r] = keys_in[i];
            v[r] = vals_in[i];
        } else {
            k[r] = 0;
            v[r] = 0;
        }
    }
    // tile histogram (reuse run[] as the counter array)
    run[tid] = 0;
    global_base[tid] = offsets[(int64_t)tid * tiles + blockIdx.x];
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        bool valid = r * kSortThreads + tid < tile_n;
        uint32_t d = valid ? (uint32_t)((k[r] >> shift) & 255u) : 256u + lane;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        if (valid && (peers & lanemask_lt()) == 0) atomicAdd(&run[d], (uint32_t)__popc(peers));
    }
    __syncthreads();
    uint32_t cnt = run[tid];
    uint32_t b = block_scan_256(cnt, warp_tot);
    tile_base[tid] = b;
    run[tid] = 0;
    __syncthreads();

    const uint32_t lt = lanemask_lt();
#pragma unroll 1
    for (int r = 0; r < kSortItems; ++r) {
#pragma unroll
        for (int w = 0; w < kWarps; ++w) warp_cnt[w * 256 + tid] = 0;
        __syncthreads();
        bool valid = r * kSortThreads + tid < tile_n;
        uint32_t d = valid ? (uint32_t)((k[r] >> shift) & 255u) : 256u + lane;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t rank = __popc(peers & lt);
        if (valid && rank == 0) warp_cnt[warp * 256 + d] = __popc(peers);
        __syncthreads();
        {
            uint32_t acc = run[tid];
#pragma unroll
            for (int w = 0; w < kWarps; ++w) {
                uint32_t c = warp_cnt[w * 256 + tid];
                warp_cnt[w * 256 + tid] = acc;
                acc += c;
            }
            run[tid] = acc;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = tile_base[d] + warp_cnt[warp * 256 + d] + rank;
            skeys[pos] = k[r];
            svals[pos] = v[r];
        }
        __syncthreads();
    }
    for (int j = tid; j < tile_n; j += kSortThreads) {
        KeyT key = skeys[j];
        uint32_t d = (uint32_t)((key >> shift) & 255u);
        uint32_t dst = global_base[d] + (uint32_t)j - tile_base[d];
        keys_out[dst] = key;
        vals_out[dst] = svals[j];
    }
}

template <typename KeyT>
size_t scatter_smem_bytes() {
    return (size_t)kTile * sizeof(KeyT) + (size_t)kTile * sizeof(int32_t) +
           (256 + 256 + kWarps * 256 + kWarps + 256) * sizeof(uint32_t);
}

// ---- exclusive scan ------------------------------------------------------

__global__ void __launch_bounds__(kScanThreads) k_scan_chunk(uint32_t* __restrict__ data,
                                                              int64_t m,
                                                              uint32_t* __restrict__ chunk_sums) {
    __shared__ uint32_t warp_tot[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t base = (int64_t)blockIdx.x * kScanChunk + (int64_t)tid * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = (base + i < m) ? data[base + i] : 0u;
        s += v[i];
    }
    uint32_t x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = warp_tot[lane];
        uint32_t u = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, u, o);
            if (lane >= o) u += y;
        }
        warp_tot[lane] = u - t;  // exclusive
        if (lane == 31 && chunk_sums) chunk_sums[blockIdx.x] = u;
    }
    __syncthreads();
    uint32_t run = warp_tot[warp] + x - s;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < m) data[base + i] = run;
        run += v[i];
    }
}

__global__ void k_scan_add(uint32_t* __restrict__ data, int64_t m,
                           const uint32_t* __restrict__ chunk_off) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) data[i] += chunk_off[i / kScanChunk];
}

__global__ void k_scan_total(const uint32_t* __restrict__ data, const uint32_t* __restrict__ orig_last,
                             int64_t m, uint32_t* total) {
    // total = exclusive[m-1] + original last value (saved before the scan)
    total[0] = data[m - 1] + orig_last[0];
}

__global__ void k_save_last(const uint32_t* __restrict__ data, int64_t m, uint32_t* out) {
    out[0] = data[m - 1];
}

int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

size_t scan_workspace_bytes(int64_t m) {
    size_t bytes = 256;  // saved last value
    int64_t level = m;
    while (level > kScanChunk) {
        level = ceil_div(level, kScanChunk);
        bytes += align256((size_t)level * sizeof(uint32_t));
    }
    return bytes;
}

static cudaError_t scan_rec(uint32_t* data, int64_t m, unsigned char* ws, cudaStream_t st) {
    int64_t chunks = ceil_div(m, kScanChunk);
    if (chunks <= 1) {
        k_scan_chunk<<<1, kScanThreads, 0, st>>>(data, m, nullptr); note_launch();
        return cudaGetLastError();
    }
    uint32_t* sums = reinterpret_cast<uint32_t*>(ws);
    k_scan_chunk<<<(unsigned)chunks, kScanThreads, 0, st>>>(data, m, sums); note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = scan_rec(sums, chunks, ws + align256((size_t)chunks * sizeof(uint32_t)), st);
    if (e != cudaSuccess) return e;
    k_scan_add<<<(unsigned)ceil_div(m, 256), 256, 0, st>>>(data, m, sums); note_launch();
    return cudaGetLastError();
}

cudaError_t exclusive_scan_u32(uint32_t* data, int64_t m, uint32_t* total, void* workspace,
                               size_t workspace_bytes, cudaStream_t stream) {
    if (m <= 0) {
        if (total) return cudaMemsetAsync(total, 0, sizeof(uint32_t), stream);
        return cudaSuccess;
    }
    if (workspace_bytes < scan_workspace_bytes(m)) return cudaErrorInvalidValue;
    unsigned char* ws = static_cast<unsigned char*>(workspace);
    uint32_t* last = reinterpret_cast<uint32_t*>(ws);
    if (total) {
        k_save_last<<<1, 1, 0, stream>>>(data, m, last); note_launch();
    }
    cudaError_t e = scan_rec(data, m, ws + 256, stream);
    if (e != cudaSuccess) return e;
    if (total) {
        k_scan_total<<<1, 1, 0, stream>>>(data, last, m, total); note_launch();
        e = cudaGetLastError();
    }
    return e;
}

size_t radix_sort_workspace_bytes(int64_t n) {
    int64_t tiles = std::max<int64_t>(1, ceil_div(n, kTile));
    int64_t m = tiles * 256;
    return align256((size_t)m * sizeof(uint32_t)) + scan_workspace_bytes(m);
}

template <typename KeyT>
cudaError_t radix_sort_pairs(KeyT* keys, int32_t* vals, KeyT* keys_alt, int32_t* vals_alt,
                             int64_t n, int begin_bit, int end_bit, void* workspace,
                             size_t workspace_bytes, cudaStream_t stream, bool* in_alt) {
    *in_alt = false;
    if (n <= 1 || end_bit <= begin_bit) return cudaSuccess;
    if (workspace_bytes < radix_sort_workspace_bytes(n)) return cudaErrorInvalidValue;
    const size_t smem = scatter_smem_bytes<KeyT>();
    {
        cudaError_t e = ensure_smem_limit(reinterpret_cast<const void*>(k_scatter<KeyT>), smem);
        if (e != cudaSuccess) return e;
    }
    const int tiles = (int)ceil_div(n, kTile);
    const int64_t m = (int64_t)tiles * 256;
    unsigned char* ws = static_cast<unsigned char*>(workspace);
    uint32_t* counts = reinterpret_cast<uint32_t*>(ws);
    unsigned char* scan_ws = ws + align256((size_t)m * sizeof(uint32_t));
    const size_t scan_bytes = workspace_bytes - align256((size_t)m * sizeof(uint32_t));

    KeyT *ki = keys, *ko = keys_alt;
    int32_t *vi = vals, *vo = vals_alt;
    bool alt = false;
    for (int shift = begin_bit; shift < end_bit; shift += 8) {
        k_digit_hist<KeyT><<<tiles, kSortThreads, 0, stream>>>(ki, n, shift, counts, tiles); note_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        e = exclusive_scan_u32(counts, m, nullptr, scan_ws, scan_bytes, stream);
        if (e != cudaSuccess) return e;
        k_scatter<KeyT><<<tiles, kSortThreads, smem, stream>>>(ki, vi, ko, vo, n, shift, counts, tiles); note_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        std::swap(ki, ko);
        std::swap(vi, vo);
        alt = !alt;
    }
    *in_alt = alt;
    return cudaSuccess;
}

template cudaError_t radix_sort_pairs<uint32_t>(uint32_t*, int32_t*, uint32_t*, int32_t*, int64_t,
                                                int, int, void*, size_t, cudaStream_t, bool*);
template cudaError_t radix_sort_pairs<uint64_t>(uint64_t*, int32_t*, uint64_t*, int32_t*, int64_t,
                                                int, int, void*, size_t, cudaStream_t, bool*);

}  // namespace cpq
