// sort.cu — stable LSD radix sort and exclusive scan (see sort.cuh).
//
// One pass over B digit bits (B = 8 or 10, D = 2^B buckets) = three launches:
//   k_digit_hist   per-tile digit counts, written digit-major
//                  (counts[d * tiles + tile]);
//   exclusive scan of that array: the global start of (digit d, tile t);
//   k_scatter      ranks the tile's keys, stages them in shared memory in
//                  digit order and writes digit runs out contiguously.
// A tile is 256 threads x IT keys (IT = 32 for 32-bit keys, 8 for 64-bit):
// with 1024 digits, an 8192-key tile writes runs of 8 keys (a full 32-byte
// sector) where a 4096-key tile wrote half sectors — the ordering of 16M
// queries took 1.24 ms instead of 1.50 (48 keys per thread: 1.34).
// Ranking needs no block-wide barrier per round: warp w owns the tile's keys
// [w*32*IT, (w+1)*32*IT) and ranks them round by round (32 consecutive keys,
// lanes in order) against its own digit counters — one ballot per digit bit
// groups equal digits (cheaper than match_any here), the group's first lane
// reads and advances the warp counter.  The histogram pass uses one shared-
// memory atomic per key.  (16M 30-bit keys, 3 passes: 0.64 ms.)  One
// block-wide pass then turns the warp counters into per-warp offsets and the
// tile's digit starts.  Keys are ranked in (warp, round, lane) order, which is
// input order, so every pass is stable.  Ten-bit digits are used when they
// save a pass (30-bit Hilbert keys: 3 passes; 63-bit build keys: 7).
#include "sort.cuh"

#include <algorithm>

namespace cpq {

namespace {

constexpr int kSortThreads = 256;
constexpr int kWarps = kSortThreads / 32;
constexpr int kMaxDigits = 1024;
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanChunk = kScanThreads * kScanItems;

template <typename KeyT>
constexpr int items_per_thread() {
    return sizeof(KeyT) == 4 ? 32 : 8;
}
template <typename KeyT>
constexpr int tile_keys() {
    return kSortThreads * items_per_thread<KeyT>();
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <typename KeyT>
__device__ __forceinline__ uint32_t digit_of(KeyT k, int shift, uint32_t mask) {
    return (uint32_t)(k >> shift) & mask;
}

template <typename KeyT, int B>
__global__ void __launch_bounds__(kSortThreads) k_digit_hist(const KeyT* __restrict__ keys,
                                                              int64_t n, int shift, uint32_t mask,
                                                              uint32_t* __restrict__ counts,
                                                              int tiles) {
    constexpr int D = 1 << B, IT = items_per_thread<KeyT>(), TILE = tile_keys<KeyT>();
    __shared__ uint32_t hist[D];
    for (int d = threadIdx.x; d < D; d += kSortThreads) hist[d] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * TILE;
    // one shared-memory atomic per key: 1024 bins take the few collisions
    // of a warp's near-random digits at less cost than grouping them first
#pragma unroll 8
    for (int r = 0; r < IT; ++r) {
        const int64_t i = base + r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&hist[digit_of(keys[i], shift, mask)], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < D; d += kSortThreads) counts[(int64_t)d * tiles + blockIdx.x] = hist[d];
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

template <typename KeyT, int B>
constexpr size_t scatter_smem_bytes() {
    constexpr int D = 1 << B, TILE = tile_keys<KeyT>();
    return (size_t)TILE * sizeof(KeyT) + (size_t)TILE * sizeof(int32_t) +
           (size_t)(kWarps * D + D + D + kWarps) * sizeof(uint32_t);
}

template <typename KeyT, int B>
__global__ void __launch_bounds__(kSortThreads) k_scatter(const KeyT* __restrict__ keys_in,
                                                           const int32_t* __restrict__ vals_in,
                                                           KeyT* __restrict__ keys_out,
                                                           int32_t* __restrict__ vals_out,
                                                           int64_t n, int shift, uint32_t mask,
                                                           const uint32_t* __restrict__ offsets,
                                                           int tiles) {
    constexpr int D = 1 << B, IT = items_per_thread<KeyT>(), TILE = tile_keys<KeyT>();
    constexpr int DPT = D / kSortThreads;  // digits per thread in the block-wide passes
    extern __shared__ __align__(16) unsigned char smem_raw[];
    KeyT* skeys = reinterpret_cast<KeyT*>(smem_raw);
    int32_t* svals = reinterpret_cast<int32_t*>(skeys + TILE);
    uint32_t* wcnt = reinterpret_cast<uint32_t*>(svals + TILE);  // [warp][digit]
    uint32_t* tile_base = wcnt + kWarps * D;                     // D
    uint32_t* global_base = tile_base + D;                       // D
    uint32_t* warp_tot = global_base + D;                        // kWarps

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t base = (int64_t)blockIdx.x * TILE;
    const int tile_n = (int)((n - base) < (int64_t)TILE ? (n - base) : (int64_t)TILE);
    const int wbase = warp * 32 * IT;  // this warp's keys within the tile

    KeyT k[IT];
    int32_t v[IT];
#pragma unroll
    for (int r = 0; r < IT; ++r) {
        const int j = wbase + r * 32 + lane;
        if (j < tile_n) {
            k[r] = keys_in[base + j];
            v[r] = vals_in ? vals_in[base + j] : (int32_t)(base + j);  // no values: the identity
        } else {
            k[r] = 0;
            v[r] = 0;
        }
    }
    for (int j = tid; j < kWarps * D; j += kSortThreads) wcnt[j] = 0;
    for (int d = tid; d < D; d += kSortThreads) global_base[d] = offsets[(int64_t)d * tiles + blockIdx.x];
    __syncthreads();

    // rank within the warp, round by round; the counters are this warp's own
    uint32_t* my = wcnt + warp * D;
    const uint32_t lt = lanemask_lt();
    uint32_t rank[IT];
#pragma unroll
    for (int r = 0; r < IT; ++r) {
        const bool valid = wbase + r * 32 + lane < tile_n;
        const uint32_t d = valid ? digit_of(k[r], shift, mask) : 0u;
        // lanes with this lane's digit: one ballot per digit bit
        uint32_t peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const bool bit = (d >> b) & 1u;
            const uint32_t m = __ballot_sync(0xffffffffu, bit);
            peers &= bit ? m : ~m;
        }
        if (!valid) peers = 1u << lane;
        const int leader = __ffs(peers) - 1;
        uint32_t old = 0;
        if (valid && lane == leader) {
            old = my[d];
            my[d] = old + (uint32_t)__popc(peers);
        }
        old = __shfl_sync(0xffffffffu, old, leader);
        rank[r] = old + (uint32_t)__popc(peers & lt);
        __syncwarp();
    }
    __syncthreads();

    // per digit: exclusive prefix over warps, then the tile's digit starts
    uint32_t tot[DPT];
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < DPT; ++j) {
        const int d = tid * DPT + j;
        uint32_t acc = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t c = wcnt[w * D + d];
            wcnt[w * D + d] = acc;
            acc += c;
        }
        tot[j] = acc;
        sum += acc;
    }
    uint32_t run = block_scan_256(sum, warp_tot);
#pragma unroll
    for (int j = 0; j < DPT; ++j) {
        tile_base[tid * DPT + j] = run;
        run += tot[j];
    }
    __syncthreads();

    // stage in digit order
#pragma unroll
    for (int r = 0; r < IT; ++r) {
        if (wbase + r * 32 + lane < tile_n) {
            const uint32_t d = digit_of(k[r], shift, mask);
            const uint32_t pos = tile_base[d] + wcnt[warp * D + d] + rank[r];
            skeys[pos] = k[r];
            svals[pos] = v[r];
        }
    }
    __syncthreads();
    for (int j = tid; j < tile_n; j += kSortThreads) {
        const KeyT key = skeys[j];
        const uint32_t d = digit_of(key, shift, mask);
        const uint32_t dst = global_base[d] + (uint32_t)j - tile_base[d];
        keys_out[dst] = key;
        vals_out[dst] = svals[j];
    }
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
    // the largest per-pass count array: the smaller (64-bit key) tile and
    // ten-bit digits
    int64_t tiles = std::max<int64_t>(1, ceil_div(n, tile_keys<uint64_t>()));
    int64_t m = tiles * kMaxDigits;
    return align256((size_t)m * sizeof(uint32_t)) + scan_workspace_bytes(m);
}

namespace {

template <typename KeyT, int B>
cudaError_t sort_pass(const KeyT* ki, const int32_t* vi, KeyT* ko, int32_t* vo, int64_t n,
                      int shift, int bits, uint32_t* counts, unsigned char* scan_ws,
                      size_t scan_bytes, cudaStream_t stream) {
    constexpr int D = 1 << B;
    const int tiles = (int)ceil_div(n, tile_keys<KeyT>());
    const int64_t m = (int64_t)tiles * D;
    const uint32_t mask = (bits >= 32 ? 0xffffffffu : ((1u << bits) - 1u));
    const size_t smem = scatter_smem_bytes<KeyT, B>();
    cudaError_t e = ensure_smem_limit(reinterpret_cast<const void*>(k_scatter<KeyT, B>), smem);
    if (e != cudaSuccess) return e;
    k_digit_hist<KeyT, B><<<tiles, kSortThreads, 0, stream>>>(ki, n, shift, mask, counts, tiles); note_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = exclusive_scan_u32(counts, m, nullptr, scan_ws, scan_bytes, stream);
    if (e != cudaSuccess) return e;
    k_scatter<KeyT, B><<<tiles, kSortThreads, smem, stream>>>(ki, vi, ko, vo, n, shift, mask, counts,
                                                             tiles); note_launch();
    return cudaGetLastError();
}

}  // namespace

template <typename KeyT>
cudaError_t radix_sort_pairs(KeyT* keys, int32_t* vals, KeyT* keys_alt, int32_t* vals_alt,
                             int64_t n, int begin_bit, int end_bit, void* workspace,
                             size_t workspace_bytes, cudaStream_t stream, bool* in_alt, bool identity_vals) {
    *in_alt = false;
    if (n <= 1 || end_bit <= begin_bit) return cudaSuccess;
    if (workspace_bytes < radix_sort_workspace_bytes(n)) return cudaErrorInvalidValue;
    const int nbits = end_bit - begin_bit;
    // ten-bit digits when they take fewer passes than eight-bit ones
    const int digit_bits = (nbits + 9) / 10 < (nbits + 7) / 8 ? 10 : 8;
    unsigned char* ws = static_cast<unsigned char*>(workspace);
    const int64_t max_m = std::max<int64_t>(1, ceil_div(n, tile_keys<uint64_t>())) * kMaxDigits;
    uint32_t* counts = reinterpret_cast<uint32_t*>(ws);
    unsigned char* scan_ws = ws + align256((size_t)max_m * sizeof(uint32_t));
    const size_t scan_bytes = workspace_bytes - align256((size_t)max_m * sizeof(uint32_t));

    KeyT *ki = keys, *ko = keys_alt;
    int32_t *vi = vals, *vo = vals_alt;
    bool alt = false;
    bool first = true;
    for (int shift = begin_bit; shift < end_bit; shift += digit_bits) {
        const int bits = std::min(digit_bits, end_bit - shift);
        const int32_t* vin = first && identity_vals ? nullptr : vi;  // the first pass makes the identity
        first = false;
        cudaError_t e = digit_bits == 10
                            ? sort_pass<KeyT, 10>(ki, vin, ko, vo, n, shift, bits, counts, scan_ws, scan_bytes, stream)
                            : sort_pass<KeyT, 8>(ki, vin, ko, vo, n, shift, bits, counts, scan_ws, scan_bytes, stream);
        if (e != cudaSuccess) return e;
        std::swap(ki, ko);
        std::swap(vi, vo);
        alt = !alt;
    }
    *in_alt = alt;
    return cudaSuccess;
}

template cudaError_t radix_sort_pairs<uint32_t>(uint32_t*, int32_t*, uint32_t*, int32_t*, int64_t,
                                                int, int, void*, size_t, cudaStream_t, bool*, bool);
template cudaError_t radix_sort_pairs<uint64_t>(uint64_t*, int32_t*, uint64_t*, int32_t*, int64_t,
                                                int, int, void*, size_t, cudaStream_t, bool*, bool);

}  // namespace cpq
