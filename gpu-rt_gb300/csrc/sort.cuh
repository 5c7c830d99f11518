// sort.cuh — stable LSD radix sort of (key, int32 value) pairs and an
// exclusive prefix sum, both hand-written for the GB300 build and query
// pipelines (no CUB).  Every launch goes on the given stream and nothing
// synchronises the host, so the calls can be captured in a CUDA graph.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cpq {

// Host side: count one kernel launch of this library (defined in api.cu).
void note_launch();

// Host side: raise a kernel's dynamic shared-memory limit once per device
// (defined in api.cu).
cudaError_t ensure_smem_limit(const void* kernel, size_t smem);

// Bytes of workspace radix_sort_pairs needs for n keys.
size_t radix_sort_workspace_bytes(int64_t n);

// Sort keys[0..n) ascending with their values, stably, on bits
// [begin_bit, end_bit) (8 or 10 bits per pass).  keys_alt / vals_alt are
// buffers of n elements.  With identity_vals the values are 0..n-1 and vals
// is not read (the first pass makes them).  On return *in_alt tells which
// pair of buffers holds the result.  KeyT is uint32_t or uint64_t.
template <typename KeyT>
cudaError_t radix_sort_pairs(KeyT* keys, int32_t* vals, KeyT* keys_alt, int32_t* vals_alt,
                             int64_t n, int begin_bit, int end_bit, void* workspace,
                             size_t workspace_bytes, cudaStream_t stream, bool* in_alt,
                             bool identity_vals = false);

// Bytes of workspace exclusive_scan_u32 needs for m elements.
size_t scan_workspace_bytes(int64_t m);

// In-place exclusive prefix sum of m uint32 values.  If total != nullptr the
// sum of all values is written there (device pointer).
cudaError_t exclusive_scan_u32(uint32_t* data, int64_t m, uint32_t* total, void* workspace,
                               size_t workspace_bytes, cudaStream_t stream);

}  // namespace cpq
