// noalloc.cu — cp_query_noalloc: the closest-point query for callers that
// must not allocate device memory while they run.
//
// Some callers cannot call cudaMalloc at query time: a renderer or simulation
// loop that forbids device allocation after start-up (an allocation can
// synchronise the device and stall the frame), a plugin whose host framework
// owns all device memory and refuses side allocations, or code that runs
// while an allocator of its own holds a lock.  cp_query needs scratch memory
// (the work counter, the query bounding box, the ordering keys and values and
// the radix-sort counts) and either takes it from the caller or allocates it.
// This variant takes it from a fixed area that the library owns instead: a
// file-scope device array of kScratchBytes, which a GPU holds from the moment
// the array is loaded on it until the process exits.
//
// In host code the array's name is only a host-side stand-in, not a device
// address.  Every call asks the runtime for the real address
// (cudaGetSymbolAddress, with the caller's device current) rather than
// keeping one: after cudaDeviceReset the device gets a new context and the
// array a new address.  The runtime loads a library's device code lazily (the
// default since CUDA 12.2), so the array is allocated on a device by the
// first call there, which is the one call that can fail for lack of memory.
// Make that first call at start-up (a zero-count call loads the array and
// does nothing else), before the host claims the remaining device memory and
// before any stream capture.
//
// Every call shares the one array and leaves its last contents behind.  The
// query clears what must start at zero (the work counter; the query box is
// re-initialised; the sort writes every count it reads), but two calls that
// overlap on the GPU — on different streams, or from different threads —
// race on the array and give wrong results.  Order them on one stream.
#include <cuda_runtime.h>

#include <climits>
#include <string>

#include "handles.cuh"

namespace {

// 32 MiB: the work counter, the query frame, two key arrays, two value arrays
// and the radix-sort counts of kMaxSortedQueries queries (24.3 MiB) fit with
// room to spare.  Without query ordering a query needs only the counter.
constexpr size_t kScratchBytes = size_t(32) << 20;
constexpr int64_t kMaxSortedQueries = int64_t(1) << 20;

static __device__ __align__(256) unsigned char g_query_scratch[kScratchBytes];

// The array's device address in the current device's context (loading it
// there on first use).
cudaError_t scratch_address(void** out) {
    *out = nullptr;
    return cudaGetSymbolAddress(out, g_query_scratch);
}

}  // namespace

extern "C" CP_API cp_status cp_query_noalloc(const cp_mesh* mesh, const float* queries, int64_t nq,
                                             const cp_query_opts* opts, float* out_point,
                                             float* out_dist, int32_t* out_tri, float* out_bary,
                                             cp_stream_t stream) {
    using namespace cpq;
    if (!mesh) return set_error(CP_ERROR_INVALID_VALUE, "mesh is NULL");
    if (nq < 0) return set_error(CP_ERROR_INVALID_VALUE, "negative query count");
    if (nq > INT32_MAX)
        return set_error(CP_ERROR_NOT_SUPPORTED, "cp_query_noalloc: more than 2^31 - 1 queries in one call");
    // resolved before anything else, so a zero-count call loads the array
    void* ws = nullptr;
    cudaError_t e = scratch_address(&ws);
    if (e != cudaSuccess)
        return set_error(e == cudaErrorMemoryAllocation ? CP_ERROR_OUT_OF_MEMORY : CP_ERROR_CUDA,
                         std::string("cp_query_noalloc: loading the scratch array: ") +
                             cudaGetErrorString(e));
    if (nq == 0) return CP_SUCCESS;
    if (!queries) return set_error(CP_ERROR_INVALID_VALUE, "queries is NULL");
    QueryParams qp;
    cp_status s = parse_query_opts(opts, &qp);
    if (s != CP_SUCCESS) return s;
    qp.no_timing = true;  // the diagnostic timer would create CUDA events
    const size_t need = query_workspace_bytes(mesh->bvh, nq, qp);
    if ((qp.sort && nq > kMaxSortedQueries) || need > kScratchBytes)
        return set_error(CP_ERROR_SCRATCH_TOO_SMALL,
                         "cp_query_noalloc: " + std::to_string(nq) + " queries need " +
                             std::to_string(need) + " bytes of scratch; the fixed area holds " +
                             std::to_string(kScratchBytes) + " and serves at most " +
                             std::to_string(kMaxSortedQueries) +
                             " queries per call with sort_queries on; split the batch, "
                             "turn sort_queries off, or use cp_query");
    e = bvh_query(mesh->bvh, queries, nq, nullptr, qp, out_point, out_dist, out_tri, out_bary, ws,
                  kScratchBytes, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return set_error(CP_ERROR_CUDA, std::string("cp_query_noalloc: ") + cudaGetErrorString(e));
    return CP_SUCCESS;
}

extern "C" CP_API size_t cp_query_noalloc_scratch_bytes(void) { return kScratchBytes; }
