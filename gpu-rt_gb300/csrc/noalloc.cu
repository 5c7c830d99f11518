// noalloc.cu — cp_query_noalloc: the closest-point query for callers that
// must not allocate device memory while they run.
//
// Some callers cannot call cudaMalloc at query time: a renderer or simulation
// loop that forbids device allocation after start-up (an allocation can
// synchronise the device and stall the frame), a plugin whose host framework
// owns all device memory and refuses side allocations, or code that runs
// while an allocator of its own holds a lock.  cp_query needs scratch memory
// (the work counter, the query bounding box, the Morton keys and values and
// the radix-sort counts) and either takes it from the caller or allocates it.
// This variant takes it from a fixed area that the library owns instead: a
// file-scope device array of kScratchBytes, which every GPU that loads the
// library holds until the process exits.
//
// In host code the array's name is only a host-side stand-in, not a device
// address; the first call on each device asks the runtime for the real
// address (cudaGetSymbolAddress, with that device current) and keeps it.
// That first call should therefore come before any stream capture.
//
// Every call shares the one array and leaves its last contents behind.  The
// query clears what must start at zero (the work counter; the query box is
// re-initialised; the sort writes every count it reads), but two calls that
// overlap on the GPU — on different streams, or from different threads —
// race on the array and give wrong results.  Order them on one stream.
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "handles.cuh"

namespace {

// 32 MiB: the work counter, the query frame, two 64-bit key arrays, two value
// arrays and the radix-sort counts of 1,048,576 queries (24.3 MiB) fit with
// room to spare.  Without Morton ordering a query needs only the counter.
constexpr size_t kScratchBytes = size_t(32) << 20;

static __device__ __align__(256) unsigned char g_query_scratch[kScratchBytes];

std::mutex g_mu;
std::vector<void*> g_scratch_addr;  // per device; nullptr until that device is set up

cudaError_t scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_mu);
    if ((int)g_scratch_addr.size() <= dev) g_scratch_addr.resize(dev + 1, nullptr);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_query_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" CP_API cp_status cp_query_noalloc(const cp_mesh* mesh, const float* queries, int64_t nq,
                                             const cp_query_opts* opts, float* out_point,
                                             float* out_dist, int32_t* out_tri, float* out_bary,
                                             cp_stream_t stream) {
    using namespace cpq;
    if (!mesh) return set_error(CP_ERROR_INVALID_VALUE, "mesh is NULL");
    if (nq < 0) return set_error(CP_ERROR_INVALID_VALUE, "negative query count");
    if (nq == 0) return CP_SUCCESS;
    if (!queries) return set_error(CP_ERROR_INVALID_VALUE, "queries is NULL");
    QueryParams qp;
    cp_status s = parse_query_opts(opts, &qp);
    if (s != CP_SUCCESS) return s;
    qp.no_timing = true;  // the diagnostic timer would create CUDA events
    const size_t need = query_workspace_bytes(mesh->bvh, nq, qp);
    if (need > kScratchBytes)
        return set_error(CP_ERROR_SCRATCH_TOO_SMALL,
                         "cp_query_noalloc: " + std::to_string(nq) + " queries need " +
                             std::to_string(need) + " bytes of scratch but the fixed area holds " +
                             std::to_string(kScratchBytes) +
                             " (1,048,576 queries fit with sort_queries on); split the batch, "
                             "turn sort_queries off, or use cp_query");
    void* ws = nullptr;
    cudaError_t e = scratch_address(&ws);
    if (e != cudaSuccess)
        return set_error(CP_ERROR_CUDA, std::string("cp_query_noalloc: scratch address: ") +
                                            cudaGetErrorString(e));
    e = bvh_query(mesh->bvh, queries, nq, nullptr, qp, out_point, out_dist, out_tri, out_bary, ws,
                  kScratchBytes, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return set_error(CP_ERROR_CUDA, std::string("cp_query_noalloc: ") + cudaGetErrorString(e));
    return CP_SUCCESS;
}

extern "C" CP_API size_t cp_query_noalloc_scratch_bytes(void) { return kScratchBytes; }
