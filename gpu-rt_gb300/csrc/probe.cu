// probe.cu — read-bandwidth probe used for the roofline denominator of the
// traversal kernel: 128-bit loads over an L2-resident buffer (the traversal
// reads its nodes and triangle records the same way).  A diagnostic with no
// counterpart in the reference.
#include <cuda_runtime.h>

#include "../../include/cpq.h"
#include "common.cuh"

namespace {

// Four independent 128-bit loads in flight per thread per iteration.
__global__ void __launch_bounds__(256) k_probe_read(const float4* __restrict__ buf, int64_t n4,
                                                    int reps, float* __restrict__ sink) {
    float acc = 0.0f;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int r = 0; r < reps; ++r) {
        int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        for (; i + 3 * stride < n4; i += 4 * stride) {
            const float4 v0 = __ldcg(buf + i);  // L2, not L1
            const float4 v1 = __ldcg(buf + i + stride);
            const float4 v2 = __ldcg(buf + i + 2 * stride);
            const float4 v3 = __ldcg(buf + i + 3 * stride);
            acc += (v0.x + v1.y) + (v2.z + v3.w);
        }
        for (; i < n4; i += stride) {
            const float4 v = __ldcg(buf + i);
            acc += v.x;
        }
    }
    if (acc == 1234.5f) sink[0] = acc;  // keeps the loads alive
}

}  // namespace

extern "C" CP_API cp_status cp_probe_read_bandwidth(int64_t bytes, int32_t reps, double* gbs,
                                                    cp_stream_t stream) {
    if (!gbs || bytes < (1 << 20) || reps < 1) return CP_ERROR_INVALID_VALUE;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int64_t n4 = bytes / 16;
    float4* buf = nullptr;
    float* sink = nullptr;
    if (cudaMalloc(&buf, n4 * 16) != cudaSuccess) return CP_ERROR_OUT_OF_MEMORY;
    if (cudaMalloc(&sink, 4) != cudaSuccess) {
        cudaFree(buf);
        return CP_ERROR_OUT_OF_MEMORY;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaMemsetAsync(buf, 0, n4 * 16, st);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // best over 4, 8 and 16 resident blocks per SM, 5 timed launches each
    float best_ms = 1e30f;
    for (int per_sm = 4; per_sm <= 16; per_sm *= 2) {
        const unsigned grid = (unsigned)sms * per_sm;
        k_probe_read<<<grid, 256, 0, st>>>(buf, n4, 2, sink);  // warm: brings the buffer into L2
        cpq::note_launch();
        for (int t = 0; t < 5; ++t) {
            cudaEventRecord(e0, st);
            k_probe_read<<<grid, 256, 0, st>>>(buf, n4, reps, sink);
            cpq::note_launch();
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best_ms) best_ms = ms;
        }
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    cudaFree(sink);
    if (e != cudaSuccess) return CP_ERROR_CUDA;
    *gbs = (double)n4 * 16.0 * reps / (best_ms * 1e-3) / 1e9;
    return CP_SUCCESS;
}
