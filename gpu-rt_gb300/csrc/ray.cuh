// ray.cuh — ray queries through the closest-point BVH (ray.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "bvh.cuh"

namespace cpq {

struct RayParams {
    float tmin = 0.0f;
    float tmax = INFINITY;
    float det_eps = 0.0f;  // |det| <= det_eps is a miss (the reference's triangle_hit uses 1e-5)
    int any_hit = 0;       // stop at the first accepted hit (the reference's visibility())
    int sort = 1;          // walk rays in the Hilbert order of their origins
    int block = 256;
};

// Closest (or any) hit of n rays; origins and directions n x 3 floats,
// tmax_per_ray optional (segment ends).  Workspace: query_workspace_bytes(b,
// n, {sort}).  Outputs (each optional): t (+inf on a miss), triangle index
// (-1), weights (u, v) of b and c.
cudaError_t bvh_ray_query(const Bvh& b, const float* orig, const float* dir, const float* tmax_per_ray,
                          int64_t n, const int64_t* d_off, const RayParams& rp, float* out_t,
                          int32_t* out_tri, float* out_uv, void* ws, size_t ws_bytes, cudaStream_t st);

// Closest (or any) hit of n world-space rays over an instanced scene (top:
// BVH over the instances, bottom: the batch, is: the instances).  Outputs
// (each optional): t, instance, triangle local to the instance's mesh, (u, v).
// Workspace: query_workspace_bytes(top, n, {sort}).
cudaError_t scene_ray_query(const Bvh& top, const Bvh& bottom, const InstanceSet& is, const float* orig,
                            const float* dir, const float* tmax_per_ray, int64_t n, const RayParams& rp,
                            float* out_t, int32_t* out_inst, int32_t* out_tri, float* out_uv, void* ws,
                            size_t ws_bytes, cudaStream_t st);

}  // namespace cpq
