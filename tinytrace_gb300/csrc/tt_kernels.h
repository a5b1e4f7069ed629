// Kernel launch interface between the C ABI (api.cu) and the device code (integrate.cu).
#pragma once

#include <cuda_runtime.h>

#include "../../include/tinytrace_cuda.h"
#include "tt_bvh.cuh"

namespace tt {

struct RenderParams {
    DevScene sc;
    tt_constants c;
    float4* target;
    uint32_t* err;
    unsigned long long* counters;  // 6 counters, instrumented kernel only
};

void launch_integrate(const RenderParams& p, bool counted, cudaStream_t st);
void launch_tonemap(const float4* in, uint64_t n, uint32_t tonemap, uint32_t format, void* out,
                    cudaStream_t st);
void launch_bsdf_eval(const tt_material_constants* m, const float4* samples, uint32_t n,
                      float4* results, cudaStream_t st);
void launch_bsdf_sample(const tt_material_constants* m, const float4* samples, uint32_t n,
                        float4* results, cudaStream_t st);
void launch_trace(const DevScene& sc, const float4* rays, uint32_t n, uint32_t flags, uint4* hits,
                  uint32_t* err, cudaStream_t st);
void launch_math(int which, const float* x, uint64_t n, float* y, cudaStream_t st);
// Ray queries staged in the library's static device array (no device allocation).
void trace_batch_noalloc(int device, const DevScene& sc, const float* rays_host, uint32_t n,
                         uint32_t flags, uint32_t* hits_host, cudaStream_t st);

}  // namespace tt
