// Shapes of the learned radiance cache (cache.cu) shared with the integrator.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace tt {

constexpr int CACHE_LEVELS = 16;
constexpr uint32_t CACHE_TABLE = 1u << 19;  // entries per level
constexpr int CACHE_WIDTH = 64;             // network width (inputs padded to it)
constexpr int CACHE_HIDDEN_LAYERS = 4;
constexpr int CACHE_OUT_ROWS = 8;           // output layer rows (3 used)
constexpr uint32_t CACHE_PARAMS = CACHE_HIDDEN_LAYERS * CACHE_WIDTH * CACHE_WIDTH + CACHE_OUT_ROWS * CACHE_WIDTH;
constexpr uint64_t CACHE_GRID_PARAMS = 2ull * CACHE_TABLE * CACHE_LEVELS;

// One query: position in the cache's unit cube, outgoing direction, shading normal, roughness.
struct CacheQuery {
    float pos[3];
    float dir[3];
    float normal[3];
    float roughness;
    float pad[2];
};
static_assert(sizeof(CacheQuery) == 48, "48-byte cache queries");

// Device state: FP32 parameters and Adam moments, FP16 copies that the queries and the training
// forward pass read (grid features: two FP16 values per entry, one 32-bit load), gradients.
struct CacheDevice {
    float *grid, *grid_m, *grid_v, *grid_grad;  // CACHE_GRID_PARAMS each
    float *w, *w_m, *w_v, *w_grad;              // CACHE_PARAMS each
    __half* w16;                                // CACHE_PARAMS
    float* loss;                                // [0]: summed loss of the last step
    __half* grid16;                             // CACHE_GRID_PARAMS
};

// err: device error word (ERR_TENSOR_WAIT), may be null.
void cache_infer(const CacheDevice& d, const CacheQuery* q, uint32_t n, float* out, uint32_t* err, cudaStream_t st);
// One Adam step on n samples: gradients of the mean relative L2 loss.
void cache_train_step(const CacheDevice& d, const CacheQuery* q, const float* target, uint32_t n, float lr,
                      uint32_t step, uint32_t* err, cudaStream_t st);
// The gradients of one training step without the Adam update: d.w_grad / d.grid_grad receive
// the gradients of the mean relative L2 loss of the n pairs (they must start at zero; Adam
// consumes them, cache_clear_gradients zeroes them), d.loss the summed loss.
void cache_gradients(const CacheDevice& d, const CacheQuery* q, const float* target, uint32_t n, uint32_t* err,
                     cudaStream_t st);
void cache_clear_gradients(const CacheDevice& d, cudaStream_t st);
void cache_init(const CacheDevice& d, uint32_t seed, cudaStream_t st);
// Queries whose count is in device memory (at most max_n of them).
void cache_infer_queue(const __half* grid16, const __half* w16, const CacheQuery* q, const uint32_t* count,
                       uint32_t max_n, float* out, uint32_t* err, cudaStream_t st);
struct TrainRecord;
void cache_targets(const TrainRecord* rec, const uint32_t* rec_count, uint32_t cap, const float4* final_radiance,
                   CacheQuery* q, float* t, uint32_t* count, cudaStream_t st);
void cache_set_level_scales();

}  // namespace tt
