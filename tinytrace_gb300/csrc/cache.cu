// Learned radiance cache (an addition: the reference has none).  A multiresolution hash grid
// over position (Mueller, Evans, Schied & Keller 2022) plus the outgoing direction, shading
// normal and roughness feeds a small ReLU MLP predicting outgoing radiance, trained online on
// radiance the path tracer itself produces ("Real-time Neural Radiance Caching for Path
// Tracing", Mueller, Rousselle, Novak & Keller 2021).  Own implementation of the published
// methods; no third-party code.
//
//   grid      16 levels, 2^19 entries per level, 2 features per entry; level l has resolution
//             floor(16 * b^l), b = (2048 / 16)^(1/15); cells index a dense table while
//             (res + 1)^3 fits, else the spatial hash (x * 1) ^ (y * 2654435761) ^ (z * 805459861);
//             trilinear interpolation of the 8 corners.  Parameters in FP32, FP16 copy for queries.
//   MLP       64 inputs (32 grid features, direction * 0.5 + 0.5, normal * 0.5 + 0.5,
//             roughness, zero padding) -> 4 hidden layers of 64 ReLU units -> 3 outputs (RGB,
//             linear), no biases.  Weights [out][in] row-major, FP32 master copy, FP16 copy.
//   inference FP16 inputs and weights on the tensor cores (mma.sync m16n8k16, FP32
//             accumulation), 16 queries per warp, weights staged in shared memory, the hidden
//             activations passed from accumulator to operand registers between layers.
//   training  FP32 on the CUDA cores: forward, relative L2 loss (y - t)^2 / (y^2 + 0.01)
//             (y not differentiated in the denominator), backward into weight gradients
//             (shared-memory accumulation, one atomic per weight per block) and grid gradients
//             (atomics on the 8 corners), then Adam (beta 0.9 / 0.99, eps 1e-15).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "tt_cache.cuh"
#include "tt_internal.h"
#include "tt_kernels.h"

namespace tt {

// 16 * b^l, b = 128^(1/15), rounded from double precision on the host.
__constant__ float c_level_scale[CACHE_LEVELS];
__device__ __forceinline__ float level_scale(int l) { return c_level_scale[l]; }

void cache_set_level_scales() {
    float s[CACHE_LEVELS];
    for (int l = 0; l < CACHE_LEVELS; ++l) s[l] = (float)(16.0 * std::pow(128.0, (double)l / 15.0));
    check_cuda(cudaMemcpyToSymbol(c_level_scale, s, sizeof(s)), "level scales");
}

// Corner indices and trilinear weights of position p (in [0,1]^3) at level l.
__device__ __forceinline__ void grid_corners(const float3& p, int l, uint32_t* idx, float* w) {
    float scale = level_scale(l);
    uint32_t res = (uint32_t)scale + 1u;  // cells per axis + 1 corner
    float fx = p.x * scale, fy = p.y * scale, fz = p.z * scale;
    float x0 = floorf(fx), y0 = floorf(fy), z0 = floorf(fz);
    float tx = fx - x0, ty = fy - y0, tz = fz - z0;
    uint32_t ix = (uint32_t)x0, iy = (uint32_t)y0, iz = (uint32_t)z0;
    bool dense = (uint64_t)(res + 1u) * (res + 1u) * (res + 1u) <= (uint64_t)CACHE_TABLE;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        uint32_t cx = ix + (c & 1), cy = iy + ((c >> 1) & 1), cz = iz + ((c >> 2) & 1);
        uint32_t h = dense ? cx + (res + 1u) * (cy + (res + 1u) * cz)
                           : (cx * 1u) ^ (cy * 2654435761u) ^ (cz * 805459861u);
        idx[c] = h & (CACHE_TABLE - 1u);
        w[c] = ((c & 1) ? tx : 1.0f - tx) * ((c & 2) ? ty : 1.0f - ty) * ((c & 4) ? tz : 1.0f - tz);
    }
}

// The 64 network inputs of one query (FP32).
__device__ __forceinline__ void encode(const CacheQuery& q, const float* grid, float* x) {
    float3 p = make_float3(fminf(fmaxf(q.pos[0], 0.0f), 1.0f), fminf(fmaxf(q.pos[1], 0.0f), 1.0f),
                           fminf(fmaxf(q.pos[2], 0.0f), 1.0f));
    for (int l = 0; l < CACHE_LEVELS; ++l) {
        uint32_t idx[8];
        float w[8];
        grid_corners(p, l, idx, w);
        float f0 = 0.0f, f1 = 0.0f;
        const float* g = grid + 2ull * CACHE_TABLE * l;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            f0 += w[c] * g[2ull * idx[c]];
            f1 += w[c] * g[2ull * idx[c] + 1];
        }
        x[2 * l] = f0;
        x[2 * l + 1] = f1;
    }
    for (int k = 0; k < 3; ++k) {
        x[32 + k] = q.dir[k] * 0.5f + 0.5f;
        x[35 + k] = q.normal[k] * 0.5f + 0.5f;
    }
    x[38] = q.roughness;
    for (int k = 39; k < CACHE_WIDTH; ++k) x[k] = 0.0f;
}

// ---------------------------------------------------------------- inference (tensor cores)
__device__ __forceinline__ uint32_t pack_half2(float a, float b) {
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

constexpr int INF_WARPS = 4;

// out[i] = MLP(encode(q[i])) for n queries; the FP16 weights (CACHE_PARAMS halves) are copied
// to shared memory once per block.
__global__ void __launch_bounds__(INF_WARPS * 32) cache_infer_kernel(const CacheQuery* q, uint32_t n,
                                                                     const uint32_t* count, const float* grid,
                                                                     const __half* w16, float* out) {
    if (count) n = min(n, *count);  // queue length written by an earlier kernel
    __shared__ __align__(16) __half s_w[CACHE_PARAMS];
    __shared__ __align__(16) __half s_x[INF_WARPS][16][CACHE_WIDTH + 8];  // +8: spread smem banks
    for (uint32_t k = threadIdx.x; k < CACHE_PARAMS / 8; k += blockDim.x)
        reinterpret_cast<uint4*>(s_w)[k] = reinterpret_cast<const uint4*>(w16)[k];
    __syncthreads();
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t tiles = (n + 15u) / 16u;
    for (uint32_t tile = blockIdx.x * INF_WARPS + warp; tile < tiles; tile += gridDim.x * INF_WARPS) {
        // encode: two lanes per query row, the first does levels 0..7 and the extras
        uint32_t row = lane >> 1, half_ = lane & 1;
        uint32_t i = tile * 16u + row;
        float x[CACHE_WIDTH];
        if (i < n) {
            encode(q[i], grid, x);
        } else {
            for (int k = 0; k < CACHE_WIDTH; ++k) x[k] = 0.0f;
        }
        for (int k = half_ * 32; k < half_ * 32 + 32; ++k) s_x[warp][row][k] = __float2half_rn(x[k]);
        __syncwarp();
        // layer 0: A from shared memory
        uint32_t a[4][4];
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            a[kk][0] = *reinterpret_cast<const uint32_t*>(&s_x[warp][g][16 * kk + 2 * t]);
            a[kk][1] = *reinterpret_cast<const uint32_t*>(&s_x[warp][g + 8][16 * kk + 2 * t]);
            a[kk][2] = *reinterpret_cast<const uint32_t*>(&s_x[warp][g][16 * kk + 2 * t + 8]);
            a[kk][3] = *reinterpret_cast<const uint32_t*>(&s_x[warp][g + 8][16 * kk + 2 * t + 8]);
        }
        __syncwarp();
        for (int layer = 0; layer < CACHE_HIDDEN_LAYERS; ++layer) {
            const __half* W = s_w + layer * CACHE_WIDTH * CACHE_WIDTH;
            float c[8][4];
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    uint32_t b[2];
                    const __half* wr = W + (8 * nt + g) * CACHE_WIDTH + 16 * kk + 2 * t;
                    b[0] = *reinterpret_cast<const uint32_t*>(wr);
                    b[1] = *reinterpret_cast<const uint32_t*>(wr + 8);
                    mma16816(c[nt], a[kk], b);
                }
            }
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {  // ReLU, then the accumulators become the next A
                a[kk][0] = pack_half2(fmaxf(c[2 * kk][0], 0.0f), fmaxf(c[2 * kk][1], 0.0f));
                a[kk][1] = pack_half2(fmaxf(c[2 * kk][2], 0.0f), fmaxf(c[2 * kk][3], 0.0f));
                a[kk][2] = pack_half2(fmaxf(c[2 * kk + 1][0], 0.0f), fmaxf(c[2 * kk + 1][1], 0.0f));
                a[kk][3] = pack_half2(fmaxf(c[2 * kk + 1][2], 0.0f), fmaxf(c[2 * kk + 1][3], 0.0f));
            }
        }
        // output layer: 8 rows of W (3 used), one n-tile
        const __half* W = s_w + CACHE_HIDDEN_LAYERS * CACHE_WIDTH * CACHE_WIDTH;
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            uint32_t b[2];
            const __half* wr = W + g * CACHE_WIDTH + 16 * kk + 2 * t;
            b[0] = *reinterpret_cast<const uint32_t*>(wr);
            b[1] = *reinterpret_cast<const uint32_t*>(wr + 8);
            mma16816(c, a[kk], b);
        }
        // c[0], c[1]: row g, columns 2t, 2t+1; c[2], c[3]: row g + 8
        uint32_t i0 = tile * 16u + g, i1 = i0 + 8u;
        for (int h = 0; h < 2; ++h) {
            int col = 2 * t + h;
            if (col < 3) {
                if (i0 < n) out[3ull * i0 + col] = c[h];
                if (i1 < n) out[3ull * i1 + col] = c[2 + h];
            }
        }
    }
}

// ---------------------------------------------------------------- training (FP32)
constexpr int TRAIN_THREADS = 64;  // one per neuron
constexpr int TRAIN_CHUNK = 32;    // samples per pass through the network
constexpr uint32_t TRAIN_SMEM =
    sizeof(float) * (CACHE_PARAMS * 2 + 5 * TRAIN_CHUNK * CACHE_WIDTH + 2 * TRAIN_CHUNK * CACHE_WIDTH + 2 * TRAIN_CHUNK * 3);

__global__ void __launch_bounds__(TRAIN_THREADS) cache_train_kernel(const CacheQuery* q, const float* target,
                                                                    uint32_t n, const float* grid, const float* w,
                                                                    float* w_grad, float* grid_grad, float* loss,
                                                                    float inv_count) {
    extern __shared__ float sm[];
    float* s_w = sm;                                      // CACHE_PARAMS
    float* s_dw = s_w + CACHE_PARAMS;                     // CACHE_PARAMS
    float* act = s_dw + CACHE_PARAMS;                     // [5][CHUNK][64]: input, hidden 1..4
    float* delta = act + 5 * TRAIN_CHUNK * CACHE_WIDTH;   // [2][CHUNK][64]
    float* y = delta + 2 * TRAIN_CHUNK * CACHE_WIDTH;     // [CHUNK][3]
    float* dy = y + TRAIN_CHUNK * 3;                      // [CHUNK][3]
    const int j = threadIdx.x;
    for (uint32_t k = j; k < CACHE_PARAMS; k += TRAIN_THREADS) {
        s_w[k] = w[k];
        s_dw[k] = 0.0f;
    }
    float block_loss = 0.0f;
    uint32_t chunks = (n + TRAIN_CHUNK - 1) / TRAIN_CHUNK;
    for (uint32_t chunk = blockIdx.x; chunk < chunks; chunk += gridDim.x) {
        uint32_t base = chunk * TRAIN_CHUNK;
        __syncthreads();
        if (j < TRAIN_CHUNK) {
            float x[CACHE_WIDTH];
            if (base + j < n) encode(q[base + j], grid, x);
            else for (int k = 0; k < CACHE_WIDTH; ++k) x[k] = 0.0f;
            for (int k = 0; k < CACHE_WIDTH; ++k) act[j * CACHE_WIDTH + k] = x[k];
        }
        __syncthreads();
        for (int l = 0; l < CACHE_HIDDEN_LAYERS; ++l) {  // forward
            const float* W = s_w + l * CACHE_WIDTH * CACHE_WIDTH + j * CACHE_WIDTH;
            const float* in = act + l * TRAIN_CHUNK * CACHE_WIDTH;
            float* out = act + (l + 1) * TRAIN_CHUNK * CACHE_WIDTH;
            for (int s = 0; s < TRAIN_CHUNK; ++s) {
                float z = 0.0f;
                for (int k = 0; k < CACHE_WIDTH; ++k) z += W[k] * in[s * CACHE_WIDTH + k];
                out[s * CACHE_WIDTH + j] = fmaxf(z, 0.0f);
            }
            __syncthreads();
        }
        const float* Wo = s_w + CACHE_HIDDEN_LAYERS * CACHE_WIDTH * CACHE_WIDTH;
        const float* h4 = act + 4 * TRAIN_CHUNK * CACHE_WIDTH;
        if (j < 3) {  // output and loss gradient
            for (int s = 0; s < TRAIN_CHUNK; ++s) {
                float z = 0.0f;
                for (int k = 0; k < CACHE_WIDTH; ++k) z += Wo[j * CACHE_WIDTH + k] * h4[s * CACHE_WIDTH + k];
                y[s * 3 + j] = z;
                float g = 0.0f;
                if (base + s < n) {
                    float d = z - target[3ull * (base + s) + j];
                    float den = z * z + 0.01f;
                    block_loss += d * d / den;
                    g = 2.0f * d / den * inv_count;
                }
                dy[s * 3 + j] = g;
            }
        }
        __syncthreads();
        float* dcur = delta;
        float* dnext = delta + TRAIN_CHUNK * CACHE_WIDTH;
        {  // output layer: weight gradients (rows 0..2) and the delta of hidden layer 4
            for (int r = 0; r < 3; ++r) {
                float acc = 0.0f;
                for (int s = 0; s < TRAIN_CHUNK; ++s) acc += dy[s * 3 + r] * h4[s * CACHE_WIDTH + j];
                s_dw[CACHE_HIDDEN_LAYERS * CACHE_WIDTH * CACHE_WIDTH + r * CACHE_WIDTH + j] += acc;
            }
            for (int s = 0; s < TRAIN_CHUNK; ++s) {
                float d = 0.0f;
                for (int r = 0; r < 3; ++r) d += Wo[r * CACHE_WIDTH + j] * dy[s * 3 + r];
                dcur[s * CACHE_WIDTH + j] = h4[s * CACHE_WIDTH + j] > 0.0f ? d : 0.0f;
            }
        }
        __syncthreads();
        for (int l = CACHE_HIDDEN_LAYERS - 1; l >= 0; --l) {  // hidden layers, last to first
            const float* in = act + l * TRAIN_CHUNK * CACHE_WIDTH;
            const float* W = s_w + l * CACHE_WIDTH * CACHE_WIDTH;
            float* dW = s_dw + l * CACHE_WIDTH * CACHE_WIDTH;
            for (int k = 0; k < CACHE_WIDTH; ++k) {  // row j of dW_l
                float acc = 0.0f;
                for (int s = 0; s < TRAIN_CHUNK; ++s) acc += dcur[s * CACHE_WIDTH + j] * in[s * CACHE_WIDTH + k];
                dW[j * CACHE_WIDTH + k] += acc;
            }
            for (int s = 0; s < TRAIN_CHUNK; ++s) {  // delta of this layer's input, component j
                float d = 0.0f;
                for (int r = 0; r < CACHE_WIDTH; ++r) d += W[r * CACHE_WIDTH + j] * dcur[s * CACHE_WIDTH + r];
                dnext[s * CACHE_WIDTH + j] = (l == 0 || in[s * CACHE_WIDTH + j] > 0.0f) ? d : 0.0f;
            }
            __syncthreads();
            float* tmp = dcur;
            dcur = dnext;
            dnext = tmp;
        }
        // dcur: gradient of the inputs; grid features are inputs 0..31
        if (j < TRAIN_CHUNK && base + j < n) {
            const CacheQuery& qq = q[base + j];
            float3 p = make_float3(fminf(fmaxf(qq.pos[0], 0.0f), 1.0f), fminf(fmaxf(qq.pos[1], 0.0f), 1.0f),
                                   fminf(fmaxf(qq.pos[2], 0.0f), 1.0f));
            for (int l = 0; l < CACHE_LEVELS; ++l) {
                uint32_t idx[8];
                float wc[8];
                grid_corners(p, l, idx, wc);
                float g0 = dcur[j * CACHE_WIDTH + 2 * l], g1 = dcur[j * CACHE_WIDTH + 2 * l + 1];
                float* gg = grid_grad + 2ull * CACHE_TABLE * l;
                for (int c = 0; c < 8; ++c) {
                    if (g0 != 0.0f) atomicAdd(gg + 2ull * idx[c], wc[c] * g0);
                    if (g1 != 0.0f) atomicAdd(gg + 2ull * idx[c] + 1, wc[c] * g1);
                }
            }
        }
    }
    __syncthreads();
    for (uint32_t k = j; k < CACHE_PARAMS; k += TRAIN_THREADS)
        if (s_dw[k] != 0.0f) atomicAdd(w_grad + k, s_dw[k]);
    if (j < 3 && block_loss != 0.0f) atomicAdd(loss, block_loss);
}

// Adam on `count` parameters; the gradient is consumed (zeroed).  FP16 copy when w16 != null.
__global__ void cache_adam_kernel(float* p, float* m, float* v, float* grad, __half* p16, uint64_t count, float lr,
                                  float c1, float c2) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= count) return;
    float g = grad[i];
    grad[i] = 0.0f;
    float mi = 0.9f * m[i] + 0.1f * g;
    float vi = 0.99f * v[i] + 0.01f * g * g;
    m[i] = mi;
    v[i] = vi;
    float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + 1e-15f);
    p[i] = pi;
    if (p16) p16[i] = __float2half_rn(pi);
}

// Deterministic initialisation: weights uniform in +-sqrt(6 / (fan_in + fan_out)), grid
// features uniform in +-1e-4; Adam moments and gradients zero.
__device__ __forceinline__ float hash_uniform(uint64_t i, uint32_t seed) {
    uint32_t h = (uint32_t)(i * 0x9E3779B97F4A7C15ull >> 32) ^ seed;
    h ^= h >> 16;
    h *= 0x7feb352du;
    h ^= h >> 15;
    h *= 0x846ca68bu;
    h ^= h >> 16;
    return (float)(h >> 8) * (1.0f / 16777216.0f);  // [0, 1)
}
__global__ void cache_init_kernel(float* grid, float* w, __half* w16, uint32_t seed) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < CACHE_GRID_PARAMS) grid[i] = (hash_uniform(i, seed) * 2.0f - 1.0f) * 1e-4f;
    if (i < CACHE_PARAMS) {
        float bound = sqrtf(6.0f / (i < CACHE_HIDDEN_LAYERS * CACHE_WIDTH * CACHE_WIDTH ? 128.0f : 67.0f));
        bool unused = i >= CACHE_HIDDEN_LAYERS * CACHE_WIDTH * CACHE_WIDTH &&
                      (i - CACHE_HIDDEN_LAYERS * CACHE_WIDTH * CACHE_WIDTH) >= 3u * CACHE_WIDTH;
        float x = unused ? 0.0f : (hash_uniform(i + CACHE_GRID_PARAMS, seed) * 2.0f - 1.0f) * bound;
        w[i] = x;
        w16[i] = __float2half_rn(x);
    }
}

void cache_infer(const CacheDevice& d, const CacheQuery* q, uint32_t n, float* out, cudaStream_t st) {
    if (n == 0) return;
    uint32_t tiles = (n + 15u) / 16u;
    uint32_t blocks = std::min<uint32_t>((tiles + INF_WARPS - 1) / INF_WARPS, 152u * 8u);
    cache_infer_kernel<<<blocks, INF_WARPS * 32, 0, st>>>(q, n, nullptr, d.grid, d.w16, out);
}

void cache_infer_queue(const float* grid, const __half* w16, const CacheQuery* q, const uint32_t* count,
                       uint32_t max_n, float* out, cudaStream_t st) {
    if (max_n == 0) return;
    uint32_t tiles = (max_n + 15u) / 16u;
    uint32_t blocks = std::min<uint32_t>((tiles + INF_WARPS - 1) / INF_WARPS, 152u * 8u);
    cache_infer_kernel<<<blocks, INF_WARPS * 32, 0, st>>>(q, max_n, count, grid, w16, out);
}

// Training pairs of the frame's records: target = (final - before) / throughput, kept when the
// throughput is above 1e-6 in every channel and the target is finite; order not preserved.
__global__ void cache_targets_kernel(const TrainRecord* rec, const uint32_t* rec_count, uint32_t cap,
                                     const float4* final_radiance, CacheQuery* q, float* t, uint32_t* count) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t n = min(*rec_count, cap);
    if (i >= n) return;
    const TrainRecord& r = rec[i];
    float4 f = final_radiance[r.path];
    float fin[3] = {f.x, f.y, f.z};
    float tg[3];
    bool ok = true;
    for (int c = 0; c < 3; ++c) {
        ok = ok && r.thr[c] > 1e-6f;
        tg[c] = (fin[c] - r.before[c]) / r.thr[c];
        ok = ok && isfinite(tg[c]);
    }
    if (!ok) return;
    uint32_t k = atomicAdd(count, 1u);
    for (int c = 0; c < 12; ++c) reinterpret_cast<float*>(q + k)[c] = r.q[c];
    for (int c = 0; c < 3; ++c) t[3ull * k + c] = fmaxf(tg[c], 0.0f);
}

void cache_targets(const TrainRecord* rec, const uint32_t* rec_count, uint32_t cap, const float4* final_radiance,
                   CacheQuery* q, float* t, uint32_t* count, cudaStream_t st) {
    check_cuda(cudaMemsetAsync(count, 0, 4, st), "memset");
    if (cap == 0) return;
    cache_targets_kernel<<<(cap + 255) / 256, 256, 0, st>>>(rec, rec_count, cap, final_radiance, q, t, count);
}

void cache_train_step(const CacheDevice& d, const CacheQuery* q, const float* target, uint32_t n, float lr,
                      uint32_t step, cudaStream_t st) {
    if (n == 0) return;
    static bool attr = false;
    if (!attr) {
        check_cuda(cudaFuncSetAttribute(cache_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TRAIN_SMEM),
                   "train smem");
        attr = true;
    }
    uint32_t chunks = (n + TRAIN_CHUNK - 1) / TRAIN_CHUNK;
    uint32_t blocks = std::min<uint32_t>(chunks, 152u);
    check_cuda(cudaMemsetAsync(d.loss, 0, 4, st), "memset");
    cache_train_kernel<<<blocks, TRAIN_THREADS, TRAIN_SMEM, st>>>(q, target, n, d.grid, d.w, d.w_grad, d.grid_grad,
                                                                  d.loss, 1.0f / (3.0f * (float)n));
    float c1 = 1.0f - std::pow(0.9f, (float)step), c2 = 1.0f - std::pow(0.99f, (float)step);
    cache_adam_kernel<<<(CACHE_PARAMS + 255) / 256, 256, 0, st>>>(d.w, d.w_m, d.w_v, d.w_grad, d.w16, CACHE_PARAMS,
                                                                  lr, c1, c2);
    cache_adam_kernel<<<(unsigned)((CACHE_GRID_PARAMS + 255) / 256), 256, 0, st>>>(
        d.grid, d.grid_m, d.grid_v, d.grid_grad, nullptr, CACHE_GRID_PARAMS, lr, c1, c2);
}

void cache_init(const CacheDevice& d, uint32_t seed, cudaStream_t st) {
    cache_init_kernel<<<(unsigned)((CACHE_GRID_PARAMS + 255) / 256), 256, 0, st>>>(d.grid, d.w, d.w16, seed);
    check_cuda(cudaMemsetAsync(d.grid_m, 0, 4 * CACHE_GRID_PARAMS, st), "memset");
    check_cuda(cudaMemsetAsync(d.grid_v, 0, 4 * CACHE_GRID_PARAMS, st), "memset");
    check_cuda(cudaMemsetAsync(d.grid_grad, 0, 4 * CACHE_GRID_PARAMS, st), "memset");
    check_cuda(cudaMemsetAsync(d.w_m, 0, 4 * CACHE_PARAMS, st), "memset");
    check_cuda(cudaMemsetAsync(d.w_v, 0, 4 * CACHE_PARAMS, st), "memset");
    check_cuda(cudaMemsetAsync(d.w_grad, 0, 4 * CACHE_PARAMS, st), "memset");
}

}  // namespace tt
