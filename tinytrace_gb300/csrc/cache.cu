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
//   inference FP16 inputs and weights on the 5th-generation tensor cores (tcgen05.mma, FP32
//             accumulation in tensor memory), 128 queries per CTA, weights and activations in
//             shared memory, ReLU and FP16 conversion between layers on the CUDA cores.
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

// ---------------------------------------------------------------- inference (tcgen05 tensor cores)
// One CTA of 128 threads owns 128 queries at a time (thread t: query row t).  Per layer the
// activations A (128 x 64 FP16) and the layer's weights B (64 x 64 FP16, [out][in]) sit in
// shared memory in the canonical K-major layout without swizzling: 8-row x 16-byte core
// matrices, the 8 core matrices of a row group 128 bytes apart along K (leading byte offset)
// and row groups 1024 bytes apart (stride byte offset).  One thread issues the layer's four
// tcgen05.mma (M 128, N 64, K 16, FP32 accumulation in 64 TMEM columns) and commits them to
// an mbarrier; every warp then reads its 32 TMEM lanes (tcgen05.ld 32x32b), applies ReLU,
// converts to FP16 and writes the next layer's A.  The output layer uses N 16 (3 rows used).
// Waits on the mbarrier are bounded: past the limit the kernel raises ERR_TENSOR_WAIT, stops
// issuing, and still releases its TMEM.
constexpr int TC_THREADS = 128;
constexpr int TC_ROWS = 128;
constexpr uint32_t TC_TMEM_COLS = 64;
constexpr uint32_t TC_OUT_N = 16;
constexpr uint32_t TC_WAIT_LIMIT = 1u << 24;
// dynamic shared memory: hidden weights, output weights, activations, mbarrier, TMEM address
constexpr uint32_t TC_W_BYTES = CACHE_WIDTH * CACHE_WIDTH * 2;     // 8 KB per hidden layer
constexpr uint32_t TC_WOUT_BYTES = TC_OUT_N * CACHE_WIDTH * 2;     // 2 KB
constexpr uint32_t TC_A_BYTES = TC_ROWS * CACHE_WIDTH * 2;         // 16 KB
constexpr uint32_t TC_OFF_WOUT = CACHE_HIDDEN_LAYERS * TC_W_BYTES;
constexpr uint32_t TC_OFF_A = TC_OFF_WOUT + TC_WOUT_BYTES;
constexpr uint32_t TC_OFF_BAR = TC_OFF_A + TC_A_BYTES;
constexpr uint32_t TC_SMEM = TC_OFF_BAR + 16 + 1024;  // + alignment slack

// Byte offset of element (row, k) of a 64-wide K-major operand in the core-matrix layout.
__device__ __forceinline__ uint32_t core_offset(uint32_t row, uint32_t k) {
    return (row >> 3) * 1024u + (k >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, leading byte offset 128, stride byte offset
// 1024 (all >> 4), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(1024u >> 4) << 32) |
           (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, FP16 A and B, both K-major, M = 128.
__host__ __device__ constexpr uint32_t mma_idesc(uint32_t n) { return (1u << 4) | ((n >> 3) << 17) | ((128u >> 4) << 24); }

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar) : "memory");
}
// Bounded wait for the mbarrier phase `parity`; false when the limit ran out.
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t it = 0; it < TC_WAIT_LIMIT; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ uint32_t pack_half2(float a, float b) {
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

// The 64 FP16 inputs of one query written straight into row `row` of the A operand, 16 bytes
// (8 inputs) at a time: the grid features of levels 4c..4c+3 (float2 gathers of the 8 corners),
// then direction, normal, roughness and zero padding.  Same values as encode().
__device__ __forceinline__ void encode_row(const CacheQuery& q, const float* grid, uint8_t* a, uint32_t row) {
    float3 p = make_float3(fminf(fmaxf(q.pos[0], 0.0f), 1.0f), fminf(fmaxf(q.pos[1], 0.0f), 1.0f),
                           fminf(fmaxf(q.pos[2], 0.0f), 1.0f));
#pragma unroll 1
    for (int c = 0; c < CACHE_LEVELS / 4; ++c) {
        uint32_t h[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int l = 4 * c + j;
            uint32_t idx[8];
            float w[8];
            grid_corners(p, l, idx, w);
            const float2* g = reinterpret_cast<const float2*>(grid + 2ull * CACHE_TABLE * l);
            float f0 = 0.0f, f1 = 0.0f;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                float2 v = __ldg(g + idx[k]);
                f0 += w[k] * v.x;
                f1 += w[k] * v.y;
            }
            h[j] = pack_half2(f0, f1);
        }
        *reinterpret_cast<uint4*>(a + core_offset(row, 8u * c)) = make_uint4(h[0], h[1], h[2], h[3]);
    }
    *reinterpret_cast<uint4*>(a + core_offset(row, 32u)) =
        make_uint4(pack_half2(q.dir[0] * 0.5f + 0.5f, q.dir[1] * 0.5f + 0.5f),
                   pack_half2(q.dir[2] * 0.5f + 0.5f, q.normal[0] * 0.5f + 0.5f),
                   pack_half2(q.normal[1] * 0.5f + 0.5f, q.normal[2] * 0.5f + 0.5f), pack_half2(q.roughness, 0.0f));
#pragma unroll
    for (int c = 5; c < 8; ++c) *reinterpret_cast<uint4*>(a + core_offset(row, 8u * c)) = make_uint4(0u, 0u, 0u, 0u);
}
__device__ __forceinline__ void zero_row(uint8_t* a, uint32_t row) {
#pragma unroll
    for (int c = 0; c < 8; ++c) *reinterpret_cast<uint4*>(a + core_offset(row, 8u * c)) = make_uint4(0u, 0u, 0u, 0u);
}
// 16 accumulator columns (c0..c0+15) of row `row`, ReLU, FP16, into the A operand.
__device__ __forceinline__ void store_relu16(uint8_t* a, uint32_t row, uint32_t c0, const float* v) {
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const float* x = v + 8 * j;
        uint4 u = make_uint4(pack_half2(fmaxf(x[0], 0.0f), fmaxf(x[1], 0.0f)),
                             pack_half2(fmaxf(x[2], 0.0f), fmaxf(x[3], 0.0f)),
                             pack_half2(fmaxf(x[4], 0.0f), fmaxf(x[5], 0.0f)),
                             pack_half2(fmaxf(x[6], 0.0f), fmaxf(x[7], 0.0f)));
        *reinterpret_cast<uint4*>(a + core_offset(row, c0 + 8u * j)) = u;
    }
}

// out[i] = MLP(encode(q[i])) for n queries (n = min(n, *count) when count is given).
__global__ void __launch_bounds__(TC_THREADS) cache_infer_tc_kernel(const CacheQuery* q, uint32_t n,
                                                                    const uint32_t* count, const float* grid,
                                                                    const __half* w16, float* out, uint32_t* err) {
    extern __shared__ uint8_t tc_smem_raw[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023u) & ~uintptr_t(1023));
    uint8_t* s_a = sm + TC_OFF_A;
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(sm + TC_OFF_BAR);
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(sm + TC_OFF_BAR + 8);
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    if (count) n = min(n, *count);

    // weights into the core-matrix layout: hidden layers [n][k], then 16 output rows (3..15 zero)
    for (uint32_t c = tid; c < CACHE_HIDDEN_LAYERS * CACHE_WIDTH * 8u; c += TC_THREADS) {
        uint32_t layer = c / (CACHE_WIDTH * 8u), r = (c / 8u) % CACHE_WIDTH, j = c % 8u;
        uint4 v = reinterpret_cast<const uint4*>(w16 + (uint64_t)layer * CACHE_WIDTH * CACHE_WIDTH +
                                                 (uint64_t)r * CACHE_WIDTH)[j];
        *reinterpret_cast<uint4*>(sm + layer * TC_W_BYTES + core_offset(r, 8u * j)) = v;
    }
    for (uint32_t c = tid; c < TC_OUT_N * 8u; c += TC_THREADS) {
        uint32_t r = c / 8u, j = c % 8u;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (r < (uint32_t)CACHE_OUT_ROWS)
            v = reinterpret_cast<const uint4*>(w16 + (uint64_t)CACHE_HIDDEN_LAYERS * CACHE_WIDTH * CACHE_WIDTH +
                                               (uint64_t)r * CACHE_WIDTH)[j];
        *reinterpret_cast<uint4*>(sm + TC_OFF_WOUT + core_offset(r, 8u * j)) = v;
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(s_bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(s_tmem)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_tmem;
    const uint32_t bar = smem_u32(s_bar);
    const uint32_t a_addr = smem_u32(s_a), w_addr = smem_u32(sm);
    const uint32_t lane_taddr = tmem + ((32u * warp) << 16);
    uint32_t phase = 0;
    bool ok = true;
    const uint32_t tiles = (n + TC_ROWS - 1u) / TC_ROWS;
    for (uint32_t tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        uint32_t i = tile * TC_ROWS + tid;
        if (i < n) encode_row(q[i], grid, s_a, tid);
        else zero_row(s_a, tid);
        for (int layer = 0; layer <= CACHE_HIDDEN_LAYERS && ok; ++layer) {
            const bool last = layer == CACHE_HIDDEN_LAYERS;
            fence_async_smem();
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            if (tid == 0) {
                uint32_t b_addr = last ? w_addr + TC_OFF_WOUT : w_addr + (uint32_t)layer * TC_W_BYTES;
                uint32_t idesc = mma_idesc(last ? TC_OUT_N : (uint32_t)CACHE_WIDTH);
#pragma unroll
                for (uint32_t kk = 0; kk < CACHE_WIDTH / 16; ++kk)
                    mma_f16(tmem, smem_desc(a_addr + 256u * kk), smem_desc(b_addr + 256u * kk), idesc, kk);
                mma_commit(bar);
            }
            ok = __syncthreads_and(bar_wait(bar, phase) ? 1 : 0) != 0;  // one verdict for the whole CTA
            phase ^= 1u;
            tc_fence_after();
            if (!ok) break;
            if (!last) {
#pragma unroll
                for (int c = 0; c < CACHE_WIDTH; c += 16) {
                    float v[16];
                    tmem_ld16(lane_taddr + (uint32_t)c, v);
                    tmem_ld_wait();
                    store_relu16(s_a, tid, (uint32_t)c, v);
                }
            } else {
                float v[16];
                tmem_ld16(lane_taddr, v);
                tmem_ld_wait();
                if (i < n) {
                    out[3ull * i] = v[0];
                    out[3ull * i + 1] = v[1];
                    out[3ull * i + 2] = v[2];
                }
            }
        }
    }
    if (!ok && err) atomicOr(err, ERR_TENSOR_WAIT);
    // every MMA of this CTA was waited for (or the wait ran out and nothing more was issued)
    tc_fence_before();
    __syncthreads();
    if (!ok) bar_wait(bar, phase ^ 1u);  // one more bounded wait for the last commit in flight
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_TMEM_COLS)
                     : "memory");
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

static void launch_infer(const CacheQuery* q, uint32_t n, const uint32_t* count, const float* grid,
                         const __half* w16, float* out, uint32_t* err, cudaStream_t st) {
    if (n == 0) return;
    static bool attr = false;
    if (!attr) {
        check_cuda(cudaFuncSetAttribute(cache_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM),
                   "infer smem");
        attr = true;
    }
    uint32_t tiles = (n + TC_ROWS - 1u) / TC_ROWS;
    uint32_t blocks = std::min<uint32_t>(tiles, 152u * 4u);
    cache_infer_tc_kernel<<<blocks, TC_THREADS, TC_SMEM, st>>>(q, n, count, grid, w16, out, err);
}

void cache_infer(const CacheDevice& d, const CacheQuery* q, uint32_t n, float* out, uint32_t* err, cudaStream_t st) {
    launch_infer(q, n, nullptr, d.grid, d.w16, out, err, st);
}

void cache_infer_queue(const float* grid, const __half* w16, const CacheQuery* q, const uint32_t* count,
                       uint32_t max_n, float* out, uint32_t* err, cudaStream_t st) {
    launch_infer(q, max_n, count, grid, w16, out, err, st);
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
