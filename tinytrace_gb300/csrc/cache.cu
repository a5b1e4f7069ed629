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
//   training  FP16 in, FP32 accumulate on the tensor cores (tcgen05): forward keeping every
//             layer's activations, relative L2 loss (y - t)^2 / (y^2 + 0.01) (y not
//             differentiated in the denominator), backward through the layers and weight
//             gradients accumulated in TMEM, grid gradients by atomics on the 8 corners; then Adam
//             on the FP32 master parameters (beta 0.9 / 0.99, eps 1e-15).
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
__device__ __forceinline__ void encode_row(const CacheQuery& q, const __half* grid16, uint8_t* a, uint32_t row) {
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
            const uint32_t* g = reinterpret_cast<const uint32_t*>(grid16 + 2ull * CACHE_TABLE * l);
            float f0 = 0.0f, f1 = 0.0f;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                uint32_t bits = __ldg(g + idx[k]);
                float2 v = __half22float2(*reinterpret_cast<const __half2*>(&bits));
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
                                                                    const uint32_t* count, const __half* grid16,
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
        if (i < n) encode_row(q[i], grid16, s_a, tid);
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

// ---------------------------------------------------------------- training (tcgen05 tensor cores)
// One CTA (128 threads, one per sample row) takes tiles of 128 training pairs.  Forward: the
// inference layers, keeping every layer's FP16 activations H0..H4 in shared memory.  Loss and
// output gradient in FP32 per thread: g = 2 (y - t) / (y^2 + 0.01), clamped to +-2^14 (the
// factor 1 / (3 n) of the mean is applied when the FP32 gradients leave the CTA).  Backward:
// per layer, from the gradient of its output (in TMEM) the thread forms delta = g * (H > 0) in
// FP16 and writes it twice, row-major as the A operand of delta . W (the next gradient) and
// transposed as the A operand of delta^T . H (the weight gradient); H's transpose is the B
// operand.  Weight gradients accumulate in TMEM across all tiles of the CTA and are added to the
// global FP32 gradient once at the end; the input gradient's 32 grid-feature columns scatter
// onto the hash grid with atomics.  Operands (K-major core-matrix layout, no swizzle):
//   forward weights W_l [out][in], W_out [16][64]; backward weights W_l^T [in][out] and
//   W_out^T [64][16]; activations H0..H4 and delta [128][64]; output gradient [128][16];
//   transposed operands [128][128] (rows 64..127 zero) and [64][128], output gradient^T [16][128].
// TMEM (512 columns): 0..63 scratch accumulator, 64 + 64 l weight gradient of layer l (lanes =
// output neuron), 320..335 output-layer gradient transposed (lanes = input neuron).
constexpr uint32_t TT_OFF_WB = 4 * TC_W_BYTES + TC_WOUT_BYTES;      // backward weights
constexpr uint32_t TT_OFF_H = TT_OFF_WB + 4 * TC_W_BYTES + TC_WOUT_BYTES;
constexpr uint32_t TT_H_BYTES = TC_ROWS * CACHE_WIDTH * 2;            // 16 KB
constexpr uint32_t TT_OFF_G = TT_OFF_H + 5 * TT_H_BYTES;              // delta, row-major
constexpr uint32_t TT_OFF_DY = TT_OFF_G + TT_H_BYTES;                 // output gradient [128][16]
constexpr uint32_t TT_OFF_AT = TT_OFF_DY + TC_ROWS * 16 * 2;          // [128][128] transposed A
constexpr uint32_t TT_OFF_BT = TT_OFF_AT + 128 * 128 * 2;             // [64][128] transposed B
constexpr uint32_t TT_OFF_DYT = TT_OFF_BT + 64 * 128 * 2;             // [16][128]
constexpr uint32_t TT_OFF_BAR = TT_OFF_DYT + 16 * 128 * 2;
constexpr uint32_t TT_SMEM = TT_OFF_BAR + 16 + 1024;
constexpr uint32_t TT_TMEM_COLS = 512;
constexpr float TT_GRAD_CLAMP = 16384.0f;  // |dL/dy| per output, before the mean's 1 / (3 n)
constexpr float TT_GRAD_SCALE = 1.0f / 64.0f;  // FP16 headroom of the backward pass; undone at the end

// Byte offset of (row, k) in a K-major core-matrix operand whose rows are `kdim` elements long.
__device__ __forceinline__ uint32_t core_offset_k(uint32_t row, uint32_t k, uint32_t kdim) {
    return (row >> 3) * (kdim * 16u) + (k >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}
__device__ __forceinline__ uint64_t smem_desc_k(uint32_t addr, uint32_t kdim) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)((kdim * 16u) >> 4) << 32) |
           (1ull << 46);
}
__device__ __forceinline__ void store_half(uint8_t* base, uint32_t off, float v) {
    *reinterpret_cast<__half*>(base + off) = __float2half_rn(v);
}
__device__ __forceinline__ float load_half(const uint8_t* base, uint32_t off) {
    return __half2float(*reinterpret_cast<const __half*>(base + off));
}
// Issues `ksteps` MMAs of K 16 (A and B K-major with row length kdim) into TMEM column `col`.
__device__ __forceinline__ void mma_chain(uint32_t tmem_col, uint32_t a, uint32_t b, uint32_t kdim, uint32_t n,
                                          uint32_t ksteps, bool accumulate) {
    uint32_t idesc = mma_idesc(n);
    for (uint32_t kk = 0; kk < ksteps; ++kk)
        mma_f16(tmem_col, smem_desc_k(a + 256u * kk, kdim), smem_desc_k(b + 256u * kk, kdim), idesc,
                (accumulate || kk > 0) ? 1u : 0u);
}

__global__ void __launch_bounds__(TC_THREADS) cache_train_tc_kernel(const CacheQuery* q, const float* target, uint32_t n,
                                                                    const __half* grid16, const __half* w16,
                                                                    float* w_grad, float* grid_grad, float* loss,
                                                                    float inv_count, uint32_t* err) {
    inv_count = inv_count / TT_GRAD_SCALE;  // the output gradient was scaled by TT_GRAD_SCALE
    extern __shared__ uint8_t tt_smem_raw[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tt_smem_raw) + 1023u) & ~uintptr_t(1023));
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(sm + TT_OFF_BAR);
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(sm + TT_OFF_BAR + 8);
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint32_t base = smem_u32(sm);

    // weights: forward [out][in] and backward [in][out], FP16, core-matrix layout
    for (uint32_t e = tid; e < CACHE_HIDDEN_LAYERS * CACHE_WIDTH * CACHE_WIDTH; e += TC_THREADS) {
        uint32_t l = e / (CACHE_WIDTH * CACHE_WIDTH), o = (e / CACHE_WIDTH) % CACHE_WIDTH, i = e % CACHE_WIDTH;
        __half v = w16[e];
        *reinterpret_cast<__half*>(sm + l * TC_W_BYTES + core_offset_k(o, i, 64)) = v;
        *reinterpret_cast<__half*>(sm + TT_OFF_WB + l * TC_W_BYTES + core_offset_k(i, o, 64)) = v;
    }
    for (uint32_t e = tid; e < 16u * CACHE_WIDTH; e += TC_THREADS) {
        uint32_t o = e / CACHE_WIDTH, i = e % CACHE_WIDTH;
        __half v = o < (uint32_t)CACHE_OUT_ROWS ? w16[CACHE_HIDDEN_LAYERS * CACHE_WIDTH * CACHE_WIDTH + e]
                                                : __float2half_rn(0.0f);
        *reinterpret_cast<__half*>(sm + 4 * TC_W_BYTES + core_offset_k(o, i, 64)) = v;
        *reinterpret_cast<__half*>(sm + TT_OFF_WB + 4 * TC_W_BYTES + core_offset_k(i, o, 16)) = v;
    }
    // rows 64..127 of the transposed A operand stay zero
    for (uint32_t e = tid; e < 64u * 128u / 8u; e += TC_THREADS) {
        uint32_t r = 64u + e / 16u, c = (e % 16u) * 8u;
        *reinterpret_cast<uint4*>(sm + TT_OFF_AT + core_offset_k(r, c, 128)) = make_uint4(0u, 0u, 0u, 0u);
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(s_bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(s_tmem)),
                     "r"(TT_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_tmem;
    const uint32_t bar = smem_u32(s_bar);
    const uint32_t lane = tmem + ((32u * warp) << 16);
    uint32_t phase = 0;
    bool ok = true;
    uint32_t done_tiles = 0;
    float my_loss = 0.0f;

    // one MMA batch: barrier, issue by thread 0, commit, bounded wait (CTA-uniform verdict)
    auto run = [&](auto issue) {
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            issue();
            mma_commit(bar);
        }
        ok = __syncthreads_and(bar_wait(bar, phase) ? 1 : 0) != 0;
        phase ^= 1u;
        tc_fence_after();
        return ok;
    };

    const uint32_t tiles = (n + TC_ROWS - 1u) / TC_ROWS;
    for (uint32_t tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const uint32_t i = tile * TC_ROWS + tid;
        const bool valid = i < n;
        const bool acc = done_tiles > 0;
        uint8_t* h0 = sm + TT_OFF_H;
        if (valid) encode_row(q[i], grid16, h0, tid);
        else zero_row(h0, tid);
        // forward
        for (int l = 0; l < CACHE_HIDDEN_LAYERS && ok; ++l) {
            uint32_t a = base + TT_OFF_H + (uint32_t)l * TT_H_BYTES, b = base + (uint32_t)l * TC_W_BYTES;
            if (!run([&] { mma_chain(tmem, a, b, 64, 64, 4, false); })) break;
            uint8_t* hn = sm + TT_OFF_H + (uint32_t)(l + 1) * TT_H_BYTES;
#pragma unroll
            for (int c = 0; c < CACHE_WIDTH; c += 16) {
                float v[16];
                tmem_ld16(lane + (uint32_t)c, v);
                tmem_ld_wait();
                store_relu16(hn, tid, (uint32_t)c, v);
            }
        }
        if (!ok) break;
        if (!run([&] { mma_chain(tmem, base + TT_OFF_H + 4 * TT_H_BYTES, base + 4 * TC_W_BYTES, 64, 16, 4, false); }))
            break;
        // loss and output gradient (rows of padding samples are zero)
        {
            float v[16];
            tmem_ld16(lane, v);
            tmem_ld_wait();
            float g[3] = {0.0f, 0.0f, 0.0f};
            if (valid) {
                for (int c = 0; c < 3; ++c) {
                    float d = v[c] - target[3ull * i + c];
                    float den = v[c] * v[c] + 0.01f;
                    my_loss += d * d / den;
                    g[c] = fminf(fmaxf(2.0f * d / den, -TT_GRAD_CLAMP), TT_GRAD_CLAMP) * TT_GRAD_SCALE;
                }
            }
            for (uint32_t c = 0; c < 16; ++c) {
                float x = c < 3 ? g[c] : 0.0f;
                store_half(sm + TT_OFF_DY, core_offset_k(tid, c, 16), x);
                store_half(sm + TT_OFF_DYT, core_offset_k(c, tid, 128), x);
            }
            // H4^T as the A operand of the output layer's gradient, transposed: D[in][out]
            const uint8_t* h4 = sm + TT_OFF_H + 4 * TT_H_BYTES;
            for (uint32_t c = 0; c < 64; ++c)
                store_half(sm + TT_OFF_AT, core_offset_k(c, tid, 128), load_half(h4, core_offset_k(tid, c, 64)));
        }
        // dW_out^T += H4^T . dy (N 16) and the gradient of H4: dy . W_out (K 16)
        if (!run([&] {
                mma_chain(tmem + 320u, base + TT_OFF_AT, base + TT_OFF_DYT, 128, 16, 8, acc);
                mma_chain(tmem, base + TT_OFF_DY, base + TT_OFF_WB + 4 * TC_W_BYTES, 16, 64, 1, false);
            }))
            break;
        // hidden layers, last to first: delta_l = grad(H_{l+1}) * (H_{l+1} > 0)
        for (int l = CACHE_HIDDEN_LAYERS - 1; l >= 0 && ok; --l) {
            const uint8_t* hout = sm + TT_OFF_H + (uint32_t)(l + 1) * TT_H_BYTES;
            const uint8_t* hin = sm + TT_OFF_H + (uint32_t)l * TT_H_BYTES;
#pragma unroll
            for (int c = 0; c < CACHE_WIDTH; c += 16) {
                float v[16];
                tmem_ld16(lane + (uint32_t)c, v);
                tmem_ld_wait();
#pragma unroll
                for (int k = 0; k < 16; ++k) {
                    uint32_t col = (uint32_t)(c + k);
                    float d = load_half(hout, core_offset_k(tid, col, 64)) > 0.0f ? v[k] : 0.0f;
                    store_half(sm + TT_OFF_G, core_offset_k(tid, col, 64), d);
                    store_half(sm + TT_OFF_AT, core_offset_k(col, tid, 128), d);
                    store_half(sm + TT_OFF_BT, core_offset_k(col, tid, 128), load_half(hin, core_offset_k(tid, col, 64)));
                }
            }
            const uint32_t dw = tmem + 64u + 64u * (uint32_t)l;
            const uint32_t wb = base + TT_OFF_WB + (uint32_t)l * TC_W_BYTES;
            if (!run([&] {
                    mma_chain(dw, base + TT_OFF_AT, base + TT_OFF_BT, 128, 64, 8, acc);  // dW_l += delta^T . H_l
                    mma_chain(tmem, base + TT_OFF_G, wb, 64, 64, 4, false);              // grad(H_l) = delta . W_l
                }))
                break;
        }
        if (!ok) break;
        // grad(H0): the 32 grid-feature columns scatter onto the grid (the TMEM loads are
        // warp-collective, so every lane loads)
        float gx[32];
        tmem_ld16(lane, gx);
        tmem_ld16(lane + 16u, gx + 16);
        tmem_ld_wait();
        if (valid) {
            float3 p = make_float3(fminf(fmaxf(q[i].pos[0], 0.0f), 1.0f), fminf(fmaxf(q[i].pos[1], 0.0f), 1.0f),
                                   fminf(fmaxf(q[i].pos[2], 0.0f), 1.0f));
            for (int l = 0; l < CACHE_LEVELS; ++l) {
                uint32_t idx[8];
                float wgt[8];
                grid_corners(p, l, idx, wgt);
                float* gg = grid_grad + 2ull * CACHE_TABLE * l;
                float g0 = gx[2 * l] * inv_count, g1 = gx[2 * l + 1] * inv_count;
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    atomicAdd(gg + 2ull * idx[c], wgt[c] * g0);
                    atomicAdd(gg + 2ull * idx[c] + 1, wgt[c] * g1);
                }
            }
        }
        ++done_tiles;
    }
    // weight gradients leave TMEM once: lanes 0..63 hold the output neurons of each layer
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (ok && done_tiles > 0 && warp < 2) {
        for (int l = 0; l < CACHE_HIDDEN_LAYERS; ++l) {
            for (int c = 0; c < CACHE_WIDTH; c += 16) {
                float v[16];
                tmem_ld16(lane + 64u + 64u * (uint32_t)l + (uint32_t)c, v);
                tmem_ld_wait();
                float* dst = w_grad + (uint64_t)l * CACHE_WIDTH * CACHE_WIDTH + (uint64_t)tid * CACHE_WIDTH + c;
                for (int k = 0; k < 16; ++k) atomicAdd(dst + k, v[k] * inv_count);
            }
        }
        float v[16];
        tmem_ld16(lane + 320u, v);  // lane = input neuron, columns = outputs
        tmem_ld_wait();
        for (int o = 0; o < 3; ++o)
            atomicAdd(w_grad + CACHE_HIDDEN_LAYERS * CACHE_WIDTH * CACHE_WIDTH + (uint64_t)o * CACHE_WIDTH + tid, v[o] * inv_count);
    }
    float block_loss = my_loss;
    for (int o = 16; o > 0; o >>= 1) block_loss += __shfl_down_sync(0xffffffffu, block_loss, o);
    if ((tid & 31u) == 0 && block_loss != 0.0f) atomicAdd(loss, block_loss);
    if (!ok && err) atomicOr(err, ERR_TENSOR_WAIT);
    tc_fence_before();
    __syncthreads();
    if (!ok) bar_wait(bar, phase ^ 1u);
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TT_TMEM_COLS)
                     : "memory");
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
__global__ void cache_init_kernel(float* grid, __half* grid16, float* w, __half* w16, uint32_t seed) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < CACHE_GRID_PARAMS) {
        float x = (hash_uniform(i, seed) * 2.0f - 1.0f) * 1e-4f;
        grid[i] = x;
        grid16[i] = __float2half_rn(x);
    }
    if (i < CACHE_PARAMS) {
        float bound = sqrtf(6.0f / (i < CACHE_HIDDEN_LAYERS * CACHE_WIDTH * CACHE_WIDTH ? 128.0f : 67.0f));
        bool unused = i >= CACHE_HIDDEN_LAYERS * CACHE_WIDTH * CACHE_WIDTH &&
                      (i - CACHE_HIDDEN_LAYERS * CACHE_WIDTH * CACHE_WIDTH) >= 3u * CACHE_WIDTH;
        float x = unused ? 0.0f : (hash_uniform(i + CACHE_GRID_PARAMS, seed) * 2.0f - 1.0f) * bound;
        w[i] = x;
        w16[i] = __float2half_rn(x);
    }
}

static void launch_infer(const CacheQuery* q, uint32_t n, const uint32_t* count, const __half* grid16,
                         const __half* w16, float* out, uint32_t* err, cudaStream_t st) {
    if (n == 0) return;
    static bool attr[64] = {};  // per device: the shared-memory opt-in is a per-device function attribute
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= 64 || !attr[dev]) {
        check_cuda(cudaFuncSetAttribute(cache_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM),
                   "infer smem");
        if (dev >= 0 && dev < 64) attr[dev] = true;
    }
    uint32_t tiles = (n + TC_ROWS - 1u) / TC_ROWS;
    uint32_t blocks = std::min<uint32_t>(tiles, 152u * 4u);
    cache_infer_tc_kernel<<<blocks, TC_THREADS, TC_SMEM, st>>>(q, n, count, grid16, w16, out, err);
}

void cache_infer(const CacheDevice& d, const CacheQuery* q, uint32_t n, float* out, uint32_t* err, cudaStream_t st) {
    launch_infer(q, n, nullptr, d.grid16, d.w16, out, err, st);
}

void cache_infer_queue(const __half* grid16, const __half* w16, const CacheQuery* q, const uint32_t* count,
                       uint32_t max_n, float* out, uint32_t* err, cudaStream_t st) {
    launch_infer(q, max_n, count, grid16, w16, out, err, st);
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

// The training kernel's gradient pass: accumulates the gradients of the mean relative L2 loss
// of n pairs into d.w_grad / d.grid_grad (which must start at zero) and the summed loss into
// d.loss.
static void cache_gradient_pass(const CacheDevice& d, const CacheQuery* q, const float* target, uint32_t n,
                                uint32_t* err, cudaStream_t st) {
    static bool attr[64] = {};  // per device: the shared-memory opt-in is a per-device function attribute
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= 64 || !attr[dev]) {
        check_cuda(cudaFuncSetAttribute(cache_train_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TT_SMEM),
                   "train smem");
        if (dev >= 0 && dev < 64) attr[dev] = true;
    }
    uint32_t tiles = (n + TC_ROWS - 1u) / TC_ROWS;
    uint32_t blocks = std::min<uint32_t>(tiles, 152u);
    check_cuda(cudaMemsetAsync(d.loss, 0, 4, st), "memset");
    cache_train_tc_kernel<<<blocks, TC_THREADS, TT_SMEM, st>>>(q, target, n, d.grid16, d.w16, d.w_grad, d.grid_grad,
                                                               d.loss, 1.0f / (3.0f * (float)n), err);
}

void cache_gradients(const CacheDevice& d, const CacheQuery* q, const float* target, uint32_t n, uint32_t* err,
                     cudaStream_t st) {
    if (n == 0) return;
    cache_gradient_pass(d, q, target, n, err, st);
}

void cache_clear_gradients(const CacheDevice& d, cudaStream_t st) {
    check_cuda(cudaMemsetAsync(d.grid_grad, 0, 4 * CACHE_GRID_PARAMS, st), "memset");
    check_cuda(cudaMemsetAsync(d.w_grad, 0, 4 * CACHE_PARAMS, st), "memset");
}

void cache_train_step(const CacheDevice& d, const CacheQuery* q, const float* target, uint32_t n, float lr,
                      uint32_t step, uint32_t* err, cudaStream_t st) {
    if (n == 0) return;
    cache_gradient_pass(d, q, target, n, err, st);
    float c1 = 1.0f - std::pow(0.9f, (float)step), c2 = 1.0f - std::pow(0.99f, (float)step);
    cache_adam_kernel<<<(CACHE_PARAMS + 255) / 256, 256, 0, st>>>(d.w, d.w_m, d.w_v, d.w_grad, d.w16, CACHE_PARAMS,
                                                                  lr, c1, c2);
    cache_adam_kernel<<<(unsigned)((CACHE_GRID_PARAMS + 255) / 256), 256, 0, st>>>(
        d.grid, d.grid_m, d.grid_v, d.grid_grad, d.grid16, CACHE_GRID_PARAMS, lr, c1, c2);
}

void cache_init(const CacheDevice& d, uint32_t seed, cudaStream_t st) {
    cache_init_kernel<<<(unsigned)((CACHE_GRID_PARAMS + 255) / 256), 256, 0, st>>>(d.grid, d.grid16, d.w, d.w16,
                                                                                   seed);
    check_cuda(cudaMemsetAsync(d.grid_m, 0, 4 * CACHE_GRID_PARAMS, st), "memset");
    check_cuda(cudaMemsetAsync(d.grid_v, 0, 4 * CACHE_GRID_PARAMS, st), "memset");
    check_cuda(cudaMemsetAsync(d.grid_grad, 0, 4 * CACHE_GRID_PARAMS, st), "memset");
    check_cuda(cudaMemsetAsync(d.w_m, 0, 4 * CACHE_PARAMS, st), "memset");
    check_cuda(cudaMemsetAsync(d.w_v, 0, 4 * CACHE_PARAMS, st), "memset");
    check_cuda(cudaMemsetAsync(d.w_grad, 0, 4 * CACHE_PARAMS, st), "memset");
}

}  // namespace tt
