// GPU LBVH build: the replacement for the driver-side BLAS/TLAS builds of the reference
// (src/scene.rs:130-171 -> crates/tinytrace_backend/src/resource.rs:728-880, 891-1085).
//
// Two structures share the pipeline below.  Two-level: one pass builds every mesh's BLAS at
// once (segment = mesh), a second pass the TLAS over instances.  Flat: one pass over the world
// boxes of all (instance, triangle) pairs (one segment).
//   1. primitive boxes (triangles: dequantised snorm16 vertices, transformed to world space for
//      the flat structure; instances: the 8 transformed corners of their mesh box) and
//      per-segment centroid bounds (float atomics);
//   2. 30-bit Morton codes of the centroids, normalised per segment, prefixed by the segment
//      (mesh) index: key = segment << 30 | morton;
//   3. stable onesweep LSD radix sort of (key, primitive) in 8-bit digits;
//   4. Karras (2012) binary radix tree over the sorted keys (index tie-break for duplicates);
//      each segment's primitives form exactly one subtree;
//   5. bottom-up box refit with one atomic visit counter per node;
//   6. collapse to 4-wide nodes level by level from the segment roots (greedy expansion of
//      the largest-area child, subtrees of <= leaf_max primitives become leaves), child boxes
//      stored as float planes (128-byte nodes).
// Every step is deterministic; the CPU oracle restates the same build and the tests compare
// the node arrays byte for byte.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "tt_common.cuh"
#include "tt_internal.h"

namespace tt {
namespace {

constexpr int SCAN_THREADS = 1024;
constexpr int SORT_THREADS = 256;
constexpr int SORT_WARPS = SORT_THREADS / 32;

inline unsigned grid_for(uint64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// ---------------------------------------------------------------- stream-ordered scratch
struct Scratch {
    cudaStream_t stream;
    std::vector<void*> ptrs;
    explicit Scratch(cudaStream_t s) : stream(s) {}
    ~Scratch() {
        for (void* p : ptrs) cudaFreeAsync(p, stream);
    }
    template <class T>
    T* get(uint64_t count) {
        void* p = nullptr;
        size_t bytes = std::max<uint64_t>(count, 1) * sizeof(T);
        check_cuda(cudaMallocAsync(&p, bytes, stream), "cudaMallocAsync (bvh scratch)");
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
};

// ---------------------------------------------------------------- exclusive scan (u32)
__global__ void scan_block_kernel(uint32_t* data, uint32_t* block_sums, uint64_t n) {
    __shared__ uint32_t warp_tot[SCAN_THREADS / 32];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_THREADS * 4;
    uint32_t v[4];
    uint32_t local = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        uint64_t i = base + (uint64_t)threadIdx.x * 4 + k;
        v[k] = i < n ? data[i] : 0u;
        local += v[k];
    }
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_tot[lane];
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        warp_tot[lane] = wi - w;
    }
    __syncthreads();
    uint32_t run = warp_tot[warp] + incl - local;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        uint64_t i = base + (uint64_t)threadIdx.x * 4 + k;
        if (i < n) data[i] = run;
        run += v[k];
    }
    if (threadIdx.x == SCAN_THREADS - 1 && block_sums) block_sums[blockIdx.x] = run;
}
__global__ void scan_add_kernel(uint32_t* data, const uint32_t* block_sums, uint64_t n) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) data[i] += block_sums[i / (SCAN_THREADS * 4)];
}
// In-place exclusive scan of n u32 values.
void exclusive_scan(uint32_t* data, uint64_t n, Scratch& sc) {
    if (n == 0) return;
    const uint64_t per_block = SCAN_THREADS * 4;
    uint64_t blocks = (n + per_block - 1) / per_block;
    if (blocks == 1) {
        scan_block_kernel<<<1, SCAN_THREADS, 0, sc.stream>>>(data, nullptr, n);
        return;
    }
    uint32_t* sums = sc.get<uint32_t>(blocks);
    scan_block_kernel<<<(unsigned)blocks, SCAN_THREADS, 0, sc.stream>>>(data, sums, n);
    exclusive_scan(sums, blocks, sc);
    scan_add_kernel<<<grid_for(n, 256), 256, 0, sc.stream>>>(data, sums, n);
}

// ---------------------------------------------------------------- radix sort (u64 key, u32 value)
// Onesweep LSD radix sort (after Adinets & Merrill 2022), 8-bit digits: one up-front pass counts
// the keys of every digit position, a small kernel turns the counts into each digit's global
// offsets, and then one kernel per digit position ranks and scatters the keys.  That kernel
// takes tiles of SORT_ITEMS x SORT_THREADS keys in the order its blocks claim them (an atomic
// tile counter, so every predecessor of a tile belongs to a block that is already running),
// ranks its keys stably per digit (warp match over SORT_ITEMS rounds of SORT_THREADS
// consecutive keys), publishes its per-digit counts, and finds each digit's exclusive prefix
// over the preceding tiles by decoupled look-back: it adds predecessors' published counts until
// it meets a published inclusive prefix, then publishes its own inclusive prefix.  A status word
// holds a 2-bit flag over a 30-bit value; the look-back wait is bounded (SORT_WAIT_LIMIT polls,
// then ERR_SORT_WAIT and the pass goes on with a wrong prefix, reported after the sort).
constexpr int SORT_ITEMS = 8;
constexpr uint32_t SORT_TILE = SORT_THREADS * SORT_ITEMS;
constexpr int SORT_MAX_PASSES = 8;
constexpr uint32_t SORT_FLAG_AGGREGATE = 1u << 30, SORT_FLAG_INCLUSIVE = 2u << 30;
constexpr uint32_t SORT_VALUE_MASK = (1u << 30) - 1u, SORT_FLAG_MASK = 3u << 30;
constexpr uint32_t SORT_WAIT_LIMIT = 1u << 24;
constexpr uint32_t ERR_SORT_WAIT = 1u;

// counts[p][d]: keys whose digit p (bits 8p..8p+7) is d, for passes p < passes.
__global__ void __launch_bounds__(SORT_THREADS) sort_count_kernel(const uint64_t* keys, uint32_t n, int passes,
                                                                  uint32_t* counts) {
    __shared__ uint32_t h[SORT_MAX_PASSES][256];
    for (int p = 0; p < passes; ++p) h[p][threadIdx.x] = 0u;
    __syncthreads();
    for (uint32_t i = blockIdx.x * SORT_THREADS + threadIdx.x; i < n; i += gridDim.x * SORT_THREADS) {
        uint64_t k = keys[i];
        for (int p = 0; p < passes; ++p) atomicAdd(&h[p][(uint32_t)(k >> (8 * p)) & 0xffu], 1u);
    }
    __syncthreads();
    for (int p = 0; p < passes; ++p)
        if (h[p][threadIdx.x]) atomicAdd(&counts[p * 256 + threadIdx.x], h[p][threadIdx.x]);
}

// offsets[p][d] = sum of counts[p][d'] for d' < d (one block of 256 threads per pass).
__global__ void __launch_bounds__(256) sort_offsets_kernel(const uint32_t* counts, uint32_t* offsets) {
    __shared__ uint32_t w[8];
    uint32_t c = counts[blockIdx.x * 256 + threadIdx.x];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) w[warp] = incl;
    __syncthreads();
    uint32_t before = 0u;
    for (int k = 0; k < warp; ++k) before += w[k];
    offsets[blockIdx.x * 256 + threadIdx.x] = before + incl - c;
}

// One digit pass: kin/vin -> kout/vout by digit `pass`.  status holds (tiles x 256) words and
// *tile_counter 0 at launch.
__global__ void __launch_bounds__(SORT_THREADS) sort_pass_kernel(const uint64_t* kin, const uint32_t* vin,
                                                                 uint64_t* kout, uint32_t* vout, uint32_t n,
                                                                 int pass, const uint32_t* offsets,
                                                                 uint32_t* status, uint32_t* tile_counter,
                                                                 uint32_t* err) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_warp[SORT_WARPS][256];
    __shared__ uint32_t s_run[256];
    const uint32_t t = threadIdx.x;
    const int lane = t & 31, warp = t >> 5;
    if (t == 0) s_tile = atomicAdd(tile_counter, 1u);
    s_run[t] = 0u;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint64_t base = (uint64_t)tile * SORT_TILE;
    const int shift = 8 * pass;
    uint64_t key[SORT_ITEMS];
    uint32_t val[SORT_ITEMS], digit[SORT_ITEMS], off[SORT_ITEMS];
#pragma unroll
    for (int k = 0; k < SORT_ITEMS; ++k) {
        uint64_t i = base + (uint64_t)k * SORT_THREADS + t;
        bool valid = i < n;
        key[k] = valid ? kin[i] : 0ull;
        val[k] = valid ? vin[i] : 0u;
        digit[k] = valid ? ((uint32_t)(key[k] >> shift) & 0xffu) : 256u;
    }
    // stable ranks inside the tile: round k covers keys k * SORT_THREADS .. + SORT_THREADS - 1
#pragma unroll
    for (int k = 0; k < SORT_ITEMS; ++k) {
#pragma unroll
        for (int w = 0; w < SORT_WARPS; ++w) s_warp[w][t] = 0u;
        __syncthreads();
        uint32_t peers = __match_any_sync(0xffffffffu, digit[k]);
        uint32_t rank = (uint32_t)__popc(peers & ((1u << lane) - 1u));
        if (digit[k] < 256u && lane == __ffs(peers) - 1) s_warp[warp][digit[k]] = (uint32_t)__popc(peers);
        __syncthreads();
        uint32_t run = s_run[t];
#pragma unroll
        for (int w = 0; w < SORT_WARPS; ++w) {
            uint32_t c = s_warp[w][t];
            s_warp[w][t] = run;
            run += c;
        }
        s_run[t] = run;
        __syncthreads();
        off[k] = digit[k] < 256u ? s_warp[warp][digit[k]] + rank : 0u;
        __syncthreads();
    }
    // decoupled look-back, one digit per thread
    const uint32_t count = s_run[t];
    uint32_t* mine = status + (uint64_t)tile * 256 + t;
    uint32_t excl = 0u;
    if (tile == 0) {
        atomicExch(mine, SORT_FLAG_INCLUSIVE | count);
    } else {
        atomicExch(mine, SORT_FLAG_AGGREGATE | count);
        uint32_t j = tile - 1u, polls = 0u;
        while (true) {
            uint32_t v = __ldcv(status + (uint64_t)j * 256 + t);
            uint32_t flag = v & SORT_FLAG_MASK;
            if (flag == 0u) {
                if (++polls > SORT_WAIT_LIMIT) {
                    atomicOr(err, ERR_SORT_WAIT);
                    break;
                }
                continue;
            }
            excl += v & SORT_VALUE_MASK;
            if (flag == SORT_FLAG_INCLUSIVE || j == 0u) break;
            --j;
        }
        atomicExch(mine, SORT_FLAG_INCLUSIVE | ((excl + count) & SORT_VALUE_MASK));
    }
    __syncthreads();  // every s_run read above is done
    s_run[t] = offsets[pass * 256 + t] + excl;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SORT_ITEMS; ++k) {
        uint32_t pos = digit[k] < 256u ? s_run[digit[k]] + off[k] : n;
        if (pos < n) {  // always, unless a look-back wait ran out (reported by ERR_SORT_WAIT)
            kout[pos] = key[k];
            vout[pos] = val[k];
        }
    }
}

// Stable sort of (keys, vals) by the low `bits` bits of the keys (bits <= 64). Result in
// keys/vals.  Synchronises the stream once, to report a look-back wait that ran out.
void radix_sort(uint64_t*& keys, uint32_t*& vals, uint32_t n, int bits, Scratch& sc) {
    if (n <= 1) return;
    if (n > SORT_VALUE_MASK) fail(TT_ERR_OVERFLOW, "more than 2^30 keys for the radix sort");
    const int passes = (bits + 7) / 8;
    const uint32_t tiles = (uint32_t)((n + SORT_TILE - 1) / SORT_TILE);
    uint64_t* k2 = sc.get<uint64_t>(n);
    uint32_t* v2 = sc.get<uint32_t>(n);
    // counts, offsets, per-pass tile counters and the error word in one zeroed block; the
    // status words of a pass (tiles x 256) are cleared before it
    const uint64_t words = 2ull * SORT_MAX_PASSES * 256 + SORT_MAX_PASSES + 1;
    uint32_t* w = sc.get<uint32_t>(words);
    check_cuda(cudaMemsetAsync(w, 0, 4ull * words, sc.stream), "memset");
    uint32_t* counts = w;
    uint32_t* offsets = counts + SORT_MAX_PASSES * 256;
    uint32_t* tile_counter = offsets + SORT_MAX_PASSES * 256;
    uint32_t* err = tile_counter + SORT_MAX_PASSES;
    uint32_t* status = sc.get<uint32_t>((uint64_t)tiles * 256);
    sort_count_kernel<<<std::min<unsigned>(tiles, 1024u), SORT_THREADS, 0, sc.stream>>>(keys, n, passes, counts);
    sort_offsets_kernel<<<passes, 256, 0, sc.stream>>>(counts, offsets);
    for (int p = 0; p < passes; ++p) {
        check_cuda(cudaMemsetAsync(status, 0, 4ull * tiles * 256, sc.stream), "memset");
        sort_pass_kernel<<<tiles, SORT_THREADS, 0, sc.stream>>>(keys, vals, k2, v2, n, p, offsets, status,
                                                                 tile_counter + p, err);
        std::swap(keys, k2);
        std::swap(vals, v2);
    }
    uint32_t host_err = 0;
    check_cuda(cudaMemcpyAsync(&host_err, err, 4, cudaMemcpyDeviceToHost, sc.stream), "sort error word");
    check_cuda(cudaStreamSynchronize(sc.stream), "cudaStreamSynchronize");
    if (host_err) fail(TT_ERR_TIMEOUT, "radix sort: a look-back wait ran out");
}

// ---------------------------------------------------------------- float atomics
__device__ __forceinline__ void atomic_min_f(float* a, float v) {
    if (v >= 0.0f) atomicMin(reinterpret_cast<int*>(a), __float_as_int(v));
    else atomicMax(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float* a, float v) {
    if (v >= 0.0f) atomicMax(reinterpret_cast<int*>(a), __float_as_int(v));
    else atomicMin(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}
__device__ __forceinline__ float canon(float v) { return v + 0.0f; }  // -0 -> +0

// ---------------------------------------------------------------- primitives
// Triangle boxes + records for all meshes.  mesh_tri_base: prefix of triangle counts.
__global__ void triangle_prims_kernel(const int16_t* positions, const uint32_t* indices,
                                      const tt_mesh* meshes, const uint32_t* mesh_tri_base,
                                      uint32_t mesh_count, uint32_t n, float4* lo, float4* hi,
                                      uint32_t* seg, float4* recs) {
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    // last mesh with base <= g
    uint32_t a = 0, b = mesh_count;
    while (b - a > 1) {
        uint32_t m = (a + b) / 2;
        if (mesh_tri_base[m] <= g) a = m;
        else b = m;
    }
    // skip meshes without triangles that share the same base
    while (a + 1 < mesh_count && mesh_tri_base[a + 1] <= g) ++a;
    const tt_mesh me = meshes[a];
    uint32_t p = g - mesh_tri_base[a];
    uint32_t base = me.index_offset + 3u * p;
    f3 q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int16_t* s = positions + 3ull * (me.vertex_offset + indices[base + k]);
        q[k] = f3{dequant_snorm16(s[0]), dequant_snorm16(s[1]), dequant_snorm16(s[2])};
    }
    f3 l = f3{fmn(fmn(q[0].x, q[1].x), q[2].x), fmn(fmn(q[0].y, q[1].y), q[2].y),
              fmn(fmn(q[0].z, q[1].z), q[2].z)};
    f3 h = f3{fmx(fmx(q[0].x, q[1].x), q[2].x), fmx(fmx(q[0].y, q[1].y), q[2].y),
              fmx(fmx(q[0].z, q[1].z), q[2].z)};
    lo[g] = make_float4(canon(l.x), canon(l.y), canon(l.z), 0.0f);
    hi[g] = make_float4(canon(h.x), canon(h.y), canon(h.z), 0.0f);
    seg[g] = a;
    recs[3ull * g + 0] = make_float4(q[0].x, q[0].y, q[0].z, __uint_as_float(p));
    recs[3ull * g + 1] = make_float4(q[1].x, q[1].y, q[1].z, __uint_as_float(a));
    recs[3ull * g + 2] = make_float4(q[2].x, q[2].y, q[2].z, 0.0f);
}

// Instance world boxes from the mesh boxes (8 transformed corners).
__global__ void instance_prims_kernel(const tt_instance* inst, const uint32_t* ids, uint32_t n,
                                      const float4* mesh_lo, const float4* mesh_hi, float4* lo,
                                      float4* hi, uint32_t* seg) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const tt_instance& in = inst[ids[i]];
    float4 ml = mesh_lo[in.mesh_index], mh = mesh_hi[in.mesh_index];
    f3 l = splat(__int_as_float(0x7f800000)), h = splat(__int_as_float(0xff800000));
    for (int k = 0; k < 8; ++k) {
        f3 c = f3{(k & 1) ? mh.x : ml.x, (k & 2) ? mh.y : ml.y, (k & 4) ? mh.z : ml.z};
        f3 w = mat43_point(in.transform, c);
        l = f3{fmn(l.x, w.x), fmn(l.y, w.y), fmn(l.z, w.z)};
        h = f3{fmx(h.x, w.x), fmx(h.y, w.y), fmx(h.z, w.z)};
    }
    lo[i] = make_float4(canon(l.x), canon(l.y), canon(l.z), 0.0f);
    hi[i] = make_float4(canon(h.x), canon(h.y), canon(h.z), 0.0f);
    seg[i] = 0u;
}

// World boxes and records of all (instance, triangle) pairs, instance-major.  inst_tri_base:
// prefix of the instances' triangle counts.
__global__ void flat_prims_kernel(const int16_t* positions, const uint32_t* indices, const tt_instance* inst,
                                  const uint32_t* inst_tri_base, uint32_t instance_count, uint32_t n, float4* lo,
                                  float4* hi, uint32_t* seg, float4* recs) {
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    uint32_t a = 0, b = instance_count;
    while (b - a > 1) {
        uint32_t m = (a + b) / 2;
        if (inst_tri_base[m] <= g) a = m;
        else b = m;
    }
    while (a + 1 < instance_count && inst_tri_base[a + 1] <= g) ++a;
    const tt_instance& in = inst[a];
    uint32_t p = g - inst_tri_base[a];
    uint32_t base = in.index_offset + 3u * p;
    f3 q[3], w[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int16_t* s = positions + 3ull * (in.vertex_offset + indices[base + k]);
        q[k] = f3{dequant_snorm16(s[0]), dequant_snorm16(s[1]), dequant_snorm16(s[2])};
        w[k] = mat43_point(in.transform, q[k]);
    }
    f3 l = f3{fmn(fmn(w[0].x, w[1].x), w[2].x), fmn(fmn(w[0].y, w[1].y), w[2].y), fmn(fmn(w[0].z, w[1].z), w[2].z)};
    f3 h = f3{fmx(fmx(w[0].x, w[1].x), w[2].x), fmx(fmx(w[0].y, w[1].y), w[2].y), fmx(fmx(w[0].z, w[1].z), w[2].z)};
    lo[g] = make_float4(canon(l.x), canon(l.y), canon(l.z), 0.0f);
    hi[g] = make_float4(canon(h.x), canon(h.y), canon(h.z), 0.0f);
    seg[g] = 0u;
    recs[3ull * g + 0] = make_float4(q[0].x, q[0].y, q[0].z, __uint_as_float(p));
    recs[3ull * g + 1] = make_float4(q[1].x, q[1].y, q[1].z, __uint_as_float(a));
    recs[3ull * g + 2] = make_float4(q[2].x, q[2].y, q[2].z, 0.0f);
}

__global__ void init_bounds_kernel(float* b, uint32_t* cnt, uint32_t segs) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= segs) return;
    for (int a = 0; a < 3; ++a) {
        b[6 * s + a] = __int_as_float(0x7f800000);
        b[6 * s + 3 + a] = __int_as_float(0xff800000);
    }
    cnt[s] = 0u;
}
// Per-segment centroid bounds and primitive counts.  Segments are contiguous runs of
// primitives, so most warps lie inside one segment: those reduce their lanes with shuffles
// and lane 0 issues one atomic per bound (min/max are exact, so the grouping does not change
// the result).  A NaN centroid (non-finite transform) leaves the bounds unchanged, as fminf /
// fmaxf do in the sequential restatement.
__global__ void centroid_bounds_kernel(const float4* lo, const float4* hi, const uint32_t* seg,
                                       uint32_t n, float* b, uint32_t* cnt) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i - (threadIdx.x & 31u) >= n) return;  // whole warp past the end
    bool valid = i < n;
    float cmin[3] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000)};
    float cmax[3] = {__int_as_float(0xff800000), __int_as_float(0xff800000), __int_as_float(0xff800000)};
    uint32_t s = 0xffffffffu;
    if (valid) {
        float4 l = lo[i], h = hi[i];
        cmin[0] = cmax[0] = canon((l.x + h.x) * 0.5f);
        cmin[1] = cmax[1] = canon((l.y + h.y) * 0.5f);
        cmin[2] = cmax[2] = canon((l.z + h.z) * 0.5f);
        s = seg[i];
    }
    uint32_t s0 = __shfl_sync(0xffffffffu, s, 0);  // lane 0 is valid
    if (__all_sync(0xffffffffu, !valid || s == s0)) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                cmin[a] = fmn(cmin[a], __shfl_xor_sync(0xffffffffu, cmin[a], off));
                cmax[a] = fmx(cmax[a], __shfl_xor_sync(0xffffffffu, cmax[a], off));
            }
        }
        uint32_t k = (uint32_t)__popc(__ballot_sync(0xffffffffu, valid));
        if ((threadIdx.x & 31u) != 0u) return;
        s = s0;
        atomicAdd(&cnt[s], k);
    } else {
        if (!valid) return;
        atomicAdd(&cnt[s], 1u);
    }
    for (int a = 0; a < 3; ++a) {
        if (cmin[a] == cmin[a]) atomic_min_f(&b[6 * s + a], cmin[a]);
        if (cmax[a] == cmax[a]) atomic_max_f(&b[6 * s + 3 + a], cmax[a]);
    }
}

__device__ __forceinline__ uint32_t expand_bits10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
__device__ __forceinline__ uint32_t quantize_axis(float c, float lo, float hi) {
    float ext = hi - lo;
    if (!(ext > 0.0f)) return 0u;
    float f = (c - lo) / ext;
    float s = fmn(fmx(f * 1024.0f, 0.0f), 1023.0f);
    return (uint32_t)s;
}
__global__ void morton_kernel(const float4* lo, const float4* hi, const uint32_t* seg, uint32_t n,
                              const float* b, uint64_t* keys, uint32_t* vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 l = lo[i], h = hi[i];
    float c[3] = {canon((l.x + h.x) * 0.5f), canon((l.y + h.y) * 0.5f), canon((l.z + h.z) * 0.5f)};
    uint32_t s = seg[i];
    const float* bb = b + 6 * s;
    uint32_t x = quantize_axis(c[0], bb[0], bb[3]);
    uint32_t y = quantize_axis(c[1], bb[1], bb[4]);
    uint32_t z = quantize_axis(c[2], bb[2], bb[5]);
    uint32_t code = (expand_bits10(x) << 2) | (expand_bits10(y) << 1) | expand_bits10(z);
    keys[i] = ((uint64_t)s << 30) | code;
    vals[i] = i;
}

// ---------------------------------------------------------------- Karras hierarchy
__device__ __forceinline__ int kdelta(const uint64_t* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint64_t a = k[i], b = k[j];
    if (a != b) return __clzll((long long)(a ^ b));
    return 64 + __clz((int)((uint32_t)i ^ (uint32_t)j));
}
__global__ void karras_kernel(const uint64_t* k, int n, int* left, int* right, int* first,
                              int* last, int* parent) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int ni = n - 1;
    if (i >= ni) return;
    int d = (kdelta(k, n, i, i + 1) - kdelta(k, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = kdelta(k, n, i, i - d);
    int lmax = 2;
    while (kdelta(k, n, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (kdelta(k, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = kdelta(k, n, i, j);
    int s = 0;
    for (int div = 2;; div *= 2) {
        int t = (l + div - 1) / div;
        if (kdelta(k, n, i, i + (s + t) * d) > dnode) s += t;
        if (t == 1) break;
    }
    int gamma = i + s * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    int lc = (lo == gamma) ? (ni + gamma) : gamma;
    int rc = (hi == gamma + 1) ? (ni + gamma + 1) : (gamma + 1);
    left[i] = lc;
    right[i] = rc;
    first[i] = lo;
    last[i] = hi;
    parent[lc] = i;
    parent[rc] = i;
}

// ---------------------------------------------------------------- refit
// Node boxes: index r < ni internal, r >= ni leaf (r - ni = sorted position).
__global__ void refit_kernel(int n, const uint32_t* order, const float4* plo, const float4* phi,
                             const int* left, const int* right, const int* parent, float4* blo,
                             float4* bhi, uint32_t* visits) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int ni = n - 1;
    int r = ni + j;
    blo[r] = plo[order[j]];
    bhi[r] = phi[order[j]];
    if (ni == 0) return;
    int p = parent[r];
    while (p >= 0) {
        __threadfence();
        if (atomicAdd(&visits[p], 1u) == 0u) return;
        int a = left[p], b = right[p];
        float4 al = __ldcg(&blo[a]), ah = __ldcg(&bhi[a]);
        float4 bl = __ldcg(&blo[b]), bh = __ldcg(&bhi[b]);
        blo[p] = make_float4(fmn(al.x, bl.x), fmn(al.y, bl.y), fmn(al.z, bl.z), 0.0f);
        bhi[p] = make_float4(fmx(ah.x, bh.x), fmx(ah.y, bh.y), fmx(ah.z, bh.z), 0.0f);
        p = parent[p];
    }
}

__global__ void segment_roots_kernel(const uint32_t* seg_first, const uint32_t* seg_count,
                                     uint32_t segs, int n, const int* first, const int* last,
                                     int* level) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= segs) return;
    int ni = n - 1;
    int a = (int)seg_first[s], c = (int)seg_count[s];
    int b = a + c - 1;
    int r;
    if (c == 0) r = -1;
    else if (c == 1) r = ni + a;
    else if (first[a] == a && last[a] == b) r = a;
    else r = b;
    level[s] = r;
}

// ---------------------------------------------------------------- collapse to BVH4
struct TreeView {
    int n, ni;
    const int *left, *right, *first, *last;
    const float4 *blo, *bhi;
    __device__ bool is_leaf(int r) const { return r >= ni; }
    __device__ int nfirst(int r) const { return is_leaf(r) ? r - ni : first[r]; }
    __device__ int ncount(int r) const { return is_leaf(r) ? 1 : last[r] - first[r] + 1; }
    __device__ float half_area(int r) const {
        float4 l = blo[r], h = bhi[r];
        float ex = h.x - l.x, ey = h.y - l.y, ez = h.z - l.z;
        return ex * ey + ey * ez + ez * ex;
    }
};

__global__ void collapse_choose_kernel(TreeView t, const int* level, uint32_t L, int leaf_max,
                                       int* chosen, uint32_t* internal_count) {
    uint32_t li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= L) return;
    int r = level[li];
    int ch[4] = {-1, -1, -1, -1};
    int cnt = 0;
    if (r < 0) {
        cnt = 0;
    } else if (t.is_leaf(r) || t.ncount(r) <= leaf_max) {
        ch[0] = r;
        cnt = 1;
    } else {
        ch[0] = t.left[r];
        ch[1] = t.right[r];
        cnt = 2;
        while (cnt < 4) {
            int best = -1;
            float best_area = -1.0f;
            for (int c = 0; c < cnt; ++c) {
                if (t.is_leaf(ch[c]) || t.ncount(ch[c]) <= leaf_max) continue;
                float a = t.half_area(ch[c]);
                if (best < 0 || a > best_area) {
                    best = c;
                    best_area = a;
                }
            }
            if (best < 0) break;
            int v = ch[best];
            for (int c = cnt; c > best + 1; --c) ch[c] = ch[c - 1];
            ch[best] = t.left[v];
            ch[best + 1] = t.right[v];
            cnt++;
        }
    }
    uint32_t internal = 0;
    for (int c = 0; c < 4; ++c) {
        chosen[4 * li + c] = ch[c];
        if (c < cnt && !(t.is_leaf(ch[c]) || t.ncount(ch[c]) <= leaf_max)) internal++;
    }
    internal_count[li] = internal;
}

__global__ void collapse_emit_kernel(TreeView t, const int* level, uint32_t L, int leaf_max,
                                     const int* chosen, const uint32_t* next_offset,
                                     uint64_t node_base, uint64_t next_base, uint4* nodes,
                                     int* next_level, const uint32_t* order,
                                     const uint32_t* leaf_ids, int leaf_by_prim) {
    uint32_t li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= L) return;
    int r = level[li];
    int cnt = 0;
    uint32_t child[4] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu};
    uint32_t k = next_offset[li];
    float clo[4][3], chi[4][3];
    for (int c = 0; c < 4; ++c) {
        int v = chosen[4 * li + c];
        if (v < 0) break;
        cnt++;
        float4 l = t.blo[v], h = t.bhi[v];
        clo[c][0] = l.x; clo[c][1] = l.y; clo[c][2] = l.z;
        chi[c][0] = h.x; chi[c][1] = h.y; chi[c][2] = h.z;
        if (t.is_leaf(v) || t.ncount(v) <= leaf_max) {
            uint32_t f = (uint32_t)t.nfirst(v);
            uint32_t kk = (uint32_t)t.ncount(v);
            if (leaf_by_prim) {
                uint32_t id = leaf_ids ? leaf_ids[order[f]] : order[f];
                child[c] = 0x80000000u | id;
            } else {
                child[c] = 0x80000000u | ((kk - 1u) << 27) | f;
            }
        } else {
            child[c] = (uint32_t)(next_base + k);
            next_level[k] = v;
            k++;
        }
    }
    float bx[6][4];
    for (int c = 0; c < 4; ++c)
        for (int a = 0; a < 3; ++a) {
            bx[2 * a][c] = c < cnt ? clo[c][a] : __int_as_float(0x7f800000);
            bx[2 * a + 1][c] = c < cnt ? chi[c][a] : __int_as_float(0xff800000);
        }
    float4* nd = reinterpret_cast<float4*>(nodes) + 8ull * (node_base + li);
    for (int k = 0; k < 6; ++k) nd[k] = make_float4(bx[k][0], bx[k][1], bx[k][2], bx[k][3]);
    uint4* nu = reinterpret_cast<uint4*>(nd);
    nu[6] = make_uint4(child[0], child[1], child[2], child[3]);
    nu[7] = make_uint4((uint32_t)cnt, 0u, 0u, 0u);
    (void)r;
}

__global__ void gather_records_kernel(const float4* in, const uint32_t* order, uint32_t n,
                                      float4* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t s = order[i];
    out[3ull * i + 0] = in[3ull * s + 0];
    out[3ull * i + 1] = in[3ull * s + 1];
    out[3ull * i + 2] = in[3ull * s + 2];
}

// tri_record[tri_base[instance] + primitive] = record, over the records in leaf order.
__global__ void tri_record_kernel(const float4* recs, const uint32_t* tri_base, uint32_t n, uint32_t* tri_record) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t prim = __float_as_uint(recs[3ull * i].w), inst = __float_as_uint(recs[3ull * i + 1].w);
    tri_record[tri_base[inst] + prim] = i;
}

__global__ void segment_boxes_kernel(const int* roots, uint32_t segs, const float4* blo,
                                     const float4* bhi, float4* slo, float4* shi) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= segs) return;
    int r = roots[s];
    if (r < 0) {
        slo[s] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        shi[s] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    slo[s] = blo[r];
    shi[s] = bhi[r];
}

struct Build4 {
    uint64_t nodes = 0;
    uint32_t levels = 0;
    std::vector<uint64_t> level_start;  // first node of each level (levels + 1 entries)
    uint32_t* order = nullptr;  // scratch, sorted position -> primitive
    float4* blo = nullptr;      // scratch, binary node boxes
    float4* bhi = nullptr;
    int* roots = nullptr;       // scratch, segment root binary refs
};

// Binary LBVH over primitive boxes grouped in non-decreasing segments: centroid bounds,
// Morton keys, stable radix sort, Karras hierarchy, bottom-up boxes; each segment's root
// binary reference in `roots` (device, -1 for an empty segment).
struct Binary {
    TreeView tv;
    uint32_t* order = nullptr;  // sorted position -> primitive
    float4* blo = nullptr;      // binary node boxes (internal r < ni, leaf ni + sorted position)
    float4* bhi = nullptr;
    int* roots = nullptr;
};

Binary build_binary(const float4* plo, const float4* phi, const uint32_t* seg, uint32_t n, uint32_t segs,
                    Scratch& sc) {
    cudaStream_t st = sc.stream;
    Binary out;
    float* bounds = sc.get<float>(6ull * segs);
    uint32_t* seg_count = sc.get<uint32_t>(segs);
    init_bounds_kernel<<<grid_for(segs, 256), 256, 0, st>>>(bounds, seg_count, segs);
    if (n > 0)
        centroid_bounds_kernel<<<grid_for(n, 256), 256, 0, st>>>(plo, phi, seg, n, bounds, seg_count);
    uint64_t* keys = sc.get<uint64_t>(n);
    uint32_t* vals = sc.get<uint32_t>(n);
    if (n > 0) morton_kernel<<<grid_for(n, 256), 256, 0, st>>>(plo, phi, seg, n, bounds, keys, vals);
    int seg_bits = 0;
    while ((1u << seg_bits) < segs) ++seg_bits;
    radix_sort(keys, vals, n, 30 + seg_bits, sc);
    out.order = vals;
    // segment first positions
    uint32_t* seg_first = sc.get<uint32_t>(segs);
    check_cuda(cudaMemcpyAsync(seg_first, seg_count, 4ull * segs, cudaMemcpyDeviceToDevice, st), "copy");
    exclusive_scan(seg_first, segs, sc);
    // hierarchy
    int ni = n > 0 ? (int)n - 1 : 0;
    int* left = sc.get<int>(ni);
    int* right = sc.get<int>(ni);
    int* first = sc.get<int>(ni);
    int* last = sc.get<int>(ni);
    int* parent = sc.get<int>(ni + n);
    uint32_t* visits = sc.get<uint32_t>(ni);
    float4* blo = sc.get<float4>(ni + n);
    float4* bhi = sc.get<float4>(ni + n);
    check_cuda(cudaMemsetAsync(parent, 0xff, sizeof(int) * (size_t)std::max<uint64_t>(ni + n, 1), st), "memset");
    check_cuda(cudaMemsetAsync(visits, 0, sizeof(uint32_t) * (size_t)std::max(ni, 1), st), "memset");
    if (ni > 0) karras_kernel<<<grid_for(ni, 256), 256, 0, st>>>(keys, (int)n, left, right, first, last, parent);
    if (n > 0)
        refit_kernel<<<grid_for(n, 256), 256, 0, st>>>((int)n, vals, plo, phi, left, right, parent,
                                                       blo, bhi, visits);
    out.blo = blo;
    out.bhi = bhi;
    out.roots = sc.get<int>(segs);
    segment_roots_kernel<<<grid_for(segs, 256), 256, 0, st>>>(seg_first, seg_count, segs, (int)n,
                                                               first, last, out.roots);
    out.tv = TreeView{(int)n, ni, left, right, first, last, blo, bhi};
    return out;
}

// Generic BVH4 build over primitive boxes grouped in non-decreasing segments.
Build4 build_bvh4(const float4* plo, const float4* phi, const uint32_t* seg, uint32_t n,
                  uint32_t segs, int leaf_max, bool leaf_by_prim, const uint32_t* leaf_ids,
                  DeviceBuffer& node_buf, Scratch& sc) {
    cudaStream_t st = sc.stream;
    Build4 out;
    Binary bin = build_binary(plo, phi, seg, n, segs, sc);
    uint32_t* vals = bin.order;
    out.order = vals;
    out.blo = bin.blo;
    out.bhi = bin.bhi;
    // collapse
    uint64_t cap = (uint64_t)n + segs + 1;
    node_buf.alloc(cap * 128ull);
    int* lvl_a = sc.get<int>(cap);
    int* lvl_b = sc.get<int>(cap);
    int* chosen = sc.get<int>(4 * cap);
    uint32_t* icount = sc.get<uint32_t>(cap + 1);
    check_cuda(cudaMemcpyAsync(lvl_a, bin.roots, sizeof(int) * segs, cudaMemcpyDeviceToDevice, st), "copy");
    out.roots = bin.roots;
    TreeView tv = bin.tv;
    uint64_t base = 0;
    uint32_t L = segs;
    while (L > 0) {
        out.levels++;
        out.level_start.push_back(base);
        collapse_choose_kernel<<<grid_for(L, 128), 128, 0, st>>>(tv, lvl_a, L, leaf_max, chosen, icount);
        check_cuda(cudaMemsetAsync(icount + L, 0, 4, st), "memset");
        exclusive_scan(icount, (uint64_t)L + 1, sc);
        uint32_t next = 0;
        check_cuda(cudaMemcpyAsync(&next, icount + L, 4, cudaMemcpyDeviceToHost, st), "copy");
        check_cuda(cudaStreamSynchronize(st), "sync");
        if (base + L + next > cap) fail(TT_ERR_OVERFLOW, "bvh node capacity exceeded");
        collapse_emit_kernel<<<grid_for(L, 128), 128, 0, st>>>(
            tv, lvl_a, L, leaf_max, chosen, icount, base, base + L, node_buf.as<uint4>(), lvl_b,
            vals, leaf_ids, leaf_by_prim ? 1 : 0);
        base += L;
        L = next;
        std::swap(lvl_a, lvl_b);
    }
    out.nodes = base;
    out.level_start.push_back(base);
    return out;
}

// ---------------------------------------------------------------- collapse to the compressed 8-wide format
// The flat structure's wide format (oracle/ref_bvh.h collapse_wide restates it; the node arrays
// must match byte for byte): level by level from the root, each node expands the largest-area
// internal child until it holds eight children (subtrees of at most WIDE_LEAF_MAX primitives are
// leaf children), assigns them to slots by octant direction, and quantises their boxes to 8 bits
// per plane (outwards) relative to the node's low corner with a power-of-two scale per axis.
// 80-byte node: origin xyz, biased exponents and the internal-slot mask; child base, triangle
// base, eight meta bytes (leaf slot: offset | unary count << 5); qlo/qhi bytes per axis.
#ifndef TT_WIDE_LEAF_MAX
#define TT_WIDE_LEAF_MAX 3
#endif
constexpr int WIDE_LEAF_MAX = TT_WIDE_LEAF_MAX;

__device__ __forceinline__ bool wide_leafish(const TreeView& t, int r) {
    return t.is_leaf(r) || t.ncount(r) <= WIDE_LEAF_MAX;
}

__device__ __forceinline__ uint32_t wide_exponent(float extent) {
    float x = extent / 255.0f;
    uint32_t bits = __float_as_uint(x);
    uint32_t e = (bits >> 23) & 0xffu;
    if (e == 0u) e = 1u;
    else if ((bits & 0x7fffffu) != 0u) e += 1u;
    while (e < 254u && 255.0f * __uint_as_float(e << 23) < extent) e += 1u;
    return e > 254u ? 254u : e;
}
__device__ __forceinline__ uint32_t wide_q(float q) { return (uint32_t)(q < 0.0f ? 0.0f : (q > 255.0f ? 255.0f : q)); }

__global__ void wide_choose_kernel(TreeView t, const int* level, uint32_t L, int* slot_child, uint32_t* icount,
                                   uint32_t* tcount) {
    uint32_t li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= L) return;
    int r = level[li];
    int ch[8];
    int cnt = 0;
    if (r >= 0) {
        if (wide_leafish(t, r)) {
            ch[0] = r;
            cnt = 1;
        } else {
            ch[0] = t.left[r];
            ch[1] = t.right[r];
            cnt = 2;
            while (cnt < 8) {
                int best = -1;
                float best_area = -1.0f;
                for (int c = 0; c < cnt; ++c) {
                    if (wide_leafish(t, ch[c])) continue;
                    float a = t.half_area(ch[c]);
                    if (best < 0 || a > best_area) {
                        best = c;
                        best_area = a;
                    }
                }
                if (best < 0) break;
                int v = ch[best];
                for (int c = cnt; c > best + 1; --c) ch[c] = ch[c - 1];
                ch[best] = t.left[v];
                ch[best + 1] = t.right[v];
                cnt++;
            }
        }
    }
    // node box and child centroids
    float lo[3] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000)};
    float hi[3] = {__int_as_float(0xff800000), __int_as_float(0xff800000), __int_as_float(0xff800000)};
    float cc[8][3];
    for (int c = 0; c < cnt; ++c) {
        float4 l = t.blo[ch[c]], h = t.bhi[ch[c]];
        lo[0] = fminf(lo[0], l.x); lo[1] = fminf(lo[1], l.y); lo[2] = fminf(lo[2], l.z);
        hi[0] = fmaxf(hi[0], h.x); hi[1] = fmaxf(hi[1], h.y); hi[2] = fmaxf(hi[2], h.z);
        cc[c][0] = (l.x + h.x) * 0.5f;
        cc[c][1] = (l.y + h.y) * 0.5f;
        cc[c][2] = (l.z + h.z) * 0.5f;
    }
    // slots: greedy cheapest (child, slot) pairs, cost = centroid offset along the slot's octant
    float pc[3] = {(lo[0] + hi[0]) * 0.5f, (lo[1] + hi[1]) * 0.5f, (lo[2] + hi[2]) * 0.5f};
    float cost[8][8];
    for (int c = 0; c < cnt; ++c) {
        float dx = cc[c][0] - pc[0], dy = cc[c][1] - pc[1], dz = cc[c][2] - pc[2];
        for (int s = 0; s < 8; ++s) {
            float sx = (s & 1) ? -dx : dx, sy = (s & 2) ? -dy : dy, sz = (s & 4) ? -dz : dz;
            cost[c][s] = __fadd_rn(__fadd_rn(sx, sy), sz);
        }
    }
    int child_at[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
    uint32_t child_done = 0u, slot_used = 0u;
    for (int k = 0; k < cnt; ++k) {
        int bc = -1, bs = -1;
        float best = 0.0f;
        for (int s = 0; s < 8; ++s) {
            if ((slot_used >> s) & 1u) continue;
            for (int c = 0; c < cnt; ++c) {
                if ((child_done >> c) & 1u) continue;
                if (bc < 0 || cost[c][s] < best) {
                    bc = c;
                    bs = s;
                    best = cost[c][s];
                }
            }
        }
        child_done |= 1u << bc;
        slot_used |= 1u << bs;
        child_at[bs] = ch[bc];
    }
    uint32_t internal = 0, tris = 0;
    for (int s = 0; s < 8; ++s) {
        int v = child_at[s];
        slot_child[8 * li + s] = v;
        if (v < 0) continue;
        if (wide_leafish(t, v)) tris += (uint32_t)t.ncount(v);
        else internal++;
    }
    icount[li] = internal;
    tcount[li] = tris;
}

__global__ void wide_emit_kernel(TreeView t, const int* level, uint32_t L, const int* slot_child,
                                 const uint32_t* ioff, const uint32_t* toff, uint64_t next_base, uint32_t tri_level_base,
                                 uint64_t node_base, uint4* nodes, int* next_level, uint32_t* tri_order) {
    uint32_t li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= L) return;
    int child_at[8];
    int cnt = 0;
    float lo[3] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000)};
    float hi[3] = {__int_as_float(0xff800000), __int_as_float(0xff800000), __int_as_float(0xff800000)};
    for (int s = 0; s < 8; ++s) {
        int v = slot_child[8 * li + s];
        child_at[s] = v;
        if (v < 0) continue;
        cnt++;
        float4 l = t.blo[v], h = t.bhi[v];
        lo[0] = fminf(lo[0], l.x); lo[1] = fminf(lo[1], l.y); lo[2] = fminf(lo[2], l.z);
        hi[0] = fmaxf(hi[0], h.x); hi[1] = fmaxf(hi[1], h.y); hi[2] = fmaxf(hi[2], h.z);
    }
    uint32_t w[20];
    uint32_t e[3];
    float scale[3], org[3];
    for (int a = 0; a < 3; ++a) {
        org[a] = cnt > 0 ? lo[a] : 0.0f;
        e[a] = cnt > 0 ? wide_exponent(__fsub_rn(hi[a], lo[a])) : 127u;
        scale[a] = __uint_as_float(e[a] << 23);
        w[a] = __float_as_uint(org[a]);
    }
    uint32_t child_base = (uint32_t)(next_base + ioff[li]);
    uint32_t tri_base = tri_level_base + toff[li];
    uint32_t imask = 0u, meta[2] = {0u, 0u}, q[12] = {};
    uint32_t tri_off = 0u, rank = 0u;
    for (int s = 0; s < 8; ++s) {
        int v = child_at[s];
        uint32_t qb[6];
        if (v < 0) {
            qb[0] = qb[2] = qb[4] = 255u;  // lo planes
            qb[1] = qb[3] = qb[5] = 0u;    // hi planes
        } else {
            float4 l = t.blo[v], h = t.bhi[v];
            const float cl[3] = {l.x, l.y, l.z}, chh[3] = {h.x, h.y, h.z};
            for (int a = 0; a < 3; ++a) {
                qb[2 * a] = wide_q(floorf(__fdiv_rn(__fsub_rn(cl[a], org[a]), scale[a])));
                qb[2 * a + 1] = wide_q(ceilf(__fdiv_rn(__fsub_rn(chh[a], org[a]), scale[a])));
            }
            if (wide_leafish(t, v)) {
                uint32_t k = (uint32_t)t.ncount(v), f = (uint32_t)t.nfirst(v);
                uint32_t m = tri_off | (((1u << k) - 1u) << 5);
                meta[s >> 2] |= m << (8 * (s & 3));
                for (uint32_t j = 0; j < k; ++j) tri_order[tri_base + tri_off + j] = f + j;
                tri_off += k;
            } else {
                imask |= 1u << s;
                next_level[ioff[li] + rank] = v;
                rank++;
            }
        }
        // q words: [qlo_x 0..3, qlo_x 4..7, qhi_x 0..3, qhi_x 4..7, qlo_y ..., qhi_z 4..7]
        for (int a = 0; a < 3; ++a) {
            q[4 * a + (s >> 2)] |= qb[2 * a] << (8 * (s & 3));
            q[4 * a + 2 + (s >> 2)] |= qb[2 * a + 1] << (8 * (s & 3));
        }
    }
    w[3] = e[0] | (e[1] << 8) | (e[2] << 16) | (imask << 24);
    w[4] = child_base;
    w[5] = tri_base;
    w[6] = meta[0];
    w[7] = meta[1];
    for (int k = 0; k < 12; ++k) w[8 + k] = q[k];
    uint4* nd = nodes + 5ull * (node_base + li);
    for (int k = 0; k < 5; ++k) nd[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
}

__global__ void gather_wide_records_kernel(const float4* in, const uint32_t* order, const uint32_t* tri_order,
                                           uint32_t n, float4* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t s = order[tri_order[i]];
    out[3ull * i + 0] = in[3ull * s + 0];
    out[3ull * i + 1] = in[3ull * s + 1];
    out[3ull * i + 2] = in[3ull * s + 2];
}

struct Build8 {
    uint64_t nodes = 0;
    uint32_t levels = 0;
    std::vector<uint64_t> level_start;
};

// The wide format of one segment's binary LBVH into `node_buf` (80-byte nodes); `tri_order`
// (n entries) receives the sorted position of each wide triangle record.
Build8 collapse_wide(const Binary& bin, uint32_t n, DeviceBuffer& node_buf, uint32_t* tri_order, Scratch& sc) {
    cudaStream_t st = sc.stream;
    Build8 out;
    uint64_t cap = (uint64_t)n + 2;
    node_buf.alloc(cap * 80ull);
    int* lvl_a = sc.get<int>(cap);
    int* lvl_b = sc.get<int>(cap);
    int* slot_child = sc.get<int>(8 * cap);
    uint32_t* icount = sc.get<uint32_t>(cap + 1);
    uint32_t* tcount = sc.get<uint32_t>(cap + 1);
    check_cuda(cudaMemcpyAsync(lvl_a, bin.roots, sizeof(int), cudaMemcpyDeviceToDevice, st), "copy");
    uint64_t base = 0;
    uint32_t L = 1, tri_level_base = 0;
    while (L > 0) {
        out.levels++;
        out.level_start.push_back(base);
        wide_choose_kernel<<<grid_for(L, 128), 128, 0, st>>>(bin.tv, lvl_a, L, slot_child, icount, tcount);
        check_cuda(cudaMemsetAsync(icount + L, 0, 4, st), "memset");
        check_cuda(cudaMemsetAsync(tcount + L, 0, 4, st), "memset");
        exclusive_scan(icount, (uint64_t)L + 1, sc);
        exclusive_scan(tcount, (uint64_t)L + 1, sc);
        uint32_t totals[2] = {0u, 0u};
        check_cuda(cudaMemcpyAsync(&totals[0], icount + L, 4, cudaMemcpyDeviceToHost, st), "copy");
        check_cuda(cudaMemcpyAsync(&totals[1], tcount + L, 4, cudaMemcpyDeviceToHost, st), "copy");
        check_cuda(cudaStreamSynchronize(st), "sync");
        if (base + L + totals[0] > cap || (uint64_t)tri_level_base + totals[1] > n)
            fail(TT_ERR_OVERFLOW, "wide bvh capacity exceeded");
        wide_emit_kernel<<<grid_for(L, 128), 128, 0, st>>>(bin.tv, lvl_a, L, slot_child, icount, tcount, base + L,
                                                           tri_level_base, base, node_buf.as<uint4>(), lvl_b,
                                                           tri_order);
        base += L;
        tri_level_base += totals[1];
        L = totals[0];
        std::swap(lvl_a, lvl_b);
    }
    out.nodes = base;
    out.level_start.push_back(base);
    return out;
}

}  // namespace

// Max |coordinate| of the root box of a built tree (the bound of the slab-test margins).
static float root_bound(const int* roots, const float4* blo, const float4* bhi, cudaStream_t stream) {
    int root = 0;
    check_cuda(cudaMemcpyAsync(&root, roots, sizeof(int), cudaMemcpyDeviceToHost, stream), "root");
    check_cuda(cudaStreamSynchronize(stream), "sync");
    float4 rb[2];
    check_cuda(cudaMemcpyAsync(&rb[0], blo + root, 16, cudaMemcpyDeviceToHost, stream), "root box");
    check_cuda(cudaMemcpyAsync(&rb[1], bhi + root, 16, cudaMemcpyDeviceToHost, stream), "root box");
    check_cuda(cudaStreamSynchronize(stream), "sync");
    float bound = 0.0f;
    for (float v : {rb[0].x, rb[0].y, rb[0].z, rb[1].x, rb[1].y, rb[1].z}) bound = std::max(bound, std::fabs(v));
    return bound;
}

static void build_flat(const BuildInput& in, cudaStream_t stream, int leaf_max, bool wide, BvhResult& out) {
    Scratch sc(stream);
    out.flat = true;
    out.wide = wide;
    std::vector<uint32_t> base(in.instance_count + 1, 0);
    for (uint32_t i = 0; i < in.instance_count; ++i)
        base[i + 1] = base[i] + in.meshes_host[in.instances_host[i].mesh_index].index_count / 3u;
    uint32_t n = base[in.instance_count];
    out.flat_tri_count = n;
    out.flat_tris.alloc(std::max<uint64_t>(n, 1) * 48ull);
    if (n == 0) {
        out.flat_nodes_buf.alloc(0);
        out.flat_nodes = 0;
        out.flat_levels = 0;
        check_cuda(cudaStreamSynchronize(stream), "bvh build");
        return;
    }
    tt_instance* d_inst = sc.get<tt_instance>(in.instance_count);
    uint32_t* d_base = sc.get<uint32_t>(in.instance_count + 1);
    check_cuda(cudaMemcpyAsync(d_inst, in.instances_host, sizeof(tt_instance) * in.instance_count,
                               cudaMemcpyHostToDevice, stream), "instances");
    check_cuda(cudaMemcpyAsync(d_base, base.data(), 4ull * (in.instance_count + 1), cudaMemcpyHostToDevice, stream),
               "bases");
    float4* plo = sc.get<float4>(n);
    float4* phi = sc.get<float4>(n);
    uint32_t* seg = sc.get<uint32_t>(n);
    float4* recs = sc.get<float4>(3ull * n);
    flat_prims_kernel<<<grid_for(n, 256), 256, 0, stream>>>(in.positions, in.indices, d_inst, d_base,
                                                             in.instance_count, n, plo, phi, seg, recs);
    if (wide) {
        Binary bin = build_binary(plo, phi, seg, n, 1, sc);
        uint32_t* tri_order = sc.get<uint32_t>(n);
        Build8 b = collapse_wide(bin, n, out.flat_nodes_buf, tri_order, sc);
        out.flat_nodes = b.nodes;
        out.flat_levels = b.levels;
        out.flat_level_start = b.level_start;
        gather_wide_records_kernel<<<grid_for(n, 256), 256, 0, stream>>>(recs, bin.order, tri_order, n,
                                                                          out.flat_tris.as<float4>());
        out.flat_bound = root_bound(bin.roots, bin.blo, bin.bhi, stream);
        check_cuda(cudaStreamSynchronize(stream), "bvh build");
        check_cuda(cudaGetLastError(), "bvh build kernels");
        return;
    }
    Build4 b = build_bvh4(plo, phi, seg, n, 1, leaf_max, false, nullptr, out.flat_nodes_buf, sc);
    out.flat_nodes = b.nodes;
    out.flat_levels = b.levels;
    out.flat_level_start = b.level_start;
    gather_records_kernel<<<grid_for(n, 256), 256, 0, stream>>>(recs, b.order, n, out.flat_tris.as<float4>());
    out.flat_tri_base.alloc(4ull * (in.instance_count + 1));
    out.flat_tri_record.alloc(4ull * n);
    check_cuda(cudaMemcpyAsync(out.flat_tri_base.ptr, base.data(), 4ull * (in.instance_count + 1),
                               cudaMemcpyHostToDevice, stream), "triangle bases");
    tri_record_kernel<<<grid_for(n, 256), 256, 0, stream>>>(out.flat_tris.as<float4>(), out.flat_tri_base.as<uint32_t>(),
                                                            n, out.flat_tri_record.as<uint32_t>());
    out.flat_bound = root_bound(b.roots, b.blo, b.bhi, stream);
    check_cuda(cudaStreamSynchronize(stream), "bvh build");
    check_cuda(cudaGetLastError(), "bvh build kernels");
}

// ---------------------------------------------------------------- refit (instance update)
// Child boxes of node j: the union of its planes over its children.
static __device__ __forceinline__ void node_box(const uint4* nodes, uint32_t j, f3& lo, f3& hi) {
    const float4* p = reinterpret_cast<const float4*>(nodes) + 8ull * j;
    uint32_t cnt = reinterpret_cast<const uint4*>(p)[7].x;
    float4 lx = p[0], hx = p[1], ly = p[2], hy = p[3], lz = p[4], hz = p[5];
    const float al[3][4] = {{lx.x, lx.y, lx.z, lx.w}, {ly.x, ly.y, ly.z, ly.w}, {lz.x, lz.y, lz.z, lz.w}};
    const float ah[3][4] = {{hx.x, hx.y, hx.z, hx.w}, {hy.x, hy.y, hy.z, hy.w}, {hz.x, hz.y, hz.z, hz.w}};
    float l[3], h[3];
    for (int a = 0; a < 3; ++a) {
        l[a] = __int_as_float(0x7f800000);
        h[a] = __int_as_float(0xff800000);
        for (uint32_t c = 0; c < cnt; ++c) {
            l[a] = fmn(l[a], al[a][c]);
            h[a] = fmx(h[a], ah[a][c]);
        }
    }
    lo = f3{l[0], l[1], l[2]};
    hi = f3{h[0], h[1], h[2]};
}

// World box of one flat record (object-space vertices, instance in b.w) under the instance's
// current transform: the flat build's box (flat_prims_kernel).
static __device__ __forceinline__ void record_box(const float4* recs, uint32_t q, const tt_instance* inst, f3& lo, f3& hi) {
    float4 a = recs[3ull * q], b = recs[3ull * q + 1], c = recs[3ull * q + 2];
    const tt_instance& in = inst[__float_as_uint(b.w)];
    f3 w0 = mat43_point(in.transform, f3{a.x, a.y, a.z});
    f3 w1 = mat43_point(in.transform, f3{b.x, b.y, b.z});
    f3 w2 = mat43_point(in.transform, f3{c.x, c.y, c.z});
    lo = f3{canon(fmn(fmn(w0.x, w1.x), w2.x)), canon(fmn(fmn(w0.y, w1.y), w2.y)), canon(fmn(fmn(w0.z, w1.z), w2.z))};
    hi = f3{canon(fmx(fmx(w0.x, w1.x), w2.x)), canon(fmx(fmx(w0.y, w1.y), w2.y)), canon(fmx(fmx(w0.z, w1.z), w2.z))};
}

// World box of an instance from its mesh's BLAS root box (instance_prims_kernel).
static __device__ __forceinline__ void instance_box(const tt_instance& in, const uint4* blas, f3& lo, f3& hi) {
    f3 ml, mh;
    node_box(blas, in.mesh_index, ml, mh);
    f3 l = splat(__int_as_float(0x7f800000)), h = splat(__int_as_float(0xff800000));
    for (int k = 0; k < 8; ++k) {
        f3 c = f3{(k & 1) ? mh.x : ml.x, (k & 2) ? mh.y : ml.y, (k & 4) ? mh.z : ml.z};
        f3 w = mat43_point(in.transform, c);
        l = f3{fmn(l.x, w.x), fmn(l.y, w.y), fmn(l.z, w.z)};
        h = f3{fmx(h.x, w.x), fmx(h.y, w.y), fmx(h.z, w.z)};
    }
    lo = f3{canon(l.x), canon(l.y), canon(l.z)};
    hi = f3{canon(h.x), canon(h.y), canon(h.z)};
}

// Refits the nodes [start, end) of one level from their children (deeper levels are done).
static __global__ void refit_level_kernel(uint4* nodes, uint64_t start, uint64_t end, const float4* recs,
                                   const tt_instance* inst, const uint4* blas, int tlas) {
    uint64_t i = start + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= end) return;
    float4* p = reinterpret_cast<float4*>(nodes) + 8ull * i;
    uint4 ch = reinterpret_cast<uint4*>(p)[6];
    uint32_t cnt = reinterpret_cast<uint4*>(p)[7].x;
    const uint32_t child[4] = {ch.x, ch.y, ch.z, ch.w};
    float bx[6][4];
    for (int c = 0; c < 4; ++c) {
        f3 lo = splat(__int_as_float(0x7f800000)), hi = splat(__int_as_float(0xff800000));
        if ((uint32_t)c < cnt) {
            uint32_t r = child[c];
            if (r & 0x80000000u) {
                if (tlas) {
                    instance_box(inst[r & 0x07ffffffu], blas, lo, hi);
                } else {
                    uint32_t f = r & 0x07ffffffu, k = ((r >> 27) & 0xfu) + 1u;
                    for (uint32_t q = f; q < f + k; ++q) {
                        f3 l, h;
                        record_box(recs, q, inst, l, h);
                        lo = f3{fmn(lo.x, l.x), fmn(lo.y, l.y), fmn(lo.z, l.z)};
                        hi = f3{fmx(hi.x, h.x), fmx(hi.y, h.y), fmx(hi.z, h.z)};
                    }
                }
            } else {
                node_box(nodes, r, lo, hi);
            }
        }
        bx[0][c] = lo.x;
        bx[1][c] = hi.x;
        bx[2][c] = lo.y;
        bx[3][c] = hi.y;
        bx[4][c] = lo.z;
        bx[5][c] = hi.z;
    }
    for (int k = 0; k < 6; ++k) p[k] = make_float4(bx[k][0], bx[k][1], bx[k][2], bx[k][3]);
}

// Root-node bound: max |coordinate| over the root's child boxes.
static float root_node_bound(const DeviceBuffer& nodes, cudaStream_t stream) {
    float4 pl[8];
    check_cuda(cudaMemcpyAsync(pl, nodes.ptr, 128, cudaMemcpyDeviceToHost, stream), "root node");
    check_cuda(cudaStreamSynchronize(stream), "sync");
    uint32_t cnt = reinterpret_cast<const uint4*>(pl)[7].x;
    float bound = 0.0f;
    for (int k = 0; k < 6; ++k) {
        const float v[4] = {pl[k].x, pl[k].y, pl[k].z, pl[k].w};
        for (uint32_t c = 0; c < cnt; ++c) bound = std::max(bound, std::fabs(v[c]));
    }
    return bound;
}

void refit_scene_bvh(const tt_instance* d_instances, cudaStream_t stream, BvhResult& b) {
    if (b.wide) fail(TT_ERR_UNSUPPORTED, "the compressed wide format is rebuilt, not refitted");
    bool flat = b.flat;
    DeviceBuffer& nodes = flat ? b.flat_nodes_buf : b.tlas;
    const std::vector<uint64_t>& ls = flat ? b.flat_level_start : b.tlas_level_start;
    if ((flat ? b.flat_nodes : b.tlas_nodes) == 0) return;
    for (size_t l = ls.size() - 1; l-- > 0;) {
        uint64_t start = ls[l], end = ls[l + 1];
        if (end <= start) continue;
        refit_level_kernel<<<grid_for(end - start, 128), 128, 0, stream>>>(
            nodes.as<uint4>(), start, end, flat ? b.flat_tris.as<float4>() : nullptr, d_instances,
            flat ? nullptr : b.blas.as<uint4>(), flat ? 0 : 1);
    }
    check_cuda(cudaGetLastError(), "refit");
    float bound = root_node_bound(nodes, stream);
    if (flat) b.flat_bound = bound;
    else b.tlas_bound = bound;
}

void build_scene_bvh(const BuildInput& in, cudaStream_t stream, int leaf_max, bool flat, bool wide, BvhResult& out) {
    if (flat) {
        build_flat(in, stream, leaf_max, wide, out);
        return;
    }
    Scratch sc(stream);
    // triangle primitives (mesh order)
    std::vector<uint32_t> tri_base(in.mesh_count + 1, 0);
    for (uint32_t m = 0; m < in.mesh_count; ++m)
        tri_base[m + 1] = tri_base[m] + in.meshes_host[m].index_count / 3u;
    uint32_t n = tri_base[in.mesh_count];
    uint32_t segs = std::max<uint32_t>(in.mesh_count, 1);
    tt_mesh* d_meshes = sc.get<tt_mesh>(segs);
    uint32_t* d_base = sc.get<uint32_t>(in.mesh_count + 1);
    if (in.mesh_count) {
        check_cuda(cudaMemcpyAsync(d_meshes, in.meshes_host, sizeof(tt_mesh) * in.mesh_count,
                                   cudaMemcpyHostToDevice, stream), "upload meshes");
        check_cuda(cudaMemcpyAsync(d_base, tri_base.data(), 4ull * (in.mesh_count + 1),
                                   cudaMemcpyHostToDevice, stream), "upload bases");
    }
    if (in.mesh_count == 0) {  // empty scene: no BLAS, no TLAS, every ray misses
        out.blas.alloc(0);
        out.tris.alloc(0);
        out.tlas.alloc(0);
        out.blas_nodes = out.tlas_nodes = out.tri_count = 0;
        out.blas_levels = out.tlas_levels = 0;
        return;
    }
    float4* plo = sc.get<float4>(n);
    float4* phi = sc.get<float4>(n);
    uint32_t* seg = sc.get<uint32_t>(n);
    float4* recs = sc.get<float4>(3ull * n);
    if (n > 0)
        triangle_prims_kernel<<<grid_for(n, 256), 256, 0, stream>>>(
            in.positions, in.indices, d_meshes, d_base, in.mesh_count, n, plo, phi, seg, recs);
    Build4 b = build_bvh4(plo, phi, seg, n, in.mesh_count, leaf_max, false, nullptr, out.blas, sc);
    out.blas_nodes = b.nodes;
    out.blas_levels = b.levels;
    out.tri_count = n;
    out.tris.alloc(std::max<uint64_t>(n, 1) * 48ull);
    if (n > 0)
        gather_records_kernel<<<grid_for(n, 256), 256, 0, stream>>>(recs, b.order, n, out.tris.as<float4>());
    // mesh boxes -> instance primitives
    float4* mlo = sc.get<float4>(segs);
    float4* mhi = sc.get<float4>(segs);
    if (in.mesh_count)
        segment_boxes_kernel<<<grid_for(in.mesh_count, 256), 256, 0, stream>>>(b.roots, in.mesh_count,
                                                                              b.blo, b.bhi, mlo, mhi);
    std::vector<uint32_t> ids;
    for (uint32_t i = 0; i < in.instance_count; ++i) {
        uint32_t m = in.instances_host[i].mesh_index;
        if (in.meshes_host[m].index_count / 3u > 0) ids.push_back(i);
    }
    uint32_t ni = (uint32_t)ids.size();
    uint32_t* d_ids = sc.get<uint32_t>(ni);
    tt_instance* d_inst = sc.get<tt_instance>(std::max<uint32_t>(in.instance_count, 1));
    if (ni) {
        check_cuda(cudaMemcpyAsync(d_ids, ids.data(), 4ull * ni, cudaMemcpyHostToDevice, stream), "ids");
        check_cuda(cudaMemcpyAsync(d_inst, in.instances_host, sizeof(tt_instance) * in.instance_count,
                                   cudaMemcpyHostToDevice, stream), "instances");
    }
    float4* ilo = sc.get<float4>(ni);
    float4* ihi = sc.get<float4>(ni);
    uint32_t* iseg = sc.get<uint32_t>(ni);
    if (ni)
        instance_prims_kernel<<<grid_for(ni, 128), 128, 0, stream>>>(d_inst, d_ids, ni, mlo, mhi,
                                                                     ilo, ihi, iseg);
    if (ni > 0) {
        Build4 tb = build_bvh4(ilo, ihi, iseg, ni, 1, 1, true, d_ids, out.tlas, sc);
        out.tlas_nodes = tb.nodes;
        out.tlas_levels = tb.levels;
        out.tlas_level_start = tb.level_start;
        out.tlas_bound = root_bound(tb.roots, tb.blo, tb.bhi, stream);  // bound of the world-space slab margins
    } else {
        out.tlas_nodes = 0;
        out.tlas_levels = 0;
    }
    check_cuda(cudaStreamSynchronize(stream), "bvh build");
    check_cuda(cudaGetLastError(), "bvh build kernels");
}

void exclusive_scan_u32(uint32_t* data, uint64_t n, cudaStream_t stream) {
    Scratch sc(stream);
    exclusive_scan(data, n, sc);
}

}  // namespace tt
