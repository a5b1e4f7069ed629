// BVH4 traversal on sm_103a: the replacement for the RT-core ray queries of the reference
// (GL_EXT_ray_query in src/integrate/integrate.glsl:112-127 and 168-185).  A scene carries one
// of two acceleration structures: the two-level one (a TLAS over instances whose leaves enter
// per-mesh BLAS in object space) or the flat one (a single BVH over the world boxes of every
// (instance, triangle) pair, whose records keep object-space vertices and the instance index).
// Both find the same closest hit, bit for bit.
//
// Semantics (identical to the CPU oracle's ray queries):
//   * instances are intersected in object space, o' = inverse_transform * (o, 1),
//     d' = mat3(inverse_transform) * d, sharing the ray parameter t;
//   * object-space vertices are the dequantised snorm16 positions, value / 32767;
//   * watertight ray/triangle test (Woop, Benthin & Wald, JCGT 2013) with the
//     double-precision fallback when an edge function is exactly zero; front faces have
//     det > 0 (geometric normal cross(p1-p0, p2-p0) facing the ray origin);
//   * hits count for tmin <= t <= tmax; the closest hit is the smallest t with ties broken
//     by the smaller (instance, primitive) pair, so any traversal order gives the same hit;
//   * child boxes are tested conservatively: slab distances are widened by
//     2^-20 (B + |o|) |1/d| per axis (B bounds the box coordinates: 1 in object space, where
//     vertices are snorm16, the scene bound in world space), more than their rounding error.
//
// Layout in HBM: BVH4 nodes are 128-byte records (six float4 of child-box planes, the child
// references, the child count) read as seven 16-byte vector loads; the
// triangles of each mesh are stored in leaf order as 48-byte records (three float4), so a
// leaf is one contiguous run; per-instance traversal data is a 64-byte record (the three
// rows of the world-to-object matrix and the mesh index).  The traversal stack lives in
// shared memory, one column per thread.
#pragma once

#include "tt_common.cuh"

namespace tt {

// Wide-format traversal variants (build-time switches): NEAREST descends into the nearest hit
// internal child of each node before its siblings; FAST_DECODE folds the byte-to-float bias of the
// quantised planes into the slab bases (one instruction less per plane, boxes one step looser).
#ifndef TT_WIDE_NEAREST
#define TT_WIDE_NEAREST 0
#endif
#ifndef TT_WIDE_FAST_DECODE
#define TT_WIDE_FAST_DECODE 0
#endif

constexpr uint32_t CHILD_LEAF = 0x80000000u;
constexpr uint32_t STACK_MARKER = 0xffffffffu;
#ifndef TT_TRAVERSAL_STACK
#define TT_TRAVERSAL_STACK 64
#endif
constexpr int TRAVERSAL_STACK = TT_TRAVERSAL_STACK;  // entries per thread, in shared memory
// The wavefront trace kernel also comes with this shorter stack, used for scenes that need no
// more: less shared memory per block leaves more of the SM's L1 to cache nodes.
constexpr int SHORT_TRAVERSAL_STACK = 48;
constexpr uint32_t TRAVERSAL_ITERATION_LIMIT = 1u << 24;
constexpr uint32_t ERR_STACK_OVERFLOW = 1u;
constexpr uint32_t ERR_ITERATION_LIMIT = 2u;
constexpr uint32_t ERR_TENSOR_WAIT = 4u;  // a tensor-core completion wait ran out (cache queries)
constexpr uint32_t ERR_PRIMARY_MISMATCH = 8u;  // a camera ray's rasterised closest hit failed its own ray test

TT_HD uint32_t leaf_first(uint32_t r) { return r & 0x07ffffffu; }
TT_HD uint32_t leaf_count(uint32_t r) { return ((r >> 27) & 0xfu) + 1u; }

// One texture: format (TEX_*), mip levels, level-0 extent and the byte offset of every level
// in the scene's texture data (levels of max(1, w >> k) x max(1, h >> k) texels, 16-byte aligned).
struct DevTexture {
    uint32_t format, levels, width, height;
    uint64_t offset[16];
};

struct DevScene {
    const int16_t* positions;
    const uint32_t* indices;
    const tt_vertex* vertices;
    const tt_material* materials;
    const tt_instance* instances;
    const tt_mesh* meshes;
    const tt_emissive_triangle* emissive;
    const uint32_t* light_prim;  // primitive index of each emissive triangle in its instance's mesh
    const uint4* blas;        // 8 x uint4 per node (two-level only)
    const float4* tris;       // 3 x float4 per triangle record
    const uint4* tlas;        // 8 x uint4 per node: the TLAS, or the flat BVH
    const float4* inst_xform; // 4 x float4 per instance: inverse rows 0..2, (mesh, material, index_offset, vertex_offset)
    const uint8_t* inst_bucket;  // shading-queue bucket of each instance's material (wavefront integrator)
    uint32_t bucket_lobes;       // byte b: the union of the lobe sets (lobe_set_of) of bucket b's materials
    uint32_t emissive_count;
    uint32_t instance_count;
    uint32_t has_tlas;
    float tlas_bound;  // max |coordinate| of the world boxes in `tlas`
    uint32_t flat;     // 1: `tlas`/`tris` hold the flat BVH
    uint32_t wide;     // 1: the flat BVH is in the compressed 8-wide format (80-byte nodes in `tlas`)
    uint32_t stack_need;  // traversal stack entries the structure can need (3 per level + 1)
    const DevTexture* textures;  // texture table (null when the scene has no textures)
    const uint8_t* tex_data;     // all texture levels
    const float* srgb;           // 256-entry sRGB-to-linear table
    uint32_t textured;           // 1 when some material samples a texture
    uint32_t light_exact;        // TT_LIGHT_VISIBILITY_TRIANGLE: shadow rays test the sampled triangle itself
    uint32_t light_power;        // TT_LIGHT_SELECTION_POWER: lights picked through `light_alias`
    const float4* light_alias;   // per emissive triangle: (keep probability, alias index bits, pdf, 0)
    const float4* light_rec;     // per emissive triangle: LIGHT_RECORD float4 (light_records_kernel)
    // flat BVH4 scenes: the scene triangle index of (instance, primitive) is tri_base[instance] +
    // primitive (so it orders hits as the closest-hit tie-break does), tri_record maps it to its
    // record in `tris`; null for the other structures
    const uint32_t* tri_base;    // instance_count + 1 entries
    const uint32_t* tri_record;  // tri_count entries
    uint32_t tri_count;          // records in `tris` (flat BVH4 scenes)
};
// A light record: what light sampling derives from an emissive triangle, computed once per
// scene and instance update.  float4 0..2: world vertices p0, p1, p2 with w = area, instance
// bits, hash bits; 3: unit normal, emission-texture slots of the material; 4: the material's
// constant emission, material index bits; 5: packed texture coordinates of the three corners,
// primitive index bits.
constexpr int LIGHT_RECORD = 6;

struct Hit {
    int hit;
    float t, u, v;
    uint32_t instance, prim;
};

struct Counters {
    uint32_t blas_nodes, tlas_nodes, triangles, instances;
};

struct RayPre {
    f3 o;
    uint32_t k;  // kx | ky << 2 | kz << 4
    float sx, sy, sz;
};
TT_HD float comp(f3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
TT_HD RayPre ray_precompute(f3 o, f3 d) {
    RayPre r;
    r.o = o;
    int kz = 0;
    if (fabsf(d.y) > fabsf(d.x)) kz = 1;
    if (fabsf(d.z) > fabsf(comp(d, kz))) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (comp(d, kz) < 0.0f) {
        int t = kx;
        kx = ky;
        ky = t;
    }
    r.k = (uint32_t)kx | ((uint32_t)ky << 2) | ((uint32_t)kz << 4);
    float dz = comp(d, kz);
    r.sx = comp(d, kx) / dz;
    r.sy = comp(d, ky) / dz;
    r.sz = 1.0f / dz;
    return r;
}

TT_HD bool intersect_triangle(const RayPre& r, f3 p0, f3 p1, f3 p2, bool cull_back, float tmin,
                              float tmax, float& t_out, float& u_out, float& v_out) {
    f3 A = p0 - r.o, B = p1 - r.o, C = p2 - r.o;
    int kx = (int)(r.k & 3u), ky = (int)((r.k >> 2) & 3u), kz = (int)(r.k >> 4);
    float Akz = comp(A, kz), Bkz = comp(B, kz), Ckz = comp(C, kz);
    float Ax = comp(A, kx) - r.sx * Akz;
    float Ay = comp(A, ky) - r.sy * Akz;
    float Bx = comp(B, kx) - r.sx * Bkz;
    float By = comp(B, ky) - r.sy * Bkz;
    float Cx = comp(C, kx) - r.sx * Ckz;
    float Cy = comp(C, ky) - r.sy * Ckz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {  // rare: resolve edges in double precision
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    bool neg = U < 0.0f || V < 0.0f || W < 0.0f;
    bool pos = U > 0.0f || V > 0.0f || W > 0.0f;
    float det = U + V + W;
    float T = U * (r.sz * Akz) + V * (r.sz * Bkz) + W * (r.sz * Ckz);
    float rcp = 1.0f / det;
    float t = T * rcp;
    bool ok = (cull_back ? !neg : !(neg && pos)) && det != 0.0f && t >= tmin && t <= tmax;
    t_out = t;
    u_out = V * rcp;
    v_out = W * rcp;
    return ok;
}

TT_HD bool closer(float t, uint32_t inst, uint32_t prim, const Hit& best) {
    if (!best.hit) return true;
    if (t < best.t) return true;
    if (t > best.t) return false;
    if (inst != best.instance) return inst < best.instance;
    return prim < best.prim;
}
TT_HD bool finite3(f3 d) { return isfinite(d.x) && isfinite(d.y) && isfinite(d.z); }
TT_HD float safe_inv(float d) {
    float a = fabsf(d) < 1e-20f ? (d < 0.0f ? -1e-20f : 1e-20f) : d;
    return 1.0f / a;
}

// Per-ray data of the slab test: per axis the inverse direction, the near-plane selector and
// -o/d widened by the conservative margin towards the near and the far side.
struct NodeRay {
    f3 inv, nob_near, nob_far;
    uint32_t near;  // bit a set: the near plane of axis a is the high bound (1/d < 0)
};
TT_HD NodeRay node_ray(f3 o, f3 d, float bound) {
    NodeRay r;
    r.inv = f3{safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
    const float oa[3] = {o.x, o.y, o.z}, ia[3] = {r.inv.x, r.inv.y, r.inv.z};
    float nn[3], nf[3];
    r.near = 0u;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float nob = -(oa[a] * ia[a]);
        float E = (bound + fabsf(oa[a])) * fabsf(ia[a]) * 9.5367431640625e-07f;
        nn[a] = nob - E;
        nf[a] = nob + E;
        if (!(ia[a] >= 0.0f)) r.near |= 1u << a;
    }
    r.nob_near = f3{nn[0], nn[1], nn[2]};
    r.nob_far = f3{nf[0], nf[1], nf[2]};
    return r;
}

// Slab test of the (up to) four children of node `i`; returns the hit mask, entry distances
// and child references.  Empty slots hold +inf/-inf planes and never pass.
TT_HD int node_hits(const uint4* nodes, uint32_t i, const NodeRay& r, float tmin, float tbest, float* tn_out,
                    uint32_t* child) {
    const float4* p = reinterpret_cast<const float4*>(nodes) + 8ull * i;
    float4 nx = __ldg(p + ((r.near & 1u) ? 1 : 0)), fx = __ldg(p + ((r.near & 1u) ? 0 : 1));
    float4 ny = __ldg(p + ((r.near & 2u) ? 3 : 2)), fy = __ldg(p + ((r.near & 2u) ? 2 : 3));
    float4 nz = __ldg(p + ((r.near & 4u) ? 5 : 4)), fz = __ldg(p + ((r.near & 4u) ? 4 : 5));
    uint4 ch = __ldg(reinterpret_cast<const uint4*>(p + 6));
    child[0] = ch.x;
    child[1] = ch.y;
    child[2] = ch.z;
    child[3] = ch.w;
    const float n4x[4] = {nx.x, nx.y, nx.z, nx.w}, f4x[4] = {fx.x, fx.y, fx.z, fx.w};
    const float n4y[4] = {ny.x, ny.y, ny.z, ny.w}, f4y[4] = {fy.x, fy.y, fy.z, fy.w};
    const float n4z[4] = {nz.x, nz.y, nz.z, nz.w}, f4z[4] = {fz.x, fz.y, fz.z, fz.w};
    int mask = 0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float tn = fmx(fmx(__fmaf_rn(n4x[c], r.inv.x, r.nob_near.x), __fmaf_rn(n4y[c], r.inv.y, r.nob_near.y)),
                       fmx(__fmaf_rn(n4z[c], r.inv.z, r.nob_near.z), tmin));
        float tf = fmn(fmn(__fmaf_rn(f4x[c], r.inv.x, r.nob_far.x), __fmaf_rn(f4y[c], r.inv.y, r.nob_far.y)),
                       fmn(__fmaf_rn(f4z[c], r.inv.z, r.nob_far.z), tbest));
        tn_out[c] = tn;
        if (tn <= tf) mask |= 1 << c;
    }
    return mask;
}

TT_HD f3 tri_vertex(float4 v) { return f3{v.x, v.y, v.z}; }

// Resumable closest-hit traversal through the TLAS/BLAS.  trace_init() sets a ray up and
// trace_step() performs one step; it returns true when the traversal is finished and the
// result is in `best`.  A step does at most one triangle test (from the lane's pending leaf
// range) and at most one stack pop or node visit, so that the lanes of a warp execute the
// same two pieces of code each step instead of one lane's long run of leaf triangles: a node
// visit sorts its hit children by entry distance, makes the nearest internal child the next
// node, makes the nearest leaf the pending triangle range when that range is empty, and
// pushes the rest.  `stack` is the thread's column in shared memory (element k at
// stack[k * stride]); `err` receives ERR_* bits when the stack or the iteration limit would
// be exceeded, in which case the traversal ends.
struct TraceState {
    f3 o, d;     // world ray
    NodeRay nr;  // slab-test data of the current level (world at the top, object inside instances)
    RayPre rp;   // triangle-test data of the instance `inst` (object space)
    Hit best;
    float tmin, tbest;
    uint32_t inst, cur, iterations;
    uint32_t tri_next, tri_left;  // pending triangles
    int sp;
    bool in_blas;  // two-level: inside an instance; flat: the object ray of `inst` is not finite
    bool have, cull;
    // wide format: the node group being expanded (first child node, and hit slots in visiting
    // order in bits 24..31 above the node's internal-slot mask) and the pending triangle group
    // (first record, and the records still to test as a bit mask)
    uint32_t ng_base, ng_bits, tg_base, tg_bits;
};

TT_HD void trace_init(TraceState& st, const DevScene& sc, f3 o, f3 d, float tmin, float tmax, bool cull) {
    st.best.hit = 0;
    st.best.t = 0.0f;
    st.best.u = 0.0f;
    st.best.v = 0.0f;
    st.best.instance = 0u;
    st.best.prim = 0u;
    st.o = o;
    st.d = d;
    st.tmin = tmin;
    st.tbest = tmax;
    st.cull = cull;
    st.nr = node_ray(o, d, sc.tlas_bound);
    st.rp = ray_precompute(o, d);
    st.inst = sc.flat ? 0xffffffffu : 0u;  // flat: no object ray set up yet
    st.in_blas = false;
    st.sp = 0;
    st.cur = 0u;
    st.iterations = 0u;
    st.tri_next = 0u;
    st.tri_left = 0u;
    st.have = finite3(d) && sc.has_tlas != 0u;  // a NaN/inf direction or an empty scene misses
    // wide format: the root (node 0) as the only member of a group whose slots map to nodes 0..7
    st.ng_base = 0u;
    st.ng_bits = (st.have && !TT_WIDE_NEAREST) ? ((1u << (24u + st.nr.near)) | 0xffu) : 0u;  // NEAREST: `cur`
    st.tg_base = 0u;
    st.tg_bits = 0u;
}

// Makes the next trace_step finish with the current result (the ray traces nothing more).
TT_HD void trace_stop(TraceState& st) {
    st.have = false;
    st.ng_bits = 0u;
    st.tg_bits = 0u;
}

template <bool COUNT, int STACK = TRAVERSAL_STACK>
__device__ __forceinline__ bool trace_push(TraceState& st, uint32_t* stack, int stride, uint32_t* err,
                                           uint32_t v) {
    if (st.sp >= STACK) {
        atomicOr(err, ERR_STACK_OVERFLOW);
        return false;
    }
    stack[(st.sp++) * stride] = v;
    return true;
}

// The object-space ray of instance `inst`: o' = inverse * (o, 1), d' = mat3(inverse) * d.
__device__ __forceinline__ void instance_ray(const DevScene& sc, uint32_t inst, f3 o, f3 d, f3& oo, f3& od,
                                             uint32_t& mesh) {
    const float4* x = sc.inst_xform + 4ull * inst;
    float4 r0 = __ldg(x + 0), r1 = __ldg(x + 1), r2 = __ldg(x + 2);
    mesh = __float_as_uint(__ldg(x + 3).x);
    oo = f3{r0.x * o.x + r0.y * o.y + r0.z * o.z + r0.w * 1.0f, r1.x * o.x + r1.y * o.y + r1.z * o.z + r1.w * 1.0f,
            r2.x * o.x + r2.y * o.y + r2.z * o.z + r2.w * 1.0f};
    od = f3{r0.x * d.x + r0.y * d.y + r0.z * d.z, r1.x * d.x + r1.y * d.y + r1.z * d.z,
            r2.x * d.x + r2.y * d.y + r2.z * d.z};
}

// Sorts the hit children of a node by entry distance and splits them into the nearest
// internal child (the next node), the nearest leaf (the pending triangle range, when that is
// free and `leaves` is set) and the rest, pushed farthest first.  Returns false on overflow.
template <int STACK = TRAVERSAL_STACK>
__device__ __forceinline__ bool visit_children(TraceState& st, int mask, const float* tn, const uint32_t* ch,
                                               bool leaves, uint32_t* stack, int stride, uint32_t* err) {
    float key[4];
    uint32_t val[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        bool take = ((mask >> c) & 1) && tn[c] <= st.tbest;
        key[c] = take ? tn[c] : __int_as_float(0x7f800000);
        val[c] = take ? ch[c] : STACK_MARKER;
    }
#define TT_SWAP(i, j)                                                  \
    {                                                                  \
        bool sw = key[j] < key[i];                                     \
        float k0 = sw ? key[j] : key[i], k1 = sw ? key[i] : key[j];    \
        uint32_t v0 = sw ? val[j] : val[i], v1 = sw ? val[i] : val[j]; \
        key[i] = k0; key[j] = k1; val[i] = v0; val[j] = v1;            \
    }
    TT_SWAP(0, 1) TT_SWAP(2, 3) TT_SWAP(0, 2) TT_SWAP(1, 3) TT_SWAP(1, 2)
#undef TT_SWAP
    int next = -1, leaf = -1, npush = 0;
    uint32_t next_ref = 0u, leaf_ref = 0u;
    bool push[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        bool valid = val[c] != STACK_MARKER;
        bool is_leaf = leaves && (val[c] & CHILD_LEAF);
        bool take_leaf = valid && is_leaf && leaf < 0 && st.tri_left == 0u;
        bool take_next = valid && !is_leaf && next < 0;
        leaf = take_leaf ? c : leaf;
        leaf_ref = take_leaf ? val[c] : leaf_ref;
        next = take_next ? c : next;
        next_ref = take_next ? val[c] : next_ref;
        push[c] = valid && !take_leaf && !take_next;
        npush += push[c] ? 1 : 0;
    }
    if (st.sp + npush > STACK) {
        atomicOr(err, ERR_STACK_OVERFLOW);
        return false;
    }
#pragma unroll
    for (int c = 3; c >= 0; --c) {
        if (push[c]) stack[st.sp * stride] = val[c];
        st.sp += push[c] ? 1 : 0;
    }
    st.tri_next = leaf >= 0 ? leaf_first(leaf_ref) : st.tri_next;
    st.tri_left = leaf >= 0 ? leaf_count(leaf_ref) : st.tri_left;
    st.have = next >= 0;
    st.cur = next >= 0 ? next_ref : st.cur;
    return true;
}

// One step through the flat BVH: the pending triangle (setting up the object ray of its
// instance when it differs from the last one), then one pop or node visit.  Internal nodes
// are popped while triangles are pending; a leaf waits until the pending range is done.
// Node visits are counted as TLAS nodes, object-ray set-ups as instances.
//
// EARLY: the pop and the node this step visits are decided before the triangle test (they
// depend only on the pending count after it) and the node's 128-byte line is prefetched into
// L1, so that its fetch overlaps the triangle test.  Measured on GB300 this pays for shadow
// rays (whose seeded tbest prunes most subtrees: shadow stage 18.8 -> 16.6 ms per frame of
// the 1080p benchmark) and costs extension rays 4 % (81.2 -> 84.6 ms), so the trace kernel
// enables it for shadow rays only.  Either order finds the same hit.
template <bool COUNT, bool EARLY = false, int STACK = TRAVERSAL_STACK>
__device__ __forceinline__ bool trace_step_flat(TraceState& st, const DevScene& sc, uint32_t* stack, int stride,
                                                uint32_t* err, Counters& cnt) {
    if (++st.iterations > TRAVERSAL_ITERATION_LIMIT) {
        atomicOr(err, ERR_ITERATION_LIMIT);
        return true;
    }
    bool visit = st.have, pop_leaf = false;
    uint32_t e = 0u;
    if (EARLY) {
        if (!visit && st.sp > 0) {
            uint32_t left = st.tri_left - (st.tri_left > 0u ? 1u : 0u);
            e = stack[(st.sp - 1) * stride];
            if (!(e & CHILD_LEAF)) {
                --st.sp;
                st.cur = e;
                visit = true;
            } else if (left == 0u) {
                --st.sp;
                pop_leaf = true;
            }
        }
        if (visit) asm volatile("prefetch.global.L1 [%0];" ::"l"(sc.tlas + 8ull * st.cur));
    }
    if (st.tri_left > 0u) {
        const float4* tr = sc.tris + 3ull * st.tri_next;
        float4 a = __ldg(tr + 0), b = __ldg(tr + 1), cc = __ldg(tr + 2);
        uint32_t prim = __float_as_uint(a.w), inst = __float_as_uint(b.w);
        if (inst != st.inst) {
            f3 oo, od;
            uint32_t mesh;
            instance_ray(sc, inst, st.o, st.d, oo, od, mesh);
            st.inst = inst;
            st.in_blas = !finite3(od);
            st.rp = ray_precompute(oo, od);
            if (COUNT) cnt.instances++;
        }
        if (COUNT) cnt.triangles++;
        float t, u, v;
        bool better = !st.in_blas &&
                      intersect_triangle(st.rp, tri_vertex(a), tri_vertex(b), tri_vertex(cc), st.cull, st.tmin,
                                         st.tbest, t, u, v) &&
                      closer(t, st.inst, prim, st.best);
        st.best.hit = better ? 1 : st.best.hit;
        st.best.t = better ? t : st.best.t;
        st.best.u = better ? u : st.best.u;
        st.best.v = better ? v : st.best.v;
        st.best.instance = better ? st.inst : st.best.instance;
        st.best.prim = better ? prim : st.best.prim;
        st.tbest = better ? t : st.tbest;
        st.tri_next++;
        st.tri_left--;
    }
    if (EARLY) {
        if (pop_leaf) {
            st.tri_next = leaf_first(e);
            st.tri_left = leaf_count(e);
        }
        if (!visit) return st.sp == 0 && st.tri_left == 0u;  // finished, waiting, or a leaf made pending
    } else if (!st.have) {
        if (st.sp == 0) return st.tri_left == 0u;
        e = stack[(st.sp - 1) * stride];
        if (e & CHILD_LEAF) {
            if (st.tri_left > 0u) return false;
            --st.sp;
            st.tri_next = leaf_first(e);
            st.tri_left = leaf_count(e);
            return false;
        }
        --st.sp;
        st.cur = e;
        st.have = true;
    }
    if (COUNT) cnt.tlas_nodes++;
    float tn[4];
    uint32_t ch[4];
    int mask = node_hits(sc.tlas, st.cur, st.nr, st.tmin, st.tbest, tn, ch);
    return !visit_children<STACK>(st, mask, tn, ch, true, stack, stride, err);
}

// Closest-hit traversal of the flat BVH by a whole warp, for coherent rays (camera rays of
// neighbouring pixels).  The warp walks one stack of (node or leaf reference, lane mask) entries
// in shared memory: every lane in an entry's mask tests the node's children (or the leaf's
// records) against its own ray with its own closest distance so far, and a child is pushed with
// the mask of the lanes whose ray enters it, farthest first by the entry distances of the lowest
// such lane.  A lane therefore tests every node and record its ray would test traced alone
// (and possibly more, with a larger closest distance at the time), so it finds the same closest
// hit, while each node is fetched once for the warp and all lanes run the same instructions.
// Every lane of the warp must call it; lanes with !valid take no part.  `stack` holds
// PACKET_STACK entries; overflow and the iteration limit set ERR_* bits and end the traversal.
constexpr int PACKET_STACK = 64;
__device__ __forceinline__ Hit packet_trace_flat(const DevScene& sc, f3 o, f3 d, bool valid, float tmin, float tmax,
                                                 bool cull, uint2* stack, uint32_t* err) {
    const uint32_t lane = threadIdx.x & 31u;
    Hit best;
    best.hit = 0;
    best.t = best.u = best.v = 0.0f;
    best.instance = best.prim = 0u;
    float tbest = tmax;
    const NodeRay nr = node_ray(o, d, sc.tlas_bound);
    RayPre rp = ray_precompute(o, d);
    uint32_t inst = 0xffffffffu;  // the instance whose object ray `rp` holds
    bool inst_bad = false;        // that object ray is not finite
    bool have = valid && finite3(d) && sc.has_tlas != 0u;
    uint32_t root = __ballot_sync(0xffffffffu, have);
    int sp = 0;
    if (root) {
        if (lane == 0u) stack[0] = make_uint2(0u, root);
        sp = 1;
    }
    __syncwarp();
    uint32_t iterations = 0u;
    while (sp > 0) {
        if (++iterations > TRAVERSAL_ITERATION_LIMIT) {
            if (lane == 0u) atomicOr(err, ERR_ITERATION_LIMIT);
            break;
        }
        const uint2 e = stack[sp - 1];
        --sp;
        __syncwarp();  // every lane has read the entry before lane 0 writes over it
        const bool mine = (e.y >> lane) & 1u;
        if (e.x & CHILD_LEAF) {
            const uint32_t first = leaf_first(e.x), count = leaf_count(e.x);
            for (uint32_t k = 0; k < count; ++k) {
                const float4* tr = sc.tris + 3ull * (first + k);
                float4 a = __ldg(tr + 0), b = __ldg(tr + 1), cc = __ldg(tr + 2);
                if (mine) {
                    uint32_t prim = __float_as_uint(a.w), in = __float_as_uint(b.w);
                    if (in != inst) {
                        f3 oo, od;
                        uint32_t mesh;
                        instance_ray(sc, in, o, d, oo, od, mesh);
                        inst = in;
                        inst_bad = !finite3(od);
                        rp = ray_precompute(oo, od);
                    }
                    float t, u, v;
                    bool better = !inst_bad &&
                                  intersect_triangle(rp, tri_vertex(a), tri_vertex(b), tri_vertex(cc), cull, tmin, tbest,
                                                     t, u, v) &&
                                  closer(t, inst, prim, best);
                    if (better) {
                        best.hit = 1;
                        best.t = t;
                        best.u = u;
                        best.v = v;
                        best.instance = inst;
                        best.prim = prim;
                        tbest = t;
                    }
                }
            }
            continue;
        }
        float tn[4];
        uint32_t ch[4];
        const int hm = node_hits(sc.tlas, e.x, nr, tmin, tbest, tn, ch) & (mine ? 0xf : 0);
        uint32_t cm[4], any = 0u;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            cm[c] = __ballot_sync(0xffffffffu, (hm >> c) & 1);
            any |= cm[c];
        }
        if (!any) continue;
        const int rep = __ffs(any) - 1;
        // the entered children, farthest first (a sorting network on lane-uniform keys; children
        // no lane enters sort last with key -inf and are not pushed)
        float key[4];
        uint2 ent[4];
        int npush = 0;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            float k = __shfl_sync(0xffffffffu, tn[c], rep);
            key[c] = cm[c] ? k : __int_as_float(0xff800000);
            ent[c] = make_uint2(ch[c], cm[c]);
            npush += cm[c] ? 1 : 0;
        }
#define TT_DESC(i, j)                                               \
    {                                                               \
        bool sw = key[j] > key[i];                                  \
        float k0 = sw ? key[j] : key[i], k1 = sw ? key[i] : key[j]; \
        uint2 e0 = sw ? ent[j] : ent[i], e1 = sw ? ent[i] : ent[j]; \
        key[i] = k0; key[j] = k1; ent[i] = e0; ent[j] = e1;         \
    }
        TT_DESC(0, 1) TT_DESC(2, 3) TT_DESC(0, 2) TT_DESC(1, 3) TT_DESC(1, 2)
#undef TT_DESC
        if (sp + npush > PACKET_STACK) {
            if (lane == 0u) atomicOr(err, ERR_STACK_OVERFLOW);
            break;
        }
        if (lane == 0u) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (i < npush) stack[sp + i] = ent[i];
        }
        sp += npush;
        __syncwarp();
    }
    return best;
}

// ---------------------------------------------------------------- compressed 8-wide format
// Node (80 bytes, five 16-byte loads): origin xyz and, in the fourth word, the biased exponents
// of the per-axis scales and the internal-slot mask; child base, triangle base and eight meta
// bytes (a leaf slot's first record offset | unary record count << 5); then the child boxes as
// bytes, per axis the eight low planes and the eight high planes.  A child plane is
// origin + q 2^(exponent - 127); the slab distance enters as fma(q, 2^(e - 127) / d,
// fma(origin, 1/d, -o/d -+ E)), conservative with the margin E of node_ray.
//
// Traversal (after Ylitie, Karras & Laine, HPG 2017): the hit internal children of a node form a
// node group visited in the order the slots were assigned for the ray's direction octant (slot s
// at position s ^ octant, lowest position first), the hit leaf children a triangle group (a mask
// of records).  A step tests at most one record of the pending triangle group and visits at most
// one node; the remainder of a node group, and a triangle group produced while another is
// pending, wait on the stack as two-word entries (node groups have hit bits in 24..31, triangle
// groups do not).

// Byte k of `w` as a float plane coordinate: the bits 0x4b0000bb (byte bb of w below the exponent
// of 2^23) are the float 2^23 + bb; minus 2^23 unless the caller folds the bias into its bases.
__device__ __forceinline__ float wide_plane(uint32_t w, uint32_t k) {
    float biased = __uint_as_float(__byte_perm(w, 0x4bu, 0x4550u | k));
    return TT_WIDE_FAST_DECODE ? biased : biased - 8388608.0f;
}
// Bit i of the result is bit i ^ o of `m` (8 bits).
__device__ __forceinline__ uint32_t permute_octant(uint32_t m, uint32_t o) {
    if (o & 1u) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
    if (o & 2u) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
    if (o & 4u) m = ((m & 0x0fu) << 4) | ((m >> 4) & 0x0fu);
    return m;
}

template <int STACK>
__device__ __forceinline__ bool wide_push(TraceState& st, uint32_t* stack, int stride, uint32_t* err, uint32_t base,
                                          uint32_t bits) {
    if (2 * st.sp + 2 > STACK) {
        atomicOr(err, ERR_STACK_OVERFLOW);
        return false;
    }
    stack[(2 * st.sp) * stride] = base;
    stack[(2 * st.sp + 1) * stride] = bits;
    st.sp++;
    return true;
}

template <bool COUNT, int STACK = TRAVERSAL_STACK>
__device__ __forceinline__ bool trace_step_wide(TraceState& st, const DevScene& sc, uint32_t* stack, int stride,
                                                uint32_t* err, Counters& cnt) {
    if (++st.iterations > TRAVERSAL_ITERATION_LIMIT) {
        atomicOr(err, ERR_ITERATION_LIMIT);
        return true;
    }
    // 1. one record of the pending triangle group
    if (st.tg_bits != 0u) {
        uint32_t j = (uint32_t)(__ffs(st.tg_bits) - 1);
        st.tg_bits &= st.tg_bits - 1u;
        const float4* tr = sc.tris + 3ull * (st.tg_base + j);
        float4 a = __ldg(tr + 0), b = __ldg(tr + 1), cc = __ldg(tr + 2);
        uint32_t prim = __float_as_uint(a.w), inst = __float_as_uint(b.w);
        if (inst != st.inst) {
            f3 oo, od;
            uint32_t mesh;
            instance_ray(sc, inst, st.o, st.d, oo, od, mesh);
            st.inst = inst;
            st.in_blas = !finite3(od);
            st.rp = ray_precompute(oo, od);
            if (COUNT) cnt.instances++;
        }
        if (COUNT) cnt.triangles++;
        float t, u, v;
        bool better = !st.in_blas &&
                      intersect_triangle(st.rp, tri_vertex(a), tri_vertex(b), tri_vertex(cc), st.cull, st.tmin,
                                         st.tbest, t, u, v) &&
                      closer(t, st.inst, prim, st.best);
        st.best.hit = better ? 1 : st.best.hit;
        st.best.t = better ? t : st.best.t;
        st.best.u = better ? u : st.best.u;
        st.best.v = better ? v : st.best.v;
        st.best.instance = better ? st.inst : st.best.instance;
        st.best.prim = better ? prim : st.best.prim;
        st.tbest = better ? t : st.tbest;
    }
    // 2. the next node: the pending nearest child, else the next child of the node group, else
    // the stack
    uint32_t node;
    if (TT_WIDE_NEAREST && st.have) {
        node = st.cur;
        st.have = false;
    } else {
        if ((st.ng_bits >> 24) == 0u) {
            if (st.sp == 0) return st.tg_bits == 0u;
            uint32_t base = stack[(2 * st.sp - 2) * stride], bits = stack[(2 * st.sp - 1) * stride];
            if ((bits >> 24) == 0u) {  // a triangle group: it becomes pending once the current one is done
                if (st.tg_bits != 0u) return false;
                --st.sp;
                st.tg_base = base;
                st.tg_bits = bits;
                return false;
            }
            --st.sp;
            st.ng_base = base;
            st.ng_bits = bits;
        }
        uint32_t pos = (uint32_t)(__ffs(st.ng_bits >> 24) - 1);
        st.ng_bits &= ~(1u << (24u + pos));
        uint32_t slot = pos ^ st.nr.near;
        node = st.ng_base + (uint32_t)__popc(st.ng_bits & 0xffu & ((1u << slot) - 1u));
        if (!TT_WIDE_NEAREST && (st.ng_bits >> 24) != 0u &&
            !wide_push<STACK>(st, stack, stride, err, st.ng_base, st.ng_bits))
            return true;
    }
    if (COUNT) cnt.tlas_nodes++;
    const uint4* nd = sc.tlas + 5ull * node;
    uint4 w0 = __ldg(nd + 0), w1 = __ldg(nd + 1), qx = __ldg(nd + 2), qy = __ldg(nd + 3), qz = __ldg(nd + 4);
    const float ia[3] = {st.nr.inv.x, st.nr.inv.y, st.nr.inv.z};
    const float nn[3] = {st.nr.nob_near.x, st.nr.nob_near.y, st.nr.nob_near.z};
    const float nf[3] = {st.nr.nob_far.x, st.nr.nob_far.y, st.nr.nob_far.z};
    const float org[3] = {__uint_as_float(w0.x), __uint_as_float(w0.y), __uint_as_float(w0.z)};
    const uint4 q[3] = {qx, qy, qz};
    float step[3], bn[3], bf[3];
    uint32_t qn[3][2], qf[3][2];  // near / far plane bytes per axis, slots 0..3 and 4..7
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        step[a] = __uint_as_float(((w0.w >> (8 * a)) & 0xffu) << 23) * ia[a];
        bn[a] = __fmaf_rn(org[a], ia[a], nn[a]);
        bf[a] = __fmaf_rn(org[a], ia[a], nf[a]);
        if (TT_WIDE_FAST_DECODE) {
            // planes enter as the biased floats 2^23 + q: fold -2^23 step into the bases and widen
            // them by one quantisation step, which covers the rounding of the folded bases
            float big = step[a] * 8388608.0f, one = fabsf(step[a]);
            bn[a] = (bn[a] - big) - one;
            bf[a] = (bf[a] - big) + one;
        }
        bool neg = (st.nr.near >> a) & 1u;  // the near plane is the high one
        qn[a][0] = neg ? q[a].z : q[a].x;
        qn[a][1] = neg ? q[a].w : q[a].y;
        qf[a][0] = neg ? q[a].x : q[a].z;
        qf[a][1] = neg ? q[a].y : q[a].w;
    }
    const uint32_t imask = w0.w >> 24;
    const uint32_t meta[2] = {w1.z, w1.w};
    uint32_t hit = 0u, tmask = 0u;
    float tnear[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        uint32_t h = c >> 2, k = c & 3;
        float tn = fmx(fmx(__fmaf_rn(wide_plane(qn[0][h], k), step[0], bn[0]),
                           __fmaf_rn(wide_plane(qn[1][h], k), step[1], bn[1])),
                       fmx(__fmaf_rn(wide_plane(qn[2][h], k), step[2], bn[2]), st.tmin));
        float tf = fmn(fmn(__fmaf_rn(wide_plane(qf[0][h], k), step[0], bf[0]),
                           __fmaf_rn(wide_plane(qf[1][h], k), step[1], bf[1])),
                       fmn(__fmaf_rn(wide_plane(qf[2][h], k), step[2], bf[2]), st.tbest));
        tnear[c] = tn;
        uint32_t m = (meta[h] >> (8 * k)) & 0xffu;
        bool valid = ((imask >> c) & 1u) || m != 0u;
        bool in = valid && tn <= tf;
        hit |= in ? (1u << c) : 0u;
        bool leaf = in && !((imask >> c) & 1u);
        tmask |= leaf ? ((m >> 5) << (m & 31u)) : 0u;
    }
    uint32_t ihit = hit & imask;
    if (TT_WIDE_NEAREST) {
        // descend into the nearest internal child next; its hit siblings form the new node group
        int best = -1;
        float bt = 0.0f;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            bool take = ((ihit >> c) & 1u) && (best < 0 || tnear[c] < bt);
            best = take ? c : best;
            bt = take ? tnear[c] : bt;
        }
        if (best >= 0) {
            uint32_t rest = ihit & ~(1u << best);
            if (rest != 0u) {
                if ((st.ng_bits >> 24) != 0u && !wide_push<STACK>(st, stack, stride, err, st.ng_base, st.ng_bits))
                    return true;
                st.ng_base = w1.x;
                st.ng_bits = (permute_octant(rest, st.nr.near) << 24) | imask;
            }
            st.cur = w1.x + (uint32_t)__popc(imask & ((1u << best) - 1u));
            st.have = true;
        }
    } else {
        st.ng_base = w1.x;
        st.ng_bits = (permute_octant(ihit, st.nr.near) << 24) | imask;
    }
    if (tmask != 0u) {
        if (st.tg_bits == 0u) {
            st.tg_base = w1.y;
            st.tg_bits = tmask;
        } else if (!wide_push<STACK>(st, stack, stride, err, w1.y, tmask)) {
            return true;
        }
    }
    return false;
}

// ACCEL: ACCEL_ANY dispatches on the scene at run time; ACCEL_FLAT_ONLY, ACCEL_TWO_LEVEL_ONLY and
// ACCEL_WIDE_ONLY compile one structure's step (the caller has checked sc.flat and sc.wide);
// ACCEL_NO_WIDE dispatches between the flat and the two-level step (no scene is wide).  Kernels
// compile the variant they need: every step compiled into a loop enlarges it, and a loop that
// holds all three ran the ReSTIR passes measurably slower on flat scenes.
constexpr int ACCEL_ANY = 0, ACCEL_FLAT_ONLY = 1, ACCEL_TWO_LEVEL_ONLY = 2, ACCEL_WIDE_ONLY = 3, ACCEL_NO_WIDE = 4;

template <bool COUNT, int ACCEL = ACCEL_ANY, bool EARLY = false, int STACK = TRAVERSAL_STACK>
__device__ __forceinline__ bool trace_step(TraceState& st, const DevScene& sc, uint32_t* stack, int stride,
                                           uint32_t* err, Counters& cnt) {
    if (ACCEL == ACCEL_WIDE_ONLY || (ACCEL == ACCEL_ANY && sc.wide))
        return trace_step_wide<COUNT, STACK>(st, sc, stack, stride, err, cnt);
    if (ACCEL == ACCEL_FLAT_ONLY || ((ACCEL == ACCEL_ANY || ACCEL == ACCEL_NO_WIDE) && sc.flat))
        return trace_step_flat<COUNT, EARLY, STACK>(st, sc, stack, stride, err, cnt);
    if (++st.iterations > TRAVERSAL_ITERATION_LIMIT) {
        atomicOr(err, ERR_ITERATION_LIMIT);
        return true;
    }
    // 1. one pending triangle
    if (st.tri_left > 0u) {
        const float4* tr = sc.tris + 3ull * st.tri_next;
        float4 a = __ldg(tr + 0), b = __ldg(tr + 1), cc = __ldg(tr + 2);
        if (COUNT) cnt.triangles++;
        float t, u, v;
        uint32_t prim = __float_as_uint(a.w);
        bool better = intersect_triangle(st.rp, tri_vertex(a), tri_vertex(b), tri_vertex(cc), st.cull, st.tmin,
                                         st.tbest, t, u, v) &&
                      closer(t, st.inst, prim, st.best);
        st.best.hit = better ? 1 : st.best.hit;
        st.best.t = better ? t : st.best.t;
        st.best.u = better ? u : st.best.u;
        st.best.v = better ? v : st.best.v;
        st.best.instance = better ? st.inst : st.best.instance;
        st.best.prim = better ? prim : st.best.prim;
        st.tbest = better ? t : st.tbest;
        st.tri_next++;
        st.tri_left--;
    }
    // 2. one pop or node visit
    if (!st.have) {
        if (st.tri_left > 0u) return false;  // leave the instance only after its pending triangles
        if (st.sp == 0) return true;
        uint32_t e = stack[(--st.sp) * stride];
        if (e == STACK_MARKER) {
            st.in_blas = false;
            st.nr = node_ray(st.o, st.d, sc.tlas_bound);
            return false;
        }
        if (st.in_blas && (e & CHILD_LEAF)) {  // a postponed leaf becomes the pending range
            st.tri_next = leaf_first(e);
            st.tri_left = leaf_count(e);
            return false;
        }
        st.cur = e;
        st.have = true;
    }
    if (!st.in_blas && (st.cur & CHILD_LEAF)) {
        st.inst = leaf_first(st.cur);
        f3 oo, od;
        uint32_t mesh;
        instance_ray(sc, st.inst, st.o, st.d, oo, od, mesh);
        if (COUNT) cnt.instances++;
        if (!finite3(od)) {
            st.have = false;
            return false;
        }
        if (!trace_push<COUNT, STACK>(st, stack, stride, err, STACK_MARKER)) return true;
        st.rp = ray_precompute(oo, od);
        st.nr = node_ray(oo, od, 1.0f);
        st.in_blas = true;
        st.cur = mesh;
        return false;
    }
    if (COUNT) {
        if (st.in_blas) cnt.blas_nodes++;
        else cnt.tlas_nodes++;
    }
    float tn[4];
    uint32_t ch[4];
    int mask = node_hits(st.in_blas ? sc.blas : sc.tlas, st.cur, st.nr, st.tmin, st.tbest, tn, ch);
    return !visit_children<STACK>(st, mask, tn, ch, st.in_blas, stack, stride, err);
}

// Closest hit, run to completion.
template <bool COUNT, int ACCEL = ACCEL_ANY>
__device__ __forceinline__ Hit trace_closest(const DevScene& sc, f3 o, f3 d, float tmin, float tmax, bool cull,
                                             uint32_t* stack, int stride, uint32_t* err, Counters& cnt) {
    TraceState st;
    trace_init(st, sc, o, d, tmin, tmax, cull);
    while (!trace_step<COUNT, ACCEL>(st, sc, stack, stride, err, cnt)) {
    }
    return st.best;
}

}  // namespace tt
