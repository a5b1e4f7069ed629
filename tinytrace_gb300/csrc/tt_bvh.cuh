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
    uint32_t emissive_count;
    uint32_t instance_count;
    uint32_t has_tlas;
    float tlas_bound;  // max |coordinate| of the world boxes in `tlas`
    uint32_t flat;     // 1: `tlas`/`tris` hold the flat BVH
    uint32_t stack_need;  // traversal stack entries the structure can need (3 per level + 1)
    const DevTexture* textures;  // texture table (null when the scene has no textures)
    const uint8_t* tex_data;     // all texture levels
    const float* srgb;           // 256-entry sRGB-to-linear table
    uint32_t textured;           // 1 when some material samples a texture
    uint32_t light_exact;        // TT_LIGHT_VISIBILITY_TRIANGLE: shadow rays test the sampled triangle itself
    uint32_t light_power;        // TT_LIGHT_SELECTION_POWER: lights picked through `light_alias`
    const float4* light_alias;   // per emissive triangle: (keep probability, alias index bits, pdf, 0)
    const float4* light_rec;     // per emissive triangle: LIGHT_RECORD float4 (light_records_kernel)
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

// ACCEL: ACCEL_ANY dispatches on the scene at run time; ACCEL_FLAT_ONLY and ACCEL_TWO_LEVEL_ONLY
// compile one structure's step (the caller has checked sc.flat).
constexpr int ACCEL_ANY = 0, ACCEL_FLAT_ONLY = 1, ACCEL_TWO_LEVEL_ONLY = 2;

template <bool COUNT, int ACCEL = ACCEL_ANY, bool EARLY = false, int STACK = TRAVERSAL_STACK>
__device__ __forceinline__ bool trace_step(TraceState& st, const DevScene& sc, uint32_t* stack, int stride,
                                           uint32_t* err, Counters& cnt) {
    if (ACCEL == ACCEL_FLAT_ONLY || (ACCEL == ACCEL_ANY && sc.flat))
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
template <bool COUNT>
__device__ __forceinline__ Hit trace_closest(const DevScene& sc, f3 o, f3 d, float tmin, float tmax, bool cull,
                                             uint32_t* stack, int stride, uint32_t* err, Counters& cnt) {
    TraceState st;
    trace_init(st, sc, o, d, tmin, tmax, cull);
    while (!trace_step<COUNT>(st, sc, stack, stride, err, cnt)) {
    }
    return st.best;
}

}  // namespace tt
