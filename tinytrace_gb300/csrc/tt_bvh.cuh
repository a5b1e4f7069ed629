// Two-level BVH4 traversal on sm_103a: the replacement for the RT-core ray queries of the
// reference (GL_EXT_ray_query in src/integrate/integrate.glsl:112-127 and 168-185).
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
//   * node boxes are quantised to 8 bits per axis relative to the node box and tested
//     conservatively (slab bounds widened by 2^-20 of their magnitudes).
//
// Layout in HBM: BVH4 nodes are 64-byte records read as four 16-byte vector loads; the
// triangles of each mesh are stored in leaf order as 48-byte records (three float4), so a
// leaf is one contiguous run; per-instance traversal data is a 64-byte record (the three
// rows of the world-to-object matrix and the mesh index).  The traversal stack lives in
// shared memory, one column per thread.
#pragma once

#include "tt_common.cuh"

namespace tt {

constexpr uint32_t CHILD_LEAF = 0x80000000u;
constexpr uint32_t STACK_MARKER = 0xffffffffu;
constexpr int TRAVERSAL_STACK = 64;
constexpr uint32_t TRAVERSAL_ITERATION_LIMIT = 1u << 24;
constexpr uint32_t ERR_STACK_OVERFLOW = 1u;
constexpr uint32_t ERR_ITERATION_LIMIT = 2u;

TT_HD uint32_t leaf_first(uint32_t r) { return r & 0x07ffffffu; }
TT_HD uint32_t leaf_count(uint32_t r) { return ((r >> 27) & 0xfu) + 1u; }

struct DevScene {
    const int16_t* positions;
    const uint32_t* indices;
    const tt_vertex* vertices;
    const tt_material* materials;
    const tt_instance* instances;
    const tt_emissive_triangle* emissive;
    const uint4* blas;        // 4 x uint4 per node
    const float4* tris;       // 3 x float4 per triangle record
    const uint4* tlas;        // 4 x uint4 per node
    const float4* inst_xform; // 4 x float4 per instance: inverse rows 0..2, (mesh, material, index_offset, vertex_offset)
    uint32_t emissive_count;
    uint32_t instance_count;
    uint32_t has_tlas;
    uint32_t pad;
};

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
    int kx, ky, kz;
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
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    float dz = comp(d, kz);
    r.sx = comp(d, kx) / dz;
    r.sy = comp(d, ky) / dz;
    r.sz = 1.0f / dz;
    return r;
}

TT_HD bool intersect_triangle(const RayPre& r, f3 p0, f3 p1, f3 p2, bool cull_back, float tmin,
                              float tmax, float& t_out, float& u_out, float& v_out) {
    f3 A = p0 - r.o, B = p1 - r.o, C = p2 - r.o;
    float Akz = comp(A, r.kz), Bkz = comp(B, r.kz), Ckz = comp(C, r.kz);
    float Ax = comp(A, r.kx) - r.sx * Akz;
    float Ay = comp(A, r.ky) - r.sy * Akz;
    float Bx = comp(B, r.kx) - r.sx * Bkz;
    float By = comp(B, r.ky) - r.sy * Bkz;
    float Cx = comp(C, r.kx) - r.sx * Ckz;
    float Cy = comp(C, r.ky) - r.sy * Ckz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if (cull_back) {
        if (U < 0.0f || V < 0.0f || W < 0.0f) return false;
    } else {
        if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    }
    float det = U + V + W;
    if (det == 0.0f) return false;
    float T = U * (r.sz * Akz) + V * (r.sz * Bkz) + W * (r.sz * Ckz);
    float rcp = 1.0f / det;
    float t = T * rcp;
    if (!(t >= tmin && t <= tmax)) return false;
    t_out = t;
    u_out = V * rcp;
    v_out = W * rcp;
    return true;
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

struct NodeRay {
    f3 o, inv;
};

struct NodeData {
    uint4 q0, q1, q2, q3;
};
TT_HD NodeData load_node(const uint4* nodes, uint32_t i) {
    const uint4* p = nodes + 4ull * i;
    NodeData n;
    n.q0 = __ldg(p + 0);
    n.q1 = __ldg(p + 1);
    n.q2 = __ldg(p + 2);
    n.q3 = __ldg(p + 3);
    return n;
}
TT_HD uint32_t byte_of(uint32_t w, int b) { return (w >> (8 * b)) & 0xffu; }

// Conservative slab test of the (up to) four children; returns the hit mask and entry t.
TT_HD int node_hits(const NodeData& nd, const NodeRay& r, float tmin, float tbest, float* tn_out,
                    uint32_t* child) {
    float org[3] = {__uint_as_float(nd.q0.x), __uint_as_float(nd.q0.y), __uint_as_float(nd.q0.z)};
    uint32_t meta = nd.q0.w;  // exp bytes 0..2, count byte 3
    int count = (int)byte_of(meta, 3);
    const float o[3] = {r.o.x, r.o.y, r.o.z};
    const float inv[3] = {r.inv.x, r.inv.y, r.inv.z};
    float A[3], Blo[3], Bhi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float scale = __uint_as_float(byte_of(meta, a) << 23);
        A[a] = scale * inv[a];
        float B = (org[a] - o[a]) * inv[a];
        float M = __fmaf_rn(256.0f, fabsf(A[a]), fabsf(B)) * 9.5367431640625e-07f;
        float s = inv[a] >= 0.0f ? M : -M;
        Blo[a] = B - s;
        Bhi[a] = B + s;
    }
    child[0] = nd.q1.x;
    child[1] = nd.q1.y;
    child[2] = nd.q1.z;
    child[3] = nd.q1.w;
    // q2: qlo x[4], qlo y[4], qlo z[4], qhi x[4]; q3: qhi y[4], qhi z[4], pad
    uint32_t lo[3] = {nd.q2.x, nd.q2.y, nd.q2.z};
    uint32_t hi[3] = {nd.q2.w, nd.q3.x, nd.q3.y};
    int mask = 0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float tn = tmin, tf = tbest;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            float t0 = __fmaf_rn((float)byte_of(lo[a], c), A[a], Blo[a]);
            float t1 = __fmaf_rn((float)byte_of(hi[a], c), A[a], Bhi[a]);
            tn = fmx(tn, fmn(t0, t1));
            tf = fmn(tf, fmx(t0, t1));
        }
        tn_out[c] = tn;
        if (c < count && tn <= tf) mask |= 1 << c;
    }
    return mask;
}

TT_HD f3 tri_vertex(float4 v) { return f3{v.x, v.y, v.z}; }

// Closest hit through the TLAS/BLAS.  `stack` is this thread's column in shared memory
// (element k at stack[k * stride]).  `err` receives ERR_* bits on overflow/limit.
template <bool COUNT>
__device__ __forceinline__ Hit trace_closest(const DevScene& sc, f3 o, f3 d, float tmin,
                                             float tmax, bool cull, uint32_t* stack, int stride,
                                             uint32_t* err, Counters& cnt) {
    Hit best;
    best.hit = 0;
    best.t = 0.0f;
    best.u = 0.0f;
    best.v = 0.0f;
    best.instance = 0u;
    best.prim = 0u;
    if (!finite3(d) || !sc.has_tlas) return best;
    float tbest = tmax;
    NodeRay world{o, f3{safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)}};
    NodeRay obj = world;
    RayPre rp = ray_precompute(o, d);
    uint32_t inst = 0;
    bool in_blas = false;
    int sp = 0;
    uint32_t cur = 0;
    bool have = true;
    uint32_t iterations = 0;
    while (true) {
        if (++iterations > TRAVERSAL_ITERATION_LIMIT) {
            atomicOr(err, ERR_ITERATION_LIMIT);
            break;
        }
        if (!have) {
            if (sp == 0) break;
            uint32_t e = stack[(--sp) * stride];
            if (e == STACK_MARKER) {
                in_blas = false;
                continue;
            }
            cur = e;
            have = true;
        }
        if (!in_blas && (cur & CHILD_LEAF)) {
            inst = leaf_first(cur);
            const float4* x = sc.inst_xform + 4ull * inst;
            float4 r0 = __ldg(x + 0), r1 = __ldg(x + 1), r2 = __ldg(x + 2);
            uint32_t mesh = __float_as_uint(__ldg(x + 3).x);
            f3 oo = f3{r0.x * o.x + r0.y * o.y + r0.z * o.z + r0.w * 1.0f,
                       r1.x * o.x + r1.y * o.y + r1.z * o.z + r1.w * 1.0f,
                       r2.x * o.x + r2.y * o.y + r2.z * o.z + r2.w * 1.0f};
            f3 od = f3{r0.x * d.x + r0.y * d.y + r0.z * d.z, r1.x * d.x + r1.y * d.y + r1.z * d.z,
                       r2.x * d.x + r2.y * d.y + r2.z * d.z};
            if (COUNT) cnt.instances++;
            if (!finite3(od)) {
                have = false;
                continue;
            }
            if (sp >= TRAVERSAL_STACK) {
                atomicOr(err, ERR_STACK_OVERFLOW);
                break;
            }
            stack[(sp++) * stride] = STACK_MARKER;
            rp = ray_precompute(oo, od);
            obj = NodeRay{oo, f3{safe_inv(od.x), safe_inv(od.y), safe_inv(od.z)}};
            in_blas = true;
            cur = mesh;
            continue;
        }
        NodeData nd = load_node(in_blas ? sc.blas : sc.tlas, cur);
        if (COUNT) {
            if (in_blas) cnt.blas_nodes++;
            else cnt.tlas_nodes++;
        }
        float tn[4];
        uint32_t ch[4];
        int mask = node_hits(nd, in_blas ? obj : world, tmin, tbest, tn, ch);
        // triangle leaves first (in child order)
        if (in_blas) {
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                if (!((mask >> c) & 1) || !(ch[c] & CHILD_LEAF)) continue;
                uint32_t f = leaf_first(ch[c]), k = leaf_count(ch[c]);
                for (uint32_t q = f; q < f + k; ++q) {
                    const float4* tr = sc.tris + 3ull * q;
                    float4 a = __ldg(tr + 0), b = __ldg(tr + 1), cc = __ldg(tr + 2);
                    if (COUNT) cnt.triangles++;
                    float t, u, v;
                    uint32_t prim = __float_as_uint(a.w);
                    if (!intersect_triangle(rp, tri_vertex(a), tri_vertex(b), tri_vertex(cc), cull,
                                            tmin, tbest, t, u, v))
                        continue;
                    if (closer(t, inst, prim, best)) {
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
        }
        // remaining descendants: internal nodes (and instance leaves at the top level),
        // sorted by entry distance; the nearest is visited next, the others are pushed.
        float key[4];
        uint32_t val[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            bool take = ((mask >> c) & 1) && (!in_blas || !(ch[c] & CHILD_LEAF)) && tn[c] <= tbest;
            key[c] = take ? tn[c] : __int_as_float(0x7f800000);
            val[c] = take ? ch[c] : STACK_MARKER;
        }
#define TT_SWAP(i, j)                                            \
    if (key[j] < key[i]) {                                       \
        float tk = key[i]; key[i] = key[j]; key[j] = tk;         \
        uint32_t tv = val[i]; val[i] = val[j]; val[j] = tv;      \
    }
        TT_SWAP(0, 1) TT_SWAP(2, 3) TT_SWAP(0, 2) TT_SWAP(1, 3) TT_SWAP(1, 2)
#undef TT_SWAP
        have = false;
        if (val[0] != STACK_MARKER) {
            cur = val[0];
            have = true;
#pragma unroll
            for (int c = 3; c >= 1; --c) {
                if (val[c] == STACK_MARKER) continue;
                if (sp >= TRAVERSAL_STACK) {
                    atomicOr(err, ERR_STACK_OVERFLOW);
                    return best;
                }
                stack[(sp++) * stride] = val[c];
            }
        }
    }
    return best;
}

}  // namespace tt
