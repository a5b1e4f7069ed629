// TEST INFRASTRUCTURE — the CPU oracle for the tinytrace rendering hot path (the checker,
// never the product; only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg
// may load it).
//
// Ray queries without RT cores.  The reference delegates acceleration-structure build and
// traversal to the Vulkan driver (src/scene.rs:130-171, src/integrate/integrate.glsl:112-127,
// 168-185), so there is no reference source for this part: this header states the
// semantics the GPU implementation must reproduce and restates the project's LBVH build on
// the CPU so that the GPU build can be compared node for node.
//
// Ray-query semantics (the reference's GL_EXT_ray_query use):
//   * instances are intersected in object space: o' = inverse_transform * (o, 1),
//     d' = mat3(inverse_transform) * d; the ray parameter t is shared across instances;
//   * object-space vertices are the dequantised snorm16 positions, value / 32767;
//   * triangle test: watertight ray/triangle intersection (Woop, Benthin & Wald, JCGT 2013)
//     with its double-precision fallback when an edge function is exactly zero;
//     barycentrics (u, v) = (V/det, W/det) so that hit = (1-u-v) p0 + u p1 + v p2;
//   * front faces are those whose geometric normal cross(p1-p0, p2-p0) faces the ray origin
//     (det > 0); gl_RayFlagsCullBackFacingTrianglesEXT keeps only front faces;
//   * a hit counts when tmin <= t <= tmax; the closest hit is the smallest t, ties broken by
//     the smaller (instance, primitive) pair, so the result does not depend on traversal order.
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

#include "ref_scene.h"

namespace ref {

struct Aabb {
    v3 lo, hi;
};
inline Aabb aabb_empty() {
    return Aabb{splat3(INFINITY), splat3(-INFINITY)};
}
inline Aabb aabb_union(const Aabb& a, const Aabb& b) {
    return Aabb{v3{fmn(a.lo.x, b.lo.x), fmn(a.lo.y, b.lo.y), fmn(a.lo.z, b.lo.z)},
                v3{fmx(a.hi.x, b.hi.x), fmx(a.hi.y, b.hi.y), fmx(a.hi.z, b.hi.z)}};
}
inline Aabb aabb_point(Aabb a, v3 p) { return aabb_union(a, Aabb{p, p}); }
// Box coordinates and centroids are canonicalised (-0 -> +0) so that min/max are unambiguous.
inline float canon(float v) { return v + 0.0f; }
inline v3 canon3(v3 v) { return v3{canon(v.x), canon(v.y), canon(v.z)}; }
inline Aabb canon_box(Aabb b) { return Aabb{canon3(b.lo), canon3(b.hi)}; }
// Half surface area: ex*ey + ey*ez + ez*ex.
inline float aabb_half_area(const Aabb& a) {
    v3 e = a.hi - a.lo;
    return e.x * e.y + e.y * e.z + e.z * e.x;
}

// ---------------------------------------------------------------- BVH4 node (128 bytes)
// Child boxes as float planes: box[2a][c] = low bound of child c on axis a, box[2a+1][c] the
// high bound (empty slots: +inf / -inf); then the four child references and the child count.
struct Node4 {
    float box[6][4];
    uint32_t child[4];
    uint32_t count;
    uint32_t pad[3];
};
static_assert(sizeof(Node4) == 128, "Node4 is 128 bytes");
constexpr uint32_t CHILD_LEAF = 0x80000000u;
inline uint32_t leaf_ref(uint32_t first, uint32_t count) {
    return CHILD_LEAF | ((count - 1u) << 27) | first;
}
inline uint32_t leaf_first(uint32_t ref) { return ref & 0x07ffffffu; }
inline uint32_t leaf_count(uint32_t ref) { return ((ref >> 27) & 0xfu) + 1u; }

// BLAS triangle record (48 bytes): v0.xyz + primitive index bits, v1.xyz, v2.xyz.
struct TriRecord {
    float v0[3];
    uint32_t prim;
    float v1[3];
    uint32_t mesh;
    float v2[3];
    uint32_t pad;
};
static_assert(sizeof(TriRecord) == 48, "TriRecord is 48 bytes");

// ---------------------------------------------------------------- LBVH build
inline uint32_t expand_bits10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
inline uint32_t quantize_axis(float c, float lo, float hi) {
    float ext = hi - lo;
    if (!(ext > 0.0f)) return 0u;
    float f = (c - lo) / ext;
    float s = fmn(fmx(f * 1024.0f, 0.0f), 1023.0f);
    return (uint32_t)s;
}
inline uint32_t morton30(v3 c, v3 lo, v3 hi) {
    uint32_t x = quantize_axis(c.x, lo.x, hi.x);
    uint32_t y = quantize_axis(c.y, lo.y, hi.y);
    uint32_t z = quantize_axis(c.z, lo.z, hi.z);
    return (expand_bits10(x) << 2) | (expand_bits10(y) << 1) | expand_bits10(z);
}
inline int clz64(uint64_t v) { return v == 0 ? 64 : __builtin_clzll(v); }
inline int clz32(uint32_t v) { return v == 0 ? 32 : __builtin_clz(v); }

struct BinaryTree {
    // internal nodes [0, n-1), leaves referenced as n-1 + leaf index in `left/right`.
    int n = 0;
    std::vector<int> left, right, first, last;  // per internal node
    std::vector<Aabb> ibox;                     // per internal node
    std::vector<Aabb> lbox;                     // per leaf (sorted order)
};

struct BvhBuild {
    std::vector<Node4> nodes;
    std::vector<uint32_t> order;  // sorted position -> primitive index
    std::vector<uint32_t> segment_root_kind;  // 0 empty, 1 ok
    int levels = 0;
};

// Karras (2012) common-prefix function with the index tie-break for duplicate keys.
inline int karras_delta(const std::vector<uint64_t>& k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    if (k[i] != k[j]) return clz64(k[i] ^ k[j]);
    return 64 + clz32((uint32_t)i ^ (uint32_t)j);
}

// Child boxes of a node (empty slots get +inf / -inf so that no ray enters them).
inline void fill_node(Node4& nd, const Aabb* cbox, int count) {
    for (int c = 0; c < 4; ++c) {
        const float* lo = &cbox[c].lo.x;
        const float* hi = &cbox[c].hi.x;
        for (int a = 0; a < 3; ++a) {
            nd.box[2 * a][c] = c < count ? lo[a] : INFINITY;
            nd.box[2 * a + 1][c] = c < count ? hi[a] : -INFINITY;
        }
    }
    nd.count = (uint32_t)count;
}

// Binary LBVH over primitives grouped in segments: Morton keys of the centroids normalised per
// segment, stable sort, Karras hierarchy, exact bottom-up boxes; `roots` holds each segment's
// root as a binary node reference (internal r < n - 1, leaf n - 1 + sorted position, -1 empty).
struct BinaryBuild {
    BinaryTree t;
    std::vector<uint32_t> order;  // sorted position -> primitive index
    std::vector<int> roots;
    int ni = 0;
    bool is_leaf(int r) const { return r >= ni; }
    int nfirst(int r) const { return is_leaf(r) ? r - ni : t.first[r]; }
    int ncount(int r) const { return is_leaf(r) ? 1 : t.last[r] - t.first[r] + 1; }
    const Aabb& nbox(int r) const { return is_leaf(r) ? t.lbox[r - ni] : t.ibox[r]; }
};

inline BinaryBuild build_binary(const std::vector<Aabb>& prim_box, const std::vector<uint32_t>& segment,
                                uint32_t segment_count) {
    BinaryBuild out;
    const int n = (int)prim_box.size();
    // 1. centroid bounds per segment
    std::vector<Aabb> cb(segment_count, aabb_empty());
    std::vector<v3> cent(n);
    for (int i = 0; i < n; ++i) {
        cent[i] = canon3((prim_box[i].lo + prim_box[i].hi) * 0.5f);
        cb[segment[i]] = aabb_point(cb[segment[i]], cent[i]);
    }
    // 2. keys, 3. stable sort
    std::vector<uint64_t> key(n);
    for (int i = 0; i < n; ++i) {
        const Aabb& b = cb[segment[i]];
        key[i] = ((uint64_t)segment[i] << 30) | morton30(cent[i], b.lo, b.hi);
    }
    std::vector<uint32_t> order(n);
    for (int i = 0; i < n; ++i) order[i] = (uint32_t)i;
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t a, uint32_t b) { return key[a] < key[b]; });
    std::vector<uint64_t> sk(n);
    for (int i = 0; i < n; ++i) sk[i] = key[order[i]];
    // 4. Karras hierarchy
    BinaryTree& t = out.t;
    t.n = n;
    int ni = n > 1 ? n - 1 : 0;
    out.ni = ni;
    t.left.assign(ni, 0);
    t.right.assign(ni, 0);
    t.first.assign(ni, 0);
    t.last.assign(ni, 0);
    for (int i = 0; i < ni; ++i) {
        int d = (karras_delta(sk, n, i, i + 1) - karras_delta(sk, n, i, i - 1)) >= 0 ? 1 : -1;
        int dmin = karras_delta(sk, n, i, i - d);
        int lmax = 2;
        while (karras_delta(sk, n, i, i + lmax * d) > dmin) lmax *= 2;
        int l = 0;
        for (int tt = lmax / 2; tt >= 1; tt /= 2)
            if (karras_delta(sk, n, i, i + (l + tt) * d) > dmin) l += tt;
        int j = i + l * d;
        int dnode = karras_delta(sk, n, i, j);
        int s = 0;
        for (int div = 2;; div *= 2) {
            int tt = (l + div - 1) / div;
            if (karras_delta(sk, n, i, i + (s + tt) * d) > dnode) s += tt;
            if (tt == 1) break;
        }
        int gamma = i + s * d + std::min(d, 0);
        int lo = std::min(i, j), hi = std::max(i, j);
        t.left[i] = (lo == gamma) ? (ni + gamma) : gamma;
        t.right[i] = (hi == gamma + 1) ? (ni + gamma + 1) : (gamma + 1);
        t.first[i] = lo;
        t.last[i] = hi;
    }
    // 5. boxes (bottom-up; exact min/max, so any order gives the same result)
    t.lbox.resize(n);
    for (int i = 0; i < n; ++i) t.lbox[i] = prim_box[order[i]];
    t.ibox.assign(ni, aabb_empty());
    std::vector<char> done(ni, 0);
    // iterative post-order
    {
        std::vector<int> st;
        if (ni > 0) st.push_back(0);
        while (!st.empty()) {
            int v = st.back();
            int l = t.left[v], r = t.right[v];
            bool ready = true;
            if (l < ni && !done[l]) { st.push_back(l); ready = false; }
            if (r < ni && !done[r]) { st.push_back(r); ready = false; }
            if (!ready) continue;
            st.pop_back();
            Aabb bl = l < ni ? t.ibox[l] : t.lbox[l - ni];
            Aabb br = r < ni ? t.ibox[r] : t.lbox[r - ni];
            t.ibox[v] = aabb_union(bl, br);
            done[v] = 1;
        }
    }
    // 6. segment roots: the node whose range equals the segment's sorted range
    std::vector<int> seg_first(segment_count, 0), seg_count(segment_count, 0);
    for (int i = 0; i < n; ++i) seg_count[segment[i]]++;
    for (uint32_t s = 1; s < segment_count; ++s) seg_first[s] = seg_first[s - 1] + seg_count[s - 1];
    for (uint32_t s = 0; s < segment_count; ++s) {
        int a = seg_first[s], b = a + seg_count[s] - 1;
        if (seg_count[s] == 0) out.roots.push_back(-1);
        else if (seg_count[s] == 1) out.roots.push_back(ni + a);
        else if (t.first[a] == a && t.last[a] == b) out.roots.push_back(a);
        else out.roots.push_back(b);
    }
    out.order = std::move(order);
    return out;
}

// Build BVH4s over primitives grouped in segments (one BVH root per segment, node index =
// segment index).  `segment` must be non-decreasing in primitive order.  `leaf_max` bounds
// the primitives per leaf child; `leaf_by_prim` stores the primitive index instead of the
// sorted position in leaf references (used for the instance level, where leaf_max == 1).
inline BvhBuild build_bvh4(const std::vector<Aabb>& prim_box, const std::vector<uint32_t>& segment,
                           uint32_t segment_count, int leaf_max, bool leaf_by_prim) {
    BvhBuild out;
    BinaryBuild bb = build_binary(prim_box, segment, segment_count);
    const BinaryTree& t = bb.t;
    const std::vector<uint32_t>& order = bb.order;
    auto is_leaf = [&](int r) { return bb.is_leaf(r); };
    auto nfirst = [&](int r) { return bb.nfirst(r); };
    auto ncount = [&](int r) { return bb.ncount(r); };
    auto nbox = [&](int r) { return bb.nbox(r); };
    std::vector<int> level = bb.roots;  // binary node refs of the current BVH4 level (-1 = empty)
    // 7. collapse to BVH4, level by level
    while (!level.empty()) {
        out.levels++;
        std::vector<int> next;
        size_t base = out.nodes.size();
        size_t next_base = base + level.size();
        out.nodes.resize(base + level.size());
        for (size_t li = 0; li < level.size(); ++li) {
            Node4& nd = out.nodes[base + li];
            std::memset(&nd, 0, sizeof(nd));
            int r = level[li];
            int ch[4];
            int cnt = 0;
            if (r < 0) {
                cnt = 0;
            } else if (is_leaf(r) || ncount(r) <= leaf_max) {
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
                        if (is_leaf(ch[c]) || ncount(ch[c]) <= leaf_max) continue;
                        float a = aabb_half_area(nbox(ch[c]));
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
            Aabb cbx[4];
            for (int c = 0; c < cnt; ++c) {
                int v = ch[c];
                cbx[c] = nbox(v);
                if (is_leaf(v) || ncount(v) <= leaf_max) {
                    uint32_t f = (uint32_t)nfirst(v);
                    uint32_t k = (uint32_t)ncount(v);
                    nd.child[c] = leaf_by_prim ? leaf_ref(order[f], 1u) : leaf_ref(f, k);
                } else {
                    nd.child[c] = (uint32_t)(next_base + next.size());
                    next.push_back(v);
                }
            }
            for (int c = cnt; c < 4; ++c) nd.child[c] = 0xffffffffu;
            fill_node(nd, cbx, cnt);
        }
        level.swap(next);
    }
    out.order = order;
    return out;
}

// ---------------------------------------------------------------- compressed 8-wide node (80 bytes)
// A node of the flat structure's wide format (after the compressed wide BVHs of Ylitie, Karras &
// Laine, HPG 2017): up to eight children whose boxes are quantised to 8 bits per plane relative
// to the node's origin (its box's low corner) with one power-of-two scale per axis,
//   plane = origin[a] + q * 2^(exponent[a] - 127),  q in 0..255,
// rounded outwards (low planes down, high planes up), so that a decoded child box contains the
// child's exact box.  Internal children are stored contiguously from `child_base` in slot order
// (child of slot s: child_base + number of internal slots below s); the triangle records of the
// leaf children are stored contiguously from `tri_base`, each leaf slot naming its first record
// (meta bits 0..4, offset from tri_base) and its 1..3 records as a unary count (meta bits 5..7).
// Children occupy slots by direction: slot s preferably holds the child lying farthest towards
// the octant whose axis a is negative when bit a of s is set, so a ray whose direction has sign
// bits o reaches the children roughly nearest first when it visits slots o ^ 0, o ^ 1, ... o ^ 7.
struct Node8 {
    float origin[3];
    uint8_t exponent[3];  // biased exponents of the per-axis scales
    uint8_t imask;        // bit s: slot s holds an internal child
    uint32_t child_base;
    uint32_t tri_base;
    uint8_t meta[8];
    uint8_t qlo_x[8], qhi_x[8], qlo_y[8], qhi_y[8], qlo_z[8], qhi_z[8];
};
static_assert(sizeof(Node8) == 80, "Node8 is 80 bytes");
constexpr int WIDE_LEAF_MAX = 3;  // records per leaf child

// Biased exponent e (scale 2^(e - 127), e in 1..254) of the smallest power-of-two scale whose 255
// steps cover `extent`.
inline uint8_t wide_exponent(float extent) {
    float x = extent / 255.0f;
    uint32_t bits = fbits(x);
    uint32_t e = (bits >> 23) & 0xffu;
    if (e == 0u) e = 1u;                               // zero or subnormal: the smallest normal scale
    else if ((bits & 0x7fffffu) != 0u) e += 1u;        // round x up to a power of two
    while (e < 254u && 255.0f * bitsf(e << 23) < extent) e += 1u;
    return (uint8_t)(e > 254u ? 254u : e);
}
inline uint8_t wide_quantize_lo(float v, float origin, float scale) {
    float q = std::floor((v - origin) / scale);
    return (uint8_t)(q < 0.0f ? 0.0f : (q > 255.0f ? 255.0f : q));
}
inline uint8_t wide_quantize_hi(float v, float origin, float scale) {
    float q = std::ceil((v - origin) / scale);
    return (uint8_t)(q < 0.0f ? 0.0f : (q > 255.0f ? 255.0f : q));
}

// Slot assignment of `cnt` children with centroids `cc` in a node with centroid `pc`: the cost of
// child c in slot s is the distance of its centroid along the octant direction of s
// ((-1)^(bit a of s) per axis); pairs are taken greedily, cheapest first (ties: lower slot, then
// lower child).  slot_of[c] receives the slot of child c.
inline void wide_assign_slots(const v3* cc, v3 pc, int cnt, int* slot_of) {
    float cost[8][8];
    for (int c = 0; c < cnt; ++c) {
        v3 d = cc[c] - pc;
        for (int s = 0; s < 8; ++s) {
            float sx = (s & 1) ? -d.x : d.x, sy = (s & 2) ? -d.y : d.y, sz = (s & 4) ? -d.z : d.z;
            cost[c][s] = (sx + sy) + sz;
        }
    }
    bool child_done[8] = {}, slot_used[8] = {};
    for (int k = 0; k < cnt; ++k) {
        int bc = -1, bs = -1;
        float best = 0.0f;
        for (int s = 0; s < 8; ++s) {
            if (slot_used[s]) continue;
            for (int c = 0; c < cnt; ++c) {
                if (child_done[c]) continue;
                if (bc < 0 || cost[c][s] < best) {
                    bc = c;
                    bs = s;
                    best = cost[c][s];
                }
            }
        }
        child_done[bc] = true;
        slot_used[bs] = true;
        slot_of[bc] = bs;
    }
}

struct WideBuild {
    std::vector<Node8> nodes;
    std::vector<uint32_t> tri_order;  // wide record position -> sorted position of the binary build
    int levels = 0;
};

// The wide format over the binary LBVH of one segment, level by level from the root: each node
// expands the largest-area internal child of its current children until it holds eight (subtrees
// of at most WIDE_LEAF_MAX primitives are leaf children), assigns the children to slots, and
// quantises their boxes; the next level lists the internal children of this level's nodes in
// node order, each node's in slot order.
inline WideBuild collapse_wide(const BinaryBuild& bb) {
    WideBuild out;
    std::vector<int> level = bb.roots;
    uint32_t tri_next = 0;
    auto leafish = [&](int r) { return bb.is_leaf(r) || bb.ncount(r) <= WIDE_LEAF_MAX; };
    while (!level.empty()) {
        out.levels++;
        size_t base = out.nodes.size();
        size_t next_base = base + level.size();
        std::vector<int> next;
        out.nodes.resize(base + level.size());
        for (size_t li = 0; li < level.size(); ++li) {
            Node8& nd = out.nodes[base + li];
            std::memset(&nd, 0, sizeof(nd));
            int r = level[li];
            int ch[8];
            int cnt = 0;
            if (r < 0) {
                cnt = 0;
            } else if (leafish(r)) {
                ch[0] = r;
                cnt = 1;
            } else {
                ch[0] = bb.t.left[r];
                ch[1] = bb.t.right[r];
                cnt = 2;
                while (cnt < 8) {
                    int best = -1;
                    float best_area = -1.0f;
                    for (int c = 0; c < cnt; ++c) {
                        if (leafish(ch[c])) continue;
                        float a = aabb_half_area(bb.nbox(ch[c]));
                        if (best < 0 || a > best_area) {
                            best = c;
                            best_area = a;
                        }
                    }
                    if (best < 0) break;
                    int v = ch[best];
                    for (int c = cnt; c > best + 1; --c) ch[c] = ch[c - 1];
                    ch[best] = bb.t.left[v];
                    ch[best + 1] = bb.t.right[v];
                    cnt++;
                }
            }
            // node box, centroids, slots
            Aabb box = aabb_empty();
            v3 cc[8];
            for (int c = 0; c < cnt; ++c) {
                const Aabb& b = bb.nbox(ch[c]);
                box = aabb_union(box, b);
                cc[c] = (b.lo + b.hi) * 0.5f;
            }
            int slot_of[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            int child_at[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
            if (cnt > 0) {
                wide_assign_slots(cc, (box.lo + box.hi) * 0.5f, cnt, slot_of);
                for (int c = 0; c < cnt; ++c) child_at[slot_of[c]] = ch[c];
            }
            const float* lo = &box.lo.x;
            const float* hi = &box.hi.x;
            float scale[3];
            for (int a = 0; a < 3; ++a) {
                nd.origin[a] = cnt > 0 ? lo[a] : 0.0f;
                nd.exponent[a] = cnt > 0 ? wide_exponent(hi[a] - lo[a]) : (uint8_t)127;
                scale[a] = bitsf((uint32_t)nd.exponent[a] << 23);
            }
            nd.child_base = (uint32_t)(next_base + next.size());
            nd.tri_base = tri_next;
            uint32_t tri_off = 0;
            for (int s = 0; s < 8; ++s) {
                int v = child_at[s];
                if (v < 0) {  // empty slot: an inverted box (never entered), meta 0
                    nd.qlo_x[s] = nd.qlo_y[s] = nd.qlo_z[s] = 255;
                    nd.qhi_x[s] = nd.qhi_y[s] = nd.qhi_z[s] = 0;
                    continue;
                }
                const Aabb& b = bb.nbox(v);
                nd.qlo_x[s] = wide_quantize_lo(b.lo.x, nd.origin[0], scale[0]);
                nd.qhi_x[s] = wide_quantize_hi(b.hi.x, nd.origin[0], scale[0]);
                nd.qlo_y[s] = wide_quantize_lo(b.lo.y, nd.origin[1], scale[1]);
                nd.qhi_y[s] = wide_quantize_hi(b.hi.y, nd.origin[1], scale[1]);
                nd.qlo_z[s] = wide_quantize_lo(b.lo.z, nd.origin[2], scale[2]);
                nd.qhi_z[s] = wide_quantize_hi(b.hi.z, nd.origin[2], scale[2]);
                if (leafish(v)) {
                    uint32_t k = (uint32_t)bb.ncount(v), f = (uint32_t)bb.nfirst(v);
                    nd.meta[s] = (uint8_t)(tri_off | (((1u << k) - 1u) << 5));
                    for (uint32_t j = 0; j < k; ++j) out.tri_order.push_back(f + j);
                    tri_off += k;
                } else {
                    nd.imask |= (uint8_t)(1u << s);
                    next.push_back(v);
                }
            }
            tri_next += tri_off;
        }
        level.swap(next);
    }
    return out;
}

// ---------------------------------------------------------------- ray queries
struct Hit {
    int hit;
    float t, u, v;
    uint32_t instance, prim;
};

struct RayPre {
    v3 o, d;
    int kx, ky, kz;
    float sx, sy, sz;
};
inline float comp(v3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
inline RayPre ray_precompute(v3 o, v3 d) {
    RayPre r;
    r.o = o;
    r.d = d;
    int kz = 0;
    if (std::fabs(d.y) > std::fabs(d.x)) kz = 1;
    if (std::fabs(d.z) > std::fabs(comp(d, kz))) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (comp(d, kz) < 0.0f) std::swap(kx, ky);
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.sx = comp(d, kx) / comp(d, kz);
    r.sy = comp(d, ky) / comp(d, kz);
    r.sz = 1.0f / comp(d, kz);
    return r;
}
// Watertight ray/triangle test. Returns true and (t, u, v) on a hit within [tmin, tmax].
inline bool intersect_triangle(const RayPre& r, v3 p0, v3 p1, v3 p2, bool cull_back, float tmin,
                               float tmax, float& t_out, float& u_out, float& v_out) {
    v3 A = p0 - r.o, B = p1 - r.o, C = p2 - r.o;
    float Ax = comp(A, r.kx) - r.sx * comp(A, r.kz);
    float Ay = comp(A, r.ky) - r.sy * comp(A, r.kz);
    float Bx = comp(B, r.kx) - r.sx * comp(B, r.kz);
    float By = comp(B, r.ky) - r.sy * comp(B, r.kz);
    float Cx = comp(C, r.kx) - r.sx * comp(C, r.kz);
    float Cy = comp(C, r.ky) - r.sy * comp(C, r.kz);
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
    float Az = r.sz * comp(A, r.kz);
    float Bz = r.sz * comp(B, r.kz);
    float Cz = r.sz * comp(C, r.kz);
    float T = U * Az + V * Bz + W * Cz;
    float rcp = 1.0f / det;
    float t = T * rcp;
    if (!(t >= tmin && t <= tmax)) return false;
    t_out = t;
    u_out = V * rcp;
    v_out = W * rcp;
    return true;
}
inline bool closer(float t, uint32_t inst, uint32_t prim, const Hit& best) {
    if (!best.hit) return true;
    if (t < best.t) return true;
    if (t > best.t) return false;
    if (inst != best.instance) return inst < best.instance;
    return prim < best.prim;
}
inline bool finite3(v3 d) { return std::isfinite(d.x) && std::isfinite(d.y) && std::isfinite(d.z); }

// Scene geometry as seen by the ray queries.
struct Geometry {
    const int16_t* positions;
    const uint32_t* indices;
    const Instance* instances;
    uint32_t instance_count;
    const Mesh* meshes;
    uint32_t mesh_count;
};
inline void triangle_object(const Geometry& g, const Instance& in, uint32_t prim, v3& p0, v3& p1,
                            v3& p2) {
    uint32_t base = in.index_offset + 3u * prim;
    p0 = dequantize_snorm3(g.positions + 3u * (in.vertex_offset + g.indices[base + 0]));
    p1 = dequantize_snorm3(g.positions + 3u * (in.vertex_offset + g.indices[base + 1]));
    p2 = dequantize_snorm3(g.positions + 3u * (in.vertex_offset + g.indices[base + 2]));
}
inline void object_ray(const Instance& in, v3 o, v3 d, v3& oo, v3& od) {
    oo = mat43_point(in.inverse_transform, o);
    od = mat3_vec(in.inverse_transform, d);
}

// Brute force closest hit over every triangle of every instance.
inline Hit trace_brute(const Geometry& g, v3 o, v3 d, float tmin, float tmax, bool cull_back) {
    Hit best{0, 0.0f, 0.0f, 0.0f, 0u, 0u};
    if (!finite3(d)) return best;
    for (uint32_t i = 0; i < g.instance_count; ++i) {
        const Instance& in = g.instances[i];
        const Mesh& m = g.meshes[in.mesh_index];
        v3 oo, od;
        object_ray(in, o, d, oo, od);
        RayPre r = ray_precompute(oo, od);
        uint32_t tris = m.index_count / 3u;
        for (uint32_t p = 0; p < tris; ++p) {
            v3 p0, p1, p2;
            triangle_object(g, in, p, p0, p1, p2);
            float t, u, v;
            if (!intersect_triangle(r, p0, p1, p2, cull_back, tmin, tmax, t, u, v)) continue;
            if (closer(t, i, p, best)) best = Hit{1, t, u, v, i, p};
        }
    }
    return best;
}

// Conservative slab test of one node against a ray.  Per axis, the near plane is the low
// bound when the inverse direction is non-negative and the high bound otherwise; entry and exit
// distances are widened by E = 2^-20 (B + |o|) |1/d|, where B bounds the box coordinates, which
// exceeds the rounding error of fma(plane, 1/d, -o/d), so float rounding never culls a box the
// ray enters.
struct NodeRay {
    v3 o, inv;
    float nob_near[3], nob_far[3];
    int near[3];
};
inline float safe_inv(float d) {
    float a = std::fabs(d) < 1e-20f ? (d < 0.0f ? -1e-20f : 1e-20f) : d;
    return 1.0f / a;
}
inline NodeRay node_ray(v3 o, v3 d, float bound) {
    NodeRay r;
    r.o = o;
    r.inv = v3{safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
    const float oa[3] = {o.x, o.y, o.z}, ia[3] = {r.inv.x, r.inv.y, r.inv.z};
    for (int a = 0; a < 3; ++a) {
        float nob = -(oa[a] * ia[a]);
        float E = (bound + std::fabs(oa[a])) * std::fabs(ia[a]) * 9.5367431640625e-07f;
        r.nob_near[a] = nob - E;
        r.nob_far[a] = nob + E;
        r.near[a] = ia[a] >= 0.0f ? 0 : 1;
    }
    return r;
}
inline int node_hits(const Node4& nd, const NodeRay& r, float tmin, float tbest, float* tnear) {
    const float ia[3] = {r.inv.x, r.inv.y, r.inv.z};
    int mask = 0;
    for (int c = 0; c < 4; ++c) {
        float tn = tmin, tf = tbest;
        for (int a = 0; a < 3; ++a) {
            float t0 = std::fmaf(nd.box[2 * a + r.near[a]][c], ia[a], r.nob_near[a]);
            float t1 = std::fmaf(nd.box[2 * a + 1 - r.near[a]][c], ia[a], r.nob_far[a]);
            tn = fmx(tn, t0);
            tf = fmn(tf, t1);
        }
        if (c < (int)nd.count && tn <= tf) {
            mask |= 1 << c;
            tnear[c] = tn;
        }
    }
    return mask;
}

struct SceneBvh {
    std::vector<Node4> blas;   // node index == mesh index for BLAS roots
    std::vector<TriRecord> tris;
    std::vector<Node4> tlas;   // root = 0
    int blas_levels = 0, tlas_levels = 0;
    float tlas_bound = 0.0f;   // max |coordinate| of the instance world boxes
    // single-level ("flat") BVH over the world boxes of every (instance, triangle) pair;
    // its triangle records keep object-space vertices and hold the instance in `mesh`
    std::vector<Node4> flat;
    std::vector<TriRecord> flat_tris;
    int flat_levels = 0;
    float flat_bound = 0.0f;   // max |coordinate| of the triangle world boxes
    // the same structure in the compressed 8-wide format (build_wide_bvh)
    std::vector<Node8> wide;
    std::vector<TriRecord> wide_tris;
    int wide_levels = 0;
};

// The flat BVH: primitives are the (instance, triangle) pairs in instance order; a primitive's
// box is the box of its three vertices transformed to world space.
inline void build_flat_bvh(const Geometry& g, int leaf_max, SceneBvh& s) {
    std::vector<Aabb> boxes;
    std::vector<uint32_t> seg;
    std::vector<TriRecord> recs;
    for (uint32_t i = 0; i < g.instance_count; ++i) {
        const Instance& in = g.instances[i];
        const Mesh& me = g.meshes[in.mesh_index];
        uint32_t tris = me.index_count / 3u;
        for (uint32_t p = 0; p < tris; ++p) {
            v3 q[3];
            triangle_object(g, in, p, q[0], q[1], q[2]);
            v3 w0 = mat43_point(in.transform, q[0]), w1 = mat43_point(in.transform, q[1]),
               w2 = mat43_point(in.transform, q[2]);
            Aabb b = canon_box(aabb_point(aabb_point(Aabb{w0, w0}, w1), w2));
            boxes.push_back(b);
            seg.push_back(0);
            const float* lo = &b.lo.x;
            const float* hi = &b.hi.x;
            for (int a = 0; a < 3; ++a) s.flat_bound = fmx(s.flat_bound, fmx(std::fabs(lo[a]), std::fabs(hi[a])));
            TriRecord tr;
            tr.v0[0] = q[0].x; tr.v0[1] = q[0].y; tr.v0[2] = q[0].z;
            tr.v1[0] = q[1].x; tr.v1[1] = q[1].y; tr.v1[2] = q[1].z;
            tr.v2[0] = q[2].x; tr.v2[1] = q[2].y; tr.v2[2] = q[2].z;
            tr.prim = p;
            tr.mesh = i;
            tr.pad = 0;
            recs.push_back(tr);
        }
    }
    BvhBuild b = build_bvh4(boxes, seg, 1, leaf_max, false);
    s.flat = b.nodes;
    s.flat_levels = b.levels;
    s.flat_tris.resize(recs.size());
    for (size_t k = 0; k < recs.size(); ++k) s.flat_tris[k] = recs[b.order[k]];
}

// The flat structure in the compressed 8-wide format: the same primitives, boxes, records and
// binary LBVH as build_flat_bvh, collapsed by collapse_wide; records in the wide order.
inline void build_wide_bvh(const Geometry& g, SceneBvh& s) {
    std::vector<Aabb> boxes;
    std::vector<TriRecord> recs;
    for (uint32_t i = 0; i < g.instance_count; ++i) {
        const Instance& in = g.instances[i];
        const Mesh& me = g.meshes[in.mesh_index];
        uint32_t tris = me.index_count / 3u;
        for (uint32_t p = 0; p < tris; ++p) {
            v3 q[3];
            triangle_object(g, in, p, q[0], q[1], q[2]);
            v3 w0 = mat43_point(in.transform, q[0]), w1 = mat43_point(in.transform, q[1]),
               w2 = mat43_point(in.transform, q[2]);
            boxes.push_back(canon_box(aabb_point(aabb_point(Aabb{w0, w0}, w1), w2)));
            TriRecord tr;
            tr.v0[0] = q[0].x; tr.v0[1] = q[0].y; tr.v0[2] = q[0].z;
            tr.v1[0] = q[1].x; tr.v1[1] = q[1].y; tr.v1[2] = q[1].z;
            tr.v2[0] = q[2].x; tr.v2[1] = q[2].y; tr.v2[2] = q[2].z;
            tr.prim = p;
            tr.mesh = i;
            tr.pad = 0;
            recs.push_back(tr);
        }
    }
    s.wide.clear();
    s.wide_tris.clear();
    s.wide_levels = 0;
    if (boxes.empty()) return;
    std::vector<uint32_t> seg(boxes.size(), 0u);
    BinaryBuild bb = build_binary(boxes, seg, 1);
    WideBuild w = collapse_wide(bb);
    s.wide = std::move(w.nodes);
    s.wide_levels = w.levels;
    s.wide_tris.resize(w.tri_order.size());
    for (size_t k = 0; k < w.tri_order.size(); ++k) s.wide_tris[k] = recs[bb.order[w.tri_order[k]]];
}

// BLAS over all meshes (segment = mesh) and TLAS over instances (leaf = instance index).
inline SceneBvh build_scene_bvh(const Geometry& g, int leaf_max) {
    SceneBvh s;
    std::vector<Aabb> pbox;
    std::vector<uint32_t> seg;
    std::vector<TriRecord> recs;
    for (uint32_t m = 0; m < g.mesh_count; ++m) {
        const Mesh& me = g.meshes[m];
        uint32_t tris = me.index_count / 3u;
        for (uint32_t p = 0; p < tris; ++p) {
            uint32_t base = me.index_offset + 3u * p;
            v3 q[3];
            for (int k = 0; k < 3; ++k)
                q[k] = dequantize_snorm3(g.positions + 3u * (me.vertex_offset + g.indices[base + k]));
            Aabb b = aabb_point(aabb_point(Aabb{q[0], q[0]}, q[1]), q[2]);
            pbox.push_back(canon_box(b));
            seg.push_back(m);
            TriRecord tr;
            tr.v0[0] = q[0].x; tr.v0[1] = q[0].y; tr.v0[2] = q[0].z;
            tr.v1[0] = q[1].x; tr.v1[1] = q[1].y; tr.v1[2] = q[1].z;
            tr.v2[0] = q[2].x; tr.v2[1] = q[2].y; tr.v2[2] = q[2].z;
            tr.prim = p;
            tr.mesh = m;
            tr.pad = 0;
            recs.push_back(tr);
        }
    }
    BvhBuild b = build_bvh4(pbox, seg, g.mesh_count, leaf_max, false);
    s.blas = b.nodes;
    s.blas_levels = b.levels;
    s.tris.resize(recs.size());
    for (size_t i = 0; i < recs.size(); ++i) s.tris[i] = recs[b.order[i]];
    // instance level: world box = box of the 8 transformed corners of the mesh box
    std::vector<Aabb> mesh_box(g.mesh_count, aabb_empty());
    for (size_t i = 0; i < pbox.size(); ++i) mesh_box[seg[i]] = aabb_union(mesh_box[seg[i]], pbox[i]);
    std::vector<Aabb> ibox;
    std::vector<uint32_t> iseg;
    std::vector<uint32_t> ids;
    for (uint32_t i = 0; i < g.instance_count; ++i) {
        const Instance& in = g.instances[i];
        const Mesh& me = g.meshes[in.mesh_index];
        if (me.index_count / 3u == 0) continue;
        const Aabb& mb = mesh_box[in.mesh_index];
        Aabb wb = aabb_empty();
        for (int k = 0; k < 8; ++k) {
            v3 c = v3{(k & 1) ? mb.hi.x : mb.lo.x, (k & 2) ? mb.hi.y : mb.lo.y,
                      (k & 4) ? mb.hi.z : mb.lo.z};
            wb = aabb_point(wb, mat43_point(in.transform, c));
        }
        ibox.push_back(canon_box(wb));
        iseg.push_back(0);
        ids.push_back(i);
    }
    for (const Aabb& b : ibox) {
        const float* lo = &b.lo.x;
        const float* hi = &b.hi.x;
        for (int a = 0; a < 3; ++a) s.tlas_bound = fmx(s.tlas_bound, fmx(std::fabs(lo[a]), std::fabs(hi[a])));
    }
    BvhBuild tb = build_bvh4(ibox, iseg, 1, 1, true);
    // leaf references hold positions in `ibox`; map them to instance indices
    for (Node4& nd : tb.nodes)
        for (int c = 0; c < nd.count; ++c)
            if (nd.child[c] & CHILD_LEAF) nd.child[c] = leaf_ref(ids[leaf_first(nd.child[c])], 1u);
    s.tlas = tb.nodes;
    s.tlas_levels = tb.levels;
    build_flat_bvh(g, leaf_max, s);
    return s;
}

// ---------------------------------------------------------------- refit (instance update)
// Union of a node's child boxes.
inline Aabb node_union(const Node4& nd) {
    Aabb b = aabb_empty();
    for (uint32_t c = 0; c < nd.count; ++c)
        b = aabb_union(b, Aabb{v3{nd.box[0][c], nd.box[2][c], nd.box[4][c]}, v3{nd.box[1][c], nd.box[3][c], nd.box[5][c]}});
    return b;
}
inline void set_child_box(Node4& nd, int c, const Aabb& b) {
    nd.box[0][c] = b.lo.x;
    nd.box[1][c] = b.hi.x;
    nd.box[2][c] = b.lo.y;
    nd.box[3][c] = b.hi.y;
    nd.box[4][c] = b.lo.z;
    nd.box[5][c] = b.hi.z;
}
inline float root_bound(const std::vector<Node4>& nodes) {
    float bound = 0.0f;
    if (nodes.empty()) return bound;
    const Node4& r = nodes[0];
    for (int k = 0; k < 6; ++k)
        for (uint32_t c = 0; c < r.count; ++c) bound = fmx(bound, std::fabs(r.box[k][c]));
    return bound;
}
// Refits the flat BVH and the TLAS to the instances' current transforms (topology kept):
// children have larger node indices than their parents, so one reverse pass suffices.
inline void refit_world_structures(const Geometry& g, SceneBvh& s) {
    for (size_t i = s.flat.size(); i-- > 0;) {
        Node4& nd = s.flat[i];
        for (uint32_t c = 0; c < nd.count; ++c) {
            uint32_t r = nd.child[c];
            Aabb b = aabb_empty();
            if (r & CHILD_LEAF) {
                for (uint32_t q = leaf_first(r); q < leaf_first(r) + leaf_count(r); ++q) {
                    const TriRecord& tr = s.flat_tris[q];
                    const Instance& in = g.instances[tr.mesh];
                    v3 w0 = mat43_point(in.transform, v3{tr.v0[0], tr.v0[1], tr.v0[2]});
                    v3 w1 = mat43_point(in.transform, v3{tr.v1[0], tr.v1[1], tr.v1[2]});
                    v3 w2 = mat43_point(in.transform, v3{tr.v2[0], tr.v2[1], tr.v2[2]});
                    b = aabb_union(b, canon_box(aabb_point(aabb_point(Aabb{w0, w0}, w1), w2)));
                }
            } else {
                b = node_union(s.flat[r]);
            }
            set_child_box(nd, (int)c, b);
        }
    }
    s.flat_bound = root_bound(s.flat);
    for (size_t i = s.tlas.size(); i-- > 0;) {
        Node4& nd = s.tlas[i];
        for (uint32_t c = 0; c < nd.count; ++c) {
            uint32_t r = nd.child[c];
            Aabb b = aabb_empty();
            if (r & CHILD_LEAF) {
                const Instance& in = g.instances[leaf_first(r)];
                Aabb mb = node_union(s.blas[in.mesh_index]);
                for (int k = 0; k < 8; ++k) {
                    v3 cc = v3{(k & 1) ? mb.hi.x : mb.lo.x, (k & 2) ? mb.hi.y : mb.lo.y, (k & 4) ? mb.hi.z : mb.lo.z};
                    b = aabb_point(b, mat43_point(in.transform, cc));
                }
                b = canon_box(b);
            } else {
                b = node_union(s.tlas[r]);
            }
            set_child_box(nd, (int)c, b);
        }
    }
    s.tlas_bound = root_bound(s.tlas);
}

inline void trace_blas(const SceneBvh& s, uint32_t root, uint32_t inst, const RayPre& rp,
                       const NodeRay& nr, bool cull_back, float tmin, Hit& best, float& tbest) {
    uint32_t stack[256];
    int sp = 0;
    stack[sp++] = root;
    while (sp > 0) {
        const Node4& nd = s.blas[stack[--sp]];
        float tn[4];
        int mask = node_hits(nd, nr, tmin, tbest, tn);
        for (int c = 0; c < nd.count; ++c) {
            if (!(mask & (1 << c))) continue;
            uint32_t ch = nd.child[c];
            if (ch & CHILD_LEAF) {
                uint32_t f = leaf_first(ch), k = leaf_count(ch);
                for (uint32_t q = f; q < f + k; ++q) {
                    const TriRecord& tr = s.tris[q];
                    float t, u, v;
                    if (!intersect_triangle(rp, v3{tr.v0[0], tr.v0[1], tr.v0[2]},
                                            v3{tr.v1[0], tr.v1[1], tr.v1[2]},
                                            v3{tr.v2[0], tr.v2[1], tr.v2[2]}, cull_back, tmin,
                                            tbest, t, u, v))
                        continue;
                    if (closer(t, inst, tr.prim, best)) {
                        best = Hit{1, t, u, v, inst, tr.prim};
                        tbest = t;
                    }
                }
            } else {
                stack[sp++] = ch;
            }
        }
    }
}

// Closest hit through the two-level BVH.
inline Hit trace_bvh(const Geometry& g, const SceneBvh& s, v3 o, v3 d, float tmin, float tmax,
                     bool cull_back) {
    Hit best{0, 0.0f, 0.0f, 0.0f, 0u, 0u};
    if (!finite3(d) || s.tlas.empty()) return best;
    float tbest = tmax;
    NodeRay wr = node_ray(o, d, s.tlas_bound);
    uint32_t stack[256];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const Node4& nd = s.tlas[stack[--sp]];
        float tn[4];
        int mask = node_hits(nd, wr, tmin, tbest, tn);
        for (int c = 0; c < nd.count; ++c) {
            if (!(mask & (1 << c))) continue;
            uint32_t ch = nd.child[c];
            if (ch & CHILD_LEAF) {
                uint32_t inst = leaf_first(ch);
                const Instance& in = g.instances[inst];
                v3 oo, od;
                object_ray(in, o, d, oo, od);
                if (!finite3(od)) continue;
                RayPre rp = ray_precompute(oo, od);
                NodeRay nr = node_ray(oo, od, 1.0f);
                trace_blas(s, in.mesh_index, inst, rp, nr, cull_back, tmin, best, tbest);
            } else {
                stack[sp++] = ch;
            }
        }
    }
    return best;
}

// Conservative slab test of the eight children of a wide node: the decoded planes
// origin + q 2^(e - 127) enter the slab distances as fma(q, 2^(e - 127) / d, fma(origin, 1/d,
// -o/d -+ E)) (the margin E of node_ray); empty slots (neither internal nor leaf) never pass.
inline int wide_node_hits(const Node8& nd, const NodeRay& r, float tmin, float tbest) {
    const float ia[3] = {r.inv.x, r.inv.y, r.inv.z};
    const uint8_t* qlo[3] = {nd.qlo_x, nd.qlo_y, nd.qlo_z};
    const uint8_t* qhi[3] = {nd.qhi_x, nd.qhi_y, nd.qhi_z};
    float step[3], base_near[3], base_far[3];
    for (int a = 0; a < 3; ++a) {
        step[a] = bitsf((uint32_t)nd.exponent[a] << 23) * ia[a];
        base_near[a] = std::fmaf(nd.origin[a], ia[a], r.nob_near[a]);
        base_far[a] = std::fmaf(nd.origin[a], ia[a], r.nob_far[a]);
    }
    int mask = 0;
    for (int c = 0; c < 8; ++c) {
        if (!((nd.imask >> c) & 1) && nd.meta[c] == 0) continue;
        float tn = tmin, tf = tbest;
        for (int a = 0; a < 3; ++a) {
            float qn = (float)(r.near[a] ? qhi[a][c] : qlo[a][c]);
            float qf = (float)(r.near[a] ? qlo[a][c] : qhi[a][c]);
            tn = fmx(tn, std::fmaf(qn, step[a], base_near[a]));
            tf = fmn(tf, std::fmaf(qf, step[a], base_far[a]));
        }
        if (tn <= tf) mask |= 1 << c;
    }
    return mask;
}

// Closest hit through the wide format of the flat structure (checks its decoding and layout; the
// GPU traversal visits the same nodes in another order and finds the same hit).
inline Hit trace_wide(const Geometry& g, const SceneBvh& s, v3 o, v3 d, float tmin, float tmax, bool cull_back) {
    Hit best{0, 0.0f, 0.0f, 0.0f, 0u, 0u};
    if (!finite3(d) || s.wide.empty()) return best;
    float tbest = tmax;
    NodeRay wr = node_ray(o, d, s.flat_bound);
    uint32_t cur = 0xffffffffu;
    bool skip = false;
    RayPre rp{};
    std::vector<uint32_t> stack;
    stack.push_back(0u);
    while (!stack.empty()) {
        const Node8& nd = s.wide[stack.back()];
        stack.pop_back();
        int mask = wide_node_hits(nd, wr, tmin, tbest);
        uint32_t rank = 0;
        for (int c = 0; c < 8; ++c) {
            bool internal = (nd.imask >> c) & 1;
            if (internal && (mask >> c) & 1) stack.push_back(nd.child_base + rank);
            rank += internal ? 1u : 0u;
            if (internal || !((mask >> c) & 1)) continue;
            uint32_t off = nd.meta[c] & 31u, units = nd.meta[c] >> 5;
            for (uint32_t j = 0; units >> j; ++j) {
                const TriRecord& tr = s.wide_tris[nd.tri_base + off + j];
                if (tr.mesh != cur) {
                    cur = tr.mesh;
                    v3 oo, od;
                    object_ray(g.instances[cur], o, d, oo, od);
                    skip = !finite3(od);
                    rp = ray_precompute(oo, od);
                }
                float t, u, v;
                if (skip) continue;
                if (!intersect_triangle(rp, v3{tr.v0[0], tr.v0[1], tr.v0[2]}, v3{tr.v1[0], tr.v1[1], tr.v1[2]},
                                        v3{tr.v2[0], tr.v2[1], tr.v2[2]}, cull_back, tmin, tbest, t, u, v))
                    continue;
                if (closer(t, cur, tr.prim, best)) {
                    best = Hit{1, t, u, v, cur, tr.prim};
                    tbest = t;
                }
            }
        }
    }
    return best;
}

// Closest hit through the flat BVH: each triangle is tested in its instance's object space.
inline Hit trace_flat(const Geometry& g, const SceneBvh& s, v3 o, v3 d, float tmin, float tmax, bool cull_back) {
    Hit best{0, 0.0f, 0.0f, 0.0f, 0u, 0u};
    if (!finite3(d) || s.flat.empty()) return best;
    float tbest = tmax;
    NodeRay wr = node_ray(o, d, s.flat_bound);
    uint32_t cur = 0xffffffffu;
    bool skip = false;  // the object ray of instance `cur` is not finite: its triangles miss
    RayPre rp{};
    uint32_t stack[256];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const Node4& nd = s.flat[stack[--sp]];
        float tn[4];
        int mask = node_hits(nd, wr, tmin, tbest, tn);
        for (int c = 0; c < (int)nd.count; ++c) {
            if (!(mask & (1 << c))) continue;
            uint32_t ch = nd.child[c];
            if (!(ch & CHILD_LEAF)) {
                stack[sp++] = ch;
                continue;
            }
            for (uint32_t q = leaf_first(ch); q < leaf_first(ch) + leaf_count(ch); ++q) {
                const TriRecord& tr = s.flat_tris[q];
                if (tr.mesh != cur) {
                    cur = tr.mesh;
                    v3 oo, od;
                    object_ray(g.instances[cur], o, d, oo, od);
                    skip = !finite3(od);
                    rp = ray_precompute(oo, od);
                }
                float t, u, v;
                if (skip) continue;
                if (!intersect_triangle(rp, v3{tr.v0[0], tr.v0[1], tr.v0[2]}, v3{tr.v1[0], tr.v1[1], tr.v1[2]},
                                        v3{tr.v2[0], tr.v2[1], tr.v2[2]}, cull_back, tmin, tbest, t, u, v))
                    continue;
                if (closer(t, cur, tr.prim, best)) {
                    best = Hit{1, t, u, v, cur, tr.prim};
                    tbest = t;
                }
            }
        }
    }
    return best;
}

}  // namespace ref
