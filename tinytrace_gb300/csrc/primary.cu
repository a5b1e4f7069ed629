// Primary visibility by rasterisation, for flat BVH4 scenes (PrimaryParams in tt_kernels.h).
//
// The reference traces camera rays like any other ray (the ray query of
// src/integrate/integrate.glsl:112-127 at bounce 0).  Here the closest hit of every camera ray
// of a sample chunk is found before the chunk's first extension pass: every camera ray starts
// at the camera position, so each triangle record can be bounded on the screen, and only the
// samples inside its rectangle are tested against it, with the traversal's own ray set-up and
// watertight ray/triangle test.  A sample keeps the smallest key (t bits << 32 | scene triangle
// index); t >= tmin > 0 orders as its bits do, and the scene triangle index
// (tri_base[instance] + primitive) orders as (instance, primitive), so the smallest key is the
// hit the traversal's closest-hit rule selects, whatever the order of the tests.
//
// The bound of a record is conservative:
//   * the sample's direction is d = normalize(B (ndc.x, ndc.y, 1)) with B from the inverse
//     projection and view matrices (camera_ray_direction), so in an instance's object space a
//     point p on a camera ray satisfies C^-1 (p - oo) = lambda (ndc.x, ndc.y, 1), C = X B (X the
//     object-from-world 3x3), lambda = t / |B (ndc, 1)| > 0: the record's vertices, mapped this
//     way, project to the ndc of the rays through them (C^-1 per instance in double precision,
//     the per-record projection in float; records that cross lambda_clip in double);
//   * oo is the float origin instance_ray computes, so the bound and the test share the origin;
//   * the pixel-position rectangle and the three edge functions of the projected triangle are
//     widened by a margin: BASE_MARGIN_PX (the float rounding of the camera ray and of the
//     ray/triangle test is ~1e-3 pixel), plus COND_MARGIN x cond(X) x the camera's pixels per
//     radian (the direction error an ill-conditioned instance matrix adds to the float
//     object-space ray), plus PROJ_MARGIN x cond(C) x the screen width (the float projection
//     errs by at most ~17 eps cond(C) in ndc on screen); the edge functions also carry their own
//     evaluation error;
//   * parts of a record with lambda < lambda_clip (half the least lambda of a hit at tmin) are
//     clipped away, so records that cross the camera plane keep a finite rectangle (and no edge
//     functions);
//   * records facing away from the camera beyond a cosine of BACKFACE_COS plus the rounding
//     bound of their normal are dropped (extension rays cull back faces, and such a record
//     yields det < 0 for every camera ray);
//   * an instance whose matrices are singular, non-finite or too badly conditioned has no
//     bound: its records cover the whole screen.
// The key pass runs over (record, pixel) pairs of the records with pixels, listed densely;
// samples that pass a record's rectangle and edges are queued per warp and tested 32 at a time.
// If the frame's pixel-record pairs exceed PAIR_LIMIT the keys are not built (ok = 0) and the
// extension kernel traverses the camera rays instead.
#include <algorithm>
#include <cmath>

#include "tt_internal.h"
#include "tt_kernels.h"
#include "tt_shade.cuh"

namespace tt {
namespace {

constexpr double BASE_MARGIN_PX = 0.05;
constexpr double COND_MARGIN = 2.0e-6;
constexpr double PROJ_MARGIN = 2.0e-6;  // float bound: per unit condition number of C, per pixel of width
constexpr float BACKFACE_COS = 1.0e-3f;
constexpr float EDGE_EVAL_MARGIN = 1.0e-3f;  // pixels: rounding of an edge function's evaluation
constexpr float EDGE_MAX_COORD = 1.0e5f;     // edge functions only for vertices within this many pixels
constexpr double MAX_PROJECTION_COND = 1.0e6;  // beyond this the float bound is not used
constexpr unsigned long long PAIR_LIMIT = 1ull << 31;
constexpr int RASTER_BLOCK = 256;
// 4 resident blocks per SM (61 registers, 32 warps): the 1080p 64-spp key pass 2.38 -> 2.17 ms
// (set-up included) against 3 blocks (75 registers)
#ifndef TT_RASTER_MIN_BLOCKS
#define TT_RASTER_MIN_BLOCKS 4
#endif
constexpr int RASTER_WARPS = RASTER_BLOCK / 32;
constexpr int SAMPLE_GROUP = 8;
constexpr int QUEUE_CAP = 32 + 32 * SAMPLE_GROUP;  // < 32 left over + one group's entries

__host__ __device__ inline void mul3(const double* a, const double* b, double* out) {  // row-major
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) out[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
}
__host__ __device__ inline bool inverse3(const double* m, double* out) {
    double c0 = m[4] * m[8] - m[5] * m[7], c1 = m[5] * m[6] - m[3] * m[8], c2 = m[3] * m[7] - m[4] * m[6];
    double det = m[0] * c0 + m[1] * c1 + m[2] * c2;
    if (!(det != 0.0) || !isfinite(det)) return false;
    double r = 1.0 / det;
    out[0] = c0 * r;
    out[1] = (m[2] * m[7] - m[1] * m[8]) * r;
    out[2] = (m[1] * m[5] - m[2] * m[4]) * r;
    out[3] = c1 * r;
    out[4] = (m[0] * m[8] - m[2] * m[6]) * r;
    out[5] = (m[2] * m[3] - m[0] * m[5]) * r;
    out[6] = c2 * r;
    out[7] = (m[1] * m[6] - m[0] * m[7]) * r;
    out[8] = (m[0] * m[4] - m[1] * m[3]) * r;
    for (int k = 0; k < 9; ++k)
        if (!isfinite(out[k])) return false;
    return true;
}
__host__ __device__ inline double frobenius(const double* m) {
    double s = 0.0;
    for (int k = 0; k < 9; ++k) s += m[k] * m[k];
    return sqrt(s);
}

__device__ __forceinline__ f3 xyz3(float4 v) { return f3{v.x, v.y, v.z}; }
__device__ __forceinline__ uint32_t lanes_below() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// The pixels whose samples can fall in the pixel-position rectangle [lo, hi] (pixel p covers
// positions [p - 0.5, p + 0.5)); a > b when none.
__device__ __forceinline__ void pixel_span(float lo, float hi, uint32_t n, int& a, int& b) {
    a = max(0, (int)ceilf(lo - 0.5f));
    b = min((int)n - 1, (int)floorf(hi + 0.5f));
}

// Per instance, in double precision: the projection C^-1 = (X B)^-1 and the margin.  The margin
// adds to BASE_MARGIN_PX the direction error an ill-conditioned X adds to the float rays
// (COND_MARGIN x cond(X) x pixels per radian) and the error of evaluating the projection in float
// (PROJ_MARGIN x cond(C) x the screen width: |delta v| / |v| <= 5 eps cond(C) for v = C^-1 q with
// rounded C^-1 and q, ndc = v.xy / v.z then errs by at most ~17 eps cond(C) on screen).
__global__ void primary_instance_kernel(const __grid_constant__ DevScene sc, f3 camera,
                                        const __grid_constant__ PrimaryParams v, uint32_t W, uint32_t H) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.instance_count) return;
    f3 oo, od;
    uint32_t mesh;
    instance_ray(sc, i, camera, f3{0.0f, 0.0f, 1.0f}, oo, od, mesh);
    const float4* x = sc.inst_xform + 4ull * i;
    float4 r0 = x[0], r1 = x[1], r2 = x[2];
    double X[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
    double C[9], Ci[9], Xi[9];
    mul3(X, v.B, C);
    bool ok = inverse3(C, Ci) && inverse3(X, Xi) && finite3(oo);
    double cond_c = ok ? frobenius(C) * frobenius(Ci) : 0.0;
    ok = ok && cond_c < MAX_PROJECTION_COND;
    double margin = BASE_MARGIN_PX + COND_MARGIN * frobenius(X) * frobenius(Xi) * v.pixel_scale +
                    PROJ_MARGIN * cond_c * (double)max(W, H);
    PrimaryInstance& I = v.inst[i];
    I.oo[0] = oo.x;
    I.oo[1] = oo.y;
    I.oo[2] = oo.z;
    for (int k = 0; k < 9; ++k) I.ci[k] = ok ? (float)Ci[k] : 0.0f;
    I.margin = __double2float_ru(margin);
    I.ok = ok && isfinite(margin) && margin < 1.0e6 ? 1u : 0u;
    I.pad[0] = I.pad[1] = 0.0f;
}

struct P3 {
    double x, y, l;  // C^-1 (p - oo): lambda (ndc.x, ndc.y, 1)
};

// The rare records that cross lambda_clip: clipped (Sutherland-Hodgman against one plane) and
// projected in double precision; false when nothing is left.
__device__ __noinline__ bool clipped_bounds(const PrimaryInstance& I, float4 va, float4 vb, float4 vc, double lc,
                                            double W, double H, double& xlo, double& ylo, double& xhi, double& yhi) {
    P3 p[3];
    const float4 vtx[3] = {va, vb, vc};
    for (int k = 0; k < 3; ++k) {
        double q[3] = {(double)vtx[k].x - I.oo[0], (double)vtx[k].y - I.oo[1], (double)vtx[k].z - I.oo[2]};
        const float* m = I.ci;
        p[k].x = (double)m[0] * q[0] + (double)m[1] * q[1] + (double)m[2] * q[2];
        p[k].y = (double)m[3] * q[0] + (double)m[4] * q[1] + (double)m[5] * q[2];
        p[k].l = (double)m[6] * q[0] + (double)m[7] * q[1] + (double)m[8] * q[2];
    }
    P3 poly[4];
    int np = 0;
    for (int k = 0; k < 3; ++k) {
        const P3& s = p[k];
        const P3& e = p[(k + 1) % 3];
        bool sin = s.l >= lc, ein = e.l >= lc;
        if (sin) poly[np++] = s;
        if (sin != ein) {
            double f = (lc - s.l) / (e.l - s.l);
            poly[np++] = P3{s.x + (e.x - s.x) * f, s.y + (e.y - s.y) * f, lc};
        }
    }
    if (np == 0) return false;
    xlo = ylo = INFINITY;
    xhi = yhi = -INFINITY;
    for (int k = 0; k < np; ++k) {
        double l = fmax(poly[k].l, lc);
        double px = (poly[k].x / l + 1.0) * 0.5 * W;
        double py = (poly[k].y / l + 1.0) * 0.5 * H;
        xlo = fmin(xlo, px);
        xhi = fmax(xhi, px);
        ylo = fmin(ylo, py);
        yhi = fmax(yhi, py);
    }
    if (!(isfinite(xlo) && isfinite(xhi) && isfinite(ylo) && isfinite(yhi))) {
        xlo = ylo = -4.0;
        xhi = W + 4.0;
        yhi = H + 4.0;
    }
    return true;
}

// Per record: the pixel-position rectangle (widened by the instance's margin), its pixel count,
// and, for records wholly in front of lambda_clip, the three edge functions of the projected
// triangle moved out by the margin (a sample outside them cannot hit the record).  float
// arithmetic; the margin covers its rounding.
__global__ void primary_rect_kernel(const __grid_constant__ DevScene sc, const __grid_constant__ PrimaryParams v,
                                    uint32_t W, uint32_t H) {
    uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t cnt = 0u;
    float4 rect = make_float4(1.0f, 1.0f, 0.0f, 0.0f);
    const float4 pass = make_float4(0.0f, 0.0f, 1.0f, 0.0f);  // an edge function every sample passes
    float4 edge[3] = {pass, pass, pass};
    if (r < v.records) {
        const float4 va = sc.tris[3ull * r], vb = sc.tris[3ull * r + 1], vc = sc.tris[3ull * r + 2];
        const PrimaryInstance& I = v.inst[__float_as_uint(vb.w)];
        const float Wf = (float)W, Hf = (float)H;
        bool any = false;
        float xlo = 0.0f, ylo = 0.0f, xhi = 0.0f, yhi = 0.0f;
        if (!I.ok) {
            any = true;
            xlo = ylo = -4.0f;
            xhi = Wf + 4.0f;
            yhi = Hf + 4.0f;
        } else {
            const f3 oo = f3{I.oo[0], I.oo[1], I.oo[2]};
            f3 a = xyz3(va), b = xyz3(vb), c = xyz3(vc);
            // back faces (extension rays cull them): object-space vertices are within the unit
            // cube, so each edge's float difference errs by at most 1e-7 per unit of length
            f3 e1 = b - a, e2 = c - a, q0 = a - oo;
            f3 n = cross(e1, e2);
            float l1 = length(e1), l2 = length(e2);
            float nerr = 1.0e-7f * (l1 + l2) + 2.4e-7f * l1 * l2;
            // front faces have their normal towards the ray origin, dot(n, oo - a) > 0
            bool back = dot(n, q0) > (BACKFACE_COS * length(n) + 4.0f * nerr) * length(q0);
            if (!back) {
                const float* m = I.ci;
                f3 q[3] = {q0, b - oo, c - oo};
                float px[3], py[3], pl[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    px[k] = m[0] * q[k].x + m[1] * q[k].y + m[2] * q[k].z;
                    py[k] = m[3] * q[k].x + m[4] * q[k].y + m[5] * q[k].z;
                    pl[k] = m[6] * q[k].x + m[7] * q[k].y + m[8] * q[k].z;
                }
                const float lc = (float)v.lambda_clip;
                if (pl[0] >= lc && pl[1] >= lc && pl[2] >= lc) {
                    float sx[3], sy[3];
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        sx[k] = (px[k] / pl[k] + 1.0f) * (0.5f * Wf);
                        sy[k] = (py[k] / pl[k] + 1.0f) * (0.5f * Hf);
                    }
                    any = true;
                    xlo = fminf(fminf(sx[0], sx[1]), sx[2]);
                    xhi = fmaxf(fmaxf(sx[0], sx[1]), sx[2]);
                    ylo = fminf(fminf(sy[0], sy[1]), sy[2]);
                    yhi = fmaxf(fmaxf(sy[0], sy[1]), sy[2]);
                    float big = fmaxf(fmaxf(fabsf(xlo), fabsf(xhi)), fmaxf(fabsf(ylo), fabsf(yhi)));
                    if (!isfinite(big)) {
                        xlo = ylo = -4.0f;
                        xhi = Wf + 4.0f;
                        yhi = Hf + 4.0f;
                    } else if (big < EDGE_MAX_COORD) {
                        float area = (sx[1] - sx[0]) * (sy[2] - sy[0]) - (sy[1] - sy[0]) * (sx[2] - sx[0]);
                        float em = I.margin + EDGE_EVAL_MARGIN + 4.0e-7f * big;
                        float4 ed[3];
                        bool usable = fabsf(area) > 1.0e-4f;
#pragma unroll
                        for (int k = 0; k < 3; ++k) {
                            const int k1 = k == 2 ? 0 : k + 1;
                            float dx = sx[k1] - sx[k], dy = sy[k1] - sy[k];
                            float len = sqrtf(dx * dx + dy * dy);
                            usable = usable && len > 1.0e-2f;
                            float s = (area > 0.0f ? 1.0f : -1.0f) / fmaxf(len, 1.0e-2f);
                            float na = -dy * s, nb = dx * s;  // unit normal towards the inside
                            ed[k] = make_float4(na, nb, em - (na * sx[k] + nb * sy[k]), 0.0f);
                        }
                        if (usable) {
                            edge[0] = ed[0];
                            edge[1] = ed[1];
                            edge[2] = ed[2];
                        }
                    }
                    xlo -= I.margin;
                    ylo -= I.margin;
                    xhi += I.margin;
                    yhi += I.margin;
                } else if (pl[0] >= lc || pl[1] >= lc || pl[2] >= lc) {
                    double dxlo, dylo, dxhi, dyhi;
                    if (clipped_bounds(I, va, vb, vc, v.lambda_clip, W, H, dxlo, dylo, dxhi, dyhi)) {
                        any = true;
                        xlo = __double2float_rd(fmax(dxlo, -1.0e9) - I.margin);
                        ylo = __double2float_rd(fmax(dylo, -1.0e9) - I.margin);
                        xhi = __double2float_ru(fmin(dxhi, 1.0e9) + I.margin);
                        yhi = __double2float_ru(fmin(dyhi, 1.0e9) + I.margin);
                    }
                }
            }
        }
        if (any) {
            xlo = fminf(fmaxf(xlo, -4.0f), Wf + 4.0f);
            xhi = fminf(fmaxf(xhi, -4.0f), Wf + 4.0f);
            ylo = fminf(fmaxf(ylo, -4.0f), Hf + 4.0f);
            yhi = fminf(fmaxf(yhi, -4.0f), Hf + 4.0f);
            float4 f = make_float4(xlo, ylo, xhi, yhi);
            int x0, x1, y0, y1;
            pixel_span(f.x, f.z, W, x0, x1);
            pixel_span(f.y, f.w, H, y0, y1);
            if (x0 <= x1 && y0 <= y1) {
                rect = f;
                unsigned long long pixels = (unsigned long long)(x1 - x0 + 1) * (unsigned long long)(y1 - y0 + 1);
                cnt = pixels > 0xffffffffull ? 0xffffffffu : (uint32_t)pixels;
            }
        }
        v.rect[r] = rect;
        v.edge[3ull * r] = edge[0];
        v.edge[3ull * r + 1] = edge[1];
        v.edge[3ull * r + 2] = edge[2];
    }
    if (r <= v.records) v.count[r] = cnt;  // count[records] = 0: the exclusive prefix ends with the total
    unsigned long long sum = cnt;
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31u) == 0u && sum) atomicAdd(v.total, sum);
}

__global__ void primary_finish_kernel(const __grid_constant__ PrimaryParams v) {
    *v.ok = *v.total < PAIR_LIMIT ? 1u : 0u;
}

// The records with pixels, listed densely (after the scan of the counts): each has at least one
// pair, so the 32 pairs a warp takes lie in at most 32 consecutive listed records.
__global__ void primary_live_flag_kernel(const __grid_constant__ PrimaryParams v) {
    uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r > v.records) return;
    v.live_pos[r] = r < v.records && v.count[r + 1] > v.count[r] ? 1u : 0u;
}
__global__ void primary_live_scatter_kernel(const __grid_constant__ PrimaryParams v) {
    uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r > v.records) return;
    if (r == v.records) {
        const uint32_t n = v.live_pos[r];
        *v.live_n = n;
        v.live_first[n] = v.count[r];
        return;
    }
    if (v.count[r + 1] > v.count[r]) {
        const uint32_t i = v.live_pos[r];
        v.live_rec[i] = r;
        v.live_first[i] = v.count[r];
    }
}

__device__ __forceinline__ bool inside_edge(float4 e, float px, float py) {
    return __fmaf_rn(e.x, px, __fmaf_rn(e.y, py, e.z)) >= 0.0f;
}

// Each warp takes 32 pixel-record pairs at a time, one per lane.  A lane draws its pixel's
// samples in order (the draws of pixel_ndc) and queues those whose position passes the record's
// rectangle and edge functions; the warp then tests queued samples 32 at a time, every lane busy,
// with the traversal's ray set-up and ray/triangle test, reading the pair from its lane.  A
// queue entry is the lane (5 bits), the sample (6 bits) and the two draws' mantissas (23 bits
// each).
__global__ void __launch_bounds__(RASTER_BLOCK, TT_RASTER_MIN_BLOCKS) primary_raster_kernel(const __grid_constant__ RenderParams p,
                                                                      const __grid_constant__ PrimaryParams v,
                                                                      uint32_t chunk_sample0, uint32_t chunk_spp,
                                                                      const __grid_constant__ XsJump jump,
                                                                      uint32_t range_pairs) {
    __shared__ unsigned long long s_queue[RASTER_WARPS][QUEUE_CAP];
    if (*v.ok == 0u) return;
    const tt_constants& c = p.c;
    const DevScene& sc = p.sc;
    const uint32_t W = c.screen_size[0], H = c.screen_size[1];
    const uint64_t WH = (uint64_t)W * H;
    const uint32_t live = *v.live_n;
    const uint32_t total = v.live_first[live];
    const uint32_t frame_hash = jenkins_hash(c.frame_index);
    const f3 camera = f3{c.camera_position[0], c.camera_position[1], c.camera_position[2]};
    const uint32_t lane = threadIdx.x & 31u;
    unsigned long long* queue = s_queue[threadIdx.x >> 5];

    // tests queue entry `e` (have: the lane holds one) of the pair of lane e & 31; every lane calls
    auto test = [&](unsigned long long e, bool have, uint32_t rec, uint32_t x, uint32_t y, uint32_t t, uint32_t tri) {
        const uint32_t owner = (uint32_t)e & 31u;
        const uint32_t orec = __shfl_sync(0xffffffffu, rec, owner), ox_ = __shfl_sync(0xffffffffu, x, owner),
                       oy_ = __shfl_sync(0xffffffffu, y, owner), ot = __shfl_sync(0xffffffffu, t, owner),
                       otri = __shfl_sync(0xffffffffu, tri, owner);
        if (!have) return;
        const uint32_t s = (uint32_t)(e >> 5) & 63u;
        const float ox = mantissa_float((uint32_t)(e >> 11) & 0x7fffffu), oy = mantissa_float((uint32_t)(e >> 34) & 0x7fffffu);
        f3 d = camera_ray_direction(c, pixel_ndc_from_draws(ox_, oy_, W, H, ox, oy));
        if (!finite3(d)) return;
        const float4 a = __ldg(sc.tris + 3ull * orec), b = __ldg(sc.tris + 3ull * orec + 1),
                     cc = __ldg(sc.tris + 3ull * orec + 2);
        f3 oo, od;
        uint32_t mesh;
        instance_ray(sc, __float_as_uint(b.w), camera, d, oo, od, mesh);
        if (!finite3(od)) return;
        RayPre rp = ray_precompute(oo, od);
        float th, u, w;
        if (!intersect_triangle(rp, tri_vertex(a), tri_vertex(b), tri_vertex(cc), true, EXTENSION_TMIN, EXTENSION_TMAX,
                                th, u, w))
            return;
        unsigned long long key = ((unsigned long long)__float_as_uint(th) << 32) | otri;
        unsigned long long* dst = v.key + (uint64_t)s * WH + ot;
        if (key < *dst) atomicMin(dst, key);
    };

    // warps claim ranges of pairs (a multiple of 32: about six ranges per warp of the wave, at most
    // range_pairs, fewer when the pairs carry more samples, so that the last ranges end
    // together) and take them 32 at a time: one search for the range's first listed record, then
    // each batch's first record follows from the previous batch's last
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t share = (uint32_t)(((uint64_t)total / (6ull * warps) + 31ull) & ~31ull);
    const uint32_t range = share < 128u ? 128u : (share > range_pairs ? range_pairs : share);
    while (true) {
        uint32_t begin = 0u;
        if (lane == 0u) begin = atomicAdd(v.next, range);
        begin = __shfl_sync(0xffffffffu, begin, 0);
        if (begin >= total) break;
        const uint32_t end = total - begin > range ? begin + range : total;
        uint32_t r0 = 0u;
        if (lane == 0u) {
            uint32_t lo = 0u, hi = live;  // live_first[lo] <= begin < live_first[hi]
            while (hi - lo > 1u) {
                uint32_t mid = (lo + hi) >> 1;
                if (__ldg(v.live_first + mid) <= begin) lo = mid;
                else hi = mid;
            }
            r0 = lo;
        }
        r0 = __shfl_sync(0xffffffffu, r0, 0);
        for (uint32_t base = begin; base < end; base += 32u) {
            const uint32_t k = base + lane;
            const bool valid = k < end;
            uint32_t rec = 0u, x = 0u, y = 0u, t = 0u, tri = 0u, pg = 0u;
            float4 rect = make_float4(1.0f, 1.0f, 0.0f, 0.0f), e0 = rect, e1 = rect, e2 = rect;
            // each lane's listed record within the 32 from r0 (the record of pair `base`):
            // live_first[r0 + i] >= base + i for i >= 1, so pair base + 31 lies before r0 + 32
            const uint32_t window = r0 + lane < live ? __ldg(v.live_first + r0 + lane) : 0xffffffffu;
            uint32_t wlo = 0u, whi = 32u;  // window[wlo] <= k < window[whi] (window[32] > base + 31)
    #pragma unroll
            for (int step = 0; step < 5; ++step) {
                const uint32_t mid = (wlo + whi) >> 1;
                const uint32_t wv = __shfl_sync(0xffffffffu, window, mid);
                if (wv <= k) wlo = mid;
                else whi = mid;
            }
            const uint32_t first = __shfl_sync(0xffffffffu, window, wlo);
            if (valid) {
                rec = __ldg(v.live_rec + r0 + wlo);
                rect = v.rect[rec];
                e0 = v.edge[3ull * rec];
                e1 = v.edge[3ull * rec + 1];
                e2 = v.edge[3ull * rec + 2];
                int x0, x1, y0, y1;
                pixel_span(rect.x, rect.z, W, x0, x1);
                pixel_span(rect.y, rect.w, H, y0, y1);
                const uint32_t bw = (uint32_t)(x1 - x0 + 1);
                const uint32_t j = k - first;
                x = (uint32_t)x0 + j % bw;
                y = (uint32_t)y0 + j / bw;
                t = band_index(x, y, W, H);
                const uint32_t prim = __float_as_uint(__ldg(sc.tris + 3ull * rec).w);
                const uint32_t inst = __float_as_uint(__ldg(sc.tris + 3ull * rec + 1).w);
                tri = __ldg(sc.tri_base + inst) + prim;
                pg = jenkins_hash((x + y * W) ^ frame_hash);
                if (chunk_sample0) pg = xs_apply(jump, pg);
            }
            uint32_t queued = 0u;  // warp-uniform
            for (uint32_t s0 = 0; s0 < chunk_spp; s0 += SAMPLE_GROUP) {
    #pragma unroll
                for (uint32_t j = 0; j < (uint32_t)SAMPLE_GROUP; ++j) {
                    const uint32_t s = s0 + j;
                    bool in = false;
                    uint32_t mx = 0u, my = 0u;
                    if (valid && s < chunk_spp) {
                        // the draws of pixel_ndc: the generator ends two steps on, at the next sample's
                        mx = random_mantissa(pg);
                        my = random_mantissa(pg);
                        const float px = (float)x + (mantissa_float(mx) - 0.5f), py = (float)y + (mantissa_float(my) - 0.5f);
                        in = px >= rect.x && px <= rect.z && py >= rect.y && py <= rect.w && inside_edge(e0, px, py) &&
                             inside_edge(e1, px, py) && inside_edge(e2, px, py);
                    }
                    const uint32_t m = __ballot_sync(0xffffffffu, in);
                    if (in)
                        queue[queued + __popc(m & lanes_below())] =
                            lane | (s << 5) | ((unsigned long long)mx << 11) | ((unsigned long long)my << 34);
                    queued += __popc(m);
                }
                __syncwarp();
                while (queued >= 32u) {
                    queued -= 32u;
                    test(queue[queued + lane], true, rec, x, y, t, tri);
                }
                __syncwarp();
            }
            if (queued) {
                const bool have = lane < queued;
                test(have ? queue[lane] : 0ull, have, rec, x, y, t, tri);
            }
            __syncwarp();
            // the record of pair base + 32: lane 31's record, or the next one if that starts there
            const uint32_t last = r0 + __shfl_sync(0xffffffffu, wlo, 31);
            uint32_t next = last;
            if (lane == 0u && last + 1u < live && __ldg(v.live_first + last + 1u) <= base + 32u) next = last + 1u;
            r0 = __shfl_sync(0xffffffffu, next, 0);
        }
    }
}

__global__ void primary_round_keys_kernel(const BatchRequest* reqs, BatchRound* round) {
    uint32_t keys = round->keys;
    for (uint32_t r = 0; r < round->nreq && keys; ++r) keys = reqs[r].vis_ok != nullptr && *reqs[r].vis_ok != 0u;
    round->keys = keys ? 1u : 0u;
}

}  // namespace

void primary_round_keys(const BatchRequest* reqs, BatchRound* round, cudaStream_t st) {
    primary_round_keys_kernel<<<1, 1, 0, st>>>(reqs, round);
    check_cuda(cudaGetLastError(), "primary round keys");
}

bool primary_camera(const tt_constants& c, PrimaryParams& v) {
    const float* IP = c.inverse_proj;
    const float* IV = c.inverse_view;
    double A[9], V[9];
    for (int r = 0; r < 3; ++r) {
        A[3 * r + 0] = -(double)IP[0 * 4 + r];
        A[3 * r + 1] = -(double)IP[1 * 4 + r];
        A[3 * r + 2] = (double)IP[2 * 4 + r] + (double)IP[3 * 4 + r];
        for (int j = 0; j < 3; ++j) V[3 * r + j] = IV[j * 4 + r];
    }
    mul3(V, A, v.B);
    double Bi[9];
    if (!inverse3(v.B, Bi)) return false;
    const double W = c.screen_size[0], H = c.screen_size[1];
    if (W < 1.0 || H < 1.0) return false;
    // the largest |B (ndc, 1)| over the screen (ndc reaches 1 + 1/W past the edges with the jitter)
    double ex = 1.0 + 1.0 / W + 0.01, ey = 1.0 + 1.0 / H + 0.01, maxb = 0.0;
    for (int sx = -1; sx <= 1; sx += 2)
        for (int sy = -1; sy <= 1; sy += 2) {
            double n[3] = {sx * ex, sy * ey, 1.0}, len = 0.0;
            for (int r = 0; r < 3; ++r) {
                double d = v.B[3 * r] * n[0] + v.B[3 * r + 1] * n[1] + v.B[3 * r + 2] * n[2];
                len += d * d;
            }
            maxb = std::max(maxb, std::sqrt(len));
        }
    if (!(maxb > 0.0) || !std::isfinite(maxb)) return false;
    v.lambda_clip = 0.5 * (double)EXTENSION_TMIN / maxb;
    // |d ndc| <= |B^-1| |dd| (1 + |ndc|) |B (ndc, 1)| for a unit direction error dd; pixels are
    // W / 2 and H / 2 ndc units
    v.pixel_scale = 0.5 * std::max(W, H) * frobenius(Bi) * (1.0 + std::sqrt(ex * ex + ey * ey)) * maxb;
    return std::isfinite(v.pixel_scale) && std::isfinite(v.lambda_clip);
}

void primary_setup(const RenderParams& p, const PrimaryParams& v, cudaStream_t st) {
    const DevScene& sc = p.sc;
    f3 camera = f3{p.c.camera_position[0], p.c.camera_position[1], p.c.camera_position[2]};
    check_cuda(cudaMemsetAsync(v.total, 0, 8, st), "memset");
    if (sc.instance_count)
        primary_instance_kernel<<<(sc.instance_count + 127) / 128, 128, 0, st>>>(sc, camera, v, p.c.screen_size[0],
                                                                                p.c.screen_size[1]);
    primary_rect_kernel<<<(unsigned)((v.records + 1ull + 255) / 256), 256, 0, st>>>(sc, v, p.c.screen_size[0],
                                                                                   p.c.screen_size[1]);
    check_cuda(cudaGetLastError(), "primary bounds");
    exclusive_scan_u32(v.count, (uint64_t)v.records + 1, st);
    const unsigned g = (unsigned)((v.records + 1ull + 255) / 256);
    primary_live_flag_kernel<<<g, 256, 0, st>>>(v);
    exclusive_scan_u32(v.live_pos, (uint64_t)v.records + 1, st);
    primary_live_scatter_kernel<<<g, 256, 0, st>>>(v);
    primary_finish_kernel<<<1, 1, 0, st>>>(v);
    check_cuda(cudaGetLastError(), "primary finish");
}

void primary_chunk(const RenderParams& p, const PrimaryParams& v, const WfParams& w, cudaStream_t st) {
    uint64_t WH = (uint64_t)p.c.screen_size[0] * p.c.screen_size[1];
    check_cuda(cudaMemsetAsync(v.key, 0xff, 8ull * WH * w.chunk_spp, st), "memset");
    check_cuda(cudaMemsetAsync(v.next, 0, 4, st), "memset");
    // one wave of resident blocks; ranges of at most 512 / spp batches (8..128)
    int occupancy = 0;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occupancy, primary_raster_kernel, RASTER_BLOCK, 0),
               "occupancy");
    const uint32_t batches = std::min<uint32_t>(128u, std::max<uint32_t>(8u, 512u / std::max(w.chunk_spp, 1u)));
    if (v.records)
        primary_raster_kernel<<<v.sms * std::max(occupancy, 1), RASTER_BLOCK, 0, st>>>(
            p, v, w.chunk_sample0, w.chunk_spp, w.chunk_jump, 32u * batches);
    check_cuda(cudaGetLastError(), "primary raster");
}

}  // namespace tt
