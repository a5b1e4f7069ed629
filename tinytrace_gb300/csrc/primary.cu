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
// The rectangle is conservative:
//   * the sample's direction is d = normalize(B (ndc.x, ndc.y, 1)) with B from the inverse
//     projection and view matrices (camera_ray_direction), so in an instance's object space a
//     point p on a camera ray satisfies C^-1 (p - oo) = lambda (ndc.x, ndc.y, 1), C = X B (X the
//     object-from-world 3x3), lambda = t / |B (ndc, 1)| > 0: the record's vertices, mapped this
//     way in double precision, project to the ndc the rays through them have;
//   * oo is the float origin instance_ray computes, so the bound and the test share the origin;
//   * the rectangle is widened by BASE_MARGIN_PX (the float rounding of the camera ray and of the
//     ray/triangle test is ~1e-3 pixel) plus COND_MARGIN x the condition number of X x the pixels
//     per radian of the camera (the direction error an ill-conditioned instance matrix can add);
//   * parts of a record with lambda < lambda_clip (half the least lambda of a hit at tmin) are
//     clipped away, so records that cross the camera plane keep a finite rectangle;
//   * records facing away from the camera beyond a cosine of BACKFACE_COS are dropped (extension
//     rays cull back faces, and such a record yields det < 0 for every camera ray);
//   * an instance whose matrices are singular or non-finite has no bound: its records cover the
//     whole screen.
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
constexpr double BACKFACE_COS = 1.0e-4;
constexpr double MAX_PROJECTION_COND = 1.0e8;  // beyond this the double projection is not trusted
constexpr unsigned long long PAIR_LIMIT = 1ull << 31;
constexpr int RASTER_BLOCK = 256;

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

// Index of pixel (x, y) in the band order of the integrator's work items (the inverse of
// band_pixel: bands of 8 rows, column by column within a band).
__device__ __forceinline__ uint32_t band_index(uint32_t x, uint32_t y, uint32_t W, uint32_t H) {
    uint32_t band = y / 8u;
    uint32_t rows = min(8u, H - 8u * band);
    return band * 8u * W + x * rows + (y - 8u * band);
}

// The pixels whose samples can fall in the pixel-position rectangle [lo, hi] (pixel p covers
// positions [p - 0.5, p + 0.5)); a > b when none.
__device__ __forceinline__ void pixel_span(float lo, float hi, uint32_t n, int& a, int& b) {
    a = max(0, (int)ceilf(lo - 0.5f));
    b = min((int)n - 1, (int)floorf(hi + 0.5f));
}

__global__ void primary_instance_kernel(const __grid_constant__ DevScene sc, f3 camera,
                                        const __grid_constant__ PrimaryParams v) {
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
    bool ok = inverse3(C, Ci) && inverse3(X, Xi) && finite3(oo) &&
              frobenius(C) * frobenius(Ci) < MAX_PROJECTION_COND;
    PrimaryInstance& I = v.inst[i];
    I.oo[0] = oo.x;
    I.oo[1] = oo.y;
    I.oo[2] = oo.z;
    for (int k = 0; k < 9; ++k) I.ci[k] = ok ? Ci[k] : 0.0;
    double margin = BASE_MARGIN_PX + COND_MARGIN * frobenius(X) * frobenius(Xi) * v.pixel_scale;
    I.margin = margin;
    I.ok = ok && isfinite(margin) ? 1u : 0u;
}

struct P3 {
    double x, y, l;  // C^-1 (p - oo): lambda (ndc.x, ndc.y, 1)
};

__global__ void primary_rect_kernel(const __grid_constant__ DevScene sc, const __grid_constant__ PrimaryParams v,
                                    uint32_t W, uint32_t H) {
    uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t cnt = 0u;
    float4 rect = make_float4(1.0f, 1.0f, 0.0f, 0.0f);
    if (r < v.records) {
        float4 a = sc.tris[3ull * r], b = sc.tris[3ull * r + 1], c = sc.tris[3ull * r + 2];
        const PrimaryInstance& I = v.inst[__float_as_uint(b.w)];
        bool any = false;
        double xlo = 0.0, ylo = 0.0, xhi = 0.0, yhi = 0.0;
        if (!I.ok) {
            any = true;
            xlo = ylo = -4.0;
            xhi = (double)W + 4.0;
            yhi = (double)H + 4.0;
        } else {
            double q[3][3] = {{a.x - I.oo[0], a.y - I.oo[1], a.z - I.oo[2]},
                              {b.x - I.oo[0], b.y - I.oo[1], b.z - I.oo[2]},
                              {c.x - I.oo[0], c.y - I.oo[1], c.z - I.oo[2]}};
            double e1[3] = {q[1][0] - q[0][0], q[1][1] - q[0][1], q[1][2] - q[0][2]};
            double e2[3] = {q[2][0] - q[0][0], q[2][1] - q[0][1], q[2][2] - q[0][2]};
            double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
            // front faces have their normal towards the ray origin: dot(n, oo - p0) > 0
            double facing = -(n[0] * q[0][0] + n[1] * q[0][1] + n[2] * q[0][2]);
            double scale = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]) *
                           sqrt(q[0][0] * q[0][0] + q[0][1] * q[0][1] + q[0][2] * q[0][2]);
            bool back = facing < -BACKFACE_COS * scale;
            if (!back) {
                P3 p[3];
                for (int k = 0; k < 3; ++k) {
                    const double* m = I.ci;
                    p[k].x = m[0] * q[k][0] + m[1] * q[k][1] + m[2] * q[k][2];
                    p[k].y = m[3] * q[k][0] + m[4] * q[k][1] + m[5] * q[k][2];
                    p[k].l = m[6] * q[k][0] + m[7] * q[k][1] + m[8] * q[k][2];
                }
                // clip to lambda >= lambda_clip (Sutherland-Hodgman against one plane)
                P3 poly[4];
                int np = 0;
                const double lc = v.lambda_clip;
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
                if (np > 0) {
                    any = true;
                    xlo = ylo = INFINITY;
                    xhi = yhi = -INFINITY;
                    for (int k = 0; k < np; ++k) {
                        double l = fmax(poly[k].l, lc);
                        double px = (poly[k].x / l + 1.0) * 0.5 * (double)W;
                        double py = (poly[k].y / l + 1.0) * 0.5 * (double)H;
                        xlo = fmin(xlo, px);
                        xhi = fmax(xhi, px);
                        ylo = fmin(ylo, py);
                        yhi = fmax(yhi, py);
                    }
                    if (!(isfinite(xlo) && isfinite(xhi) && isfinite(ylo) && isfinite(yhi))) {
                        xlo = ylo = -4.0;
                        xhi = (double)W + 4.0;
                        yhi = (double)H + 4.0;
                    }
                    xlo -= I.margin;
                    ylo -= I.margin;
                    xhi += I.margin;
                    yhi += I.margin;
                }
            }
        }
        if (any) {
            xlo = fmin(fmax(xlo, -4.0), (double)W + 4.0);
            xhi = fmin(fmax(xhi, -4.0), (double)W + 4.0);
            ylo = fmin(fmax(ylo, -4.0), (double)H + 4.0);
            yhi = fmin(fmax(yhi, -4.0), (double)H + 4.0);
            float4 f = make_float4(__double2float_rd(xlo), __double2float_rd(ylo), __double2float_ru(xhi),
                                   __double2float_ru(yhi));
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
    }
    if (r <= v.records) v.count[r] = cnt;  // count[records] = 0: the exclusive prefix ends with the total
    unsigned long long sum = cnt;
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31u) == 0u && sum) atomicAdd(v.total, sum);
}

__global__ void primary_finish_kernel(const __grid_constant__ PrimaryParams v) {
    *v.ok = *v.total < PAIR_LIMIT ? 1u : 0u;
}

// One thread per pixel-record pair (grid-stride): every sample of the chunk in the pixel whose
// position lies in the record's rectangle is tested against the record.
__global__ void __launch_bounds__(RASTER_BLOCK) primary_raster_kernel(const __grid_constant__ RenderParams p,
                                                                      const __grid_constant__ PrimaryParams v,
                                                                      uint32_t chunk_sample0, uint32_t chunk_spp,
                                                                      const __grid_constant__ XsJump jump) {
    if (*v.ok == 0u) return;
    const tt_constants& c = p.c;
    const DevScene& sc = p.sc;
    const uint32_t W = c.screen_size[0], H = c.screen_size[1];
    const uint64_t WH = (uint64_t)W * H;
    const uint32_t total = v.count[v.records];
    const uint32_t frame_hash = jenkins_hash(c.frame_index);
    const f3 camera = f3{c.camera_position[0], c.camera_position[1], c.camera_position[2]};
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
        uint32_t lo = 0u, hi = v.records;  // count[lo] <= k < count[hi]
        while (hi - lo > 1u) {
            uint32_t mid = (lo + hi) >> 1;
            if (__ldg(v.count + mid) <= k) lo = mid;
            else hi = mid;
        }
        const float4 rect = v.rect[lo];
        int x0, x1, y0, y1;
        pixel_span(rect.x, rect.z, W, x0, x1);
        pixel_span(rect.y, rect.w, H, y0, y1);
        const uint32_t bw = (uint32_t)(x1 - x0 + 1);
        const uint32_t j = k - __ldg(v.count + lo);
        const uint32_t x = (uint32_t)x0 + j % bw, y = (uint32_t)y0 + j / bw;
        const float4 a = __ldg(sc.tris + 3ull * lo), b = __ldg(sc.tris + 3ull * lo + 1), cc = __ldg(sc.tris + 3ull * lo + 2);
        const uint32_t prim = __float_as_uint(a.w), inst = __float_as_uint(b.w);
        const unsigned long long tri = (unsigned long long)(__ldg(sc.tri_base + inst) + prim);
        unsigned long long* dst = v.key + band_index(x, y, W, H);
        uint32_t pg = jenkins_hash((x + y * W) ^ frame_hash);
        if (chunk_sample0) pg = xs_apply(jump, pg);
        for (uint32_t s = 0; s < chunk_spp; ++s, dst += WH) {
            // the draws of pixel_ndc: the sample's generator ends two steps on, at the next sample's
            float ox = random_float(pg);
            float oy = random_float(pg);
            float px = (float)x + (ox - 0.5f), py = (float)y + (oy - 0.5f);
            if (px < rect.x || px > rect.z || py < rect.y || py > rect.w) continue;
            f3 d = camera_ray_direction(c, pixel_ndc_from_draws(x, y, W, H, ox, oy));
            if (!finite3(d)) continue;
            f3 oo, od;
            uint32_t mesh;
            instance_ray(sc, inst, camera, d, oo, od, mesh);
            if (!finite3(od)) continue;
            RayPre rp = ray_precompute(oo, od);
            float t, u, w;
            if (!intersect_triangle(rp, tri_vertex(a), tri_vertex(b), tri_vertex(cc), true, EXTENSION_TMIN,
                                    EXTENSION_TMAX, t, u, w))
                continue;
            unsigned long long key = ((unsigned long long)__float_as_uint(t) << 32) | tri;
            if (key < *dst) atomicMin(dst, key);
        }
    }
}

}  // namespace

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
        primary_instance_kernel<<<(sc.instance_count + 127) / 128, 128, 0, st>>>(sc, camera, v);
    primary_rect_kernel<<<(unsigned)((v.records + 1ull + 255) / 256), 256, 0, st>>>(sc, v, p.c.screen_size[0],
                                                                                   p.c.screen_size[1]);
    check_cuda(cudaGetLastError(), "primary bounds");
    exclusive_scan_u32(v.count, (uint64_t)v.records + 1, st);
    primary_finish_kernel<<<1, 1, 0, st>>>(v);
    check_cuda(cudaGetLastError(), "primary finish");
}

void primary_chunk(const RenderParams& p, const PrimaryParams& v, const WfParams& w, cudaStream_t st) {
    uint64_t WH = (uint64_t)p.c.screen_size[0] * p.c.screen_size[1];
    check_cuda(cudaMemsetAsync(v.key, 0xff, 8ull * WH * w.chunk_spp, st), "memset");
    if (v.records)
        primary_raster_kernel<<<v.raster_blocks, RASTER_BLOCK, 0, st>>>(p, v, w.chunk_sample0, w.chunk_spp,
                                                                        w.chunk_jump);
    check_cuda(cudaGetLastError(), "primary raster");
}

}  // namespace tt
