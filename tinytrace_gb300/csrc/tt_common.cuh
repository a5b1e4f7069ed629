// Device-side vector algebra, deterministic elementary functions, the RNG, the scene byte
// layouts and light sampling of the tinytrace rendering hot path (sm_103a).
//
// Determinism contract: this file is compiled with -fmad=false and without fast math, so
// every float expression below is evaluated as written with IEEE-754 single-precision
// rounding (division and sqrt correctly rounded).  Fused multiply-adds appear only where
// they are written explicitly (__fmaf_rn).  The elementary functions are implemented here
// from published methods rather than taken from the CUDA math library, so that results are
// bit-identical on any IEEE-754 machine that evaluates the same operations:
//   * sin/cos: Cody & Waite additive reduction by pi/2 (three-part constant), Maclaurin
//     series of sin and cos on [-pi/4, pi/4];
//   * exp: Cody & Waite reduction by ln 2, Maclaurin series through r^7, two-step scaling;
//   * log: exponent/mantissa split, log(m) = 2 atanh((m-1)/(m+1)) series through s^11;
//   * acos: pi/2 - asin(x) for |x| <= 1/2, 2 asin(sqrt((1-x)/2)) beyond, Maclaurin series of
//     asin through y^21.
#pragma once

#include <cstdint>

#include "../../include/tinytrace_cuda.h"

#define TT_HD __device__ __forceinline__

namespace tt {

struct f2 {
    float x, y;
};
struct f3 {
    float x, y, z;
};

TT_HD f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
TT_HD f3 splat(float s) { return f3{s, s, s}; }
TT_HD f3 operator+(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
TT_HD f3 operator-(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
TT_HD f3 operator*(f3 a, f3 b) { return f3{a.x * b.x, a.y * b.y, a.z * b.z}; }
TT_HD f3 operator/(f3 a, f3 b) { return f3{a.x / b.x, a.y / b.y, a.z / b.z}; }
TT_HD f3 operator*(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
TT_HD f3 operator*(float s, f3 a) { return f3{s * a.x, s * a.y, s * a.z}; }
TT_HD f3 operator/(f3 a, float s) { return f3{a.x / s, a.y / s, a.z / s}; }
TT_HD f3 operator/(float s, f3 a) { return f3{s / a.x, s / a.y, s / a.z}; }
TT_HD f3 operator-(f3 a) { return f3{-a.x, -a.y, -a.z}; }
TT_HD f3 operator-(float s, f3 a) { return f3{s - a.x, s - a.y, s - a.z}; }
TT_HD f3& operator+=(f3& a, f3 b) { a = a + b; return a; }
TT_HD f3& operator*=(f3& a, f3 b) { a = a * b; return a; }

TT_HD float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
TT_HD f3 cross(f3 a, f3 b) {
    return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
TT_HD float length(f3 v) { return sqrtf(dot(v, v)); }
TT_HD f3 normalize(f3 v) {
    float inv = 1.0f / sqrtf(dot(v, v));
    return v * inv;
}
TT_HD float fmn(float a, float b) { return fminf(a, b); }
TT_HD float fmx(float a, float b) { return fmaxf(a, b); }
TT_HD float clampf(float v, float lo, float hi) { return fmn(fmx(v, lo), hi); }
TT_HD float saturate(float v) { return clampf(v, 0.0f, 1.0f); }
TT_HD float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
TT_HD f3 mix3(f3 a, f3 b, float t) { return a * (1.0f - t) + b * t; }
TT_HD float signf(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
TT_HD f3 reflect(f3 i, f3 n) { return i - (2.0f * dot(n, i)) * n; }
TT_HD f3 xyz4(float4 v) { return f3{v.x, v.y, v.z}; }

// ---------------------------------------------------------------- elementary functions
constexpr float PIO2_1 = 1.5707963705062866f;
constexpr float PIO2_2 = -4.371138828673793e-08f;
constexpr float PIO2_3 = -1.7151245100058819e-15f;
constexpr float TWO_OVER_PI = 0.6366197466850281f;
constexpr float PI_1 = 3.1415927410125732f;
constexpr float PI_2 = -8.742277657347586e-08f;
constexpr float LN2_HI = 0.693145751953125f;
constexpr float LN2_LO = 1.428606765330187e-06f;
constexpr float LOG2E = 1.4426950216293335f;

TT_HD void tsincos(float x, float* s, float* c) {
    if (!(fabsf(x) <= 1.0e7f)) {
        if (x != x || isinf(x)) {
            *s = *c = __int_as_float(0x7fffffff);
            return;
        }
        x = fmodf(x, 6.2831854820251465f);
    }
    float j = rintf(x * TWO_OVER_PI);
    float r = __fmaf_rn(-j, PIO2_1, x);
    r = __fmaf_rn(-j, PIO2_2, r);
    r = __fmaf_rn(-j, PIO2_3, r);
    float r2 = r * r;
    float ps = __fmaf_rn(r2, 2.7557319223985893e-06f, -0.00019841270113829523f);
    ps = __fmaf_rn(r2, ps, 0.008333333767950535f);
    ps = __fmaf_rn(r2, ps, -0.1666666716337204f);
    float sn = __fmaf_rn(r * r2, ps, r);
    float pc = __fmaf_rn(r2, -2.755731922398589e-07f, 2.4801587642286904e-05f);
    pc = __fmaf_rn(r2, pc, -0.0013888889225199819f);
    pc = __fmaf_rn(r2, pc, 0.0416666679084301f);
    pc = __fmaf_rn(r2, pc, -0.5f);
    float cs = __fmaf_rn(r2, pc, 1.0f);
    int q = ((int)j) & 3;
    float so = (q & 1) ? cs : sn;
    float co = (q & 1) ? sn : cs;
    if (q == 2 || q == 3) so = -so;
    if (q == 1 || q == 2) co = -co;
    *s = so;
    *c = co;
}

TT_HD float texp(float x) {
    if (x != x) return x;
    if (x > 88.72283935546875f) return __int_as_float(0x7f800000);
    if (x < -103.972084045410f) return 0.0f;
    float k = rintf(x * LOG2E);
    float r = __fmaf_rn(-k, LN2_HI, x);
    r = __fmaf_rn(-k, LN2_LO, r);
    float p = __fmaf_rn(r, 0.00019841270113829523f, 0.0013888889225199819f);
    p = __fmaf_rn(r, p, 0.008333333767950535f);
    p = __fmaf_rn(r, p, 0.0416666679084301f);
    p = __fmaf_rn(r, p, 0.1666666716337204f);
    p = __fmaf_rn(r, p, 0.5f);
    p = __fmaf_rn(r, p, 1.0f);
    p = __fmaf_rn(r, p, 1.0f);
    int ki = (int)k;
    int k1 = ki / 2;
    int k2 = ki - k1;
    float s1 = __int_as_float((k1 + 127) << 23);
    float s2 = __int_as_float((k2 + 127) << 23);
    return (p * s1) * s2;
}

TT_HD float tlog(float x) {
    if (x != x) return x;
    if (x < 0.0f) return __int_as_float(0x7fffffff);
    if (x == 0.0f) return __int_as_float(0xff800000);
    if (isinf(x)) return x;
    int e = 0;
    uint32_t b = __float_as_uint(x);
    if (b < 0x00800000u) {
        x = x * 8388608.0f;
        b = __float_as_uint(x);
        e = -23;
    }
    e += (int)((b >> 23) & 0xffu) - 127;
    float m = __uint_as_float((b & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421353816986083984f) {
        m = m * 0.5f;
        e += 1;
    }
    float s = (m - 1.0f) / (m + 1.0f);
    float z = s * s;
    float p = __fmaf_rn(z, 0.09090909090909091f, 0.1111111119389534f);
    p = __fmaf_rn(z, p, 0.1428571492433548f);
    p = __fmaf_rn(z, p, 0.2000000029802322f);
    p = __fmaf_rn(z, p, 0.3333333432674408f);
    float s2 = 2.0f * s;
    float lm = __fmaf_rn(s2 * z, p, s2);
    float fe = (float)e;
    return __fmaf_rn(fe, LN2_HI, __fmaf_rn(fe, LN2_LO, lm));
}

TT_HD float asin_small(float y) {
    float z = y * y;
    float p = __fmaf_rn(z, 0.008390335366129875f, 0.009761609137058258f);
    p = __fmaf_rn(z, p, 0.01155180111527443f);
    p = __fmaf_rn(z, p, 0.013964843936264515f);
    p = __fmaf_rn(z, p, 0.017352763563394547f);
    p = __fmaf_rn(z, p, 0.022372158244252205f);
    p = __fmaf_rn(z, p, 0.0303819440305233f);
    p = __fmaf_rn(z, p, 0.0446428582072258f);
    p = __fmaf_rn(z, p, 0.07500000298023224f);
    p = __fmaf_rn(z, p, 0.1666666716337204f);
    return __fmaf_rn(y * z, p, y);
}

TT_HD float tacos(float x) {
    if (x != x) return x;
    float ax = fabsf(x);
    if (ax > 1.0f) return __int_as_float(0x7fffffff);
    if (ax <= 0.5f) return (PIO2_1 - asin_small(x)) + PIO2_2;
    if (x > 0.0f) {
        float y = sqrtf((1.0f - x) * 0.5f);
        return 2.0f * asin_small(y);
    }
    float y = sqrtf((1.0f + x) * 0.5f);
    return (PI_1 - 2.0f * asin_small(y)) + PI_2;
}

// atan(t) for 0 <= t <= 1: two half-angle steps atan(t) = 2 atan(t / (1 + sqrt(1 + t^2)))
// bring the argument below tan(pi/16), then the Maclaurin series of atan through r^15.
TT_HD float atan_unit(float t) {
    float r = t / (1.0f + sqrtf(__fmaf_rn(t, t, 1.0f)));
    r = r / (1.0f + sqrtf(__fmaf_rn(r, r, 1.0f)));
    float z = r * r;
    float p = __fmaf_rn(z, -0.0666666666666667f, 0.0769230769230769f);
    p = __fmaf_rn(z, p, -0.0909090909090909f);
    p = __fmaf_rn(z, p, 0.1111111111111111f);
    p = __fmaf_rn(z, p, -0.1428571428571429f);
    p = __fmaf_rn(z, p, 0.2f);
    p = __fmaf_rn(z, p, -0.3333333333333333f);
    return 4.0f * __fmaf_rn(r * z, p, r);
}

// atan2(y, x) by octant: atan_unit of min/max, reflected about pi/4 and pi/2, signed by y.
TT_HD float tatan2(float y, float x) {
    if (x != x || y != y) return x + y;
    float ax = fabsf(x), ay = fabsf(y);
    float a;
    if (ax == 0.0f && ay == 0.0f) {
        a = 0.0f;
    } else if (ax == ay) {
        a = 0.785398185253143310546875f;  // pi/4, also for two infinities
    } else if (ay > ax) {
        a = (PIO2_1 - atan_unit(ax / ay)) + PIO2_2;
    } else {
        a = atan_unit(ay / ax);
    }
    if (signbit(x)) a = (PI_1 - a) + PI_2;
    return signbit(y) ? -a : a;
}

// ---------------------------------------------------------------- constants
constexpr float PI = 3.1415926535897932f;
constexpr float TAU = 6.283185307179586f;
constexpr float INVERSE_PI = 1.0f / PI;
constexpr uint32_t LIGHT_SAMPLING_NEE = 2u;

// ---------------------------------------------------------------- RNG (random.glsl:4-50)
TT_HD uint32_t jenkins_hash(uint32_t x) {
    x += x << 10;
    x ^= x >> 6;
    x += x << 3;
    x ^= x >> 11;
    x += x << 15;
    return x;
}
TT_HD uint32_t xor_shift(uint32_t& s) {
    s ^= s << 13;
    s ^= s >> 17;
    s ^= s << 5;
    return s;
}
// Jump-ahead of xor_shift: each step is linear over GF(2), so k steps map a state x to M^k x
// for one 32 x 32 bit matrix M.  A matrix is stored as its 32 columns (the images of 1 << j),
// and applying it XORs the columns of the set bits of x: k steps for any k in 32 selects.
struct XsJump {
    uint32_t col[32];
};
__host__ __device__ constexpr uint32_t xs_step(uint32_t s) {
    s ^= s << 13;
    s ^= s >> 17;
    s ^= s << 5;
    return s;
}
__host__ __device__ constexpr uint32_t xs_apply(const XsJump& m, uint32_t x) {
    uint32_t acc = 0u;
    for (int j = 0; j < 32; ++j) acc ^= m.col[j] & (0u - ((x >> j) & 1u));
    return acc;
}
__host__ __device__ constexpr XsJump xs_compose(const XsJump& a, const XsJump& b) {  // a after b
    XsJump r{};
    for (int j = 0; j < 32; ++j) r.col[j] = xs_apply(a, b.col[j]);
    return r;
}
__host__ __device__ constexpr XsJump xs_power(uint64_t k) {  // M^k by squaring
    XsJump base{}, r{};
    for (int j = 0; j < 32; ++j) {
        base.col[j] = xs_step(1u << j);
        r.col[j] = 1u << j;
    }
    while (k) {
        if (k & 1u) r = xs_compose(base, r);
        base = xs_compose(base, base);
        k >>= 1;
    }
    return r;
}

// random_float split in two: the 23 mantissa bits a step draws, and the float in [0, 1) they give
TT_HD uint32_t random_mantissa(uint32_t& s) { return xor_shift(s) >> 9; }
TT_HD float mantissa_float(uint32_t m) { return __uint_as_float(0x3f800000u | m) - 1.0f; }
TT_HD float random_float(uint32_t& s) { return mantissa_float(random_mantissa(s)); }
TT_HD f2 random_vec2(uint32_t& s) {
    float a = random_float(s);
    float b = random_float(s);
    return f2{a, b};
}

// ---------------------------------------------------------------- sample.glsl:7-30
TT_HD f3 sample_triangle(f2 r) {
    r.x = r.x / 2.0f;
    r.y = r.y / 2.0f;
    float offset = r.y - r.x;
    if (offset > 0.0f) r.y += offset;
    else r.x -= offset;
    return f3{r.x, r.y, 1.0f - r.x - r.y};
}
TT_HD f3 cosine_hemisphere_sample(f2 r) {
    float rr = sqrtf(r.x);
    float theta = 2.0f * PI * r.y;
    float s, c;
    tsincos(theta, &s, &c);
    float x = rr * c, y = rr * s;
    float z = sqrtf(fmx(0.0f, 1.0f - x * x - y * y));
    return f3{x, y, z};
}
TT_HD float cosine_hemisphere_density(float nds) {
    if (nds <= 1e-6f) return 1e-6f / PI;
    return nds / PI;
}

// ---------------------------------------------------------------- scene data
// Instance transforms, column-major (src/scene.rs:236-246).
TT_HD f3 mat43_point(const float* m, f3 p) {
    return f3{m[0] * p.x + m[4] * p.y + m[8] * p.z + m[12] * 1.0f,
              m[1] * p.x + m[5] * p.y + m[9] * p.z + m[13] * 1.0f,
              m[2] * p.x + m[6] * p.y + m[10] * p.z + m[14] * 1.0f};
}
TT_HD f3 mat3_vec(const float* m, f3 v) {
    return f3{m[0] * v.x + m[4] * v.y + m[8] * v.z, m[1] * v.x + m[5] * v.y + m[9] * v.z,
              m[2] * v.x + m[6] * v.y + m[10] * v.z};
}
TT_HD float4 mat4_mul(const float* m, float4 v) {
    float4 r;
    r.x = m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w;
    r.y = m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w;
    r.z = m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w;
    r.w = m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w;
    return r;
}
TT_HD float dequant_snorm16(int v) { return (float)v / 32767.0f; }

// octahedron.glsl:16-24
TT_HD f3 octahedron_decode(f2 o) {
    f2 s = f2{o.x * 2.0f - 1.0f, o.y * 2.0f - 1.0f};
    f3 n = f3{s.x, s.y, 1.0f - fabsf(s.x) - fabsf(s.y)};
    float t = clampf(-n.z, 0.0f, 1.0f);
    n.x += n.x >= 0.0f ? -t : t;
    n.y += n.y >= 0.0f ? -t : t;
    return normalize(n);
}
TT_HD float dequant_unorm(uint32_t bits, uint32_t value) {
    return (float)value / (float)((1u << bits) - 1u);
}
struct TangentFrame {
    f3 normal, tangent;
    float bitangent_sign;
};
// scene.glsl:29-64
TT_HD TangentFrame decode_tangent_frame(uint32_t enc) {
    TangentFrame tf;
    f2 uv = f2{dequant_unorm(10, enc & 0x3ffu), dequant_unorm(10, (enc >> 10) & 0x3ffu)};
    tf.normal = octahedron_decode(uv);
    f3 ortho = fabsf(tf.normal.x) > fabsf(tf.normal.z) ? f3{-tf.normal.y, tf.normal.x, 0.0f}
                                                         : f3{0.0f, -tf.normal.z, tf.normal.y};
    float angle = dequant_unorm(11, (enc >> 20) & 0x7ffu) * TAU;
    float s, c;
    tsincos(angle, &s, &c);
    tf.tangent = ortho * c + cross(tf.normal, ortho) * s;
    tf.bitangent_sign = (enc >> 31) == 1u ? 1.0f : -1.0f;
    return tf;
}

struct Basis {
    f3 normal, tangent, bitangent;
};
TT_HD f3 transform_to_basis(const Basis& b, f3 d) {
    return normalize(d.x * b.tangent + d.y * b.bitangent + d.z * b.normal);
}
TT_HD f3 transform_from_basis(const Basis& b, f3 d) {
    return normalize(f3{dot(d, b.tangent), dot(d, b.bitangent), dot(d, b.normal)});
}
TT_HD f3 gram_schmidt(f3 n, f3 t) { return normalize(t - n * dot(n, t)); }
TT_HD f3 interp3(f3 b, f3 a0, f3 a1, f3 a2) { return b.x * a0 + b.y * a1 + b.z * a2; }

}  // namespace tt
