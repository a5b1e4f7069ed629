// TEST INFRASTRUCTURE — the CPU oracle for the tinytrace rendering hot path.
// Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may load this code.
// It is the checker, never the product.
//
// Vector helpers and deterministic elementary functions for the oracle.
//
// Every vector operation has one fixed evaluation order (written out below), so that an
// independent CUDA implementation compiled with contraction disabled (-fmad=false) produces
// the same IEEE-754 single-precision bits.  The oracle is compiled with
// -ffp-contract=off -fno-fast-math; fmaf() below is an explicit, correctly rounded fused
// multiply-add on both x86-64 (glibc) and aarch64 (fmadd).
//
// The elementary functions follow published methods, not any vendor library:
//   * sin/cos: Cody & Waite additive range reduction by pi/2 with a three-part constant
//     ("Software Manual for the Elementary Functions", 1980), then the Maclaurin series of
//     sin and cos on [-pi/4, pi/4] (truncation < 3e-9 relative).
//   * exp: Cody & Waite reduction by ln 2 (two-part constant), Maclaurin series of e^r on
//     |r| <= ln2/2 through r^7, exact scaling by 2^k in two steps.
//   * log: mantissa/exponent split with m in [sqrt(1/2), sqrt(2)), then
//     log(m) = 2 atanh(s), s = (m-1)/(m+1), atanh series through s^11.
//   * acos: acos(x) = pi/2 - asin(x) for |x| <= 1/2 and the half-angle identity
//     acos(x) = 2 asin(sqrt((1-x)/2)) beyond, with the Maclaurin series of asin through y^21.
// GLSL pow(s, 3.0) (the only pow on the path, src/material/diffuse_brdf.glsl:14) is s*s*s.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace ref {

struct v2 {
    float x, y;
};
struct v3 {
    float x, y, z;
};
struct v4 {
    float x, y, z, w;
};

inline v2 mk2(float x, float y) { return v2{x, y}; }
inline v3 mk3(float x, float y, float z) { return v3{x, y, z}; }
inline v3 splat3(float s) { return v3{s, s, s}; }
inline v3 xyz(const v4& v) { return v3{v.x, v.y, v.z}; }

inline v3 operator+(v3 a, v3 b) { return v3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline v3 operator-(v3 a, v3 b) { return v3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline v3 operator*(v3 a, v3 b) { return v3{a.x * b.x, a.y * b.y, a.z * b.z}; }
inline v3 operator/(v3 a, v3 b) { return v3{a.x / b.x, a.y / b.y, a.z / b.z}; }
inline v3 operator*(v3 a, float s) { return v3{a.x * s, a.y * s, a.z * s}; }
inline v3 operator*(float s, v3 a) { return v3{s * a.x, s * a.y, s * a.z}; }
inline v3 operator/(v3 a, float s) { return v3{a.x / s, a.y / s, a.z / s}; }
inline v3 operator-(v3 a) { return v3{-a.x, -a.y, -a.z}; }
inline v3 operator-(float s, v3 a) { return v3{s - a.x, s - a.y, s - a.z}; }
inline v3 operator/(float s, v3 a) { return v3{s / a.x, s / a.y, s / a.z}; }
inline v3& operator+=(v3& a, v3 b) { a = a + b; return a; }
inline v3& operator*=(v3& a, v3 b) { a = a * b; return a; }
inline v2 operator+(v2 a, v2 b) { return v2{a.x + b.x, a.y + b.y}; }
inline v2 operator-(v2 a, v2 b) { return v2{a.x - b.x, a.y - b.y}; }
inline v2 operator*(v2 a, v2 b) { return v2{a.x * b.x, a.y * b.y}; }
inline v2 operator*(float s, v2 a) { return v2{s * a.x, s * a.y}; }
inline v2 operator/(v2 a, v2 b) { return v2{a.x / b.x, a.y / b.y}; }

inline float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot2(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }
inline v3 cross(v3 a, v3 b) {
    return v3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float length(v3 v) { return std::sqrt(dot(v, v)); }
// normalize(v) = v * (1 / length(v)).
inline v3 normalize(v3 v) {
    float inv = 1.0f / std::sqrt(dot(v, v));
    return v * inv;
}
// GLSL min/max/clamp use fmin/fmax semantics (a NaN operand yields the other operand).
inline float fmn(float a, float b) { return std::fmin(a, b); }
inline float fmx(float a, float b) { return std::fmax(a, b); }
inline float clampf(float v, float lo, float hi) { return fmn(fmx(v, lo), hi); }
inline float saturate(float v) { return clampf(v, 0.0f, 1.0f); }
inline v3 fmx3(v3 a, float b) { return v3{fmx(a.x, b), fmx(a.y, b), fmx(a.z, b)}; }
// mix(a, b, t) = a * (1 - t) + b * t  (GLSL definition).
inline float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
inline v3 mix3(v3 a, v3 b, float t) { return a * (1.0f - t) + b * t; }
inline float signf(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
// reflect(I, N) = I - (2 * dot(N, I)) * N
inline v3 reflect(v3 i, v3 n) { return i - (2.0f * dot(n, i)) * n; }

inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float bitsf(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// IEEE binary16 -> binary32 (exact).
inline float half_to_float(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t exp = (h >> 10) & 0x1fu;
    uint32_t man = h & 0x3ffu;
    if (exp == 0) {
        if (man == 0) return bitsf(sign);
        // subnormal half: man * 2^-24
        float v = (float)man * 5.9604644775390625e-08f;
        return sign ? -v : v;
    }
    if (exp == 31) return bitsf(sign | 0x7f800000u | (man << 13));
    return bitsf(sign | ((exp + 112u) << 23) | (man << 13));
}

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

inline void tsincos(float x, float* s, float* c) {
    if (!(std::fabs(x) <= 1.0e7f)) {
        if (x != x || std::isinf(x)) {
            *s = *c = NAN;
            return;
        }
        x = std::fmod(x, 6.2831854820251465f);
    }
    float j = std::rint(x * TWO_OVER_PI);
    float r = std::fmaf(-j, PIO2_1, x);
    r = std::fmaf(-j, PIO2_2, r);
    r = std::fmaf(-j, PIO2_3, r);
    float r2 = r * r;
    // sin(r) = r + r^3 (-1/6 + r^2 (1/120 + r^2 (-1/5040 + r^2 / 362880)))
    float ps = std::fmaf(r2, 2.7557319223985893e-06f, -0.00019841270113829523f);
    ps = std::fmaf(r2, ps, 0.008333333767950535f);
    ps = std::fmaf(r2, ps, -0.1666666716337204f);
    float sn = std::fmaf(r * r2, ps, r);
    // cos(r) = 1 + r^2 (-1/2 + r^2 (1/24 + r^2 (-1/720 + r^2 (1/40320 - r^2/3628800))))
    float pc = std::fmaf(r2, -2.755731922398589e-07f, 2.4801587642286904e-05f);
    pc = std::fmaf(r2, pc, -0.0013888889225199819f);
    pc = std::fmaf(r2, pc, 0.0416666679084301f);
    pc = std::fmaf(r2, pc, -0.5f);
    float cs = std::fmaf(r2, pc, 1.0f);
    int q = ((int)j) & 3;
    float so, co;
    switch (q) {
        case 0: so = sn; co = cs; break;
        case 1: so = cs; co = -sn; break;
        case 2: so = -sn; co = -cs; break;
        default: so = -cs; co = sn; break;
    }
    *s = so;
    *c = co;
}
inline float tsin(float x) { float s, c; tsincos(x, &s, &c); return s; }
inline float tcos(float x) { float s, c; tsincos(x, &s, &c); return c; }

inline float texp(float x) {
    if (x != x) return x;
    if (x > 88.72283935546875f) return INFINITY;
    if (x < -103.972084045410f) return 0.0f;
    float k = std::rint(x * LOG2E);
    float r = std::fmaf(-k, LN2_HI, x);
    r = std::fmaf(-k, LN2_LO, r);
    float p = std::fmaf(r, 0.00019841270113829523f, 0.0013888889225199819f);
    p = std::fmaf(r, p, 0.008333333767950535f);
    p = std::fmaf(r, p, 0.0416666679084301f);
    p = std::fmaf(r, p, 0.1666666716337204f);
    p = std::fmaf(r, p, 0.5f);
    p = std::fmaf(r, p, 1.0f);
    p = std::fmaf(r, p, 1.0f);
    int ki = (int)k;
    int k1 = ki / 2;
    int k2 = ki - k1;
    float s1 = bitsf((uint32_t)(k1 + 127) << 23);
    float s2 = bitsf((uint32_t)(k2 + 127) << 23);
    return (p * s1) * s2;
}

inline float tlog(float x) {
    if (x != x) return x;
    if (x < 0.0f) return NAN;
    if (x == 0.0f) return -INFINITY;
    if (std::isinf(x)) return x;
    int e = 0;
    uint32_t b = fbits(x);
    if (b < 0x00800000u) {
        x = x * 8388608.0f;
        b = fbits(x);
        e = -23;
    }
    e += (int)((b >> 23) & 0xffu) - 127;
    float m = bitsf((b & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421353816986083984f) {
        m = m * 0.5f;
        e += 1;
    }
    float s = (m - 1.0f) / (m + 1.0f);
    float z = s * s;
    float p = std::fmaf(z, 0.09090909090909091f, 0.1111111119389534f);
    p = std::fmaf(z, p, 0.1428571492433548f);
    p = std::fmaf(z, p, 0.2000000029802322f);
    p = std::fmaf(z, p, 0.3333333432674408f);
    float s2 = 2.0f * s;
    float lm = std::fmaf(s2 * z, p, s2);
    float fe = (float)e;
    return std::fmaf(fe, LN2_HI, std::fmaf(fe, LN2_LO, lm));
}
inline float tlog2(float x) { return tlog(x) * LOG2E; }

// asin(y) for 0 <= |y| <= 1/2: y + y^3 * P(y^2), P = Maclaurin coefficients c1..c10.
inline float asin_small(float y) {
    float z = y * y;
    float p = std::fmaf(z, 0.008390335366129875f, 0.009761609137058258f);
    p = std::fmaf(z, p, 0.01155180111527443f);
    p = std::fmaf(z, p, 0.013964843936264515f);
    p = std::fmaf(z, p, 0.017352763563394547f);
    p = std::fmaf(z, p, 0.022372158244252205f);
    p = std::fmaf(z, p, 0.0303819440305233f);
    p = std::fmaf(z, p, 0.0446428582072258f);
    p = std::fmaf(z, p, 0.07500000298023224f);
    p = std::fmaf(z, p, 0.1666666716337204f);
    return std::fmaf(y * z, p, y);
}

inline float tacos(float x) {
    if (x != x) return x;
    float ax = std::fabs(x);
    if (ax > 1.0f) return NAN;
    if (ax <= 0.5f) return (PIO2_1 - asin_small(x)) + PIO2_2;
    if (x > 0.0f) {
        float y = std::sqrt((1.0f - x) * 0.5f);
        return 2.0f * asin_small(y);
    }
    float y = std::sqrt((1.0f + x) * 0.5f);
    return (PI_1 - 2.0f * asin_small(y)) + PI_2;
}

// atan(t) for 0 <= t <= 1: two half-angle steps atan(t) = 2 atan(t / (1 + sqrt(1 + t^2)))
// bring the argument below tan(pi/16), then the Maclaurin series of atan through r^15.
inline float atan_unit(float t) {
    float r = t / (1.0f + std::sqrt(std::fmaf(t, t, 1.0f)));
    r = r / (1.0f + std::sqrt(std::fmaf(r, r, 1.0f)));
    float z = r * r;
    float p = std::fmaf(z, -0.0666666666666667f, 0.0769230769230769f);
    p = std::fmaf(z, p, -0.0909090909090909f);
    p = std::fmaf(z, p, 0.1111111111111111f);
    p = std::fmaf(z, p, -0.1428571428571429f);
    p = std::fmaf(z, p, 0.2f);
    p = std::fmaf(z, p, -0.3333333333333333f);
    return 4.0f * std::fmaf(r * z, p, r);
}

// atan2(y, x) by octant: atan_unit of min/max, reflected about pi/4 and pi/2, signed by y.
inline float tatan2(float y, float x) {
    if (x != x || y != y) return x + y;
    float ax = std::fabs(x), ay = std::fabs(y);
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
    if (std::signbit(x)) a = (PI_1 - a) + PI_2;
    return std::signbit(y) ? -a : a;
}

// IEEE binary32 -> binary16, round to nearest even (f16::from_f32 of the half crate).
inline uint16_t float_to_half(float f) {
    uint32_t u = fbits(f);
    uint16_t sign = (uint16_t)((u >> 16) & 0x8000u);
    uint32_t a = u & 0x7fffffffu;
    if (a > 0x7f800000u) return sign | 0x7e00u;   // NaN
    if (a >= 0x47800000u) return sign | 0x7c00u;  // >= 65536 (and infinity)
    if (a < 0x38800000u) {                        // below 2^-14: subnormal half or zero
        float v = bitsf(a) * 16777216.0f;          // in units of 2^-24, exact
        float r = (v + 12582912.0f) - 12582912.0f;  // round to an integer, ties to even
        return sign | (uint16_t)r;
    }
    uint32_t h = (a >> 13) - (112u << 10);
    uint32_t rem = a & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h += 1u;
    return sign | (uint16_t)h;
}

}  // namespace ref
