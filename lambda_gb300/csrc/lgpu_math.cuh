/*
 * Host/device maths for the path tracer: float3 helpers with the reference's operation order
 * (src/maths/vec3.h, maths.h), std::min/std::max semantics (NaN handling matters for parity),
 * the spectrum value type, and the spectral tables in constant memory.
 */
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include "lgpu_rng.h"
#include "lgpu_scene.h"
#include "spectral_tables.h"

#define HD __host__ __device__ __forceinline__

namespace lg {

#define LG_PI 3.14159265358979323846f
static constexpr float PI = 3.14159265358979323846f;
static constexpr float PI2 = 2.0f * 3.14159265358979323846f;
static constexpr float INV_PI = 1.0f / 3.14159265358979323846f;
static constexpr float INV_PI2 = 1.0f / (2.0f * 3.14159265358979323846f);
static constexpr float INV_PI4 = 1.0f / (4.0f * 3.14159265358979323846f);
static constexpr float SURFACE_EPSILON = 1e-5f;
static constexpr float HERO_RANGE = 340.0f;

HD float bits_to_float(int v) {
    union { int i; float f; } u;
    u.i = v;
    return u.f;
}
HD int float_to_bits(float f) {
    union { float f; int i; } u;
    u.f = f;
    return u.i;
}
HD float finf() { return bits_to_float(0x7f800000); }
HD float fmaxreal() { return 3.402823466e+38f; }
/* std::max / std::min exactly: the first argument's NaN propagates. */
HD float smax(float a, float b) { return (a < b) ? b : a; }
HD float smin(float a, float b) { return (b < a) ? b : a; }
HD float clampr(float v, float lo, float hi) { return smax(smin(v, hi), lo); }
HD float lerpf(float a, float b, float r) { return a + (b - a) * r; }
/* Separately rounded multiply / add: no FMA contraction, so sensitive expressions (noise hashes
 * that feed sin() at large arguments) round exactly like the CPU restatement. */
#if defined(__CUDA_ARCH__)
HD float mul_rn(float a, float b) { return __fmul_rn(a, b); }
HD float add_rn(float a, float b) { return __fadd_rn(a, b); }
#else
HD float mul_rn(float a, float b) { return a * b; }
HD float add_rn(float a, float b) { return a + b; }
#endif
HD float fractf(float r) { return r - floorf(r); }

HD float3 mk(float x, float y, float z) { return make_float3(x, y, z); }
HD float3 operator+(float3 a, float3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
HD float3 operator-(float3 a, float3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
HD float3 operator*(float3 a, float3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
HD float3 operator*(float3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
HD float3 operator-(float3 a) { return a * -1.0f; }
HD float3 divs(float3 a, float s) { const float inv = 1.0f / s; return mk(a.x * inv, a.y * inv, a.z * inv); }
HD float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
HD float3 cross(float3 a, float3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
HD float mag(float3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
HD float3 normalised(float3 a) { return divs(a, mag(a)); }
HD float distsq(float3 a, float3 b) { const float3 d = b - a; return d.x * d.x + d.y * d.y + d.z * d.z; }
HD float comp(float3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
HD float3 to_local(float3 v, float3 t, float3 n, float3 bt) { return mk(dot(t, v), dot(n, v), dot(bt, v)); }
HD float3 to_world(float3 v, float3 t, float3 n, float3 bt) {
    return mk(t.x * v.x + n.x * v.y + bt.x * v.z, t.y * v.x + n.y * v.y + bt.y * v.z, t.z * v.x + n.z * v.y + bt.z * v.z);
}
HD float3 spherical_dir(float s, float c, float phi) { return mk(s * cosf(phi), c, s * sinf(phi)); }
HD float spherical_theta(float3 v) { return acosf(smax(smin(v.y, 1.0f), -1.0f)); }
HD float spherical_phi(float3 v) {
    const float p = atan2f(v.z, v.x);
    return (p < 0) ? (float)((double)p + 3.14159265359 * 2.) : p;
}
HD float3 mul_cm(const float *m, float3 v) {
    return mk(m[0] * v.x + m[3] * v.y + m[6] * v.z, m[1] * v.x + m[4] * v.y + m[7] * v.z, m[2] * v.x + m[5] * v.y + m[8] * v.z);
}
HD float3 f3(float4 a) { return mk(a.x, a.y, a.z); }

/* maths::FindInterval over a sorted float array (src/maths/maths.h:77-90): predicate a[i] <= u. */
HD int find_interval(const float *a, int size, float u) {
    int first = 0, len = size;
    while (len > 0) {
        const int half = len >> 1, middle = first + half;
        if (a[middle] <= u) { first = middle + 1; len -= half + 1; }
        else len = half;
    }
    int r = first - 1;
    r = r < size - 2 ? r : size - 2;
    return r > 0 ? r : 0;
}

/* float -> unsigned as x86-64 code converts it (64-bit truncation, low 32 bits). */
HD uint32_t to_unsigned(float x) {
    if (!(x == x) || fabsf(x) >= 9.2e18f) return 0u;
    return (uint32_t)(uint64_t)(int64_t)x;
}

/* ------------------------------------------------------------------ spectrum */
template <int NS>
struct Spec {
    float c[4];
    HD Spec() { c[0] = c[1] = c[2] = c[3] = 0.f; }
    HD explicit Spec(float v) {
#pragma unroll
        for (int i = 0; i < 4; ++i) c[i] = (i < NS) ? v : 0.f;
    }
    HD static Spec from4(float4 v) { Spec s; s.c[0] = v.x; s.c[1] = v.y; s.c[2] = v.z; s.c[3] = NS == 4 ? v.w : 0.f; return s; }
    HD float4 as4() const { return make_float4(c[0], c[1], c[2], c[3]); }
#define LG_SPEC_BIN(OP)                                                        \
    HD Spec operator OP(const Spec &o) const {                                  \
        Spec r;                                                                \
        _Pragma("unroll") for (int i = 0; i < NS; ++i) r.c[i] = c[i] OP o.c[i]; \
        return r;                                                              \
    }
    LG_SPEC_BIN(+)
    LG_SPEC_BIN(-)
    LG_SPEC_BIN(*)
    LG_SPEC_BIN(/)
#undef LG_SPEC_BIN
    HD Spec operator*(float s) const { Spec r; _Pragma("unroll") for (int i = 0; i < NS; ++i) r.c[i] = c[i] * s; return r; }
    HD Spec operator/(float s) const { Spec r; _Pragma("unroll") for (int i = 0; i < NS; ++i) r.c[i] = c[i] / s; return r; }
    HD Spec operator-() const { Spec r; _Pragma("unroll") for (int i = 0; i < NS; ++i) r.c[i] = -c[i]; return r; }
    HD Spec &operator+=(const Spec &o) { _Pragma("unroll") for (int i = 0; i < NS; ++i) c[i] += o.c[i]; return *this; }
    HD Spec &operator*=(const Spec &o) { _Pragma("unroll") for (int i = 0; i < NS; ++i) c[i] *= o.c[i]; return *this; }
    HD Spec &operator*=(float s) { _Pragma("unroll") for (int i = 0; i < NS; ++i) c[i] *= s; return *this; }
    HD Spec &operator/=(float s) { _Pragma("unroll") for (int i = 0; i < NS; ++i) c[i] /= s; return *this; }
    HD bool black() const {
        bool b = true;
        _Pragma("unroll") for (int i = 0; i < NS; ++i) b = b && (c[i] == 0.f);
        return b;
    }
};
template <int NS> HD Spec<NS> sexp(const Spec<NS> &s) {
    Spec<NS> r;
#pragma unroll
    for (int i = 0; i < NS; ++i) r.c[i] = expf(s.c[i]);
    return r;
}

/* Spectral context of one path: the hero wavelengths (HERO4) or nothing (RGB3). */
struct Lambda4 { float l[4]; };

/* Spectral tables: host copies come from spectral_tables.h, device copies live in global memory
 * (hero wavelengths differ per lane, so a constant-bank broadcast would serialise). */
#if defined(__CUDACC__)
static __device__ const float d_cie_x[] = {LGPU_CIE_X_DATA};
static __device__ const float d_cie_y[] = {LGPU_CIE_Y_DATA};
static __device__ const float d_cie_z[] = {LGPU_CIE_Z_DATA};
static __device__ const float d_smits_lambda[] = {LGPU_SMITS_LAMBDA_DATA};
static __device__ const float d_smits_basis[14][32] = {LGPU_SMITS_BASIS_DATA};
#endif
#if defined(__CUDA_ARCH__)
#define LG_TAB(name) d_##name
#else
#define LG_TAB(name) lgpu_##name
#endif

/* Linear interpolation in a table sampled at 1 nm from 360 nm. */
HD float cie_at(const float *tab, float l) {
    if (l <= 360.0f) return tab[0];
    if (l >= 830.0f) return tab[LGPU_N_CIE - 1];
    int j = (int)(l - 360.0f);
    j = j < LGPU_N_CIE - 2 ? j : LGPU_N_CIE - 2;
    const float t = (l - (360.0f + (float)j)) / 1.0f;
    return tab[j] + (tab[j + 1] - tab[j]) * t;
}

}  // namespace lg
