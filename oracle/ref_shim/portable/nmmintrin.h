/*
 * Element-wise stand-in for the few SSE intrinsics the reference renderer uses (maths/vec3.h,
 * image/Colour.h), for the reference build in oracle/_ref only.  TEST INFRASTRUCTURE ONLY.
 * Each lane is one IEEE single-precision operation, as an SSE lane is, so x86 and Arm hosts compute
 * the same results (with -ffp-contract=off).
 */
#pragma once
#include <cstdint>
#include <cstring>

struct alignas(16) __m128 { float v[4]; };

static inline __m128 _mm_load_ps(const float *p) { __m128 r; std::memcpy(r.v, p, sizeof(r.v)); return r; }
static inline void _mm_store_ps(float *p, __m128 a) { std::memcpy(p, a.v, sizeof(a.v)); }
static inline __m128 _mm_set_ps1(float x) { __m128 r; r.v[0] = r.v[1] = r.v[2] = r.v[3] = x; return r; }
static inline __m128 _mm_add_ps(__m128 a, __m128 b) { for (int i = 0; i < 4; ++i) a.v[i] = a.v[i] + b.v[i]; return a; }
static inline __m128 _mm_sub_ps(__m128 a, __m128 b) { for (int i = 0; i < 4; ++i) a.v[i] = a.v[i] - b.v[i]; return a; }
static inline __m128 _mm_mul_ps(__m128 a, __m128 b) { for (int i = 0; i < 4; ++i) a.v[i] = a.v[i] * b.v[i]; return a; }
static inline __m128 _mm_div_ps(__m128 a, __m128 b) { for (int i = 0; i < 4; ++i) a.v[i] = a.v[i] / b.v[i]; return a; }
/* lanes equal: all-ones bit pattern, else zero */
static inline __m128 _mm_cmpeq_ps(__m128 a, __m128 b) {
    __m128 r;
    for (int i = 0; i < 4; ++i) {
        const uint32_t m = a.v[i] == b.v[i] ? 0xffffffffu : 0u;
        std::memcpy(&r.v[i], &m, sizeof(m));
    }
    return r;
}
/* sign bit of each lane into bit i of the result */
static inline int _mm_movemask_ps(__m128 a) {
    int m = 0;
    for (int i = 0; i < 4; ++i) {
        uint32_t u;
        std::memcpy(&u, &a.v[i], sizeof(u));
        m |= (int)(u >> 31) << i;
    }
    return m;
}
