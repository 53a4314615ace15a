/*
 * Portable stand-in for <immintrin.h> in the reference build (oracle/_ref only; TEST
 * INFRASTRUCTURE ONLY): the SSE subset of nmmintrin.h plus the BMI2 bit deposit the reference's
 * Morton-order texture addressing calls (image/Texture.h:42-50).
 */
#pragma once
#include "nmmintrin.h"

/* parallel bit deposit: the low bits of src go, in order, to the set bits of mask */
static inline uint64_t _pdep_u64(uint64_t src, uint64_t mask) {
    uint64_t r = 0;
    for (uint64_t bit = 1; mask; bit <<= 1) {
        const uint64_t lowest = mask & (~mask + 1);
        if (src & bit) r |= lowest;
        mask &= mask - 1;
    }
    return r;
}
