/*
 * Counter-based random numbers keyed by (seed, pixel, sample, dimension).
 *
 * This replaces Lambda's stateful HaltonSampler + SampleShifter (src/sampling/HaltonSampler.cpp:5-63,
 * src/sampling/SampleShifter.cpp:5-21) behind the same Sampler::Get1D / Get2D seam
 * (src/sampling/Sampler.h:9-25).  A value depends only on its key, so a path can be replayed
 * anywhere (GPU megakernel, GPU wavefront, CPU oracle) and a render resumed at any sample index
 * reproduces an uninterrupted render bit for bit.
 *
 * The mixer is the "lowbias32" integer hash (Wellons, 2018), applied in a chain over the key
 * words.  Get1D returns the top 24 bits scaled by 2^-24, so every value lies in [0, 1).
 * Get2D draws x first, then y, each from its own dimension.
 */
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define LGPU_HD __host__ __device__ __forceinline__
#else
#define LGPU_HD inline
#endif

LGPU_HD uint32_t lgpu_mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

/* Hash of the path key (seed, pixel, sample); the per-dimension value mixes this with dim. */
LGPU_HD uint32_t lgpu_path_key(uint32_t seed, uint32_t pixel, uint32_t sample) {
    uint32_t h = lgpu_mix32(seed ^ 0x9e3779b9U);
    h = lgpu_mix32(h ^ pixel);
    h = lgpu_mix32(h ^ (sample * 0x85ebca6bU + 0x68e31da4U));
    return h;
}

LGPU_HD uint32_t lgpu_rng_bits(uint32_t path_key, uint32_t dim) {
    return lgpu_mix32(path_key ^ lgpu_mix32(dim * 0xc2b2ae35U + 0x27d4eb2fU));
}

LGPU_HD float lgpu_rng_float(uint32_t path_key, uint32_t dim) {
    return (float)(lgpu_rng_bits(path_key, dim) >> 8) * (1.0f / 16777216.0f);
}

/* Dimension used for the hero-wavelength draw; outside the sequence Get1D walks through. */
#define LGPU_DIM_WAVELENGTH 0xFFFFFF00U
