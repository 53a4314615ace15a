/* Camera ray generation shared by every render kernel: the pixel jitter of Render.cpp:55-56 and
 * Camera::GenerateRay (src/camera/Camera.cpp:41-71) with the thin lens's Aperture::Sample_p
 * (src/camera/Aperture.cpp:10-36).  Random numbers come from the path's stream in the reference's
 * order: jitter x, y, then the aperture's. */
#pragma once
#include "lgpu_device.cuh"
#include "lgpu_launch.h"

namespace lg {

/* Piecewise1D::SampleContinuous (src/sampling/Piecewise.cpp:19-28) over a CDF of n + 1 entries */
__device__ __forceinline__ float pool_sample_cont(const float *cdf, int n, float u, int *off_) {
    const int off = find_interval(cdf, n + 1, u);
    if (off_) *off_ = off;
    float du = u - cdf[off];
    if ((cdf[off + 1] - cdf[off]) > 0.f) du /= (cdf[off + 1] - cdf[off]);
    return ((float)off + du) / (float)n;
}

/* Aperture::Sample_p: a point on the aperture plane */
__device__ __forceinline__ float2 aperture_sample(const CamParams &cam, const float *fpool, Rng &rng) {
    const float size = cam.ap_size;
    switch (cam.aperture) {
    case LGPU_APERTURE_BLADE: {   /* BladeAperture::Sample_p (Aperture.cpp:10-19) */
        const float d = PI2 / (float)cam.blades;
        const float rnd = PI2 * rng.next();
        const float thMin = floorf(rnd / d) * d;
        const float thMax = thMin + d;
        const float ux = rng.next(), uy = rng.next();
        return make_float2((cosf(thMin) * ux + cosf(thMax) * uy) * size, (sinf(thMin) * ux + sinf(thMax) * uy) * size);
    }
    case LGPU_APERTURE_CIRCULAR: {   /* CircularAperture::Sample_p (Aperture.cpp:25-27), SampleUnitDisk */
        const float ux = rng.next(), uy = rng.next();
        const float r = sqrtf(ux), th = uy * PI2;
        return make_float2(r * cosf(th) * size - size * .5f, r * sinf(th) * size - size * .5f);
    }
    case LGPU_APERTURE_MASKED: {   /* MaskedAperture::Sample_p (Aperture.cpp:33-36), Piecewise2D */
        const float ux = rng.next(), uy = rng.next();
        int row;
        const float d1 = pool_sample_cont(fpool + cam.mask_marg_off, cam.mask_h, uy, &row);
        const float d0 = pool_sample_cont(fpool + cam.mask_cond_off + row * (2 * cam.mask_w + 2), cam.mask_w, ux, nullptr);
        return make_float2(d0 * size - size * .5f, d1 * size - size * .5f);
    }
    default: return make_float2(0.f, 0.f);
    }
}

/* Film-plane coordinates of pixel (x, y) with jitter, then the camera's ray */
__device__ __forceinline__ void camera_ray(const CamParams &cam, const float *fpool, uint32_t x, uint32_t y, Rng &rng,
                                           float3 &o, float3 &d) {
    const float u = cam.xi * ((float)x + rng.next() - .5f);
    const float v = cam.yi * ((float)y + rng.next() - .5f);
    if (cam.type == LGPU_CAMERA_SPHERICAL) {   /* SphericalCamera::GenerateRay (Camera.cpp:66-71) */
        const float phi = PI2 * u + cam.off_phi;
        const float theta = PI * v + cam.off_theta;
        const float3 s = normalised(spherical_dir(sinf(theta), cosf(theta), phi));
        o = cam.o;
        d = cam.x * s.x + cam.y * s.y + cam.z * s.z;
        return;
    }
    const float px = u * -cam.tanFov2 + cam.tanFov, py = v * -cam.tanFov2 * cam.aspect + cam.tanFov * cam.aspect;
    if (cam.type == LGPU_CAMERA_THIN_LENS) {   /* ThinLensCamera::GenerateRay (Camera.cpp:53-58) */
        const float3 fp = cam.o + (cam.x * px + cam.y * py + cam.z) * cam.focal;
        const float2 ap = cam.aperture != LGPU_APERTURE_NONE ? aperture_sample(cam, fpool, rng) : make_float2(0.f, 0.f);
        o = cam.o + cam.x * ap.x + cam.y * ap.y;
        d = normalised(fp - o);
        return;
    }
    /* PinholeCamera::GenerateRay (Camera.cpp:41-44) */
    const float3 p = cam.o + cam.x * px + cam.y * py + cam.z;
    o = cam.o;
    d = normalised(p - cam.o);
}

}  // namespace lg
