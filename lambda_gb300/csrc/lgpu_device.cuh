/*
 * Device side of the GB300 MIS volumetric path tracer.
 *
 * Layers, each restating the reference function cited beside it:
 *   shader bytecode  -- ShaderGraph socket pulls (src/shading/graph/) compiled to a linear program
 *   BSDF leaves      -- Lambertian / Oren-Nayar / microfacet / dielectric (src/shading/surface/)
 *   media            -- HomogeneousMedium + Henyey-Greenstein (src/shading/media/)
 *   lights           -- mesh / triangle / point / spot / environment (src/lighting/)
 *   light tree       -- ManyLightSampler pick / pdf (src/lighting/ManyLightSampler.cpp)
 *   traversal        -- Embree rtcIntersect1 / rtcOccluded1 restated over a BVH2 with a TLAS
 *   integrator       -- MISVolumetricPathIntegrator::Li (src/integrators/MISVolumetricPathIntegrator.cpp)
 * Bug patches (B-ids) are the same as the CPU oracle's; everything else keeps the reference's
 * arithmetic, including std::min/max NaN behaviour.
 */
#pragma once
#include "lgpu_math.cuh"
#include "../../include/lambda_gpu.h"

namespace lg {

/* ------------------------------------------------------------------ bytecode */
enum Op : uint8_t {
    OP_CONST = 0, OP_UV, OP_POINT, OP_NORMAL, OP_NOISE, OP_MATHS, OP_VMATHS, OP_DOT, OP_CROSS, OP_LEN,
    OP_CONV, OP_BBCONST, OP_BB, OP_SEP, OP_MERGE, OP_SCHLICK, OP_IMAGE, OP_COUNT
};
/* socket value types (ShaderGraph.h:46-54) */
enum SockT : uint8_t { ST_NULL = 0, ST_SCALAR, ST_COLOUR, ST_VEC2, ST_VEC3, ST_SPECTRUM, ST_BXDF };
enum NoiseK : uint8_t { NK_PERLIN = 0, NK_VALUE, NK_CHECKER, NK_VORONOI, NK_OCTAVE };

/* Inputs a shader program can read (ScatterEvent / RayHit fields the reference nodes touch). */
struct ShadeCtx {
    float3 point;
    float3 normalS;
    float2 uv;
    float woLy;
    float eta;
    bool mediumInteraction;
    const float4 *texels;   /* texel pool of IMAGE_TEXTURE nodes */
};

/* texture_t::GetPixelUVBilinear (src/image/Texture.h:71-81) at fract(uv)
 * (ImageTextureInput::GetColour, src/shading/graph/GraphInputs.cpp:128-131); texel (x, y) at
 * off + y * w + x.  Returns the filtered texel; the four weights and the base texel index are
 * written for callers that differentiate through the fetch. */
HD float4 image_bilinear(const float4 *tex, int off, int w, int h, float2 uv, int *base = nullptr, float *wts = nullptr) {
    const float u = uv.x - floorf(uv.x), v = uv.y - floorf(uv.y);
    const float fx = fminf((float)(w - 1), fminf(fmaxf(u, 0.f), 1.f) * (float)w);
    const float fy = fminf((float)(h - 1), fminf(fmaxf(v, 0.f), 1.f) * (float)h);
    const int x = (int)fx, y = (int)fy;
    const int x1 = x + 1 < w ? x + 1 : w - 1, y1 = y + 1 < h ? y + 1 : h - 1;
    const float tx = fx - (float)x, ty = fy - (float)y;
    const float4 p00 = tex[off + y * w + x], p10 = tex[off + y * w + x1];
    const float4 p01 = tex[off + y1 * w + x], p11 = tex[off + y1 * w + x1];
    const float4 ya = make_float4(p00.x + (p10.x - p00.x) * tx, p00.y + (p10.y - p00.y) * tx,
                                  p00.z + (p10.z - p00.z) * tx, p00.w + (p10.w - p00.w) * tx);
    const float4 yb = make_float4(p01.x + (p11.x - p01.x) * tx, p01.y + (p11.y - p01.y) * tx,
                                  p01.z + (p11.z - p01.z) * tx, p01.w + (p11.w - p01.w) * tx);
    if (base) {
        base[0] = y * w + x; base[1] = y * w + x1; base[2] = y1 * w + x; base[3] = y1 * w + x1;
        wts[0] = (1.f - tx) * (1.f - ty); wts[1] = tx * (1.f - ty); wts[2] = (1.f - tx) * ty; wts[3] = tx * ty;
    }
    return make_float4(ya.x + (yb.x - ya.x) * ty, ya.y + (yb.y - ya.y) * ty, ya.z + (yb.z - ya.z) * ty,
                       ya.w + (yb.w - ya.w) * ty);
}

/* -------- spectral conversions -------- */
HD float smits_at(const float *curve, float l) {
    const float *lam = LG_TAB(smits_lambda);
    if (l <= lam[0]) return curve[0];
    if (l >= lam[LGPU_N_SMITS - 1]) return curve[LGPU_N_SMITS - 1];
    const int off = find_interval(lam, LGPU_N_SMITS, l);
    const float t = (l - lam[off]) / (lam[off + 1] - lam[off]);
    return lerpf(curve[off], curve[off + 1], t);
}
/* SampledSpectrum::FromRGB (src/core/Spectrum.cpp:104-187) evaluated at one wavelength. */
HD float smits_upsample(float r0, float r1, float r2, bool illum, float l) {
    const float(*B)[32] = LG_TAB(smits_basis) + (illum ? 7 : 0);
    float r = 0.f;
    if (r0 <= r1 && r0 <= r2) {
        r += smits_at(B[0], l) * r0;
        if (r1 <= r2) { r += smits_at(B[1], l) * (r1 - r0); r += smits_at(B[6], l) * (r2 - r1); }
        else { r += smits_at(B[1], l) * (r2 - r0); r += smits_at(B[5], l) * (r1 - r2); }
    } else if (r1 <= r0 && r1 <= r2) {
        r += smits_at(B[0], l) * r1;
        if (r0 <= r2) { r += smits_at(B[2], l) * (r0 - r1); r += smits_at(B[6], l) * (r2 - r0); }
        else { r += smits_at(B[2], l) * (r2 - r1); r += smits_at(B[4], l) * (r0 - r2); }
    } else {
        r += smits_at(B[0], l) * r2;
        if (r0 <= r1) { r += smits_at(B[3], l) * (r0 - r2); r += smits_at(B[5], l) * (r1 - r0); }
        else { r += smits_at(B[3], l) * (r1 - r2); r += smits_at(B[4], l) * (r0 - r1); }
    }
    r *= illum ? 0.86445f : 0.94f;
    return smax(r, 0.f);
}
template <int NS> HD Spec<NS> from_rgb(float r, float g, float b, bool illum, const Lambda4 &lam) {
    Spec<NS> s;
    if (NS == 3) { s.c[0] = r; s.c[1] = g; s.c[2] = b; return s; }
#pragma unroll
    for (int i = 0; i < 4; ++i) s.c[i] = smits_upsample(r, g, b, illum, lam.l[i]);
    return s;
}
/* RGBSpectrum::y (Spectrum.h:328-331); hero: Monte-Carlo luminance of the four samples. */
template <int NS> HD float spec_y(const Spec<NS> &s, const Lambda4 &lam) {
    if (NS == 3) return 0.212671f * s.c[0] + 0.715160f * s.c[1] + 0.072169f * s.c[2];
    float acc = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) acc += s.c[i] * cie_at(LG_TAB(cie_y), lam.l[i]);
    return acc * (HERO_RANGE / (4.0f * LGPU_CIE_Y_INTEGRAL));
}
/* Planck's law normalised at the Wien peak (GraphInputs.cpp:87-104). */
HD float planck(float lnm, float T) {
    const float c = 299792458.f, h = 6.62606957e-34f, kb = 1.3806488e-23f;
    const float l = (float)((double)lnm * 1e-9);
    const float l5 = l * l * l * l * l;
    return (2.0f * h * c * c) / (l5 * (expf((h * c) / (l * kb * T)) - 1.0f));
}
HD float planck_norm(float lnm, float T) {
    const float lmax = (float)(2.8977721e-3 / T * 1e9);
    return planck(lnm, T) / planck(lmax, T);
}
/* RGBSpectrum::FromSampled of a blackbody at `samples` wavelengths in [400, 700) (GraphInputs.cpp:106-116). */
HD void blackbody_rgb(float T, int samples, float out[3]) {
    float lam[8], v[8];
    if (samples > 8) samples = 8;
    const int interval = 300;
    const float inv = 1.0f / (float)samples;
    for (int i = 0; i < samples; ++i) lam[i] = 400.0f + (float)interval * inv * (float)i;
    for (int i = 0; i < samples; ++i) v[i] = planck_norm(lam[i], T);
    float xyz[3] = {0.f, 0.f, 0.f};
    for (int i = 0; i < LGPU_N_CIE; ++i) {
        const float l = 360.0f + (float)i;
        float val;
        if (l <= lam[0]) val = v[0];
        else if (l >= lam[samples - 1]) val = v[samples - 1];
        else {
            const int off = find_interval(lam, samples, l);
            val = lerpf(v[off], v[off + 1], (l - lam[off]) / (lam[off + 1] - lam[off]));
        }
        xyz[0] += val * LG_TAB(cie_x)[i];
        xyz[1] += val * LG_TAB(cie_y)[i];
        xyz[2] += val * LG_TAB(cie_z)[i];
    }
    const float scale = (float)(830.0f - 360.0f) / (float)(LGPU_CIE_Y_INTEGRAL * LGPU_N_CIE);
    xyz[0] *= scale; xyz[1] *= scale; xyz[2] *= scale;
    out[0] = (float)(3.240479 * xyz[0] - 1.537150 * xyz[1] - 0.498535 * xyz[2]);
    out[1] = (float)(-0.969256 * xyz[0] + 1.875991 * xyz[1] + 0.041556 * xyz[2]);
    out[2] = (float)(0.055648 * xyz[0] - 0.204043 * xyz[1] + 1.057311 * xyz[2]);
}

/* -------- noise (GraphTexture.cpp:8-219) -------- */
HD uint32_t hash21(uint32_t x, uint32_t y) { x *= 1597334677u; y *= 3812015801u; return (x ^ y) * 1597334677u; }
HD float grid_hash(float x, float y) { return (float)((double)hash21(to_unsigned(x), to_unsigned(y)) * (1.0 / 4294967296.0)); }
HD float quintic(float x) { return x * x * x * (x * (x * 6.f - 15.f) + 10.f); }
HD float cubicf(float x) { return x * x * (3.f - 2.f * x); }
HD float perlin2d(float u, float v, float scale) {
    u *= scale; v *= scale;
    const float gx = floorf(u), gy = floorf(v);
    float a;
    a = grid_hash(gx, gy) * PI2;           const float g00x = cosf(a), g00y = sinf(a);
    a = grid_hash(gx + 1, gy) * PI2;       const float g10x = cosf(a), g10y = sinf(a);
    a = grid_hash(gx + 1, gy + 1) * PI2;   const float g11x = cosf(a), g11y = sinf(a);
    a = grid_hash(gx, gy + 1) * PI2;       const float g01x = cosf(a), g01y = sinf(a);
    const float d00 = (u - gx) * g00x + (v - gy) * g00y;
    const float d10 = (u - (gx + 1)) * g10x + (v - gy) * g10y;
    const float d11 = (u - (gx + 1)) * g11x + (v - (gy + 1)) * g11y;
    const float d01 = (u - gx) * g01x + (v - (gy + 1)) * g01y;
    const float vx0 = lerpf(d00, d10, quintic(u - gx));
    const float vx1 = lerpf(d01, d11, quintic(u - gx));
    return lerpf(vx0, vx1, quintic(v - gy)) + 0.5f;
}
HD float value2d(float u, float v, float scale) {
    u *= scale; v *= scale;
    const float px = floorf(u), py = floorf(v);
    const float fx = u - px, fy = v - py;
    const float v00 = grid_hash(px, py), v10 = grid_hash(px + 1, py), v11 = grid_hash(px + 1, py + 1), v01 = grid_hash(px, py + 1);
    const float vx0 = lerpf(v00, v10, cubicf(fx)), vx1 = lerpf(v01, v11, cubicf(fx));
    return lerpf(vx0, vx1, cubicf(fy));
}
HD float checker2d(float u, float v, float scale) {
    u = fractf(u * scale); v = fractf(v * scale);
    return (u > .5f) == (v > .5f) ? 0.f : 1.f;
}
HD float checker3d(float3 p, float scale) {
    p = p * scale;
    p = mk(fractf(p.x), fractf(p.y), fractf(p.z));
    return ((p.x > .5f) == (p.y > .5f)) == (p.z > .5f) ? 0.f : 1.f;
}
HD float voronoi2d(float u, float v, float scale) {
    u *= scale; v *= scale;
    const float px = floorf(u), py = floorf(v);
    float m = finf();
    for (int y = -1; y < 2; ++y)
        for (int x = -1; x < 2; ++x) {
            const float ox = px + (float)x, oy = py + (float)y;
            const float hx = add_rn(mul_rn(ox, 127.1f), mul_rn(oy, 311.7f));
            const float hy = add_rn(mul_rn(ox, 269.5f), mul_rn(oy, 183.3f));
            const float sx = sinf(hx) * 18.5453f, sy = sinf(hy) * 18.5453f;
            const float rx = ox + fractf(sx) - u, ry = oy + fractf(sy) - v;
            const float d2 = add_rn(mul_rn(rx, rx), mul_rn(ry, ry));
            if (d2 < m) m = d2;
        }
    return sqrtf(m);
}
HD float3 fract3(float3 v) { return mk(fractf(v.x), fractf(v.y), fractf(v.z)); }
HD float voronoi3d(float3 p, float scale) {
    p = p * scale;
    const float3 b = mk(floorf(p.x), floorf(p.y), floorf(p.z));
    float m = finf();
    for (int z = -1; z < 2; ++z)
        for (int y = -1; y < 2; ++y)
            for (int x = -1; x < 2; ++x) {
                const float3 off = b + mk((float)x, (float)y, (float)z);
                float3 q = fract3(off * mk(.1031f, .1030f, .0973f));
                const float d = add_rn(add_rn(mul_rn(q.x, q.y + 33.33f), mul_rn(q.y, q.x + 33.33f)), mul_rn(q.z, q.z + 33.33f));
                q = q + mk(d, d, d);
                const float3 hsh = fract3((mk(q.x, q.x, q.y) + mk(q.y, q.x, q.x)) * mk(q.z, q.y, q.z));
                const float3 rp = off + hsh - p;
                const float d2 = add_rn(add_rn(mul_rn(rp.x, rp.x), mul_rn(rp.y, rp.y)), mul_rn(rp.z, rp.z));
                if (d2 < m) m = d2;
            }
    return sqrtf(m);
}
HD float noise2(int kind, float u, float v, float scale) {
    switch (kind) {
    case NK_PERLIN: return perlin2d(u, v, scale);
    case NK_VALUE: return value2d(u, v, scale);
    case NK_CHECKER: return checker2d(u, v, scale);
    case NK_VORONOI: return voronoi2d(u, v, scale);
    default: return 0.f;
    }
}
HD float noise3(int kind, float3 p, float scale) {
    switch (kind) {
    case NK_CHECKER: return checker3d(p, scale);
    case NK_VORONOI: return voronoi3d(p, scale);
    default: return 0.f;   /* PerlinNoise::Get3D / ValueNoise::Get3D return 0 (B13) */
    }
}

/* Run one program: registers are float4; spectra occupy xyz (RGB3) or xyzw (HERO4). */
template <int NS>
__host__ __device__ __noinline__ void run_prog(const DIns *p, int n, const ShadeCtx &c, const Lambda4 &lam, float4 *R) {
    for (int i = 0; i < n; ++i) {
        const DIns in = p[i];
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
        switch (in.op) {
        case OP_CONST: r = make_float4(in.k[0], in.k[1], in.k[2], in.k[3]); break;
        case OP_UV: r = make_float4(c.uv.x, c.uv.y, 0.f, 0.f); break;
        case OP_POINT: r = make_float4(c.point.x, c.point.y, c.point.z, 0.f); break;
        case OP_NORMAL: r = make_float4(c.normalS.x, c.normalS.y, c.normalS.z, 0.f); break;
        case OP_IMAGE: {   /* k = (texel offset bits, width, height); sub 0 colour, 1 scalar (red) */
            r = image_bilinear(c.texels, float_to_bits(in.k[0]), (int)in.k[1], (int)in.k[2], c.uv);
            if (in.sub == 1) r = make_float4(r.x, 0.f, 0.f, 0.f);
            break;
        }
        case OP_NOISE: {
            float v = 0.f;
            if (in.sub == NK_OCTAVE) {   /* OctaveNoise::Get2D / Get3D (GraphTexture.cpp:157-175) */
                float amp = .5f, scl = 1.f;
                const int oct = (int)in.k[1];
                for (int o = 0; o < oct; ++o) {
                    if (c.mediumInteraction) v += noise3(in.c, c.point * in.k[0] * scl, in.k[2]) * amp;
                    else v += noise2(in.c, c.uv.x * in.k[0] * scl, c.uv.y * in.k[0] * scl, in.k[2]) * amp;
                    scl *= 2.f; amp *= .5f;
                }
            } else {
                v = c.mediumInteraction ? noise3(in.sub, c.point, in.k[0]) : noise2(in.sub, c.uv.x, c.uv.y, in.k[0]);
            }
            r.x = v;
            break;
        }
        case OP_MATHS: {
            const float a = R[in.a].x, b = R[in.b].x;
            switch (in.sub) {
            case LGPU_MATHS_ADD: r.x = a + b; break;
            case LGPU_MATHS_SUBTRACT: r.x = a - b; break;
            case LGPU_MATHS_MULTIPLY: r.x = a * b; break;
            case LGPU_MATHS_DIVIDE: r.x = a / b; break;
            case LGPU_MATHS_SQRT: r.x = sqrtf(a); break;
            default: r.x = powf(a, b); break;
            }
            break;
        }
        case OP_VMATHS: {
            const float4 a = R[in.a], b = R[in.b];
            switch (in.sub) {
            case LGPU_MATHS_ADD: r = make_float4(a.x + b.x, a.y + b.y, a.z + b.z, 0.f); break;
            case LGPU_MATHS_SUBTRACT: r = make_float4(a.x - b.x, a.y - b.y, a.z - b.z, 0.f); break;
            case LGPU_MATHS_MULTIPLY: r = make_float4(a.x * b.x, a.y * b.y, a.z * b.z, 0.f); break;
            case LGPU_MATHS_DIVIDE: r = make_float4(a.x / b.x, a.y / b.y, a.z / b.z, 0.f); break;
            default: break;
            }
            break;
        }
        case OP_DOT: r.x = dot(f3(R[in.a]), f3(R[in.b])); break;
        case OP_CROSS: { const float3 v = cross(f3(R[in.a]), f3(R[in.b])); r = make_float4(v.x, v.y, v.z, 0.f); break; }
        case OP_LEN: r.x = mag(f3(R[in.a])); break;
        case OP_CONV: {   /* Socket::GetAs<T> / GetAsSpectrum (ShaderGraph.h:90-251) */
            const float4 a = R[in.a];
            const int from = in.sub >> 4, to = in.sub & 15;
            if (to == ST_SCALAR) {
                switch (from) {
                case ST_SCALAR: r.x = a.x; break;
                case ST_COLOUR: r.x = a.x * .3f + a.y * .59f + a.z * .11f; break;
                case ST_VEC2: r.x = (a.x + a.y) * .5f; break;
                case ST_VEC3: r.x = (a.x + a.y + a.z) * .333333333333f; break;
                case ST_SPECTRUM: r.x = spec_y<NS>(Spec<NS>::from4(a), lam); break;
                default: r.x = 0.f;
                }
            } else if (to == ST_COLOUR) {
                switch (from) {
                case ST_COLOUR: r = a; break;
                case ST_SCALAR: r = make_float4(a.x, a.x, a.x, 1.f); break;
                case ST_SPECTRUM: r = make_float4(a.x, a.y, a.z, 1.f); break;
                case ST_VEC3: r = make_float4(a.x, a.y, a.z, 1.f); break;
                case ST_VEC2: { const float m = (a.x + a.y) * .5f; r = make_float4(m, m, m, 1.f); break; }
                default: r = make_float4(1.f, 0.f, 1.f, 1.f);
                }
            } else if (to == ST_VEC2) {
                if (from == ST_VEC2 || from == ST_VEC3) r = make_float4(a.x, a.y, 0.f, 0.f);
                else if (from == ST_SCALAR) r = make_float4(a.x, a.x, 0.f, 0.f);
            } else if (to == ST_VEC3) {
                if (from == ST_VEC3) r = make_float4(a.x, a.y, a.z, 0.f);
                else if (from == ST_VEC2) r = make_float4(a.x, a.y, 0.f, 0.f);
                else if (from == ST_SCALAR) r = make_float4(a.x, a.x, a.x, 0.f);
            } else if (to == ST_SPECTRUM) {
                if (from == ST_COLOUR) r = from_rgb<NS>(a.x, a.y, a.z, in.c != 0, lam).as4();
                else if (from == ST_SCALAR) r = Spec<NS>(a.x).as4();
                else if (from == ST_SPECTRUM) r = a;
            }
            break;
        }
        case OP_BBCONST: {   /* constant-temperature blackbody: RGB folded at compile time */
            if (NS == 3) r = make_float4(in.k[0], in.k[1], in.k[2], 0.f);
            else r = make_float4(planck_norm(lam.l[0], in.k[3]), planck_norm(lam.l[1], in.k[3]),
                                 planck_norm(lam.l[2], in.k[3]), planck_norm(lam.l[3], in.k[3]));
            break;
        }
        case OP_BB: {
            const float T = R[in.a].x;
            if (NS == 3) { float o[3]; blackbody_rgb(T, (int)in.k[0], o); r = make_float4(o[0], o[1], o[2], 0.f); }
            else r = make_float4(planck_norm(lam.l[0], T), planck_norm(lam.l[1], T), planck_norm(lam.l[2], T), planck_norm(lam.l[3], T));
            break;
        }
        case OP_SEP: { const float4 a = R[in.a]; r.x = in.sub == 0 ? a.x : (in.sub == 1 ? a.y : (in.sub == 2 ? a.z : a.w)); break; }
        case OP_MERGE: r = make_float4(R[in.a].x, R[in.b].x, R[in.c].x, in.sub == 255 ? 0.f : R[in.sub].x); break;
        case OP_SCHLICK: {   /* FresnelInput::SchlickApprox (GraphInputs.cpp:183-196) */
            const float n1 = c.eta, n2 = R[in.a].x;
            float R0 = (n1 - n2) / (n1 + n2);
            R0 *= R0;
            const float cc = 1.f - c.woLy;
            r.x = R0 + (1.f - R0) * cc * cc * cc * cc * cc;
            break;
        }
        default: break;
        }
        R[in.dst] = r;
    }
}

/* ------------------------------------------------------------------ BSDF leaves */
HD bool same_hemi(float3 a, float3 b) { return a.y * b.y > 0.f; }
HD float cos2t(float3 w) { return w.y * w.y; }
HD float sin2t(float3 w) { return smax(0.f, 1.f - cos2t(w)); }
HD float sint(float3 w) { return sqrtf(sin2t(w)); }
HD float cosphi(float3 w) { const float s = sint(w); return (s < 0.000001f) ? 0.f : clampr(w.x / s, -1.f, 1.f); }
HD float sinphi(float3 w) { const float s = sint(w); return (s < 0.000001f) ? 0.f : clampr(w.z / s, -1.f, 1.f); }
HD float cos2phi(float3 w) { return cosphi(w) * cosphi(w); }
HD float sin2phi(float3 w) { return sinphi(w) * sinphi(w); }
HD float tan2t(float3 w) { return sin2t(w) / cos2t(w); }
HD float tant(float3 w) { return sint(w) / w.y; }
HD float cos_hemi_pdf(float3 wo, float3 wi) { return same_hemi(wo, wi) ? fabsf(wi.y) * INV_PI : 0.f; }
HD float3 sample_cos_hemi(float u0, float u1) {   /* Sampling.h:9-19 */
    const float r = sqrtf(u0);
    const float th = u1 * PI2;
    const float dx = r * cosf(th), dy = r * sinf(th);
    return mk(dx, sqrtf(smax(0.f, 1.f - dx * dx - dy * dy)), dy);
}
HD float3 reflect(float3 w, float3 n) { return w - n * 2.f * dot(n, w); }
HD bool refract(float3 w, float3 n, float eta, float3 *wr) {
    const float cosI = dot(w, n);
    const float sin2I = smax(0.f, 1.f - cosI * cosI);
    const float sin2T = eta * eta * sin2I;
    if (sin2T >= 1.f) { *wr = mk(-1.f, 1.f, -1.f) * w; return false; }
    const float cosT = sqrtf(1.f - sin2T);
    *wr = w * -eta + n * (eta * cosI - cosT);
    return true;
}
/* Fresnel::FrDielectric (Fresnel.cpp:5-20) */
HD float fr_dielectric(float cosI, float etaI, float etaT) {
    cosI = clampr(cosI, -1.f, 1.f);
    if (cosI < 0.f) { const float t = etaI; etaI = etaT; etaT = t; cosI = fabsf(cosI); }
    const float sinI = sqrtf(smax(0.f, 1.f - cosI * cosI));
    const float sinT = etaI / etaT * sinI;
    if (sinT >= 1.f) return 1.f;
    const float cosT = sqrtf(smax(0.f, 1.f - sinT * sinT));
    const float rPa = (etaT * cosI - etaI * cosT) / (etaT * cosI + etaI * cosT);
    const float rPe = (etaI * cosI - etaT * cosT) / (etaI * cosI + etaT * cosT);
    return (rPa * rPa + rPe * rPe) * .5f;
}
/* MicrofacetDistribution.cpp:11-71 (isotropic alpha) */
HD float md_D(int dist, float3 wh, float a) {
    const float t2 = tan2t(wh);
    if (isinf(t2)) return 0.f;
    const float c4 = cos2t(wh) * cos2t(wh);
    if (dist == LGPU_DIST_BECKMANN) return expf(-t2 * (cos2phi(wh) / (a * a) + sin2phi(wh) / (a * a))) / (PI * a * a * c4);
    const float e = (cos2phi(wh) / (a * a) + sin2phi(wh) / (a * a)) * t2;
    return 1.f / (PI * a * a * c4 * (1.f + e) * (1.f + e));
}
HD float md_lambda(int dist, float3 w, float a) {
    const float at = fabsf(tant(w));
    if (isinf(at)) return 0.f;
    const float alpha = sqrtf(cos2phi(w) * a * a + sin2phi(w) * a * a);
    if (dist == LGPU_DIST_BECKMANN) {
        const float aa = 1.f / (alpha * at);
        if (aa >= 1.6f) return 0.f;
        return (1.f - 1.259f * aa + 0.396f * aa * aa) / (3.535f * aa + 2.181f * aa * aa);
    }
    const float a2 = (alpha * at) * (alpha * at);
    return (-1.f + sqrtf(1.f + a2)) / 2.f;
}
HD float md_G(int dist, float3 wo, float3 wi, float a) { return 1.f / (1.f + md_lambda(dist, wo, a) + md_lambda(dist, wi, a)); }
HD float md_pdf(int dist, float3 wh, float a) { return md_D(dist, wh, a) * fabsf(wh.y); }
HD float3 md_sample(int dist, float u0, float u1, float3 wo, float a) {
    if (dist == LGPU_DIST_BECKMANN) {
        const float lg = u0 == 1.f ? 0.f : logf(1.f - u0);
        const float phi = PI2 * u1;
        const float t2 = -a * a * lg;
        const float cT = 1.f / sqrtf(1.f + t2);
        const float sT = sqrtf(smax(0.f, 1.f - cT * cT));
        const float3 h = spherical_dir(sT, cT, phi);
        return !same_hemi(wo, h) ? -h : h;
    }
    const float phi = PI2 * u1;
    const float t2 = a * a * u0 / (1.f - u0);
    const float cT = 1.f / sqrtf(1.f + t2);
    const float sT = sqrtf(smax(0.f, 1.f - cT * cT));
    float3 wh = spherical_dir(sT, cT, phi);
    if (!same_hemi(wo, wh)) wh = -wh;
    return wh;
}
HD float to_alpha(float r) {   /* Microfacet.cpp:49-54 */
    r = smax(r, 1e-3f);
    const float x = logf(r);
    return 1.62142f + 0.819955f * x + 0.1734f * x * x + 0.0171201f * x * x * x + 0.000640711f * x * x * x * x;
}
HD float oren_nayar_term(float3 wiL, float3 woL, float sigma) {   /* OrenNayar.cpp:10-21 */
    const float thI = acosf(clampr(wiL.y, -1.f, 1.f));
    const float thO = acosf(clampr(woL.y, -1.f, 1.f));
    const float al = smax(thI, thO), be = smin(thI, thO);
    const float phI = acosf(cosphi(wiL)), phO = acosf(cosphi(woL));
    const float s2 = sigma * sigma;
    const float A = 1.f - s2 / (2.f * (s2 + .33f));
    const float B = (.45f * s2) / (s2 + .09f);
    return A + B * smax(0.f, cosf(phI - phO) * clampr(sinf(al), -1.f, 1.f) * clampr(tanf(be), -1.f, 1.f));
}

/* ------------------------------------------------------------------ rays / hits / events */
struct RayHit {
    float3 point, nG, nS, tan, bitan;
    float2 uv;
    int obj;
    float tFar;
    int prim;
};
struct Event {
    float3 wo, wi, woL, wiL;
    int sidedness;
    int medium;
    float eta;
    bool mediumInteraction;
};
HD float3 ev_local(const RayHit &h, float3 v) { return to_local(v, h.tan, h.nS, h.bitan); }
HD float3 ev_world(const RayHit &h, float3 v) { return to_world(v, h.tan, h.nS, h.bitan); }

struct Rng {
    uint32_t key, dim;
    HD float next() { return lgpu_rng_float(key, dim++); }
};

/* One material's BSDF after its program ran: leaf parameters + mix tree. */
template <int NS>
struct Bsdf {
    const DMaterial *m;
    Spec<NS> alb[LGPU_MAX_LEAVES];
    float rough[LGPU_MAX_LEAVES];
    float ratio[2 * LGPU_MAX_LEAVES - 1];
};

template <int NS>
HD Spec<NS> leaf_f(const DLeaf &L, const Spec<NS> &alb, float rough, const Event &ev) {
    switch (L.type) {
    case LGPU_NODE_BXDF_LAMBERTIAN: return alb * INV_PI;
    case LGPU_NODE_BXDF_OREN_NAYAR_R:
    case LGPU_NODE_BXDF_OREN_NAYAR_T: { const float on = oren_nayar_term(ev.wiL, ev.woL, rough); return alb * INV_PI * on; }
    case LGPU_NODE_BXDF_MICROFACET_R: {   /* Microfacet.cpp:12-27 */
        const float cO = fabsf(ev.woL.y), cI = fabsf(ev.wiL.y);
        float3 wh = ev.wiL + ev.woL;
        if (cI == 0.f || cO == 0.f) return Spec<NS>(0.f);
        if (wh.x == 0.f && wh.y == 0.f && wh.z == 0.f) return Spec<NS>(0.f);
        wh = normalised(wh);
        const float3 wiL = mk(ev.wiL.x, clampr(ev.wiL.y, 0.f, 1.f), ev.wiL.z);
        const float F = fr_dielectric(dot(wiL, wh), L.eta, 0.00001f);
        const float a = to_alpha(rough);
        const float D = md_D(L.dist, wh, a);
        const float G = md_G(L.dist, ev.woL, wiL, a);
        return alb * D * G * Spec<NS>(F) / (4.f * cI * cO);
    }
    default: return Spec<NS>(0.f);
    }
}
HD float leaf_pdf(const DLeaf &L, float rough, float3 wo, float3 wi) {
    switch (L.type) {
    case LGPU_NODE_BXDF_MICROFACET_R: {
        if (!same_hemi(wo, wi)) return 0.f;
        const float3 wh = normalised(wo + wi);
        return md_pdf(L.dist, wh, to_alpha(rough)) / (4.f * dot(wo, wh));
    }
    case LGPU_NODE_BXDF_FRESNEL:
    case LGPU_NODE_BXDF_SPECULAR_T: return 0.f;
    default: return cos_hemi_pdf(wo, wi);
    }
}
/* Mix trees are at most two levels deep; the depth is a template parameter so no device function
 * recurses (the stack size stays statically known). */
template <int NS, int D>
struct MixEval {
    HD static Spec<NS> f(const Bsdf<NS> &b, int slot, const Event &ev) {
        const DBsdfNode nd = b.m->tree[slot];
        if (nd.kind == 0) return leaf_f<NS>(b.m->leaves[nd.a], b.alb[nd.a], b.rough[nd.a], ev);
        const float r = b.ratio[slot];
        return MixEval<NS, D + 1>::f(b, nd.a, ev) * (1.f - r) + MixEval<NS, D + 1>::f(b, nd.b, ev) * r;
    }
    HD static float pdf(const Bsdf<NS> &b, int slot, float3 wo, float3 wi) {
        const DBsdfNode nd = b.m->tree[slot];
        if (nd.kind == 0) return leaf_pdf(b.m->leaves[nd.a], b.rough[nd.a], wo, wi);
        const float r = b.ratio[slot];
        return MixEval<NS, D + 1>::pdf(b, nd.a, wo, wi) * (1.f - r) + MixEval<NS, D + 1>::pdf(b, nd.b, wo, wi) * r;
    }
};
template <int NS>
struct MixEval<NS, 3> {
    HD static Spec<NS> f(const Bsdf<NS> &b, int slot, const Event &ev) {
        const DBsdfNode nd = b.m->tree[slot];
        if (nd.kind == 0) return leaf_f<NS>(b.m->leaves[nd.a], b.alb[nd.a], b.rough[nd.a], ev);
        return Spec<NS>(0.f);
    }
    HD static float pdf(const Bsdf<NS> &b, int slot, float3 wo, float3 wi) {
        const DBsdfNode nd = b.m->tree[slot];
        if (nd.kind == 0) return leaf_pdf(b.m->leaves[nd.a], b.rough[nd.a], wo, wi);
        return 0.f;
    }
};
template <int NS> HD Spec<NS> bsdf_f(const Bsdf<NS> &b, const Event &ev) { return MixEval<NS, 0>::f(b, 0, ev); }
template <int NS> HD float bsdf_pdf(const Bsdf<NS> &b, float3 wo, float3 wi) { return MixEval<NS, 0>::pdf(b, 0, wo, wi); }

/* BxDF::Sample_f of one leaf; moves hit.point off the surface as each reference lobe does. */
template <int NS>
HD Spec<NS> leaf_sample(const Bsdf<NS> &b, int li, Event &ev, RayHit &h, Rng &rng, float &pdf) {
    const DLeaf &L = b.m->leaves[li];
    switch (L.type) {
    case LGPU_NODE_BXDF_MICROFACET_R: {   /* Microfacet.cpp:29-42 */
        if (ev.woL.y == 0.f) return Spec<NS>(0.f);
        const float a = to_alpha(b.rough[li]);
        const float u0 = rng.next(), u1 = rng.next();
        const float3 wh = normalised(md_sample(L.dist, u0, u1, ev.woL, a));
        ev.wiL = reflect(-ev.woL, wh);
        if (!same_hemi(ev.woL, ev.wiL)) { pdf = 0.f; return Spec<NS>(0.f); }
        pdf = md_pdf(L.dist, wh, a) / (4.f * dot(ev.woL, wh));
        ev.wi = ev_world(h, ev.wiL);
        h.point = h.point + h.nG * SURFACE_EPSILON;
        return leaf_f<NS>(L, b.alb[li], b.rough[li], ev);
    }
    case LGPU_NODE_BXDF_OREN_NAYAR_T: {   /* OrenNayar.cpp:37-44 */
        const float u0 = rng.next(), u1 = rng.next();
        ev.wiL = sample_cos_hemi(u0, u1);
        pdf = cos_hemi_pdf(ev.woL, ev.wiL);
        ev.wiL.y *= (float)-ev.sidedness;
        ev.wi = ev_world(h, ev.wiL);
        h.point = h.point + h.nG * (float)-ev.sidedness * SURFACE_EPSILON;
        return leaf_f<NS>(L, b.alb[li], b.rough[li], ev);
    }
    case LGPU_NODE_BXDF_FRESNEL: {   /* Specular.cpp:18-45 */
        const bool entering = ev.woL.y > 0.f;
        const float ior = b.rough[li];
        const float fr = fr_dielectric(ev.woL.y, 1.f, ior);
        if (rng.next() < fr) {
            ev.wiL = mk(-ev.woL.x, ev.woL.y, -ev.woL.z);
            ev.wi = ev_world(h, ev.wiL);
            const float cT = fabsf(ev.wiL.y);
            h.point = h.point + h.nG * (entering ? SURFACE_EPSILON : -SURFACE_EPSILON);
            pdf = fr;
            return b.alb[li] * fr / cT;
        }
        const float etaI = entering ? 1.f : ior;
        ev.eta = etaI;
        const float etaT = entering ? ior : 1.f;
        const float3 nf = (ev.woL.y < 0.f) ? mk(0.f, -1.f, 0.f) : mk(0.f, 1.f, 0.f);
        if (!refract(ev.woL, nf, etaI / etaT, &ev.wiL)) { pdf = 0.f; return Spec<NS>(0.f); }
        Spec<NS> ft = b.alb[li] * (1.f - fr);
        ft *= (etaI * etaI) / (etaT * etaT);
        const float cT = fabsf(ev.wiL.y);
        ev.wi = ev_world(h, ev.wiL);
        h.point = h.point + h.nG * (entering ? -SURFACE_EPSILON * 2.f : SURFACE_EPSILON * 2.f);
        pdf = 1.f - fr;
        return ft / cT;
    }
    case LGPU_NODE_BXDF_SPECULAR_R: {   /* Specular.cpp:62-68 */
        pdf = 1.f;
        ev.wiL = mk(-ev.woL.x, ev.woL.y, -ev.woL.z);
        ev.wi = ev_world(h, ev.wiL);
        h.point = h.point + h.nG * SURFACE_EPSILON;
        return b.alb[li] / fabsf(ev.wiL.y);
    }
    default: {   /* BxDF::Sample_f (BxDF.cpp:7-14): cosine hemisphere */
        const float u0 = rng.next(), u1 = rng.next();
        ev.wiL = sample_cos_hemi(u0, u1);
        if (ev.woL.y < 0.f) ev.wiL.y *= -1.f;
        pdf = cos_hemi_pdf(ev.woL, ev.wiL);
        ev.wi = ev_world(h, ev.wiL);
        h.point = h.point + h.nG * SURFACE_EPSILON * (float)ev.sidedness;
        return leaf_f<NS>(L, b.alb[li], b.rough[li], ev);
    }
    }
}
/* MixBSDF::Sample_f (BxDF.cpp:51-60) over the mix tree: descend choosing a child per level
 * (one Get1D each), sample the leaf, then combine on the way up with the other children's f. */
template <int NS>
HD Spec<NS> bsdf_sample(const Bsdf<NS> &b, Event &ev, RayHit &h, Rng &rng, float &pdf) {
    int path[3];
    bool tookA[3];
    int depth = 0;
    int slot = 0;
    while (b.m->tree[slot].kind == 1 && depth < 2) {
        const DBsdfNode nd = b.m->tree[slot];
        const bool a = rng.next() > b.ratio[slot];
        path[depth] = slot;
        tookA[depth] = a;
        ++depth;
        slot = a ? nd.a : nd.b;
    }
    if (b.m->tree[slot].kind == 1) { pdf = 0.f; return Spec<NS>(0.f); }
    Spec<NS> v = leaf_sample<NS>(b, b.m->tree[slot].a, ev, h, rng, pdf);
    for (int k = depth - 1; k >= 0; --k) {
        const DBsdfNode nd = b.m->tree[path[k]];
        const float r = b.ratio[path[k]];
        if (tookA[k]) v = v * (1.f - r) + MixEval<NS, 1>::f(b, nd.b, ev) * r;
        else v = v * r + MixEval<NS, 1>::f(b, nd.a, ev) * (1.f - r);
    }
    return v;
}

/* ------------------------------------------------------------------ media */
template <int NS> HD Spec<NS> medium_sigma(const float *v) {
    Spec<NS> s;
    if (NS == 3) { s.c[0] = v[0]; s.c[1] = v[1]; s.c[2] = v[2]; return s; }
    return Spec<NS>((v[0] + v[1] + v[2]) * (1.f / 3.f));
}
template <int NS> HD Spec<NS> medium_tr(const DMedium &m, float t) {
    const Spec<NS> st = medium_sigma<NS>(m.sa) + medium_sigma<NS>(m.ss);
    return sexp<NS>(-st * smin(t, fmaxreal()));
}
/* HomogeneousMedium::SampleDistance (HomogeneousMedium.cpp:17-38) */
template <int NS>
HD Spec<NS> medium_sample_distance(const DMedium &m, Rng &rng, Event &ev, const RayHit &h, float *t_, float *pdf_) {
    const Spec<NS> sS = medium_sigma<NS>(m.ss);
    const Spec<NS> st = medium_sigma<NS>(m.sa) + sS;
    const float u0 = rng.next(), u1 = rng.next();
    unsigned ch = (unsigned)(u0 * (float)NS);
    ch = ch < (unsigned)NS - 1 ? ch : (unsigned)NS - 1;
    const float dist = -logf(1.f - u1) / st.c[ch];
    const float t = smin(dist, h.tFar);
    ev.mediumInteraction = t < h.tFar;
    const Spec<NS> Tr = sexp<NS>(-st * smin(t, fmaxreal()));
    const Spec<NS> dens = ev.mediumInteraction ? (st * Tr) : Tr;
    float pdf = 0.f;
#pragma unroll
    for (int i = 0; i < NS; ++i) pdf += dens.c[i];
    pdf *= 1.f / (float)NS;
    if (pdf == 0.f) pdf = 1.f;
    *t_ = t;
    *pdf_ = pdf;
    return ev.mediumInteraction ? (Tr * sS / pdf) : (Tr / pdf);
}
template <int NS> HD float medium_pdf_distance(const DMedium &m, float t) {   /* B3 patched */
    const Spec<NS> st = medium_sigma<NS>(m.sa) + medium_sigma<NS>(m.ss);
    const Spec<NS> Tr = sexp<NS>(-st * smin(t, fmaxreal()));
    float pdf = 0.f;
#pragma unroll
    for (int i = 0; i < NS; ++i) pdf += st.c[i] * Tr.c[i];
    pdf *= 1.f / (float)NS;
    return pdf;
}
/* SampleEquiangular (HomogeneousMedium.cpp:49-77): B2 t = min(dist, tFar), B4 origin = ray.o. */
template <int NS>
HD Spec<NS> medium_sample_equiangular(const DMedium &m, float3 ro, float3 rd, Rng &rng, Event &ev, const RayHit &h,
                                      float3 lp, float *t_, float *pdf_) {
    const float3 delta = lp - ro;
    const float l = dot(rd, delta);
    const float D = sqrtf(dot(delta, delta) - l * l);
    const float thA = -atan2f(l, D);
    const float thB = atan2f(h.tFar - l, D);
    const float eps = rng.next();
    const float dist = D * tanf(lerpf(thB, thA, eps));
    const float t = smin(dist, h.tFar);
    *t_ = t;
    ev.mediumInteraction = t < h.tFar;
    rng.next(); rng.next();   /* channel draw, unused (HomogeneousMedium.cpp:70-71) */
    const float pdf = D / ((thB - thA) * (D * D + t * t));
    *pdf_ = pdf;
    const Spec<NS> st = medium_sigma<NS>(m.sa) + medium_sigma<NS>(m.ss);
    const Spec<NS> Tr = sexp<NS>(-st * smin(t, fmaxreal()));
    return Tr * medium_sigma<NS>(m.ss) / pdf;
}
HD float medium_pdf_equiangular(float3 ro, float3 rd, float3 lp, float tFar, float t) {
    const float3 delta = lp - ro;
    const float l = dot(rd, delta);
    const float D = sqrtf(dot(delta, delta) - l * l);
    const float thA = -atan2f(l, D);
    const float thB = atan2f(tFar - l, D);
    return D / ((thB - thA) * (D * D + t * t));
}
HD float phase_hg(float cosT, float g) {   /* HenyeyGreenstein.cpp:8-13 */
    const float g2 = g * g;
    const float den = 1.f + g2 + 2.f * g * cosT;
    return INV_PI4 * (1.f - g2) / (den * sqrtf(den));
}
HD float hg_sample(float g, float3 wo, float3 *wi, Rng &rng) {   /* HenyeyGreenstein.cpp:19-36 */
    const float u0 = rng.next(), u1 = rng.next();
    float cT;
    if (fabsf(g) < 1e-3f) cT = 1.f - 2.f * u0;
    else { const float sq = (1.f - g * g) / (1.f - g + 2.f * g * u0); cT = (1.f + g * g - sq * sq) / (2.f * g); }
    const float sT = sqrtf(smax(0.f, 1.f - cT * cT));
    const float phi = 2.f * PI * u1;
    const float3 wn = -wo;
    const float3 v1 = cross(wn, mk(0.f, 1.f, 0.f));
    const float3 v2 = cross(wn, v1);
    const float3 d = spherical_dir(sT, cT, phi);
    *wi = v1 * d.x + wn * d.y + v2 * d.z;
    return phase_hg(-cT, g);
}

/* ------------------------------------------------------------------ traversal */
struct TravStats { uint32_t nodes, tris, rays; };

#define LG_LEAF_BITS 4
#define LG_MARKER (-1)

HD bool tri_test(float3 o, float3 d, const DTri &T, float tmax, bool closedMax, float *t, float *u, float *v) {
    const float3 e1 = f3(T.e1), e2 = f3(T.e2);
    const float3 pv = cross(d, e2);
    const float det = dot(e1, pv);
    if (det == 0.f) return false;
    const float inv = 1.f / det;
    const float3 tv = o - f3(T.v0);
    const float uu = dot(tv, pv) * inv;
    if (uu < 0.f || uu > 1.f) return false;
    const float3 qv = cross(tv, e1);
    const float vv = dot(d, qv) * inv;
    if (vv < 0.f || uu + vv > 1.f) return false;
    const float tt = dot(e2, qv) * inv;
    if (!(tt > 0.f)) return false;
    if (closedMax ? !(tt <= tmax) : !(tt < tmax)) return false;
    *t = tt; *u = uu; *v = vv;
    return true;
}

struct HitRec { float t, u, v; int prim, obj; };

#if defined(__CUDACC__)
__device__ __forceinline__ float4 ldg4(const float4 *p) { return __ldg(p); }
__device__ __forceinline__ int4 ldg4i(const int4 *p) { return __ldg(p); }
#endif

/* Traversal stacks: per-thread local array, or a column of a shared-memory block array
 * (entry i of thread t at i * LG_SMEM_STRIDE + t: every lane hits its own bank). */
struct LocalStack {
    int v[LGPU_STACK];
    __device__ __forceinline__ int &operator[](int i) { return v[i]; }
};
#define LG_SMEM_STRIDE 128
struct SmemStack {
    int *p;
    __device__ __forceinline__ int &operator[](int i) { return p[i * LG_SMEM_STRIDE]; }
};

#if LGPU_BVH_WIDE
/* One 8-wide node against a ray: keys[k] = (entry distance bits with the low 3 bits replaced by
 * k) for each child box the ray enters before `best`, sorted ascending; ~0u for the others.
 * Slab distances take one multiply-add per plane, t = q * (s * inv) + (p - o) * inv, with the near
 * and far planes of each axis chosen by the sign of the direction once per node.  A plane byte q
 * becomes a float without the conversion pipe: a byte permute writes it into the low mantissa of
 * 2^23 (0x4B0000qq) and subtracting 2^23 leaves q exactly. */
__device__ __forceinline__ void wide_keys(const float4 h0, const int4 qa, const int4 qb, const int4 qc, float3 o,
                                          float3 inv, float best, uint32_t key[8]) {
    const uint32_t eb = __float_as_uint(h0.w);
    const int nch = (int)(eb >> 24);
    const float ax = __fmul_rn(__fsub_rn(h0.x, o.x), inv.x), ay = __fmul_rn(__fsub_rn(h0.y, o.y), inv.y);
    const float az = __fmul_rn(__fsub_rn(h0.z, o.z), inv.z);
    const float bx = __fmul_rn(__uint_as_float((eb & 0xffu) << 23), inv.x);
    const float by = __fmul_rn(__uint_as_float(((eb >> 8) & 0xffu) << 23), inv.y);
    const float bz = __fmul_rn(__uint_as_float(((eb >> 16) & 0xffu) << 23), inv.z);
    /* byte words: qa = lo x (children 0-3, 4-7), lo y; qb = lo z, hi x; qc = hi y, hi z */
    const bool sx = inv.x < 0.f, sy = inv.y < 0.f, sz = inv.z < 0.f;
    const uint32_t nx0 = sx ? qb.z : qa.x, nx1 = sx ? qb.w : qa.y, fx0 = sx ? qa.x : qb.z, fx1 = sx ? qa.y : qb.w;
    const uint32_t ny0 = sy ? qc.x : qa.z, ny1 = sy ? qc.y : qa.w, fy0 = sy ? qa.z : qc.x, fy1 = sy ? qa.w : qc.y;
    const uint32_t nz0 = sz ? qc.z : qb.x, nz1 = sz ? qc.w : qb.y, fz0 = sz ? qb.x : qc.z, fz1 = sz ? qb.y : qc.w;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
#define LG_QF(w0, w1) __fsub_rn(__uint_as_float(__byte_perm((k < 4 ? (w0) : (w1)), 0x4B000000u, 0x7440u | (uint32_t)(k & 3))), 8388608.f)
        const float tnx = __fmaf_rn(LG_QF(nx0, nx1), bx, ax), tfx = __fmaf_rn(LG_QF(fx0, fx1), bx, ax);
        const float tny = __fmaf_rn(LG_QF(ny0, ny1), by, ay), tfy = __fmaf_rn(LG_QF(fy0, fy1), by, ay);
        const float tnz = __fmaf_rn(LG_QF(nz0, nz1), bz, az), tfz = __fmaf_rn(LG_QF(fz0, fz1), bz, az);
#undef LG_QF
        const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, 0.f));
        const float tf = fminf(fminf(tfx, tfy), fminf(tfz, best));
        key[k] = (k < nch && tn <= tf) ? ((__float_as_uint(tn) & ~7u) | (uint32_t)k) : 0xffffffffu;
    }
    /* Batcher's odd-even merge network for eight keys (19 compare-exchanges) */
#define LG_CX(i, j) { const uint32_t lo = umin(key[i], key[j]); key[j] = umax(key[i], key[j]); key[i] = lo; }
    LG_CX(0, 1) LG_CX(2, 3) LG_CX(4, 5) LG_CX(6, 7) LG_CX(0, 2) LG_CX(1, 3) LG_CX(4, 6) LG_CX(5, 7) LG_CX(1, 2)
    LG_CX(5, 6) LG_CX(0, 4) LG_CX(3, 7) LG_CX(1, 5) LG_CX(2, 6) LG_CX(1, 4) LG_CX(3, 6) LG_CX(2, 4) LG_CX(3, 5)
    LG_CX(3, 4)
#undef LG_CX
}
#endif

/* Closest hit (any_hit = false) or occlusion (any_hit = true) over TLAS + BLAS.  The entry being
 * visited is held in `e`; a node continues with its nearest hit child and pushes the others far to
 * near, so the next nearest is popped first.  Every push is checked against the stack: the host
 * refuses scenes whose worst case exceeds it, so the check only reports a broken bound. */
template <bool COUNT, class STK>
__device__ __forceinline__ bool traverse_t(const DeviceScene &S, float3 wo, float3 wd, float tmax, bool any_hit, HitRec *hr,
                                           TravStats *st, STK &stack) {
    int sp = 0;
    int e = S.root;   /* encoded child ref of the root */
    float3 o = wo, d = wd;
    float3 inv = mk(1.f / d.x, 1.f / d.y, 1.f / d.z);
    const float3 winv = inv;   /* world-space 1/d, restored when the ray leaves an instance */
#if LGPU_BOX_FMA
    float3 oi = mk(o.x * inv.x, o.y * inv.y, o.z * inv.z);   /* slab distance = fma(plane, inv, -oi) */
#endif
    float best = tmax;
    int inst_obj = -1;
    bool hit = false;
    bool in_blas = !S.use_tlas;
    if (COUNT) st->rays++;
    while (true) {
        if (e == LG_MARKER) {
            o = wo; d = wd; inv = winv;
#if LGPU_BOX_FMA
            oi = mk(o.x * inv.x, o.y * inv.y, o.z * inv.z);
#endif
            in_blas = false; inst_obj = -1;
            if (sp == 0) break;
            e = stack[--sp];
            continue;
        }
        const int ref = e >> LG_LEAF_BITS, cnt = e & ((1 << LG_LEAF_BITS) - 1);
        if (cnt == 0) {
#if !LGPU_BVH_WIDE
            const DNode *n = S.nodes + ref;
            const float4 xs = ldg4(&n->xs), ys = ldg4(&n->ys), zs = ldg4(&n->zs);
            const int4 ch = ldg4i(&n->ch);
            if (COUNT) st->nodes++;
#if LGPU_BOX_FMA
#define LG_SLAB(p, a) __fmaf_rn((p), inv.a, -oi.a)
#else
#define LG_SLAB(p, a) (((p) - o.a) * inv.a)
#endif
            const float ax0 = LG_SLAB(xs.x, x), ax1 = LG_SLAB(xs.y, x);
            const float ay0 = LG_SLAB(ys.x, y), ay1 = LG_SLAB(ys.y, y);
            const float az0 = LG_SLAB(zs.x, z), az1 = LG_SLAB(zs.y, z);
            const float bx0 = LG_SLAB(xs.z, x), bx1 = LG_SLAB(xs.w, x);
            const float by0 = LG_SLAB(ys.z, y), by1 = LG_SLAB(ys.w, y);
            const float bz0 = LG_SLAB(zs.z, z), bz1 = LG_SLAB(zs.w, z);
#undef LG_SLAB
            const float an = fmaxf(fmaxf(fminf(ax0, ax1), fminf(ay0, ay1)), fmaxf(fminf(az0, az1), 0.f));
            const float af = fminf(fminf(fmaxf(ax0, ax1), fmaxf(ay0, ay1)), fminf(fmaxf(az0, az1), best));
            const float bn = fmaxf(fmaxf(fminf(bx0, bx1), fminf(by0, by1)), fmaxf(fminf(bz0, bz1), 0.f));
            const float bf = fminf(fminf(fmaxf(bx0, bx1), fmaxf(by0, by1)), fminf(fmaxf(bz0, bz1), best));
            const bool ha = an <= af, hb = bn <= bf;
            if (ha || hb) {
                if (ha && hb) {
                    if (sp + 1 > LGPU_STACK) {
                        atomicOr(S.err, 1);
                        return hit;
                    }
                    const bool aFirst = an <= bn;
                    stack[sp++] = aFirst ? ch.y : ch.x;
                    e = aFirst ? ch.x : ch.y;
                } else {
                    e = ha ? ch.x : ch.y;
                }
                continue;
            }
#else
            const float4 *np = reinterpret_cast<const float4 *>(S.nodes + ref);
            const float4 h0 = ldg4(np);
            const int4 h1 = ldg4i(reinterpret_cast<const int4 *>(np) + 1);
            const int4 qa = ldg4i(reinterpret_cast<const int4 *>(np) + 2);
            const int4 qb = ldg4i(reinterpret_cast<const int4 *>(np) + 3);
            const int4 qc = ldg4i(reinterpret_cast<const int4 *>(np) + 4);
            if (COUNT) st->nodes++;
            uint32_t key[8];
            wide_keys(h0, qa, qb, qc, o, inv, best, key);
            if (key[0] != 0xffffffffu) {
                int nhit = 1;
#pragma unroll
                for (int k = 1; k < 8; ++k) nhit += key[k] != 0xffffffffu ? 1 : 0;
                if (sp + nhit - 1 > LGPU_STACK) {
                    atomicOr(S.err, 1);
                    return hit;
                }
#define LG_ENT(kk) ([&] {                                                                        \
        const int ch = (int)((kk) & 7u);                                                          \
        const uint32_t mb = ((uint32_t)(ch < 4 ? h1.z : h1.w) >> (8 * (ch & 3))) & 0xffu;         \
        const int c = (int)(mb & 7u), off = (int)(mb >> 3);                                       \
        return c ? (((h1.y + off) << LG_LEAF_BITS) | c) : ((h1.x + off) << LG_LEAF_BITS);         \
    }())
#pragma unroll
                for (int k = 7; k >= 1; --k)
                    if (key[k] != 0xffffffffu) stack[sp++] = LG_ENT(key[k]);
                e = LG_ENT(key[0]);
#undef LG_ENT
                continue;
            }
#endif
        } else if (!in_blas) {
            /* TLAS leaf: one instance record */
            const DInst *I = S.insts + ref;
            const float4 r0 = ldg4(&I->r0), r1 = ldg4(&I->r1), r2 = ldg4(&I->r2);
            /* inv * (o - t) and inv * d, unfused, in the order of the host's column-major product */
            const float3 v = mk(__fsub_rn(wo.x, r0.w), __fsub_rn(wo.y, r1.w), __fsub_rn(wo.z, r2.w));
            o = mk(add_rn(add_rn(mul_rn(r0.x, v.x), mul_rn(r0.y, v.y)), mul_rn(r0.z, v.z)),
                   add_rn(add_rn(mul_rn(r1.x, v.x), mul_rn(r1.y, v.y)), mul_rn(r1.z, v.z)),
                   add_rn(add_rn(mul_rn(r2.x, v.x), mul_rn(r2.y, v.y)), mul_rn(r2.z, v.z)));
            d = mk(add_rn(add_rn(mul_rn(r0.x, wd.x), mul_rn(r0.y, wd.y)), mul_rn(r0.z, wd.z)),
                   add_rn(add_rn(mul_rn(r1.x, wd.x), mul_rn(r1.y, wd.y)), mul_rn(r1.z, wd.z)),
                   add_rn(add_rn(mul_rn(r2.x, wd.x), mul_rn(r2.y, wd.y)), mul_rn(r2.z, wd.z)));
            inv = mk(1.f / d.x, 1.f / d.y, 1.f / d.z);
#if LGPU_BOX_FMA
            oi = mk(o.x * inv.x, o.y * inv.y, o.z * inv.z);
#endif
            inst_obj = __ldg(&I->object);
            in_blas = true;
            if (sp + 1 > LGPU_STACK) {
                atomicOr(S.err, 1);
                return hit;
            }
            stack[sp++] = LG_MARKER;
            e = __ldg(&I->root);
            continue;
        } else {
            for (int k = 0; k < cnt; ++k) {
                const DTri *tp = S.tris + ref + k;
                DTri T;
                T.v0 = ldg4(&tp->v0); T.e1 = ldg4(&tp->e1); T.e2 = ldg4(&tp->e2);
                if (COUNT) st->tris++;
                float t, u, v;
                if (tri_test(o, d, T, best, any_hit, &t, &u, &v)) {
                    if (any_hit) return true;
                    best = t; hit = true;
                    hr->t = t; hr->u = u; hr->v = v;
                    hr->prim = __float_as_int(T.v0.w);
                    hr->obj = inst_obj >= 0 ? inst_obj : __float_as_int(T.e1.w);
                }
            }
        }
        if (sp == 0) break;
        e = stack[--sp];
    }
    return hit;
}

template <bool COUNT>
__device__ __noinline__ bool traverse(const DeviceScene &S, float3 wo, float3 wd, float tmax, bool any_hit, HitRec *hr, TravStats *st) {
    LocalStack stk;
    return traverse_t<COUNT>(S, wo, wd, tmax, any_hit, hr, st, stk);
}

/* Object::Hit + TriangleMesh/Instance::ProcessHit (Object.h:27-35, TriangleMesh.cpp:80-114,
 * Instance.cpp:36-43); B18 transforms Ng, B26 uses the instance that was hit. */
static __device__ __noinline__ void process_hit(const DeviceScene &S, float3 o, float3 d, const HitRec &hr, RayHit &h) {
    const DObject &ob = S.objects[hr.obj];
    const DMesh me = S.meshes[ob.mesh];
    const uint4 ti = __ldg(&S.tri_idx[me.tri_off + hr.prim]);
    const float3 p0 = f3(__ldg(&S.pos[me.vtx_off + ti.x]));
    const float3 p1 = f3(__ldg(&S.pos[me.vtx_off + ti.y]));
    const float3 p2 = f3(__ldg(&S.pos[me.vtx_off + ti.z]));
    h.tFar = hr.t;
    h.point = mk(o.x + d.x * hr.t, o.y + d.y * hr.t, o.z + d.z * hr.t);
    const float3 ng = cross(p1 - p0, p2 - p0);
    h.nG = normalised(ng);
    const float u = hr.u, v = hr.v;
    if (me.flags & 2) {
        const float2 a = __ldg(&S.uv[me.vtx_off + ti.x]), b = __ldg(&S.uv[me.vtx_off + ti.y]), c = __ldg(&S.uv[me.vtx_off + ti.z]);
        h.uv = make_float2(a.x + (b.x - a.x) * u + (c.x - a.x) * v, a.y + (b.y - a.y) * u + (c.y - a.y) * v);
    }
    if (me.flags & 1) {
        const float3 n0 = f3(__ldg(&S.nrm[me.vtx_off + ti.x])), n1 = f3(__ldg(&S.nrm[me.vtx_off + ti.y])), n2 = f3(__ldg(&S.nrm[me.vtx_off + ti.z]));
        const float4 t0 = __ldg(&S.tan[me.vtx_off + ti.x]), t1 = __ldg(&S.tan[me.vtx_off + ti.y]), t2 = __ldg(&S.tan[me.vtx_off + ti.z]);
        h.nS = normalised(n0 + (n1 - n0) * u + (n2 - n0) * v);
        h.tan = normalised(f3(t0) + (f3(t1) - f3(t0)) * u + (f3(t2) - f3(t0)) * v);
        const float3 b0 = cross(n0, f3(t0)) * t0.w, b1 = cross(n1, f3(t1)) * t1.w, b2 = cross(n2, f3(t2)) * t2.w;
        h.bitan = normalised(b0 + (b1 - b0) * u + (b2 - b0) * v);
    } else {
        h.nS = h.nG;
        const float3 c1 = cross(h.nG, mk(0.f, 0.f, 1.f));
        const float3 c2 = cross(h.nG, mk(0.f, 1.f, 0.f));
        h.tan = dot(c1, c1) > dot(c2, c2) ? c1 : c2;
        h.bitan = cross(h.tan, h.nG);
    }
    if (ob.kind == 1 && !ob.identity) {
        h.nS = normalised(mul_cm(ob.m, h.nS));
        h.tan = normalised(mul_cm(ob.m, h.tan));
        h.bitan = normalised(mul_cm(ob.m, h.bitan));
        h.nG = normalised(mul_cm(ob.nrm, ng));
    }
    h.obj = hr.obj;
    h.prim = hr.prim;
}

}  // namespace lg
