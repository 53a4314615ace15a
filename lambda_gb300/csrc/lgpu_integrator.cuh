/*
 * Lights, light sampling, transmittance queries and the MIS volumetric integrator on the GPU.
 * Restates src/lighting/ (Light.cpp, MeshLight.cpp, PointLight.cpp, Spotlight.cpp,
 * EnvironmentLight.cpp, LightSampler.cpp, ManyLightSampler.cpp), src/core/Scene.cpp:28-107 and
 * src/integrators/MISVolumetricPathIntegrator.cpp:23-215 for one path per thread.
 */
#pragma once
#include "lgpu_device.cuh"

namespace lg {

/* A light as the integrator sees it: `tri` >= 0 selects a TriangleLight of mesh light `light`
 * (the light tree's unit), tri = -1 the light itself.  Equality is pointer equality in the
 * reference (`nl != l`). */
struct LRef { int light, tri; };

#define LG_MAX_TREE_DEPTH 64
HD bool lref_eq(LRef a, LRef b) { return a.light == b.light && a.tri == b.tri; }

/* Adjoint replay arguments: dLoss/dI per pixel and the gradient targets. */
struct AdjArgs {
    const float4 *dloss;   /* per pixel: dLoss / d(pixel mean), rgb */
    float4 *grad_tex;      /* per texel of the differentiated texture (rgb accumulated) */
    float *grad_scalar;    /* roughness, sigma_a, sigma_s (accumulated) */
    int tex_material, tex_off, tex_w, tex_h;
    int rough_material, medium;
    float inv_spp;
};

template <int NS, bool COUNT>
struct Tracer {
    const DeviceScene &S;
    Rng &rng;
    const Lambda4 &lam;
    TravStats *st;
    float *trlen = nullptr;   /* adjoint replay: accumulates the path length inside medium trmed */
    int trmed = -1;

    /* ---------------------------------------------------------------- scene queries */
    __device__ bool intersect(float3 o, float3 d, RayHit &h) {   /* Scene::Intersect (Scene.cpp:28-43) */
        HitRec hr;
        if (!traverse<COUNT>(S, o, d, finf(), false, &hr, st)) return false;
        if (!(hr.t > 0.f) || !(hr.t < finf())) return false;
        process_hit(S, o, d, hr, h);
        return true;
    }
    __device__ bool occluded(float3 o, float3 d, float tmax) {
        HitRec hr;
        return traverse<COUNT>(S, o, d, tmax, true, &hr, st);
    }
    __device__ const DMaterial &mat(const RayHit &h) { return S.materials[S.objects[h.obj].material]; }
    __device__ int get_medium(const DMaterial &m, float3 w, float3 n) { return dot(w, n) < 0.f ? m.medium_interior : m.medium_exterior; }

    /* Scene::IntersectTr (Scene.cpp:45-81); maxT < 0 selects the unbounded form. */
    __device__ __noinline__ bool intersect_tr(float3 o, float3 d, RayHit &h, int med, Spec<NS> *Tr, float maxT) {
        float tFar = 0.f;
        for (int guard = 0; guard < 256; ++guard) {
            if (!intersect(o, d, h)) return false;
            tFar += h.tFar;
            bool term = false;
            if (maxT >= 0.f) {
                term = tFar > maxT;
                if (term) { const float delta = tFar - maxT; tFar -= delta; h.tFar -= delta; }
            }
            if (med >= 0 && Tr) *Tr *= medium_tr<NS>(S.media[med], h.tFar);
            if (trlen && med >= 0 && med == trmed) *trlen += h.tFar;
            const DMaterial &m = mat(h);
            if (term || m.has_bsdf || m.light >= 0) { h.tFar = tFar; return true; }
            med = get_medium(m, d, h.nG);
            o = h.point + h.nG * (dot(h.nG, d) < 0.f ? -SURFACE_EPSILON : SURFACE_EPSILON);
        }
        return false;
    }
    /* Light::MutualVisibility / PointMutualVisibility (Light.cpp:10-38); bounded = point form. */
    __device__ bool light_visibility(float3 p1, float3 p2, Event &ev, Spec<NS> *Tr, bool bounded) {
        const float3 diff = p2 - p1;
        const float m = mag(diff);
        const float3 dir = divs(diff, m);
        if (S.has_volumes) {
            const float minT = m - SURFACE_EPSILON * 10.f;
            ev.wi = dir;
            RayHit hh;
            hh.tFar = finf();
            intersect_tr(p1, dir, hh, ev.medium, Tr, bounded ? m : -1.f);
            return hh.tFar > minT;
        }
        ev.wi = dir;   /* Scene::MutualVisibility (Scene.cpp:83-95) */
        return !occluded(p1, dir, (float)(m - .00001));
    }
    /* Light::RayEscapes (Light.cpp:40-49) */
    __device__ bool ray_escapes(float3 o, float3 d, const Event &ev, Spec<NS> *Tr) {
        if (S.has_volumes) {
            RayHit hh;
            return !intersect_tr(o, d, hh, ev.medium, Tr, -1.f);
        }
        return !occluded(o, d, finf());
    }

    /* ---------------------------------------------------------------- emission programs */
    __device__ __noinline__ Spec<NS> emission(const DLight &L, const Event &ev, const RayHit &h, bool illum) {
        if (NS == 3 && L.em_folded) return Spec<NS>::from4(illum ? L.em[0] : L.em[1]);
        float4 R[LGPU_MAX_REGS];
        ShadeCtx c;
        c.point = h.point; c.normalS = h.nS; c.uv = h.uv; c.woLy = ev.woL.y; c.eta = ev.eta;
        c.mediumInteraction = ev.mediumInteraction;
        c.texels = S.env_tex;
        run_prog<NS>(S.prog + L.prog_off, L.prog_len, c, lam, R);
        /* the program ends with a conversion to a spectrum; the reflectance variant sits one
         * register above the illuminant one */
        return Spec<NS>::from4(R[L.out_reg + (illum ? 0 : 1)]);
    }

    /* ---------------------------------------------------------------- environment light */
    __device__ Spec<NS> env_texel_uv(float u, float v) {   /* TextureAdapter::GetUV, bilinear (Texture.h:71-81) */
        const DEnv &E = S.env;
        u = fractf(u); v = fractf(v);
        const float fx = fminf((float)(E.w - 1), clampr(u, 0.f, 1.f) * (float)E.w);
        const float fy = fminf((float)(E.h - 1), clampr(v, 0.f, 1.f) * (float)E.h);
        const unsigned x = (unsigned)fx, y = (unsigned)fy;
        const unsigned x1 = min(x + 1, (unsigned)E.w - 1), y1 = min(y + 1, (unsigned)E.h - 1);
        const float4 a = __ldg(&S.env_tex[E.tex_off + y * E.w + x]), b = __ldg(&S.env_tex[E.tex_off + y * E.w + x1]);
        const float4 c = __ldg(&S.env_tex[E.tex_off + y1 * E.w + x]), d = __ldg(&S.env_tex[E.tex_off + y1 * E.w + x1]);
        const float tx = fx - (float)x, ty = fy - (float)y;
        const float r = lerpf(lerpf(a.x, b.x, tx), lerpf(c.x, d.x, tx), ty);
        const float g = lerpf(lerpf(a.y, b.y, tx), lerpf(c.y, d.y, tx), ty);
        const float bb = lerpf(lerpf(a.z, b.z, tx), lerpf(c.z, d.z, tx), ty);
        return from_rgb<NS>(r, g, bb, true, lam);
    }
    __device__ Spec<NS> env_le(float3 w) {   /* EnvironmentLight::Le (EnvironmentLight.h:47-50) */
        const DEnv &E = S.env;
        const float u = fractf((spherical_phi(w) - E.offx) * INV_PI2);
        const float v = fractf((spherical_theta(w) - E.offy) * INV_PI);
        return env_texel_uv(u, v) * E.intensity;
    }
    __device__ float p1d_sample_cont(int cdf_off, int n, float integral, float u, float *pdf, int *off_) {
        const float *cdf = S.fpool + cdf_off;
        const int off = find_interval(cdf, n + 1, u);
        if (off_) *off_ = off;
        float du = u - cdf[off];
        if ((cdf[off + 1] - cdf[off]) > 0.f) du /= (cdf[off + 1] - cdf[off]);
        *pdf = S.fpool[cdf_off + n + 1 + off] / integral;
        return ((float)off + du) / (float)n;
    }
    __device__ __noinline__ Spec<NS> env_sample_li(Event &ev, const RayHit &h, float &pdf) {   /* EnvironmentLight.cpp:24-45 */
        const DEnv &E = S.env;
        const float u0 = rng.next(), u1 = rng.next();
        float pm, pc; int row;
        const float d1 = p1d_sample_cont(E.marg_off, E.h, E.marg_integral, u1, &pm, &row);
        const int co = E.cond_off + row * (2 * E.w + 2);
        const float d0 = p1d_sample_cont(co, E.w, S.fpool[co + 2 * E.w + 1], u0, &pc, nullptr);
        pdf = pc * pm;
        if (pdf == 0.f) return Spec<NS>(0.f);
        const float theta = d1 * PI + E.offy;
        const float phi = d0 * PI2 + E.offx;
        const float cT = cosf(theta), sT = sinf(theta);
        if (sT == 0.f) { pdf = 0.f; return Spec<NS>(0.f); }
        ev.wi = spherical_dir(sT, cT, phi);
        Spec<NS> Tr(1.f);
        if (ray_escapes(h.point + h.nG * SURFACE_EPSILON, ev.wi, ev, &Tr)) {
            ev.wiL = ev_local(h, ev.wi);
            pdf /= 2.f * PI * PI * sT;
            return env_texel_uv(d0, d1) * Tr * E.intensity;
        }
        pdf = 0.f;
        return Spec<NS>(0.f);
    }
    __device__ __noinline__ float env_pdf_li(const Event &ev) {   /* EnvironmentLight.cpp:60-67 + Piecewise2D::PDF */
        const DEnv &E = S.env;
        const float theta = spherical_theta(ev.wi) - E.offy;
        const float phi = spherical_phi(ev.wi) - E.offx;
        const float sT = sinf(theta);
        if (sT == 0.f) return 0.f;
        const float u = fractf(phi * INV_PI2), v = fractf(theta * INV_PI);
        const int iu = max(min((int)(u * (float)E.w), E.w - 1), 0);
        const int iv = max(min((int)(v * (float)E.h), E.h - 1), 0);
        const int co = E.cond_off + iv * (2 * E.w + 2);
        const float p = S.fpool[co + E.w + 1 + iu] / E.marg_integral;
        return p / (2.f * PI * PI * sT);
    }

    /* ---------------------------------------------------------------- mesh / triangle lights */
    __device__ void tri_verts(const DLight &L, int t, float3 &a, float3 &b, float3 &c) {
        const DObject &ob = S.objects[L.object];
        const DMesh me = S.meshes[ob.mesh];
        const uint4 ti = __ldg(&S.tri_idx[me.tri_off + t]);
        a = f3(__ldg(&S.pos[me.vtx_off + ti.x]));
        b = f3(__ldg(&S.pos[me.vtx_off + ti.y]));
        c = f3(__ldg(&S.pos[me.vtx_off + ti.z]));
    }
    __device__ float2 tri_uv(const DLight &L, int t, float u, float v) {
        const DObject &ob = S.objects[L.object];
        const DMesh me = S.meshes[ob.mesh];
        const uint4 ti = __ldg(&S.tri_idx[me.tri_off + t]);
        const float2 a = S.uv[me.vtx_off + ti.x], b = S.uv[me.vtx_off + ti.y], c = S.uv[me.vtx_off + ti.z];
        return make_float2(a.x + (b.x - a.x) * u + (c.x - a.x) * v, a.y + (b.y - a.y) * u + (c.y - a.y) * v);
    }
    __device__ bool mesh_has_uv(const DLight &L) { return (S.meshes[S.objects[L.object].mesh].flags & 2) != 0; }
    HD static void area_normal(float3 a, float3 b, float3 c, float *area, float3 *n) {   /* TriangleMesh.h:59-63 */
        const float3 cr = cross(b - a, c - a);
        *area = mag(cr) * .5f;
        if (n) *n = divs(cr, (float)(*area * 2.));
    }
    __device__ int mesh_pick(const DLight &L, float u, float *pdf) {   /* Piecewise1D::SampleDiscrete */
        const float *cdf = S.fpool + L.dist_off;
        const int off = find_interval(cdf, L.num_tris + 1, u);
        *pdf = S.fpool[L.dist_off + L.num_tris + 1 + off] / (L.integral * (float)L.num_tris);
        return off;
    }

    /* Light::Sample_Li for every light kind. */
    __device__ __noinline__ Spec<NS> sample_li(LRef r, Event &ev, RayHit &h, float &pdf) {
        if (r.light < 0) { pdf = 0.f; return Spec<NS>(0.f); }   /* no light to sample */
        const DLight &L = S.lights[r.light];
        if (L.type == LT_ENV) return env_sample_li(ev, h, pdf);
        if (L.type == LT_POINT || L.type == LT_SPOT) {   /* PointLight.cpp:18-29, Spotlight.cpp:44-55 */
            const float3 p = h.point + h.nG * SURFACE_EPSILON * (float)ev.sidedness;
            Spec<NS> Tr(1.f);
            if (light_visibility(p, L.pos, ev, &Tr, true)) {
                pdf = 1.f;
                const float d2 = distsq(L.pos, h.point);
                ev.wiL = ev_local(h, ev.wi);
                Spec<NS> e = emission(L, ev, h, false) * Tr;
                if (L.type == LT_SPOT) e = e * spot_falloff(L, -ev.wi);
                return e * L.intensity / d2;
            }
            pdf = 0.f;
            return Spec<NS>(0.f);
        }
        /* mesh light: whole mesh (MeshLight.cpp:22-42) or one triangle (TriangleLight, :134-151) */
        int t = r.tri;
        float u0, u1;
        if (t < 0) {
            t = mesh_pick(L, rng.next(), &pdf);
            u0 = rng.next(); u1 = rng.next();
        } else {
            u0 = rng.next(); u1 = rng.next();
        }
        float3 a, b, c;
        tri_verts(L, t, a, b, c);
        const float3 pL = a + (b - a) * u0 + (c - a) * u1;
        const float3 pS = h.point + h.nG * SURFACE_EPSILON * (float)ev.sidedness;
        Spec<NS> Tr(1.f);
        if (light_visibility(pS, pL, ev, &Tr, false)) {
            float area; float3 n;
            area_normal(a, b, c, &area, &n);
            const float cT = fabsf(dot(n, -ev.wi));
            if (cT > 0.f) {
                ev.wiL = ev_local(h, ev.wi);
                if (r.tri < 0) pdf *= distsq(h.point, pL) / (cT * area);
                else pdf = distsq(h.point, pL) / (cT * area);   /* B10 */
                return emission(L, ev, h, true) * Tr * L.intensity * INV_PI;
            }
        }
        pdf = 0.f;
        return Spec<NS>(0.f);
    }
    __device__ float spot_falloff(const DLight &L, float3 w) {   /* Spotlight.cpp:21-27 */
        const float c = dot(w, L.axis);
        if (c < L.cosCone) return 0.f;
        if (c > L.cosFall) return 1.f;
        const float d = (c - L.cosCone) / (L.cosFall - L.cosCone);
        return (d * d) * (d * d);
    }
    /* Light::PDF_Li(event) at the new hit (MeshLight.cpp:44-53, :158-165, EnvironmentLight.cpp:60-67). */
    __device__ __noinline__ float pdf_li(LRef r, const Event &ev, const RayHit &h) {
        const DLight &L = S.lights[r.light];
        if (L.type == LT_ENV) return env_pdf_li(ev);
        if (L.type != LT_MESH) return 0.f;
        if (h.prim >= L.num_tris) return 0.f;   /* hit object does not carry this light's mesh */
        if (dot(ev.wi, h.nG) > 0.f) return 0.f;
        const float distSq = h.tFar * h.tFar;
        float3 a, b, c;
        tri_verts(L, h.prim, a, b, c);
        float area;
        area_normal(a, b, c, &area, nullptr);
        const float cT = fabsf(dot(h.nG, -ev.wi));
        if (r.tri < 0) {
            const float triPdf = S.fpool[L.dist_off + L.num_tris + 1 + h.prim];   /* raw area (Piecewise1D::PDF) */
            return triPdf * distSq / (cT * area);
        }
        return distSq / (cT * area);
    }
    /* Light::PDF_Li(event, sampler): the pdf of direction ev.wi from the shading point h, found
     * with a ray query -- MeshLight.cpp:43-54 (no triangle-selection factor; TriangleLight delegates
     * to its mesh light, :153-155), EnvironmentLight.cpp:47-58 (the ray must escape), 0 for delta
     * lights.  Used by DirectLightingIntegrator's BSDF-sampled strategy. */
    __device__ __noinline__ float pdf_li_dir(LRef r, const Event &ev, const RayHit &h) {
        if (r.light < 0) return 0.f;
        const DLight &L = S.lights[r.light];
        if (L.type == LT_ENV) {
            const DEnv &E = S.env;
            const float theta = spherical_theta(ev.wi) - E.offy;
            const float phi = spherical_phi(ev.wi) - E.offx;
            const float sT = sinf(theta);
            if (sT == 0.f) return 0.f;
            const float3 wOff = spherical_dir(sT, cosf(theta), phi);
            if (!ray_escapes(h.point, wOff, ev, nullptr)) return 0.f;
            const float u = fractf(phi * INV_PI2), v = fractf(theta * INV_PI);
            const int iu = max(min((int)(u * (float)E.w), E.w - 1), 0);
            const int iv = max(min((int)(v * (float)E.h), E.h - 1), 0);
            const int co = E.cond_off + iv * (2 * E.w + 2);
            return S.fpool[co + E.w + 1 + iu] / E.marg_integral / (2.f * PI * PI * sT);
        }
        if (L.type != LT_MESH) return 0.f;
        const float3 o = h.point + h.nG * (SURFACE_EPSILON * (float)ev.sidedness);
        RayHit hh;
        hh.tFar = finf(); hh.uv = make_float2(0.f, 0.f);
        const bool hit = S.has_volumes ? intersect_tr(o, ev.wi, hh, ev.medium, nullptr, -1.f) : intersect(o, ev.wi, hh);
        if (!hit || mat(hh).light != r.light || hh.prim >= L.num_tris) return 0.f;
        float3 a, b, c, n;
        tri_verts(L, hh.prim, a, b, c);
        float area;
        area_normal(a, b, c, &area, &n);
        const float cT = fabsf(dot(n, -ev.wi));
        return cT > 0.f ? distsq(h.point, hh.point) / (cT * area) : 0.f;
    }
    /* Light::SamplePoint (MeshLight.cpp:55-70, :167-181, PointLight.cpp:40-44). */
    __device__ __noinline__ Spec<NS> sample_point(LRef r, Event &ev, RayHit &h, float3 &lpoint, float3 &lnormal, float &lpdf) {
        if (r.light < 0) { lpdf = 0.f; lpoint = h.point; return Spec<NS>(0.f); }
        const DLight &L = S.lights[r.light];
        if (L.type == LT_ENV) { lpdf *= 0.f; lpoint = mk(0.f, 0.f, 0.f); return Spec<NS>(0.f); }
        if (L.type == LT_POINT || L.type == LT_SPOT) { lpoint = L.pos; return emission(L, ev, h, true) * L.intensity; }
        int t = r.tri;
        float3 a, b, c;
        if (t < 0) {
            float dp;
            t = mesh_pick(L, rng.next(), &dp);
            tri_verts(L, t, a, b, c);
            float area;
            area_normal(a, b, c, &area, &lnormal);
            lpdf *= dp / area;
        } else {
            tri_verts(L, t, a, b, c);
            float area;
            area_normal(a, b, c, &area, nullptr);
            lpdf /= area;
        }
        const float u0 = rng.next(), u1 = rng.next();
        if (mesh_has_uv(L)) h.uv = tri_uv(L, t, u0, u1);
        lpoint = a + (b - a) * u0 + (c - a) * u1;
        return emission(L, ev, h, true) * L.intensity * INV_PI;
    }
    /* Light::Visibility (MeshLight.cpp:72-81, :183-192, PointLight.cpp:46-55, Spotlight.cpp:69-78, EnvironmentLight.cpp:76-84). */
    __device__ __noinline__ Spec<NS> visibility(LRef r, float3 p, Event &ev, RayHit &h, float3 lpoint, float3 lnormal, float &lpdf) {
        if (r.light < 0) { lpdf = 0.f; return Spec<NS>(0.f); }
        const DLight &L = S.lights[r.light];
        Spec<NS> Tr(1.f);
        if (L.type == LT_ENV) {
            const float3 wi = normalised(lpoint - p);
            if (ray_escapes(p, wi, ev, &Tr)) return Tr;
            lpdf = 0.f;
            return Spec<NS>(0.f);
        }
        if (L.type == LT_POINT || L.type == LT_SPOT) {
            const float3 q = p + h.nG * SURFACE_EPSILON * (float)ev.sidedness;
            if (light_visibility(q, lpoint, ev, &Tr, true)) {
                Spec<NS> v = Tr;
                if (L.type == LT_SPOT) v = v * spot_falloff(L, -ev.wi);
                return v / distsq(L.pos, h.point);
            }
            lpdf = 0.f;
            return Spec<NS>(0.f);
        }
        if (light_visibility(p, lpoint, ev, &Tr, false)) {
            const float cT = r.tri < 0 ? fabsf(dot(lnormal, -ev.wi)) : fabsf(dot(h.nG, -ev.wi));
            lpdf *= distsq(p, lpoint) / cT;
            return Tr;
        }
        lpdf = 0.f;
        return Spec<NS>(0.f);
    }
    /* Light::L at the new hit (MeshLight::L) */
    __device__ __noinline__ Spec<NS> light_L(LRef r, const Event &ev, const RayHit &h) {
        const DLight &L = S.lights[r.light];
        if (L.type == LT_ENV) return env_le(ev.wi);
        if (L.type == LT_MESH) return emission(L, ev, h, true) * L.intensity * INV_PI;
        return Spec<NS>(0.f);
    }
    __device__ Spec<NS> light_Le(LRef r, float3 d) {
        const DLight &L = S.lights[r.light];
        if (L.type == LT_ENV) return env_le(d);
        return Spec<NS>(0.f);
    }

    /* ---------------------------------------------------------------- light samplers */
    /* ManyLightSampler::ImportanceMeasure (ManyLightSampler.cpp:305-326), useSplits = true:
     *   theta  = acos(delta . axis), thetaU = atan(r / d), thetaDash = max(theta - thetaO - thetaU, 0)
     *   I = cos(max(thetaI - thetaU, 0)) * E / d^2 * cos(thetaDash)   if thetaDash < thetaE (= pi/2)
     * evaluated with cosine/sine identities instead of acos / atan / cos.  The reference's angles come
     * from acos of the rounded dot products, so the dot products are rounded as the reference rounds
     * them (products, then sums) and the sines are taken as sqrt((1 - c)(1 + c)), which keeps full
     * relative precision for cosines near 1, where acos is ill-conditioned.  The reference's NaN
     * cases are kept: a cone cosine outside [-1, 1] gives 0, a normal cosine outside [-1, 1] NaN. */
    static __device__ __forceinline__ float dot_rn(float3 a, float3 b) {
        return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
    }
    static __device__ __forceinline__ float sin_of_cos(float c) { return sqrtf(smax(0.f, (1.f - c) * (1.f + c))); }
    __device__ __forceinline__ float importance(float3 p, float3 nS, const DLNode &n) {
        float3 delta = n.center - p;
        const float d2 = dot_rn(delta, delta);
        const float dd = sqrtf(d2);
        const float invD = 1.f / dd;
        delta = make_float3(__fmul_rn(delta.x, invD), __fmul_rn(delta.y, invD), __fmul_rn(delta.z, invD));
        const float cosT = dot_rn(delta, n.axis);
        if (!(cosT >= -1.f && cosT <= 1.f)) return 0.f;
        const float tU = (n.diag * .5f) * invD;
        const float cosU = 1.f / sqrtf(1.f + tU * tU), sinU = tU * cosU;
        const float cosA = n.cosO * cosU - n.sinO * sinU;   /* a = thetaO + thetaU */
        const float sinA = n.sinO * cosU + n.cosO * sinU;
        float cosDash = 1.f;
        if (!(sinA < 0.f || cosT >= cosA)) {               /* theta > a (and a <= pi) */
            cosDash = cosT * cosA + sin_of_cos(cosT) * sinA;
            if (!(cosDash > 0.f)) return 0.f;               /* thetaDash >= thetaE = pi/2 */
        }
        const float cosI = dot_rn(delta, nS);
        if (!(cosI >= -1.f && cosI <= 1.f)) return __int_as_float(0x7fc00000);
        float cosTerm = 1.f;
        if (cosI < cosU)                                    /* thetaI > thetaU */
            cosTerm = cosI * cosU + sin_of_cos(cosI) * sinU;
        return (cosTerm * n.power) / d2 * cosDash;
    }
    __device__ LRef tree_light_ref(int idx) {
        const int2 tl = __ldg(&S.tree_lights[idx]);
        LRef r; r.light = tl.x; r.tri = tl.y;
        return r;
    }
    /* LightSampler::Sample: PowerLightSampler (LightSampler.cpp:17-19) or ManyLightSampler (:17-27, :355-378). */
    __device__ __noinline__ LRef sample_light(float3 p, float3 nS, float *pdf) {
        if (S.light_strategy == LGPU_LIGHT_STRATEGY_POWER) {
            const float *cdf = S.fpool + S.power_cdf_off;
            const float u = rng.next();
            const int off = find_interval(cdf, S.num_lights + 1, u);
            *pdf = S.fpool[S.power_cdf_off + S.num_lights + 1 + off] / (S.power_integral * (float)S.num_lights);
            LRef r; r.light = off; r.tri = -1;
            return r;
        }
        float eps = rng.next();
        const float pTree = S.tree_power / (S.inf_power + S.tree_power);
        if (eps < pTree) {
            eps /= pTree;
            *pdf *= pTree;
            float e = rng.next();   /* B6: a fresh draw drives the descent */
            /* the chosen child's record, loaded with its sibling, is the next level's node: one
             * round of (two independent) loads per level */
            DLNode n = S.lnodes[S.tree_root];
            for (int guard = 0; guard < 64; ++guard) {
                if (n.child0 < 0) {
                    const float *cdf = S.fpool + n.dist_off;
                    const int off = find_interval(cdf, n.num + 1, e);
                    *pdf *= S.fpool[n.dist_off + n.num + 1 + off] / (n.integral * (float)n.num);
                    return tree_light_ref(n.first + off);
                }
                const DLNode cl = S.lnodes[n.child0], cr = S.lnodes[n.child0 + 1];
                const float IL = importance(p, nS, cl);
                const float IR = importance(p, nS, cr);
                const float PL = IL / (IL + IR);
                const float PR = 1.f - PL;
                if (e < PL) { e /= PL; *pdf *= PL; n = cl; }
                else { e = (e - PL) / PR; *pdf *= PR; n = cr; }
            }
        }
        *pdf *= 1.f - pTree;
        LRef r; r.light = S.env_light; r.tri = -1;
        return r;
    }
    /* LightSampler::Pdf (LightSampler.cpp:21-23, ManyLightSampler.cpp:29-35 + RecursivePDF :380-393, B7, B8). */
    __device__ __noinline__ float light_pdf(float3 p, float3 nS, int prim, LRef l) {
        const DLight &L = S.lights[l.light];
        if (S.light_strategy == LGPU_LIGHT_STRATEGY_POWER) return L.power * S.inv_total_power;
        if (L.type == LT_ENV) return S.inf_power / (S.inf_power + S.tree_power);
        int ti;
        if (L.type == LT_MESH) {
            const int t = l.tri >= 0 ? l.tri : prim;
            if (t < 0 || t >= L.num_tris) return 0.f;
            ti = L.tri_base + t;
        } else ti = S.light_slot[l.light];
        if (ti < 0 || ti >= S.num_tree_lights) return 0.f;
        const int2 slot = __ldg(&S.tree_slot[ti]);
        DLNode cur = S.lnodes[slot.x];
        const float pdf = S.fpool[cur.dist_off + cur.num + 1 + slot.y];   /* raw power (Piecewise1D::PDF) */
        /* branch probabilities multiplied leaf-up (the reference's recursion multiplies root-down;
         * the two orders agree to a few ulps).  Sibling pairs are (even, even + 1) records, so the
         * sibling is index ^ 1 and the left child is the even one; the sibling and the parent are
         * independent loads of each level. */
        int child = slot.x;
        float acc = 1.f;
        for (int depth = 0; cur.parent >= 0 && depth < LG_MAX_TREE_DEPTH; ++depth) {
            const DLNode sib = S.lnodes[child ^ 1];
            const DLNode par = S.lnodes[cur.parent];
            const bool left = (child & 1) == 0;
            const float IL = importance(p, nS, left ? cur : sib);
            const float IR = importance(p, nS, left ? sib : cur);
            const float p0 = IL / (IL + IR);
            acc = (left ? p0 : 1.f - p0) * acc;
            child = cur.parent;
            cur = par;
        }
        return pdf * acc;
    }

    /* ---------------------------------------------------------------- BSDF setup */
    __device__ __noinline__ void setup_bsdf(Bsdf<NS> &b, const DMaterial &m, const Event &ev, const RayHit &h) {
        b.m = &m;
        if (NS == 3 && m.folded) {   /* context-free graph evaluated at scene compile */
            for (int i = 0; i < m.num_leaves; ++i) { b.alb[i] = Spec<NS>::from4(m.kalb[i]); b.rough[i] = m.krough[i]; }
            for (int i = 0; i < m.num_tree; ++i) b.ratio[i] = m.kratio[i];
            return;
        }
        float4 R[LGPU_MAX_REGS];
        ShadeCtx c;
        c.point = h.point; c.normalS = h.nS; c.uv = h.uv; c.woLy = ev.woL.y; c.eta = ev.eta;
        c.mediumInteraction = ev.mediumInteraction;
        c.texels = S.env_tex;
        run_prog<NS>(S.prog + m.prog_off, m.prog_len, c, lam, R);
        for (int i = 0; i < m.num_leaves; ++i) {
            b.alb[i] = Spec<NS>::from4(R[m.leaves[i].albedo]);
            b.rough[i] = R[m.leaves[i].rough].x;
        }
        for (int i = 0; i < m.num_tree; ++i) b.ratio[i] = m.tree[i].kind ? R[m.tree[i].ratio].x : 0.f;
    }

    /* ---------------------------------------------------------------- integrator */
    HD static float power_heuristic(float f, float g) { return (f * f) / (f * f + g * g); }

    /* LdMediumPoint (MISVolumetricPathIntegrator.cpp:23-69) */
    __device__ __noinline__ Spec<NS> ld_medium_point(Event &ev, RayHit &hit, float3 p, LRef lsLight, float3 lsPoint, float3 lsNormal,
                                        Spec<NS> lsLe, float &lsPdf, float3 &wiOut, float3 sp, float3 sn) {
        /* lsPdf is the PartialLightSample's pdf: Visibility completes it in place, so the second
         * call (equiangular point) starts from the value the first call left. */
        const DMedium &med = S.media[ev.medium];
        float partialLightPDF = lsPdf;
        hit.point = p;
        Spec<NS> Li = lsLe * visibility(lsLight, p, ev, hit, lsPoint, lsNormal, lsPdf);
        float scatteringPDF, lightPDF = lsPdf;
        Spec<NS> Ld(0.f);
        if (lightPDF > 0.f && !Li.black()) {
            scatteringPDF = phase_hg(dot(ev.wo, ev.wi), med.g);
            if (scatteringPDF > 0.f) {
                const float w = power_heuristic(lightPDF, scatteringPDF);
                Ld += Li * Spec<NS>(scatteringPDF) * w / lightPDF;
            }
        }
        scatteringPDF = hg_sample(med.g, ev.wo, &ev.wi, rng);
        wiOut = ev.wi;
        const float3 ro = p, rd = ev.wi;
        Spec<NS> Tr(1.f);
        const bool hs = intersect_tr(ro, rd, hit, ev.medium, &Tr, -1.f);
        if (scatteringPDF > 0.f) {
            LRef nl; nl.light = hs ? mat(hit).light : S.env_light; nl.tri = -1;
            if (nl.light >= 0) {
                if (!lref_eq(nl, lsLight)) partialLightPDF = light_pdf(sp, sn, hit.prim, nl);
                lightPDF = partialLightPDF * pdf_li(nl, ev, hit);
                Li = hs ? light_L(nl, ev, hit) : light_Le(nl, rd);
                const float w = power_heuristic(scatteringPDF, lightPDF);
                if (!Li.black() && lightPDF > 0.f) Ld += Li * Tr * w / scatteringPDF;
            }
        }
        return Ld;
    }

    /* ---------------------------------------------------------------- the other integrators
     * PathIntegrator::Li (src/integrators/PathIntegrator.cpp:15-88): the surface branch of the MIS
     * integrator with media ignored (null surfaces are crossed, no medium is entered).  B7 patched
     * as in Li: the light-tree pdf of a BSDF-sampled emitter is evaluated at the shading point. */
    __device__ Spec<NS> Li_path(float3 ro, float3 rd, int maxBounces, int minBounces) {
        Spec<NS> L(0.f), beta(1.f);
        RayHit hit;
        hit.tFar = finf(); hit.uv = make_float2(0.f, 0.f);
        Event ev;
        ev.wo = -rd; ev.wi = mk(0.f, 0.f, 0.f); ev.woL = ev.wi; ev.wiL = ev.wi;
        ev.sidedness = 1; ev.medium = -1; ev.eta = 1.001f; ev.mediumInteraction = false;
        bool scatterIntersect = false;
        int nullCrossings = 0;
        for (int bounces = 0; bounces < maxBounces; ++bounces) {
            if (bounces == 0 ? intersect(ro, rd, hit) : scatterIntersect) {
                const DMaterial &m = mat(hit);
                if (bounces == 0 && m.light >= 0) { LRef lr; lr.light = m.light; lr.tri = -1; L += light_L(lr, ev, hit); }
                if (m.has_bsdf) {
                    ev.wo = -rd;
                    ev.woL = ev_local(hit, ev.wo);
                    ev.wiL = ev_local(hit, ev.wi);
                    ev.sidedness = (ev.woL.y > 0.f) ? 1 : -1;
                    Bsdf<NS> b;
                    setup_bsdf(b, m, ev, hit);
                    float lightDistPdf = 1.f;
                    const float3 sp = hit.point, sn = hit.nS;
                    const LRef l = sample_light(hit.point, hit.nS, &lightDistPdf);
                    Spec<NS> Ld(0.f);
                    float scatteringPDF = 0.f, lightPDF = 0.f;
                    Spec<NS> Li = sample_li(l, ev, hit, lightPDF);
                    Spec<NS> f;
                    lightPDF *= lightDistPdf;
                    if (lightPDF > 0.f && !Li.black()) {
                        f = bsdf_f<NS>(b, ev) * fabsf(ev.wiL.y);
                        scatteringPDF = bsdf_pdf<NS>(b, ev.woL, ev.wiL);
                        if (!f.black() && scatteringPDF > 0.f) Ld += Li * f * power_heuristic(lightPDF, scatteringPDF) / lightPDF;
                    }
                    f = bsdf_sample<NS>(b, ev, hit, rng, scatteringPDF);
                    f *= fabsf(ev.wiL.y);
                    ro = hit.point;
                    rd = ev.wi;
                    scatterIntersect = intersect(ro, rd, hit);
                    if (scatteringPDF > 0.f && !f.black()) {
                        LRef nl; nl.light = scatterIntersect ? mat(hit).light : S.env_light; nl.tri = -1;
                        if (nl.light >= 0) {
                            if (!lref_eq(nl, l)) lightDistPdf = light_pdf(sp, sn, hit.prim, nl);
                            lightPDF = lightDistPdf * pdf_li(nl, ev, hit);
                            Li = scatterIntersect ? light_L(nl, ev, hit) : light_Le(nl, rd);
                            if (!Li.black() && lightPDF > 0.f) Ld += Li * f * power_heuristic(scatteringPDF, lightPDF) / scatteringPDF;
                        }
                    } else break;
                    L += beta * Ld;
                    beta *= f / scatteringPDF;
                } else {
                    ro = hit.point + hit.nG * (dot(rd, hit.nG) < 0.f ? -SURFACE_EPSILON : SURFACE_EPSILON);
                    if (bounces > 0) scatterIntersect = intersect(ro, rd, hit);
                    if (++nullCrossings > 256) break;
                    bounces--;
                    continue;
                }
                if (bounces > minBounces) {
                    const float q = smax(.05f, 1.f - spec_y<NS>(beta, lam));
                    if (rng.next() < q) break;
                    beta /= 1.f - q;
                }
            } else {
                if (bounces == 0 && S.env_light >= 0) L += env_le(rd);
                break;
            }
        }
        return L;
    }

    /* VolumetricPathIntegrator::Li (src/integrators/VolumetricPathIntegrator.cpp:20-160): distance
     * sampling only (no equiangular), medium vertices with light sampling + phase MIS, the medium
     * contribution weighted by the throughput.  B7 patched at surface and medium vertices; an
     * absent environment light contributes nothing on escape (the reference dereferences null). */
    __device__ Spec<NS> Li_volpath(float3 ro, float3 rd, int maxBounces, int minBounces) {
        Spec<NS> L(0.f), beta(1.f);
        RayHit hit;
        hit.tFar = finf(); hit.uv = make_float2(0.f, 0.f);
        Event ev;
        ev.wo = -rd; ev.wi = mk(0.f, 0.f, 0.f); ev.woL = ev.wi; ev.wiL = ev.wi;
        ev.sidedness = 1; ev.medium = -1; ev.eta = 1.001f; ev.mediumInteraction = false;
        bool scatterIntersect = false;
        int nullCrossings = 0;
        for (int bounces = 0; bounces < maxBounces; ++bounces) {
            if (bounces == 0 ? intersect(ro, rd, hit) : scatterIntersect) {
                if (bounces == 0 && mat(hit).light >= 0) {
                    LRef lr; lr.light = mat(hit).light; lr.tri = -1;
                    if (ev.medium >= 0) L += light_L(lr, ev, hit) * medium_tr<NS>(S.media[ev.medium], hit.tFar);
                    else L += light_L(lr, ev, hit);
                }
                float distanceT = 0.f, distPdf = 0.f;
                if (ev.medium >= 0) beta *= medium_sample_distance<NS>(S.media[ev.medium], rng, ev, hit, &distanceT, &distPdf);
                else ev.mediumInteraction = false;
                if (!ev.mediumInteraction) {
                    const DMaterial &m = mat(hit);
                    if (m.has_bsdf) {
                        ev.wo = -rd;
                        ev.woL = ev_local(hit, ev.wo);
                        ev.wiL = ev_local(hit, ev.wi);
                        ev.sidedness = (ev.woL.y > 0.f) ? 1 : -1;
                        Bsdf<NS> b;
                        setup_bsdf(b, m, ev, hit);
                        float lightDistPdf = 1.f;
                        const float3 sp = hit.point, sn = hit.nS;
                        const LRef l = sample_light(hit.point, hit.nS, &lightDistPdf);
                        Spec<NS> Ld(0.f);
                        float scatteringPDF = 0.f, lightPDF = 0.f;
                        Spec<NS> Li = sample_li(l, ev, hit, lightPDF);
                        Spec<NS> f;
                        lightPDF *= lightDistPdf;
                        if (lightPDF > 0.f && !Li.black()) {
                            f = bsdf_f<NS>(b, ev) * fabsf(ev.wiL.y);
                            scatteringPDF = bsdf_pdf<NS>(b, ev.woL, ev.wiL);
                            if (!f.black() && scatteringPDF > 0.f) Ld += Li * f * power_heuristic(lightPDF, scatteringPDF) / lightPDF;
                        }
                        f = bsdf_sample<NS>(b, ev, hit, rng, scatteringPDF);
                        f *= fabsf(ev.wiL.y);
                        ro = hit.point;
                        rd = ev.wi;
                        ev.medium = get_medium(m, ev.wi, hit.nG);
                        scatterIntersect = intersect(ro, rd, hit);
                        if (scatteringPDF > 0.f && !f.black()) {
                            LRef nl; nl.light = scatterIntersect ? mat(hit).light : S.env_light; nl.tri = -1;
                            if (nl.light >= 0) {
                                if (!lref_eq(nl, l)) lightDistPdf = light_pdf(sp, sn, hit.prim, nl);
                                lightPDF = lightDistPdf * pdf_li(nl, ev, hit);
                                Li = scatterIntersect ? light_L(nl, ev, hit) : light_Le(nl, rd);
                                if (!Li.black() && lightPDF > 0.f) Ld += Li * f * power_heuristic(scatteringPDF, lightPDF) / scatteringPDF;
                            }
                        } else break;
                        L += beta * Ld;
                        beta *= f / scatteringPDF;
                    } else {
                        ev.medium = get_medium(m, rd, hit.nG);
                        ro = hit.point + hit.nG * (dot(hit.nG, rd) < 0.f ? -SURFACE_EPSILON : SURFACE_EPSILON);
                        if (bounces > 0) scatterIntersect = intersect(ro, rd, hit);
                        if (++nullCrossings > 256) break;
                        bounces--;
                        continue;
                    }
                } else if (ev.medium >= 0) {
                    const DMedium &med = S.media[ev.medium];
                    ev.wo = -rd;
                    const float3 scatterPoint = ro + rd * distanceT;
                    hit.point = scatterPoint;   /* the surface hit's normal stays (the reference reuses the hit) */
                    float lightDistPdf = 1.f;
                    const float3 sp = hit.point, sn = hit.nS;
                    const LRef l = sample_light(hit.point, hit.nS, &lightDistPdf);
                    Spec<NS> Ld(0.f);
                    float scatteringPDF = 0.f, lightPDF = 0.f;
                    Spec<NS> Li = sample_li(l, ev, hit, lightPDF);
                    lightPDF *= lightDistPdf;
                    if (lightPDF > 0.f && !Li.black()) {
                        scatteringPDF = phase_hg(dot(ev.wo, ev.wi), med.g);
                        if (scatteringPDF > 0.f) Ld += Li * Spec<NS>(scatteringPDF) * power_heuristic(lightPDF, scatteringPDF) / lightPDF;
                    }
                    scatteringPDF = hg_sample(med.g, ev.wo, &ev.wi, rng);
                    ro = hit.point;
                    rd = ev.wi;
                    Spec<NS> Tr(1.f);
                    scatterIntersect = intersect_tr(ro, rd, hit, ev.medium, &Tr, -1.f);
                    if (scatteringPDF > 0.f) {
                        LRef nl; nl.light = scatterIntersect ? mat(hit).light : S.env_light; nl.tri = -1;
                        if (nl.light >= 0) {
                            if (!lref_eq(nl, l)) lightDistPdf = light_pdf(sp, sn, hit.prim, nl);
                            lightPDF = lightDistPdf * pdf_li(nl, ev, hit);
                            Li = scatterIntersect ? light_L(nl, ev, hit) : light_Le(nl, rd);
                            if (!Li.black() && lightPDF > 0.f) Ld += Li * Tr * power_heuristic(scatteringPDF, lightPDF) / scatteringPDF;
                        }
                    } else break;
                    ro = scatterPoint;
                    scatterIntersect = intersect(ro, rd, hit);
                    L += beta * Ld;
                }
                if (bounces > minBounces) {
                    const float q = smax(.05f, 1.f - spec_y<NS>(beta, lam));
                    if (rng.next() < q) break;
                    beta /= 1.f - q;
                }
            } else {
                if (bounces == 0 && S.env_light >= 0) L += env_le(rd) * beta;
                break;
            }
        }
        return L;
    }

    /* DirectLightingIntegrator::Li (src/integrators/DirectLightingIntegrator.cpp:13-29) with
     * Integrator::SampleOneLight / EstimateDirect (src/integrators/Integrator.cpp:5-55).  The
     * reference's quirks are kept: the BSDF-sampled light pdf is PDF_Li(event, sampler) (a ray query
     * from the shading point, without the mesh's triangle-selection factor), and the BSDF-sampled
     * hit counts only if its light is the sampled light object itself.  Null surfaces
     * are crossed with a 1e-4 offset (at most 256 times); an absent environment light gives 0, so does
     * a light-selection pdf that is not positive (the reference divides by it). */
    __device__ Spec<NS> Li_direct(float3 ro, float3 rd) {
        RayHit hit;
        hit.tFar = finf(); hit.uv = make_float2(0.f, 0.f);
        for (int guard = 0; guard < 256; ++guard) {
            if (!intersect(ro, rd, hit)) return S.env_light >= 0 ? env_le(rd) : Spec<NS>(0.f);
            const DMaterial &m = mat(hit);
            if (!m.has_bsdf) { ro = hit.point + rd * .0001f; continue; }
            Event ev;
            ev.wo = -rd; ev.wi = mk(0.f, 0.f, 0.f);
            ev.woL = ev_local(hit, ev.wo); ev.wiL = ev_local(hit, ev.wi);
            ev.sidedness = (ev.woL.y > 0.f) ? 1 : -1; ev.medium = -1; ev.eta = 1.001f; ev.mediumInteraction = false;
            Bsdf<NS> b;
            setup_bsdf(b, m, ev, hit);
            float lightPdf = 1.f;
            const LRef l = sample_light(hit.point, hit.nS, &lightPdf);
            if (l.light < 0) return Spec<NS>(0.f);
            const bool pdfOk = lightPdf > 0.f;   /* a zero or NaN selection pdf would make the estimate NaN */
            /* EstimateDirect */
            Spec<NS> Ld(0.f);
            float scatteringPDF = 0.f, lightPDF = 0.f;
            Spec<NS> Li = sample_li(l, ev, hit, lightPDF);
            if (lightPDF > 0.f && !Li.black()) {
                const Spec<NS> f = bsdf_f<NS>(b, ev) * fabsf(ev.wiL.y);
                scatteringPDF = bsdf_pdf<NS>(b, ev.woL, ev.wiL);
                if (!f.black() && scatteringPDF > 0.f) Ld += Li * f * power_heuristic(lightPDF, scatteringPDF) / lightPDF;
            }
            Spec<NS> f = bsdf_sample<NS>(b, ev, hit, rng, scatteringPDF);   /* moves hit.point off the surface */
            f *= fabsf(ev.wiL.y);
            if (scatteringPDF > 0.f && !f.black()) {
                lightPDF = pdf_li_dir(l, ev, hit);
                if (lightPDF == 0.f) return pdfOk ? Ld / lightPdf : Spec<NS>(0.f);
                const float w = power_heuristic(scatteringPDF, lightPDF);
                const float3 o2 = hit.point + hit.nG * .00001f;
                RayHit lh;
                lh.tFar = finf(); lh.uv = make_float2(0.f, 0.f);
                Spec<NS> Lc(0.f);
                if (intersect(o2, ev.wi, lh)) {
                    if (l.tri < 0 && mat(lh).light == l.light) {
                        Event be = ev;
                        be.wo = -ev.wi;
                        LRef lr; lr.light = l.light; lr.tri = -1;
                        Lc = light_L(lr, be, lh);
                    }
                } else {
                    Lc = light_Le(l, ev.wi);
                }
                if (!Lc.black()) Ld += f * Lc * w / scatteringPDF;
            }
            return pdfOk ? Ld / lightPdf : Spec<NS>(0.f);
        }
        return Spec<NS>(0.f);
    }

    /* UtilityIntegrator::Li of NormalPass (shading normal; the reference's green channel is
     * n.y / 2 + 1) and DepthPass(max depth 100, power 1, background (1, 0, 1))
     * (src/integrators/UtilityIntegrators.cpp:7-53), converted as Spectrum::FromRGB (reflectance). */
    __device__ Spec<NS> Li_pass(float3 ro, float3 rd, bool normal) {
        RayHit hit;
        hit.tFar = finf(); hit.uv = make_float2(0.f, 0.f);
        float3 c;
        if (intersect(ro, rd, hit)) {
            if (normal) c = mk(hit.nS.x * .5f + .5f, hit.nS.y * .5f + 1.f, hit.nS.z * .5f + .5f);
            else { const float d = powf(mag(hit.point - ro) / 100.f, 1.f); c = mk(d, d, d); }
        } else {
            c = normal ? mk(0.f, 0.f, 0.f) : mk(1.f, 0.f, 1.f);
        }
        return from_rgb<NS>(c.x, c.y, c.z, false, lam);
    }

    /* ---------------------------------------------------------------- path-replay adjoint
     * The same estimator as Li, replayed with the same random numbers, carrying forward the
     * log-derivatives of the path throughput with respect to the differentiated parameters:
     * every radiance contribution C added to L credits dLoss/dI . C . dlnC/dtheta to the
     * gradient.  Sampling decisions are held fixed (detached): the derivative of an estimator
     * f L / p with p fixed is (df / f) f L / p, and MIS weights summing to one need no derivative.
     * The reference's MIS weights do not always sum to one over the strategies (its light pdf for
     * a BSDF-sampled hit is the mesh light's, the sampled one the triangle's), so the weights are
     * differentiated too: d ln w of the power heuristic through the parameter-dependent pdf.
     * The reference also drops a surface vertex's light-sampled estimate when the BSDF sample
     * that follows it fails (a microfacet reflection below the horizon ends the path before the
     * estimate is added), so that estimate's expectation is scaled by the probability P(alpha)
     * of a valid BSDF sample.  Its derivative dP = integral over valid directions of dp/dalpha is
     * estimated on the same sample by (dp/dalpha) / p of the sampled direction, added to the
     * light-sampled estimate's log-derivative.
     * Parameters: texels of an image-texture albedo (Lambertian, linear), the roughness of one
     * material's first BSDF leaf (central difference of the BSDF value), the grey sigma_a and
     * sigma_s of one homogeneous medium (transmittance exp(-sigma_t len) and the sigma_s factor of
     * a scattering event).  RGB3 only. */
    struct TexEntry { int idx[4]; float w[4]; float3 inv; };

    __device__ void credit(const AdjArgs &A, const TexEntry *E, int ne, const Spec<NS> &C, float3 dl,
                           const Spec<NS> &Dr, const Spec<NS> &Dsa, const Spec<NS> &Dss, float g[3]) {
        const float cx = dl.x * C.c[0], cy = dl.y * C.c[1], cz = dl.z * C.c[2];
        g[0] += cx * Dr.c[0] + cy * Dr.c[1] + cz * Dr.c[2];
        g[1] += cx * Dsa.c[0] + cy * Dsa.c[1] + cz * Dsa.c[2];
        g[2] += cx * Dss.c[0] + cy * Dss.c[1] + cz * Dss.c[2];
        for (int e = 0; e < ne; ++e) {
            const float gx = cx * E[e].inv.x, gy = cy * E[e].inv.y, gz = cz * E[e].inv.z;
            for (int t = 0; t < 4; ++t) {
                if (E[e].w[t] == 0.f) continue;
                float *q = reinterpret_cast<float *>(&A.grad_tex[E[e].idx[t]]);
                atomicAdd(q + 0, gx * E[e].w[t]);
                atomicAdd(q + 1, gy * E[e].w[t]);
                atomicAdd(q + 2, gz * E[e].w[t]);
            }
        }
    }
    /* d ln f / d roughness of leaf 0 at the event's (woL, wiL): central difference */
    __device__ Spec<NS> dlnf_rough(const Bsdf<NS> &b, const Event &ev) {
        const float r = b.rough[0], h = 1e-3f * fmaxf(r, 0.05f);
        Bsdf<NS> bp = b, bm = b;
        bp.rough[0] = r + h;
        bm.rough[0] = r - h;
        const Spec<NS> f0 = bsdf_f<NS>(b, ev), fp = bsdf_f<NS>(bp, ev), fm = bsdf_f<NS>(bm, ev);
        Spec<NS> d(0.f);
        for (int c = 0; c < NS; ++c) d.c[c] = f0.c[c] > 0.f ? (fp.c[c] - fm.c[c]) / (2.f * h * f0.c[c]) : 0.f;
        return d;
    }
    /* d pdf / d roughness of leaf 0 at the event's directions: central difference */
    __device__ float dpdf_rough(const Bsdf<NS> &b, const Event &ev) {
        const float r = b.rough[0], h = 1e-3f * fmaxf(r, 0.05f);
        Bsdf<NS> bp = b, bm = b;
        bp.rough[0] = r + h;
        bm.rough[0] = r - h;
        return (bsdf_pdf<NS>(bp, ev.woL, ev.wiL) - bsdf_pdf<NS>(bm, ev.woL, ev.wiL)) / (2.f * h);
    }
    /* LdMediumPoint split into its light-sampled and phase-sampled terms, with the length each
     * term's transmittance spent inside the differentiated medium */
    __device__ void ld_medium_point_adj(Event &ev, RayHit &hit, float3 p, LRef lsLight, float3 lsPoint, float3 lsNormal,
                                        Spec<NS> lsLe, float &lsPdf, float3 &wiOut, float3 sp, float3 sn,
                                        Spec<NS> &T1, float &len1, Spec<NS> &T2, float &len2) {
        const DMedium &med = S.media[ev.medium];
        float partialLightPDF = lsPdf;
        hit.point = p;
        *trlen = 0.f;
        Spec<NS> Li = lsLe * visibility(lsLight, p, ev, hit, lsPoint, lsNormal, lsPdf);
        len1 = *trlen;
        float scatteringPDF, lightPDF = lsPdf;
        T1 = Spec<NS>(0.f);
        T2 = Spec<NS>(0.f);
        if (lightPDF > 0.f && !Li.black()) {
            scatteringPDF = phase_hg(dot(ev.wo, ev.wi), med.g);
            if (scatteringPDF > 0.f) {
                const float w = power_heuristic(lightPDF, scatteringPDF);
                T1 += Li * Spec<NS>(scatteringPDF) * w / lightPDF;
            }
        }
        scatteringPDF = hg_sample(med.g, ev.wo, &ev.wi, rng);
        wiOut = ev.wi;
        const float3 ro = p, rd = ev.wi;
        Spec<NS> Tr(1.f);
        *trlen = 0.f;
        const bool hs = intersect_tr(ro, rd, hit, ev.medium, &Tr, -1.f);
        len2 = *trlen;
        if (scatteringPDF > 0.f) {
            LRef nl; nl.light = hs ? mat(hit).light : S.env_light; nl.tri = -1;
            if (nl.light >= 0) {
                if (!lref_eq(nl, lsLight)) partialLightPDF = light_pdf(sp, sn, hit.prim, nl);
                lightPDF = partialLightPDF * pdf_li(nl, ev, hit);
                Li = hs ? light_L(nl, ev, hit) : light_Le(nl, rd);
                const float w = power_heuristic(scatteringPDF, lightPDF);
                if (!Li.black() && lightPDF > 0.f) T2 += Li * Tr * w / scatteringPDF;
            }
        }
    }

    /* Replay of Li (same control flow and random numbers) accumulating gradients; g = (roughness,
     * sigma_a, sigma_s), texel gradients go to A.grad_tex with atomics.  dl = dLoss/dI of the
     * path's pixel divided by the samples per pixel.  Returns the replayed radiance. */
    __device__ Spec<NS> Li_adj(float3 ro, float3 rd, int maxBounces, int minBounces, const AdjArgs &A, float3 dl, float g[3]) {
        Spec<NS> L(0.f), beta(1.f);
        Spec<NS> Dr(0.f), Dsa(0.f), Dss(0.f);   /* log-derivatives of beta */
        const Spec<NS> zero(0.f);
        TexEntry E[8];
        int ne = 0;
        float seglen = 0.f;
        trlen = &seglen;
        trmed = A.medium;
        const float invSigS = (A.medium >= 0 && S.media[A.medium].ss[0] > 0.f) ? 1.f / S.media[A.medium].ss[0] : 0.f;
        RayHit hit;
        hit.tFar = finf(); hit.uv = make_float2(0.f, 0.f);
        Event ev;
        ev.wo = -rd; ev.wi = mk(0.f, 0.f, 0.f); ev.woL = ev.wi; ev.wiL = ev.wi;
        ev.sidedness = 1; ev.medium = -1; ev.eta = 1.001f; ev.mediumInteraction = false;
        bool scatterIntersect = false;
        int nullCrossings = 0;
        for (int bounces = 0; bounces < maxBounces; ++bounces) {
            if (bounces == 0 ? intersect(ro, rd, hit) : scatterIntersect) {
                if (bounces == 0) {
                    const int li = mat(hit).light;
                    if (li >= 0) {
                        LRef lr; lr.light = li; lr.tri = -1;
                        if (ev.medium >= 0) {
                            const Spec<NS> C = light_L(lr, ev, hit) * medium_tr<NS>(S.media[ev.medium], hit.tFar);
                            L += C;
                            if (ev.medium == A.medium) credit(A, E, 0, C, dl, zero, Spec<NS>(-hit.tFar), Spec<NS>(-hit.tFar), g);
                        } else L += light_L(lr, ev, hit);
                    }
                }
                if (ev.medium >= 0) {
                    const DMedium &med = S.media[ev.medium];
                    const bool dm = ev.medium == A.medium;
                    float lsPdf = 1.f;
                    const float3 sp = hit.point, sn = hit.nS;
                    const LRef lsLight = sample_light(hit.point, hit.nS, &lsPdf);
                    float3 lsPoint, lsNormal = mk(0.f, 0.f, 0.f);
                    const Spec<NS> lsLe = sample_point(lsLight, ev, hit, lsPoint, lsNormal, lsPdf);
                    const int choice = (rng.next() > 0.5f) ? 0 : 1;
                    float distT, distPdf, eqT, eqPdf;
                    const Spec<NS> mTrD = medium_sample_distance<NS>(med, rng, ev, hit, &distT, &distPdf);
                    const bool intD = ev.mediumInteraction;
                    const Spec<NS> mTrE = medium_sample_equiangular<NS>(med, ro, rd, rng, ev, hit, lsPoint, &eqT, &eqPdf);
                    const bool intE = ev.mediumInteraction;
                    ev.mediumInteraction = intD && intE;
                    if (!ev.mediumInteraction) {
                        /* the distance sample's weight: Tr / P(pass) past the segment, or, when only
                         * the equiangular sample left the segment, the scattering form Tr sigma_s / pdf */
                        beta *= mTrD;
                        if (dm) { Dsa += Spec<NS>(-distT); Dss += Spec<NS>(-distT + (intD ? invSigS : 0.f)); }
                    }
                    if (ev.mediumInteraction) {
                        ev.wo = -rd;
                        const float3 mpD = ro + rd * distT, mpE = ro + rd * eqT;
                        const float distPdf2 = medium_pdf_distance<NS>(med, eqT);
                        const float eqPdf2 = medium_pdf_equiangular(ro, rd, lsPoint, hit.tFar, distT);
                        const float distW = power_heuristic(distPdf, eqPdf2);
                        const float eqW = power_heuristic(eqPdf, distPdf2);
                        float3 wiD, wiE;
                        Spec<NS> t1, t2;
                        float l1, l2;
                        /* the reference adds the medium-vertex estimate to L without the throughput */
                        ld_medium_point_adj(ev, hit, mpD, lsLight, lsPoint, lsNormal, lsLe, lsPdf, wiD, sp, sn, t1, l1, t2, l2);
                        const float sD = dm ? -distT : 0.f, sE = dm ? -eqT : 0.f, ks = dm ? invSigS : 0.f;
                        /* MIS weights through the distance-sampling pdf sigma_t exp(-sigma_t t) */
                        float wD = 0.f, wE = 0.f;
                        if (dm) {
                            const float sigT = S.media[A.medium].sa[0] + S.media[A.medium].ss[0];
                            const float a2 = distPdf * distPdf, b2 = eqPdf2 * eqPdf2;
                            const float c2 = eqPdf * eqPdf, d2 = distPdf2 * distPdf2;
                            if (a2 + b2 > 0.f) wD = 2.f * (1.f / sigT - distT) * b2 / (a2 + b2);
                            if (c2 + d2 > 0.f) wE = -2.f * (1.f / sigT - eqT) * d2 / (c2 + d2);
                        }
                        Spec<NS> C = t1 * mTrD * distW;
                        L += C;
                        credit(A, E, 0, C, dl, zero, Spec<NS>(sD - l1 + wD), Spec<NS>(sD - l1 + ks + wD), g);
                        C = t2 * mTrD * distW;
                        L += C;
                        credit(A, E, 0, C, dl, zero, Spec<NS>(sD - l2 + wD), Spec<NS>(sD - l2 + ks + wD), g);
                        ld_medium_point_adj(ev, hit, mpE, lsLight, lsPoint, lsNormal, lsLe, lsPdf, wiE, sp, sn, t1, l1, t2, l2);
                        C = t1 * mTrE * eqW;
                        L += C;
                        credit(A, E, 0, C, dl, zero, Spec<NS>(sE - l1 + wE), Spec<NS>(sE - l1 + ks + wE), g);
                        C = t2 * mTrE * eqW;
                        L += C;
                        credit(A, E, 0, C, dl, zero, Spec<NS>(sE - l2 + wE), Spec<NS>(sE - l2 + ks + wE), g);
                        ro = choice == 0 ? mpD : mpE;
                        rd = choice == 0 ? wiD : wiE;
                        scatterIntersect = intersect(ro, rd, hit);
                        beta *= (choice == 0 ? mTrD : mTrE);
                        const float s = choice == 0 ? sD : sE;
                        Dsa += Spec<NS>(s);
                        Dss += Spec<NS>(s + ks);
                    }
                } else ev.mediumInteraction = false;

                if (!ev.mediumInteraction) {
                    const DMaterial &m = mat(hit);
                    const int mi = S.objects[hit.obj].material;
                    if (m.has_bsdf) {
                        ev.wo = -rd;
                        ev.woL = ev_local(hit, ev.wo);
                        ev.wiL = ev_local(hit, ev.wi);
                        ev.sidedness = (ev.woL.y > 0.f) ? 1 : -1;
                        Bsdf<NS> b;
                        setup_bsdf(b, m, ev, hit);
                        if (mi == A.tex_material && ne < 8) {   /* albedo = bilinear texel blend */
                            TexEntry &e = E[ne++];
                            image_bilinear(S.env_tex, A.tex_off, A.tex_w, A.tex_h, hit.uv, e.idx, e.w);
                            const Spec<NS> a = b.alb[0];
                            e.inv = make_float3(a.c[0] > 0.f ? 1.f / a.c[0] : 0.f, a.c[1] > 0.f ? 1.f / a.c[1] : 0.f,
                                                a.c[2] > 0.f ? 1.f / a.c[2] : 0.f);
                        }
                        const bool dr = mi == A.rough_material;
                        float lightDistPdf = 1.f;
                        const float3 sp = hit.point, sn = hit.nS;
                        const LRef l = sample_light(hit.point, hit.nS, &lightDistPdf);
                        Spec<NS> LdN(0.f), LdS(0.f), DrN(0.f), DrS(0.f);
                        float scatteringPDF = 0.f, lightPDF = 0.f;
                        seglen = 0.f;
                        Spec<NS> Li = sample_li(l, ev, hit, lightPDF);
                        const float lenN = seglen;
                        Spec<NS> f;
                        lightPDF *= lightDistPdf;
                        if (lightPDF > 0.f && !Li.black()) {
                            f = bsdf_f<NS>(b, ev) * fabsf(ev.wiL.y);
                            scatteringPDF = bsdf_pdf<NS>(b, ev.woL, ev.wiL);
                            if (!f.black() && scatteringPDF > 0.f) {
                                const float w = power_heuristic(lightPDF, scatteringPDF);
                                LdN += Li * f * w / lightPDF;
                                if (dr) {
                                    const float pL2 = lightPDF * lightPDF, pS = scatteringPDF;
                                    DrN = dlnf_rough(b, ev) + Spec<NS>(-2.f * pS * dpdf_rough(b, ev) / (pL2 + pS * pS));
                                }
                            }
                        }
                        f = bsdf_sample<NS>(b, ev, hit, rng, scatteringPDF);
                        f *= fabsf(ev.wiL.y);
                        float dpS = 0.f;
                        if (dr) { DrS = dlnf_rough(b, ev); dpS = dpdf_rough(b, ev); }
                        Spec<NS> DwS(0.f);
                        ro = hit.point;
                        rd = ev.wi;
                        ev.medium = get_medium(m, ev.wi, hit.nG);
                        scatterIntersect = intersect(ro, rd, hit);
                        if (scatteringPDF > 0.f && !f.black()) {
                            LRef nl; nl.light = scatterIntersect ? mat(hit).light : S.env_light; nl.tri = -1;
                            if (nl.light >= 0) {
                                if (!lref_eq(nl, l)) lightDistPdf = light_pdf(sp, sn, hit.prim, nl);
                                lightPDF = lightDistPdf * pdf_li(nl, ev, hit);
                                Li = scatterIntersect ? light_L(nl, ev, hit) : light_Le(nl, rd);
                                const float w = power_heuristic(scatteringPDF, lightPDF);
                                if (!Li.black() && lightPDF > 0.f) {
                                    LdS += Li * f * w / scatteringPDF;
                                    if (dr) {
                                        const float pL2 = lightPDF * lightPDF, pS = scatteringPDF;
                                        DwS = Spec<NS>(2.f * dpS / pS * pL2 / (pL2 + pS * pS));
                                    }
                                }
                            }
                        } else break;
                        const Spec<NS> CN = beta * LdN, CS = beta * LdS;
                        L += CN + CS;
                        /* dpS / pS: score of the BSDF sample's validity, which keeps the light estimate */
                        credit(A, E, ne, CN, dl, Dr + DrN + Spec<NS>(dpS / scatteringPDF), Dsa + Spec<NS>(-lenN),
                               Dss + Spec<NS>(-lenN), g);
                        credit(A, E, ne, CS, dl, Dr + DrS + DwS, Dsa, Dss, g);
                        beta *= f / scatteringPDF;
                        Dr += DrS;
                    } else {
                        ev.medium = get_medium(m, rd, hit.nG);
                        ro = hit.point + hit.nG * (dot(hit.nG, rd) < 0.f ? -SURFACE_EPSILON : SURFACE_EPSILON);
                        if (bounces > 0) scatterIntersect = intersect(ro, rd, hit);
                        if (++nullCrossings > 256) break;
                        bounces--;
                        continue;
                    }
                }
                if (bounces > minBounces) {
                    const float q = smax(.05f, 1.f - spec_y<NS>(beta, lam));
                    if (rng.next() < q) break;
                    beta /= 1.f - q;
                }
            } else {
                if (bounces == 0 && S.env_light >= 0) L += env_le(rd) * beta;
                break;
            }
        }
        trlen = nullptr;
        return L;
    }

    /* MISVolumetricPathIntegrator::Li (MISVolumetricPathIntegrator.cpp:71-215) */
    __device__ Spec<NS> Li(float3 ro, float3 rd, int maxBounces, int minBounces) {
        Spec<NS> L(0.f), beta(1.f);
        RayHit hit;
        hit.tFar = finf(); hit.uv = make_float2(0.f, 0.f);
        Event ev;
        ev.wo = -rd; ev.wi = mk(0.f, 0.f, 0.f); ev.woL = ev.wi; ev.wiL = ev.wi;
        ev.sidedness = 1; ev.medium = -1; ev.eta = 1.001f; ev.mediumInteraction = false;
        bool scatterIntersect = false;
        int nullCrossings = 0;   /* null surfaces do not count as bounces; bound them (256) */
        for (int bounces = 0; bounces < maxBounces; ++bounces) {
            if (bounces == 0 ? intersect(ro, rd, hit) : scatterIntersect) {
                if (bounces == 0) {
                    const int li = mat(hit).light;
                    if (li >= 0) {
                        LRef lr; lr.light = li; lr.tri = -1;
                        if (ev.medium >= 0) L += light_L(lr, ev, hit) * medium_tr<NS>(S.media[ev.medium], hit.tFar);
                        else L += light_L(lr, ev, hit);
                    }
                }
                if (ev.medium >= 0) {
                    const DMedium &med = S.media[ev.medium];
                    float lsPdf = 1.f;                                   /* B5 */
                    const float3 sp = hit.point, sn = hit.nS;            /* B7 */
                    const LRef lsLight = sample_light(hit.point, hit.nS, &lsPdf);
                    float3 lsPoint, lsNormal = mk(0.f, 0.f, 0.f);
                    const Spec<NS> lsLe = sample_point(lsLight, ev, hit, lsPoint, lsNormal, lsPdf);
                    const int choice = (rng.next() > 0.5f) ? 0 : 1;
                    float distT, distPdf, eqT, eqPdf;
                    const Spec<NS> mTrD = medium_sample_distance<NS>(med, rng, ev, hit, &distT, &distPdf);
                    const bool intD = ev.mediumInteraction;
                    const Spec<NS> mTrE = medium_sample_equiangular<NS>(med, ro, rd, rng, ev, hit, lsPoint, &eqT, &eqPdf);
                    const bool intE = ev.mediumInteraction;
                    ev.mediumInteraction = intD && intE;
                    if (!ev.mediumInteraction) beta *= mTrD;
                    if (ev.mediumInteraction) {
                        ev.wo = -rd;
                        Spec<NS> Ld(0.f);
                        const float3 mpD = ro + rd * distT, mpE = ro + rd * eqT;
                        const float distPdf2 = medium_pdf_distance<NS>(med, eqT);
                        const float eqPdf2 = medium_pdf_equiangular(ro, rd, lsPoint, hit.tFar, distT);
                        const float distW = power_heuristic(distPdf, eqPdf2);
                        const float eqW = power_heuristic(eqPdf, distPdf2);
                        float3 wiD, wiE;
                        const Spec<NS> liD = ld_medium_point(ev, hit, mpD, lsLight, lsPoint, lsNormal, lsLe, lsPdf, wiD, sp, sn);
                        Ld += liD * mTrD * distW;
                        const Spec<NS> liE = ld_medium_point(ev, hit, mpE, lsLight, lsPoint, lsNormal, lsLe, lsPdf, wiE, sp, sn);
                        Ld += liE * mTrE * eqW;
                        ro = choice == 0 ? mpD : mpE;
                        rd = choice == 0 ? wiD : wiE;
                        scatterIntersect = intersect(ro, rd, hit);
                        L += Ld;
                        beta *= (choice == 0 ? mTrD : mTrE);
                    }
                } else ev.mediumInteraction = false;

                if (!ev.mediumInteraction) {
                    const DMaterial &m = mat(hit);
                    if (m.has_bsdf) {
                        ev.wo = -rd;
                        ev.woL = ev_local(hit, ev.wo);
                        ev.wiL = ev_local(hit, ev.wi);
                        ev.sidedness = (ev.woL.y > 0.f) ? 1 : -1;
                        Bsdf<NS> b;
                        setup_bsdf(b, m, ev, hit);
                        float lightDistPdf = 1.f;
                        const float3 sp = hit.point, sn = hit.nS;   /* B7 */
                        const LRef l = sample_light(hit.point, hit.nS, &lightDistPdf);
                        Spec<NS> Ld(0.f);
                        float scatteringPDF = 0.f, lightPDF = 0.f;
                        Spec<NS> Li = sample_li(l, ev, hit, lightPDF);
                        Spec<NS> f;
                        lightPDF *= lightDistPdf;
                        if (lightPDF > 0.f && !Li.black()) {
                            f = bsdf_f<NS>(b, ev) * fabsf(ev.wiL.y);
                            scatteringPDF = bsdf_pdf<NS>(b, ev.woL, ev.wiL);
                            if (!f.black() && scatteringPDF > 0.f) {
                                const float w = power_heuristic(lightPDF, scatteringPDF);
                                Ld += Li * f * w / lightPDF;
                            }
                        }
                        f = bsdf_sample<NS>(b, ev, hit, rng, scatteringPDF);
                        f *= fabsf(ev.wiL.y);
                        ro = hit.point;
                        rd = ev.wi;
                        ev.medium = get_medium(m, ev.wi, hit.nG);
                        scatterIntersect = intersect(ro, rd, hit);
                        if (scatteringPDF > 0.f && !f.black()) {
                            LRef nl; nl.light = scatterIntersect ? mat(hit).light : S.env_light; nl.tri = -1;
                            if (nl.light >= 0) {
                                if (!lref_eq(nl, l)) lightDistPdf = light_pdf(sp, sn, hit.prim, nl);
                                lightPDF = lightDistPdf * pdf_li(nl, ev, hit);
                                Li = scatterIntersect ? light_L(nl, ev, hit) : light_Le(nl, rd);
                                const float w = power_heuristic(scatteringPDF, lightPDF);
                                if (!Li.black() && lightPDF > 0.f) Ld += Li * f * w / scatteringPDF;
                            }
                        } else break;
                        L += beta * Ld;
                        beta *= f / scatteringPDF;
                    } else {
                        ev.medium = get_medium(m, rd, hit.nG);
                        ro = hit.point + hit.nG * (dot(hit.nG, rd) < 0.f ? -SURFACE_EPSILON : SURFACE_EPSILON);
                        if (bounces > 0) scatterIntersect = intersect(ro, rd, hit);
                        if (++nullCrossings > 256) break;
                        bounces--;
                        continue;
                    }
                }
                if (bounces > minBounces) {
                    const float q = smax(.05f, 1.f - spec_y<NS>(beta, lam));
                    if (rng.next() < q) break;
                    beta /= 1.f - q;
                }
            } else {
                if (bounces == 0 && S.env_light >= 0) L += env_le(rd) * beta;
                break;
            }
        }
        return L;
    }
};

}  // namespace lg
