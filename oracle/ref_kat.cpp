/*
 * ref_kat.cpp -- golden-vector driver over the reference renderer's OWN translation units.
 * TEST INFRASTRUCTURE ONLY: built by oracle/build_ref.py into oracle/_ref/ together with the
 * reference's Fresnel.cpp, HenyeyGreenstein.cpp, HomogeneousMedium.cpp, Spectrum.cpp,
 * SPD_Data.cpp, Piecewise.cpp, Camera.cpp, Aperture.cpp and TextureEncoding.cpp compiled where they
 * lie; used to pin the oracle's restatement of those functions (tests/golden).  Each entry point calls the reference function named beside it
 * with fixed inputs; random numbers come from a sampler that replays given values.
 */
#include <Lambda.h>
#include <camera/Camera.h>
#include <image/Texture.h>
#include <sampling/Sampling.h>
#include <core/Ray.h>
#include <core/Spectrum.h>
#include <sampling/Piecewise.h>
#include <sampling/Sampler.h>
#include <shading/Fresnel.h>
#include <shading/ScatterEvent.h>
#include <shading/media/HenyeyGreenstein.h>
#include <shading/media/HomogeneousMedium.h>

using namespace lambda;

namespace {

/* Sampler (sampling/Sampler.h:9-25) replaying a fixed list of numbers. */
struct ReplaySampler : Sampler {
    const float *u;
    int n, i = 0;
    ReplaySampler(const float *u_, int n_) : u(u_), n(n_) {}
    Sampler *clone() const override { return nullptr; }
    void NextSample() override {}
    void SetSample(const unsigned) override {}
    Real Get1D() override { return i < n ? u[i++] : (Real).5; }
    Vec2 Get2D() override { const Real a = Get1D(); const Real b = Get1D(); return Vec2(a, b); }
};

Spectrum spec3(const float *v) { Spectrum s; s[0] = v[0]; s[1] = v[1]; s[2] = v[2]; return s; }

}  // namespace

#define REF_API extern "C" __attribute__((visibility("default")))

/* Fresnel::FrDielectric (shading/Fresnel.cpp:5-20) */
REF_API float ref_fr_dielectric(float c, float ei, float et) { return Fresnel::FrDielectric(c, ei, et); }

/* FresnelDielectric(etaT).Evaluate(cosI, etaArg) (shading/Fresnel.cpp:55-57), first channel */
REF_API float ref_fresnel_dielectric_eval(float etaT, float cosI, float etaArg) {
    FresnelDielectric f(etaT);
    return f.Evaluate(cosI, etaArg)[0];
}

/* HenyeyGreenstein::p (shading/media/HenyeyGreenstein.cpp:18-20) */
REF_API float ref_hg_p(float g, const float *wo, const float *wi) {
    HenyeyGreenstein h(g);
    return h.p(Vec3(wo[0], wo[1], wo[2]), Vec3(wi[0], wi[1], wi[2]));
}

/* HenyeyGreenstein::Sample_p (HenyeyGreenstein.cpp:22-36): returns the pdf, writes wi */
REF_API float ref_hg_sample(float g, const float *wo, float u0, float u1, float *wi) {
    HenyeyGreenstein h(g);
    const float u[2] = {u0, u1};
    ReplaySampler s(u, 2);
    Vec3 w;
    const float pdf = h.Sample_p(Vec3(wo[0], wo[1], wo[2]), &w, s);
    wi[0] = w.x; wi[1] = w.y; wi[2] = w.z;
    return pdf;
}

/* HomogeneousMedium (shading/media/HomogeneousMedium.cpp): out[0..2] = Tr(tFar),
 * out[3] = SampleDistance t, out[4] = its pdf, out[5..7] = its weight, out[8] = mediumInteraction,
 * out[9] = PDFDistance(tFar), out[10] = PDFEquiangular(ray, light point, tFar, t_eq) */
REF_API void ref_medium(const float *sa, const float *ss, const float *ray6, float tFar, float u0, float u1,
                        const float *lp, float t_eq, float *out) {
    HomogeneousMedium m(spec3(sa), spec3(ss));
    const Ray r(Vec3(ray6[0], ray6[1], ray6[2]), Vec3(ray6[3], ray6[4], ray6[5]));
    const float u[2] = {u0, u1};
    ReplaySampler s(u, 2);
    const Spectrum tr = m.Tr(r, tFar, s);
    out[0] = tr[0]; out[1] = tr[1]; out[2] = tr[2];
    RayHit hit;
    hit.tFar = tFar;
    ScatterEvent ev;
    ev.hit = &hit;
    Real t = 0, pdf = 0;
    const Spectrum w = m.SampleDistance(r, s, ev, &t, &pdf);
    out[3] = t; out[4] = pdf; out[5] = w[0]; out[6] = w[1]; out[7] = w[2];
    out[8] = ev.mediumInteraction ? 1.f : 0.f;
    out[9] = m.PDFDistance(tFar);
    out[10] = m.PDFEquiangular(r, Vec3(lp[0], lp[1], lp[2]), tFar, t_eq);
}

/* RGBSpectrum::FromSampled (core/Spectrum.h:353-372) */
REF_API void ref_rgb_from_sampled(const float *lam, const float *v, int n, float *rgb) {
    const Spectrum s = RGBSpectrum::FromSampled(lam, v, (unsigned)n);
    rgb[0] = s[0]; rgb[1] = s[1]; rgb[2] = s[2];
}

/* SpectrumUtils::XYZToRGB / RGBToXYZ (core/Spectrum.h:194-205), RGBSpectrum::y (:328-331) */
REF_API void ref_xyz_to_rgb(const float *xyz, float *rgb) { SpectrumUtils::XYZToRGB(xyz, rgb); }
REF_API void ref_rgb_to_xyz(const float *rgb, float *xyz) { SpectrumUtils::RGBToXYZ(rgb, xyz); }
REF_API float ref_rgb_y(const float *rgb) { return spec3(rgb).y(); }

/* SampledSpectrum::FromRGB (core/Spectrum.cpp:104-187): 32 bins over [400, 700] nm */
REF_API int ref_sampled_from_rgb(const float *rgb, int illum, float *out) {
    static bool init = false;
    if (!init) { SampledSpectrum::Init(); init = true; }
    const SampledSpectrum s = SampledSpectrum::FromRGB(rgb, illum ? SpectrumType::Illuminant : SpectrumType::Reflectance);
    for (unsigned i = 0; i < nSpectralSamples; ++i) out[i] = s[i];
    return (int)nSpectralSamples;
}

/* Distribution::Piecewise1D (sampling/Piecewise.cpp:9-44): out = SampleContinuous value, pdf,
 * offset; SampleDiscrete index, pdf, remapped u; PDF(index) */
REF_API void ref_piecewise1d(const float *f, int n, float u, float *out) {
    Distribution::Piecewise1D d(f, (unsigned)n);
    Real pdf = 0; int off = 0;
    out[0] = d.SampleContinuous(u, &pdf, &off);
    out[1] = pdf; out[2] = (float)off;
    Real dp = 0, ur = 0;
    const unsigned i = d.SampleDiscrete(u, &dp, &ur);
    out[3] = (float)i; out[4] = dp; out[5] = ur;
    out[6] = d.PDF(i);
}

/* Distribution::Piecewise2D (sampling/Piecewise.cpp:50-76): out = sample x, y, pdf, PDF(x, y) */
REF_API void ref_piecewise2d(const float *f, int nu, int nv, float u0, float u1, float *out) {
    Distribution::Piecewise2D d(f, (unsigned)nu, (unsigned)nv);
    Real pdf = 0;
    const Vec2 x = d.SampleContinuous(Vec2(u0, u1), &pdf);
    out[0] = x.x; out[1] = x.y; out[2] = pdf; out[3] = d.PDF(x);
}

/* PinholeCamera / ThinLensCamera / SphericalCamera::GenerateRay (camera/Camera.cpp:41-71) with a
 * CircularAperture or BladeAperture (camera/Aperture.cpp:10-27) drawing from ap_u.
 * type 0 pinhole, 1 thin lens, 2 spherical; aperture 0 none, 1 circular, 2 blade. */
REF_API void ref_camera_ray(int type, const float *org, const float *xh, const float *yh, const float *zh, float fov,
                            int W, int H, float focal, int aperture, float size, int blades, float offPhi,
                            float offTheta, float u, float v, const float *ap_u, float *o, float *d) {
    ReplaySampler s(ap_u, 8);
    const Vec3 origin(org[0], org[1], org[2]);
    std::unique_ptr<Aperture> ap;
    if (aperture == 1) ap.reset(new CircularAperture(size));
    if (aperture == 2) ap.reset(new BladeAperture((unsigned)blades, size));
    std::unique_ptr<Camera> cam;
    if (type == 1) cam.reset(new ThinLensCamera(origin, (Real)W, (Real)H, focal, ap.get()));
    else if (type == 2) {
        SphericalCamera *sc = new SphericalCamera(origin);
        sc->offsetPhi = offPhi;
        sc->offsetTheta = offTheta;
        cam.reset(sc);
    } else cam.reset(new PinholeCamera(origin, (Real)W, (Real)H));
    cam->SetAxes(Vec3(xh[0], xh[1], xh[2]), Vec3(yh[0], yh[1], yh[2]), Vec3(zh[0], zh[1], zh[2]));
    cam->SetFov(fov);
    const Ray r = cam->GenerateRay(u, v, s);
    for (int k = 0; k < 3; ++k) { o[k] = r.o[k]; d[k] = r.d[k]; }
}

/* texture_t<Colour>::GetPixelUV -> GetPixelUVBilinear (image/Texture.h:71-81, 159-168) over w x h RGBA texels */
REF_API void ref_texture_bilinear(const float *rgba, int w, int h, float u, float v, float *out) {
    texture_t<Colour> t((unsigned)w, (unsigned)h);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const float *p = rgba + 4 * ((size_t)y * w + x);
            t.SetPixelCoord((unsigned)x, (unsigned)y, Colour(p[0], p[1], p[2], p[3]));
        }
    const Colour c = t.GetPixelUV(u, v);   /* interpolation defaults to INTERP_BILINEAR (Texture.h:84) */
    out[0] = c.r; out[1] = c.g; out[2] = c.b; out[3] = c.a;
}

/* Sampling::SampleCosineHemisphere (sampling/Sampling.h:15-19) */
REF_API void ref_cos_hemisphere(float u0, float u1, float *out) {
    const Vec3 w = Sampling::SampleCosineHemisphere(Vec2(u0, u1));
    out[0] = w.x; out[1] = w.y; out[2] = w.z;
}
