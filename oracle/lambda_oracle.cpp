/*
 * lambda_oracle.cpp -- CPU ORACLE.  TEST INFRASTRUCTURE ONLY.
 *
 * A scalar C++ restatement of the Lambda renderer's MIS volumetric path-tracing hot path, written
 * function by function after the reference sources cited beside each piece.  It is the checker
 * for the GPU module (tests, __graft_entry__.smoke, and bench.py's CPU baseline leg) and is never
 * linked into, called by, or shipped with the product library.
 *
 * Structure follows the reference: a virtual Light hierarchy, pull-based shader-graph sockets,
 * BxDFs that call back into sockets, a pointer-linked light tree, and a per-path recursive
 * integrator.  Embree (absent) is restated as a two-level binned-SAH BVH2 with a two-sided
 * Moller-Trumbore triangle test: tnear = 0, closest hit, u/v with p = (1-u-v)p0 + u p1 + v p2,
 * unnormalised Ng = cross(v1 - v0, v2 - v0), occlusion = any hit with t in (0, tfar].
 *
 * Where the reference has undefined behaviour or an outright defect on the hot path, the oracle
 * applies the documented patch (ids B2..B26); every other quirk is kept so results match the
 * reference's own arithmetic.  Build with -ffp-contract=off so x86 and Arm hosts agree.
 *
 * Parity status: partly pinned.  Fresnel, Henyey-Greenstein, the homogeneous medium, the spectrum
 * conversions (RGB from samples, XYZ to RGB, luminance, Smits upsampling) and the piecewise
 * distributions are checked against golden vectors computed by the reference's own translation
 * units (oracle/build_ref.py, tests/golden).  Everything that includes the reference's shader
 * graph (BSDFs, microfacet distributions, graph nodes and noise, blackbody, lights, light tree,
 * integrator) cannot be compiled here -- g++ rejects ShaderGraph.h's class-scope explicit
 * specialisations and Embree/TBB are absent -- so those parts are parity unpinned: they rest on
 * this restatement read against the reference source.
 */
#include "../include/lambda_gpu.h"
#include "../lambda_gb300/csrc/lgpu_rng.h"
#include "../lambda_gb300/csrc/spectral_tables.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <list>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <vector>

namespace orc {

typedef float Real;
static const Real INF = std::numeric_limits<Real>::infinity();
static const Real MAX_REAL = std::numeric_limits<Real>::max();
constexpr Real PI = (Real)3.14159265358979323846264338;      /* maths.h:31 */
constexpr Real PI2 = (Real)2 * PI;
constexpr Real INV_PI = (Real)1 / PI;
constexpr Real INV_PI2 = (Real)1 / ((Real)2 * PI);
constexpr Real INV_PI4 = (Real)1 / ((Real)4 * PI);
constexpr Real SURFACE_EPSILON = (Real)1e-5;                   /* ScatterEvent.h:8 */

/* std::max / std::min exactly (NaN propagation of the first argument matters). */
static inline Real smax(Real a, Real b) { return (a < b) ? b : a; }
static inline Real smin(Real a, Real b) { return (b < a) ? b : a; }
static inline Real clampr(Real v, Real lo, Real hi) { return smax(smin(v, hi), lo); }

/* ------------------------------------------------------------------ vectors (maths/vec3.h) */
struct V3 {
    Real x = 0, y = 0, z = 0;
    V3() {}
    V3(Real a, Real b, Real c) : x(a), y(b), z(c) {}
    V3 operator+(const V3 &o) const { return V3(x + o.x, y + o.y, z + o.z); }
    V3 operator-(const V3 &o) const { return V3(x - o.x, y - o.y, z - o.z); }
    V3 operator*(const V3 &o) const { return V3(x * o.x, y * o.y, z * o.z); }
    V3 operator*(Real s) const { return V3(x * s, y * s, z * s); }
    V3 operator/(Real s) const { const Real inv = (Real)1 / s; return V3(x * inv, y * inv, z * inv); }
    V3 operator-() const { return *this * (Real)-1; }
    V3 &operator+=(const V3 &o) { x += o.x; y += o.y; z += o.z; return *this; }
    Real operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    Real Magnitude() const { return std::sqrt(x * x + y * y + z * z); }
    V3 Normalised() const { return *this / Magnitude(); }
};
struct V2 {
    Real x = 0, y = 0;
    V2() {}
    V2(Real a, Real b) : x(a), y(b) {}
    V2 operator+(const V2 &o) const { return V2(x + o.x, y + o.y); }
    V2 operator-(const V2 &o) const { return V2(x - o.x, y - o.y); }
    V2 operator*(Real s) const { return V2(x * s, y * s); }
};
static inline Real Dot(const V3 &a, const V3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline Real Dot2(const V2 &a, const V2 &b) { return a.x * b.x + a.y * b.y; }
static inline V3 Cross(const V3 &a, const V3 &b) {
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline Real DistSq(const V3 &a, const V3 &b) { const V3 d = b - a; return d.x * d.x + d.y * d.y + d.z * d.z; }
static inline V3 WorldToLocal(const V3 &v, const V3 &t, const V3 &n, const V3 &bt) {
    return V3(Dot(t, v), Dot(n, v), Dot(bt, v));
}
static inline V3 LocalToWorld(const V3 &v, const V3 &t, const V3 &n, const V3 &bt) {
    return V3(t.x * v.x + n.x * v.y + bt.x * v.z, t.y * v.x + n.y * v.y + bt.y * v.z,
              t.z * v.x + n.z * v.y + bt.z * v.z);
}
static inline V3 SphericalDirection(Real s, Real c, Real phi) {
    return V3(s * std::cos(phi), c, s * std::sin(phi));
}
static inline Real SphericalTheta(const V3 &v) { return std::acos(smax(smin(v.y, (Real)1), (Real)-1)); }
static inline Real SphericalPhi(const V3 &v) {
    const Real p = std::atan2(v.z, v.x);
    return (p < 0) ? (Real)(p + 3.14159265359 * 2.) : p;
}
static inline Real Lerp(Real a, Real b, Real r) { return a + (b - a) * r; }
static inline Real Fract(Real r) { return r - std::floor(r); }
template <class T> static inline T Bary(const T &a, const T &b, const T &c, Real u, Real v) {
    return a + (b - a) * u + (c - a) * v;
}
/* maths::Rotate, src/maths/vec3.h:230-234 (axis not normalised; sin from cos). */
static inline V3 Rotate(const V3 &v, const V3 &axis, Real theta) {
    const Real c = std::cos(theta);
    const Real s = std::sqrt((Real)1 - c * c);
    return v * c + Cross(axis, v) * s + axis * Dot(axis, v) * ((Real)1 - c);
}

struct Bounds {
    V3 min, max;   /* default-constructed bounds is the origin box (maths/bounds.h:12-15) */
    Bounds() {}
    Bounds(const V3 &p) : min(p), max(p) {}
    Bounds(const V3 &a, const V3 &b) : min(a), max(b) {}
    Real SurfaceArea() const { const V3 s = max - min; return (s.x * s.y + s.y * s.z + s.x * s.z) * (Real)2; }
    Real MaxLength() const { const V3 b = max - min; return smax(smax(b.x, b.y), b.z); }
    V3 Center() const { return min + (max - min) * (Real).5; }
    Real DiagonalLength() const { return (max - min).Magnitude(); }
    V3 Offset(const V3 &p) const { const V3 o = p - min, d = max - min; return V3(o.x / d.x, o.y / d.y, o.z / d.z); }
};
static inline Bounds Union(const Bounds &a, const Bounds &b) {
    return Bounds(V3(std::min(a.min.x, b.min.x), std::min(a.min.y, b.min.y), std::min(a.min.z, b.min.z)),
                  V3(std::max(a.max.x, b.max.x), std::max(a.max.y, b.max.y), std::max(a.max.z, b.max.z)));
}
static inline Bounds Union(const Bounds &b, const V3 &p) {
    return Bounds(V3(std::min(p.x, b.min.x), std::min(p.y, b.min.y), std::min(p.z, b.min.z)),
                  V3(std::max(p.x, b.max.x), std::max(p.y, b.max.y), std::max(p.z, b.max.z)));
}

/* maths::FindInterval, src/maths/maths.h:77-90 */
template <class P> static inline unsigned FindInterval(int size, const P &pred) {
    int first = 0, len = size;
    while (len > 0) {
        int half = len >> 1, middle = first + half;
        if (pred(middle)) { first = middle + 1; len -= half + 1; }
        else len = half;
    }
    return (unsigned)std::max(std::min(first - 1, size - 2), 0);
}

/* float -> unsigned as x86-64 g++ emits it (cvttss2si to 64 bits, keep low 32): NaN/inf -> 0. */
static inline unsigned ToUnsigned(Real x) {
    if (!(x == x) || std::isinf(x) || x >= 9.2e18f || x <= -9.2e18f) return 0u;
    return (unsigned)(uint64_t)(int64_t)x;
}

/* ------------------------------------------------------------------ spectrum (core/Spectrum.*) */
static int g_ns = 3;                         /* 3 = RGBSpectrum, 4 = hero wavelengths */
static thread_local Real t_lambda[4];        /* current path's hero wavelengths (nm) */

struct Spec {
    Real c[4] = {0, 0, 0, 0};
    Spec() {}
    explicit Spec(Real v) { for (int i = 0; i < 4; ++i) c[i] = (i < g_ns) ? v : 0; }
    Spec operator+(const Spec &o) const { Spec r; for (int i = 0; i < g_ns; ++i) r.c[i] = c[i] + o.c[i]; return r; }
    Spec operator-(const Spec &o) const { Spec r; for (int i = 0; i < g_ns; ++i) r.c[i] = c[i] - o.c[i]; return r; }
    Spec operator*(const Spec &o) const { Spec r; for (int i = 0; i < g_ns; ++i) r.c[i] = c[i] * o.c[i]; return r; }
    Spec operator/(const Spec &o) const { Spec r; for (int i = 0; i < g_ns; ++i) r.c[i] = c[i] / o.c[i]; return r; }
    Spec operator*(Real s) const { Spec r; for (int i = 0; i < g_ns; ++i) r.c[i] = c[i] * s; return r; }
    Spec operator/(Real s) const { Spec r; for (int i = 0; i < g_ns; ++i) r.c[i] = c[i] / s; return r; }
    Spec operator-() const { Spec r; for (int i = 0; i < g_ns; ++i) r.c[i] = -c[i]; return r; }
    Spec &operator+=(const Spec &o) { for (int i = 0; i < g_ns; ++i) c[i] += o.c[i]; return *this; }
    Spec &operator*=(const Spec &o) { for (int i = 0; i < g_ns; ++i) c[i] *= o.c[i]; return *this; }
    Spec &operator*=(Real s) { for (int i = 0; i < g_ns; ++i) c[i] *= s; return *this; }
    Spec &operator/=(Real s) { for (int i = 0; i < g_ns; ++i) c[i] /= s; return *this; }
    bool IsBlack() const { for (int i = 0; i < g_ns; ++i) if (c[i] != 0) return false; return true; }
    Real y() const;
};
static Spec SExp(const Spec &s) { Spec r; for (int i = 0; i < g_ns; ++i) r.c[i] = std::exp(s.c[i]); return r; }

/* CIE y-bar at a wavelength: linear interpolation in the 1 nm table. */
static inline Real CieAt(const float *tab, Real l) {
    if (l <= lgpu_cie_lambda[0]) return tab[0];
    if (l >= lgpu_cie_lambda[LGPU_N_CIE - 1]) return tab[LGPU_N_CIE - 1];
    const int i = (int)(l - lgpu_cie_lambda[0]);
    const int j = std::min(i, LGPU_N_CIE - 2);
    const Real t = (l - lgpu_cie_lambda[j]) / (lgpu_cie_lambda[j + 1] - lgpu_cie_lambda[j]);
    return tab[j] + (tab[j + 1] - tab[j]) * t;
}
static const Real HERO_RANGE = 340.0f;   /* 380-720 nm */

/* RGBSpectrum::y (Spectrum.h:328-331); hero mode: Monte-Carlo luminance of the 4 samples. */
Real Spec::y() const {
    if (g_ns == 3) {
        const Real YWeight[3] = {0.212671f, 0.715160f, 0.072169f};
        return YWeight[0] * c[0] + YWeight[1] * c[1] + YWeight[2] * c[2];
    }
    Real s = 0;
    for (int i = 0; i < 4; ++i) s += c[i] * CieAt(lgpu_cie_y, t_lambda[i]);
    return s * (HERO_RANGE / (4.0f * LGPU_CIE_Y_INTEGRAL));
}

/* InterpolateSpectrumSamples over the 32-knot Smits grid (Spectrum.cpp:195-201). */
static inline Real SmitsAt(const float *curve, Real l) {
    if (l <= lgpu_smits_lambda[0]) return curve[0];
    if (l >= lgpu_smits_lambda[LGPU_N_SMITS - 1]) return curve[LGPU_N_SMITS - 1];
    const unsigned off = FindInterval(LGPU_N_SMITS, [&](int i) { return lgpu_smits_lambda[i] <= l; });
    const Real t = (l - lgpu_smits_lambda[off]) / (lgpu_smits_lambda[off + 1] - lgpu_smits_lambda[off]);
    return Lerp(curve[off], curve[off + 1], t);
}

/* SampledSpectrum::FromRGB (Spectrum.cpp:104-187) evaluated at one wavelength. */
static Real SmitsUpsample(const Real rgb[3], bool illum, Real l) {
    const float(*B)[32] = lgpu_smits_basis + (illum ? 7 : 0);
    enum { W = 0, C = 1, M = 2, Y = 3, R = 4, G = 5, Bl = 6 };
    Real r = 0;
    if (rgb[0] <= rgb[1] && rgb[0] <= rgb[2]) {
        r += SmitsAt(B[W], l) * rgb[0];
        if (rgb[1] <= rgb[2]) { r += SmitsAt(B[C], l) * (rgb[1] - rgb[0]); r += SmitsAt(B[Bl], l) * (rgb[2] - rgb[1]); }
        else { r += SmitsAt(B[C], l) * (rgb[2] - rgb[0]); r += SmitsAt(B[G], l) * (rgb[1] - rgb[2]); }
    } else if (rgb[1] <= rgb[0] && rgb[1] <= rgb[2]) {
        r += SmitsAt(B[W], l) * rgb[1];
        if (rgb[0] <= rgb[2]) { r += SmitsAt(B[M], l) * (rgb[0] - rgb[1]); r += SmitsAt(B[Bl], l) * (rgb[2] - rgb[0]); }
        else { r += SmitsAt(B[M], l) * (rgb[2] - rgb[1]); r += SmitsAt(B[R], l) * (rgb[0] - rgb[2]); }
    } else {
        r += SmitsAt(B[W], l) * rgb[2];
        if (rgb[0] <= rgb[1]) { r += SmitsAt(B[Y], l) * (rgb[0] - rgb[2]); r += SmitsAt(B[G], l) * (rgb[1] - rgb[0]); }
        else { r += SmitsAt(B[Y], l) * (rgb[1] - rgb[2]); r += SmitsAt(B[R], l) * (rgb[0] - rgb[1]); }
    }
    r *= illum ? 0.86445f : (Real).94;
    return smax(r, 0);
}

/* Spectrum::FromRGB: identity for RGBSpectrum (Spectrum.h:341-347); hero mode upsamples. */
static Spec FromRGB(const Real rgb[3], bool illum) {
    Spec s;
    if (g_ns == 3) { s.c[0] = rgb[0]; s.c[1] = rgb[1]; s.c[2] = rgb[2]; return s; }
    for (int i = 0; i < 4; ++i) s.c[i] = SmitsUpsample(rgb, illum, t_lambda[i]);
    return s;
}

/* XYZToRGB (Spectrum.h:194-198), double-precision constants as in the reference. */
static void XYZToRGB(const Real xyz[3], Real rgb[3]) {
    rgb[0] = (Real)(3.240479 * xyz[0] - 1.537150 * xyz[1] - 0.498535 * xyz[2]);
    rgb[1] = (Real)(-0.969256 * xyz[0] + 1.875991 * xyz[1] + 0.041556 * xyz[2]);
    rgb[2] = (Real)(0.055648 * xyz[0] - 0.204043 * xyz[1] + 1.057311 * xyz[2]);
}

/* RGBSpectrum::FromSampled (Spectrum.h:355-372) -> RGB.  Unsorted samples are first sorted by
 * (wavelength, value) pairs (SpectrumSamplesSorted / SortSpectrumSamples, Spectrum.cpp:23-39). */
static void RGBFromSampled(const Real *lam, const Real *v, unsigned n, Real out[3]) {
    for (unsigned i = 0; i + 1 < n; ++i) {
        if (lam[i] > lam[i + 1]) {
            std::vector<std::pair<Real, Real>> sv;
            for (unsigned k = 0; k < n; ++k) sv.push_back(std::make_pair(lam[k], v[k]));
            std::sort(sv.begin(), sv.end());
            std::vector<Real> sl(n), svv(n);
            for (unsigned k = 0; k < n; ++k) { sl[k] = sv[k].first; svv[k] = sv[k].second; }
            RGBFromSampled(sl.data(), svv.data(), n, out);
            return;
        }
    }
    Real xyz[3] = {0, 0, 0};
    for (int i = 0; i < LGPU_N_CIE; ++i) {
        const Real l = lgpu_cie_lambda[i];
        Real val;
        if (l <= lam[0]) val = v[0];
        else if (l >= lam[n - 1]) val = v[n - 1];
        else {
            const unsigned off = FindInterval((int)n, [&](int k) { return lam[k] <= l; });
            const Real t = (l - lam[off]) / (lam[off + 1] - lam[off]);
            val = Lerp(v[off], v[off + 1], t);
        }
        xyz[0] += val * lgpu_cie_x[i];
        xyz[1] += val * lgpu_cie_y[i];
        xyz[2] += val * lgpu_cie_z[i];
    }
    const Real scale = (Real)(lgpu_cie_lambda[LGPU_N_CIE - 1] - lgpu_cie_lambda[0]) / (Real)(LGPU_CIE_Y_INTEGRAL * LGPU_N_CIE);
    xyz[0] *= scale; xyz[1] *= scale; xyz[2] *= scale;
    XYZToRGB(xyz, out);
}

/* Planck's law and its peak normalisation (GraphInputs.cpp:87-104). */
static void Blackbody(const Real *lam, int n, Real T, Real *Le) {
    const Real c = 299792458;
    const Real h = 6.62606957e-34f;
    const Real kb = 1.3806488e-23f;
    for (int i = 0; i < n; ++i) {
        const Real l = (Real)((double)lam[i] * 1e-9);
        const Real lambda5 = l * l * l * l * l;
        Le[i] = ((Real)2 * h * c * c) / (lambda5 * (std::exp((h * c) / (l * kb * T)) - (Real)1));
    }
}
static void BlackbodyNormalized(const Real *lam, int n, Real T, Real *Le) {
    Blackbody(lam, n, T, Le);
    const Real lambdaMax = (Real)(2.8977721e-3 / T * 1e9);
    Real maxL;
    Blackbody(&lambdaMax, 1, T, &maxL);
    for (int i = 0; i < n; ++i) Le[i] /= maxL;
}
/* BlackbodyInput::MakeBlackbodySpectrum (GraphInputs.cpp:106-116). */
static Spec MakeBlackbody(Real T, unsigned samples) {
    Spec s;
    if (g_ns == 4) { BlackbodyNormalized(t_lambda, 4, T, s.c); return s; }
    std::vector<Real> lam(samples), v(samples);
    const int interval = 700 - 400;
    const Real inv = (Real)1 / samples;
    for (unsigned i = 0; i < samples; ++i) lam[i] = (Real)400 + (Real)interval * inv * (Real)i;
    BlackbodyNormalized(lam.data(), (int)samples, T, v.data());
    Real rgb[3];
    RGBFromSampled(lam.data(), v.data(), samples, rgb);
    s.c[0] = rgb[0]; s.c[1] = rgb[1]; s.c[2] = rgb[2];
    return s;
}

/* ------------------------------------------------------------------ sampler seam */
struct Sampler {
    uint32_t key = 0, dim = 0;
    const float *replay = nullptr;   /* known-answer tests only: replay these numbers instead */
    Real Get1D() { return replay ? replay[dim++] : lgpu_rng_float(key, dim++); }
    V2 Get2D() { const Real a = Get1D(); const Real b = Get1D(); return V2(a, b); }
};

/* ------------------------------------------------------------------ rays / hits / events */
struct Ray { V3 o, d; };
struct ObjectRec;
struct RayHit {
    V3 point, normalG, normalS, tangent, bitangent;
    V2 uv;
    const ObjectRec *object = nullptr;
    Real tFar = INF;
    unsigned primId = 0;
};
struct Medium;
struct Scene;
struct ScatterEvent {
    V3 wo, wi, woL, wiL;
    RayHit *hit = nullptr;
    int sidedness = 1;
    const Medium *medium = nullptr;
    const Scene *scene = nullptr;
    Real eta = 1.001f;
    bool mediumInteraction = false;
    V3 ToLocal(const V3 &v) const { return WorldToLocal(v, hit->tangent, hit->normalS, hit->bitangent); }
    V3 ToWorld(const V3 &v) const { return LocalToWorld(v, hit->tangent, hit->normalS, hit->bitangent); }
    void SurfaceLocalise() { woL = ToLocal(wo); wiL = ToLocal(wi); sidedness = (woL.y > 0) ? 1 : -1; }
};
static inline bool SameHemisphere(const V3 &a, const V3 &b) { return a.y * b.y > 0; }
static inline V3 Reflect(const V3 &w, const V3 &n) { return w - n * (Real)2 * Dot(n, w); }
static inline bool Refract(const V3 &w, const V3 &n, Real eta, V3 *wr) {
    const Real cosI = Dot(w, n);
    const Real sin2I = smax((Real)0, (Real)1 - cosI * cosI);
    const Real sin2T = eta * eta * sin2I;
    if (sin2T >= 1) { *wr = V3(-1, 1, -1) * w; return false; }
    const Real cosT = std::sqrt(1 - sin2T);
    *wr = w * -eta + n * (eta * cosI - cosT);
    return true;
}
static inline Real Cos2Theta(const V3 &w) { return w.y * w.y; }
static inline Real Sin2Theta(const V3 &w) { return smax((Real)0, (Real)1 - Cos2Theta(w)); }
static inline Real SinTheta(const V3 &w) { return std::sqrt(Sin2Theta(w)); }
static inline Real CosPhi(const V3 &w) { const Real s = SinTheta(w); return (s < (Real)0.000001) ? 0 : clampr(w.x / s, -1, 1); }
static inline Real SinPhi(const V3 &w) { const Real s = SinTheta(w); return (s < (Real)0.000001) ? 0 : clampr(w.z / s, -1, 1); }
static inline Real Cos2Phi(const V3 &w) { return CosPhi(w) * CosPhi(w); }
static inline Real Sin2Phi(const V3 &w) { return SinPhi(w) * SinPhi(w); }
static inline Real Tan2Theta(const V3 &w) { return Sin2Theta(w) / Cos2Theta(w); }
static inline Real TanTheta(const V3 &w) { return SinTheta(w) / w.y; }

/* ------------------------------------------------------------------ shader graph (src/shading/graph/) */
enum SockT { T_NULL = 0, T_SCALAR, T_COLOUR, T_VEC2, T_VEC3, T_SPECTRUM, T_BXDF };
struct Val {
    SockT t = T_NULL;
    Real v[4] = {0, 0, 0, 0};
    Spec s;
    int bxdf = -1;
};
/* texture_t::GetPixelUVBilinear (Texture.h:71-81) over RGBA texels in scanline rows */
static void TexBilinear(const float *t, int w, int h, Real u, Real v, Real out[4]) {
    const Real fx = std::min((float)(w - 1), clampr(u, 0.f, 1.f) * (float)w);
    const Real fy = std::min((float)(h - 1), clampr(v, 0.f, 1.f) * (float)h);
    const unsigned x = (unsigned)fx, y = (unsigned)fy;
    const unsigned x1 = std::min(x + 1, (unsigned)w - 1), y1 = std::min(y + 1, (unsigned)h - 1);
    for (int k = 0; k < 4; ++k) {
        const Real ya = Lerp(t[4 * ((size_t)y * w + x) + k], t[4 * ((size_t)y * w + x1) + k], fx - (float)x);
        const Real yb = Lerp(t[4 * ((size_t)y1 * w + x) + k], t[4 * ((size_t)y1 * w + x1) + k], fx - (float)x);
        out[k] = Lerp(ya, yb, fy - (float)y);
    }
}
struct Graph;
static Val EvalOutput(const Graph &g, int node, int out, const ScatterEvent &ev);

struct Graph {
    std::vector<lgpu_node_desc> nodes;
    std::vector<std::vector<float>> tex;   /* image textures: RGBA texels, scanline rows */
    std::vector<int> texW, texH;
    static SockT OutType(int type, int out) {
        switch (type) {
        case LGPU_NODE_BXDF_MIX: case LGPU_NODE_BXDF_LAMBERTIAN: case LGPU_NODE_BXDF_OREN_NAYAR_R:
        case LGPU_NODE_BXDF_OREN_NAYAR_T: case LGPU_NODE_BXDF_MICROFACET_R: case LGPU_NODE_BXDF_FRESNEL:
        case LGPU_NODE_BXDF_SPECULAR_R: case LGPU_NODE_BXDF_SPECULAR_T: case LGPU_NODE_BXDF_GHOST: return T_BXDF;
        case LGPU_NODE_SEPARATE_XYZ: case LGPU_NODE_SEPARATE_RGBA: return T_SCALAR;
        case LGPU_NODE_MERGE_XYZ: return T_VEC3;
        case LGPU_NODE_MERGE_RGBA: return T_COLOUR;
        case LGPU_NODE_SCALAR: return T_SCALAR;
        case LGPU_NODE_VECTOR3: return T_VEC3;
        case LGPU_NODE_VECTOR2: return T_VEC2;
        case LGPU_NODE_RGB: return T_COLOUR;
        case LGPU_NODE_SPECTRUM: case LGPU_NODE_BLACKBODY: return T_SPECTRUM;
        case LGPU_NODE_SURFACE_INFO: return T_VEC3;
        case LGPU_NODE_IMAGE_TEXTURE: return out == 0 ? T_COLOUR : T_SCALAR;
        case LGPU_NODE_MATHS: case LGPU_NODE_DOT_PRODUCT: case LGPU_NODE_VECTOR_MAGNITUDE: return T_SCALAR;
        case LGPU_NODE_VECTOR_MATHS: case LGPU_NODE_CROSS_PRODUCT: return T_VEC3;
        case LGPU_NODE_PERLIN_NOISE: case LGPU_NODE_VALUE_NOISE: case LGPU_NODE_OCTAVE_NOISE:
        case LGPU_NODE_CHECKER: case LGPU_NODE_VORONOI: return T_SCALAR;
        default: return T_NULL;
        }
    }
};

/* Socket::GetAs<Real> (ShaderGraph.h:90-127) */
static Real AsReal(const Val &v) {
    switch (v.t) {
    case T_SCALAR: return v.v[0];
    case T_COLOUR: return v.v[0] * (Real).3 + v.v[1] * (Real).59 + v.v[2] * (Real).11;
    case T_VEC2: return (v.v[0] + v.v[1]) * (Real).5;
    case T_VEC3: return (v.v[0] + v.v[1] + v.v[2]) * (Real).333333333333;
    case T_SPECTRUM: return v.s.y();
    default: return 0;
    }
}
/* GetAs<Colour> (ShaderGraph.h:129-167) */
static void AsColour(const Val &v, Real c[4]) {
    switch (v.t) {
    case T_COLOUR: for (int i = 0; i < 4; ++i) c[i] = v.v[i]; return;
    case T_SCALAR: c[0] = c[1] = c[2] = v.v[0]; c[3] = 1; return;
    case T_SPECTRUM: c[0] = v.s.c[0]; c[1] = v.s.c[1]; c[2] = v.s.c[2]; c[3] = 1; return;
    case T_VEC3: c[0] = v.v[0]; c[1] = v.v[1]; c[2] = v.v[2]; c[3] = 1; return;
    case T_VEC2: c[0] = c[1] = c[2] = (v.v[0] + v.v[1]) * (Real).5; c[3] = 1; return;
    default: c[0] = 1; c[1] = 0; c[2] = 1; c[3] = 1; return;
    }
}
static V2 AsVec2(const Val &v) {
    switch (v.t) {
    case T_VEC2: case T_VEC3: return V2(v.v[0], v.v[1]);
    case T_SCALAR: return V2(v.v[0], v.v[0]);
    default: return V2(0, 0);
    }
}
static V3 AsVec3(const Val &v) {
    switch (v.t) {
    case T_VEC3: return V3(v.v[0], v.v[1], v.v[2]);
    case T_VEC2: return V3(v.v[0], v.v[1], 0);
    case T_SCALAR: return V3(v.v[0], v.v[0], v.v[0]);
    default: return V3(0, 0, 0);
    }
}
/* Socket::GetAsSpectrum (ShaderGraph.h:232-251) */
static Spec AsSpectrum(const Val &v, bool illum) {
    switch (v.t) {
    case T_COLOUR: { Real c[4]; AsColour(v, c); return FromRGB(c, illum); }
    case T_SCALAR: return Spec(AsReal(v));
    case T_SPECTRUM: return v.s;
    default: return Spec(0);
    }
}

/* SocketRef input i of node n: linked socket or inline default (ShaderGraph.h:254-287). */
struct In {
    const Graph &g; int n; int i; const ScatterEvent &ev;
    bool linked() const { return g.nodes[n].in_node[i] >= 0; }
    Val pull() const { return EvalOutput(g, g.nodes[n].in_node[i], g.nodes[n].in_socket[i], ev); }
    const float *def() const { return g.nodes[n].in_default[i]; }
    Real real() const { return linked() ? AsReal(pull()) : def()[0]; }
    V2 vec2() const { return linked() ? AsVec2(pull()) : V2(def()[0], def()[1]); }
    V3 vec3() const { return linked() ? AsVec3(pull()) : V3(def()[0], def()[1], def()[2]); }
    void colour(Real c[4]) const { if (linked()) AsColour(pull(), c); else for (int k = 0; k < 4; ++k) c[k] = def()[k]; }
    /* SocketRef::GetAsSpectrum: unlinked -> raw data as a Spectrum (RGB); hero mode upsamples it. */
    Spec spectrum() const {
        if (linked()) return AsSpectrum(pull(), false);
        const Real rgb[3] = {def()[0], def()[1], def()[2]};
        return FromRGB(rgb, false);
    }
    int bxdf() const { return linked() ? pull().bxdf : -1; }
    SockT linkedType() const { return linked() ? Graph::OutType(g.nodes[g.nodes[n].in_node[i]].type, g.nodes[n].in_socket[i]) : T_NULL; }
};

/* Noise helpers (GraphTexture.cpp:8-50) */
static const double inv32 = 1. / 4294967296.;
static inline uint32_t Hash21(uint32_t x, uint32_t y) { x *= 1597334677u; y *= 3812015801u; return (x ^ y) * 1597334677u; }
static inline V2 Hash22(V2 v) {
    v = V2(Dot2(v, V2((Real)127.1, (Real)311.7)), Dot2(v, V2((Real)269.5, (Real)183.3)));
    const V2 s = V2(std::sin(v.x), std::sin(v.y)) * (Real)18.5453;
    return V2(Fract(s.x), Fract(s.y));
}
static inline V2 Gradient2D(Real u) { u *= PI2; return V2(std::cos(u), std::sin(u)); }
static inline Real Quintic(Real x) { return x * x * x * (x * (x * 6.f - 15.f) + 10.f); }
static inline Real Cubic(Real x) { return x * x * (3 - 2 * x); }
static inline uint32_t GridU(Real g) { return ToUnsigned(g); }
static Real Perlin2D(V2 tc, Real scale) {
    tc = tc * scale;
    const Real gx = std::floor(tc.x), gy = std::floor(tc.y);
    const V2 p00(gx, gy), p10(gx + 1, gy), p11(gx + 1, gy + 1), p01(gx, gy + 1);
    const V2 g00 = Gradient2D((Real)(Hash21(GridU(p00.x), GridU(p00.y)) * inv32));
    const V2 g10 = Gradient2D((Real)(Hash21(GridU(p10.x), GridU(p10.y)) * inv32));
    const V2 g11 = Gradient2D((Real)(Hash21(GridU(p11.x), GridU(p11.y)) * inv32));
    const V2 g01 = Gradient2D((Real)(Hash21(GridU(p01.x), GridU(p01.y)) * inv32));
    const Real d00 = Dot2(tc - p00, g00), d10 = Dot2(tc - p10, g10), d11 = Dot2(tc - p11, g11), d01 = Dot2(tc - p01, g01);
    const Real vx0 = Lerp(d00, d10, Quintic(tc.x - gx));
    const Real vx1 = Lerp(d01, d11, Quintic(tc.x - gx));
    return Lerp(vx0, vx1, Quintic(tc.y - gy)) + (Real).5;
}
static Real Value2D(V2 tc, Real scale) {
    tc = tc * scale;
    const V2 p00(std::floor(tc.x), std::floor(tc.y));
    const V2 p = tc - p00;
    const Real v00 = (Real)(Hash21(GridU(p00.x), GridU(p00.y)) * inv32);
    const Real v10 = (Real)(Hash21(GridU(p00.x + 1), GridU(p00.y)) * inv32);
    const Real v11 = (Real)(Hash21(GridU(p00.x + 1), GridU(p00.y + 1)) * inv32);
    const Real v01 = (Real)(Hash21(GridU(p00.x), GridU(p00.y + 1)) * inv32);
    const Real vx0 = Lerp(v00, v10, Cubic(p.x)), vx1 = Lerp(v01, v11, Cubic(p.x));
    return Lerp(vx0, vx1, Cubic(p.y));
}
static Real Checker2D(V2 tc, Real scale) {
    tc = tc * scale;
    tc = V2(Fract(tc.x), Fract(tc.y));
    return (tc.x > .5f) == (tc.y > .5f) ? 0 : 1;
}
static Real Checker3D(V3 p, Real scale) {
    p = p * scale;
    p = V3(Fract(p.x), Fract(p.y), Fract(p.z));
    return ((p.x > .5) == (p.y > .5)) == (p.z > .5) ? 0 : 1;
}
static Real Voronoi2D(V2 tc, Real scale) {
    tc = tc * scale;
    const V2 p00(std::floor(tc.x), std::floor(tc.y));
    Real m = INF;
    for (int y = -1; y < 2; ++y)
        for (int x = -1; x < 2; ++x) {
            const V2 off = p00 + V2((Real)x, (Real)y);
            const V2 rp = off + Hash22(off) - tc;
            const Real d2 = Dot2(rp, rp);
            if (d2 < m) m = d2;
        }
    return std::sqrt(m);
}
static inline V3 Fract3(const V3 &v) { return V3(Fract(v.x), Fract(v.y), Fract(v.z)); }
static inline V3 Hash33(V3 p) {
    p = Fract3(p * V3((Real).1031, (Real).1030, (Real).0973));
    const Real d = Dot(p, V3(p.y, p.x, p.z) + V3((Real)33.33, (Real)33.33, (Real)33.33));
    p = p + V3(d, d, d);
    return Fract3((V3(p.x, p.x, p.y) + V3(p.y, p.x, p.x)) * V3(p.z, p.y, p.z));
}
static Real Voronoi3D(V3 pt, Real scale) {
    pt = pt * scale;
    const V3 p00(std::floor(pt.x), std::floor(pt.y), std::floor(pt.z));
    Real m = INF;
    for (int z = -1; z < 2; ++z)
        for (int y = -1; y < 2; ++y)
            for (int x = -1; x < 2; ++x) {
                const V3 off = p00 + V3((Real)x, (Real)y, (Real)z);
                const V3 rp = off + Hash33(off) - pt;
                const Real d2 = Dot(rp, rp);
                if (d2 < m) m = d2;
            }
    return std::sqrt(m);
}
/* Noise::Get2D / Get3D dispatch for the node kinds usable inside OctaveNoise. */
static Real Noise2D(const Graph &g, int node, V2 tc) {
    const lgpu_node_desc &d = g.nodes[node];
    switch (d.type) {
    case LGPU_NODE_PERLIN_NOISE: return Perlin2D(tc, d.params[0]);
    case LGPU_NODE_VALUE_NOISE: return Value2D(tc, d.params[0]);
    case LGPU_NODE_CHECKER: return Checker2D(tc, d.params[0]);
    case LGPU_NODE_VORONOI: return Voronoi2D(tc, d.params[0]);
    case LGPU_NODE_OCTAVE_NOISE: {
        Real out = 0, amp = .5, scl = 1;
        const unsigned oct = (unsigned)d.params[1];
        for (unsigned i = 0; i < oct; ++i) { out += Noise2D(g, d.in_node[0], tc * d.params[0] * scl) * amp; scl *= 2; amp *= .5; }
        return out;
    }
    default: return 0;
    }
}
static Real Noise3D(const Graph &g, int node, V3 p) {
    const lgpu_node_desc &d = g.nodes[node];
    switch (d.type) {
    case LGPU_NODE_PERLIN_NOISE: return 0;    /* PerlinNoise::Get3D returns 0 (B13) */
    case LGPU_NODE_VALUE_NOISE: return 0;     /* ValueNoise::Get3D returns 0 (B13) */
    case LGPU_NODE_CHECKER: return Checker3D(p, d.params[0]);
    case LGPU_NODE_VORONOI: return Voronoi3D(p, d.params[0]);
    case LGPU_NODE_OCTAVE_NOISE: {
        Real out = 0, amp = .5, scl = 1;
        const unsigned oct = (unsigned)d.params[1];
        for (unsigned i = 0; i < oct; ++i) { out += Noise3D(g, d.in_node[0], p * d.params[0] * scl) * amp; scl *= 2; amp *= .5; }
        return out;
    }
    default: return 0;
    }
}

static Val EvalOutput(const Graph &g, int node, int out, const ScatterEvent &ev) {
    const lgpu_node_desc &d = g.nodes[node];
    Val r;
    r.t = Graph::OutType(d.type, out);
    auto in = [&](int i) { return In{g, node, i, ev}; };
    switch (d.type) {
    case LGPU_NODE_SCALAR: r.v[0] = d.params[0]; break;
    case LGPU_NODE_VECTOR2: r.v[0] = d.params[0]; r.v[1] = d.params[1]; break;
    case LGPU_NODE_VECTOR3: r.v[0] = d.params[0]; r.v[1] = d.params[1]; r.v[2] = d.params[2]; break;
    case LGPU_NODE_RGB: r.v[0] = d.params[0]; r.v[1] = d.params[1]; r.v[2] = d.params[2]; r.v[3] = 1; break;
    case LGPU_NODE_SPECTRUM: { const Real rgb[3] = {d.params[0], d.params[1], d.params[2]}; r.s = FromRGB(rgb, false); break; }
    case LGPU_NODE_BLACKBODY: r.s = MakeBlackbody(in(0).real(), (unsigned)d.params[0]); break;
    case LGPU_NODE_SURFACE_INFO: r.v[0] = ev.hit->normalS.x; r.v[1] = ev.hit->normalS.y; r.v[2] = ev.hit->normalS.z; break;
    case LGPU_NODE_IMAGE_TEXTURE: {   /* ImageTextureInput::GetColour / GetScalar (GraphInputs.cpp:128-136) */
        const int ti = (int)d.params[0];
        const std::vector<float> &t = g.tex[ti];
        const int w = g.texW[ti], h = g.texH[ti];
        TexBilinear(t.data(), w, h, Fract(ev.hit->uv.x), Fract(ev.hit->uv.y), r.v);
        if (out == 1) { r.v[1] = r.v[2] = r.v[3] = 0; }
        break;
    }
    case LGPU_NODE_SEPARATE_XYZ: {        /* B14: every output reads input 0 */
        const V3 v = in(0).vec3();
        r.v[0] = out == 0 ? v.x : (out == 1 ? v.y : v.z);
        break;
    }
    case LGPU_NODE_SEPARATE_RGBA: { Real c[4]; in(0).colour(c); r.v[0] = c[out]; break; }
    case LGPU_NODE_MERGE_XYZ: r.v[0] = in(0).real(); r.v[1] = in(1).real(); r.v[2] = in(2).real(); break;
    case LGPU_NODE_MERGE_RGBA: for (int i = 0; i < 4; ++i) r.v[i] = in(i).real(); break;
    case LGPU_NODE_MATHS: {
        const Real a = in(0).real();
        const Real b = (d.op == LGPU_MATHS_SQRT) ? 0 : in(1).real();
        switch (d.op) {
        case LGPU_MATHS_ADD: r.v[0] = a + b; break;
        case LGPU_MATHS_SUBTRACT: r.v[0] = a - b; break;
        case LGPU_MATHS_MULTIPLY: r.v[0] = a * b; break;
        case LGPU_MATHS_DIVIDE: r.v[0] = a / b; break;
        case LGPU_MATHS_SQRT: r.v[0] = std::sqrt(a); break;     /* B15 */
        case LGPU_MATHS_POWER: r.v[0] = std::pow(a, b); break;   /* B15 */
        }
        break;
    }
    case LGPU_NODE_VECTOR_MATHS: {
        const V3 a = in(0).vec3(), b = in(1).vec3();
        V3 o;
        switch (d.op) {
        case LGPU_MATHS_ADD: o = a + b; break;
        case LGPU_MATHS_SUBTRACT: o = a - b; break;
        case LGPU_MATHS_MULTIPLY: o = a * b; break;
        case LGPU_MATHS_DIVIDE: o = V3(a.x / b.x, a.y / b.y, a.z / b.z); break;
        default: break;
        }
        r.v[0] = o.x; r.v[1] = o.y; r.v[2] = o.z;
        break;
    }
    case LGPU_NODE_DOT_PRODUCT: r.v[0] = Dot(in(0).vec3(), in(1).vec3()); break;
    case LGPU_NODE_CROSS_PRODUCT: { const V3 o = Cross(in(0).vec3(), in(1).vec3()); r.v[0] = o.x; r.v[1] = o.y; r.v[2] = o.z; break; }
    case LGPU_NODE_VECTOR_MAGNITUDE: r.v[0] = in(0).vec3().Magnitude(); break;
    case LGPU_NODE_PERLIN_NOISE: case LGPU_NODE_VALUE_NOISE: case LGPU_NODE_OCTAVE_NOISE:
    case LGPU_NODE_CHECKER: case LGPU_NODE_VORONOI:
        r.v[0] = ev.mediumInteraction ? Noise3D(g, node, ev.hit->point) : Noise2D(g, node, ev.hit->uv);
        break;
    default:
        if (r.t == T_BXDF) r.bxdf = node;
        break;
    }
    return r;
}

/* ------------------------------------------------------------------ BxDFs (src/shading/surface/) */
static inline Real CosineHemispherePdf(const V3 &wo, const V3 &wi) { return SameHemisphere(wo, wi) ? std::abs(wi.y) * INV_PI : 0; }
static inline V3 SampleCosineHemisphere(const V2 &u) {   /* Sampling.h:9-19 */
    const Real r = std::sqrt(u.x);
    const Real theta = u.y * PI2;
    const V2 d(r * std::cos(theta), r * std::sin(theta));
    const Real up = std::sqrt(smax((Real)0, 1 - d.x * d.x - d.y * d.y));
    return V3(d.x, up, d.y);
}
/* Fresnel::FrDielectric (Fresnel.cpp:5-20) */
static Real FrDielectric(Real cosI, Real etaI, Real etaT) {
    cosI = clampr(cosI, -1, 1);
    if (cosI < 0) { std::swap(etaI, etaT); cosI = std::abs(cosI); }
    const Real sinI = std::sqrt(smax((Real)0, 1 - cosI * cosI));
    const Real sinT = etaI / etaT * sinI;
    if (sinT >= 1) return 1;
    const Real cosT = std::sqrt(smax((Real)0, 1 - sinT * sinT));
    const Real rPara = (etaT * cosI - etaI * cosT) / (etaT * cosI + etaI * cosT);
    const Real rPerp = (etaI * cosI - etaT * cosT) / (etaI * cosI + etaT * cosT);
    return (rPara * rPara + rPerp * rPerp) * (Real).5;
}
/* MicrofacetDistribution.cpp:11-71 */
static Real DistD(int dist, const V3 &wh, V2 a) {
    const Real tan2 = Tan2Theta(wh);
    if (std::isinf(tan2)) return 0.;
    const Real cos4 = Cos2Theta(wh) * Cos2Theta(wh);
    if (dist == LGPU_DIST_BECKMANN)
        return std::exp(-tan2 * (Cos2Phi(wh) / (a.x * a.x) + Sin2Phi(wh) / (a.y * a.y))) / (PI * a.x * a.y * cos4);
    const Real e = (Cos2Phi(wh) / (a.x * a.x) + Sin2Phi(wh) / (a.y * a.y)) * tan2;
    return (Real)1 / (PI * a.x * a.y * cos4 * (1 + e) * (1 + e));
}
static Real DistLambda(int dist, const V3 &w, V2 a) {
    const Real absTan = std::abs(TanTheta(w));
    if (std::isinf(absTan)) return 0.;
    const Real alpha = std::sqrt(Cos2Phi(w) * a.x * a.x + Sin2Phi(w) * a.y * a.y);
    if (dist == LGPU_DIST_BECKMANN) {
        const Real aa = 1 / (alpha * absTan);
        if (aa >= 1.6f) return 0;
        return (1 - 1.259f * aa + 0.396f * aa * aa) / (3.535f * aa + 2.181f * aa * aa);
    }
    const Real a2t2 = (alpha * absTan) * (alpha * absTan);
    return (-1 + std::sqrt(1.f + a2t2)) / 2;
}
static Real DistG(int dist, const V3 &wo, const V3 &wi, V2 a) { return (Real)1 / ((Real)1 + DistLambda(dist, wo, a) + DistLambda(dist, wi, a)); }
static Real DistPdf(int dist, const V3 &wh, V2 a) { return DistD(dist, wh, a) * std::abs(wh.y); }
static V3 DistSampleWh(int dist, Sampler &s, const V3 &wo, V2 a) {
    const V2 u = s.Get2D();
    if (dist == LGPU_DIST_BECKMANN) {
        const Real lg = u.x == 1 ? 0 : std::log(1 - u.x);
        const Real phi = PI2 * u.y;
        const Real tan2 = -a.x * a.x * lg;
        const Real cosT = 1 / std::sqrt(1 + tan2);
        const Real sinT = std::sqrt(smax((Real)0, 1 - cosT * cosT));
        const V3 h = SphericalDirection(sinT, cosT, phi);
        return !SameHemisphere(wo, h) ? -h : h;
    }
    const Real phi = (PI2)*u.y;
    const Real tan2 = a.x * a.x * u.x / (1 - u.x);
    const Real cosT = 1 / std::sqrt(1 + tan2);
    const Real sinT = std::sqrt(smax((Real)0., (Real)1. - cosT * cosT));
    V3 wh = SphericalDirection(sinT, cosT, phi);
    if (!SameHemisphere(wo, wh)) wh = -wh;
    return wh;
}
/* ToAlpha (Microfacet.cpp:49-54) */
static inline Real ToAlpha(Real r) {
    r = smax(r, (Real)1e-3);
    Real x = std::log(r);
    return (Real)1.62142 + (Real)0.819955 * x + (Real)0.1734 * x * x + (Real)0.0171201 * x * x * x + (Real)0.000640711 * x * x * x * x;
}
/* OrenNayarTerm (OrenNayar.cpp:10-21) */
static Real OrenNayarTerm(const ScatterEvent &ev, Real sigma) {
    const Real thetaI = std::acos(clampr(ev.wiL.y, -1, 1));
    const Real thetaO = std::acos(clampr(ev.woL.y, -1, 1));
    const Real alpha = smax(thetaI, thetaO);
    const Real beta = smin(thetaI, thetaO);
    const Real phiI = std::acos(CosPhi(ev.wiL));
    const Real phiO = std::acos(CosPhi(ev.woL));
    const Real s2 = sigma * sigma;
    const Real A = (Real)1 - s2 / ((Real)2 * (s2 + (Real).33));
    const Real B = ((Real).45 * s2) / (s2 + (Real).09);
    return A + B * smax((Real)0, std::cos(phiI - phiO) * clampr(std::sin(alpha), -1, 1) * clampr(std::tan(beta), -1, 1));
}

struct Bxdf {
    const Graph &g;
    In in(int node, int i, const ScatterEvent &ev) const { return In{g, node, i, ev}; }
    /* Microfacet.cpp:56-69: the roughness SocketRef is declared TYPE_SCALAR, so the isotropic
     * branch is the one taken. */
    V2 RoughnessToAlpha(int node, const ScatterEvent &ev) const {
        const Real a = ToAlpha(in(node, 1, ev).real());
        return V2(a, a);
    }
    Spec f(int node, const ScatterEvent &ev) const {
        const int type = g.nodes[node].type;
        switch (type) {
        case LGPU_NODE_BXDF_LAMBERTIAN: return in(node, 0, ev).spectrum() * INV_PI;     /* BxDF.cpp:30-32 */
        case LGPU_NODE_BXDF_MIX: {                                                       /* BxDF.cpp:46-49 */
            const Real ratio = in(node, 2, ev).real();
            return f(in(node, 0, ev).bxdf(), ev) * ((Real)1 - ratio) + f(in(node, 1, ev).bxdf(), ev) * ratio;
        }
        case LGPU_NODE_BXDF_OREN_NAYAR_R: case LGPU_NODE_BXDF_OREN_NAYAR_T: {           /* OrenNayar.cpp:23-27 */
            const Real oN = OrenNayarTerm(ev, in(node, 1, ev).real());
            return in(node, 0, ev).spectrum() * INV_PI * oN;
        }
        case LGPU_NODE_BXDF_MICROFACET_R: {                                              /* Microfacet.cpp:12-27 */
            const Real cosO = std::abs(ev.woL.y), cosI = std::abs(ev.wiL.y);
            V3 wh = ev.wiL + ev.woL;
            if (cosI == 0 || cosO == 0) return Spec(0);
            if (wh.x == 0 && wh.y == 0 && wh.z == 0) return Spec(0);
            wh = wh.Normalised();
            const V3 wiL(ev.wiL.x, clampr(ev.wiL.y, 0, 1), ev.wiL.z);
            const Real etaT = (Real)0.00001;                                             /* Microfacet.h:10 */
            const Real F = FrDielectric(Dot(wiL, wh), g.nodes[node].params[1], etaT);   /* FresnelDielectric::Evaluate (B12 kept) */
            const V2 alpha = RoughnessToAlpha(node, ev);
            const int dist = (int)g.nodes[node].params[0];
            const Real D = DistD(dist, wh, alpha);
            const Real G = DistG(dist, ev.woL, wiL, alpha);
            const Spec alb = in(node, 0, ev).spectrum();
            return alb * D * G * Spec(F) / (4 * cosI * cosO);
        }
        default: return Spec(0);   /* FresnelBSDF / specular lobes: delta, f = 0 */
        }
    }
    Real Pdf(int node, const V3 &wo, const V3 &wi, const ScatterEvent &ev) const {
        const int type = g.nodes[node].type;
        switch (type) {
        case LGPU_NODE_BXDF_MIX: {
            const Real ratio = in(node, 2, ev).real();
            return Pdf(in(node, 0, ev).bxdf(), wo, wi, ev) * ((Real)1 - ratio) + Pdf(in(node, 1, ev).bxdf(), wo, wi, ev) * ratio;
        }
        case LGPU_NODE_BXDF_MICROFACET_R: {
            if (!SameHemisphere(wo, wi)) return 0;
            const V3 wh = (wo + wi).Normalised();
            const V2 alpha = RoughnessToAlpha(node, ev);
            return DistPdf((int)g.nodes[node].params[0], wh, alpha) / (4 * Dot(wo, wh));
        }
        case LGPU_NODE_BXDF_FRESNEL: case LGPU_NODE_BXDF_SPECULAR_T: return 0;
        default: return CosineHemispherePdf(wo, wi);
        }
    }
    Spec Sample_f(int node, ScatterEvent &ev, Sampler &s, Real &pdf) const {
        const int type = g.nodes[node].type;
        switch (type) {
        case LGPU_NODE_BXDF_MIX: {                                                       /* BxDF.cpp:51-60 */
            const Real ratio = in(node, 2, ev).real();
            if (s.Get1D() > ratio) {
                const Spec af = Sample_f(in(node, 0, ev).bxdf(), ev, s, pdf);
                return af * ((Real)1 - ratio) + f(in(node, 1, ev).bxdf(), ev) * ratio;
            } else {
                const Spec bf = Sample_f(in(node, 1, ev).bxdf(), ev, s, pdf);
                return bf * ratio + f(in(node, 0, ev).bxdf(), ev) * ((Real)1 - ratio);
            }
        }
        case LGPU_NODE_BXDF_MICROFACET_R: {                                              /* Microfacet.cpp:29-42 */
            if (ev.woL.y == 0) return Spec(0);
            const V2 alpha = RoughnessToAlpha(node, ev);
            const int dist = (int)g.nodes[node].params[0];
            const V3 wh = DistSampleWh(dist, s, ev.woL, alpha).Normalised();
            ev.wiL = Reflect(-ev.woL, wh);
            if (!SameHemisphere(ev.woL, ev.wiL)) { pdf = 0; return Spec(0); }
            pdf = DistPdf(dist, wh, alpha) / (4 * Dot(ev.woL, wh));
            ev.wi = ev.ToWorld(ev.wiL);
            ev.hit->point += ev.hit->normalG * SURFACE_EPSILON;
            return f(node, ev);
        }
        case LGPU_NODE_BXDF_OREN_NAYAR_T: {                                              /* OrenNayar.cpp:37-44 */
            ev.wiL = SampleCosineHemisphere(s.Get2D());
            pdf = CosineHemispherePdf(ev.woL, ev.wiL);
            ev.wiL.y *= (Real)-ev.sidedness;
            ev.wi = ev.ToWorld(ev.wiL);
            ev.hit->point += ev.hit->normalG * (Real)-ev.sidedness * SURFACE_EPSILON;
            return f(node, ev);
        }
        case LGPU_NODE_BXDF_FRESNEL: {                                                   /* Specular.cpp:18-45 */
            const bool entering = ev.woL.y > 0;
            const Real ior = in(node, 1, ev).real();
            const Real fr = FrDielectric(ev.woL.y, 1, ior);
            if (s.Get1D() < fr) {
                ev.wiL = V3(-ev.woL.x, ev.woL.y, -ev.woL.z);
                ev.wi = ev.ToWorld(ev.wiL);
                const Real cosT = std::abs(ev.wiL.y);
                ev.hit->point += ev.hit->normalG * (entering ? SURFACE_EPSILON : -SURFACE_EPSILON);
                pdf = fr;
                return in(node, 0, ev).spectrum() * fr / cosT;
            }
            const Real etaI = ev.eta = entering ? 1 : ior;
            const Real etaT = entering ? ior : 1;
            const V3 nf = (Dot(V3(0, 1, 0), ev.woL) < (Real)0) ? V3(0, -1, 0) : V3(0, 1, 0);
            const bool refr = Refract(ev.woL, nf, etaI / etaT, &ev.wiL);
            if (!refr) { pdf = 0; return Spec(0); }     /* unreachable: fr == 1 on TIR; pdf left 0 */
            Spec ft = in(node, 0, ev).spectrum() * (1 - fr);
            ft *= (etaI * etaI) / (etaT * etaT);
            const Real cosT = std::abs(ev.wiL.y);
            ev.wi = ev.ToWorld(ev.wiL);
            ev.hit->point += ev.hit->normalG * (entering ? -SURFACE_EPSILON * 2 : SURFACE_EPSILON * 2);
            pdf = (Real)1 - fr;
            return ft / cosT;
        }
        case LGPU_NODE_BXDF_SPECULAR_R: {                                                /* Specular.cpp:62-68 */
            pdf = 1;
            ev.wiL = V3(-ev.woL.x, ev.woL.y, -ev.woL.z);
            ev.wi = ev.ToWorld(ev.wiL);
            ev.hit->point += ev.hit->normalG * SURFACE_EPSILON;
            return in(node, 0, ev).spectrum() / std::abs(ev.wiL.y);
        }
        default: {                                                                       /* BxDF::Sample_f BxDF.cpp:7-14 */
            ev.wiL = SampleCosineHemisphere(s.Get2D());
            if (ev.woL.y < 0) ev.wiL.y *= -1;
            pdf = CosineHemispherePdf(ev.woL, ev.wiL);
            ev.wi = ev.ToWorld(ev.wiL);
            ev.hit->point += ev.hit->normalG * SURFACE_EPSILON * (Real)ev.sidedness;
            return f(node, ev);
        }
        }
    }
};

/* ------------------------------------------------------------------ media (src/shading/media/) */
struct Medium {
    Spec sigmaA, sigmaS;
    Real g = 0;
    Real sa[3], ss[3];
    /* RGB mode: the coefficients as given.  Hero mode: spectrally constant at the RGB mean. */
    void Prepare() {
        if (g_ns == 3) { for (int i = 0; i < 3; ++i) { sigmaA.c[i] = sa[i]; sigmaS.c[i] = ss[i]; } sigmaA.c[3] = sigmaS.c[3] = 0; return; }
        sigmaA = Spec((sa[0] + sa[1] + sa[2]) * ((Real)1 / 3));
        sigmaS = Spec((ss[0] + ss[1] + ss[2]) * ((Real)1 / 3));
    }
    /* HomogeneousMedium::Tr (HomogeneousMedium.cpp:12-15) */
    Spec Tr(Real tFar) const { const Spec st = sigmaA + sigmaS; return SExp(-st * smin(tFar, MAX_REAL)); }
    /* SampleDistance (HomogeneousMedium.cpp:17-38) */
    Spec SampleDistance(Sampler &s, ScatterEvent &ev, Real *t_, Real *pdf_) const {
        const Spec st = sigmaA + sigmaS;
        const V2 u = s.Get2D();
        const unsigned ch = std::min((unsigned)(u.x * (Real)g_ns), (unsigned)g_ns - 1);
        const Real dist = -std::log(1 - u.y) / st.c[ch];
        const Real t = smin(dist, ev.hit->tFar);
        ev.mediumInteraction = t < ev.hit->tFar;
        const Spec Tr = SExp(-st * smin(t, MAX_REAL));
        const Spec density = ev.mediumInteraction ? (st * Tr) : Tr;
        Real pdf = 0;
        for (int i = 0; i < g_ns; ++i) pdf += density.c[i];
        pdf *= 1 / (Real)g_ns;
        if (pdf == 0) pdf = 1;
        if (t_) *t_ = t;
        if (pdf_) *pdf_ = pdf;
        return ev.mediumInteraction ? (Tr * sigmaS / pdf) : (Tr / pdf);
    }
    /* PDFDistance (HomogeneousMedium.cpp:40-47), B3 patched: 1.f / nSamples */
    Real PDFDistance(Real t) const {
        const Spec st = sigmaA + sigmaS;
        const Spec Tr = SExp(-st * smin(t, MAX_REAL));
        Real pdf = 0;
        for (int i = 0; i < g_ns; ++i) pdf += st.c[i] * Tr.c[i];
        pdf *= 1.f / (Real)g_ns;
        return pdf;
    }
    /* SampleEquiangular (HomogeneousMedium.cpp:49-77); B2 t := min(dist, tFar), B4 origin := ray.o.
     * The sampled distance is measured from the foot of the perpendicular (kept as in the reference). */
    Spec SampleEquiangular(const Ray &r, Sampler &s, ScatterEvent &ev, const V3 &lp, Real *t_, Real *pdf_) const {
        const V3 delta = lp - r.o;
        const Real l = Dot(r.d, delta);
        const Real D = std::sqrt(Dot(delta, delta) - l * l);
        const Real thetaA = -std::atan2(l, D);
        const Real thetaB = std::atan2(ev.hit->tFar - l, D);
        const Real eps = s.Get1D();
        const Real dist = D * std::tan(Lerp(thetaB, thetaA, eps));
        const Real t = smin(dist, ev.hit->tFar);
        *t_ = t;
        ev.mediumInteraction = t < ev.hit->tFar;
        (void)s.Get2D();                                  /* channel draw, unused (HomogeneousMedium.cpp:70-71) */
        const Real pdf = D / ((thetaB - thetaA) * (D * D + t * t));
        *pdf_ = pdf;
        const Spec st = sigmaA + sigmaS;
        const Spec Tr = SExp(-st * smin(t, MAX_REAL));
        return Tr * sigmaS / pdf;
    }
    /* PDFEquiangular (HomogeneousMedium.cpp:80-92) */
    Real PDFEquiangular(const Ray &r, const V3 &lp, Real tFar, Real t) const {
        const V3 delta = lp - r.o;
        const Real l = Dot(r.d, delta);
        const Real D = std::sqrt(Dot(delta, delta) - l * l);
        const Real thetaA = -std::atan2(l, D);
        const Real thetaB = std::atan2(tFar - l, D);
        return D / ((thetaB - thetaA) * (D * D + t * t));
    }
    /* HenyeyGreenstein (HenyeyGreenstein.cpp:8-36) */
    static Real PhaseHG(Real cosT, Real g) {
        const Real g2 = g * g;
        const Real denom = 1 + g2 + 2 * g * cosT;
        return INV_PI4 * (1 - g2) / (denom * std::sqrt(denom));
    }
    Real p(const V3 &wo, const V3 &wi) const { return PhaseHG(Dot(wo, wi), g); }
    Real Sample_p(const V3 &wo, V3 *wi, Sampler &s) const {
        const V2 u = s.Get2D();
        Real cosT;
        if (std::abs(g) < 1e-3) cosT = 1 - 2 * u.x;
        else { const Real sq = (1 - g * g) / (1 - g + 2 * g * u.x); cosT = (1 + g * g - sq * sq) / (2 * g); }
        const Real sinT = std::sqrt(smax((Real)0, 1 - cosT * cosT));
        const Real phi = 2 * PI * u.y;
        const V3 woNeg = -wo;
        const V3 v1 = Cross(woNeg, V3(0, 1, 0));      /* frame not normalised, kept as in the reference */
        const V3 v2 = Cross(woNeg, v1);
        const V3 d = SphericalDirection(sinT, cosT, phi);
        *wi = v1 * d.x + woNeg * d.y + v2 * d.z;
        return PhaseHG(-cosT, g);
    }
};

/* ------------------------------------------------------------------ geometry + BVH (Embree restated) */
struct Tri { uint32_t v0, v1, v2; };
struct MeshRec {
    std::vector<V3> verts;
    std::vector<Tri> tris;
    std::vector<V3> normals;
    std::vector<V3> tangents; std::vector<Real> tsign;
    std::vector<V2> uvs;
    bool smooth = false, hasUV = false;
    /* BVH2 over triangles */
    struct Node { Bounds b; int left = -1, right = -1, first = 0, count = 0; };
    std::vector<Node> nodes;
    std::vector<uint32_t> triIdx;
    void GetAreaNormal(unsigned i, Real *area, V3 *normal) const {   /* TriangleMesh.h:59-63 */
        const Tri &t = tris[i];
        const V3 c = Cross(verts[t.v1] - verts[t.v0], verts[t.v2] - verts[t.v0]);
        *area = c.Magnitude() * (Real).5;
        if (normal) *normal = c / (Real)(*area * 2.);
    }
    V3 SamplePoint(unsigned i, V2 u) const {                          /* TriangleMesh.h:73-79 */
        const Tri &t = tris[i];
        const V3 &a = verts[t.v0], &b = verts[t.v1], &c = verts[t.v2];
        return a + (b - a) * u.x + (c - a) * u.y;
    }
    void Build();
};

static void BuildBVH(std::vector<MeshRec::Node> &nodes, std::vector<uint32_t> &idx,
                     const std::vector<Bounds> &pb, const std::vector<V3> &pc, int leafMax) {
    const size_t n = pb.size();
    idx.resize(n);
    for (size_t i = 0; i < n; ++i) idx[i] = (uint32_t)i;
    nodes.clear();
    nodes.reserve(2 * n + 1);
    struct Job { int node, first, count; };
    std::vector<Job> stack;
    nodes.push_back(MeshRec::Node());
    stack.push_back({0, 0, (int)n});
    const int NB = 16;
    while (!stack.empty()) {
        Job j = stack.back(); stack.pop_back();
        Bounds b = pb[idx[j.first]], cb(pc[idx[j.first]]);
        for (int i = j.first; i < j.first + j.count; ++i) { b = Union(b, pb[idx[i]]); cb = Union(cb, pc[idx[i]]); }
        nodes[j.node].b = b;
        if (j.count <= leafMax) { nodes[j.node].first = j.first; nodes[j.node].count = j.count; continue; }
        int bestAxis = -1, bestSplit = -1; Real bestCost = INF;
        for (int ax = 0; ax < 3; ++ax) {
            const Real lo = cb.min[ax], hi = cb.max[ax];
            if (!(hi > lo)) continue;
            Bounds bb[NB]; int cnt[NB] = {0}; bool init[NB] = {false};
            for (int i = j.first; i < j.first + j.count; ++i) {
                int k = (int)((pc[idx[i]][ax] - lo) / (hi - lo) * NB); if (k >= NB) k = NB - 1; if (k < 0) k = 0;
                bb[k] = init[k] ? Union(bb[k], pb[idx[i]]) : pb[idx[i]]; init[k] = true; cnt[k]++;
            }
            Real rightA[NB]; int rightC[NB];
            { Bounds acc; bool ai = false; int c = 0;
              for (int k = NB - 1; k > 0; --k) { if (init[k]) { acc = ai ? Union(acc, bb[k]) : bb[k]; ai = true; } c += cnt[k]; rightA[k] = ai ? acc.SurfaceArea() : 0; rightC[k] = c; } }
            Bounds acc; bool ai = false; int c = 0;
            for (int k = 0; k < NB - 1; ++k) {
                if (init[k]) { acc = ai ? Union(acc, bb[k]) : bb[k]; ai = true; }
                c += cnt[k];
                if (c == 0 || rightC[k + 1] == 0) continue;
                const Real cost = acc.SurfaceArea() * c + rightA[k + 1] * rightC[k + 1];
                if (cost < bestCost) { bestCost = cost; bestAxis = ax; bestSplit = k; }
            }
        }
        int mid;
        if (bestAxis < 0) mid = j.first + j.count / 2;
        else {
            const Real lo = cb.min[bestAxis], hi = cb.max[bestAxis];
            uint32_t *beg = &idx[j.first], *end = beg + j.count;
            uint32_t *m = std::partition(beg, end, [&](uint32_t p) {
                int k = (int)((pc[p][bestAxis] - lo) / (hi - lo) * NB); if (k >= NB) k = NB - 1; if (k < 0) k = 0;
                return k <= bestSplit; });
            mid = (int)(m - &idx[0]);
            if (mid == j.first || mid == j.first + j.count) mid = j.first + j.count / 2;
        }
        const int l = (int)nodes.size(); nodes.push_back(MeshRec::Node());
        const int r = (int)nodes.size(); nodes.push_back(MeshRec::Node());
        nodes[j.node].left = l; nodes[j.node].right = r;
        stack.push_back({l, j.first, mid - j.first});
        stack.push_back({r, mid, j.first + j.count - mid});
    }
}

void MeshRec::Build() {
    std::vector<Bounds> pb(tris.size());
    std::vector<V3> pc(tris.size());
    for (size_t i = 0; i < tris.size(); ++i) {
        Bounds b(verts[tris[i].v0]); b = Union(b, verts[tris[i].v1]); b = Union(b, verts[tris[i].v2]);
        pb[i] = b; pc[i] = b.Center();
    }
    BuildBVH(nodes, triIdx, pb, pc, 4);
}

/* Moller-Trumbore, two-sided; the triangle test both sides of the parity check use. */
static inline bool IntersectTri(const V3 &o, const V3 &d, const V3 &p0, const V3 &p1, const V3 &p2,
                                Real tmax, Real *t, Real *u, Real *v) {
    const V3 e1 = p1 - p0, e2 = p2 - p0;
    const V3 pv = Cross(d, e2);
    const Real det = Dot(e1, pv);
    if (det == 0) return false;
    const Real inv = (Real)1 / det;
    const V3 tv = o - p0;
    const Real uu = Dot(tv, pv) * inv;
    if (uu < 0 || uu > 1) return false;
    const V3 qv = Cross(tv, e1);
    const Real vv = Dot(d, qv) * inv;
    if (vv < 0 || uu + vv > 1) return false;
    const Real tt = Dot(e2, qv) * inv;
    if (!(tt > 0) || !(tt < tmax)) return false;
    *t = tt; *u = uu; *v = vv;
    return true;
}
static inline bool HitBox(const Bounds &b, const V3 &o, const V3 &inv, Real tmax, Real *tn) {
    Real t0 = 0, t1 = tmax;
    for (int a = 0; a < 3; ++a) {
        Real ta = (b.min[a] - o[a]) * inv[a], tb = (b.max[a] - o[a]) * inv[a];
        if (ta > tb) std::swap(ta, tb);
        if (!(ta <= tb)) { ta = -INF; tb = INF; }      /* 0 * inf on a slab plane: treat as inside */
        t0 = ta > t0 ? ta : t0; t1 = tb < t1 ? tb : t1;
        if (t0 > t1) return false;
    }
    *tn = t0;
    return true;
}

struct ObjectRec {
    int mesh = 0, kind = 0, material = 0, index = 0;
    Real m[9], t[3];        /* column-major linear part + translation */
    Real minv[9];
    Real nrm[9];            /* inverse transpose (normal matrix) */
    bool identity = true;
    Bounds worldBounds;
};

struct LightBase;
struct Material { int bxdf = -1; const LightBase *light = nullptr; int mi = -1, me = -1; };

/* ------------------------------------------------------------------ lights (src/lighting/) */
struct PartialLightSample { V3 point, normal; Spec Le; const LightBase *light = nullptr; Real pdf = 1; };

struct LightBase {
    virtual ~LightBase() {}
    virtual Spec Sample_Li(ScatterEvent &ev, Sampler &s, Real &pdf) const = 0;
    virtual Real PDF_Li(const ScatterEvent &ev) const = 0;
    /* Light::PDF_Li(event, sampler): the pdf of direction ev.wi from the shading point, found with
     * a ray query (EstimateDirect's BSDF-sampled strategy); 0 for delta lights */
    virtual Real PDF_Li_S(const ScatterEvent &, Sampler &) const { return 0; }
    virtual Spec SamplePoint(Sampler &s, ScatterEvent &ev, PartialLightSample *ls) const = 0;
    virtual Spec Visibility(const V3 &p, ScatterEvent &ev, Sampler &s, PartialLightSample *ls) const = 0;
    virtual Spec Le(const Ray &) const { return Spec(0); }
    virtual Spec L(const ScatterEvent &) const { return Spec(0); }
    virtual Real Irradiance() const = 0;
    virtual Real Area() const = 0;
    Real Power() const { return Irradiance() * Area(); }
    virtual Bounds GetBounds() const = 0;
    virtual V3 GetDirection() const = 0;
    virtual bool IsMesh() const { return false; }
    virtual bool IsEnv() const { return false; }
};

struct LightSampler {
    virtual ~LightSampler() {}
    virtual const LightBase *Sample(const ScatterEvent &ev, Sampler &s, Real *pdf) const = 0;
    /* B7: the tree importance is evaluated at the point/normal the sample was drawn for. */
    virtual Real Pdf(const V3 &p, const V3 &nS, unsigned primId, const LightBase *l) const = 0;
};

struct Scene {
    std::vector<MeshRec> meshes;
    std::vector<ObjectRec> objects;
    std::vector<Material> materials;
    std::vector<std::unique_ptr<LightBase>> lightStore;
    std::vector<const LightBase *> lights;
    const LightBase *envLight = nullptr;
    std::unique_ptr<LightSampler> lightSampler;
    std::vector<Medium> media;
    Graph graph;
    bool hasVolumes = false;
    std::vector<MeshRec::Node> tlas;
    std::vector<uint32_t> tlasIdx;
    Bounds sceneBounds;

    bool Intersect(const Ray &r, RayHit &h) const;
    bool Occluded(const V3 &o, const V3 &d, Real tmax) const;
    bool IntersectTr(Ray r, RayHit &h, Sampler &s, const Medium *med, Spec *Tr) const;
    bool IntersectTr(Ray r, RayHit &h, Sampler &s, const Medium *med, Spec *Tr, Real maxT) const;
    bool MutualVisibility(const V3 &p1, const V3 &p2, V3 *w) const;
    bool RayEscapes(const Ray &r) const { return !Occluded(r.o, r.d, INF); }
    const Medium *GetMedium(const Material &m, const V3 &w, const V3 &n) const {
        const int id = Dot(w, n) < 0 ? m.mi : m.me;                              /* Media.h:53-55 */
        return id >= 0 ? &media[id] : nullptr;
    }
};

static inline V3 MulCM(const Real *m, const V3 &v) {
    return V3(m[0] * v.x + m[3] * v.y + m[6] * v.z, m[1] * v.x + m[4] * v.y + m[7] * v.z, m[2] * v.x + m[5] * v.y + m[8] * v.z);
}

/* Closest hit over the two-level BVH (Scene::Intersect, Scene.cpp:28-43 with Object::Hit and
 * TriangleMesh/Instance::ProcessHit).  B26: an instance hit is processed by the instance that was
 * hit (the reference calls objects[geomID], the proxy-local id, i.e. objects[0]). */
bool Scene::Intersect(const Ray &r, RayHit &h) const {
    Real best = INF, bu = 0, bv = 0; int bobj = -1; unsigned bprim = 0;
    const V3 inv(1 / r.d.x, 1 / r.d.y, 1 / r.d.z);
    int stack[128]; int sp = 0; stack[sp++] = 0;
    while (sp) {
        const MeshRec::Node &nd = tlas[stack[--sp]];
        Real tn;
        if (!HitBox(nd.b, r.o, inv, best, &tn)) continue;
        if (nd.left < 0) {
            for (int k = nd.first; k < nd.first + nd.count; ++k) {
                const ObjectRec &ob = objects[tlasIdx[k]];
                const MeshRec &me = meshes[ob.mesh];
                V3 o = r.o, d = r.d;
                if (!ob.identity) { o = MulCM(ob.minv, r.o - V3(ob.t[0], ob.t[1], ob.t[2])); d = MulCM(ob.minv, r.d); }
                const V3 oinv(1 / d.x, 1 / d.y, 1 / d.z);
                int st2[128]; int sp2 = 0; st2[sp2++] = 0;
                while (sp2) {
                    const MeshRec::Node &bn = me.nodes[st2[--sp2]];
                    Real t2;
                    if (!HitBox(bn.b, o, oinv, best, &t2)) continue;
                    if (bn.left < 0) {
                        for (int q = bn.first; q < bn.first + bn.count; ++q) {
                            const unsigned ti = me.triIdx[q];
                            const Tri &tr = me.tris[ti];
                            Real tt, uu, vv;
                            if (IntersectTri(o, d, me.verts[tr.v0], me.verts[tr.v1], me.verts[tr.v2], best, &tt, &uu, &vv)) {
                                best = tt; bu = uu; bv = vv; bobj = ob.index; bprim = ti;
                            }
                        }
                    } else { st2[sp2++] = bn.right; st2[sp2++] = bn.left; }
                }
            }
        } else { stack[sp++] = nd.right; stack[sp++] = nd.left; }
    }
    if (bobj < 0 || !(best > 0) || !(best < INF)) return false;
    const ObjectRec &ob = objects[bobj];
    const MeshRec &me = meshes[ob.mesh];
    const Tri &tr = me.tris[bprim];
    h.tFar = best;
    h.point = V3(r.o.x + r.d.x * best, r.o.y + r.d.y * best, r.o.z + r.d.z * best);
    const V3 ng = Cross(me.verts[tr.v1] - me.verts[tr.v0], me.verts[tr.v2] - me.verts[tr.v0]);
    h.normalG = ng.Normalised();
    /* TriangleMesh::ProcessHit (TriangleMesh.cpp:80-114) */
    if (me.hasUV) h.uv = Bary(me.uvs[tr.v0], me.uvs[tr.v1], me.uvs[tr.v2], bu, bv);
    if (me.smooth) {
        const V3 &n0 = me.normals[tr.v0], &n1 = me.normals[tr.v1], &n2 = me.normals[tr.v2];
        const V3 &t0 = me.tangents[tr.v0], &t1 = me.tangents[tr.v1], &t2 = me.tangents[tr.v2];
        h.normalS = Bary(n0, n1, n2, bu, bv).Normalised();
        h.tangent = Bary(t0, t1, t2, bu, bv).Normalised();
        h.bitangent = Bary(Cross(n0, t0) * me.tsign[tr.v0], Cross(n1, t1) * me.tsign[tr.v1], Cross(n2, t2) * me.tsign[tr.v2], bu, bv).Normalised();
    } else {
        h.normalS = h.normalG;
        const V3 c1 = Cross(h.normalG, V3(0, 0, 1));
        const V3 c2 = Cross(h.normalG, V3(0, 1, 0));
        h.tangent = (Dot(c1, c1) > Dot(c2, c2) ? c1 : c2);
        h.bitangent = Cross(h.tangent, h.normalG);
    }
    if (ob.kind == 1 && !ob.identity) {   /* Instance::ProcessHit (Instance.cpp:36-43) + B18 */
        h.normalS = MulCM(ob.m, h.normalS).Normalised();
        h.tangent = MulCM(ob.m, h.tangent).Normalised();
        h.bitangent = MulCM(ob.m, h.bitangent).Normalised();
        h.normalG = MulCM(ob.nrm, ng).Normalised();
    }
    h.object = &ob;
    h.primId = bprim;
    return true;
}

/* Any hit with t in (0, tmax] (rtcOccluded1). */
bool Scene::Occluded(const V3 &ro, const V3 &rd, Real tmax) const {
    const V3 inv(1 / rd.x, 1 / rd.y, 1 / rd.z);
    const Real lim = std::nextafter(tmax, INF);
    int stack[128]; int sp = 0; stack[sp++] = 0;
    while (sp) {
        const MeshRec::Node &nd = tlas[stack[--sp]];
        Real tn;
        if (!HitBox(nd.b, ro, inv, lim, &tn)) continue;
        if (nd.left < 0) {
            for (int k = nd.first; k < nd.first + nd.count; ++k) {
                const ObjectRec &ob = objects[tlasIdx[k]];
                const MeshRec &me = meshes[ob.mesh];
                V3 o = ro, d = rd;
                if (!ob.identity) { o = MulCM(ob.minv, ro - V3(ob.t[0], ob.t[1], ob.t[2])); d = MulCM(ob.minv, rd); }
                const V3 oinv(1 / d.x, 1 / d.y, 1 / d.z);
                int st2[128]; int sp2 = 0; st2[sp2++] = 0;
                while (sp2) {
                    const MeshRec::Node &bn = me.nodes[st2[--sp2]];
                    Real t2;
                    if (!HitBox(bn.b, o, oinv, lim, &t2)) continue;
                    if (bn.left < 0) {
                        for (int q = bn.first; q < bn.first + bn.count; ++q) {
                            const Tri &tr = me.tris[me.triIdx[q]];
                            Real tt, uu, vv;
                            if (IntersectTri(o, d, me.verts[tr.v0], me.verts[tr.v1], me.verts[tr.v2], lim, &tt, &uu, &vv)) return true;
                        }
                    } else { st2[sp2++] = bn.right; st2[sp2++] = bn.left; }
                }
            }
        } else { stack[sp++] = nd.right; stack[sp++] = nd.left; }
    }
    return false;
}

/* Scene::IntersectTr (Scene.cpp:45-59) */
bool Scene::IntersectTr(Ray r, RayHit &h, Sampler &s, const Medium *med, Spec *Tr) const {
    (void)s;
    Real tFar = 0;
    while (Intersect(r, h)) {
        tFar += h.tFar;
        if (med && Tr) *Tr *= med->Tr(h.tFar);
        const Material &m = materials[h.object->material];
        if (m.bxdf >= 0 || m.light) { h.tFar = tFar; return true; }
        med = GetMedium(m, r.d, h.normalG);
        r.o = h.point + h.normalG * (Dot(h.normalG, r.d) < 0 ? -SURFACE_EPSILON : SURFACE_EPSILON);
    }
    return false;
}
/* Scene::IntersectTr with maxT (Scene.cpp:61-81) */
bool Scene::IntersectTr(Ray r, RayHit &h, Sampler &s, const Medium *med, Spec *Tr, Real maxT) const {
    (void)s;
    Real tFar = 0;
    while (Intersect(r, h)) {
        tFar += h.tFar;
        const bool term = tFar > maxT;
        if (term) { const Real delta = tFar - maxT; tFar -= delta; h.tFar -= delta; }
        if (med && Tr) *Tr *= med->Tr(h.tFar);
        const Material &m = materials[h.object->material];
        if (term || m.bxdf >= 0 || m.light) { h.tFar = tFar; return true; }
        med = GetMedium(m, r.d, h.normalG);
        r.o = h.point + h.normalG * (Dot(h.normalG, r.d) < 0 ? -SURFACE_EPSILON : SURFACE_EPSILON);
    }
    return false;
}
/* Scene::MutualVisibility (Scene.cpp:83-95) */
bool Scene::MutualVisibility(const V3 &p1, const V3 &p2, V3 *w) const {
    const V3 diff = p2 - p1;
    const Real mag = diff.Magnitude();
    const V3 dir = diff / mag;
    if (w) *w = dir;
    return !Occluded(p1, dir, (Real)(mag - .00001));
}

/* Light::MutualVisibility / PointMutualVisibility / RayEscapes (Light.cpp:10-49) */
static bool LMutualVisibility(const V3 &p1, const V3 &p2, ScatterEvent &ev, const Scene &sc, Sampler &s, Spec *Tr) {
    if (sc.hasVolumes) {
        const V3 diff = p2 - p1;
        const Real mag = diff.Magnitude();
        const V3 dir = diff / mag;
        const Real minT = mag - SURFACE_EPSILON * 10;
        ev.wi = dir;
        RayHit hit;
        sc.IntersectTr(Ray{p1, dir}, hit, s, ev.medium, Tr);
        return hit.tFar > minT;
    }
    return sc.MutualVisibility(p1, p2, &ev.wi);
}
static bool LPointMutualVisibility(const V3 &p1, const V3 &p2, ScatterEvent &ev, const Scene &sc, Sampler &s, Spec *Tr) {
    if (sc.hasVolumes) {
        const V3 diff = p2 - p1;
        const Real mag = diff.Magnitude();
        const V3 dir = diff / mag;
        const Real minT = mag - SURFACE_EPSILON * 10;
        ev.wi = dir;
        RayHit hit;
        sc.IntersectTr(Ray{p1, dir}, hit, s, ev.medium, Tr, mag);
        return hit.tFar > minT;
    }
    return sc.MutualVisibility(p1, p2, &ev.wi);
}
static bool LRayEscapes(const Ray &r, const ScatterEvent &ev, Sampler &s, Spec *Tr) {
    if (ev.scene->hasVolumes) {
        RayHit hit;
        return !ev.scene->IntersectTr(r, hit, s, ev.medium, Tr);
    }
    return ev.scene->RayEscapes(r);
}

struct Piecewise1D {   /* sampling/Piecewise.cpp:9-38 */
    std::vector<Real> pdf, cdf;
    Real integral = 0;
    Piecewise1D() {}
    Piecewise1D(const Real *d, unsigned n) : pdf(d, d + n), cdf(n + 1) {
        cdf[0] = 0;
        for (unsigned i = 1; i < n + 1; ++i) cdf[i] = cdf[i - 1] + pdf[i - 1] / n;
        integral = cdf[n];
        if (integral == 0) { for (unsigned i = 1; i < n + 1; ++i) cdf[i] = Real(i) / Real(n); }
        else { for (unsigned i = 1; i < n + 1; ++i) cdf[i] /= integral; }
    }
    Real SampleContinuous(Real u, Real *p, int *off_) const {
        const unsigned off = FindInterval((int)cdf.size(), [&](int i) { return cdf[i] <= u; });
        if (off_) *off_ = (int)off;
        Real du = u - cdf[off];
        if ((cdf[off + 1] - cdf[off]) > 0) du /= (cdf[off + 1] - cdf[off]);
        if (p) *p = pdf[off] / integral;
        return (off + du) / pdf.size();
    }
    unsigned SampleDiscrete(Real u, Real *p) const {
        const unsigned off = FindInterval((int)cdf.size(), [&](int i) { return cdf[i] <= u; });
        if (p) *p = pdf[off] / (integral * pdf.size());
        return off;
    }
    Real PDF(unsigned i) const { return pdf[i]; }     /* raw value, Piecewise.h:26-28 */
};
struct Piecewise2D {   /* Piecewise.cpp:40-76 */
    std::vector<Piecewise1D> cond;
    Piecewise1D marg;
    Piecewise2D() {}
    Piecewise2D(const Real *f, unsigned nu, unsigned nv) {
        for (unsigned v = 0; v < nv; ++v) cond.emplace_back(&f[v * nu], nu);
        std::vector<Real> m;
        for (unsigned v = 0; v < nv; ++v) m.push_back(cond[v].integral);
        marg = Piecewise1D(m.data(), nv);
    }
    V2 SampleContinuous(const V2 &u, Real *pdf) const {
        Real p[2]; int v;
        const Real d1 = marg.SampleContinuous(u.y, &p[1], &v);
        const Real d0 = cond[v].SampleContinuous(u.x, &p[0], nullptr);
        *pdf = p[0] * p[1];
        return V2(d0, d1);
    }
    Real PDF(const V2 &uv) const {
        const int iu = std::max(std::min(int(uv.x * cond[0].pdf.size()), (int)cond[0].pdf.size() - 1), 0);
        const int iv = std::max(std::min(int(uv.y * marg.pdf.size()), (int)marg.pdf.size() - 1), 0);
        return cond[iv].pdf[iu] / marg.integral;
    }
};

static Spec EvalEmission(const Scene &sc, int node, int sock, const ScatterEvent &ev) {
    return AsSpectrum(EvalOutput(sc.graph, node, sock, ev), true);
}

struct MeshLight;
struct TriangleLight : LightBase {
    const MeshLight *ml; unsigned tri;
    TriangleLight(const MeshLight *m, unsigned i) : ml(m), tri(i) {}
    Spec Sample_Li(ScatterEvent &ev, Sampler &s, Real &pdf) const override;
    Real PDF_Li(const ScatterEvent &ev) const override;
    Real PDF_Li_S(const ScatterEvent &ev, Sampler &s) const override;
    Spec SamplePoint(Sampler &s, ScatterEvent &ev, PartialLightSample *ls) const override;
    Spec Visibility(const V3 &p, ScatterEvent &ev, Sampler &s, PartialLightSample *ls) const override;
    Spec L(const ScatterEvent &ev) const override;
    Real Irradiance() const override;
    Real Area() const override;
    Bounds GetBounds() const override;
    V3 GetDirection() const override;
};
struct MeshLight : LightBase {   /* MeshLight.cpp:1-125 */
    const Scene *sc; const ObjectRec *obj; const MeshRec *mesh;
    int enode, esock; Real intensity;
    Piecewise1D triDist;
    std::vector<TriangleLight> triLights;
    bool IsMesh() const override { return true; }
    void Init() {
        std::vector<Real> a(mesh->tris.size());
        for (size_t i = 0; i < a.size(); ++i) mesh->GetAreaNormal((unsigned)i, &a[i], nullptr);
        triDist = Piecewise1D(a.data(), (unsigned)a.size());
        for (size_t i = 0; i < a.size(); ++i) triLights.emplace_back(this, (unsigned)i);
    }
    Spec Emit(const ScatterEvent &ev) const { return EvalEmission(*sc, enode, esock, ev) * intensity * INV_PI; }
    Spec Sample_Li(ScatterEvent &ev, Sampler &s, Real &pdf) const override {
        const unsigned i = triDist.SampleDiscrete(s.Get1D(), &pdf);
        const V2 u = s.Get2D();
        const V3 pL = mesh->SamplePoint(i, u);
        const V3 pS = ev.hit->point + ev.hit->normalG * SURFACE_EPSILON * (Real)ev.sidedness;
        Spec Tr(1);
        if (LMutualVisibility(pS, pL, ev, *ev.scene, s, &Tr)) {
            Real area; V3 n;
            mesh->GetAreaNormal(i, &area, &n);
            const Real cosT = std::abs(Dot(n, -ev.wi));
            if (cosT > 0) {
                ev.wiL = ev.ToLocal(ev.wi);
                pdf *= DistSq(ev.hit->point, pL) / (cosT * area);
                return Emit(ev) * Tr;
            }
        }
        pdf = 0;
        return Spec(0);
    }
    /* MeshLight::PDF_Li(event, sampler) (MeshLight.cpp:43-54): no triangle-selection factor */
    Real PDF_Li_S(const ScatterEvent &ev, Sampler &s) const override {
        RayHit h;
        const Ray r{ev.hit->point + ev.hit->normalG * SURFACE_EPSILON * (Real)ev.sidedness, ev.wi};
        const bool hit = sc->hasVolumes ? sc->IntersectTr(r, h, s, ev.medium, nullptr) : sc->Intersect(r, h);
        if (!hit) return 0;
        if (sc->materials[h.object->material].light != this) return 0;
        Real area; V3 n;
        mesh->GetAreaNormal(h.primId, &area, &n);
        const Real cosT = std::abs(Dot(n, -ev.wi));
        if (cosT > 0) return DistSq(ev.hit->point, h.point) / (cosT * area);
        return 0;
    }
    Real PDF_Li(const ScatterEvent &ev) const override {
        if (Dot(ev.wi, ev.hit->normalG) > 0) return 0;
        const Real triPdf = triDist.PDF(ev.hit->primId);
        const Real distSq = ev.hit->tFar * ev.hit->tFar;
        Real area; mesh->GetAreaNormal(ev.hit->primId, &area, nullptr);
        const Real cosT = std::abs(Dot(ev.hit->normalG, -ev.wi));
        return triPdf * distSq / (cosT * area);
    }
    Spec SamplePoint(Sampler &s, ScatterEvent &ev, PartialLightSample *ls) const override {
        Real distPdf;
        const unsigned i = triDist.SampleDiscrete(s.Get1D(), &distPdf);
        Real area;
        mesh->GetAreaNormal(i, &area, &ls->normal);
        ls->pdf *= distPdf / area;
        const V2 u = s.Get2D();
        const Tri &t = mesh->tris[i];
        if (mesh->hasUV) ev.hit->uv = Bary(mesh->uvs[t.v0], mesh->uvs[t.v1], mesh->uvs[t.v2], u.x, u.y);
        ls->point = mesh->SamplePoint(i, u);
        return Emit(ev);
    }
    Spec Visibility(const V3 &p, ScatterEvent &ev, Sampler &s, PartialLightSample *ls) const override {
        Spec Tr(1);
        if (LMutualVisibility(p, ls->point, ev, *ev.scene, s, &Tr)) {
            const Real cosT = std::abs(Dot(ls->normal, -ev.wi));
            ls->pdf *= DistSq(p, ls->point) / cosT;
            return Tr;
        }
        ls->pdf = 0;
        return Spec(0);
    }
    Spec L(const ScatterEvent &ev) const override { return Emit(ev); }
    Real Irradiance() const override { return intensity; }
    Real Area() const override { Real a = 0; for (size_t i = 0; i < mesh->tris.size(); ++i) {
        const Tri &t = mesh->tris[i]; a += Cross(mesh->verts[t.v1] - mesh->verts[t.v0], mesh->verts[t.v2] - mesh->verts[t.v0]).Magnitude(); }
        return a * (Real).5; }
    Bounds GetBounds() const override { Bounds b; for (auto &v : mesh->verts) b = Union(b, v); return b; }
    V3 GetDirection() const override { return V3(0, 0, 0); }
};
/* TriangleLight (MeshLight.cpp:129-238); B10: pdf = dist^2 / (cos * A). */
Spec TriangleLight::Sample_Li(ScatterEvent &ev, Sampler &s, Real &pdf) const {
    const V3 pL = ml->mesh->SamplePoint(tri, s.Get2D());
    const V3 pS = ev.hit->point + ev.hit->normalG * SURFACE_EPSILON * (Real)ev.sidedness;
    Spec Tr(1);
    if (LMutualVisibility(pS, pL, ev, *ev.scene, s, &Tr)) {
        Real area; V3 n;
        ml->mesh->GetAreaNormal(tri, &area, &n);
        const Real cosT = std::abs(Dot(n, -ev.wi));
        if (cosT > 0) {
            ev.wiL = ev.ToLocal(ev.wi);
            pdf = DistSq(ev.hit->point, pL) / (cosT * area);
            return ml->Emit(ev) * Tr;
        }
    }
    pdf = 0;
    return Spec(0);
}
/* TriangleLight::PDF_Li(event, sampler) (MeshLight.cpp:153-155) */
Real TriangleLight::PDF_Li_S(const ScatterEvent &ev, Sampler &s) const { return ml->PDF_Li_S(ev, s); }
Real TriangleLight::PDF_Li(const ScatterEvent &ev) const {
    if (Dot(ev.wi, ev.hit->normalG) > 0) return 0;
    const Real distSq = ev.hit->tFar * ev.hit->tFar;
    Real area; ml->mesh->GetAreaNormal(ev.hit->primId, &area, nullptr);
    const Real cosT = std::abs(Dot(ev.hit->normalG, -ev.wi));
    return distSq / (cosT * area);
}
Spec TriangleLight::SamplePoint(Sampler &s, ScatterEvent &ev, PartialLightSample *ls) const {
    const MeshRec &m = *ml->mesh;
    const Tri &t = m.tris[tri];
    Real area; m.GetAreaNormal(tri, &area, nullptr);
    ls->pdf /= area;
    const V2 u = s.Get2D();
    if (m.hasUV) ev.hit->uv = Bary(m.uvs[t.v0], m.uvs[t.v1], m.uvs[t.v2], u.x, u.y);
    ls->point = m.SamplePoint(tri, u);
    return ml->Emit(ev);
}
Spec TriangleLight::Visibility(const V3 &p, ScatterEvent &ev, Sampler &s, PartialLightSample *ls) const {
    Spec Tr(1);
    if (LMutualVisibility(p, ls->point, ev, *ev.scene, s, &Tr)) {
        const Real cosT = std::abs(Dot(ev.hit->normalG, -ev.wi));
        ls->pdf *= DistSq(p, ls->point) / cosT;
        return Tr;
    }
    ls->pdf = 0;
    return Spec(0);
}
Spec TriangleLight::L(const ScatterEvent &ev) const { return ml->L(ev); }
Real TriangleLight::Irradiance() const {   /* MeshLight.cpp:205-218, tree build in RGB semantics */
    const MeshRec &m = *ml->mesh;
    const Tri &t = m.tris[tri];
    const unsigned n = 3; const Real inv = (Real)1 / (Real)n;
    ScatterEvent fe; RayHit fh; fe.hit = &fh;
    const int keep = g_ns; g_ns = 3;
    Real irr = 0;
    for (unsigned a = 0; a < n; ++a)
        for (unsigned b = 0; b < n; ++b) {
            if (m.hasUV) fh.uv = Bary(m.uvs[t.v0], m.uvs[t.v1], m.uvs[t.v2], (Real)a * inv, (Real)b * inv);
            irr += EvalEmission(*ml->sc, ml->enode, ml->esock, fe).y();
        }
    g_ns = keep;
    return irr * inv * inv * ml->intensity;
}
Real TriangleLight::Area() const { Real a; ml->mesh->GetAreaNormal(tri, &a, nullptr); return a; }
Bounds TriangleLight::GetBounds() const {
    const MeshRec &m = *ml->mesh; const Tri &t = m.tris[tri];
    Bounds b(m.verts[t.v0]); b = Union(b, m.verts[t.v1]); b = Union(b, m.verts[t.v2]); return b;
}
V3 TriangleLight::GetDirection() const { Real a; V3 n; ml->mesh->GetAreaNormal(tri, &a, &n); return n; }

struct PointLightO : LightBase {   /* PointLight.cpp:18-71 */
    const Scene *sc; V3 pos; int enode, esock; Real intensity;
    Spec Emit(const ScatterEvent &ev, bool illum) const { return AsSpectrum(EvalOutput(sc->graph, enode, esock, ev), illum); }
    Spec Sample_Li(ScatterEvent &ev, Sampler &s, Real &pdf) const override {
        const V3 p = ev.hit->point + ev.hit->normalG * SURFACE_EPSILON * (Real)ev.sidedness;
        Spec Tr(1);
        if (LPointMutualVisibility(p, pos, ev, *ev.scene, s, &Tr)) {
            pdf = 1;
            const Real d2 = DistSq(pos, ev.hit->point);
            ev.wiL = ev.ToLocal(ev.wi);
            return Emit(ev, false) * Tr * intensity / d2;
        }
        pdf = 0;
        return Spec(0);
    }
    Real PDF_Li(const ScatterEvent &) const override { return 0; }
    Spec SamplePoint(Sampler &, ScatterEvent &ev, PartialLightSample *ls) const override { ls->point = pos; return Emit(ev, true) * intensity; }
    Spec Visibility(const V3 &sp, ScatterEvent &ev, Sampler &s, PartialLightSample *ls) const override {
        const V3 p = sp + ev.hit->normalG * SURFACE_EPSILON * (Real)ev.sidedness;
        Spec Tr(1);
        if (LPointMutualVisibility(p, ls->point, ev, *ev.scene, s, &Tr)) return Tr / DistSq(pos, ev.hit->point);
        ls->pdf = 0;
        return Spec(0);
    }
    Real Irradiance() const override { return intensity; }
    Real Area() const override { return 4 * PI; }
    Bounds GetBounds() const override { return Bounds(pos); }
    V3 GetDirection() const override { return V3(0, 1, 0); }
};
struct SpotLightO : LightBase {   /* Spotlight.cpp:21-81 */
    const Scene *sc; V3 pos, axis; Real cosCone, cosFall; int enode, esock; Real intensity;
    Real Falloff(const V3 &w) const {
        const Real c = Dot(w, axis);
        if (c < cosCone) return 0;
        if (c > cosFall) return 1;
        const Real d = (c - cosCone) / (cosFall - cosCone);
        return (d * d) * (d * d);
    }
    Spec Emit(const ScatterEvent &ev, bool illum) const { return AsSpectrum(EvalOutput(sc->graph, enode, esock, ev), illum); }
    Spec Sample_Li(ScatterEvent &ev, Sampler &s, Real &pdf) const override {
        const V3 p = ev.hit->point + ev.hit->normalG * SURFACE_EPSILON * (Real)ev.sidedness;
        Spec Tr(1);
        if (LPointMutualVisibility(p, pos, ev, *ev.scene, s, &Tr)) {
            pdf = 1;
            const Real d2 = DistSq(pos, ev.hit->point);
            ev.wiL = ev.ToLocal(ev.wi);
            return Emit(ev, false) * Tr * Falloff(-ev.wi) * intensity / d2;
        }
        pdf = 0;
        return Spec(0);
    }
    Real PDF_Li(const ScatterEvent &) const override { return 0; }
    Spec SamplePoint(Sampler &, ScatterEvent &ev, PartialLightSample *ls) const override { ls->point = pos; return Emit(ev, true) * intensity; }
    Spec Visibility(const V3 &sp, ScatterEvent &ev, Sampler &s, PartialLightSample *ls) const override {
        const V3 p = sp + ev.hit->normalG * SURFACE_EPSILON * (Real)ev.sidedness;
        Spec Tr(1);
        if (LPointMutualVisibility(p, ls->point, ev, *ev.scene, s, &Tr)) return Tr * Falloff(-ev.wi) / DistSq(pos, ev.hit->point);
        ls->pdf = 0;
        return Spec(0);
    }
    Real Irradiance() const override { return intensity; }
    Real Area() const override { return PI2 - (1 - (Real).5 * (cosFall + cosCone)); }
    Bounds GetBounds() const override { return Bounds(pos); }
    V3 GetDirection() const override { return axis; }
};
struct EnvLightO : LightBase {   /* EnvironmentLight.cpp:7-108 */
    int w = 0, h = 0; std::vector<Real> tex; Real intensity = 1; V2 offset; Real radius = 0; Bounds bounds;
    Piecewise2D dist;
    bool IsEnv() const override { return true; }
    void Texel(int x, int y, Real c[3]) const { const Real *p = &tex[3 * ((size_t)y * w + x)]; c[0] = p[0]; c[1] = p[1]; c[2] = p[2]; }
    Spec GetUV(V2 uv) const {   /* TextureAdapter::GetUV + GetPixelUVBilinear (Texture.h:71-81) */
        uv = V2(Fract(uv.x), Fract(uv.y));
        const Real fx = std::min((float)(w - 1), clampr(uv.x, 0.f, 1.f) * (float)w);
        const Real fy = std::min((float)(h - 1), clampr(uv.y, 0.f, 1.f) * (float)h);
        const unsigned x = (unsigned)fx, y = (unsigned)fy;
        const unsigned x1 = std::min(x + 1, (unsigned)w - 1), y1 = std::min(y + 1, (unsigned)h - 1);
        Real a[3], b[3], c[3], d[3], rgb[3];
        Texel(x, y, a); Texel(x1, y, b); Texel(x, y1, c); Texel(x1, y1, d);
        for (int k = 0; k < 3; ++k) {
            const Real ya = Lerp(a[k], b[k], fx - (float)x);
            const Real yb = Lerp(c[k], d[k], fx - (float)x);
            rgb[k] = Lerp(ya, yb, fy - (float)y);
        }
        return FromRGB(rgb, true);
    }
    void Init() {
        std::vector<Real> img((size_t)w * h);
        const int keep = g_ns; g_ns = 3;
        for (int y = 0; y < h; ++y) {
            const Real vp = (Real)y / (Real)h;
            const Real sinT = std::sin(PI * Real(y + .5) / Real(h));
            for (int x = 0; x < w; ++x) {
                const Real up = (Real)x / (Real)w;
                img[x + (size_t)y * w] = std::abs(GetUV(V2(up, vp)).y());
                img[x + (size_t)y * w] *= sinT;
            }
        }
        g_ns = keep;
        dist = Piecewise2D(img.data(), w, h);
    }
    Spec LeDir(const V3 &wd) const {
        const V2 uv(Fract((SphericalPhi(wd) - offset.x) * INV_PI2), Fract((SphericalTheta(wd) - offset.y) * INV_PI));
        return GetUV(uv) * intensity;
    }
    Spec Sample_Li(ScatterEvent &ev, Sampler &s, Real &pdf) const override {
        const V2 uv = dist.SampleContinuous(s.Get2D(), &pdf);
        if (pdf == 0) return Spec(0);
        const Real theta = uv.y * PI + offset.y;
        const Real phi = uv.x * PI2 + offset.x;
        const Real cosT = std::cos(theta), sinT = std::sin(theta);
        if (sinT == 0) { pdf = 0; return Spec(0); }
        ev.wi = SphericalDirection(sinT, cosT, phi);
        Spec Tr(1);
        if (LRayEscapes(Ray{ev.hit->point + ev.hit->normalG * SURFACE_EPSILON, ev.wi}, ev, s, &Tr)) {
            ev.wiL = ev.ToLocal(ev.wi);
            pdf /= 2 * PI * PI * sinT;
            return GetUV(uv) * Tr * intensity;
        }
        pdf = 0;
        return Spec(0);
    }
    Real PDF_Li(const ScatterEvent &ev) const override {
        const Real theta = SphericalTheta(ev.wi) - offset.y;
        const Real phi = SphericalPhi(ev.wi) - offset.x;
        const Real sinT = std::sin(theta);
        if (sinT == 0) return 0;
        return dist.PDF(V2(Fract(phi * INV_PI2), Fract(theta * INV_PI))) / ((Real)2 * PI * PI * sinT);
    }
    /* EnvironmentLight::PDF_Li(event, sampler) (EnvironmentLight.cpp:47-58) */
    Real PDF_Li_S(const ScatterEvent &ev, Sampler &s) const override {
        const Real theta = SphericalTheta(ev.wi) - offset.y;
        const Real phi = SphericalPhi(ev.wi) - offset.x;
        const Real sinT = std::sin(theta);
        if (sinT == 0) return 0;
        const V3 wOff = SphericalDirection(sinT, std::cos(theta), phi);
        if (LRayEscapes(Ray{ev.hit->point, wOff}, ev, s, nullptr))
            return dist.PDF(V2(Fract(phi * INV_PI2), Fract(theta * INV_PI))) / ((Real)2 * PI * PI * sinT);
        return 0;
    }
    Spec SamplePoint(Sampler &, ScatterEvent &, PartialLightSample *ls) const override { ls->pdf *= 0; ls->point = V3(0, 0, 0); return Spec(0); }
    Spec Visibility(const V3 &sp, ScatterEvent &ev, Sampler &s, PartialLightSample *ls) const override {
        const V3 wi = (ls->point - sp).Normalised();
        Spec Tr(1);
        if (LRayEscapes(Ray{sp, wi}, ev, s, &Tr)) return Tr;
        ls->pdf = 0;
        return Spec(0);
    }
    Spec Le(const Ray &r) const override { return LeDir(r.d); }
    Spec L(const ScatterEvent &ev) const override { return LeDir(ev.wi); }
    Real Area() const override { return PI * radius * radius; }
    Real Irradiance() const override { return intensity; }
    Bounds GetBounds() const override { return bounds; }
    V3 GetDirection() const override { return V3(0, 0, 0); }
};

/* PowerLightSampler (LightSampler.cpp:14-35) */
struct PowerSamplerO : LightSampler {
    const Scene *sc; Piecewise1D d; Real invTotal = 0;
    void Commit() {
        std::vector<Real> imp(sc->lights.size()); Real tot = 0;
        for (size_t i = 0; i < imp.size(); ++i) { imp[i] = sc->lights[i]->Power(); tot += imp[i]; }
        d = Piecewise1D(imp.data(), (unsigned)imp.size());
        invTotal = (Real)1 / tot;
    }
    const LightBase *Sample(const ScatterEvent &, Sampler &s, Real *pdf) const override { return sc->lights[d.SampleDiscrete(s.Get1D(), pdf)]; }
    Real Pdf(const V3 &, const V3 &, unsigned, const LightBase *l) const override { return l->Power() * invTotal; }
};

/* ManyLightSampler (ManyLightSampler.cpp) */
struct Cone { V3 axis = V3(0, 1, 0); Real thetaO = 0, thetaE = 0; };
static Cone MakeCone(const V3 &axis) { Cone c; c.axis = axis; c.thetaO = 0; c.thetaE = PI / (Real)2; return c; }
/* OrientationCone::Union (ManyLightSampler.cpp:50-64), including its in-place swap of the operands. */
static Cone ConeUnion(Cone *a, Cone *b) {
    if (b->thetaO > a->thetaO) std::swap(*a, *b);
    const Real thetaE = std::max(a->thetaE, b->thetaE);
    const Real thetaD = std::acos(clampr(Dot(a->axis, b->axis), 0, 1));
    if (std::min(thetaD + b->thetaO, (Real)PI) <= a->thetaO) { Cone r; r.axis = a->axis; r.thetaO = a->thetaO; r.thetaE = thetaE; return r; }
    const Real thetaO = (a->thetaO + thetaD + b->thetaO) * (Real).5;
    if (thetaO >= PI) { Cone r; r.axis = a->axis; r.thetaO = PI; r.thetaE = thetaE; return r; }
    const Real thetaR = thetaO - a->thetaO;
    Cone r; r.axis = Rotate(a->axis, Cross(a->axis, b->axis), thetaR); r.thetaO = thetaO; r.thetaE = thetaE;
    return r;
}
static Cone ConeUnionT(Cone a, Cone b) { return ConeUnion(&a, &b); }
static Real MOmega(const Cone &c) {   /* :71-78 */
    const Real cosO = std::cos(c.thetaO);
    const Real sinO = std::sqrt(1 - cosO * cosO);
    const Real a = PI2 * ((Real)1 - cosO);
    const Real thetaW2 = std::min(c.thetaO + c.thetaE, (Real)PI) * (Real)2;
    const Real b = thetaW2 * sinO - std::cos(c.thetaO - thetaW2) - (Real)2 * c.thetaO * sinO + cosO;
    return a + PI * (Real).5 * b;
}
struct TreeSamplerO : LightSampler {
    struct Node { Node *ch[2] = {nullptr, nullptr}; Node *parent = nullptr; unsigned first = 0, num = 0; Bounds b; Cone cone; Real power = 0, var = 0; };
    struct Bucket { Real power = 0; Bounds b; Cone cone; };
    const Scene *sc;
    std::vector<const LightBase *> lights;
    const LightBase *inf = nullptr;
    Real treePower = 0, infPower = 0;   /* B11: initialised */
    std::vector<std::unique_ptr<Node>> store;
    Node *root = nullptr;
    std::map<unsigned, Piecewise1D> leafDist;
    std::map<const LightBase *, std::pair<Node *, unsigned>> leafOf;
    std::map<std::pair<const LightBase *, unsigned>, const LightBase *> triMap;   /* (MeshLight, prim) -> TriangleLight */

    Node *NewNode() { store.emplace_back(new Node()); return store.back().get(); }
    Real PowerVariance(unsigned first, unsigned n) const {
        std::vector<Real> p(n); Real mean = 0;
        for (unsigned i = 0; i < n; ++i) { p[i] = lights[i + first]->Power(); mean += p[i]; }
        mean /= (Real)n;
        Real sum = 0;
        for (unsigned i = 0; i < n; ++i) { const Real t = p[i] - mean; sum += t * t; }
        return sum / (Real)(n - 1);
    }
    static Real SAOH(const Node &P, const Bucket &R, const Bucket &L, unsigned axis) {
        const V3 box = P.b.max - P.b.min;
        const Real lenMax = std::max(std::max(box.x, box.y), box.z);
        const Real Kr = lenMax / box[axis];
        const Real m = P.b.SurfaceArea() * MOmega(P.cone);
        const Real mL = L.power * L.b.SurfaceArea() * MOmega(L.cone);
        const Real mR = R.power * R.b.SurfaceArea() * MOmega(R.cone);
        return Kr * (mL + mR) / m;
    }
    void InitLeaf(Node *n) {
        std::vector<Real> d(n->num);
        for (unsigned i = 0; i < n->num; ++i) {
            d[i] = lights[n->first + i]->Power();
            leafOf[lights[n->first + i]] = {n, i};
            treePower += d[i];
        }
        leafDist[n->first] = Piecewise1D(d.data(), n->num);
        n->ch[0] = n->ch[1] = nullptr;
    }
    bool SplitAxis(Node *n, unsigned axis, Real *minCost, unsigned *bi, Bucket *lb, Bucket *rb) {
        const unsigned NB = 12;
        Bucket bk[NB]; bool init[NB] = {false};
        for (unsigned i = n->first; i < n->first + n->num; ++i) {
            const LightBase *l = lights[i];
            unsigned b = ToUnsigned((Real)NB * n->b.Offset(l->GetBounds().Center())[axis]);
            if (b == NB) b = NB - 1;
            if (b > NB) b = 0;    /* out-of-range conversion never occurs for offsets in [0, 1] */
            if (!init[b]) { bk[b].power = l->Power(); bk[b].b = l->GetBounds(); bk[b].cone = MakeCone(l->GetDirection()); init[b] = true; }
            else { bk[b].power += l->Power(); bk[b].b = Union(bk[b].b, l->GetBounds()); bk[b].cone = ConeUnionT(bk[b].cone, MakeCone(l->GetDirection())); }
        }
        bool cheaper = false;
        for (unsigned i = 0; i < NB - 1; ++i) {
            Bucket bL; bL.power = 0; bL.b = bk[0].b; bL.cone = bk[0].cone;
            Bucket bR; bR.power = 0; bR.b = bk[i + 1].b; bR.cone = bk[i + 1].cone;
            for (unsigned j = 0; j <= i; ++j) { bL.b = Union(bL.b, bk[j].b); bL.cone = ConeUnion(&bL.cone, &bk[j].cone); bL.power += bk[j].power; }
            for (unsigned j = i + 1; j < NB; ++j) { bR.b = Union(bR.b, bk[j].b); bR.cone = ConeUnion(&bR.cone, &bk[j].cone); bR.power += bk[j].power; }
            const Real cost = SAOH(*n, bR, bL, axis);
            if (cost < *minCost) { *minCost = cost; *lb = bL; *rb = bR; *bi = i; cheaper = true; }
        }
        return cheaper;
    }
    void RecursiveBuild(Node *n) {
        n->b = lights[n->first]->GetBounds();
        n->cone = MakeCone(lights[n->first]->GetDirection());
        for (unsigned i = 0; i < n->num; ++i) {
            n->b = Union(n->b, lights[i + n->first]->GetBounds());
            n->cone = ConeUnionT(n->cone, MakeCone(lights[i + n->first]->GetDirection()));
        }
        Bucket lb, rb; Real minCost = INF; unsigned bi = 0; int axis = -1;
        for (int i = 0; i < 3; ++i) if (SplitAxis(n, (unsigned)i, &minCost, &bi, &lb, &rb)) axis = i;
        if (n->num > 1 && minCost < n->power) {
            auto pred = [&](const LightBase *l) {
                unsigned b = ToUnsigned(n->b.Offset(l->GetBounds().Center())[axis] * (Real)12);
                if (b == 12) b--;
                return b <= bi;
            };
            const LightBase **beg = &lights[n->first];
            const LightBase **it = std::partition(beg, beg + n->num, pred);
            const unsigned pivot = (unsigned)(it - &lights[0]);
            const unsigned ln = pivot - n->first, rn = n->num - ln;
            if (ln != 0 && rn != 0) {
                Node *L = NewNode(); Node *R = NewNode();
                L->parent = n; L->first = n->first; L->num = ln; L->b = lb.b; L->cone = lb.cone; L->power = lb.power; L->var = PowerVariance(n->first, ln);
                R->parent = n; R->first = pivot; R->num = rn; R->b = rb.b; R->cone = rb.cone; R->power = rb.power; R->var = PowerVariance(pivot, rn);
                n->ch[0] = L; n->ch[1] = R;
                RecursiveBuild(L); RecursiveBuild(R);
            } else InitLeaf(n);
        } else InitLeaf(n);
    }
    /* InitLights (ManyLightSampler.cpp:250-303).  Triangle lights come first, ordered by mesh light
     * then triangle index (the reference uses unordered_map iteration order here). */
    void Commit() {
        std::vector<const LightBase *> rest;
        for (const LightBase *l : sc->lights) {
            if (l->IsEnv()) { inf = l; continue; }
            if (l->IsMesh()) {
                const MeshLight *ml = static_cast<const MeshLight *>(l);
                for (size_t i = 0; i < ml->triLights.size(); ++i) {
                    lights.push_back(&ml->triLights[i]);
                    triMap[{l, (unsigned)i}] = &ml->triLights[i];
                }
            } else rest.push_back(l);
        }
        for (auto *l : rest) lights.push_back(l);
        if (!lights.empty()) {
            root = NewNode();
            root->num = (unsigned)lights.size(); root->first = 0;
            root->b = lights[0]->GetBounds(); root->power = 0; root->var = 0;
            root->cone = MakeCone(lights[0]->GetDirection());
            for (unsigned i = 0; i < root->num; ++i) {
                root->b = Union(root->b, lights[i]->GetBounds());
                root->cone = ConeUnionT(root->cone, MakeCone(lights[i]->GetDirection()));
                root->power += lights[i]->Power();
            }
        }
        treePower = 0;
        if (inf) infPower = inf->Power() * (Real).1;
        if (!lights.empty()) RecursiveBuild(root);
    }
    /* ImportanceMeasure (:305-326), useSplits = true */
    static Real Importance(const V3 &p, const V3 &nS, const Node *n) {
        V3 delta = n->b.Center() - p;
        const Real diam = n->b.DiagonalLength();
        const Real d2 = Dot(delta, delta);
        const Real d = std::sqrt(d2);
        const Real invD = (Real)1 / d;
        delta = delta * invD;
        const Real theta = std::acos(Dot(delta, n->cone.axis));
        const Real thetaU = std::atan((diam * (Real).5) * invD);
        const Real thetaDash = smax(theta - n->cone.thetaO - thetaU, (Real)0);
        if (thetaDash < n->cone.thetaE) {
            const Real E = n->power;
            const Real thetaI = std::acos(Dot(delta, nS));
            return (std::cos(smax(thetaI - thetaU, (Real)0)) * E) / d2 * std::cos(thetaDash);
        }
        return 0;
    }
    const LightBase *Pick(const V3 &p, const V3 &nS, Real eps, const Node *n, Real *pdf) const {   /* :355-378 */
        if (!n->ch[0] && !n->ch[1]) {
            Real lp = 1;
            const unsigned i = leafDist.at(n->first).SampleDiscrete(eps, &lp);
            *pdf *= lp;
            return lights[n->first + i];
        }
        const Real IL = Importance(p, nS, n->ch[0]);
        const Real IR = Importance(p, nS, n->ch[1]);
        const Real PL = IL / (IL + IR);
        const Real PR = 1 - PL;
        if (eps < PL) { eps /= PL; *pdf *= PL; return Pick(p, nS, eps, n->ch[0], pdf); }
        eps = (eps - PL) / PR; *pdf *= PR;
        return Pick(p, nS, eps, n->ch[1], pdf);
    }
    Real RecursivePDF(const V3 &p, const V3 &nS, const Node *n, const Node *child) const {   /* :380-393, B8 */
        if (child) {
            const int side = child == n->ch[0] ? 0 : 1;
            const Real IL = Importance(p, nS, n->ch[0]);
            const Real IR = Importance(p, nS, n->ch[1]);
            Real pd[2];
            pd[0] = IL / (IL + IR);
            pd[1] = 1 - pd[0];
            if (n->parent) pd[side] *= RecursivePDF(p, nS, n->parent, n);
            return pd[side];
        }
        if (n->parent) return RecursivePDF(p, nS, n->parent, n);
        return 1;
    }
    const LightBase *Sample(const ScatterEvent &ev, Sampler &s, Real *pdf) const override {   /* :17-27 */
        Real eps = s.Get1D();
        const Real pTree = treePower / (infPower + treePower);
        if (eps < pTree) {
            eps /= pTree;
            *pdf *= pTree;
            return Pick(ev.hit->point, ev.hit->normalS, s.Get1D(), root, pdf);
        }
        *pdf *= 1 - pTree;
        return inf;
    }
    Real Pdf(const V3 &p, const V3 &nS, unsigned primId, const LightBase *l) const override {   /* :29-35 */
        if (l == inf) return infPower / (infPower + treePower);
        auto tl = triMap.find({l, primId});
        if (tl != triMap.end()) l = tl->second;
        const auto &ref = leafOf.at(l);
        return leafDist.at(ref.first->first).PDF(ref.second) * RecursivePDF(p, nS, ref.first, nullptr);
    }
};

/* ------------------------------------------------------------------ integrator */
static inline Real PowerHeuristic(Real f, Real g) { return (f * f) / (f * f + g * g); }

struct Integrator {
    const Scene &sc;
    Bxdf bx;
    int maxBounces, minBounces;
    Integrator(const Scene &s, int maxB, int minB) : sc(s), bx{s.graph}, maxBounces(maxB), minBounces(minB) {}

    const Material &Mat(const RayHit &h) const { return sc.materials[h.object->material]; }

    /* LdMediumPoint (MISVolumetricPathIntegrator.cpp:23-69) */
    Spec LdMediumPoint(ScatterEvent &ev, Sampler &s, const V3 &p, PartialLightSample *ls, V3 *wiOut,
                       const V3 &sampPoint, const V3 &sampNormal) const {
        RayHit &hit = *ev.hit;
        Real partialLightPDF = ls->pdf;
        hit.point = p;
        Spec Li(0);
        if (ls->light) Li = ls->Le * ls->light->Visibility(p, ev, s, ls);
        else ls->pdf = 0;
        Real scatteringPDF, lightPDF = ls->pdf;
        Spec Ld(0);
        if (lightPDF > 0 && !Li.IsBlack()) {
            scatteringPDF = ev.medium->p(ev.wo, ev.wi);
            if (scatteringPDF > 0) {
                const Real w = PowerHeuristic(lightPDF, scatteringPDF);
                Ld += Li * Spec(scatteringPDF) * w / lightPDF;
            }
        }
        scatteringPDF = ev.medium->Sample_p(ev.wo, &ev.wi, s);
        *wiOut = ev.wi;
        Ray r{p, ev.wi};
        Spec Tr(1);
        const bool hitSurf = sc.IntersectTr(r, hit, s, ev.medium, &Tr);
        if (scatteringPDF > 0) {
            const LightBase *nl = hitSurf ? Mat(hit).light : sc.envLight;
            if (nl) {
                if (nl != ls->light) partialLightPDF = sc.lightSampler->Pdf(sampPoint, sampNormal, hit.primId, nl);
                lightPDF = partialLightPDF * nl->PDF_Li(ev);
                Li = Spec(0);
                if (hitSurf) Li = nl->L(ev); else Li = nl->Le(r);
                const Real w = PowerHeuristic(scatteringPDF, lightPDF);
                if (!Li.IsBlack() && lightPDF > 0) Ld += Li * Tr * w / scatteringPDF;
            }
        }
        return Ld;
    }

    /* PathIntegrator::Li (PathIntegrator.cpp:15-88); B7 patched (tree pdf at the shading point);
     * at most 256 null-surface crossings. */
    Spec LiPath(Ray r, Sampler &s) const {
        Spec L(0), beta(1);
        RayHit hit;
        ScatterEvent ev;
        ev.hit = &hit;
        ev.scene = &sc;
        ev.wo = -r.d;
        bool scatterIntersect = false;
        int nullCrossings = 0;
        for (int bounces = 0; bounces < maxBounces; ++bounces) {
            if (bounces == 0 ? sc.Intersect(r, hit) : scatterIntersect) {
                if (bounces == 0 && Mat(hit).light) L += Mat(hit).light->L(ev);
                const Material &m = Mat(hit);
                if (m.bxdf >= 0) {
                    ev.wo = -r.d;
                    ev.SurfaceLocalise();
                    Real lightDistPdf = 1;
                    const V3 sp = hit.point, sn = hit.normalS;
                    const LightBase *l = sc.lightSampler->Sample(ev, s, &lightDistPdf);
                    Spec Ld(0);
                    Real scatteringPDF = 0, lightPDF = 0;
                    Spec f, Li = l ? l->Sample_Li(ev, s, lightPDF) : Spec(0);
                    lightPDF *= lightDistPdf;
                    if (lightPDF > 0 && !Li.IsBlack()) {
                        f = bx.f(m.bxdf, ev) * std::abs(ev.wiL.y);
                        scatteringPDF = bx.Pdf(m.bxdf, ev.woL, ev.wiL, ev);
                        if (!f.IsBlack() && scatteringPDF > 0) Ld += Li * f * PowerHeuristic(lightPDF, scatteringPDF) / lightPDF;
                    }
                    f = bx.Sample_f(m.bxdf, ev, s, scatteringPDF);
                    f *= std::abs(ev.wiL.y);
                    r.o = hit.point;
                    r.d = ev.wi;
                    scatterIntersect = sc.Intersect(r, hit);
                    if (scatteringPDF > 0 && !f.IsBlack()) {
                        const LightBase *nl = scatterIntersect ? Mat(hit).light : sc.envLight;
                        if (nl) {
                            if (nl != l) lightDistPdf = sc.lightSampler->Pdf(sp, sn, hit.primId, nl);
                            lightPDF = lightDistPdf * nl->PDF_Li(ev);
                            Li = scatterIntersect ? nl->L(ev) : nl->Le(r);
                            if (!Li.IsBlack() && lightPDF > 0) Ld += Li * f * PowerHeuristic(scatteringPDF, lightPDF) / scatteringPDF;
                        }
                    } else break;
                    L += beta * Ld;
                    beta *= f / scatteringPDF;
                } else {
                    r.o = hit.point + hit.normalG * (Dot(r.d, hit.normalG) < 0 ? -SURFACE_EPSILON : SURFACE_EPSILON);
                    if (bounces > 0) scatterIntersect = sc.Intersect(r, hit);
                    if (++nullCrossings > 256) break;
                    bounces--;
                    continue;
                }
                if (bounces > minBounces) {
                    const Real q = smax((Real).05, 1 - beta.y());
                    if (s.Get1D() < q) break;
                    beta /= (Real)1 - q;
                }
            } else {
                if (bounces == 0 && sc.envLight) L += sc.envLight->Le(r);
                break;
            }
        }
        return L;
    }

    /* VolumetricPathIntegrator::Li (VolumetricPathIntegrator.cpp:20-160); B7 patched at surface
     * and medium vertices; no environment light: nothing on escape (the reference dereferences
     * null); at most 256 null-surface crossings. */
    Spec LiVolPath(Ray r, Sampler &s) const {
        Spec L(0), beta(1);
        RayHit hit;
        ScatterEvent ev;
        ev.hit = &hit;
        ev.scene = &sc;
        ev.wo = -r.d;
        bool scatterIntersect = false;
        int nullCrossings = 0;
        ev.medium = nullptr;
        for (int bounces = 0; bounces < maxBounces; ++bounces) {
            if (bounces == 0 ? sc.Intersect(r, hit) : scatterIntersect) {
                if (bounces == 0 && Mat(hit).light) {
                    if (ev.medium) L += Mat(hit).light->L(ev) * ev.medium->Tr(hit.tFar);
                    else L += Mat(hit).light->L(ev);
                }
                Real distanceT = 0, distPdf = 0;
                if (ev.medium) beta *= ev.medium->SampleDistance(s, ev, &distanceT, &distPdf);
                else ev.mediumInteraction = false;
                if (!ev.mediumInteraction) {
                    const Material &m = Mat(hit);
                    if (m.bxdf >= 0) {
                        ev.wo = -r.d;
                        ev.SurfaceLocalise();
                        Real lightDistPdf = 1;
                        const V3 sp = hit.point, sn = hit.normalS;
                        const LightBase *l = sc.lightSampler->Sample(ev, s, &lightDistPdf);
                        Spec Ld(0);
                        Real scatteringPDF = 0, lightPDF = 0;
                        Spec f, Li = l ? l->Sample_Li(ev, s, lightPDF) : Spec(0);
                        lightPDF *= lightDistPdf;
                        if (lightPDF > 0 && !Li.IsBlack()) {
                            f = bx.f(m.bxdf, ev) * std::abs(ev.wiL.y);
                            scatteringPDF = bx.Pdf(m.bxdf, ev.woL, ev.wiL, ev);
                            if (!f.IsBlack() && scatteringPDF > 0) Ld += Li * f * PowerHeuristic(lightPDF, scatteringPDF) / lightPDF;
                        }
                        f = bx.Sample_f(m.bxdf, ev, s, scatteringPDF);
                        f *= std::abs(ev.wiL.y);
                        r.o = hit.point;
                        r.d = ev.wi;
                        ev.medium = sc.GetMedium(m, ev.wi, hit.normalG);
                        scatterIntersect = sc.Intersect(r, hit);
                        if (scatteringPDF > 0 && !f.IsBlack()) {
                            const LightBase *nl = scatterIntersect ? Mat(hit).light : sc.envLight;
                            if (nl) {
                                if (nl != l) lightDistPdf = sc.lightSampler->Pdf(sp, sn, hit.primId, nl);
                                lightPDF = lightDistPdf * nl->PDF_Li(ev);
                                Li = scatterIntersect ? nl->L(ev) : nl->Le(r);
                                if (!Li.IsBlack() && lightPDF > 0) Ld += Li * f * PowerHeuristic(scatteringPDF, lightPDF) / scatteringPDF;
                            }
                        } else break;
                        L += beta * Ld;
                        beta *= f / scatteringPDF;
                    } else {
                        ev.medium = sc.GetMedium(m, r.d, hit.normalG);
                        r.o = hit.point + hit.normalG * (Dot(hit.normalG, r.d) < 0 ? -SURFACE_EPSILON : SURFACE_EPSILON);
                        if (bounces > 0) scatterIntersect = sc.Intersect(r, hit);
                        if (++nullCrossings > 256) break;
                        bounces--;
                        continue;
                    }
                } else if (ev.medium) {
                    ev.wo = -r.d;
                    const V3 scatterPoint = r.o + r.d * distanceT;
                    hit.point = scatterPoint;
                    Real lightDistPdf = 1;
                    const V3 sp = hit.point, sn = hit.normalS;
                    const LightBase *l = sc.lightSampler->Sample(ev, s, &lightDistPdf);
                    Spec Ld(0);
                    Real scatteringPDF = 0, lightPDF = 0;
                    Spec Li = l ? l->Sample_Li(ev, s, lightPDF) : Spec(0);
                    lightPDF *= lightDistPdf;
                    if (lightPDF > 0 && !Li.IsBlack()) {
                        scatteringPDF = ev.medium->p(ev.wo, ev.wi);
                        if (scatteringPDF > 0) Ld += Li * Spec(scatteringPDF) * PowerHeuristic(lightPDF, scatteringPDF) / lightPDF;
                    }
                    scatteringPDF = ev.medium->Sample_p(ev.wo, &ev.wi, s);
                    r.o = hit.point;
                    r.d = ev.wi;
                    Spec Tr(1);
                    const Medium *med = ev.medium;
                    scatterIntersect = sc.IntersectTr(r, hit, s, med, &Tr);
                    if (scatteringPDF > 0) {
                        const LightBase *nl = scatterIntersect ? Mat(hit).light : sc.envLight;
                        if (nl) {
                            if (nl != l) lightDistPdf = sc.lightSampler->Pdf(sp, sn, hit.primId, nl);
                            lightPDF = lightDistPdf * nl->PDF_Li(ev);
                            Li = scatterIntersect ? nl->L(ev) : nl->Le(r);
                            if (!Li.IsBlack() && lightPDF > 0) Ld += Li * Tr * PowerHeuristic(scatteringPDF, lightPDF) / scatteringPDF;
                        }
                    } else break;
                    r.o = scatterPoint;
                    scatterIntersect = sc.Intersect(r, hit);
                    L += beta * Ld;
                }
                if (bounces > minBounces) {
                    const Real q = smax((Real).05, 1 - beta.y());
                    if (s.Get1D() < q) break;
                    beta /= (Real)1 - q;
                }
            } else {
                if (bounces == 0 && sc.envLight) L += sc.envLight->Le(r) * beta;
                break;
            }
        }
        return L;
    }

    /* DirectLightingIntegrator::Li (DirectLightingIntegrator.cpp:13-29) with SampleOneLight and
     * EstimateDirect (Integrator.cpp:5-55), quirks kept; null surfaces crossed iteratively (256 at
     * most); no environment light or no light: 0 (the reference dereferences null); a light-selection
     * pdf that is not positive gives 0 (the reference divides by it). */
    Spec LiDirect(Ray r, Sampler &s) const {
        RayHit hit;
        for (int guard = 0; guard < 256; ++guard) {
            if (!sc.Intersect(r, hit)) return sc.envLight ? sc.envLight->Le(r) : Spec(0);
            const Material &m = Mat(hit);
            if (m.bxdf < 0) { r.o = hit.point + r.d * (Real).0001; continue; }
            ScatterEvent ev;
            ev.hit = &hit;
            ev.scene = &sc;
            ev.wo = -r.d;
            ev.SurfaceLocalise();
            Real lightPdf = 1;
            const LightBase *l = sc.lightSampler->Sample(ev, s, &lightPdf);
            if (!l) return Spec(0);
            const bool pdfOk = lightPdf > 0;   /* a zero or NaN selection pdf would make the estimate NaN */
            Spec Ld(0);
            Real scatteringPDF = 0, lightPDF = 0;
            Spec Li = l->Sample_Li(ev, s, lightPDF);
            if (lightPDF > 0 && !Li.IsBlack()) {
                const Spec f = bx.f(m.bxdf, ev) * std::abs(ev.wiL.y);
                scatteringPDF = bx.Pdf(m.bxdf, ev.woL, ev.wiL, ev);
                if (!f.IsBlack() && scatteringPDF > 0) Ld += Li * f * PowerHeuristic(lightPDF, scatteringPDF) / lightPDF;
            }
            Spec f = bx.Sample_f(m.bxdf, ev, s, scatteringPDF);
            f *= std::abs(ev.wiL.y);
            if (scatteringPDF > 0 && !f.IsBlack()) {
                lightPDF = l->PDF_Li_S(ev, s);
                if (lightPDF == 0) return pdfOk ? Ld / lightPdf : Spec(0);
                const Real w = PowerHeuristic(scatteringPDF, lightPDF);
                RayHit lh;
                ScatterEvent be;
                be.scene = &sc;
                be.hit = &lh;
                be.wo = -ev.wi;
                const Ray br{hit.point + hit.normalG * (Real).00001, ev.wi};
                Spec Lc(0);
                if (sc.Intersect(br, lh)) {
                    if (Mat(lh).light == l) Lc = Mat(lh).light->L(be);
                } else {
                    Lc = l->Le(br);
                }
                if (!Lc.IsBlack()) Ld += f * Lc * w / scatteringPDF;
            }
            return pdfOk ? Ld / lightPdf : Spec(0);
        }
        return Spec(0);
    }

    /* NormalPass / DepthPass (UtilityIntegrators.cpp:7-53) as UtilityIntegrator::Li. */
    Spec LiPass(Ray r, bool normal) const {
        RayHit hit;
        Real c[3];
        if (sc.Intersect(r, hit)) {
            if (normal) { c[0] = hit.normalS.x * (Real).5 + (Real).5; c[1] = hit.normalS.y * (Real).5 + 1; c[2] = hit.normalS.z * (Real).5 + (Real).5; }
            else { const Real d = std::pow((hit.point - r.o).Magnitude() / (Real)100, (Real)1); c[0] = c[1] = c[2] = d; }
        } else if (normal) { c[0] = c[1] = c[2] = 0; }
        else { c[0] = 1; c[1] = 0; c[2] = 1; }
        return FromRGB(c, false);
    }

    /* MISVolumetricPathIntegrator::Li (MISVolumetricPathIntegrator.cpp:71-215) */
    Spec Li(Ray r, Sampler &s) const {
        Spec L(0), beta(1);
        RayHit hit;
        ScatterEvent ev;
        ev.hit = &hit;
        ev.scene = &sc;
        ev.wo = -r.d;
        bool scatterIntersect = false;
        int nullCrossings = 0;   /* null surfaces do not count as bounces; bound them (256) */
        ev.medium = nullptr;   /* InMedium: camera outside all media (B19) */
        for (int bounces = 0; bounces < maxBounces; ++bounces) {
            if (bounces == 0 ? sc.Intersect(r, hit) : scatterIntersect) {
                if (bounces == 0) {
                    if (Mat(hit).light) {
                        if (ev.medium) L += Mat(hit).light->L(ev) * ev.medium->Tr(hit.tFar);
                        else L += Mat(hit).light->L(ev);
                    }
                }
                if (ev.medium) {
                    PartialLightSample ls;                       /* B5: pdf starts at 1 */
                    const V3 sp = hit.point, sn = hit.normalS;   /* B7: sample point/normal */
                    ls.light = sc.lightSampler->Sample(ev, s, &ls.pdf);
                    if (ls.light) ls.Le = ls.light->SamplePoint(s, ev, &ls);
                    else { ls.pdf = 0; ls.point = hit.point; }
                    const int DISTANCE = 0, EQUIANGULAR = 1;
                    const int choice = (s.Get1D() > 0.5) ? DISTANCE : EQUIANGULAR;
                    Real distT, distPdf, eqT, eqPdf;
                    Spec mTr[2]; bool mInt[2];
                    mTr[DISTANCE] = ev.medium->SampleDistance(s, ev, &distT, &distPdf);
                    mInt[DISTANCE] = ev.mediumInteraction;
                    mTr[EQUIANGULAR] = ev.medium->SampleEquiangular(r, s, ev, ls.point, &eqT, &eqPdf);
                    mInt[EQUIANGULAR] = ev.mediumInteraction;
                    ev.mediumInteraction = mInt[DISTANCE] && mInt[EQUIANGULAR];
                    if (!ev.mediumInteraction) beta *= mTr[DISTANCE];
                    if (ev.mediumInteraction) {
                        ev.wo = -r.d;
                        Spec Ld(0);
                        V3 mp[2];
                        mp[DISTANCE] = r.o + r.d * distT;
                        mp[EQUIANGULAR] = r.o + r.d * eqT;
                        const Real distPdf2 = ev.medium->PDFDistance(eqT);
                        const Real eqPdf2 = ev.medium->PDFEquiangular(r, ls.point, hit.tFar, distT);
                        const Real distW = PowerHeuristic(distPdf, eqPdf2);
                        const Real eqW = PowerHeuristic(eqPdf, distPdf2);
                        V3 wi[2];
                        const Spec liD = LdMediumPoint(ev, s, mp[DISTANCE], &ls, &wi[DISTANCE], sp, sn);
                        Ld += liD * mTr[DISTANCE] * distW;
                        const Spec liE = LdMediumPoint(ev, s, mp[EQUIANGULAR], &ls, &wi[EQUIANGULAR], sp, sn);
                        Ld += liE * mTr[EQUIANGULAR] * eqW;
                        r.o = mp[choice];
                        r.d = wi[choice];
                        scatterIntersect = sc.Intersect(r, hit);
                        L += Ld;
                        beta *= mTr[choice];
                    }
                } else ev.mediumInteraction = false;

                if (!ev.mediumInteraction) {
                    const Material &m = Mat(hit);
                    if (m.bxdf >= 0) {
                        ev.wo = -r.d;
                        ev.SurfaceLocalise();
                        Real lightDistPdf = 1;
                        const V3 sp = hit.point, sn = hit.normalS;   /* B7 */
                        const LightBase *l = sc.lightSampler->Sample(ev, s, &lightDistPdf);
                        Spec Ld(0);
                        Real scatteringPDF = 0, lightPDF = 0;
                        Spec f, Li = l ? l->Sample_Li(ev, s, lightPDF) : Spec(0);
                        lightPDF *= lightDistPdf;
                        if (lightPDF > 0 && !Li.IsBlack()) {
                            f = bx.f(m.bxdf, ev) * std::abs(ev.wiL.y);
                            scatteringPDF = bx.Pdf(m.bxdf, ev.woL, ev.wiL, ev);
                            if (!f.IsBlack() && scatteringPDF > 0) {
                                const Real w = PowerHeuristic(lightPDF, scatteringPDF);
                                Ld += Li * f * w / lightPDF;
                            }
                        }
                        f = bx.Sample_f(m.bxdf, ev, s, scatteringPDF);
                        f *= std::abs(ev.wiL.y);
                        r.o = hit.point;
                        r.d = ev.wi;
                        ev.medium = sc.GetMedium(m, ev.wi, hit.normalG);
                        scatterIntersect = sc.Intersect(r, hit);
                        if (scatteringPDF > 0 && !f.IsBlack()) {
                            const LightBase *nl = scatterIntersect ? Mat(hit).light : sc.envLight;
                            if (nl) {
                                if (nl != l) lightDistPdf = sc.lightSampler->Pdf(sp, sn, hit.primId, nl);
                                lightPDF = lightDistPdf * nl->PDF_Li(ev);
                                Li = Spec(0);
                                if (scatterIntersect) Li = nl->L(ev); else Li = nl->Le(r);
                                const Real w = PowerHeuristic(scatteringPDF, lightPDF);
                                if (!Li.IsBlack() && lightPDF > 0) Ld += Li * f * w / scatteringPDF;
                            }
                        } else break;
                        L += beta * Ld;
                        beta *= f / scatteringPDF;
                    } else {
                        ev.medium = sc.GetMedium(m, r.d, hit.normalG);
                        r.o = hit.point + hit.normalG * (Dot(ev.hit->normalG, r.d) < 0 ? -SURFACE_EPSILON : SURFACE_EPSILON);
                        if (bounces > 0) scatterIntersect = sc.Intersect(r, hit);
                        if (++nullCrossings > 256) break;
                        bounces--;
                        continue;
                    }
                }
                if (bounces > minBounces) {
                    const Real q = smax((Real).05, 1 - beta.y());
                    if (s.Get1D() < q) break;
                    beta /= (Real)1 - q;
                }
            } else {
                if (bounces == 0 && sc.envLight) L += sc.envLight->Le(r) * beta;
                break;
            }
        }
        return L;
    }
};

/* ------------------------------------------------------------------ scene setup */
struct Oracle {
    Scene sc;
    std::vector<std::unique_ptr<Piecewise2D>> masks;   /* per texture: masked-aperture distribution or null */
    std::string err;
    bool Load(const lgpu_scene_desc *d);
};

static void Inverse3(const Real *m, Real *inv) {
    /* column-major m: col0 = m[0..2] */
    const double a = m[0], b = m[3], c = m[6], dd = m[1], e = m[4], f = m[7], g = m[2], h = m[5], i = m[8];
    const double A = e * i - f * h, B = -(dd * i - f * g), C = dd * h - e * g;
    const double det = a * A + b * B + c * C;
    const double id = 1.0 / det;
    const double r[9] = {A * id, -(b * i - c * h) * id, (b * f - c * e) * id,
                         B * id, (a * i - c * g) * id, -(a * f - c * dd) * id,
                         C * id, -(a * h - b * g) * id, (a * e - b * dd) * id};
    /* r is row-major inverse; store column-major */
    inv[0] = (Real)r[0]; inv[3] = (Real)r[1]; inv[6] = (Real)r[2];
    inv[1] = (Real)r[3]; inv[4] = (Real)r[4]; inv[7] = (Real)r[5];
    inv[2] = (Real)r[6]; inv[5] = (Real)r[7]; inv[8] = (Real)r[8];
}

bool Oracle::Load(const lgpu_scene_desc *d) {
    sc.graph.nodes.assign(d->nodes, d->nodes + d->num_nodes);
    for (int t = 0; t < d->num_textures; ++t) {
        const lgpu_texture_desc &td = d->textures[t];
        sc.graph.tex.emplace_back(td.rgba, td.rgba + (size_t)td.width * td.height * 4);
        sc.graph.texW.push_back(td.width);
        sc.graph.texH.push_back(td.height);
        masks.emplace_back();
        if (td.aperture_mask) {
            /* MaskedAperture::InitDistribution (Aperture.cpp:38-51): |GetPixelUV(x/w, y/h).r|,
             * bilinear (Texture.h:71-81) */
            const int w = td.width, h = td.height;
            std::vector<Real> img((size_t)w * h);
            for (int y = 0; y < h; ++y) {
                const float vp = (float)y / (float)h;
                for (int x = 0; x < w; ++x) {
                    const float up = (float)x / (float)w;
                    const float fx = std::min((float)(w - 1), clampr(up, 0.f, 1.f) * (float)w);
                    const float fy = std::min((float)(h - 1), clampr(vp, 0.f, 1.f) * (float)h);
                    const unsigned xi = (unsigned)fx, yi = (unsigned)fy;
                    const unsigned x1 = std::min(xi + 1, (unsigned)w - 1), y1 = std::min(yi + 1, (unsigned)h - 1);
                    auto R = [&](unsigned xx, unsigned yy) { return td.rgba[4 * ((size_t)yy * w + xx)]; };
                    const float ya = Lerp(R(xi, yi), R(x1, yi), fx - (float)xi);
                    const float yb = Lerp(R(xi, y1), R(x1, y1), fx - (float)xi);
                    img[x + (size_t)y * w] = std::abs(Lerp(ya, yb, fy - (float)yi));
                }
            }
            masks.back().reset(new Piecewise2D(img.data(), (unsigned)w, (unsigned)h));
        }
    }
    sc.hasVolumes = d->has_volumes != 0;
    sc.meshes.resize(d->num_meshes);
    for (int i = 0; i < d->num_meshes; ++i) {
        const lgpu_mesh_desc &md = d->meshes[i];
        MeshRec &m = sc.meshes[i];
        m.verts.resize(md.num_vertices);
        for (uint32_t k = 0; k < md.num_vertices; ++k) m.verts[k] = V3(md.vertices[3 * k], md.vertices[3 * k + 1], md.vertices[3 * k + 2]);
        m.tris.resize(md.num_triangles);
        for (uint32_t k = 0; k < md.num_triangles; ++k) m.tris[k] = Tri{md.triangles[3 * k], md.triangles[3 * k + 1], md.triangles[3 * k + 2]};
        if (md.normals && md.tangents) {
            m.smooth = true;
            m.normals.resize(md.num_vertices); m.tangents.resize(md.num_vertices); m.tsign.resize(md.num_vertices);
            for (uint32_t k = 0; k < md.num_vertices; ++k) {
                m.normals[k] = V3(md.normals[3 * k], md.normals[3 * k + 1], md.normals[3 * k + 2]);
                m.tangents[k] = V3(md.tangents[4 * k], md.tangents[4 * k + 1], md.tangents[4 * k + 2]);
                m.tsign[k] = md.tangents[4 * k + 3];
            }
        }
        if (md.uvs) {
            m.hasUV = true;
            m.uvs.resize(md.num_vertices);
            for (uint32_t k = 0; k < md.num_vertices; ++k) m.uvs[k] = V2(md.uvs[2 * k], md.uvs[2 * k + 1]);
        }
        m.Build();
    }
    sc.media.resize(d->num_media);
    for (int i = 0; i < d->num_media; ++i) {
        Medium &me = sc.media[i];
        for (int k = 0; k < 3; ++k) { me.sa[k] = d->media[i].sigma_a[k]; me.ss[k] = d->media[i].sigma_s[k]; }
        me.g = d->media[i].g;
        me.Prepare();
    }
    sc.materials.resize(d->num_materials);
    for (int i = 0; i < d->num_materials; ++i) {
        sc.materials[i].bxdf = d->materials[i].bxdf_node;
        sc.materials[i].mi = d->materials[i].medium_interior;
        sc.materials[i].me = d->materials[i].medium_exterior;
    }
    sc.objects.resize(d->num_objects);
    std::vector<Bounds> ob(d->num_objects);
    std::vector<V3> oc(d->num_objects);
    for (int i = 0; i < d->num_objects; ++i) {
        const lgpu_object_desc &od = d->objects[i];
        ObjectRec &o = sc.objects[i];
        o.mesh = od.mesh; o.kind = od.kind; o.material = od.material; o.index = i;
        for (int k = 0; k < 9; ++k) o.m[k] = (od.kind == 1) ? od.xfm[k] : ((k % 4 == 0) ? 1.f : 0.f);
        for (int k = 0; k < 3; ++k) o.t[k] = (od.kind == 1) ? od.xfm[9 + k] : 0.f;
        o.identity = true;
        const Real id[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
        for (int k = 0; k < 9; ++k) if (o.m[k] != id[k]) o.identity = false;
        for (int k = 0; k < 3; ++k) if (o.t[k] != 0) o.identity = false;
        Inverse3(o.m, o.minv);
        for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) o.nrm[c * 3 + r] = o.minv[r * 3 + c];
        const MeshRec &me = sc.meshes[o.mesh];
        Bounds b; bool first = true;
        for (const V3 &v : me.verts) {
            const V3 w = o.identity ? v : MulCM(o.m, v) + V3(o.t[0], o.t[1], o.t[2]);
            b = first ? Bounds(w) : Union(b, w); first = false;
        }
        o.worldBounds = b;
        ob[i] = b; oc[i] = b.Center();
        sc.sceneBounds = (i == 0) ? b : Union(sc.sceneBounds, b);
    }
    BuildBVH(sc.tlas, sc.tlasIdx, ob, oc, 1);
    /* lights */
    for (int i = 0; i < d->num_lights; ++i) {
        const lgpu_light_desc &ld = d->lights[i];
        LightBase *lb = nullptr;
        if (ld.type == LGPU_LIGHT_MESH) {
            MeshLight *ml = new MeshLight();
            ml->sc = &sc; ml->obj = &sc.objects[ld.object]; ml->mesh = &sc.meshes[sc.objects[ld.object].mesh];
            ml->enode = ld.emission_node; ml->esock = ld.emission_socket; ml->intensity = ld.intensity;
            ml->Init();
            lb = ml;
        } else if (ld.type == LGPU_LIGHT_POINT) {
            PointLightO *p = new PointLightO();
            p->sc = &sc; p->pos = V3(ld.position[0], ld.position[1], ld.position[2]);
            p->enode = ld.emission_node; p->esock = ld.emission_socket; p->intensity = ld.intensity;
            lb = p;
        } else if (ld.type == LGPU_LIGHT_SPOT) {
            SpotLightO *p = new SpotLightO();
            p->sc = &sc; p->pos = V3(ld.position[0], ld.position[1], ld.position[2]);
            p->axis = V3(ld.axis[0], ld.axis[1], ld.axis[2]);
            p->cosCone = std::cos(ld.cone_angle); p->cosFall = std::cos(ld.falloff_start);
            p->enode = ld.emission_node; p->esock = ld.emission_socket; p->intensity = ld.intensity;
            lb = p;
        } else if (ld.type == LGPU_LIGHT_ENVIRONMENT) {
            EnvLightO *e = new EnvLightO();
            e->w = ld.env_width; e->h = ld.env_height;
            e->tex.assign(ld.env_texture, ld.env_texture + (size_t)3 * e->w * e->h);
            e->intensity = ld.intensity; e->offset = V2(ld.offset[0], ld.offset[1]);
            e->Init();
            e->bounds = sc.sceneBounds;            /* Scene::Commit (Scene.cpp:20-23) */
            e->radius = e->bounds.MaxLength();
            sc.envLight = e;
            lb = e;
        } else { err = "unknown light type"; return false; }
        sc.lightStore.emplace_back(lb);
        sc.lights.push_back(lb);
    }
    for (int i = 0; i < d->num_materials; ++i)
        if (d->materials[i].light >= 0) sc.materials[i].light = sc.lights[d->materials[i].light];
    if (d->light_strategy == LGPU_LIGHT_STRATEGY_POWER) {
        PowerSamplerO *p = new PowerSamplerO(); p->sc = &sc; p->Commit(); sc.lightSampler.reset(p);
    } else {
        TreeSamplerO *t = new TreeSamplerO(); t->sc = &sc; t->Commit(); sc.lightSampler.reset(t);
    }
    return true;
}

}  // namespace orc

/* ------------------------------------------------------------------ C entry points (oracle only) */
using namespace orc;

struct OracleRun {
    const Oracle *o;
    const lgpu_camera_desc *cam;
    const lgpu_render_opts *opt;
};

static void SetWavelengths(uint32_t key) {
    const Real u = lgpu_rng_float(key, LGPU_DIM_WAVELENGTH);
    const Real l0 = (Real)380 + HERO_RANGE * u;
    for (int i = 0; i < 4; ++i) {
        Real l = l0 + (Real)i * (HERO_RANGE / 4.0f);
        if (l >= (Real)720) l -= HERO_RANGE;
        t_lambda[i] = l;
    }
}

/* Aperture::Sample_p (Aperture.cpp:10-36) */
static V2 ApertureSample(const Oracle *o, const lgpu_camera_desc &c, Sampler &s) {
    const Real size = c.aperture_size;
    switch (c.aperture) {
    case LGPU_APERTURE_BLADE: {   /* BladeAperture::Sample_p (Aperture.cpp:10-19) */
        const Real d = PI2 / (Real)c.blades;
        const Real rnd = PI2 * s.Get1D();
        const Real thetaMin = std::floor(rnd / d) * d;
        const Real thetaMax = thetaMin + d;
        const V2 p1(std::cos(thetaMin), std::sin(thetaMin)), p2(std::cos(thetaMax), std::sin(thetaMax));
        const Real ux = s.Get1D(), uy = s.Get1D();
        return V2((p1.x * ux + p2.x * uy) * size, (p1.y * ux + p2.y * uy) * size);
    }
    case LGPU_APERTURE_CIRCULAR: {   /* CircularAperture::Sample_p (Aperture.cpp:25-27) + SampleUnitDisk */
        const Real ux = s.Get1D(), uy = s.Get1D();
        const Real r = std::sqrt(ux), theta = uy * PI2;
        return V2(r * std::cos(theta) * size - size * (Real).5, r * std::sin(theta) * size - size * (Real).5);
    }
    case LGPU_APERTURE_MASKED: {   /* MaskedAperture::Sample_p (Aperture.cpp:33-36) */
        const Real ux = s.Get1D(), uy = s.Get1D();
        if (!o || c.aperture_mask < 0 || c.aperture_mask >= (int)o->masks.size() || !o->masks[c.aperture_mask])
            return V2(0, 0);   /* unreachable from oracle_render, which rejects such a camera */
        Real pdf;
        const V2 p = o->masks[c.aperture_mask]->SampleContinuous(V2(ux, uy), &pdf);
        return V2(p.x * size - size * (Real).5, p.y * size - size * (Real).5);
    }
    default: return V2(0, 0);
    }
}

/* Camera::GenerateRay (Camera.cpp:41-71) at film coordinates (u, v) of a W x H film; the thin lens
 * draws its aperture point from s. */
static Ray GenerateCameraRay(const Oracle *o, const lgpu_camera_desc &c, int W, int H, Real u, Real v, Sampler &s) {
    const V3 org(c.origin[0], c.origin[1], c.origin[2]);
    const V3 xh(c.x_hat[0], c.x_hat[1], c.x_hat[2]), yh(c.y_hat[0], c.y_hat[1], c.y_hat[2]), zh(c.z_hat[0], c.z_hat[1], c.z_hat[2]);
    const Real tanFov = (Real)std::tan(.5 * c.fov);
    const Real tanFov2 = 2 * tanFov;
    const Real aspect = (Real)H / (Real)W;
    if (c.type == LGPU_CAMERA_SPHERICAL) {   /* SphericalCamera::GenerateRay (Camera.cpp:66-71) */
        const Real phi = PI2 * u + c.offset_phi;
        const Real theta = PI * v + c.offset_theta;
        const V3 d = SphericalDirection(std::sin(theta), std::cos(theta), phi).Normalised();
        return Ray{org, xh * d.x + yh * d.y + zh * d.z};
    }
    if (c.type == LGPU_CAMERA_THIN_LENS) {   /* ThinLensCamera::GenerateRay (Camera.cpp:53-58) */
        const V3 fp = org + (xh * (u * -tanFov2 + tanFov) + yh * (v * -tanFov2 * aspect + tanFov * aspect) + zh) * (Real)c.focal_length;
        const V2 ap = c.aperture != LGPU_APERTURE_NONE ? ApertureSample(o, c, s) : V2(0, 0);
        const V3 ro = org + xh * ap.x + yh * ap.y;
        return Ray{ro, (fp - ro).Normalised()};
    }
    /* PinholeCamera::GenerateRay (Camera.cpp:41-44) */
    const V3 p = org + xh * (u * -tanFov2 + tanFov) + yh * (v * -tanFov2 * aspect + tanFov * aspect) + zh;
    return Ray{org, (p - org).Normalised()};
}

/* One path: pixel jitter (Render.cpp:55-56), Camera::GenerateRay, Li. */
static Spec TracePath(const OracleRun &R, uint64_t pathId, Real rgbOut[3], uint32_t *dimsOut) {
    const int W = R.opt->width, H = R.opt->height, spp = R.opt->spp;
    const uint32_t pixel = (uint32_t)(pathId / (uint64_t)spp);
    const uint32_t sIdx = (uint32_t)(pathId % (uint64_t)spp) + R.opt->sample_offset;
    const uint32_t x = pixel % (uint32_t)W, y = pixel / (uint32_t)W;
    Sampler s;
    s.key = lgpu_path_key(R.opt->seed, pixel, sIdx);
    s.dim = 0;
    if (g_ns == 4) SetWavelengths(s.key);
    const Real xi = (Real)1 / W, yi = (Real)1 / H;
    const Real u = xi * ((Real)x + s.Get1D() - (Real).5);
    const Real v = yi * ((Real)y + s.Get1D() - (Real).5);
    const Ray r = GenerateCameraRay(R.o, *R.cam, W, H, u, v, s);
    Integrator I(R.o->sc, R.opt->max_bounces, R.opt->min_bounces);
    Spec L;
    switch (R.opt->integrator) {
    case LGPU_INTEGRATOR_PATH: L = I.LiPath(r, s); break;
    case LGPU_INTEGRATOR_VOLPATH: L = I.LiVolPath(r, s); break;
    case LGPU_INTEGRATOR_DIRECT: L = I.LiDirect(r, s); break;
    case LGPU_INTEGRATOR_NORMAL: L = I.LiPass(r, true); break;
    case LGPU_INTEGRATOR_DEPTH: L = I.LiPass(r, false); break;
    default: L = I.Li(r, s); break;
    }
    if (dimsOut) *dimsOut = s.dim;
    if (g_ns == 3) { rgbOut[0] = L.c[0]; rgbOut[1] = L.c[1]; rgbOut[2] = L.c[2]; }
    else {
        Real xyz[3] = {0, 0, 0};
        for (int i = 0; i < 4; ++i) {
            const Real w = L.c[i] * (HERO_RANGE / (4.0f * LGPU_CIE_Y_INTEGRAL));
            xyz[0] += w * CieAt(lgpu_cie_x, t_lambda[i]);
            xyz[1] += w * CieAt(lgpu_cie_y, t_lambda[i]);
            xyz[2] += w * CieAt(lgpu_cie_z, t_lambda[i]);
        }
        XYZToRGB(xyz, rgbOut);
    }
    return L;
}

extern "C" {

LGPU_API void *oracle_create(const lgpu_scene_desc *d) {
    Oracle *o = new Oracle();
    if (!o->Load(d)) { delete o; return nullptr; }
    return o;
}
LGPU_API void oracle_destroy(void *o) { delete (Oracle *)o; }
/* Light-tree summary: total tree power, infinite-light power and number of tree lights. */
LGPU_API void oracle_tree_info(void *h, float *out) {
    Oracle *o = (Oracle *)h;
    out[0] = out[1] = out[2] = 0;
    if (auto *t = dynamic_cast<TreeSamplerO *>(o->sc.lightSampler.get())) {
        out[0] = t->treePower; out[1] = t->infPower; out[2] = (float)t->lights.size();
    }
}

/* Render paths [n ids or, when ids == NULL, every path of the frame].  film (optional) receives
 * summed RGB + count per pixel; path_out (optional) receives RGB + 0 per listed path. */
LGPU_API int oracle_render(void *handle, const lgpu_camera_desc *cam, const lgpu_render_opts *opt,
                           const uint64_t *ids, uint64_t n, float *film, float *path_out, int threads) {
    Oracle *o = (Oracle *)handle;
    if (cam->type == LGPU_CAMERA_THIN_LENS && cam->aperture == LGPU_APERTURE_MASKED &&
        (cam->aperture_mask < 0 || cam->aperture_mask >= (int)o->masks.size() || !o->masks[cam->aperture_mask]))
        return 1;   /* as the GPU library: a masked aperture needs a texture committed with aperture_mask */
    g_ns = (opt->spectral_mode == LGPU_SPECTRAL_HERO4) ? 4 : 3;
    for (auto &m : o->sc.media) m.Prepare();
    const uint64_t total = ids ? n : (uint64_t)opt->width * opt->height * opt->spp;
    OracleRun R{o, cam, opt};
    std::atomic<uint64_t> next(0);
    const uint64_t chunk = 256;
    std::vector<float> accum;
    auto worker = [&](std::vector<float> *acc) {
        for (;;) {
            const uint64_t b = next.fetch_add(chunk);
            if (b >= total) break;
            const uint64_t e = std::min(total, b + chunk);
            for (uint64_t i = b; i < e; ++i) {
                const uint64_t pid = ids ? ids[i] : i;
                Real rgb[3];
                uint32_t dims = 0;
                TracePath(R, pid, rgb, &dims);
                if (path_out) { path_out[4 * i] = rgb[0]; path_out[4 * i + 1] = rgb[1]; path_out[4 * i + 2] = rgb[2]; path_out[4 * i + 3] = (float)dims; }
                if (film) {
                    const uint64_t px = pid / (uint64_t)opt->spp;
                    float *f = &(*acc)[4 * px];
                    f[0] += rgb[0]; f[1] += rgb[1]; f[2] += rgb[2]; f[3] += 1;
                }
            }
        }
    };
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    const size_t npx = (size_t)opt->width * opt->height;
    std::vector<std::vector<float>> accs(film ? threads : 0, std::vector<float>());
    for (auto &a : accs) a.assign(4 * npx, 0.f);
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t) th.emplace_back(worker, film ? &accs[t] : nullptr);
    for (auto &t : th) t.join();
    if (film) for (auto &a : accs) for (size_t k = 0; k < 4 * npx; ++k) film[k] += a[k];
    return 0;
}

/* Closest hit for one world-space ray: out = {t, u, v} and ids = {objectId, primId}; returns hit. */
LGPU_API int oracle_intersect(void *handle, const float *ray, float *out, int32_t *ids) {
    Oracle *o = (Oracle *)handle;
    Ray r{V3(ray[0], ray[1], ray[2]), V3(ray[4], ray[5], ray[6])};
    RayHit h;
    if (!o->sc.Intersect(r, h)) { ids[0] = -1; ids[1] = -1; out[0] = INF; return 0; }
    out[0] = h.tFar;
    out[1] = h.normalG.x; out[2] = h.normalG.y; out[3] = h.normalG.z;
    ids[0] = h.object->index; ids[1] = (int32_t)h.primId;
    return 1;
}

/* ---- function-level known-answer entry points (pinned against the reference's own code) ---- */

/* FrDielectric(cosI, etaI, etaT) */
LGPU_API float oracle_fr_dielectric(float c, float ei, float et) { return FrDielectric(c, ei, et); }
/* Microfacet distribution D, Lambda, G for (dist, w, alpha) */
LGPU_API void oracle_microfacet(int dist, const float *wh, const float *wo, const float *wi, float ax, float ay, float *out) {
    const V3 h(wh[0], wh[1], wh[2]), o(wo[0], wo[1], wo[2]), i(wi[0], wi[1], wi[2]);
    out[0] = DistD(dist, h, V2(ax, ay));
    out[1] = DistLambda(dist, o, V2(ax, ay));
    out[2] = DistG(dist, o, i, V2(ax, ay));
    out[3] = DistPdf(dist, h, V2(ax, ay));
}
LGPU_API float oracle_to_alpha(float r) { return ToAlpha(r); }
/* texture bilinear fetch at (u, v): RGBA out (known-answer tests) */
LGPU_API void oracle_kat_texture_bilinear(const float *rgba, int w, int h, float u, float v, float *out) {
    Real o[4];
    TexBilinear(rgba, w, h, u, v, o);
    for (int k = 0; k < 4; ++k) out[k] = o[k];
}
/* Sampling::SampleCosineHemisphere (known-answer tests) */
LGPU_API void oracle_kat_cos_hemisphere(float u0, float u1, float *out) {
    const V3 w = SampleCosineHemisphere(V2(u0, u1));
    out[0] = w.x; out[1] = w.y; out[2] = w.z;
}
/* Same arguments as the reference-side driver's camera entry point: type 0 pinhole, 1 thin lens,
 * 2 spherical; aperture 0 none, 1 circular, 2 blade (known-answer tests) */
LGPU_API void oracle_kat_camera_ray(int type, const float *org, const float *xh, const float *yh, const float *zh, float fov,
                                    int W, int H, float focal, int aperture, float size, int blades, float offPhi,
                                    float offTheta, float u, float v, const float *ap_u, float *o, float *d) {
    lgpu_camera_desc c;
    std::memset(&c, 0, sizeof(c));
    for (int k = 0; k < 3; ++k) { c.origin[k] = org[k]; c.x_hat[k] = xh[k]; c.y_hat[k] = yh[k]; c.z_hat[k] = zh[k]; }
    c.fov = fov; c.type = type; c.focal_length = focal; c.aperture = aperture; c.aperture_size = size;
    c.blades = blades; c.offset_phi = offPhi; c.offset_theta = offTheta;
    Sampler s; s.replay = ap_u;
    const Ray r = GenerateCameraRay(nullptr, c, W, H, u, v, s);
    o[0] = r.o.x; o[1] = r.o.y; o[2] = r.o.z;
    d[0] = r.d.x; d[1] = r.d.y; d[2] = r.d.z;
}
/* Camera::GenerateRay at film coordinates (u, v) with the aperture's numbers replayed from ap_u
 * (known-answer tests; handle may be null unless the aperture is masked) */
LGPU_API void oracle_camera_ray(void *handle, const lgpu_camera_desc *cam, int W, int H, float u, float v,
                                const float *ap_u, float *o, float *d) {
    Sampler s; s.replay = ap_u;
    const Ray r = GenerateCameraRay((const Oracle *)handle, *cam, W, H, u, v, s);
    o[0] = r.o.x; o[1] = r.o.y; o[2] = r.o.z;
    d[0] = r.d.x; d[1] = r.d.y; d[2] = r.d.z;
}
LGPU_API float oracle_phase_hg(float c, float g) { return Medium::PhaseHG(c, g); }
/* HG Sample_p with explicit u: returns pdf, writes wi */
LGPU_API float oracle_hg_sample(float g, const float *wo, float u0, float u1, float *wi) {
    Medium m; m.g = g;
    struct FixedSampler : Sampler {};
    Sampler s;
    /* feed the two draws through a two-entry stream: emulate with a custom loop */
    const V3 w(wo[0], wo[1], wo[2]);
    Real cosT;
    if (std::abs(g) < 1e-3) cosT = 1 - 2 * u0;
    else { const Real sq = (1 - g * g) / (1 - g + 2 * g * u0); cosT = (1 + g * g - sq * sq) / (2 * g); }
    const Real sinT = std::sqrt(smax((Real)0, 1 - cosT * cosT));
    const Real phi = 2 * PI * u1;
    const V3 woNeg = -w;
    const V3 v1 = Cross(woNeg, V3(0, 1, 0));
    const V3 v2 = Cross(woNeg, v1);
    const V3 d = SphericalDirection(sinT, cosT, phi);
    const V3 r = v1 * d.x + woNeg * d.y + v2 * d.z;
    wi[0] = r.x; wi[1] = r.y; wi[2] = r.z;
    (void)s; (void)m;
    return Medium::PhaseHG(-cosT, g);
}
/* Oren-Nayar term for local wo, wi and sigma */
LGPU_API float oracle_oren_nayar(const float *wo, const float *wi, float sigma) {
    ScatterEvent ev; ev.woL = V3(wo[0], wo[1], wo[2]); ev.wiL = V3(wi[0], wi[1], wi[2]);
    return OrenNayarTerm(ev, sigma);
}
/* Blackbody RGB for a temperature (RGB mode, `samples` wavelengths) */
LGPU_API void oracle_blackbody_rgb(float T, int samples, float *rgb) {
    g_ns = 3;
    const Spec s = MakeBlackbody(T, (unsigned)samples);
    rgb[0] = s.c[0]; rgb[1] = s.c[1]; rgb[2] = s.c[2];
}
LGPU_API void oracle_blackbody_norm(const float *lam, int n, float T, float *out) { BlackbodyNormalized(lam, n, T, out); }
/* Smits upsampling at one wavelength */
LGPU_API float oracle_smits(const float *rgb, int illum, float lambda) { return SmitsUpsample(rgb, illum != 0, lambda); }
/* Noise nodes */
LGPU_API float oracle_perlin2d(float u, float v, float scale) { return Perlin2D(V2(u, v), scale); }
LGPU_API float oracle_value2d(float u, float v, float scale) { return Value2D(V2(u, v), scale); }
LGPU_API float oracle_voronoi2d(float u, float v, float scale) { return Voronoi2D(V2(u, v), scale); }
LGPU_API float oracle_checker2d(float u, float v, float scale) { return Checker2D(V2(u, v), scale); }
LGPU_API float oracle_voronoi3d(float x, float y, float z, float scale) { return Voronoi3D(V3(x, y, z), scale); }
/* ---- known-answer exports with the same signatures as oracle/ref_kat.cpp's (golden vectors) */
LGPU_API float oracle_kat_fr_dielectric(float c, float ei, float et) { return FrDielectric(c, ei, et); }
/* FresnelDielectric(etaT).Evaluate(cosI, etaArg) = FrDielectric(cosI, etaT, etaArg) (B12 kept) */
LGPU_API float oracle_kat_fresnel_dielectric_eval(float etaT, float cosI, float etaArg) { return FrDielectric(cosI, etaT, etaArg); }
LGPU_API float oracle_kat_hg_p(float g, const float *wo, const float *wi) {
    Medium m; m.g = g;
    return m.p(V3(wo[0], wo[1], wo[2]), V3(wi[0], wi[1], wi[2]));
}
LGPU_API float oracle_kat_hg_sample(float g, const float *wo, float u0, float u1, float *wi) {
    Medium m; m.g = g;
    const float u[2] = {u0, u1};
    Sampler s; s.replay = u;
    V3 w;
    const float pdf = m.Sample_p(V3(wo[0], wo[1], wo[2]), &w, s);
    wi[0] = w.x; wi[1] = w.y; wi[2] = w.z;
    return pdf;
}
LGPU_API void oracle_kat_medium(const float *sa, const float *ss, const float *ray6, float tFar, float u0, float u1,
                                const float *lp, float t_eq, float *out) {
    g_ns = 3;
    Medium m;
    for (int i = 0; i < 3; ++i) { m.sa[i] = sa[i]; m.ss[i] = ss[i]; }
    m.Prepare();
    Ray r; r.o = V3(ray6[0], ray6[1], ray6[2]); r.d = V3(ray6[3], ray6[4], ray6[5]);
    const Spec tr = m.Tr(tFar);
    out[0] = tr.c[0]; out[1] = tr.c[1]; out[2] = tr.c[2];
    const float u[2] = {u0, u1};
    Sampler s; s.replay = u;
    RayHit hit; hit.tFar = tFar;
    ScatterEvent ev; ev.hit = &hit;
    Real t = 0, pdf = 0;
    const Spec w = m.SampleDistance(s, ev, &t, &pdf);
    out[3] = t; out[4] = pdf; out[5] = w.c[0]; out[6] = w.c[1]; out[7] = w.c[2];
    out[8] = ev.mediumInteraction ? 1.f : 0.f;
    out[9] = m.PDFDistance(tFar);
    out[10] = m.PDFEquiangular(r, V3(lp[0], lp[1], lp[2]), tFar, t_eq);
}
LGPU_API void oracle_kat_rgb_from_sampled(const float *lam, const float *v, int n, float *rgb) { RGBFromSampled(lam, v, (unsigned)n, rgb); }
LGPU_API void oracle_kat_xyz_to_rgb(const float *xyz, float *rgb) { XYZToRGB(xyz, rgb); }
LGPU_API float oracle_kat_rgb_y(const float *rgb) {
    g_ns = 3;
    Spec s; s.c[0] = rgb[0]; s.c[1] = rgb[1]; s.c[2] = rgb[2];
    return s.y();
}
LGPU_API void oracle_kat_piecewise1d(const float *f, int n, float u, float *out) {
    const Piecewise1D d(f, (unsigned)n);
    Real pdf = 0; int off = 0;
    out[0] = d.SampleContinuous(u, &pdf, &off);
    out[1] = pdf; out[2] = (float)off;
    Real dp = 0;
    const unsigned i = d.SampleDiscrete(u, &dp);
    out[3] = (float)i; out[4] = dp; out[5] = (u - d.cdf[i]) / (d.cdf[i + 1] - d.cdf[i]);
    out[6] = d.PDF(i);
}
LGPU_API void oracle_kat_piecewise2d(const float *f, int nu, int nv, float u0, float u1, float *out) {
    const Piecewise2D d(f, (unsigned)nu, (unsigned)nv);
    Real pdf = 0;
    const V2 x = d.SampleContinuous(V2(u0, u1), &pdf);
    out[0] = x.x; out[1] = x.y; out[2] = pdf; out[3] = d.PDF(x);
}
/* Medium functions for a grey medium */
LGPU_API void oracle_medium(float sa, float ss, float t, float *out) {
    g_ns = 3;
    Medium m; m.sa[0] = m.sa[1] = m.sa[2] = sa; m.ss[0] = m.ss[1] = m.ss[2] = ss; m.Prepare();
    out[0] = m.Tr(t).c[0];
    out[1] = m.PDFDistance(t);
}
LGPU_API void oracle_cone_union(const float *a, const float *b, float *out) {
    Cone ca; ca.axis = V3(a[0], a[1], a[2]); ca.thetaO = a[3]; ca.thetaE = a[4];
    Cone cb; cb.axis = V3(b[0], b[1], b[2]); cb.thetaO = b[3]; cb.thetaE = b[4];
    const Cone r = ConeUnion(&ca, &cb);
    out[0] = r.axis.x; out[1] = r.axis.y; out[2] = r.axis.z; out[3] = r.thetaO; out[4] = r.thetaE;
}
LGPU_API float oracle_momega(float thetaO, float thetaE) { Cone c; c.thetaO = thetaO; c.thetaE = thetaE; return MOmega(c); }
LGPU_API uint32_t oracle_rng_bits(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t dim) {
    return lgpu_rng_bits(lgpu_path_key(seed, pixel, sample), dim);
}

}  // extern "C"
