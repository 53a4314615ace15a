"""Builds of the reference renderer's own code, used as the checker's anchor.  TEST INFRASTRUCTURE ONLY:
nothing here is linked into, loaded by or shipped with the product library, and every output stays
in oracle/_ref/ (git-ignored).

1. oracle/_ref/libref_kat.so -- golden-vector driver (oracle/ref_kat.cpp) linked with nine of the
   reference's translation units that compile unmodified, straight from the reference tree.

2. oracle/_ref/libref_li.so -- the reference's MIS volumetric path integrator with everything it
   calls (scene, meshes, instances, lights, light samplers, BSDFs, shader graph, media, spectra,
   cameras, tile renderer), driven by oracle/ref_li.cpp.  It is compiled from a PATCHED COPY of the
   reference sources in oracle/_ref/src, made by prepare() from the reference tree.  The copy is
   needed because the sources do not build as shipped:
     * g++ rejects the class-scope explicit specialisations of Socket::GetAs (ShaderGraph.h) and a
       string literal bound to `constexpr char *` (M1, M2); Texture.cpp calls std::powf (M3);
     * Embree 3 is absent: oracle/ref_shim/embree3/rtcore.h declares its API and
       oracle/ref_shim/rtcore_bvh.cpp implements the 18 calls the reference makes;
     * the x86 SSE/BMI2 intrinsics of vec3.h, Colour.h and Texture.h are supplied by portable
       element-wise versions (oracle/ref_shim/portable/), so x86 and Arm hosts compute the same
       IEEE single-precision results;
     * stb_image is compiled without its SIMD paths (STBI_NO_SIMD) for the same reason.
   Every edit is listed in EDITS with its reason.  Ids M* are mechanical (build only), S1 adds an
   accessor the counter-based sampler needs, S2 the read-only accessors of the GPU module's
   Lambda-side binding, and B* patch the reference defects on the hot path; the CPU oracle and the
   GPU module apply the same patches, so the three compute the same thing.

3. oracle/_ref/libref_binding.so -- the same units plus the GPU module's Lambda-side binding
   (lambda_gb300/binding), which only compiles against Lambda's headers, linked with the module:
   the tests drive the binding on lambda::Scene objects built by ref_li.cpp.

The copy is made on a host that has the reference tree; where the tree is absent (a GPU host) a copy
made earlier is compiled if present.

    python oracle/build_ref.py <reference_root>        (or LAMBDA_REFERENCE_ROOT=<reference_root>)
"""
import concurrent.futures as cf
import hashlib
import os
import pathlib
import re
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libref_kat.so"
LIB_LI = OUT / "libref_li.so"
COPY = OUT / "src"
SHIM = HERE / "ref_shim"


def reference_root(arg=None):
    """The reference tree: an explicit argument, else $LAMBDA_REFERENCE_ROOT; None when unset."""
    root = arg or os.environ.get("LAMBDA_REFERENCE_ROOT")
    return pathlib.Path(root) if root else None


# ---------------------------------------------------------------------------------------------
# 1. golden-vector library of unmodified units
UNITS = ["shading/Fresnel.cpp", "shading/media/HenyeyGreenstein.cpp", "shading/media/HomogeneousMedium.cpp",
         "core/Spectrum.cpp", "core/SPD_Data.cpp", "sampling/Piecewise.cpp", "camera/Camera.cpp", "camera/Aperture.cpp",
         "image/TextureEncoding.cpp"]
# camera/Aperture.cpp instantiates the reference's texture class, whose Morton-order addressing calls the
# x86 BMI2 intrinsic _pdep_u64 (image/Texture.h:46): that unit needs -mbmi2 (this x86 build only).
UNIT_FLAGS = {"camera/Aperture.cpp": ["-mbmi2"]}


def _has_bmi2():
    try:
        return "bmi2" in pathlib.Path("/proc/cpuinfo").read_text().split()
    except OSError:
        return False


def build(ref_root=None, force=False):
    """Golden-vector library.  Returns its path, or None where it cannot be built here (no reference
    tree, or a host without the BMI2 instructions the reference's texture class needs)."""
    root = reference_root(ref_root)
    if root is None or not (root / "src").is_dir() or not _has_bmi2():
        return LIB if LIB.exists() and _has_bmi2() and not force else None   # built earlier on this host
    src = root / "src"
    if LIB.exists() and not force and LIB.stat().st_mtime >= (HERE / "ref_kat.cpp").stat().st_mtime:
        return LIB
    OUT.mkdir(exist_ok=True)
    flags = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden", "-include", "cstring",
             "-I", str(src), "-I", str(src.parent), "-I", str(SHIM), "-w"]
    objs = []
    for u in UNITS:
        obj = OUT / (u.replace("/", "_") + ".o")
        subprocess.run(flags + UNIT_FLAGS.get(u, []) + ["-c", str(src / u), "-o", str(obj)], check=True)
        objs.append(str(obj))
    drv = OUT / "ref_kat.o"
    subprocess.run(flags + ["-mbmi2", "-c", str(HERE / "ref_kat.cpp"), "-o", str(drv)], check=True)   # drives texture_t too
    subprocess.run(["g++", "-shared", "-o", str(LIB), str(drv), *objs, "-Wl,--no-undefined"], check=True)
    return LIB


# ---------------------------------------------------------------------------------------------
# 2. the patched copy and the integrator library

def _shader_graph_m1(text):
    """M1: move the explicit specialisations of Socket::GetAs<T> (ShaderGraph.h:82-230) and the
    GetAsSpectrum that calls them (:232-251) out of struct Socket to namespace scope; the primary
    template (a static_assert(false) body) becomes a declaration.  Code unchanged otherwise."""
    text, n = re.subn(r'template<class T> inline T GetAs\(const ScatterEvent &_event\) \{\s*'
                      r'static_assert\(false, "GetAs\(\): Invalid template - not specialised."\);\s*\}',
                      'template<class T> T GetAs(const ScatterEvent &_event);', text)
    assert n == 1, "M1: primary GetAs template not found"
    start = text.index("template<> inline Real GetAs<Real>")
    gs = text.index("inline Spectrum GetAsSpectrum(const ScatterEvent &_event, const SpectrumType _type")
    gs_end = text.index("};", text.index("default:\n\t\t\treturn Spectrum(0);", gs))
    specs, body = text[start:gs], text[gs:gs_end]
    decl = "inline Spectrum GetAsSpectrum(const ScatterEvent &_event, const SpectrumType _type = SpectrumType::Reflectance);\n"
    text = text[:start] + decl + text[gs_end:]
    specs, n = re.subn(r"template<> inline ([A-Za-z0-9_]+\s*\**\s*)GetAs<", r"template<> inline \1Socket::GetAs<", specs)
    assert n == 5, "M1: expected five GetAs specialisations, found %d" % n
    body = body.replace("inline Spectrum GetAsSpectrum(const ScatterEvent &_event, const SpectrumType _type = SpectrumType::Reflectance)",
                        "inline Spectrum Socket::GetAsSpectrum(const ScatterEvent &_event, const SpectrumType _type)", 1)
    after = text.index("};", text.index(decl)) + 2
    return text[:after] + "\n\n" + specs + "\n" + body + "\n" + text[after:]


# (unit, id, reason, old, new[, count]); `old` must occur exactly `count` times (default once)
EDITS = [
    ("shading/graph/ShaderGraph.h", "M2", "string literal bound to constexpr char * (ill-formed in C++11 and later)",
     'template<class T> constexpr char *getSocketTag = "Null";',
     'template<class T> constexpr char const *getSocketTag = "Null";'),
    ("image/Texture.cpp", "M3", "std::powf is not declared by libstdc++",
     "std::powf", "std::pow", 3),
    ("sampling/SampleShifter.h", "S1", "accessor for the pixel index set by TileRenderers (counter-based sampler key)",
     "\t\tReal Shift(const Real _point, const unsigned _dimensionIndex) const;",
     "\t\tReal Shift(const Real _point, const unsigned _dimensionIndex) const;\n\n"
     "\t\tinline unsigned GetPixelIndex() const { return pixelIndex; }"),
    # S2: read-only accessors the GPU module's Lambda-side binding (lambda_gb300/binding) needs, the
    # getters a maintainer adds with it: the camera frame, an instance's proxy and mesh, and the
    # environment light's texture are not public
    ("shading/graph/ShaderGraph.h", "B36", "output sockets lose their owning node: Node() links them, then every node "
     "constructor overwrites them with MAKE_SOCKET, whose initialiser sets node = nullptr (GraphIterator, "
     "ShaderGraph.cpp:130, then follows null); the binding reads the owner of a linked socket",
     "MAKE_SOCKET_CALLBACK(_callback), nullptr, (_type)", "MAKE_SOCKET_CALLBACK(_callback), this, (_type)"),
    ("shading/graph/GraphBxDF.h", "B36", "the same for the BxDF nodes' MAKE_BXDF_SOCKET",
     "NodeDelegate::FromFunction<_DECLTYPE, _callback>(this), nullptr, (_type)",
     "NodeDelegate::FromFunction<_DECLTYPE, _callback>(this), this, (_type)"),
    ("camera/Camera.h", "S2", "binding: the camera frame and tan(fov / 2)",
     "\t\tvoid SetFov(const Real _fov);",
     "\t\tvoid SetFov(const Real _fov);\n\n"
     "\t\tinline void GetFrame(Vec3 *_x, Vec3 *_y, Vec3 *_z, Real *_tanFov) const { *_x = xHat; *_y = yHat; *_z = zHat; *_tanFov = tanFov; }"),
    ("core/Instance.h", "S2", "binding: the object an instance proxy wraps",
     "\t\tvoid Commit(const RTCDevice &_device);\n",
     "\t\tvoid Commit(const RTCDevice &_device);\n\n\t\tinline Object *GetObject() const { return iObject; }\n"),
    ("core/Instance.h", "S2", "binding: the proxy an instance places",
     "\t\tvoid Commit(const RTCDevice &_device) override;",
     "\t\tvoid Commit(const RTCDevice &_device) override;\n\n\t\tinline InstanceProxy *GetProxy() const { return proxy; }"),
    ("shading/TextureAdapter.h", "S2", "binding: the RGB texture behind an adapter (null for other kinds)",
     "\t\tinline void operator=(TextureR32 *_rhs) { SetTexture(_rhs); }",
     "\t\tinline void operator=(TextureR32 *_rhs) { SetTexture(_rhs); }\n\n"
     "\t\tinline const Texture *GetRGBTexture() const { return textureType == TextureType::RGB ? reinterpret_cast<const Texture *>(texture) : nullptr; }"),
    ("lighting/EnvironmentLight.h", "S2", "binding: the radiance map of an environment light",
     "\t\tEnvironmentLight(Texture *_texture, const Real _intesity = 1);",
     "\t\tEnvironmentLight(Texture *_texture, const Real _intesity = 1);\n\n"
     "\t\tinline const TextureAdapter &GetRadianceMap() const { return radianceMap; }"),
    ("shading/media/HomogeneousMedium.cpp", "B2", "SampleEquiangular reads the uninitialised `t`",
     "const Real t = std::min(t, _event.hit->tFar);", "const Real t = std::min(dist, _event.hit->tFar);"),
    ("shading/media/HomogeneousMedium.cpp", "B3", "integer division makes PDFDistance zero",
     "pdf *= 1 / Spectrum::nSamples;", "pdf *= 1.f / Spectrum::nSamples;"),
    ("shading/media/HomogeneousMedium.cpp", "B4", "equiangular sample measured from the hit point, its pdf from the ray origin",
     "const Vec3 delta = _lightPoint - _event.hit->point;", "const Vec3 delta = _lightPoint - _ray.o;"),
    ("integrators/MISVolumetricPathIntegrator.cpp", "B5", "light-sample pdf multiplied while uninitialised",
     "\t\t\t\tPartialLightSample lSample;\n",
     "\t\t\t\tPartialLightSample lSample;\n\t\t\t\tlSample.pdf = 1;\n"
     "\t\t\t\tconst Vec3 sampPoint = hit.point, sampNormal = hit.normalS;\n"),
    ("integrators/MISVolumetricPathIntegrator.cpp", "B7", "medium vertex: pass the point the light was sampled for",
     "LdMediumPoint(event, mediumPoint[DISTANCE], &lSample, &wi[DISTANCE], &phasePDF);",
     "LdMediumPoint(event, mediumPoint[DISTANCE], &lSample, &wi[DISTANCE], &phasePDF, sampPoint, sampNormal);"),
    ("integrators/MISVolumetricPathIntegrator.cpp", "B7", "medium vertex: pass the point the light was sampled for",
     "LdMediumPoint(event, mediumPoint[EQUIANGULAR], &lSample, &wi[EQUIANGULAR], &phasePDF);",
     "LdMediumPoint(event, mediumPoint[EQUIANGULAR], &lSample, &wi[EQUIANGULAR], &phasePDF, sampPoint, sampNormal);"),
    ("integrators/MISVolumetricPathIntegrator.cpp", "B7", "medium vertex: pass the point the light was sampled for",
     "Spectrum MISVolumetricPathIntegrator::LdMediumPoint(ScatterEvent &_event, const Vec3 &_p, PartialLightSample *_ls, Vec3 *_wi, Real *_f) const {",
     "Spectrum MISVolumetricPathIntegrator::LdMediumPoint(ScatterEvent &_event, const Vec3 &_p, PartialLightSample *_ls, Vec3 *_wi, Real *_f, const Vec3 &_sampPoint, const Vec3 &_sampNormal) const {"),
    ("integrators/MISVolumetricPathIntegrator.h", "B7", "medium vertex: pass the point the light was sampled for",
     "Spectrum LdMediumPoint(ScatterEvent &_event, const Vec3 &_p, PartialLightSample *_ls, Vec3 *_wi, Real *_f) const;",
     "Spectrum LdMediumPoint(ScatterEvent &_event, const Vec3 &_p, PartialLightSample *_ls, Vec3 *_wi, Real *_f, const Vec3 &_sampPoint, const Vec3 &_sampNormal) const;"),
    ("integrators/MISVolumetricPathIntegrator.cpp", "B7", "light-tree pdf evaluated at the next hit instead of the shading point",
     "\t\t\t\tpartialLightPDF = scene.lightSampler->Pdf(_event, nl); //Recalculate light distribution pdf if don't already know it",
     "\t\t\t\tconst Vec3 hp = hit.point, hn = hit.normalS;\n\t\t\t\thit.point = _sampPoint; hit.normalS = _sampNormal;\n"
     "\t\t\t\tpartialLightPDF = scene.lightSampler->Pdf(_event, nl);\n\t\t\t\thit.point = hp; hit.normalS = hn;"),
    ("integrators/MISVolumetricPathIntegrator.cpp", "B7", "light-tree pdf evaluated at the next hit instead of the shading point",
     "\t\t\t\t\tReal lightDistPdf = 1;\n",
     "\t\t\t\t\tReal lightDistPdf = 1;\n\t\t\t\t\tconst Vec3 sampPoint = hit.point, sampNormal = hit.normalS;\n"),
    ("integrators/MISVolumetricPathIntegrator.cpp", "B7", "light-tree pdf evaluated at the next hit instead of the shading point",
     "if (nl != l) lightDistPdf = _scene.lightSampler->Pdf(event, nl); //Recalculate light distribution pdf if we don't already know it",
     "if (nl != l) { const Vec3 hp = hit.point, hn = hit.normalS; hit.point = sampPoint; hit.normalS = sampNormal;"
     " lightDistPdf = _scene.lightSampler->Pdf(event, nl); hit.point = hp; hit.normalS = hn; }"),
    ("integrators/MISVolumetricPathIntegrator.cpp", "B32", "escape at bounce 0 dereferences a null environment light",
     "if (bounces == 0) L += ((Light*)_scene.envLight)->Le(r) * beta;",
     "if (bounces == 0 && _scene.envLight) L += ((Light*)_scene.envLight)->Le(r) * beta;"),
    ("integrators/PathIntegrator.cpp", "B7", "light-tree pdf evaluated at the next hit instead of the shading point",
     "Real lightDistPdf = 1;", "Real lightDistPdf = 1; const Vec3 sampPoint = hit.point, sampNormal = hit.normalS;"),
    ("integrators/PathIntegrator.cpp", "B7", "light-tree pdf evaluated at the next hit instead of the shading point",
     "if (nl != l) lightDistPdf = _scene.lightSampler->Pdf(event, nl);",
     "if (nl != l) { const Vec3 hp = hit.point, hn = hit.normalS; hit.point = sampPoint; hit.normalS = sampNormal;"
     " lightDistPdf = _scene.lightSampler->Pdf(event, nl); hit.point = hp; hit.normalS = hn; }"),
    ("integrators/VolumetricPathIntegrator.cpp", "B7", "light-tree pdf evaluated at the next hit instead of the shading point",
     "Real lightDistPdf = 1;", "Real lightDistPdf = 1; const Vec3 sampPoint = hit.point, sampNormal = hit.normalS;", 2),
    ("integrators/VolumetricPathIntegrator.cpp", "B7", "light-tree pdf evaluated at the next hit instead of the shading point",
     "if (nl != l) lightDistPdf = _scene.lightSampler->Pdf(event, nl);",
     "if (nl != l) { const Vec3 hp = hit.point, hn = hit.normalS; hit.point = sampPoint; hit.normalS = sampNormal;"
     " lightDistPdf = _scene.lightSampler->Pdf(event, nl); hit.point = hp; hit.normalS = hn; }", 2),
    ("integrators/VolumetricPathIntegrator.cpp", "B32", "escape at bounce 0 dereferences a null environment light",
     "if (bounces == 0) L += ((Light*)_scene.envLight)->Le(r) * beta;",
     "if (bounces == 0 && _scene.envLight) L += ((Light*)_scene.envLight)->Le(r) * beta;"),
    ("lighting/ManyLightSampler.cpp", "B8", "RecursivePDF: right-child probability 1 - IR instead of 1 - pdfs[0]",
     "pdfs[1] = 1 - IR;", "pdfs[1] = 1 - pdfs[0];"),
    ("lighting/ManyLightSampler.h", "B11", "infinite light and powers uninitialised when there is no environment light",
     "\t\tLight *infiniteLight;\n\t\tReal treePower, infPower;",
     "\t\tLight *infiniteLight = nullptr;\n\t\tReal treePower = 0, infPower = 0;"),
    ("lighting/ManyLightSampler.cpp", "B33", "triangle lights enter the tree in unordered_map order (pointer hashes: "
     "differs from run to run); use mesh-light order, then triangle index",
     "\tfor (auto &it : triangleLights) lights.push_back(&it.second);",
     "\tfor (Light *l0 : _lights) {\n\t\tMeshLight *ml = dynamic_cast<MeshLight *>(l0);\n\t\tif (!ml) continue;\n"
     "\t\tfor (size_t i = 0; i < ml->GetMesh().numTriangles; ++i) lights.push_back(&triangleLights.at({ ml, (unsigned)i }));\n\t}"),
    ("lighting/MeshLight.cpp", "B10", "TriangleLight::Sample_Li multiplies by cos * area instead of dividing",
     "_pdf = maths::DistSq(_event.hit->point, pL) * (cosTheta * triArea);",
     "_pdf = maths::DistSq(_event.hit->point, pL) / (cosTheta * triArea);"),
    ("lighting/MeshLight.cpp", "B35", "emitter sampling reads the texture coordinates of a mesh that has none "
     "(null dereference); the hit uv is set only when the mesh has them",
     "\t_event.hit->uvCoords = maths::BarycentricInterpolation(\n\t\tmesh->textureCoordinates[t.v0],",
     "\tif (mesh->textureCoordinates) _event.hit->uvCoords = maths::BarycentricInterpolation(\n\t\tmesh->textureCoordinates[t.v0],"),
    ("lighting/MeshLight.cpp", "B35", "emitter sampling reads the texture coordinates of a mesh that has none "
     "(null dereference); the hit uv is set only when the mesh has them",
     "\t_event.hit->uvCoords = maths::BarycentricInterpolation(\n\t\tmesh.textureCoordinates[t.v0],",
     "\tif (mesh.textureCoordinates) _event.hit->uvCoords = maths::BarycentricInterpolation(\n\t\tmesh.textureCoordinates[t.v0],"),
    ("lighting/MeshLight.cpp", "B35", "TriangleLight::Irradiance reads the texture coordinates of a mesh that has none",
     "\t\t\tfakeHit.uvCoords = maths::BarycentricInterpolation(uv0, uv1, uv2, (Real)a * invSamples, (Real)b * invSamples);",
     "\t\t\tif (meshLight->mesh->textureCoordinates) fakeHit.uvCoords = maths::BarycentricInterpolation(uv0, uv1, uv2, (Real)a * invSamples, (Real)b * invSamples);"),
    ("lighting/MeshLight.cpp", "B35", "TriangleLight::Irradiance binds references into a null texture-coordinate array",
     "\tconst Vec2 &uv0 = meshLight->mesh->textureCoordinates[meshLight->mesh->triangles[triIndex].v0];\n"
     "\tconst Vec2 &uv1 = meshLight->mesh->textureCoordinates[meshLight->mesh->triangles[triIndex].v1];\n"
     "\tconst Vec2 &uv2 = meshLight->mesh->textureCoordinates[meshLight->mesh->triangles[triIndex].v2];",
     "\tconst Vec2 *uvs = meshLight->mesh->textureCoordinates;\n"
     "\tconst Vec2 uv0 = uvs ? uvs[meshLight->mesh->triangles[triIndex].v0] : Vec2(0, 0);\n"
     "\tconst Vec2 uv1 = uvs ? uvs[meshLight->mesh->triangles[triIndex].v1] : Vec2(0, 0);\n"
     "\tconst Vec2 uv2 = uvs ? uvs[meshLight->mesh->triangles[triIndex].v2] : Vec2(0, 0);"),
    ("shading/graph/GraphConverters.cpp", "B14", "SeparateXYZ::GetY reads a second input the node does not have",
     "inputSockets[1].socket->GetAs<Vec3>(_event).y", "inputSockets[0].socket->GetAs<Vec3>(_event).y"),
    ("shading/graph/GraphConverters.cpp", "B14", "SeparateXYZ::GetZ reads a third input the node does not have",
     "inputSockets[2].socket->GetAs<Vec3>(_event).z", "inputSockets[0].socket->GetAs<Vec3>(_event).z"),
    ("shading/graph/GraphMaths.cpp", "B15", "SQRT and POWER leave the output unwritten",
     "\t\tcase ScalarOperatorType::DIVIDE:\n"
     "\t\t\t*reinterpret_cast<Real *>(_out) = inputSockets[0].socket->GetAs<Real>(_event) / inputSockets[1].socket->GetAs<Real>(_event);\n"
     "\t\t\tbreak;\n",
     "\t\tcase ScalarOperatorType::DIVIDE:\n"
     "\t\t\t*reinterpret_cast<Real *>(_out) = inputSockets[0].socket->GetAs<Real>(_event) / inputSockets[1].socket->GetAs<Real>(_event);\n"
     "\t\t\tbreak;\n"
     "\t\tcase ScalarOperatorType::SQRT:\n"
     "\t\t\t*reinterpret_cast<Real *>(_out) = std::sqrt(inputSockets[0].socket->GetAs<Real>(_event));\n"
     "\t\t\tbreak;\n"
     "\t\tcase ScalarOperatorType::POWER:\n"
     "\t\t\t*reinterpret_cast<Real *>(_out) = std::pow(inputSockets[0].socket->GetAs<Real>(_event), inputSockets[1].socket->GetAs<Real>(_event));\n"
     "\t\t\tbreak;\n"),
    ("core/Scene.cpp", "B26", "an instance hit is processed by objects[geomID] (the id inside the instanced scene)",
     "objects[rayHit.hit.geomID]->Hit(rayHit, _hit);",
     "objects[rayHit.hit.instID[0] != RTC_INVALID_GEOMETRY_ID ? rayHit.hit.instID[0] : rayHit.hit.geomID]->Hit(rayHit, _hit);"),
    ("core/Scene.cpp", "B31", "the constructor leaves envLight and lightSampler uninitialised (read by Commit)",
     "\thasVolumes = false;\n", "\thasVolumes = false;\n\tenvLight = nullptr;\n\tlightSampler = nullptr;\n"),
    ("core/Transformable.h", "B34", "the parent pointer is uninitialised and GetAffine (Instance::Commit) reads it",
     "\t\tTransformable *parent;", "\t\tTransformable *parent = nullptr;"),
    ("core/Instance.cpp", "B18", "the geometric normal of an instance hit stays in object space",
     "\tif (!xfm.IsIdentity()) {\n\t\tTransformNormal(&_hit.normalS);",
     "\tif (!xfm.IsIdentity()) {\n"
     "\t\t{\t/* Ng by the inverse transpose of the linear part (inverse in double precision) */\n"
     "\t\t\tconst double a = xfm[0], b = xfm[3], c = xfm[6], d = xfm[1], e = xfm[4], f = xfm[7], g = xfm[2], h = xfm[5], i = xfm[8];\n"
     "\t\t\tconst double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;\n"
     "\t\t\tconst double id = 1.0 / (a * A + b * B + c * C);\n"
     "\t\t\tconst float n[9] = {(float)(A * id), (float)(-(b * i - c * h) * id), (float)((b * f - c * e) * id),\n"
     "\t\t\t\t(float)(B * id), (float)((a * i - c * g) * id), (float)(-(a * f - c * d) * id),\n"
     "\t\t\t\t(float)(C * id), (float)(-(a * h - b * g) * id), (float)((a * e - b * d) * id)};\n"
     "\t\t\tconst Vec3 ng(_rtcHit.hit.Ng_x, _rtcHit.hit.Ng_y, _rtcHit.hit.Ng_z);\n"
     "\t\t\t_hit.normalG = (Vec3(n[0], n[1], n[2]) * ng.x + Vec3(n[3], n[4], n[5]) * ng.y + Vec3(n[6], n[7], n[8]) * ng.z).Normalised();\n"
     "\t\t}\n"
     "\t\tTransformNormal(&_hit.normalS);"),
]

# Units of the integrator library (src/ relative); assets, the C API, the denoiser, post-processing
# and the TBB/OpenMP mosaic renderers are not on the path.
LI_UNITS = ["core/Scene.cpp", "core/TriangleMesh.cpp", "core/Instance.cpp", "core/Spectrum.cpp", "core/SPD_Data.cpp",
            "camera/Camera.cpp", "camera/Aperture.cpp", "camera/Film.cpp", "image/Texture.cpp", "image/TextureEncoding.cpp",
            "integrators/Integrator.cpp", "integrators/MISVolumetricPathIntegrator.cpp", "integrators/PathIntegrator.cpp",
            "integrators/VolumetricPathIntegrator.cpp", "integrators/DirectLightingIntegrator.cpp",
            "lighting/Light.cpp", "lighting/LightSampler.cpp", "lighting/ManyLightSampler.cpp", "lighting/MeshLight.cpp",
            "lighting/PointLight.cpp", "lighting/Spotlight.cpp", "lighting/EnvironmentLight.cpp", "render/Render.cpp",
            "sampling/Piecewise.cpp", "sampling/SampleShifter.cpp", "sampling/HaltonSampler.cpp",
            "shading/Fresnel.cpp", "shading/Material.cpp", "shading/MicrofacetDistribution.cpp",
            "shading/graph/ShaderGraph.cpp", "shading/graph/GraphBxDF.cpp", "shading/graph/GraphConverters.cpp",
            "shading/graph/GraphInputs.cpp", "shading/graph/GraphMaths.cpp", "shading/graph/GraphTexture.cpp",
            "shading/media/HenyeyGreenstein.cpp", "shading/media/HomogeneousMedium.cpp",
            "shading/surface/BxDF.cpp", "shading/surface/Ghost.cpp", "shading/surface/Microfacet.cpp",
            "shading/surface/OrenNayar.cpp", "shading/surface/Specular.cpp", "utility/Memory.cpp", "utility/Concurrency.cpp"]
COPY_DIRS = ["Lambda.h", "camera", "core", "image", "integrators", "lighting", "maths", "render", "sampling", "shading",
             "utility"]


def _recipe_hash():
    h = hashlib.sha256()
    h.update(pathlib.Path(__file__).read_bytes())
    return h.hexdigest()[:16]


def prepare(ref_root=None, force=False):
    """Copy the reference sources into oracle/_ref/src and apply EDITS.  Returns the copy, or None
    when neither a reference tree nor an earlier copy is available."""
    stamp = COPY / ".recipe"
    if COPY.is_dir() and stamp.exists() and stamp.read_text() == _recipe_hash() and not force:
        return COPY
    root = reference_root(ref_root)
    if root is None or not (root / "src").is_dir():
        return COPY if COPY.is_dir() and stamp.exists() else None
    if COPY.exists():
        shutil.rmtree(COPY)
    COPY.mkdir(parents=True)
    for d in COPY_DIRS:
        s = root / "src" / d
        if s.is_dir():
            shutil.copytree(s, COPY / d)
        else:
            shutil.copy2(s, COPY / d)
    shutil.copytree(root / "third_party" / "stb_image", COPY / "stb_image")
    sg = COPY / "shading" / "graph" / "ShaderGraph.h"
    sg.write_text(_shader_graph_m1(sg.read_text(encoding="latin-1")), encoding="latin-1")
    log = ["M1 shading/graph/ShaderGraph.h: Socket::GetAs specialisations and GetAsSpectrum moved to namespace scope"]
    for edit in EDITS:
        unit, tag, why, old, new = edit[:5]
        want = edit[5] if len(edit) > 5 else 1
        p = COPY / unit
        t = p.read_text(encoding="latin-1")
        n = t.count(old)
        if n != want:
            raise RuntimeError("edit %s in %s: expected %d match(es), found %d" % (tag, unit, want, n))
        p.write_text(t.replace(old, new), encoding="latin-1")
        log.append("%s %s: %s" % (tag, unit, why))
    (COPY / "EDITS.txt").write_text("\n".join(log) + "\n")
    stamp.write_text(_recipe_hash())
    return COPY


def _li_flags(opt="-O3"):
    return ["g++", "-std=c++17", opt, "-fPIC", "-ffp-contract=off", "-fpermissive", "-w", "-include", "cstring",
            "-DSTBI_NO_SIMD", "-I", str(SHIM / "portable"), "-I", str(SHIM), "-I", str(COPY)]


def build_li(ref_root=None, force=False):
    """Integrator library from the patched copy.  Returns its path, or None when no copy exists."""
    if prepare(ref_root) is None:
        return None
    deps = [HERE / "ref_li.cpp", SHIM / "rtcore_bvh.cpp", SHIM / "embree3" / "rtcore.h", COPY / ".recipe",
            HERE.parent / "include" / "lambda_gpu.h", HERE.parent / "lambda_gb300" / "csrc" / "lgpu_rng.h"]
    deps += list((SHIM / "portable").glob("*.h"))
    if LIB_LI.exists() and not force and all(LIB_LI.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB_LI
    obj_dir = OUT / "li_obj"
    obj_dir.mkdir(parents=True, exist_ok=True)
    jobs = [(COPY / u, obj_dir / (u.replace("/", "_") + ".o")) for u in LI_UNITS]
    jobs += [(SHIM / "rtcore_bvh.cpp", obj_dir / "rtcore_bvh.o"), (HERE / "ref_li.cpp", obj_dir / "ref_li.o")]

    def one(job):
        src, obj = job
        if obj.exists() and not force and obj.stat().st_mtime >= max(src.stat().st_mtime, (COPY / ".recipe").stat().st_mtime):
            return
        r = subprocess.run(_li_flags() + ["-c", str(src), "-o", str(obj)], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("reference build failed on %s:\n%s" % (src, r.stderr[-4000:]))

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(one, jobs))
    tmp = LIB_LI.with_suffix(".so.tmp%d" % os.getpid())
    subprocess.run(["g++", "-shared", "-o", str(tmp), *[str(o) for _, o in jobs], "-lpthread", "-Wl,--no-undefined"],
                   check=True)
    os.replace(tmp, LIB_LI)
    return LIB_LI


LIB_BINDING = OUT / "libref_binding.so"
BINDING = HERE.parent / "lambda_gb300" / "binding"
GPU_LIB_DIR = HERE.parent / "lambda_gb300" / "_build"


def build_binding(ref_root=None, force=False):
    """The GPU module's Lambda-side binding (lambda_gb300/binding/lambda_gpu_binding.cpp) compiled
    against the patched copy and linked with the integrator library's units, ref_li.cpp built with
    REF_WITH_BINDING, and the module (lambda_gb300/_build/liblambda_gpu.so, found through the
    library's run path).  Returns its path, or None when no copy or no module library exists."""
    if build_li(ref_root) is None or not (GPU_LIB_DIR / "liblambda_gpu.so").exists():
        return None
    obj_dir = OUT / "li_obj"
    srcs = [(HERE / "ref_li.cpp", obj_dir / "ref_li_binding.o", ["-DREF_WITH_BINDING"]),
            (BINDING / "lambda_gpu_binding.cpp", obj_dir / "lambda_gpu_binding.o", [])]
    deps = [BINDING / "lambda_gpu_binding.h", BINDING / "lambda_gpu_binding.cpp", HERE / "ref_li.cpp", LIB_LI,
            GPU_LIB_DIR / "liblambda_gpu.so"]
    if LIB_BINDING.exists() and not force and all(LIB_BINDING.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB_BINDING

    def one(job):
        src, obj, extra = job
        r = subprocess.run(_li_flags() + extra + ["-c", str(src), "-o", str(obj)], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("binding build failed on %s:\n%s" % (src, r.stderr[-4000:]))

    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        list(ex.map(one, srcs))
    objs = [obj_dir / (u.replace("/", "_") + ".o") for u in LI_UNITS] + [obj_dir / "rtcore_bvh.o"]
    objs += [o for _, o, _ in srcs]
    tmp = LIB_BINDING.with_suffix(".so.tmp%d" % os.getpid())
    rpath = os.path.relpath(GPU_LIB_DIR, OUT)
    subprocess.run(["g++", "-shared", "-o", str(tmp), *[str(o) for o in objs], "-L" + str(GPU_LIB_DIR), "-llambda_gpu",
                    "-Wl,-rpath,$ORIGIN/" + rpath, "-lpthread", "-Wl,--no-undefined"], check=True)
    os.replace(tmp, LIB_BINDING)
    return LIB_BINDING


if __name__ == "__main__":
    arg = sys.argv[1] if len(sys.argv) > 1 else None
    print(build(arg, force=True))
    print(prepare(arg, force=True))
    print(build_li(arg, force=True))
