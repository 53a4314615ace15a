/*
 * ref_li.cpp -- driver of the REFERENCE renderer's own integrator.  TEST INFRASTRUCTURE ONLY.
 *
 * Linked with the patched copy of the reference sources (oracle/build_ref.py, oracle/_ref/src) into
 * oracle/_ref/libref_li.so.  It builds a lambda::Scene from the same flat scene description the GPU
 * module takes (include/lambda_gpu.h) through the reference's own classes -- TriangleMesh,
 * InstanceProxy/Instance, Material, shader-graph nodes, MeshLight/PointLight/Spotlight/
 * EnvironmentLight, ManyLightSampler/PowerLightSampler, HomogeneousMedium + HenyeyGreenstein, the
 * cameras -- and runs lambda::MISVolumetricPathIntegrator::Li (and the other integrators the C API
 * selects) with a counter-based Sampler keyed exactly like the GPU module and the CPU oracle
 * (lgpu_rng.h), so the three are compared path by path on the same random numbers.
 *
 * Entry points (C ABI, ctypes-loaded by oracle/reference.py):
 *   ref_create / ref_destroy / ref_last_error    scene from a descriptor
 *   ref_render      per-path radiance for chosen path ids (pixel jitter, Camera::GenerateRay and
 *                   Integrator::Li as TileRenderers::UniformSpp does per sample), or a whole film
 *                   through the reference's RenderMosaic + TileRenderers::UniformSpp on a pool of
 *                   std::threads (the TBB/OpenMP mosaic renderers are not built)
 *   ref_render_tiles   the same tile renderer over a caller-chosen subset of tiles (timing samples)
 *   ref_binding_*   (built with REF_WITH_BINDING into libref_binding.so) the GPU module's Lambda-side
 *                   binding on the scene built here: translation check and renders through it
 *   ref_kat_*       function-level known answers of reference units that need a scene or graph
 */
#include "../include/lambda_gpu.h"
#include "../lambda_gb300/csrc/lgpu_rng.h"
#ifdef REF_WITH_BINDING
#include "../lambda_gb300/binding/lambda_gpu_binding.h"
#endif

#include <camera/Camera.h>
#include <camera/Film.h>
#include <core/Instance.h>
#include <core/Scene.h>
#include <core/TriangleMesh.h>
#include <integrators/DirectLightingIntegrator.h>
#include <integrators/MISVolumetricPathIntegrator.h>
#include <integrators/PathIntegrator.h>
#include <integrators/VolumetricPathIntegrator.h>
#include <lighting/EnvironmentLight.h>
#include <lighting/LightSampler.h>
#include <lighting/ManyLightSampler.h>
#include <lighting/MeshLight.h>
#include <lighting/PointLight.h>
#include <lighting/Spotlight.h>
#include <render/Render.h>
#include <sampling/SampleShifter.h>
#include <shading/Fresnel.h>
#include <shading/MicrofacetDistribution.h>
#include <shading/Material.h>
#include <shading/graph/GraphBxDF.h>
#include <shading/graph/GraphConverters.h>
#include <shading/graph/GraphInputs.h>
#include <shading/graph/GraphMaths.h>
#include <shading/graph/GraphTexture.h>
#include <shading/media/HenyeyGreenstein.h>
#include <shading/media/HomogeneousMedium.h>

#include <atomic>
#include <cstring>
#include <iostream>
#include <memory>
#include <streambuf>
#include <string>
#include <thread>
#include <vector>

using namespace lambda;
namespace sg = lambda::ShaderGraph;

namespace {

thread_local std::string g_err;

/* Counter-based Sampler behind the reference's RNG seam (src/sampling/Sampler.h:9-25): the value of
 * dimension d of sample s of pixel p is lgpu_rng_float(lgpu_path_key(seed, p, s), d).  The pixel
 * comes from the SampleShifter that TileRenderers::UniformSpp points at each pixel
 * (SampleShifter::SetPixelIndex, no mask: y * width + x); Get2D draws x, then y. */
class CounterSampler : public Sampler {
  public:
    uint32_t seed = 0, offset = 0, key = 0, dim = 0;
    Sampler *clone() const override { return new CounterSampler(*this); }
    void NextSample() override { SetSample(sampleIndex + 1); }
    void SetSample(const unsigned _i) override {
        sampleIndex = _i;
        const uint32_t pixel = sampleShifter ? sampleShifter->GetPixelIndex() : 0u;
        key = lgpu_path_key(seed, pixel, _i + offset);
        dim = 0;
    }
    void SetPath(uint32_t pixel, uint32_t sample) {
        sampleIndex = sample;
        key = lgpu_path_key(seed, pixel, sample + offset);
        dim = 0;
    }
    Real Get1D() override { return lgpu_rng_float(key, dim++); }
    Vec2 Get2D() override {
        const Real a = Get1D();
        const Real b = Get1D();
        return Vec2(a, b);
    }
};

}  // namespace

/* The scene description has a VECTOR3 constant node; the reference's node factory has no class for
 * it (src/api/Material.cpp:136, commented out), so this one follows Vec2Input. */
namespace lambda {
namespace ShaderGraph {
class LgpuVec3Input : public Node {
  public:
    Vec3 vec3;
    LgpuVec3Input(const Vec3 &_v) : Node(0, 1, "Vector3 Input") {
        vec3 = _v;
        outputSockets[0] = MAKE_SOCKET(SocketType::TYPE_VEC3, &LgpuVec3Input::GetVec3, "Vector3");
    }
    void GetVec3(const ScatterEvent &, void *_out) const { *reinterpret_cast<Vec3 *>(_out) = vec3; }
};
}  // namespace ShaderGraph
}  // namespace lambda

namespace {

using Vec3Input = sg::LgpuVec3Input;

/* The reference's classes have no virtual destructors, so every object is owned through a
 * shared_ptr created with its concrete type (the deleter keeps that type). */
struct RefScene {
    std::vector<std::shared_ptr<void>> owned;
    Scene scene;
    std::vector<Object *> objects;                         /* meshes and instances, in scene order */
    std::vector<InstanceProxy *> proxies;
    std::vector<int> proxyOfMesh;
    std::vector<TriangleMesh *> meshObjectOf;              /* kind-0 object index -> its mesh */
    std::vector<Material *> materials;
    std::vector<BxDF *> bxdfOf;                            /* per desc node: the BxDF it is, or null */
    std::vector<sg::Textures::Noise *> noiseOf;            /* per desc node: the noise it is, or null */
    std::vector<Light *> lights;
    std::vector<Medium *> media;
    std::vector<Texture *> textures;
    LightSampler *lightSampler = nullptr;
    int n_desc_nodes = 0;

    template <class T, class... A> T *make(A &&...a) {
        std::shared_ptr<T> p(new T(std::forward<A>(a)...));
        owned.push_back(p);
        return p.get();
    }
};

template <class T, class... A> T *own(RefScene &R, A &&...a) { return R.make<T>(std::forward<A>(a)...); }

/* Builds one desc node as the reference's node class; records the BxDF and noise views. */
sg::Node *make_node(RefScene &R, const lgpu_node_desc &d, BxDF **bx, sg::Textures::Noise **nz) {
    *bx = nullptr;
    *nz = nullptr;
    RefScene &N = R;
    switch (d.type) {
    case LGPU_NODE_BXDF_MIX: { auto *n = own<sg::MixBxDFNode>(N); *bx = static_cast<MixBSDF *>(n); return n; }
    case LGPU_NODE_BXDF_LAMBERTIAN: { auto *n = own<sg::LambertianBRDFNode>(N); *bx = static_cast<LambertianBRDF *>(n); return n; }
    case LGPU_NODE_BXDF_OREN_NAYAR_R: { auto *n = own<sg::OrenNayarBRDFNode>(N); *bx = static_cast<OrenNayarBRDF *>(n); return n; }
    case LGPU_NODE_BXDF_OREN_NAYAR_T: { auto *n = own<sg::OrenNayarBTDFNode>(N); *bx = static_cast<OrenNayarBTDF *>(n); return n; }
    case LGPU_NODE_BXDF_MICROFACET_R: {
        MicrofacetDistribution *dist = (int)d.params[0] == LGPU_DIST_BECKMANN
                                           ? static_cast<MicrofacetDistribution *>(R.make<BeckmannDistribution>())
                                           : static_cast<MicrofacetDistribution *>(R.make<TrowbridgeReitzDistribution>());
        Fresnel *fr = R.make<FresnelDielectric>(d.params[1]);
        auto *n = own<sg::MicrofacetBRDFNode>(N, nullptr, nullptr, dist, fr);
        *bx = static_cast<MicrofacetBRDF *>(n);
        return n;
    }
    case LGPU_NODE_BXDF_GHOST: { auto *n = own<sg::GhostBTDFNode>(N); *bx = static_cast<GhostBTDF *>(n); return n; }
    case LGPU_NODE_BXDF_FRESNEL: { auto *n = own<sg::FresnelBSDFNode>(N); *bx = static_cast<FresnelBSDF *>(n); return n; }
    case LGPU_NODE_BXDF_SPECULAR_R: {
        Fresnel *fr = R.make<FresnelDielectric>(d.params[0]);
        auto *n = own<sg::SpecularBRDFNode>(N, nullptr, fr);
        *bx = static_cast<SpecularBRDF *>(n);
        return n;
    }
    case LGPU_NODE_BXDF_SPECULAR_T: { auto *n = own<sg::SpecularBTDFNode>(N, nullptr, (Real)d.params[0]); *bx = static_cast<SpecularBTDF *>(n); return n; }
    case LGPU_NODE_SEPARATE_XYZ: return own<sg::Converter::SeparateXYZ>(N);
    case LGPU_NODE_SEPARATE_RGBA: return own<sg::Converter::SeparateRGBA>(N);
    case LGPU_NODE_MERGE_XYZ: return own<sg::Converter::MergeXYZ>(N);
    case LGPU_NODE_MERGE_RGBA: return own<sg::Converter::MergeRGBA>(N);
    case LGPU_NODE_SCALAR: return own<sg::ScalarInput>(N, (Real)d.params[0]);
    case LGPU_NODE_VECTOR3: return own<Vec3Input>(N, Vec3(d.params[0], d.params[1], d.params[2]));
    case LGPU_NODE_VECTOR2: return own<sg::Vec2Input>(N, Vec2(d.params[0], d.params[1]));
    case LGPU_NODE_RGB: return own<sg::RGBInput>(N, Colour(d.params[0], d.params[1], d.params[2]));
    case LGPU_NODE_SPECTRUM: {
        const Real rgb[3] = {d.params[0], d.params[1], d.params[2]};
        return own<sg::SpectralInput>(N, Spectrum::FromRGB(rgb, SpectrumType::Reflectance));
    }
    case LGPU_NODE_BLACKBODY: return own<sg::BlackbodyInput>(N, nullptr, (unsigned)d.params[0]);
    case LGPU_NODE_IMAGE_TEXTURE: {
        const int t = (int)d.params[0];
        if (t < 0 || t >= (int)R.textures.size()) return nullptr;
        return own<sg::ImageTextureInput>(N, R.textures[t]);
    }
    case LGPU_NODE_SURFACE_INFO: return own<sg::SurfaceInfoInput>(N);
    case LGPU_NODE_MATHS: return own<sg::Maths::ScalarMathsNode>(N, (sg::Maths::ScalarOperatorType)d.op);
    case LGPU_NODE_VECTOR_MATHS: return own<sg::Maths::VectorMathsNode>(N, (sg::Maths::VectorOperatorType)d.op);
    case LGPU_NODE_DOT_PRODUCT: return own<sg::Maths::DotProductNode>(N);
    case LGPU_NODE_CROSS_PRODUCT: return own<sg::Maths::CrossProductNode>(N);
    case LGPU_NODE_VECTOR_MAGNITUDE: return own<sg::Maths::VectorLength>(N);
    case LGPU_NODE_PERLIN_NOISE: { auto *n = own<sg::Textures::PerlinNoise>(N, (Real)d.params[0]); *nz = n; return n; }
    case LGPU_NODE_VALUE_NOISE: { auto *n = own<sg::Textures::ValueNoise>(N, (Real)d.params[0]); *nz = n; return n; }
    case LGPU_NODE_OCTAVE_NOISE: { auto *n = own<sg::Textures::OctaveNoise>(N, (Real)d.params[0], (unsigned)d.params[1]); *nz = n; return n; }
    case LGPU_NODE_CHECKER: { auto *n = own<sg::Textures::Checker>(N, (Real)d.params[0]); *nz = n; return n; }
    case LGPU_NODE_VORONOI: { auto *n = own<sg::Textures::Voronoi>(N, (Real)d.params[0]); *nz = n; return n; }
    default: return nullptr;
    }
}

/* Node kinds whose callbacks read an input through `inputSockets[i].socket->` directly
 * (GraphConverters.cpp, GraphMaths.cpp, GraphInputs.cpp:84): an unlinked input there is a null
 * dereference in the reference, so its default value is fed by a constant node of the input's type. */
bool reads_socket_directly(int type) {
    switch (type) {
    case LGPU_NODE_SEPARATE_XYZ: case LGPU_NODE_SEPARATE_RGBA: case LGPU_NODE_MERGE_XYZ: case LGPU_NODE_MERGE_RGBA:
    case LGPU_NODE_MATHS: case LGPU_NODE_VECTOR_MATHS: case LGPU_NODE_DOT_PRODUCT: case LGPU_NODE_CROSS_PRODUCT:
    case LGPU_NODE_VECTOR_MAGNITUDE: case LGPU_NODE_BLACKBODY:
        return true;
    default:
        return false;
    }
}

sg::Node *constant_node(RefScene &R, sg::SocketType t, const float *v) {
    switch (t) {
    case sg::SocketType::TYPE_VEC3: return own<Vec3Input>(R, Vec3(v[0], v[1], v[2]));
    case sg::SocketType::TYPE_VEC2: return own<sg::Vec2Input>(R, Vec2(v[0], v[1]));
    case sg::SocketType::TYPE_COLOUR: return own<sg::RGBInput>(R, Colour(v[0], v[1], v[2], v[3]));
    default: return own<sg::ScalarInput>(R, (Real)v[0]);
    }
}

Vec3 v3(const float *p) { return Vec3(p[0], p[1], p[2]); }

TriangleMesh *make_mesh(RefScene &R, const lgpu_mesh_desc &md) {
    TriangleMesh *m = R.make<TriangleMesh>();
    Vec3 *verts = new Vec3[md.num_vertices];
    for (uint32_t k = 0; k < md.num_vertices; ++k) verts[k] = v3(md.vertices + 3 * k);
    Triangle *tris = new Triangle[md.num_triangles];
    for (uint32_t k = 0; k < md.num_triangles; ++k)
        tris[k] = Triangle{md.triangles[3 * k], md.triangles[3 * k + 1], md.triangles[3 * k + 2]};
    Vec3 *normals = nullptr, *tangents = nullptr;
    if (md.normals && md.tangents) {
        normals = new Vec3[md.num_vertices];
        tangents = new Vec3[md.num_vertices];
        for (uint32_t k = 0; k < md.num_vertices; ++k) {
            normals[k] = v3(md.normals + 3 * k);
            tangents[k] = v3(md.tangents + 4 * k);
            tangents[k].a = md.tangents[4 * k + 3];   /* bitangent handedness (TriangleMesh.h:27) */
        }
    }
    Vec2 *uvs = nullptr;
    if (md.uvs) {
        uvs = new Vec2[md.num_vertices];
        for (uint32_t k = 0; k < md.num_vertices; ++k) uvs[k] = Vec2(md.uvs[2 * k], md.uvs[2 * k + 1]);
    }
    m->AssignData(md.num_vertices, md.num_triangles, verts, tris, normals, tangents, nullptr, uvs);   /* the mesh frees them */
    m->smoothNormals = normals != nullptr;
    return m;
}

bool load(RefScene &R, const lgpu_scene_desc *d) {
    /* textures (texture_t<Colour>, scanline rows) */
    for (int t = 0; t < d->num_textures; ++t) {
        const lgpu_texture_desc &td = d->textures[t];
        Texture *tex = R.make<Texture>(td.width, td.height);
        for (int y = 0; y < td.height; ++y)
            for (int x = 0; x < td.width; ++x) {
                const float *p = td.rgba + 4 * ((size_t)y * td.width + x);
                tex->SetPixelCoord(x, y, Colour(p[0], p[1], p[2], p[3]));
            }
        R.textures.push_back(tex);
    }
    /* shader graph: nodes, then links and defaults */
    R.n_desc_nodes = d->num_nodes;
    std::vector<sg::Node *> node(d->num_nodes, nullptr);
    R.bxdfOf.assign(d->num_nodes, nullptr);
    R.noiseOf.assign(d->num_nodes, nullptr);
    for (int i = 0; i < d->num_nodes; ++i) {
        node[i] = make_node(R, d->nodes[i], &R.bxdfOf[i], &R.noiseOf[i]);
        if (!node[i]) { g_err = "node " + std::to_string(i) + ": type has no reference class"; return false; }
    }
    for (int i = 0; i < d->num_nodes; ++i) {
        const lgpu_node_desc &nd = d->nodes[i];
        if (nd.type == LGPU_NODE_OCTAVE_NOISE) {   /* OctaveNoise::noise: the inner noise node */
            auto *o = static_cast<sg::Textures::OctaveNoise *>(node[i]);
            const int k = nd.in_node[0];
            o->noise = (k >= 0 && k < d->num_nodes) ? R.noiseOf[k] : nullptr;
            if (!o->noise) { g_err = "octave noise without an inner noise node"; return false; }
            continue;
        }
        for (unsigned k = 0; k < node[i]->numIn && k < LGPU_NODE_MAX_INPUTS; ++k) {
            sg::SocketRef &in = node[i]->inputSockets[k];
            const int src = nd.in_node[k];
            if (src >= 0) {
                if (src >= d->num_nodes || nd.in_socket[k] < 0 || (unsigned)nd.in_socket[k] >= node[src]->numOut) {
                    g_err = "bad link";
                    return false;
                }
                in = &node[src]->outputSockets[nd.in_socket[k]];
            } else {
                for (int c = 0; c < 4; ++c) in.data[c] = nd.in_default[k][c];
                if (reads_socket_directly(nd.type)) {
                    sg::Node *cn = constant_node(R, in.socketType, nd.in_default[k]);
                    in = &cn->outputSockets[0];
                }
            }
        }
    }
    /* media */
    for (int i = 0; i < d->num_media; ++i) {
        const lgpu_medium_desc &m = d->media[i];
        HomogeneousMedium *med = R.make<HomogeneousMedium>(Spectrum::FromRGB(m.sigma_a, SpectrumType::Reflectance),
                                                           Spectrum::FromRGB(m.sigma_s, SpectrumType::Reflectance));
        med->phase = R.make<HenyeyGreenstein>(m.g);
        R.media.push_back(med);
    }
    auto medium = [&](int i) -> Medium * { return i >= 0 && i < (int)R.media.size() ? R.media[i] : nullptr; };
    /* materials (lights are attached after the lights exist) */
    for (int i = 0; i < d->num_materials; ++i) {
        const lgpu_material_desc &md = d->materials[i];
        Material *m = R.make<Material>();
        m->bxdf = nullptr;
        m->light = nullptr;
        if (md.bxdf_node >= 0) {
            if (md.bxdf_node >= d->num_nodes || !R.bxdfOf[md.bxdf_node]) { g_err = "material BxDF is not a BxDF node"; return false; }
            m->bxdf = R.bxdfOf[md.bxdf_node];
        }
        m->mediaBoundary = MediaBoundary(medium(md.medium_interior), medium(md.medium_exterior));
        R.materials.push_back(m);
    }
    /* objects: kind 0 = the mesh itself; kind 1 = Instance of an InstanceProxy over the mesh */
    R.proxyOfMesh.assign(d->num_meshes, -1);
    R.meshObjectOf.assign(d->num_objects, nullptr);
    for (int i = 0; i < d->num_objects; ++i) {
        const lgpu_object_desc &od = d->objects[i];
        if (od.mesh < 0 || od.mesh >= d->num_meshes || od.material < 0 || od.material >= d->num_materials) {
            g_err = "bad object";
            return false;
        }
        Object *o;
        if (od.kind == 0) {
            TriangleMesh *m = make_mesh(R, d->meshes[od.mesh]);
            R.meshObjectOf[i] = m;
            o = m;
        } else {
            if (R.proxyOfMesh[od.mesh] < 0) {
                TriangleMesh *pm = make_mesh(R, d->meshes[od.mesh]);
                pm->material = R.materials[od.material];
                R.proxies.push_back(R.make<InstanceProxy>(pm));
                R.proxies.back()->Commit(R.scene.device);
                R.proxyOfMesh[od.mesh] = (int)R.proxies.size() - 1;
            }
            Instance *in = R.make<Instance>(R.proxies[R.proxyOfMesh[od.mesh]]);
            for (int k = 0; k < 12; ++k) in->xfm[k] = od.xfm[k];
            o = in;
        }
        o->material = R.materials[od.material];
        R.objects.push_back(o);
    }
    /* lights, in description order (Scene::lights order feeds the light tree) */
    for (int i = 0; i < d->num_lights; ++i) {
        const lgpu_light_desc &ld = d->lights[i];
        sg::Socket *emission = nullptr;
        if (ld.type != LGPU_LIGHT_ENVIRONMENT) {
            if (ld.emission_node < 0 || ld.emission_node >= d->num_nodes) { g_err = "light without emission"; return false; }
            emission = &node[ld.emission_node]->outputSockets[ld.emission_socket];
        }
        Light *l = nullptr;
        if (ld.type == LGPU_LIGHT_MESH) {
            if (ld.object < 0 || ld.object >= d->num_objects || !R.meshObjectOf[ld.object]) { g_err = "mesh light on a non-mesh object"; return false; }
            MeshLight *ml = R.make<MeshLight>(R.meshObjectOf[ld.object]);
            ml->emission = emission;
            ml->intensity = ld.intensity;
            l = ml;
        } else if (ld.type == LGPU_LIGHT_POINT) {
            l = R.make<PointLight>(v3(ld.position), emission, ld.intensity);
        } else if (ld.type == LGPU_LIGHT_SPOT) {
            Spotlight *s = R.make<Spotlight>(v3(ld.position), v3(ld.axis), ld.cone_angle, ld.falloff_start);
            s->emission = emission;
            s->intensity = ld.intensity;
            l = s;
        } else if (ld.type == LGPU_LIGHT_ENVIRONMENT) {
            Texture *tex = R.make<Texture>(ld.env_width, ld.env_height);
            for (int y = 0; y < ld.env_height; ++y)
                for (int x = 0; x < ld.env_width; ++x) {
                    const float *p = ld.env_texture + 3 * ((size_t)y * ld.env_width + x);
                    tex->SetPixelCoord(x, y, Colour(p[0], p[1], p[2]));
                }
            EnvironmentLight *e = R.make<EnvironmentLight>(tex, ld.intensity);
            e->offset = Vec2(ld.offset[0], ld.offset[1]);
            l = e;
        } else {
            g_err = "unknown light type";
            return false;
        }
        R.lights.push_back(l);
    }
    for (int i = 0; i < d->num_materials; ++i) {
        const int li = d->materials[i].light;
        if (li >= 0 && li < (int)R.lights.size()) R.materials[i]->light = R.lights[li];
    }
    for (Object *o : R.objects) R.scene.AddObject(o, false);
    for (Light *l : R.lights) R.scene.AddLight(l);
    R.scene.hasVolumes = d->has_volumes != 0;
    if (d->light_strategy == LGPU_LIGHT_STRATEGY_POWER) R.lightSampler = R.make<PowerLightSampler>(R.scene);
    else R.lightSampler = R.make<ManyLightSampler>(R.scene);
    R.scene.lightSampler = R.lightSampler;
    R.scene.Commit();
    return true;
}

/* Camera from the descriptor (Camera.cpp:7-71); aspect = height / width. */
struct RefCamera {
    std::shared_ptr<Camera> cam;
    std::shared_ptr<Aperture> ap;
};
bool make_camera(const lgpu_camera_desc &c, int W, int H, RefCamera &out) {
    const Vec3 o = v3(c.origin);
    if (c.type == LGPU_CAMERA_SPHERICAL) {
        std::shared_ptr<SphericalCamera> s(new SphericalCamera(o));
        s->offsetPhi = c.offset_phi;      /* B29: uninitialised in the reference */
        s->offsetTheta = c.offset_theta;
        out.cam = s;
    } else if (c.type == LGPU_CAMERA_THIN_LENS) {
        if (c.aperture == LGPU_APERTURE_CIRCULAR) out.ap = std::shared_ptr<CircularAperture>(new CircularAperture(c.aperture_size));
        else if (c.aperture == LGPU_APERTURE_BLADE) out.ap = std::shared_ptr<BladeAperture>(new BladeAperture((unsigned)c.blades, c.aperture_size));
        else if (c.aperture != LGPU_APERTURE_NONE) { g_err = "masked aperture not driven here"; return false; }
        out.cam = std::shared_ptr<ThinLensCamera>(new ThinLensCamera(o, (Real)W, (Real)H, c.focal_length, out.ap.get()));
    } else {
        out.cam = std::shared_ptr<PinholeCamera>(new PinholeCamera(o, (Real)W, (Real)H));
    }
    out.cam->SetAxes(v3(c.x_hat), v3(c.y_hat), v3(c.z_hat));
    out.cam->SetFov(c.fov);
    return true;
}

std::shared_ptr<Integrator> make_integrator(const lgpu_render_opts &o, Sampler *s) {
    switch (o.integrator) {
    case LGPU_INTEGRATOR_PATH: return std::shared_ptr<PathIntegrator>(new PathIntegrator(s, o.max_bounces, o.min_bounces));
    case LGPU_INTEGRATOR_VOLPATH:
        return std::shared_ptr<VolumetricPathIntegrator>(new VolumetricPathIntegrator(s, o.max_bounces, o.min_bounces));
    case LGPU_INTEGRATOR_GPU_MISVOLPATH:
        return std::shared_ptr<MISVolumetricPathIntegrator>(new MISVolumetricPathIntegrator(s, o.max_bounces, o.min_bounces));
    default: return nullptr;
    }
}

/* f(0 .. n-1) on `threads` threads, handed out dynamically in chunks of `grain` */
template <class F> void parallel(uint64_t n, int threads, uint64_t grain, F &&f) {
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<uint64_t> next(0);
    auto work = [&]() {
        for (;;) {
            const uint64_t b = next.fetch_add(grain);
            if (b >= n) return;
            for (uint64_t i = b; i < std::min(n, b + grain); ++i) f(i);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
}

/* film (H x W float4: summed rgb, samples) through RenderMosaic + TileRenderers::UniformSpp
 * (Render.cpp:11-64) over `tiles` (all tiles when null), tiles dealt to threads dynamically */
int render_tiles(RefScene &R, const lgpu_camera_desc *cd, const lgpu_render_opts *o, const int32_t *tiles, int n_tiles,
                 float *film_out, int threads) {
    RefCamera rc;
    if (!make_camera(*cd, o->width, o->height, rc)) return 1;
    CounterSampler proto;
    proto.seed = o->seed;
    proto.offset = o->sample_offset;
    std::shared_ptr<Integrator> integ = make_integrator(*o, &proto);
    if (!integ) { g_err = "integrator not driven here"; return 1; }
    Film film(o->width, o->height);
    SampleShifter shifter(nullptr);
    RenderDirective dir;
    dir.film = &film;
    dir.scene = &R.scene;
    dir.camera = rc.cam.get();
    dir.integrator = integ.get();
    dir.sampler = &proto;
    dir.sampleShifter = &shifter;
    dir.tileSizeX = dir.tileSizeY = 16;
    dir.spp = o->spp;
    RenderMosaic mosaic(dir);
    std::vector<int> todo;
    if (tiles) {
        for (int i = 0; i < n_tiles; ++i) {
            const int t = tiles[i];
            if (t >= 0 && t < (int)mosaic.tiles.size()) todo.push_back(t);
        }
    } else {
        for (int i = 0; i < (int)mosaic.tiles.size(); ++i) todo.push_back(i);
    }
    parallel(todo.size(), threads, 1, [&](uint64_t k) { TileRenderers::UniformSpp(&mosaic.tiles[todo[k]]); });
    for (int y = 0; y < o->height; ++y)
        for (int x = 0; x < o->width; ++x) {
            const FilmPixel &p = film.filmData.GetPixelCoord(x, y);
            float *f = film_out + 4 * ((size_t)y * o->width + x);
            f[0] = p.spectrum[0]; f[1] = p.spectrum[1]; f[2] = p.spectrum[2]; f[3] = (float)p.nSamples;
        }
    return 0;
}

}  // namespace

extern "C" {

__attribute__((visibility("default"))) const char *ref_last_error() { return g_err.c_str(); }

/* ManyLightSampler::Commit reports progress on std::cout; callers of this library own stdout (a
 * benchmark prints one JSON line there), so the scene build runs with std::cout discarded. */
struct NullBuf : std::streambuf {
    int overflow(int c) override { return c; }
};

__attribute__((visibility("default"))) void *ref_create(const lgpu_scene_desc *d) {
    static NullBuf sink;
    std::streambuf *keep = std::cout.rdbuf(&sink);
    RefScene *R = new RefScene();
    const bool ok = load(*R, d);
    std::cout.rdbuf(keep);
    if (!ok) { delete R; return nullptr; }
    return R;
}

__attribute__((visibility("default"))) void ref_destroy(void *h) { delete static_cast<RefScene *>(h); }

/* paths_out: n x 4 floats (rgb, random numbers drawn) for path ids `ids` (id = pixel * spp + sample);
 * or, with ids == null, the whole film (height x width x 4) by the tile renderer.  Returns 0 on success. */
__attribute__((visibility("default"))) int ref_render(void *h, const lgpu_camera_desc *cd, const lgpu_render_opts *o,
                                                      const uint64_t *ids, uint64_t n, float *film, float *paths_out,
                                                      int threads) {
    RefScene &R = *static_cast<RefScene *>(h);
    if (!ids) return film ? render_tiles(R, cd, o, nullptr, 0, film, threads) : 1;
    RefCamera rc;
    if (!make_camera(*cd, o->width, o->height, rc)) return 1;
    {
        CounterSampler probe;
        std::shared_ptr<Integrator> t = make_integrator(*o, &probe);
        if (!t) { g_err = "integrator not driven here"; return 1; }
    }
    const int W = o->width, H = o->height;
    const Real xi = (Real)1 / W, yi = (Real)1 / H;
    parallel(n, threads, 64, [&](uint64_t i) {
        CounterSampler s;
        s.seed = o->seed;
        s.offset = o->sample_offset;
        std::shared_ptr<Integrator> integ = make_integrator(*o, &s);
        const uint64_t pid = ids[i];
        const uint32_t pixel = (uint32_t)(pid / (uint64_t)o->spp);
        const uint32_t sample = (uint32_t)(pid % (uint64_t)o->spp);
        const uint32_t x = pixel % (uint32_t)W, y = pixel / (uint32_t)W;
        s.SetPath(pixel, sample);
        /* TileRenderers::UniformSpp, one sample (Render.cpp:55-58) */
        const Real u = xi * ((Real)x + s.Get1D() - .5);
        const Real v = yi * ((Real)y + s.Get1D() - .5);
        const Ray r = rc.cam->GenerateRay(u, v, s);
        const Spectrum L = integ->Li(r, R.scene);
        float *p = paths_out + 4 * i;
        p[0] = L[0]; p[1] = L[1]; p[2] = L[2]; p[3] = (float)s.dim;
    });
    (void)H;
    return 0;
}

/* The tile renderer over chosen tiles of 16 x 16 pixels (row-major tile index over the film);
 * film as in ref_render.  Used to time a bounded sample of a frame. */
__attribute__((visibility("default"))) int ref_render_tiles(void *h, const lgpu_camera_desc *cd, const lgpu_render_opts *o,
                                                            const int32_t *tiles, int n_tiles, float *film, int threads) {
    return render_tiles(*static_cast<RefScene *>(h), cd, o, tiles, n_tiles, film, threads);
}

#ifdef REF_WITH_BINDING
/* The GPU module's Lambda-side binding (lambda_gb300/binding) run on the lambda::Scene built here:
 * the translation back to a scene description, checked on the host (lgpu_scene_check), and
 * renders through its RenderDirective and TileRenderer entry points. */

/* counts: meshes, objects, materials, nodes, lights, media, textures, has_volumes, light_strategy */
__attribute__((visibility("default"))) int ref_binding_check(void *h, char *report, size_t report_size, int32_t *counts) {
    RefScene &R = *static_cast<RefScene *>(h);
    lambda_gpu::SceneDesc sd;
    const int rc = sd.Build(R.scene);
    if (rc != LGPU_OK) {
        g_err = sd.Error();
        if (report && report_size) { std::strncpy(report, g_err.c_str(), report_size - 1); report[report_size - 1] = 0; }
        return rc;
    }
    const lgpu_scene_desc &d = sd.Desc();
    const int32_t c[9] = {d.num_meshes, d.num_objects, d.num_materials, d.num_nodes, d.num_lights, d.num_media,
                          d.num_textures, d.has_volumes, d.light_strategy};
    for (int k = 0; k < 9; ++k) counts[k] = c[k];
    return lgpu_scene_check(&d, report, report_size);
}

/* mode 0: GpuRenderer::RenderDirective over the whole film; mode 1: RenderMosaic's 16 x 16 tiles
 * through GpuTileRenderer.  film_out: height x width x 4 (summed rgb, samples). */
__attribute__((visibility("default"))) int ref_binding_render(void *h, const lgpu_camera_desc *cd, const lgpu_render_opts *o,
                                                              int mode, float *film_out) {
    RefScene &R = *static_cast<RefScene *>(h);
    RefCamera rc;
    if (!make_camera(*cd, o->width, o->height, rc)) return LGPU_ERR_INVALID_ARG;
    CounterSampler proto;
    proto.seed = o->seed;
    std::shared_ptr<Integrator> integ = make_integrator(*o, &proto);
    if (!integ) { g_err = "integrator not driven here"; return LGPU_ERR_INVALID_ARG; }
    Film film(o->width, o->height);
    SampleShifter shifter(nullptr);
    RenderDirective dir;
    dir.film = &film;
    dir.scene = &R.scene;
    dir.camera = rc.cam.get();
    dir.integrator = integ.get();
    dir.sampler = &proto;
    dir.sampleShifter = &shifter;
    dir.tileSizeX = dir.tileSizeY = 16;
    dir.spp = o->spp;
    lambda_gpu::GpuRenderer gpu(0);
    gpu.seed = o->seed;
    gpu.kernelMode = o->kernel_mode;
    int r = gpu.Commit(R.scene);
    if (r == LGPU_OK) {
        if (mode == 0) {
            r = gpu.RenderDirective(dir);
        } else {
            RenderMosaic mosaic(dir);
            lambda_gpu::SetTileRenderer(&gpu);
            for (RenderTile &t : mosaic.tiles) lambda_gpu::GpuTileRenderer(&t);
            r = lambda_gpu::TileRendererError();
            lambda_gpu::SetTileRenderer(nullptr);
        }
    }
    if (r != LGPU_OK) { g_err = gpu.LastError(); return r; }
    for (int y = 0; y < o->height; ++y)
        for (int x = 0; x < o->width; ++x) {
            const FilmPixel &p = film.filmData.GetPixelCoord(x, y);
            float *f = film_out + 4 * ((size_t)y * o->width + x);
            f[0] = p.spectrum[0]; f[1] = p.spectrum[1]; f[2] = p.spectrum[2]; f[3] = (float)p.nSamples;
        }
    return LGPU_OK;
}
#endif

}  // extern "C"
