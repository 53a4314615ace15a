/*
 * Lambda-side binding of the GPU path tracer: lambda::Scene -> lgpu_scene_desc, RenderDirective
 * and TileRenderer entry points.  See lambda_gpu_binding.h for what it needs from Lambda's headers.
 */
#include "lambda_gpu_binding.h"

#include <cmath>
#include <cstring>

#include <core/Instance.h>
#include <core/TriangleMesh.h>
#include <integrators/MISVolumetricPathIntegrator.h>
#include <integrators/PathIntegrator.h>
#include <integrators/VolumetricPathIntegrator.h>
#include <lighting/EnvironmentLight.h>
#include <lighting/LightSampler.h>
#include <lighting/ManyLightSampler.h>
#include <lighting/MeshLight.h>
#include <lighting/PointLight.h>
#include <lighting/Spotlight.h>
#include <shading/Fresnel.h>
#include <shading/Material.h>
#include <shading/MicrofacetDistribution.h>
#include <shading/graph/GraphBxDF.h>
#include <shading/graph/GraphConverters.h>
#include <shading/graph/GraphInputs.h>
#include <shading/graph/GraphMaths.h>
#include <shading/graph/GraphTexture.h>
#include <shading/media/HenyeyGreenstein.h>
#include <shading/media/HomogeneousMedium.h>

namespace lambda_gpu {

namespace sg = lambda::ShaderGraph;
using ::Real;
using ::Vec3;

namespace {

/* A float x whose cosf equals c: Spotlight keeps only cos(coneAngle) (Spotlight.cpp:17-18) and the
 * module takes the angle and evaluates std::cos(float) again, so the angle is chosen to give back
 * the same float. */
float angle_for_cos(float c) {
    const float a0 = (float)std::acos((double)c);
    float lo = a0, hi = a0;
    for (int k = 0; k < 256; ++k) {
        if (std::cos(lo) == c) return lo;
        if (std::cos(hi) == c) return hi;
        lo = std::nextafter(lo, -INFINITY);
        hi = std::nextafter(hi, INFINITY);
    }
    return a0;
}

/* A float fov with (float)tan(0.5 * fov) == tanFov (Camera::SetFov, Camera.cpp:32-35, and the
 * module's make_cam do this in double and round to float). */
float fov_for_tan(float tanFov) {
    const float f0 = (float)(2.0 * std::atan((double)tanFov));
    float lo = f0, hi = f0;
    for (int k = 0; k < 256; ++k) {
        if ((float)std::tan(.5 * (double)lo) == tanFov) return lo;
        if ((float)std::tan(.5 * (double)hi) == tanFov) return hi;
        lo = std::nextafter(lo, -INFINITY);
        hi = std::nextafter(hi, INFINITY);
    }
    return f0;
}

void copy3(float *d, const Vec3 &v) { d[0] = v.x; d[1] = v.y; d[2] = v.z; }

/* Node kinds by Node::nodeTag (the tags the constructors in src/shading/graph/*.cpp pass). */
struct TagKind { const char *tag; int type; };
const TagKind kTags[] = {
    {"Mix BSDF", LGPU_NODE_BXDF_MIX}, {"Lambertian BRDF", LGPU_NODE_BXDF_LAMBERTIAN},
    {"Oren-Nayar BRDF", LGPU_NODE_BXDF_OREN_NAYAR_R}, {"Oren-Nayar BTDF", LGPU_NODE_BXDF_OREN_NAYAR_T},
    {"Microfcet BRDF", LGPU_NODE_BXDF_MICROFACET_R}, {"Ghost BTDF", LGPU_NODE_BXDF_GHOST},
    {"Fresnel BSDF", LGPU_NODE_BXDF_FRESNEL}, {"Specular BRDF", LGPU_NODE_BXDF_SPECULAR_R},
    {"Specular BTDF", LGPU_NODE_BXDF_SPECULAR_T}, {"Separate XYZ", LGPU_NODE_SEPARATE_XYZ},
    {"Separate RGBA", LGPU_NODE_SEPARATE_RGBA}, {"Merge XYZ", LGPU_NODE_MERGE_XYZ},
    {"Merge RGBA", LGPU_NODE_MERGE_RGBA}, {"Scalar Input", LGPU_NODE_SCALAR}, {"Vector2 Input", LGPU_NODE_VECTOR2},
    {"RGB Input", LGPU_NODE_RGB}, {"Spectrum", LGPU_NODE_SPECTRUM}, {"Blackbody Spectrum", LGPU_NODE_BLACKBODY},
    {"Image Texture", LGPU_NODE_IMAGE_TEXTURE}, {"Surface Information", LGPU_NODE_SURFACE_INFO},
    {"Maths", LGPU_NODE_MATHS}, {"Vector Maths", LGPU_NODE_VECTOR_MATHS}, {"Dot", LGPU_NODE_DOT_PRODUCT},
    {"Cross", LGPU_NODE_CROSS_PRODUCT}, {"Length", LGPU_NODE_VECTOR_MAGNITUDE},
    {"Perlin Noise", LGPU_NODE_PERLIN_NOISE}, {"Value Noise", LGPU_NODE_VALUE_NOISE},
    {"Octave Noise", LGPU_NODE_OCTAVE_NOISE}, {"Checker", LGPU_NODE_CHECKER}, {"Voronoi", LGPU_NODE_VORONOI},
};

int kind_of_tag(const std::string &tag) {
    for (const TagKind &t : kTags)
        if (tag == t.tag) return t.type;
    return -1;
}

}  // namespace

/* ------------------------------------------------------------------ scene translation */

bool SceneDesc::Fail(int code, const std::string &msg) {
    if (code_ == LGPU_OK) { code_ = code; err_ = msg; }
    return false;
}

int SceneDesc::Mesh(const lambda::TriangleMesh *m) {
    auto it = meshIdx_.find(m);
    if (it != meshIdx_.end()) return it->second;
    lgpu_mesh_desc md{};
    const size_t nv = m->numVertices, nt = m->numTriangles;
    auto *v = new std::vector<float>(3 * nv);
    for (size_t k = 0; k < nv; ++k) copy3(&(*v)[3 * k], m->vertices[k]);
    floats_.emplace_back(v);
    auto *t = new std::vector<uint32_t>(3 * nt);
    for (size_t k = 0; k < nt; ++k) {
        (*t)[3 * k] = m->triangles[k].v0; (*t)[3 * k + 1] = m->triangles[k].v1; (*t)[3 * k + 2] = m->triangles[k].v2;
    }
    words_.emplace_back(t);
    md.vertices = v->data();
    md.triangles = t->data();
    /* smooth frames need normals and tangents (TriangleMesh::ProcessHit, TriangleMesh.cpp:80-114) */
    if (m->smoothNormals && m->vertexNormals && m->vertexTangents) {
        auto *n = new std::vector<float>(3 * nv), *g = new std::vector<float>(4 * nv);
        for (size_t k = 0; k < nv; ++k) {
            copy3(&(*n)[3 * k], m->vertexNormals[k]);
            copy3(&(*g)[4 * k], m->vertexTangents[k]);
            (*g)[4 * k + 3] = m->vertexTangents[k].a;   /* bitangent handedness (TriangleMesh.h:27) */
        }
        floats_.emplace_back(n);
        floats_.emplace_back(g);
        md.normals = n->data();
        md.tangents = g->data();
    }
    if (m->textureCoordinates) {
        auto *u = new std::vector<float>(2 * nv);
        for (size_t k = 0; k < nv; ++k) { (*u)[2 * k] = m->textureCoordinates[k].x; (*u)[2 * k + 1] = m->textureCoordinates[k].y; }
        floats_.emplace_back(u);
        md.uvs = u->data();
    }
    md.num_vertices = (uint32_t)nv;
    md.num_triangles = (uint32_t)nt;
    meshes_.push_back(md);
    return meshIdx_[m] = (int)meshes_.size() - 1;
}

int SceneDesc::Medium(const lambda::Medium *m) {
    if (!m) return -1;
    auto it = mediumIdx_.find(m);
    if (it != mediumIdx_.end()) return it->second;
    const auto *h = dynamic_cast<const lambda::HomogeneousMedium *>(m);
    const auto *hg = h ? dynamic_cast<const lambda::HenyeyGreenstein *>(h->phase) : nullptr;
    if (!h || !hg) return Fail(LGPU_ERR_UNSUPPORTED_NODE, "only HomogeneousMedium with a HenyeyGreenstein phase is supported"), -2;
    lgpu_medium_desc md{};
    for (int c = 0; c < 3; ++c) { md.sigma_a[c] = h->sigmaA[c]; md.sigma_s[c] = h->sigmaS[c]; }
    md.g = hg->g;
    media_.push_back(md);
    return mediumIdx_[m] = (int)media_.size() - 1;
}

int SceneDesc::Texture(const lambda::Texture *t, bool apertureMask) {
    auto it = textureIdx_.find(t);
    if (it != textureIdx_.end()) return it->second;
    const unsigned w = t->GetWidth(), h = t->GetHeight();
    auto *px = new std::vector<float>((size_t)w * h * 4);
    for (unsigned y = 0; y < h; ++y)
        for (unsigned x = 0; x < w; ++x) {
            const lambda::Colour c = t->GetPixelCoord(x, y);
            float *p = &(*px)[4 * ((size_t)y * w + x)];
            p[0] = c.r; p[1] = c.g; p[2] = c.b; p[3] = c.a;
        }
    floats_.emplace_back(px);
    lgpu_texture_desc td{};
    td.rgba = px->data();
    td.width = (int32_t)w;
    td.height = (int32_t)h;
    td.aperture_mask = apertureMask ? 1 : 0;
    textures_.push_back(td);
    return textureIdx_[t] = (int)textures_.size() - 1;
}

/* The node owning output socket `s` (Socket::node, which Node's constructor sets and the socket
 * macros keep), and the socket's index there. */
bool SceneDesc::Link(sg::Socket *s, int32_t *node, int32_t *socket) {
    sg::Node *n = s->node;
    if (!n) return Fail(LGPU_ERR_INVALID_SCENE, "a linked output socket does not record its node");
    const sg::Socket *first = n->outputSockets.get();
    if (s < first || s >= first + n->numOut) return Fail(LGPU_ERR_INVALID_SCENE, "socket not found in its node");
    const int k = Node(n);
    if (k < 0) return false;
    *node = k;
    *socket = (int32_t)(s - first);
    return true;
}

int SceneDesc::Node(sg::Node *n) {
    auto it = nodeIdx_.find(n);
    if (it != nodeIdx_.end()) return it->second;
    int type = kind_of_tag(n->nodeTag);
    float folded[4] = {0, 0, 0, 0};
    if (type < 0 && n->numIn == 0 && n->numOut == 1) {
        /* a constant node of a class the binding does not know (an application's own input node):
         * evaluated once, it becomes the input node of its output type */
        lambda::ScatterEvent ev{};
        sg::Socket &o = n->outputSockets[0];
        switch (o.socketType) {
        case sg::SocketType::TYPE_SCALAR: type = LGPU_NODE_SCALAR; folded[0] = o.GetAs<Real>(ev); break;
        case sg::SocketType::TYPE_VEC2: { const ::Vec2 v = o.GetAs<::Vec2>(ev); type = LGPU_NODE_VECTOR2; folded[0] = v.x; folded[1] = v.y; break; }
        case sg::SocketType::TYPE_VEC3: { const Vec3 v = o.GetAs<Vec3>(ev); type = LGPU_NODE_VECTOR3; copy3(folded, v); break; }
        case sg::SocketType::TYPE_COLOUR: {
            const lambda::Colour c = o.GetAs<lambda::Colour>(ev);
            type = LGPU_NODE_RGB; folded[0] = c.r; folded[1] = c.g; folded[2] = c.b;
            break;
        }
        case sg::SocketType::TYPE_SPECTRUM: {   /* e.g. SpectralInput(const Spectrum &), which passes no tag */
            const lambda::Spectrum sp = o.GetAsSpectrum(ev);
            type = LGPU_NODE_SPECTRUM; folded[0] = sp[0]; folded[1] = sp[1]; folded[2] = sp[2];
            break;
        }
        default: break;
        }
        if (type >= 0) {
            const int idx = (int)nodes_.size();
            nodeIdx_[n] = idx;
            lgpu_node_desc nd;
            std::memset(&nd, 0, sizeof(nd));
            nd.type = type;
            for (int k = 0; k < 4; ++k) nd.params[k] = folded[k];
            for (int k = 0; k < LGPU_NODE_MAX_INPUTS; ++k) nd.in_node[k] = -1;
            nodes_.push_back(nd);
            return idx;
        }
    }
    if (type < 0) return Fail(LGPU_ERR_UNSUPPORTED_NODE, "shader node \"" + n->nodeTag + "\" has no GPU implementation"), -1;
    const int idx = (int)nodes_.size();
    nodeIdx_[n] = idx;
    lgpu_node_desc nd;
    std::memset(&nd, 0, sizeof(nd));
    nd.type = type;
    for (int k = 0; k < LGPU_NODE_MAX_INPUTS; ++k) { nd.in_node[k] = -1; nd.in_socket[k] = 0; }
    nodes_.push_back(nd);
    switch (type) {
    case LGPU_NODE_BXDF_MICROFACET_R: {
        const auto *mf = static_cast<lambda::MicrofacetBRDF *>(static_cast<sg::MicrofacetBRDFNode *>(n));
        const auto *fr = dynamic_cast<const lambda::FresnelDielectric *>(mf->fresnel);
        if (!fr) return Fail(LGPU_ERR_UNSUPPORTED_NODE, "microfacet BRDF with a non-dielectric Fresnel"), -1;
        nd.params[0] = dynamic_cast<const lambda::BeckmannDistribution *>(mf->distribution) ? LGPU_DIST_BECKMANN
                                                                                              : LGPU_DIST_TROWBRIDGE_REITZ;
        nd.params[1] = fr->etaT;
        break;
    }
    case LGPU_NODE_BXDF_SPECULAR_R: {
        const auto *sp = static_cast<lambda::SpecularBRDF *>(static_cast<sg::SpecularBRDFNode *>(n));
        const auto *fr = dynamic_cast<const lambda::FresnelDielectric *>(sp->fresnel);
        if (!fr) return Fail(LGPU_ERR_UNSUPPORTED_NODE, "specular BRDF with a non-dielectric Fresnel"), -1;
        nd.params[0] = fr->etaT;
        break;
    }
    case LGPU_NODE_BXDF_SPECULAR_T:
        nd.params[0] = static_cast<lambda::SpecularBTDF *>(static_cast<sg::SpecularBTDFNode *>(n))->fresnel.etaT;
        break;
    case LGPU_NODE_SCALAR: nd.params[0] = static_cast<sg::ScalarInput *>(n)->value; break;
    case LGPU_NODE_VECTOR2: {
        const auto &v = static_cast<sg::Vec2Input *>(n)->vec2;
        nd.params[0] = v.x; nd.params[1] = v.y;
        break;
    }
    case LGPU_NODE_RGB: {
        const auto &c = static_cast<sg::RGBInput *>(n)->rgb;
        nd.params[0] = c.r; nd.params[1] = c.g; nd.params[2] = c.b;
        break;
    }
    case LGPU_NODE_SPECTRUM: {
        /* RGB spectra (the build's Spectrum is RGBSpectrum): the stored coefficients are the rgb */
        const auto &sp = static_cast<sg::SpectralInput *>(n)->spec;
        nd.params[0] = sp[0]; nd.params[1] = sp[1]; nd.params[2] = sp[2];
        break;
    }
    case LGPU_NODE_BLACKBODY: nd.params[0] = (float)static_cast<sg::BlackbodyInput *>(n)->samples; break;
    case LGPU_NODE_IMAGE_TEXTURE: {
        const auto *tex = static_cast<sg::ImageTextureInput *>(n)->tex;
        if (!tex) return Fail(LGPU_ERR_INVALID_SCENE, "image texture node without a texture"), -1;
        const int t = Texture(tex, false);
        nd.params[0] = (float)t;
        break;
    }
    case LGPU_NODE_MATHS: nd.op = (int32_t) static_cast<sg::Maths::ScalarMathsNode *>(n)->operatorType; break;
    case LGPU_NODE_VECTOR_MATHS: nd.op = (int32_t) static_cast<sg::Maths::VectorMathsNode *>(n)->operatorType; break;
    case LGPU_NODE_PERLIN_NOISE: nd.params[0] = static_cast<sg::Textures::PerlinNoise *>(n)->scale; break;
    case LGPU_NODE_VALUE_NOISE: nd.params[0] = static_cast<sg::Textures::ValueNoise *>(n)->scale; break;
    case LGPU_NODE_CHECKER: nd.params[0] = static_cast<sg::Textures::Checker *>(n)->scale; break;
    case LGPU_NODE_VORONOI: nd.params[0] = static_cast<sg::Textures::Voronoi *>(n)->scale; break;
    case LGPU_NODE_OCTAVE_NOISE: {
        auto *o = static_cast<sg::Textures::OctaveNoise *>(n);
        nd.params[0] = o->scale;
        nd.params[1] = (float)o->octaves;
        sg::Node *inner = o->noise ? dynamic_cast<sg::Node *>(o->noise) : nullptr;
        if (!inner) return Fail(LGPU_ERR_INVALID_SCENE, "octave noise without an inner noise node"), -1;
        const int k = Node(inner);
        if (k < 0) return -1;
        nd.in_node[0] = k;   /* OctaveNoise::noise, not a socket */
        break;
    }
    default: break;
    }
    if (type != LGPU_NODE_OCTAVE_NOISE) {
        if (n->numIn > LGPU_NODE_MAX_INPUTS) return Fail(LGPU_ERR_UNSUPPORTED_NODE, "node with more than four inputs"), -1;
        for (unsigned k = 0; k < n->numIn; ++k) {
            const sg::SocketRef &in = n->inputSockets[k];
            for (int c = 0; c < 4; ++c) nd.in_default[k][c] = in.data[c];
            if (in.socket && !Link(in.socket, &nd.in_node[k], &nd.in_socket[k])) return -1;
        }
    }
    nodes_[idx] = nd;
    return idx;
}

int SceneDesc::MaterialIndex(const lambda::Material *m) {
    if (!m) return Fail(LGPU_ERR_INVALID_SCENE, "object without a material"), -1;
    auto it = materialIdx_.find(m);
    if (it != materialIdx_.end()) return it->second;
    lgpu_material_desc md{};
    md.bxdf_node = -1;
    md.light = -1;
    if (m->bxdf) {
        sg::Node *n = dynamic_cast<sg::Node *>(m->bxdf);   /* BxDF nodes derive from Node and the BxDF */
        if (!n) return Fail(LGPU_ERR_UNSUPPORTED_NODE, "material BxDF is not a shader-graph node"), -1;
        md.bxdf_node = Node(n);
        if (md.bxdf_node < 0) return -1;
    }
    if (m->light) {
        auto li = lightIdx_.find(m->light);
        if (li == lightIdx_.end()) return Fail(LGPU_ERR_INVALID_SCENE, "material light is not in Scene::lights"), -1;
        md.light = li->second;
    }
    md.medium_interior = Medium(m->mediaBoundary.interior);
    md.medium_exterior = Medium(m->mediaBoundary.exterior);
    if (md.medium_interior < -1 || md.medium_exterior < -1) return -1;
    materials_.push_back(md);
    return materialIdx_[m] = (int)materials_.size() - 1;
}

int SceneDesc::Build(const lambda::Scene &scene) {
    code_ = LGPU_OK;
    err_.clear();
    for (size_t i = 0; i < scene.lights.size(); ++i) lightIdx_[scene.lights[i]] = (int)i;
    /* Scene::objects: meshes, and instances of a proxy over a mesh */
    for (lambda::Object *o : scene.objects) {
        lgpu_object_desc od;
        std::memset(&od, 0, sizeof(od));
        if (auto *m = dynamic_cast<lambda::TriangleMesh *>(o)) {
            od.kind = 0;
            od.mesh = Mesh(m);
            meshObject_[m] = (int)objects_.size();
            od.material = MaterialIndex(o->material);
        } else if (auto *in = dynamic_cast<lambda::Instance *>(o)) {
            lambda::InstanceProxy *p = in->GetProxy();
            auto *pm = p ? dynamic_cast<lambda::TriangleMesh *>(p->GetObject()) : nullptr;
            if (!pm) return Fail(LGPU_ERR_UNSUPPORTED_NODE, "instance whose proxy is not a triangle mesh"), code_;
            od.kind = 1;
            od.mesh = Mesh(pm);
            for (int k = 0; k < 12; ++k) od.xfm[k] = in->xfm[k];
            od.material = MaterialIndex(in->material ? in->material : pm->material);
        } else {
            return Fail(LGPU_ERR_UNSUPPORTED_NODE, "scene object that is neither a TriangleMesh nor an Instance"), code_;
        }
        if (od.material < 0 || code_ != LGPU_OK) return code_ != LGPU_OK ? code_ : LGPU_ERR_INVALID_SCENE;
        objects_.push_back(od);
    }
    /* Scene::lights, in order (the light tree is built over this order) */
    for (lambda::Light *l : scene.lights) {
        lgpu_light_desc ld;
        std::memset(&ld, 0, sizeof(ld));
        ld.object = -1;
        ld.emission_node = -1;
        sg::Socket *emission = nullptr;
        if (auto *ml = dynamic_cast<lambda::MeshLight *>(l)) {
            ld.type = LGPU_LIGHT_MESH;
            auto it = meshObject_.find(&ml->GetMesh());
            if (it == meshObject_.end()) return Fail(LGPU_ERR_UNSUPPORTED_NODE, "mesh light on a mesh that is not a scene object"), code_;
            ld.object = it->second;
            ld.intensity = ml->intensity;
            emission = ml->emission;
        } else if (auto *sl = dynamic_cast<lambda::Spotlight *>(l)) {
            ld.type = LGPU_LIGHT_SPOT;
            copy3(ld.position, sl->position);
            copy3(ld.axis, sl->axis);
            ld.cone_angle = angle_for_cos(sl->cosConeAngle);
            ld.falloff_start = angle_for_cos(sl->cosFalloffStart);
            ld.intensity = sl->intensity;
            emission = sl->emission;
        } else if (auto *pl = dynamic_cast<lambda::PointLight *>(l)) {
            ld.type = LGPU_LIGHT_POINT;
            copy3(ld.position, pl->position);
            ld.intensity = pl->intensity;
            emission = pl->emission;
        } else if (auto *el = dynamic_cast<lambda::EnvironmentLight *>(l)) {
            ld.type = LGPU_LIGHT_ENVIRONMENT;
            const lambda::Texture *t = el->GetRadianceMap().GetRGBTexture();
            if (!t) return Fail(LGPU_ERR_UNSUPPORTED_NODE, "environment light without an RGB texture"), code_;
            const unsigned w = t->GetWidth(), h = t->GetHeight();
            auto *px = new std::vector<float>((size_t)w * h * 3);
            for (unsigned y = 0; y < h; ++y)
                for (unsigned x = 0; x < w; ++x) {
                    const lambda::Colour c = t->GetPixelCoord(x, y);
                    float *p = &(*px)[3 * ((size_t)y * w + x)];
                    p[0] = c.r; p[1] = c.g; p[2] = c.b;
                }
            floats_.emplace_back(px);
            ld.env_texture = px->data();
            ld.env_width = (int32_t)w;
            ld.env_height = (int32_t)h;
            ld.intensity = el->intensity;
            ld.offset[0] = el->offset.x;
            ld.offset[1] = el->offset.y;
        } else {
            return Fail(LGPU_ERR_UNSUPPORTED_NODE, "light type has no GPU implementation"), code_;
        }
        if (ld.type != LGPU_LIGHT_ENVIRONMENT) {
            if (!emission) return Fail(LGPU_ERR_INVALID_SCENE, "light without an emission socket"), code_;
            if (!Link(emission, &ld.emission_node, &ld.emission_socket)) return code_;
        }
        lights_.push_back(ld);
    }
    if (code_ != LGPU_OK) return code_;
    desc_.meshes = meshes_.data(); desc_.num_meshes = (int32_t)meshes_.size();
    desc_.objects = objects_.data(); desc_.num_objects = (int32_t)objects_.size();
    desc_.materials = materials_.data(); desc_.num_materials = (int32_t)materials_.size();
    desc_.nodes = nodes_.data(); desc_.num_nodes = (int32_t)nodes_.size();
    desc_.lights = lights_.data(); desc_.num_lights = (int32_t)lights_.size();
    desc_.media = media_.data(); desc_.num_media = (int32_t)media_.size();
    desc_.textures = textures_.data(); desc_.num_textures = (int32_t)textures_.size();
    desc_.has_volumes = scene.hasVolumes ? 1 : 0;
    desc_.light_strategy = dynamic_cast<const lambda::ManyLightSampler *>(scene.lightSampler) ? LGPU_LIGHT_STRATEGY_TREE
                                                                                             : LGPU_LIGHT_STRATEGY_POWER;
    return LGPU_OK;
}

/* ------------------------------------------------------------------ rendering */

GpuRenderer::~GpuRenderer() {
    if (ctx_) lgpu_destroy(ctx_);
}

int GpuRenderer::Fail(int code, const std::string &msg) {
    err_ = msg;
    return code;
}

int GpuRenderer::Commit(const lambda::Scene &scene) {
    std::lock_guard<std::mutex> lock(mu_);
    if (!ctx_) {
        const int rc = lgpu_create(&ctx_, device_);
        if (rc != LGPU_OK) { ctx_ = nullptr; return Fail(rc, "lgpu_create failed"); }
    }
    SceneDesc sd;
    int rc = sd.Build(scene);
    if (rc != LGPU_OK) return Fail(rc, sd.Error());
    rc = lgpu_scene_commit(ctx_, &sd.Desc());
    if (rc != LGPU_OK) return Fail(rc, lgpu_last_error(ctx_));
    committed_ = true;
    passes_.clear();
    return LGPU_OK;
}

/* lgpu_camera_desc of a Lambda camera (Camera.cpp:7-71). */
int GpuRenderer::Camera(const lambda::Camera *cam, int width, int height, lgpu_camera_desc *c) {
    (void)width; (void)height;
    std::memset(c, 0, sizeof(*c));
    if (!cam) return Fail(LGPU_ERR_INVALID_ARG, "directive without a camera");
    Vec3 x, y, z;
    Real tanFov;
    cam->GetFrame(&x, &y, &z, &tanFov);
    copy3(c->origin, cam->origin);
    copy3(c->x_hat, x);
    copy3(c->y_hat, y);
    copy3(c->z_hat, z);
    c->fov = fov_for_tan(tanFov);
    c->type = LGPU_CAMERA_PINHOLE;
    c->aperture = LGPU_APERTURE_NONE;
    if (const auto *tl = dynamic_cast<const lambda::ThinLensCamera *>(cam)) {
        c->type = LGPU_CAMERA_THIN_LENS;
        c->focal_length = tl->focalLength;
        if (const auto *ca = dynamic_cast<const lambda::CircularAperture *>(tl->aperture)) {
            c->aperture = LGPU_APERTURE_CIRCULAR;
            c->aperture_size = ca->size;
        } else if (const auto *ba = dynamic_cast<const lambda::BladeAperture *>(tl->aperture)) {
            c->aperture = LGPU_APERTURE_BLADE;
            c->aperture_size = ba->size;
            c->blades = (int32_t)ba->blades;
        } else if (tl->aperture) {
            return Fail(LGPU_ERR_UNSUPPORTED_NODE, "masked apertures are committed with the scene's textures; not bound here");
        }
    } else if (const auto *sc = dynamic_cast<const lambda::SphericalCamera *>(cam)) {
        c->type = LGPU_CAMERA_SPHERICAL;
        c->offset_phi = sc->offsetPhi;
        c->offset_theta = sc->offsetTheta;
    } else if (!dynamic_cast<const lambda::PinholeCamera *>(cam)) {
        return Fail(LGPU_ERR_UNSUPPORTED_NODE, "camera type has no GPU implementation");
    }
    return LGPU_OK;
}

/* Integrator selection (Lambda.cpp:356-378) and its bounce limits. */
int GpuRenderer::Options(const lambda::Integrator *integrator, int width, int height, unsigned spp, lgpu_render_opts *o) {
    std::memset(o, 0, sizeof(*o));
    o->width = width;
    o->height = height;
    o->spp = (int32_t)spp;
    o->spectral_mode = LGPU_SPECTRAL_RGB3;   /* Lambda's Spectrum is RGBSpectrum */
    o->kernel_mode = kernelMode;
    o->seed = seed;
    if (const auto *mis = dynamic_cast<const lambda::MISVolumetricPathIntegrator *>(integrator)) {
        o->integrator = LGPU_INTEGRATOR_GPU_MISVOLPATH;
        o->max_bounces = (int32_t)mis->maxBounces;
        o->min_bounces = (int32_t)mis->minBounces;
    } else if (const auto *vp = dynamic_cast<const lambda::VolumetricPathIntegrator *>(integrator)) {
        o->integrator = LGPU_INTEGRATOR_VOLPATH;
        o->max_bounces = (int32_t)vp->maxBounces;
        o->min_bounces = (int32_t)vp->minBounces;
    } else if (const auto *pt = dynamic_cast<const lambda::PathIntegrator *>(integrator)) {
        o->integrator = LGPU_INTEGRATOR_PATH;
        o->max_bounces = (int32_t)pt->maxBounces;
        o->min_bounces = (int32_t)pt->minBounces;
    } else {
        return Fail(LGPU_ERR_UNSUPPORTED_NODE, "integrator has no GPU implementation on this binding");
    }
    return LGPU_OK;
}

/* Sample indices of the next pass on `film`: a directive takes the next spp indices; the tiles of a
 * mosaic pass share one offset, and a tile seen again starts the next pass. */
uint32_t GpuRenderer::NextSampleOffset(const lambda::Film *film, unsigned spp, int tileX, int tileY) {
    FilmPass &p = passes_[film];
    if (tileX < 0) {   /* whole directive */
        p.offset = p.next;
        p.next += spp;
        p.tiles.clear();
        return p.offset;
    }
    const uint64_t key = ((uint64_t)(uint32_t)tileX << 32) | (uint32_t)tileY;
    bool seen = false;
    for (uint64_t t : p.tiles) seen |= t == key;
    if (seen || p.tiles.empty()) {
        p.offset = p.next;
        p.next += spp;
        p.tiles.clear();
    }
    p.tiles.push_back(key);
    return p.offset;
}

int GpuRenderer::RenderDirective(const lambda::RenderDirective &rd) {
    std::lock_guard<std::mutex> lock(mu_);
    if (!ctx_ || !committed_) return Fail(LGPU_ERR_NO_SCENE, "no committed scene");
    if (!rd.film) return Fail(LGPU_ERR_INVALID_ARG, "directive without a film");
    lambda::FilmData &fd = rd.film->filmData;
    const int W = (int)fd.GetWidth(), H = (int)fd.GetHeight();
    lgpu_camera_desc cam;
    lgpu_render_opts o;
    int rc = Camera(rd.camera, W, H, &cam);
    if (rc == LGPU_OK) rc = Options(rd.integrator, W, H, rd.spp, &o);
    if (rc != LGPU_OK) return rc;
    o.sample_offset = NextSampleOffset(rd.film, rd.spp, -1, -1);
    /* the module's film is float4 (r, g, b, samples), added to as Film::AddSample adds */
    std::vector<float> film((size_t)W * H * 4);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const lambda::FilmPixel &p = fd.GetPixelCoord(x, y);
            float *f = &film[4 * ((size_t)y * W + x)];
            f[0] = p.spectrum[0]; f[1] = p.spectrum[1]; f[2] = p.spectrum[2]; f[3] = (float)p.nSamples;
        }
    rc = lgpu_render(ctx_, &cam, &o, film.data());
    if (rc != LGPU_OK) return Fail(rc, lgpu_last_error(ctx_));
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            lambda::FilmPixel &p = fd.GetPixelCoord(x, y);
            const float *f = &film[4 * ((size_t)y * W + x)];
            p.spectrum[0] = f[0]; p.spectrum[1] = f[1]; p.spectrum[2] = f[2];
            p.nSamples += rd.spp;
        }
    return LGPU_OK;
}

int GpuRenderer::RenderTile(const lambda::RenderTile &tile) {
    std::lock_guard<std::mutex> lock(mu_);
    if (!ctx_ || !committed_) return Fail(LGPU_ERR_NO_SCENE, "no committed scene");
    if (!tile.film) return Fail(LGPU_ERR_INVALID_ARG, "tile without a film");
    lambda::FilmData &fd = tile.film->filmData;
    const int W = (int)fd.GetWidth(), H = (int)fd.GetHeight();
    lgpu_camera_desc cam;
    lgpu_render_opts o;
    int rc = Camera(tile.camera, W, H, &cam);
    if (rc == LGPU_OK) rc = Options(tile.integrator.get(), W, H, tile.spp, &o);
    if (rc != LGPU_OK) return rc;
    o.sample_offset = NextSampleOffset(tile.film, tile.spp, (int)tile.x, (int)tile.y);
    const unsigned x1 = std::min<unsigned>(tile.x + tile.w, (unsigned)W), y1 = std::min<unsigned>(tile.y + tile.h, (unsigned)H);
    if (tile.x >= x1 || tile.y >= y1 || tile.spp == 0) return LGPU_OK;
    std::vector<uint64_t> ids;
    ids.reserve((size_t)(x1 - tile.x) * (y1 - tile.y) * tile.spp);
    for (unsigned y = tile.y; y < y1; ++y)
        for (unsigned x = tile.x; x < x1; ++x)
            for (unsigned s = 0; s < tile.spp; ++s) ids.push_back(((uint64_t)y * W + x) * tile.spp + s);
    std::vector<float> out(ids.size() * 4);
    rc = lgpu_render_paths(ctx_, &cam, &o, ids.data(), ids.size(), out.data());
    if (rc != LGPU_OK) return Fail(rc, lgpu_last_error(ctx_));
    size_t k = 0;
    for (unsigned y = tile.y; y < y1; ++y)
        for (unsigned x = tile.x; x < x1; ++x) {
            lambda::FilmPixel &p = fd.GetPixelCoord(x, y);
            for (unsigned s = 0; s < tile.spp; ++s, ++k) {   /* Film::AddSample per sample, in order */
                p.spectrum[0] += out[4 * k];
                p.spectrum[1] += out[4 * k + 1];
                p.spectrum[2] += out[4 * k + 2];
                p.nSamples++;
            }
        }
    return LGPU_OK;
}

namespace {
std::mutex g_tile_mu;
GpuRenderer *g_tile_renderer = nullptr;
int g_tile_error = LGPU_OK;
}  // namespace

void SetTileRenderer(GpuRenderer *renderer) {
    std::lock_guard<std::mutex> lock(g_tile_mu);
    g_tile_renderer = renderer;
    g_tile_error = LGPU_OK;
}

void GpuTileRenderer(const lambda::RenderTile *tile) {
    GpuRenderer *r;
    {
        std::lock_guard<std::mutex> lock(g_tile_mu);
        r = g_tile_renderer;
    }
    const int rc = (r && tile) ? r->RenderTile(*tile) : LGPU_ERR_NO_SCENE;
    if (rc != LGPU_OK) {
        std::lock_guard<std::mutex> lock(g_tile_mu);
        if (g_tile_error == LGPU_OK) g_tile_error = rc;
    }
}

int TileRendererError() {
    std::lock_guard<std::mutex> lock(g_tile_mu);
    return g_tile_error;
}

}  // namespace lambda_gpu
