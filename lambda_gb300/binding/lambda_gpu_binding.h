/*
 * Lambda-side binding of the GPU path tracer (include/lambda_gpu.h): the code a Lambda maintainer
 * adds so that a lambda::Scene renders on the GPU when the integrator enum selects it.
 *
 * It compiles against Lambda's own headers (the renderer's src/ tree) plus read-only accessors
 * that the binding needs because the state is not public there, and one fix: output sockets must
 * keep the node that owns them (Socket::node, ShaderGraph.h:72-76), which Node's constructor sets
 * and the MAKE_SOCKET / MAKE_BXDF_SOCKET initialisers reset to null.  The accessors:
 *   Camera::GetFrame(x, y, z, tanFov)     the camera frame (camera/Camera.h:42-44)
 *   Instance::GetProxy(), InstanceProxy::GetObject()   instanced mesh (core/Instance.h:12-28)
 *   EnvironmentLight::GetRadianceMap(), TextureAdapter::GetRGBTexture()   the environment texture
 *
 *   lambda_gpu::SceneDesc     lambda::Scene -> lgpu_scene_desc, owning every array it points to
 *                             (Scene.h:31-36 objects/lights/lightSampler/hasVolumes, TriangleMesh,
 *                             Instance, Material, the shader-graph nodes, lights and media)
 *   lambda_gpu::GpuRenderer   one lgpu_context with one committed scene; renders a RenderDirective
 *                             (render/Render.h:12-20) into its Film as Film::AddSample adds
 *   lambda_gpu::GpuTileRenderer   a TileRenderer (render/Render.h:39) for RenderMosaic,
 *                             MosaicRenderer and ProgressiveRender: renders one tile's pixels
 *
 * Errors follow the module's convention: an lgpu status code, and a message from LastError().
 * Scene, camera and film objects are only read during a call; nothing keeps pointers to them.
 */
#pragma once
#include <cstdint>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include <camera/Camera.h>
#include <camera/Film.h>
#include <core/Scene.h>
#include <core/TriangleMesh.h>
#include <image/Texture.h>
#include <integrators/Integrator.h>
#include <render/Render.h>
#include <shading/Material.h>
#include <shading/graph/ShaderGraph.h>
#include <shading/media/Media.h>

#include "../../include/lambda_gpu.h"

namespace lambda_gpu {

/* The LAMBDA_Integrator value (include/lambda/Lambda.h:106-113) that selects the GPU integrator. */
constexpr int LAMBDA_INTEGRATOR_GPU_MISVOLPATH = LGPU_INTEGRATOR_GPU_MISVOLPATH;

class SceneDesc {
  public:
    /* Translate `scene`.  Returns LGPU_OK, LGPU_ERR_UNSUPPORTED_NODE (a node, light, object or
     * medium kind the GPU module does not implement) or LGPU_ERR_INVALID_SCENE. */
    int Build(const lambda::Scene &scene);
    const lgpu_scene_desc &Desc() const { return desc_; }
    const std::string &Error() const { return err_; }

  private:
    int Mesh(const lambda::TriangleMesh *m);
    int MaterialIndex(const lambda::Material *m);
    int Medium(const lambda::Medium *m);
    int Node(lambda::ShaderGraph::Node *n);
    int Texture(const lambda::Texture *t, bool apertureMask);
    bool Link(lambda::ShaderGraph::Socket *s, int32_t *node, int32_t *socket);
    bool Fail(int code, const std::string &msg);

    lgpu_scene_desc desc_{};
    std::string err_;
    int code_ = LGPU_OK;
    std::vector<lgpu_mesh_desc> meshes_;
    std::vector<lgpu_object_desc> objects_;
    std::vector<lgpu_material_desc> materials_;
    std::vector<lgpu_node_desc> nodes_;
    std::vector<lgpu_light_desc> lights_;
    std::vector<lgpu_medium_desc> media_;
    std::vector<lgpu_texture_desc> textures_;
    std::vector<std::unique_ptr<std::vector<float>>> floats_;
    std::vector<std::unique_ptr<std::vector<uint32_t>>> words_;
    std::unordered_map<const void *, int> meshIdx_, materialIdx_, mediumIdx_, nodeIdx_, textureIdx_, lightIdx_;
    std::unordered_map<const void *, int> meshObject_;   /* kind-0 mesh -> its object index */
};

class GpuRenderer {
  public:
    explicit GpuRenderer(int device = 0) : device_(device) {}
    ~GpuRenderer();
    GpuRenderer(const GpuRenderer &) = delete;
    GpuRenderer &operator=(const GpuRenderer &) = delete;

    /* Translate and upload the scene (lgpu_scene_commit).  Call again after the scene changes. */
    int Commit(const lambda::Scene &scene);

    /* Render a whole directive: rd.spp samples per pixel of rd.film with the directive's camera
     * and integrator (MISVolumetricPathIntegrator, VolumetricPathIntegrator or PathIntegrator, with
     * their maxBounces / minBounces), added into rd.film.  Each call on the same film continues
     * with the next sample indices. */
    int RenderDirective(const lambda::RenderDirective &rd);

    /* One tile of a mosaic (TileRenderers::UniformSpp, Render.cpp:20-39, on the GPU): tile->spp
     * samples for each pixel of the tile, added into tile->film sample by sample. */
    int RenderTile(const lambda::RenderTile &tile);

    const char *LastError() const { return err_.c_str(); }
    lgpu_context *Context() const { return ctx_; }
    uint32_t seed = 1;               /* counter-based RNG key (lgpu_render_opts::seed) */
    int32_t kernelMode = LGPU_KERNEL_AUTO;

  private:
    int Camera(const lambda::Camera *cam, int width, int height, lgpu_camera_desc *out);
    int Options(const lambda::Integrator *integrator, int width, int height, unsigned spp, lgpu_render_opts *out);
    int Fail(int code, const std::string &msg);
    uint32_t NextSampleOffset(const lambda::Film *film, unsigned spp, int tileX, int tileY);

    int device_;
    lgpu_context *ctx_ = nullptr;
    bool committed_ = false;
    std::string err_;
    std::mutex mu_;
    /* sample indices already used per film, and the tiles done in the current mosaic pass */
    struct FilmPass { uint32_t offset = 0; uint32_t next = 0; std::vector<uint64_t> tiles; };
    std::unordered_map<const void *, FilmPass> passes_;
};

/* TileRenderer (render/Render.h:39): renders the tile with the GpuRenderer set by
 * SetTileRenderer; RenderMosaic / MosaicRenderer / ProgressiveRender call it once per tile and
 * pass.  Errors are reported through TileRendererError() (the TileRenderer signature has no
 * return value). */
void SetTileRenderer(GpuRenderer *renderer);
void GpuTileRenderer(const lambda::RenderTile *tile);
int TileRendererError();

}  // namespace lambda_gpu
