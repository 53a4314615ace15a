/*
 * lambda_gpu.h -- C ABI of the GB300 (sm_103a) MIS volumetric path-tracing module.
 *
 * The module replaces the per-sample CPU call chain of the Lambda renderer
 *   TileRenderers::UniformSpp (src/render/Render.cpp:43-64)
 *     -> MISVolumetricPathIntegrator::Li (src/integrators/MISVolumetricPathIntegrator.cpp:71-215)
 *       -> Scene::Intersect / IntersectTr / MutualVisibility (src/core/Scene.cpp:28-107, Embree rtcIntersect1/rtcOccluded1)
 *       -> Light / LightSampler / BxDF / Medium / shader-graph sockets
 * with one call that renders a whole film on the GPU.  A GPU integrator needs every path of a
 * frame at once, so the seam is frame granularity: the inputs are exactly the fields of
 * lambda::RenderDirective {film, scene, camera, integrator, sampler, spp} (src/render/Render.h:12-20).
 *
 * The scene is handed over as flat, caller-owned arrays that mirror Lambda's object model:
 *   meshes     <- TriangleMesh buffers        (src/core/TriangleMesh.h:13-83, include/lambda/Lambda.h:67-78)
 *   objects    <- Scene::objects / Instance   (src/core/Scene.h:31, src/core/Instance.h)
 *   materials  <- Material{bxdf, light, mediaBoundary} (src/shading/Material.h:18-32)
 *   nodes      <- ShaderGraph::Node graph     (src/shading/graph/ShaderGraph.h:254-327, include/lambda/Material.h:245-290)
 *   lights     <- Scene::lights               (src/lighting/)
 *   media      <- HomogeneousMedium + HenyeyGreenstein (src/shading/media/)
 * The module copies everything into device memory during lgpu_scene_commit and keeps no host
 * pointer past the call (Lambda's TriangleMesh::AssignData aliases caller arrays instead).
 *
 * Error convention: every entry point returns an lgpu_status; lgpu_last_error() gives a message.
 * No C++ exception crosses this boundary.  Calls on one context must be serialised by the caller.
 */
#ifndef LAMBDA_GPU_H
#define LAMBDA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define LGPU_API __declspec(dllexport)
#else
#define LGPU_API __attribute__((visibility("default")))
#endif

/* ---------------------------------------------------------------- status codes */
typedef enum lgpu_status {
    LGPU_OK = 0,
    LGPU_ERR_INVALID_ARG = 1,
    LGPU_ERR_CUDA = 2,
    LGPU_ERR_OOM = 3,
    LGPU_ERR_INVALID_SCENE = 4,
    LGPU_ERR_UNSUPPORTED_NODE = 5,
    LGPU_ERR_QUEUE_OVERFLOW = 6,
    LGPU_ERR_TIMEOUT = 7,
    LGPU_ERR_NO_SCENE = 8
} lgpu_status;

/* ---------------------------------------------------------------- enums mirrored from Lambda */

/* Integrators.  Values 0-5 are include/lambda/Lambda.h:106-113 (LAMBDA_Integrator); the GPU
 * MIS volumetric path integrator is the added value, the drop-in for
 * MISVolumetricPathIntegrator (src/integrators/MISVolumetricPathIntegrator.h:9-22). */
typedef enum lgpu_integrator {
    LGPU_INTEGRATOR_PATH = 0,
    LGPU_INTEGRATOR_VOLPATH = 1,
    LGPU_INTEGRATOR_DIRECT = 2,
    LGPU_INTEGRATOR_NORMAL = 3,
    LGPU_INTEGRATOR_DEPTH = 4,
    LGPU_INTEGRATOR_AOV = 5,
    LGPU_INTEGRATOR_GPU_MISVOLPATH = 6
} lgpu_integrator;

/* include/lambda/Lambda.h:115-118 */
typedef enum lgpu_light_strategy {
    LGPU_LIGHT_STRATEGY_POWER = 0,   /* PowerLightSampler  src/lighting/LightSampler.cpp:14-35 */
    LGPU_LIGHT_STRATEGY_TREE = 1     /* ManyLightSampler   src/lighting/ManyLightSampler.cpp */
} lgpu_light_strategy;

/* include/lambda/Material.h:232-237 */
typedef enum lgpu_light_type {
    LGPU_LIGHT_POINT = 0,
    LGPU_LIGHT_MESH = 1,
    LGPU_LIGHT_ENVIRONMENT = 2,
    LGPU_LIGHT_SPOT = 3
} lgpu_light_type;

/* Shader node types: same values as LAMBDA_ShaderNodeType, include/lambda/Material.h:245-278. */
typedef enum lgpu_node_type {
    LGPU_NODE_BXDF_MIX = 0,
    LGPU_NODE_BXDF_LAMBERTIAN = 1,
    LGPU_NODE_BXDF_OREN_NAYAR_R = 2,
    LGPU_NODE_BXDF_OREN_NAYAR_T = 3,
    LGPU_NODE_BXDF_MICROFACET_R = 4,
    LGPU_NODE_BXDF_MICROFACET_T = 5,   /* no reference implementation: rejected */
    LGPU_NODE_BXDF_GHOST = 6,
    LGPU_NODE_BXDF_FRESNEL = 7,
    LGPU_NODE_BXDF_SPECULAR_R = 8,
    LGPU_NODE_BXDF_SPECULAR_T = 9,
    LGPU_NODE_SEPARATE_XYZ = 10,
    LGPU_NODE_SEPARATE_RGBA = 11,
    LGPU_NODE_MERGE_XYZ = 12,
    LGPU_NODE_MERGE_RGBA = 13,
    LGPU_NODE_SCALAR = 14,
    LGPU_NODE_VECTOR3 = 15,
    LGPU_NODE_VECTOR2 = 16,
    LGPU_NODE_RGB = 17,
    LGPU_NODE_SPECTRUM = 18,
    LGPU_NODE_BLACKBODY = 19,
    LGPU_NODE_IMAGE_TEXTURE = 20,
    LGPU_NODE_SURFACE_INFO = 21,
    LGPU_NODE_MATHS = 22,
    LGPU_NODE_VECTOR_MATHS = 23,
    LGPU_NODE_DOT_PRODUCT = 24,
    LGPU_NODE_CROSS_PRODUCT = 25,
    LGPU_NODE_VECTOR_MAGNITUDE = 26,
    LGPU_NODE_PERLIN_NOISE = 27,
    LGPU_NODE_VALUE_NOISE = 28,
    LGPU_NODE_OCTAVE_NOISE = 29,
    LGPU_NODE_CHECKER = 30,
    LGPU_NODE_VORONOI = 31,
    LGPU_NODE_TYPE_COUNT = 32
} lgpu_node_type;

/* ScalarOperatorType / VectorOperatorType, src/shading/graph/GraphMaths.h:9-16 */
typedef enum lgpu_maths_op {
    LGPU_MATHS_ADD = 0, LGPU_MATHS_SUBTRACT = 1, LGPU_MATHS_MULTIPLY = 2,
    LGPU_MATHS_DIVIDE = 3, LGPU_MATHS_SQRT = 4, LGPU_MATHS_POWER = 5
} lgpu_maths_op;

/* Microfacet distributions, src/shading/MicrofacetDistribution.h:29-53 */
typedef enum lgpu_distribution { LGPU_DIST_TROWBRIDGE_REITZ = 0, LGPU_DIST_BECKMANN = 1 } lgpu_distribution;

/* Spectral representation.  RGB3 is the reference's `typedef RGBSpectrum Spectrum`
 * (src/core/Spectrum.h:24).  HERO4 carries 4 hero wavelengths per path over 380-720 nm. */
typedef enum lgpu_spectral_mode { LGPU_SPECTRAL_RGB3 = 0, LGPU_SPECTRAL_HERO4 = 1 } lgpu_spectral_mode;

/* ---------------------------------------------------------------- scene description */

/* TriangleMesh buffers (src/core/TriangleMesh.h:15-22).  Vertices are world space for plain mesh
 * objects and object space for meshes used through instances. */
typedef struct lgpu_mesh_desc {
    const float *vertices;      /* 3 * num_vertices */
    const uint32_t *triangles;  /* 3 * num_triangles (v0, v1, v2) */
    const float *normals;       /* optional, 3 * num_vertices; enables smooth shading frames */
    const float *tangents;      /* optional, 4 * num_vertices (xyz + handedness), needed with normals */
    const float *uvs;           /* optional, 2 * num_vertices */
    uint32_t num_vertices;
    uint32_t num_triangles;
} lgpu_mesh_desc;

/* One entry of Scene::objects.  kind 0 = the mesh itself (TriangleMesh object), kind 1 = an
 * Instance of the mesh used as an InstanceProxy, placed by a column-major 3x3 + translation
 * affine (affine3<Real>::xfm layout, src/maths/affine3.h:18-30). */
typedef struct lgpu_object_desc {
    int32_t mesh;
    int32_t kind;
    int32_t material;
    int32_t pad;
    float xfm[12];
} lgpu_object_desc;

/* Material{bxdf, light, mediaBoundary} (src/shading/Material.h:18-24).  bxdf_node = -1 is a
 * null surface (a pure media boundary, skipped by IntersectTr).  light = index into lights or -1. */
typedef struct lgpu_material_desc {
    int32_t bxdf_node;
    int32_t light;
    int32_t medium_interior;
    int32_t medium_exterior;
} lgpu_material_desc;

#define LGPU_NODE_MAX_INPUTS 4

/* One shader node.  Input i is linked to output socket in_socket[i] of node in_node[i] when
 * in_node[i] >= 0, else it reads its SocketRef default value in_default[i] (SocketRef::data,
 * ShaderGraph.h:254-284).  params hold the node's own constants:
 *   SCALAR: value | VECTOR2/VECTOR3/RGB: components | SPECTRUM: rgb of a constant spectrum
 *   BLACKBODY: samples | PERLIN/VALUE/CHECKER/VORONOI: scale | OCTAVE: scale, octaves
 *   MICROFACET_R: distribution, fresnel etaT | SPECULAR_R: fresnel etaT | SPECULAR_T: etaT
 * op: lgpu_maths_op for MATHS / VECTOR_MATHS.
 * OCTAVE_NOISE takes its inner noise node (Octave::noise) as in_node[0]. */
typedef struct lgpu_node_desc {
    int32_t type;
    int32_t op;
    float params[4];
    int32_t in_node[LGPU_NODE_MAX_INPUTS];
    int32_t in_socket[LGPU_NODE_MAX_INPUTS];
    float in_default[LGPU_NODE_MAX_INPUTS][4];
} lgpu_node_desc;

/* Lights (src/lighting/).  MESH: object = emitting object, emission = node/socket
 * (MeshLight::emission), intensity.  POINT/SPOT: position, axis, cone/falloff angles in radians,
 * emission socket, intensity.  ENVIRONMENT: RGB float texture env_width x env_height, scanline
 * rows, equirectangular (EnvironmentLight.cpp:7-22), intensity and offset. */
typedef struct lgpu_light_desc {
    int32_t type;
    int32_t object;
    int32_t emission_node;
    int32_t emission_socket;
    float intensity;
    float position[3];
    float axis[3];
    float cone_angle;
    float falloff_start;
    float offset[2];
    int32_t env_width;
    int32_t env_height;
    int32_t pad;
    const float *env_texture;
} lgpu_light_desc;

/* HomogeneousMedium(sigmaA, sigmaS) + HenyeyGreenstein(g) (src/shading/media/HomogeneousMedium.h). */
typedef struct lgpu_medium_desc {
    float sigma_a[3];
    float sigma_s[3];
    float g;
    float pad;
} lgpu_medium_desc;

/* Image texture (texture_t<Colour>, src/image/Texture.h): width * height RGBA float texels in
 * scanline-row order (texel (x, y) at (y * width + x) * 4), sampled by IMAGE_TEXTURE nodes
 * (params[0] = texture index) with GetPixelUVBilinear at fract(uv). */
typedef struct lgpu_texture_desc {
    const float *rgba;
    int32_t width, height;
    int32_t aperture_mask;    /* nonzero: also build the sampling distribution of |red| that a masked
                               * aperture over this texture draws from (MaskedAperture::InitDistribution,
                               * src/camera/Aperture.cpp:38-51), at scene commit */
    int32_t pad;
} lgpu_texture_desc;

typedef struct lgpu_scene_desc {
    const lgpu_mesh_desc *meshes;       int32_t num_meshes;
    const lgpu_object_desc *objects;    int32_t num_objects;
    const lgpu_material_desc *materials; int32_t num_materials;
    const lgpu_node_desc *nodes;        int32_t num_nodes;
    const lgpu_light_desc *lights;      int32_t num_lights;
    const lgpu_medium_desc *media;      int32_t num_media;
    int32_t has_volumes;      /* Scene::hasVolumes (src/core/Scene.h:36) */
    int32_t light_strategy;   /* lgpu_light_strategy */
    const lgpu_texture_desc *textures; int32_t num_textures;
} lgpu_scene_desc;

/* Cameras (src/camera/Camera.cpp:7-71) and apertures (src/camera/Aperture.cpp:10-51): origin, the
 * three axes and the field of view; aspect = height / width as in Camera::Camera.  A sample's
 * random numbers: pixel jitter x, y (Render.cpp:55-56), then the aperture's (blade: one for the
 * blade, two for the point; circular and masked: two), then the integrator's. */
typedef enum lgpu_camera_type {
    LGPU_CAMERA_PINHOLE = 0,      /* PinholeCamera::GenerateRay (Camera.cpp:41-44) */
    LGPU_CAMERA_THIN_LENS = 1,    /* ThinLensCamera::GenerateRay (Camera.cpp:53-58) */
    LGPU_CAMERA_SPHERICAL = 2     /* SphericalCamera::GenerateRay (Camera.cpp:66-71) */
} lgpu_camera_type;
typedef enum lgpu_aperture_type {
    LGPU_APERTURE_NONE = 0,       /* thin lens without an aperture: ap = (0, 0), no random numbers */
    LGPU_APERTURE_CIRCULAR = 1,   /* CircularAperture::Sample_p (Aperture.cpp:25-27) */
    LGPU_APERTURE_BLADE = 2,      /* BladeAperture::Sample_p (Aperture.cpp:10-19) */
    LGPU_APERTURE_MASKED = 3      /* MaskedAperture::Sample_p (Aperture.cpp:33-36) */
} lgpu_aperture_type;
typedef struct lgpu_camera_desc {
    float origin[3];
    float x_hat[3];
    float y_hat[3];
    float z_hat[3];
    float fov;
    int32_t type;             /* lgpu_camera_type */
    float focal_length;       /* thin lens: ThinLensCamera::focalLength (the C API's default is 1) */
    int32_t aperture;         /* thin lens: lgpu_aperture_type (the C API's default: circular, size 0) */
    float aperture_size;      /* Aperture::size */
    int32_t blades;           /* BladeAperture::blades (>= 3) */
    int32_t aperture_mask;    /* masked: index of a scene texture committed with aperture_mask set */
    float offset_phi, offset_theta;   /* spherical: SphericalCamera::offsetPhi / offsetTheta */
} lgpu_camera_desc;

/* RenderDirective fields (src/render/Render.h:12-20) plus the GPU-side knobs. */
typedef struct lgpu_render_opts {
    int32_t width;
    int32_t height;
    int32_t spp;
    int32_t max_bounces;      /* MISVolumetricPathIntegrator::maxBounces */
    int32_t min_bounces;      /* MISVolumetricPathIntegrator::minBounces (Russian roulette start) */
    int32_t integrator;       /* lgpu_integrator */
    int32_t spectral_mode;    /* lgpu_spectral_mode */
    uint32_t seed;            /* counter-based RNG key */
    uint32_t sample_offset;   /* first sample index: resume = same seed, offset = samples done */
    int32_t block_size;       /* threads per block of the wavefront trace kernel: 64, 128, 256 or 512 (0 = 64) */
    int32_t kernel_mode;      /* lgpu_kernel_mode */
    int32_t pool_slots;       /* wavefront path-slot pool size, 0 = default (8 Mi slots) */
} lgpu_render_opts;

/* Execution scheme of one render.  Both produce the same paths (same random-number order). */
typedef enum lgpu_kernel_mode {
    LGPU_KERNEL_AUTO = 0,        /* the lgpu_autotune result if there is one, else wavefront */
    LGPU_KERNEL_MEGAKERNEL = 1,  /* one thread runs a whole path */
    LGPU_KERNEL_WAVEFRONT = 2,   /* path state machine + separate traversal kernels */
    LGPU_KERNEL_WAVEFRONT_GRAPH = 3  /* the same kernels over resident grids, reading their queue sizes
                                      * on the device; the bounce loop is a CUDA graph replayed by
                                      * the host (no per-launch timing in lgpu_stats) */
} lgpu_kernel_mode;

/* Per-render statistics.  Traversal counters are filled only by lgpu_render_count. */
typedef struct lgpu_stats {
    double last_render_ms;
    uint64_t paths;
    uint64_t rays;            /* closest-hit + occlusion queries issued */
    uint64_t nodes_visited;   /* BVH node fetches over all queries */
    uint64_t tris_tested;     /* triangle records fetched over all queries */
    uint64_t bvh_nodes;
    uint64_t bvh_bytes;
    uint64_t tri_bytes;
    uint32_t node_bytes;      /* size of one BVH node record */
    uint32_t tri_record_bytes;/* size of one triangle record */
    uint64_t device_bytes;    /* device memory held by the committed scene */
    /* wavefront breakdown of the last render (lgpu_render, lgpu_render_device, lgpu_render_paths),
     * timed with CUDA events recorded on the render's stream around every launch: */
    double trace_ms, shade_ms, spawn_ms;
    uint32_t iterations;      /* trace + resume rounds of the last wavefront render */
    uint32_t pool_slots;
    double stage_ms[6];       /* resume time per stage: primary hit, surface extension, null-surface
                               * extension, medium extension, visibility, transmittance step */
    uint64_t resumed[6];      /* paths resumed per stage */
    uint64_t traced;          /* ray queries answered by the trace kernel */
    uint64_t spawned;         /* paths started */
    uint64_t launches;        /* kernels launched by the last render */
    double bvh_build_ms;      /* device time of the last commit's BVH builds (device builder only) */
} lgpu_stats;

typedef struct lgpu_context lgpu_context;

/* Create a context on CUDA device `device`.  Replaces lambdaCreateDevice
 * (include/lambda/Lambda.h:37) for the GPU path. */
LGPU_API int lgpu_create(lgpu_context **out, int device);

/* Free the context and every device buffer it owns (lambdaReleaseDevice, Lambda.h:40). */
LGPU_API void lgpu_destroy(lgpu_context *ctx);

/* Message of the last failed call on ctx (never NULL). */
LGPU_API const char *lgpu_last_error(const lgpu_context *ctx);

/* Compile and upload a scene: BVH build, light-tree build, shader-graph bytecode.
 * Replaces Scene::AddObject + Scene::Commit (src/core/Scene.cpp:18-26, 114-121) and
 * LightSampler::Commit (ManyLightSampler.cpp:37-44). */
LGPU_API int lgpu_scene_commit(lgpu_context *ctx, const lgpu_scene_desc *scene);

/* Compile and validate a scene on the host only, without a GPU or a context (the host half of
 * lgpu_scene_commit).  Writes a one-line report (counts, or the first error) into `report`
 * (NUL-terminated, truncated to report_size).  Returns the status lgpu_scene_commit would. */
LGPU_API int lgpu_scene_check(const lgpu_scene_desc *scene, char *report, size_t report_size);

/* Render `opts->spp` samples per pixel and ADD them to the host film `film_rgbn`
 * (width*height float4: summed RGB + sample count), the way Film::AddSample accumulates
 * (src/camera/Film.h:30-33).  Host buffers: the call copies the film to and from the device.
 * Replaces MosaicRenderer::Render over TileRenderers::UniformSpp (src/render/Render.cpp:43-64). */
LGPU_API int lgpu_render(lgpu_context *ctx, const lgpu_camera_desc *camera,
                         const lgpu_render_opts *opts, float *film_rgbn);

/* Same, on device memory: film_rgbn_dev is a device float4 film that the render adds into;
 * path_out_dev (optional, may be NULL) receives the radiance of every path, indexed
 * (y * width + x) * spp + s, as float4.  stream = cudaStream_t or NULL. */
LGPU_API int lgpu_render_device(lgpu_context *ctx, const lgpu_camera_desc *camera,
                                const lgpu_render_opts *opts, float *film_rgbn_dev,
                                float *path_out_dev, void *stream);

/* Render a chosen list of paths (path index = (y * width + x) * spp + s) and write their
 * radiance to path_out_host (n * 4 floats).  Used for per-path parity checks. */
LGPU_API int lgpu_render_paths(lgpu_context *ctx, const lgpu_camera_desc *camera,
                               const lgpu_render_opts *opts, const uint64_t *path_ids,
                               uint64_t n, float *path_out_host);

/* Render once with in-kernel traversal counters on (nodes, triangles, rays); the counts land in
 * lgpu_get_stats.  The film is not touched. */
LGPU_API int lgpu_render_count(lgpu_context *ctx, const lgpu_camera_desc *camera,
                               const lgpu_render_opts *opts);

/* Closest-hit queries for a batch of rays (Scene::Intersect, src/core/Scene.cpp:28-43).
 * rays: n * 8 floats (ox, oy, oz, tnear, dx, dy, dz, tfar), device pointer.  hits: n * 4 words
 * (t as float bits, primId, objectId, instance-or-~0), device pointer.  u, v are written to
 * uv_out (n * 2 floats, device, optional). */
LGPU_API int lgpu_intersect(lgpu_context *ctx, const float *rays_dev, uint32_t *hits_dev,
                            float *uv_out_dev, uint64_t n, void *stream);

/* Film::ToRGBTexture (src/camera/Film.cpp:11-24) on the device: rgba_dev[i] = (film rgb / sample
 * count, 1) for n_px float4 pixels (DEVICE buffers); pixels without samples give black. */
LGPU_API int lgpu_film_resolve(const float *film_dev, float *rgba_dev, uint64_t n_px, void *stream);

/* GPU counterpart of ProgressiveRender::RunPass (src/render/ProgressiveRender.cpp:40-58): `passes`
 * renders of opts->spp samples per pixel, each with the next opts->spp sample indices
 * (sample_offset advanced per pass), added into the DEVICE film; after every pass the film is
 * resolved into rgba_dev (optional) as UpdateOutputTexture does.  Returns when done. */
LGPU_API int lgpu_render_progressive(lgpu_context *ctx, const lgpu_camera_desc *camera, const lgpu_render_opts *opts,
                                     int32_t passes, float *film_dev, float *rgba_dev, void *stream);

/* One view of a batched render: a camera with its own film size, samples per pixel, depth and seed.
 * film_dev is the view's DEVICE film (width * height float4: r, g, b, sample count), which the render
 * adds into as Film::AddSample does (src/camera/Film.h:30-33). */
typedef struct lgpu_view_desc {
    lgpu_camera_desc camera;
    int32_t width, height, spp, max_bounces;
    uint32_t seed, sample_offset;
    float *film_dev;
} lgpu_view_desc;

/* Render many views of the committed scene in one wavefront (no counterpart in the reference, which
 * renders one RenderDirective at a time).  Consecutive views are packed into chunks of at most
 * 2^28 paths that share one pool of path slots, so views too small to fill the GPU are rendered
 * together; every path gives the same result as in a single-view render (same random numbers), so
 * each view's film equals the one lgpu_render_device would produce.  opts supplies the shared
 * settings (integrator, min_bounces, spectral_mode, kernel_mode, pool_slots, block_size); its width,
 * height, spp, max_bounces, seed and sample_offset are ignored in favour of each view's.
 * kernel_mode MEGAKERNEL renders the views one launch at a time instead.  Work is issued on
 * `stream`; the call returns when every film is complete. */
LGPU_API int lgpu_render_batch(lgpu_context *ctx, const lgpu_view_desc *views, int32_t n_views,
                               const lgpu_render_opts *opts, void *stream);

/* Result of lgpu_autotune: the execution scheme chosen for a workload. */
typedef struct lgpu_tuning {
    int32_t kernel_mode;      /* LGPU_KERNEL_MEGAKERNEL, _WAVEFRONT or _WAVEFRONT_GRAPH */
    int32_t pool_slots;       /* wavefront path-slot pool */
    int32_t block_size;       /* trace-kernel threads per block */
    int32_t pad;
    double mpaths_per_s;      /* throughput of the chosen scheme on the probe */
    int32_t tried;            /* candidate schemes timed */
    int32_t pad2;
} lgpu_tuning;

/* Autotuner (no counterpart in the reference): times the candidate schemes -- megakernel,
 * host-driven wavefront and graph-replayed wavefront, path-slot pools of 2^18, 2^20 and 2^22, trace
 * blocks of 64 to 512 threads -- on a probe of the given views rendered at min(spp, probe_spp)
 * samples per pixel into scratch films (the views' own films are not touched), keeps the fastest in
 * the context for every later render with kernel_mode AUTO (explicit pool_slots / block_size in
 * those opts still win) and writes it to *out.  Allocates its scratch films for the duration of
 * the call. */
LGPU_API int lgpu_autotune(lgpu_context *ctx, const lgpu_view_desc *views, int32_t n_views,
                           const lgpu_render_opts *opts, int32_t probe_spp, lgpu_tuning *out);

/* Parameters the path-replay adjoint differentiates (any of them may be -1: not differentiated). */
typedef struct lgpu_adjoint_desc {
    int32_t tex_material;     /* material whose Lambertian albedo reads an IMAGE_TEXTURE ... */
    int32_t texture;          /* ... of this scene texture: per-texel gradients */
    int32_t rough_material;   /* material whose first BSDF leaf's roughness gets a gradient */
    int32_t medium;           /* homogeneous medium whose (grey) sigma_a and sigma_s get gradients */
} lgpu_adjoint_desc;

/* Path-replay adjoint of one render (no counterpart in the reference, which has no derivatives).
 * For the image I = lgpu_render_device(camera, opts) (pixel means over opts->spp samples) and a
 * loss with dloss_dev = dLoss/dI (DEVICE, width * height float4, rgb used), ADDS dLoss/dtheta into
 * grad_texture_dev (DEVICE, texture width * height float4, rgb) and grad_scalars_dev (DEVICE,
 * 3 floats: roughness, sigma_a, sigma_s).  Every path is recomputed with the same random numbers
 * as the forward render (nothing is stored between the passes); sampling decisions are treated
 * as fixed.  RGB3 only; the forward render must use the same opts and seed.  Returns when done. */
LGPU_API int lgpu_adjoint(lgpu_context *ctx, const lgpu_camera_desc *camera, const lgpu_render_opts *opts,
                          const lgpu_adjoint_desc *params, const float *dloss_dev, float *grad_texture_dev,
                          float *grad_scalars_dev, void *stream);

/* Fixed-scratch variant of lgpu_render_paths, for callers that must not allocate.
 * No counterpart in the reference, which renders on the CPU.
 *
 * Who needs it: a host that drives the renderer from a region where allocating device memory is
 * not allowed or not affordable, e.g. a caller whose device memory is fully handed to another
 * allocator (a framework's caching pool), or a frame loop that cannot take the implicit
 * device-wide synchronisation of cudaMalloc / cudaFree.  lgpu_render_paths grows buffers inside
 * the context on demand; this entry point never does.
 *
 * Same paths, same random-number order and the same per-path result as lgpu_render_paths, but:
 *   - path_ids_dev (n ids, uint64) and path_out_dev (n x 4 floats: radiance, random numbers
 *     drawn) are DEVICE buffers owned by the caller; ids must be < width * height * spp (larger
 *     ids are not detected and give unspecified values, no out-of-bounds access);
 *   - the working memory is one array of at most LGPU_NOALLOC_SCRATCH_BYTES compiled into the
 *     library (one copy per device), holding a pool of at most LGPU_NOALLOC_MAX_SLOTS paths in
 *     flight; any n streams through that pool.  opts->pool_slots = 0 uses the whole pool, values
 *     above LGPU_NOALLOC_MAX_SLOTS are rejected with LGPU_ERR_INVALID_ARG;
 *   - the wavefront kernels always run, and they are the MIS volumetric integrator: kernel_mode
 *     MEGAKERNEL and every integrator other than LGPU_INTEGRATOR_GPU_MISVOLPATH are rejected with
 *     LGPU_ERR_INVALID_ARG; no traversal counters (lgpu_get_stats reports this call's paths,
 *     iterations, queries and launches, without stage timings).
 * The call issues its work on `stream` and returns when it has finished.  The first call on a
 * device also looks up the array's address (cudaGetSymbolAddress) and may make the driver load
 * the kernels' code, so make it before any stream capture or allocation-free region starts.
 * The scratch and its counters (which must start at zero) are cleared by the call itself.
 * The array is shared by every context on a device: overlapping calls would race on it, so calls
 * on one device are serialised by a lock inside the library; do not issue them from code that
 * cannot block.  Error paths store their message in the context (host memory). */
#define LGPU_NOALLOC_MAX_SLOTS 16384
#define LGPU_NOALLOC_SCRATCH_BYTES (16u << 20)
LGPU_API int lgpu_render_paths_noalloc(lgpu_context *ctx, const lgpu_camera_desc *camera,
                                       const lgpu_render_opts *opts, const uint64_t *path_ids_dev,
                                       uint64_t n, float *path_out_dev, void *stream);

LGPU_API int lgpu_get_stats(const lgpu_context *ctx, lgpu_stats *out);

/* Version string of the module. */
LGPU_API const char *lgpu_version(void);

/* Read bandwidth of this device for a buffer of `bytes` (rounded down to 16 B): the buffer is
 * allocated, zeroed and read once to warm the caches, then read `reps` times in one launch of a
 * read-only kernel of the module (loads cached in L2 only), timed with CUDA events;
 * *gbs = bytes * reps / time.
 * A buffer well inside L2 (e.g. 32 MiB) gives the L2 read peak that the traversal kernels are
 * compared against; one well beyond it gives the HBM read rate.  No counterpart in the reference. */
LGPU_API int lgpu_probe_bandwidth(lgpu_context *ctx, uint64_t bytes, int32_t reps, double *gbs);

/* BVH builder of the following commits: LGPU_BVH_BUILD_HOST (default) builds binned-SAH trees on
 * the host; LGPU_BVH_BUILD_DEVICE builds linear BVHs on the device (Morton order, radix tree,
 * bottom-up boxes; one primitive per leaf) in milliseconds, at some cost in traversal.  Both give
 * the same node layout and the same hits.  Replaces rtcCommitScene's build (src/core/Scene.cpp:18-26)
 * for the GPU path; lgpu_stats::bvh_build_ms reports the device build time. */
typedef enum lgpu_bvh_build { LGPU_BVH_BUILD_HOST = 0, LGPU_BVH_BUILD_DEVICE = 1 } lgpu_bvh_build;
LGPU_API int lgpu_set_bvh_builder(lgpu_context *ctx, int32_t builder);

#ifdef __cplusplus
}
#endif

#endif /* LAMBDA_GPU_H */
