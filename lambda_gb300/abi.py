"""ctypes mirror of include/lambda_gpu.h (structs, enums) shared by the Python host side."""
import ctypes as C

# lgpu_status
OK, ERR_INVALID_ARG, ERR_CUDA, ERR_OOM, ERR_INVALID_SCENE, ERR_UNSUPPORTED_NODE, \
    ERR_QUEUE_OVERFLOW, ERR_TIMEOUT, ERR_NO_SCENE = range(9)

# lgpu_integrator
INTEGRATOR_PATH, INTEGRATOR_VOLPATH, INTEGRATOR_DIRECT, INTEGRATOR_NORMAL, INTEGRATOR_DEPTH, \
    INTEGRATOR_AOV, INTEGRATOR_GPU_MISVOLPATH = range(7)
LIGHT_STRATEGY_POWER, LIGHT_STRATEGY_TREE = 0, 1
LIGHT_POINT, LIGHT_MESH, LIGHT_ENVIRONMENT, LIGHT_SPOT = 0, 1, 2, 3
SPECTRAL_RGB3, SPECTRAL_HERO4 = 0, 1
DIST_TROWBRIDGE_REITZ, DIST_BECKMANN = 0, 1
MATHS_ADD, MATHS_SUBTRACT, MATHS_MULTIPLY, MATHS_DIVIDE, MATHS_SQRT, MATHS_POWER = range(6)

NODE = dict(
    BXDF_MIX=0, BXDF_LAMBERTIAN=1, BXDF_OREN_NAYAR_R=2, BXDF_OREN_NAYAR_T=3, BXDF_MICROFACET_R=4,
    BXDF_MICROFACET_T=5, BXDF_GHOST=6, BXDF_FRESNEL=7, BXDF_SPECULAR_R=8, BXDF_SPECULAR_T=9,
    SEPARATE_XYZ=10, SEPARATE_RGBA=11, MERGE_XYZ=12, MERGE_RGBA=13, SCALAR=14, VECTOR3=15, VECTOR2=16,
    RGB=17, SPECTRUM=18, BLACKBODY=19, IMAGE_TEXTURE=20, SURFACE_INFO=21, MATHS=22, VECTOR_MATHS=23,
    DOT_PRODUCT=24, CROSS_PRODUCT=25, VECTOR_MAGNITUDE=26, PERLIN_NOISE=27, VALUE_NOISE=28,
    OCTAVE_NOISE=29, CHECKER=30, VORONOI=31)

F32P = C.POINTER(C.c_float)
U32P = C.POINTER(C.c_uint32)


class MeshDesc(C.Structure):
    _fields_ = [("vertices", F32P), ("triangles", U32P), ("normals", F32P), ("tangents", F32P),
                ("uvs", F32P), ("num_vertices", C.c_uint32), ("num_triangles", C.c_uint32)]


class ObjectDesc(C.Structure):
    _fields_ = [("mesh", C.c_int32), ("kind", C.c_int32), ("material", C.c_int32), ("pad", C.c_int32),
                ("xfm", C.c_float * 12)]


class MaterialDesc(C.Structure):
    _fields_ = [("bxdf_node", C.c_int32), ("light", C.c_int32), ("medium_interior", C.c_int32),
                ("medium_exterior", C.c_int32)]


class NodeDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("op", C.c_int32), ("params", C.c_float * 4),
                ("in_node", C.c_int32 * 4), ("in_socket", C.c_int32 * 4),
                ("in_default", (C.c_float * 4) * 4)]


class LightDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("object", C.c_int32), ("emission_node", C.c_int32),
                ("emission_socket", C.c_int32), ("intensity", C.c_float), ("position", C.c_float * 3),
                ("axis", C.c_float * 3), ("cone_angle", C.c_float), ("falloff_start", C.c_float),
                ("offset", C.c_float * 2), ("env_width", C.c_int32), ("env_height", C.c_int32),
                ("pad", C.c_int32), ("env_texture", F32P)]


class MediumDesc(C.Structure):
    _fields_ = [("sigma_a", C.c_float * 3), ("sigma_s", C.c_float * 3), ("g", C.c_float), ("pad", C.c_float)]


class TextureDesc(C.Structure):
    _fields_ = [("rgba", F32P), ("width", C.c_int32), ("height", C.c_int32), ("aperture_mask", C.c_int32),
                ("pad", C.c_int32)]


class SceneDesc(C.Structure):
    _fields_ = [("meshes", C.POINTER(MeshDesc)), ("num_meshes", C.c_int32),
                ("objects", C.POINTER(ObjectDesc)), ("num_objects", C.c_int32),
                ("materials", C.POINTER(MaterialDesc)), ("num_materials", C.c_int32),
                ("nodes", C.POINTER(NodeDesc)), ("num_nodes", C.c_int32),
                ("lights", C.POINTER(LightDesc)), ("num_lights", C.c_int32),
                ("media", C.POINTER(MediumDesc)), ("num_media", C.c_int32),
                ("has_volumes", C.c_int32), ("light_strategy", C.c_int32),
                ("textures", C.POINTER(TextureDesc)), ("num_textures", C.c_int32)]


CAMERA_PINHOLE, CAMERA_THIN_LENS, CAMERA_SPHERICAL = 0, 1, 2
APERTURE_NONE, APERTURE_CIRCULAR, APERTURE_BLADE, APERTURE_MASKED = 0, 1, 2, 3


class CameraDesc(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("x_hat", C.c_float * 3), ("y_hat", C.c_float * 3),
                ("z_hat", C.c_float * 3), ("fov", C.c_float), ("type", C.c_int32),
                ("focal_length", C.c_float), ("aperture", C.c_int32), ("aperture_size", C.c_float),
                ("blades", C.c_int32), ("aperture_mask", C.c_int32), ("offset_phi", C.c_float),
                ("offset_theta", C.c_float)]


class ViewDesc(C.Structure):
    _fields_ = [("camera", CameraDesc), ("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32),
                ("max_bounces", C.c_int32), ("seed", C.c_uint32), ("sample_offset", C.c_uint32),
                ("film_dev", C.c_void_p)]


class Tuning(C.Structure):
    _fields_ = [("kernel_mode", C.c_int32), ("pool_slots", C.c_int32), ("block_size", C.c_int32), ("pad", C.c_int32),
                ("mpaths_per_s", C.c_double), ("tried", C.c_int32), ("pad2", C.c_int32)]


class AdjointDesc(C.Structure):
    _fields_ = [("tex_material", C.c_int32), ("texture", C.c_int32), ("rough_material", C.c_int32),
                ("medium", C.c_int32)]


class RenderOpts(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32),
                ("max_bounces", C.c_int32), ("min_bounces", C.c_int32), ("integrator", C.c_int32),
                ("spectral_mode", C.c_int32), ("seed", C.c_uint32), ("sample_offset", C.c_uint32),
                ("block_size", C.c_int32), ("kernel_mode", C.c_int32), ("pool_slots", C.c_int32)]


KERNEL_AUTO, KERNEL_MEGAKERNEL, KERNEL_WAVEFRONT, KERNEL_WAVEFRONT_GRAPH = 0, 1, 2, 3
BVH_BUILD_HOST, BVH_BUILD_DEVICE = 0, 1


class Stats(C.Structure):
    _fields_ = [("last_render_ms", C.c_double), ("paths", C.c_uint64), ("rays", C.c_uint64),
                ("nodes_visited", C.c_uint64), ("tris_tested", C.c_uint64), ("bvh_nodes", C.c_uint64),
                ("bvh_bytes", C.c_uint64), ("tri_bytes", C.c_uint64), ("node_bytes", C.c_uint32),
                ("tri_record_bytes", C.c_uint32), ("device_bytes", C.c_uint64),
                ("trace_ms", C.c_double), ("shade_ms", C.c_double), ("spawn_ms", C.c_double),
                ("iterations", C.c_uint32), ("pool_slots", C.c_uint32), ("stage_ms", C.c_double * 6),
                ("resumed", C.c_uint64 * 6), ("traced", C.c_uint64), ("spawned", C.c_uint64),
                ("launches", C.c_uint64), ("bvh_build_ms", C.c_double)]


def render_opts(width, height, spp, max_bounces, min_bounces=3, seed=1, spectral=SPECTRAL_RGB3,
                sample_offset=0, integrator=INTEGRATOR_GPU_MISVOLPATH, block_size=0, kernel_mode=0, pool_slots=0):
    return RenderOpts(width, height, spp, max_bounces, min_bounces, integrator, spectral, seed,
                      sample_offset, block_size, kernel_mode, pool_slots)
