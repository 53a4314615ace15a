"""lambda_gb300: GB300-native (sm_103a) MIS volumetric path tracer behind Lambda's scene API.

The compute path is the CUDA library lambda_gb300/_build/liblambda_gpu.so (C ABI declared in
include/lambda_gpu.h); this module only binds it with ctypes.  There is no CPU fallback: if the
library or a GPU is missing, every entry point raises.
"""
import ctypes as C
import os
import pathlib

import numpy as np

from . import abi
from .scene import Camera, SceneBuilder, out  # noqa: F401

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = pathlib.Path(os.environ["LGPU_LIB_PATH"]) if os.environ.get("LGPU_LIB_PATH") else HERE / "_build" / "liblambda_gpu.so"

EXPORTS = ["lgpu_create", "lgpu_destroy", "lgpu_last_error", "lgpu_scene_commit", "lgpu_render",
           "lgpu_render_device", "lgpu_render_paths", "lgpu_render_count", "lgpu_intersect",
           "lgpu_get_stats", "lgpu_version", "lgpu_scene_check", "lgpu_render_paths_noalloc", "lgpu_render_batch", "lgpu_autotune", "lgpu_adjoint", "lgpu_film_resolve",
           "lgpu_render_progressive", "lgpu_probe_bandwidth", "lgpu_set_bvh_builder"]

_lib = None


class LambdaGPUError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("lgpu error %d: %s" % (code, msg))
        self.code = code


def build(force=False):
    """Build the extension in-tree (a no-op when LGPU_LIB_PATH selects a prebuilt tuning variant)."""
    if os.environ.get("LGPU_LIB_PATH"):
        return LIB_PATH
    from .build_ext import build as _b
    return _b(force=force)


def lib():
    """Load the CUDA extension; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError("CUDA extension %s is missing: run lambda_gb300.build()" % LIB_PATH)
        L = C.CDLL(str(LIB_PATH))
        vp = C.c_void_p
        L.lgpu_create.argtypes = [C.POINTER(vp), C.c_int]
        L.lgpu_destroy.argtypes = [vp]
        L.lgpu_destroy.restype = None
        L.lgpu_last_error.argtypes = [vp]
        L.lgpu_last_error.restype = C.c_char_p
        L.lgpu_scene_commit.argtypes = [vp, C.POINTER(abi.SceneDesc)]
        L.lgpu_render.argtypes = [vp, C.POINTER(abi.CameraDesc), C.POINTER(abi.RenderOpts), vp]
        L.lgpu_render_device.argtypes = [vp, C.POINTER(abi.CameraDesc), C.POINTER(abi.RenderOpts), vp, vp, vp]
        L.lgpu_render_paths.argtypes = [vp, C.POINTER(abi.CameraDesc), C.POINTER(abi.RenderOpts), vp, C.c_uint64, vp]
        L.lgpu_render_count.argtypes = [vp, C.POINTER(abi.CameraDesc), C.POINTER(abi.RenderOpts)]
        L.lgpu_intersect.argtypes = [vp, vp, vp, vp, C.c_uint64, vp]
        L.lgpu_get_stats.argtypes = [vp, C.POINTER(abi.Stats)]
        L.lgpu_version.restype = C.c_char_p
        L.lgpu_probe_bandwidth.argtypes = [vp, C.c_uint64, C.c_int32, C.POINTER(C.c_double)]
        L.lgpu_set_bvh_builder.argtypes = [vp, C.c_int32]
        L.lgpu_scene_check.argtypes = [C.POINTER(abi.SceneDesc), C.c_char_p, C.c_size_t]
        L.lgpu_render_batch.argtypes = [vp, C.POINTER(abi.ViewDesc), C.c_int32, C.POINTER(abi.RenderOpts), vp]
        L.lgpu_adjoint.argtypes = [vp, C.POINTER(abi.CameraDesc), C.POINTER(abi.RenderOpts),
                                   C.POINTER(abi.AdjointDesc), vp, vp, vp, vp]
        L.lgpu_film_resolve.argtypes = [vp, vp, C.c_uint64, vp]
        L.lgpu_render_progressive.argtypes = [vp, C.POINTER(abi.CameraDesc), C.POINTER(abi.RenderOpts), C.c_int32,
                                              vp, vp, vp]
        L.lgpu_autotune.argtypes = [vp, C.POINTER(abi.ViewDesc), C.c_int32, C.POINTER(abi.RenderOpts), C.c_int32,
                                    C.POINTER(abi.Tuning)]
        _lib = L
    return _lib


def scene_check(scene):
    """Compile + validate a scene on the host only (no GPU): returns (status, report)."""
    desc = scene.desc()
    buf = C.create_string_buffer(512)
    rc = lib().lgpu_scene_check(C.byref(desc), buf, 512)
    return rc, buf.value.decode()


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Renderer:
    """One GPU context holding one committed scene (lgpu_create + lgpu_scene_commit)."""

    def __init__(self, scene, device=0, bvh_builder=0):
        """bvh_builder: abi.BVH_BUILD_HOST (binned SAH on the host) or abi.BVH_BUILD_DEVICE (LBVH)."""
        L = lib()
        h = C.c_void_p()
        rc = L.lgpu_create(C.byref(h), device)
        if rc != 0:
            raise LambdaGPUError(rc, "lgpu_create failed (no CUDA device?)")
        self._h = h
        self._desc = scene.desc()
        self._scene = scene
        if bvh_builder:
            self._check(L.lgpu_set_bvh_builder(self._h, int(bvh_builder)))
        self._check(L.lgpu_scene_commit(self._h, C.byref(self._desc)))

    def _check(self, rc):
        if rc != 0:
            raise LambdaGPUError(rc, lib().lgpu_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            lib().lgpu_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def handle(self):
        return self._h

    def render(self, camera, opts, film=None):
        """Host-buffer render (lgpu_render): adds opts.spp samples into film (H, W, 4)."""
        if film is None:
            film = np.zeros((opts.height, opts.width, 4), np.float32)
        cam = camera.desc()
        self._check(lib().lgpu_render(self._h, C.byref(cam), C.byref(opts), _ptr(film)))
        return film

    def render_device(self, camera, opts, film_ptr, paths_ptr=None, stream=None):
        """Device-buffer render: film_ptr / paths_ptr are device addresses (ints)."""
        cam = camera.desc()
        self._check(lib().lgpu_render_device(self._h, C.byref(cam), C.byref(opts), C.c_void_p(film_ptr),
                                             C.c_void_p(paths_ptr) if paths_ptr else None,
                                             C.c_void_p(stream) if stream else None))

    def render_paths(self, camera, opts, path_ids):
        ids = np.ascontiguousarray(path_ids, np.uint64)
        outp = np.zeros((len(ids), 4), np.float32)
        cam = camera.desc()
        self._check(lib().lgpu_render_paths(self._h, C.byref(cam), C.byref(opts), _ptr(ids), len(ids), _ptr(outp)))
        return outp

    def render_batch(self, views, opts, stream=None):
        """Batched render (lgpu_render_batch).  views: list of (camera, width, height, spp,
        max_bounces, seed, film_ptr[, sample_offset]) with film_ptr a device address of
        width*height float4."""
        arr = self._views(views)
        self._check(lib().lgpu_render_batch(self._h, arr, len(views), C.byref(opts),
                                            C.c_void_p(stream) if stream else None))

    @staticmethod
    def _views(views):
        arr = (abi.ViewDesc * len(views))()
        for i, v in enumerate(views):
            cam, w, h, spp, depth, seed, film_ptr = v[:7]
            arr[i].camera = cam.desc()
            arr[i].width, arr[i].height, arr[i].spp, arr[i].max_bounces = w, h, spp, depth
            arr[i].seed, arr[i].sample_offset, arr[i].film_dev = seed, (v[7] if len(v) > 7 else 0), film_ptr
        return arr

    def autotune(self, views, opts, probe_spp=1):
        """lgpu_autotune over views (same tuple form as render_batch; film pointers unused)."""
        t = abi.Tuning()
        arr = self._views([v[:6] + (v[6] if len(v) > 6 else None,) for v in views])
        self._check(lib().lgpu_autotune(self._h, arr, len(views), C.byref(opts), probe_spp, C.byref(t)))
        return {f: getattr(t, f) for f, _ in abi.Tuning._fields_ if not f.startswith("pad")}

    def adjoint(self, camera, opts, params, dloss_ptr, grad_tex_ptr, grad_scalars_ptr, stream=None):
        """lgpu_adjoint: params = (tex_material, texture, rough_material, medium); pointers are device
        addresses (ints); gradients are added into the given buffers."""
        cam = camera.desc()
        p = abi.AdjointDesc(*params)
        self._check(lib().lgpu_adjoint(self._h, C.byref(cam), C.byref(opts), C.byref(p), C.c_void_p(dloss_ptr),
                                       C.c_void_p(grad_tex_ptr) if grad_tex_ptr else None,
                                       C.c_void_p(grad_scalars_ptr), C.c_void_p(stream) if stream else None))

    def render_progressive(self, camera, opts, passes, film_ptr, rgba_ptr=None, stream=None):
        """lgpu_render_progressive: passes of opts.spp samples into a device film, resolved to rgba."""
        cam = camera.desc()
        self._check(lib().lgpu_render_progressive(self._h, C.byref(cam), C.byref(opts), passes, C.c_void_p(film_ptr),
                                                  C.c_void_p(rgba_ptr) if rgba_ptr else None,
                                                  C.c_void_p(stream) if stream else None))

    def render_count(self, camera, opts):
        cam = camera.desc()
        self._check(lib().lgpu_render_count(self._h, C.byref(cam), C.byref(opts)))
        return self.stats()

    def intersect(self, rays_ptr, hits_ptr, uv_ptr, n, stream=None):
        self._check(lib().lgpu_intersect(self._h, C.c_void_p(rays_ptr), C.c_void_p(hits_ptr),
                                         C.c_void_p(uv_ptr) if uv_ptr else None, n,
                                         C.c_void_p(stream) if stream else None))

    def probe_bandwidth(self, nbytes, reps=20):
        """Read bandwidth (GB/s) of a buffer of nbytes on this renderer's device (lgpu_probe_bandwidth):
        a buffer inside L2 gives the L2 read peak, one far larger the HBM read rate."""
        g = C.c_double(0.0)
        self._check(lib().lgpu_probe_bandwidth(self._h, C.c_uint64(int(nbytes)), int(reps), C.byref(g)))
        return g.value

    def stats(self):
        s = abi.Stats()
        self._check(lib().lgpu_get_stats(self._h, C.byref(s)))
        out = {}
        for f, _ in abi.Stats._fields_:
            v = getattr(s, f)
            out[f] = list(v) if hasattr(v, "__len__") else v
        return out
