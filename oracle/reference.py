"""ctypes loader of the reference renderer's own integrator (oracle/_ref/libref_li.so, built by
oracle/build_ref.py from a patched copy of the reference sources).  TEST INFRASTRUCTURE ONLY: it is
the anchor the CPU oracle is checked against and the CPU baseline that bench.py times; the product
never loads it.

available() is False where the library cannot be built (no reference tree and no prepared copy).
BindingScene drives the GPU module's Lambda-side binding (lambda_gb300/binding, built into
oracle/_ref/libref_binding.so) on the lambda::Scene of a description."""
import ctypes as C
import os

import numpy as np

from . import build_ref

_lib = None
_why = None
_blib = None
_bwhy = None


def lib():
    global _lib, _why
    if _lib is None and _why is None:
        try:
            path = build_ref.build_li()
        except Exception as e:   # a failed compile is reported, not raised, so callers can fall back
            path, _why = None, "reference build failed: %s" % str(e).splitlines()[0]
        if path is None:
            _why = _why or "no reference tree (LAMBDA_REFERENCE_ROOT) and no prepared copy in oracle/_ref/src"
        else:
            L = C.CDLL(str(path))
            L.ref_create.restype = C.c_void_p
            L.ref_create.argtypes = [C.c_void_p]
            L.ref_destroy.argtypes = [C.c_void_p]
            L.ref_last_error.restype = C.c_char_p
            L.ref_render.restype = C.c_int
            L.ref_render.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                                     C.c_int]
            L.ref_render_tiles.restype = C.c_int
            L.ref_render_tiles.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int]
            _lib = L
    return _lib


def available():
    return lib() is not None


def unavailable_reason():
    lib()
    return _why


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Reference:
    """The reference's lambda::Scene built from one scene description, with its integrators."""

    def __init__(self, scene_builder):
        L = lib()
        if L is None:
            raise RuntimeError(_why)
        self._desc = scene_builder.desc()
        self._h = L.ref_create(C.byref(self._desc))
        if not self._h:
            raise RuntimeError("reference rejected the scene: %s" % L.ref_last_error().decode())

    def close(self):
        if self._h:
            lib().ref_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def render_paths(self, camera, opts, path_ids, threads=0):
        """Per path: rgb radiance and the number of random numbers drawn."""
        ids = np.ascontiguousarray(path_ids, np.uint64)
        out = np.zeros((len(ids), 4), np.float32)
        cam = camera.desc()
        if lib().ref_render(self._h, C.byref(cam), C.byref(opts), _p(ids), len(ids), None, _p(out), threads):
            raise ValueError(lib().ref_last_error().decode())
        return out

    def render(self, camera, opts, threads=0):
        """Whole film (H, W, 4) = summed rgb + samples, by the reference's tile renderer."""
        film = np.zeros((opts.height, opts.width, 4), np.float32)
        cam = camera.desc()
        if lib().ref_render(self._h, C.byref(cam), C.byref(opts), None, 0, _p(film), None, threads):
            raise ValueError(lib().ref_last_error().decode())
        return film

    def render_tiles(self, camera, opts, tiles, threads=0):
        """Film of the chosen 16 x 16 tiles only (row-major tile indices)."""
        t = np.ascontiguousarray(tiles, np.int32)
        film = np.zeros((opts.height, opts.width, 4), np.float32)
        cam = camera.desc()
        if lib().ref_render_tiles(self._h, C.byref(cam), C.byref(opts), _p(t), len(t), _p(film), threads):
            raise ValueError(lib().ref_last_error().decode())
        return film

    @staticmethod
    def threads():
        return os.cpu_count() or 1


def binding_lib():
    """libref_binding.so (the reference units + the GPU module's binding), or None with a reason in
    binding_unavailable_reason()."""
    global _blib, _bwhy
    if _blib is None and _bwhy is None:
        try:
            path = build_ref.build_binding()
        except Exception as e:
            path, _bwhy = None, "binding build failed: %s" % str(e).splitlines()[0]
        if path is None:
            _bwhy = _bwhy or "no prepared reference copy or no GPU module library to link the binding with"
        else:
            L = C.CDLL(str(path))
            L.ref_create.restype = C.c_void_p
            L.ref_create.argtypes = [C.c_void_p]
            L.ref_destroy.argtypes = [C.c_void_p]
            L.ref_last_error.restype = C.c_char_p
            L.ref_binding_check.restype = C.c_int
            L.ref_binding_check.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t, C.c_void_p]
            L.ref_binding_render.restype = C.c_int
            L.ref_binding_render.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
            _blib = L
    return _blib


def binding_unavailable_reason():
    binding_lib()
    return _bwhy


class BindingScene:
    """A lambda::Scene built from a description by the reference's classes, translated back by the
    binding (lambda_gpu::SceneDesc) and rendered through its RenderDirective / TileRenderer paths."""

    COUNTS = ("meshes", "objects", "materials", "nodes", "lights", "media", "textures", "has_volumes", "light_strategy")

    def __init__(self, scene_builder):
        L = binding_lib()
        if L is None:
            raise RuntimeError(_bwhy)
        self._desc = scene_builder.desc()
        self._h = L.ref_create(C.byref(self._desc))
        if not self._h:
            raise RuntimeError("reference rejected the scene: %s" % L.ref_last_error().decode())

    def close(self):
        if self._h:
            binding_lib().ref_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def check(self):
        """(status, lgpu_scene_check report, dict of counts of the translated description)."""
        rep = C.create_string_buffer(512)
        counts = np.zeros(9, np.int32)
        rc = binding_lib().ref_binding_check(self._h, rep, 512, _p(counts))
        return rc, rep.value.decode(), dict(zip(self.COUNTS, counts.tolist()))

    def render(self, camera, opts, mode=0):
        """Film (H, W, 4) through GpuRenderer::RenderDirective (mode 0) or GpuTileRenderer (mode 1)."""
        film = np.zeros((opts.height, opts.width, 4), np.float32)
        cam = camera.desc()
        rc = binding_lib().ref_binding_render(self._h, C.byref(cam), C.byref(opts), mode, _p(film))
        if rc:
            raise ValueError("binding render failed (%d): %s" % (rc, binding_lib().ref_last_error().decode()))
        return film
