"""ctypes loader and build recipe for the CPU oracle (test infrastructure only)."""
import ctypes as C
import os
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB = HERE / "_build" / "liblambda_oracle.so"
SRC = HERE / "lambda_oracle.cpp"


def build(force=False):
    """Compile the oracle with g++ (-ffp-contract=off keeps x86 and Arm results identical)."""
    deps = [SRC, HERE.parent / "include" / "lambda_gpu.h", HERE.parent / "lambda_gb300" / "csrc" / "lgpu_rng.h",
            HERE.parent / "lambda_gb300" / "csrc" / "spectral_tables.h"]
    if LIB.exists() and not force and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    LIB.parent.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp%d" % os.getpid())
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-Wall",
           "-Wno-unused-function", str(SRC), "-o", str(tmp), "-lpthread"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [C.c_void_p]
        L.oracle_destroy.argtypes = [C.c_void_p]
        L.oracle_render.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64,
                                    C.c_void_p, C.c_void_p, C.c_int]
        L.oracle_intersect.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        for name in ("oracle_fr_dielectric",):
            getattr(L, name).restype = C.c_float
            getattr(L, name).argtypes = [C.c_float] * 3
        L.oracle_to_alpha.restype = C.c_float
        L.oracle_to_alpha.argtypes = [C.c_float]
        L.oracle_phase_hg.restype = C.c_float
        L.oracle_phase_hg.argtypes = [C.c_float, C.c_float]
        L.oracle_hg_sample.restype = C.c_float
        L.oracle_hg_sample.argtypes = [C.c_float, C.c_void_p, C.c_float, C.c_float, C.c_void_p]
        L.oracle_oren_nayar.restype = C.c_float
        L.oracle_oren_nayar.argtypes = [C.c_void_p, C.c_void_p, C.c_float]
        L.oracle_microfacet.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_void_p]
        L.oracle_blackbody_rgb.argtypes = [C.c_float, C.c_int, C.c_void_p]
        L.oracle_blackbody_norm.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_void_p]
        L.oracle_smits.restype = C.c_float
        L.oracle_smits.argtypes = [C.c_void_p, C.c_int, C.c_float]
        for name in ("oracle_perlin2d", "oracle_value2d", "oracle_voronoi2d", "oracle_checker2d"):
            getattr(L, name).restype = C.c_float
            getattr(L, name).argtypes = [C.c_float] * 3
        L.oracle_voronoi3d.restype = C.c_float
        L.oracle_voronoi3d.argtypes = [C.c_float] * 4
        L.oracle_medium.argtypes = [C.c_float, C.c_float, C.c_float, C.c_void_p]
        L.oracle_cone_union.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_momega.restype = C.c_float
        L.oracle_momega.argtypes = [C.c_float, C.c_float]
        L.oracle_tree_info.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_rng_bits.restype = C.c_uint32
        L.oracle_rng_bits.argtypes = [C.c_uint32] * 4
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Oracle:
    """CPU restatement of the reference integrator bound to one scene description."""

    def __init__(self, scene_builder):
        self._desc = scene_builder.desc()
        self._h = lib().oracle_create(C.byref(self._desc))
        if not self._h:
            raise RuntimeError("oracle rejected the scene")

    def close(self):
        if self._h:
            lib().oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def render(self, camera, opts, threads=0):
        """Full frame: returns the film (H, W, 4) = summed RGB + count."""
        film = np.zeros((opts.height, opts.width, 4), np.float32)
        cam = camera.desc()
        if lib().oracle_render(self._h, C.byref(cam), C.byref(opts), None, 0, _p(film), None, threads):
            raise ValueError("oracle rejected the camera")
        return film

    def render_paths(self, camera, opts, path_ids, threads=0):
        ids = np.ascontiguousarray(path_ids, np.uint64)
        outp = np.zeros((len(ids), 4), np.float32)
        cam = camera.desc()
        if lib().oracle_render(self._h, C.byref(cam), C.byref(opts), _p(ids), len(ids), None, _p(outp), threads):
            raise ValueError("oracle rejected the camera")
        return outp

    def tree_info(self):
        out = np.zeros(3, np.float32)
        lib().oracle_tree_info(self._h, _p(out))
        return {"tree_power": float(out[0]), "inf_power": float(out[1]), "tree_lights": int(out[2])}

    def intersect(self, o, d):
        ray = np.array(list(o) + [0.0] + list(d) + [np.inf], np.float32)
        res = np.zeros(4, np.float32)
        ids = np.zeros(2, np.int32)
        hit = lib().oracle_intersect(self._h, _p(ray), _p(res), _p(ids))
        return bool(hit), float(res[0]), int(ids[0]), int(ids[1])
