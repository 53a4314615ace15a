"""Host-side scene builder: assembles the flat scene description of include/lambda_gpu.h.

It mirrors how a Lambda application builds a scene (src/core/Scene.h, src/shading/graph): meshes
become objects with materials, materials reference a BxDF node of a shader graph, a light and a
media boundary.  The builder keeps every numpy buffer alive for as long as the descriptor is used.
"""
import ctypes as C
import numpy as np

from . import abi


def _fptr(a):
    return a.ctypes.data_as(abi.F32P) if a is not None else C.cast(None, abi.F32P)


class Camera:
    """Camera with the axes convention of Camera::SetForwards (src/camera/Camera.cpp:28-32):
    z = forward, x = cross(z, up), y = cross(x, z).

    kind: "pinhole" (PinholeCamera), "thin_lens" (ThinLensCamera: focal_length, aperture "none",
    "circular", "blade" or "masked" with aperture_size, blades and aperture_mask = index of a texture
    added with aperture_mask=True) or "spherical" (SphericalCamera: offset_phi, offset_theta)."""

    KINDS = {"pinhole": abi.CAMERA_PINHOLE, "thin_lens": abi.CAMERA_THIN_LENS, "spherical": abi.CAMERA_SPHERICAL}
    APERTURES = {"none": abi.APERTURE_NONE, "circular": abi.APERTURE_CIRCULAR, "blade": abi.APERTURE_BLADE,
                 "masked": abi.APERTURE_MASKED}

    def __init__(self, origin, target, fov=1.1, up=(0.0, 1.0, 0.0), kind="pinhole", focal_length=1.0,
                 aperture="none", aperture_size=0.0, blades=6, aperture_mask=-1, offset_phi=0.0,
                 offset_theta=0.0):
        o = np.asarray(origin, np.float64)
        z = np.asarray(target, np.float64) - o
        z /= np.linalg.norm(z)
        x = np.cross(z, np.asarray(up, np.float64))
        x /= np.linalg.norm(x)
        y = np.cross(x, z)
        self.origin, self.x, self.y, self.z, self.fov = o, x, y, z, float(fov)
        self.kind, self.focal_length, self.aperture = kind, float(focal_length), aperture
        self.aperture_size, self.blades, self.aperture_mask = float(aperture_size), int(blades), int(aperture_mask)
        self.offset_phi, self.offset_theta = float(offset_phi), float(offset_theta)

    def desc(self):
        d = abi.CameraDesc()
        for name, v in (("origin", self.origin), ("x_hat", self.x), ("y_hat", self.y), ("z_hat", self.z)):
            getattr(d, name)[:] = [float(t) for t in v]
        d.fov = self.fov
        d.type = self.KINDS[self.kind]
        d.focal_length = self.focal_length
        d.aperture = self.APERTURES[self.aperture]
        d.aperture_size = self.aperture_size
        d.blades = self.blades
        d.aperture_mask = self.aperture_mask
        d.offset_phi, d.offset_theta = self.offset_phi, self.offset_theta
        return d


class SceneBuilder:
    def __init__(self):
        self.meshes, self.objects, self.materials = [], [], []
        self.nodes, self.lights, self.media = [], [], []
        self.textures = []
        self.texture_masks = []
        self.has_volumes = False
        self.light_strategy = abi.LIGHT_STRATEGY_TREE
        self._keep = []

    # ---------------------------------------------------------------- geometry
    def mesh(self, verts, tris, normals=None, tangents=None, uvs=None):
        v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(tris, np.uint32).reshape(-1, 3)
        n = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        tg = None if tangents is None else np.ascontiguousarray(tangents, np.float32).reshape(-1, 4)
        uv = None if uvs is None else np.ascontiguousarray(uvs, np.float32).reshape(-1, 2)
        self.meshes.append((v, t, n, tg, uv))
        return len(self.meshes) - 1

    def obj(self, mesh, material, xfm=None):
        """xfm: None for a plain mesh object, else 12 floats (column-major 3x3, then translation)."""
        self.objects.append((mesh, 0 if xfm is None else 1, material,
                             [1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0] if xfm is None else list(map(float, xfm))))
        return len(self.objects) - 1

    def material(self, bxdf=-1, light=-1, medium_interior=-1, medium_exterior=-1):
        self.materials.append((bxdf, light, medium_interior, medium_exterior))
        return len(self.materials) - 1

    # ---------------------------------------------------------------- shader graph
    def node(self, kind, params=(), inputs=None, op=0):
        """inputs: {index: (node, socket)} for links or {index: (v0, v1, v2, v3)} / scalar defaults."""
        d = abi.NodeDesc()
        d.type = abi.NODE[kind] if isinstance(kind, str) else int(kind)
        d.op = int(op)
        for i, p in enumerate(params):
            d.params[i] = float(p)
        for i in range(4):
            d.in_node[i] = -1
            d.in_socket[i] = 0
        for i, val in (inputs or {}).items():
            if isinstance(val, Link):
                d.in_node[i], d.in_socket[i] = val.node, val.socket
            else:
                vals = [float(val)] * 4 if np.isscalar(val) else list(map(float, val)) + [0.0] * (4 - len(val))
                for k in range(4):
                    d.in_default[i][k] = vals[k]
        self.nodes.append(d)
        return len(self.nodes) - 1

    # ---------------------------------------------------------------- lights / media
    def light_mesh(self, obj, emission, intensity):
        d = abi.LightDesc()
        d.type, d.object = abi.LIGHT_MESH, obj
        d.emission_node, d.emission_socket = emission.node, emission.socket
        d.intensity = intensity
        self.lights.append(d)
        return len(self.lights) - 1

    def light_point(self, position, emission, intensity):
        d = abi.LightDesc()
        d.type, d.object = abi.LIGHT_POINT, -1
        d.position[:] = list(map(float, position))
        d.emission_node, d.emission_socket = emission.node, emission.socket
        d.intensity = intensity
        self.lights.append(d)
        return len(self.lights) - 1

    def light_spot(self, position, axis, cone_angle, falloff_start, emission, intensity):
        d = abi.LightDesc()
        d.type, d.object = abi.LIGHT_SPOT, -1
        d.position[:] = list(map(float, position))
        a = np.asarray(axis, np.float64)
        d.axis[:] = list(map(float, a / np.linalg.norm(a)))
        d.cone_angle, d.falloff_start = cone_angle, falloff_start
        d.emission_node, d.emission_socket = emission.node, emission.socket
        d.intensity = intensity
        self.lights.append(d)
        return len(self.lights) - 1

    def light_env(self, texture_rgb, intensity=1.0, offset=(0.0, 0.0)):
        tex = np.ascontiguousarray(texture_rgb, np.float32)
        h, w, _ = tex.shape
        self._keep.append(tex)
        d = abi.LightDesc()
        d.type, d.object = abi.LIGHT_ENVIRONMENT, -1
        d.intensity = intensity
        d.offset[:] = list(offset)
        d.env_width, d.env_height = w, h
        d.env_texture = _fptr(tex)
        d.emission_node = -1
        self.lights.append(d)
        return len(self.lights) - 1

    def medium(self, sigma_a, sigma_s, g):
        sa = [sigma_a] * 3 if np.isscalar(sigma_a) else list(sigma_a)
        ss = [sigma_s] * 3 if np.isscalar(sigma_s) else list(sigma_s)
        self.media.append((sa, ss, g))
        return len(self.media) - 1

    def texture(self, rgba, aperture_mask=False):
        """Image texture (height, width, 4) float texels, row y then column x; returns its index
        for an IMAGE_TEXTURE node's params[0] or a masked aperture (aperture_mask=True builds the
        sampling distribution of its |red| channel at commit)."""
        t = np.ascontiguousarray(rgba, np.float32)
        if t.ndim == 3 and t.shape[2] == 3:
            t = np.ascontiguousarray(np.concatenate([t, np.ones(t.shape[:2] + (1,), np.float32)], 2))
        assert t.ndim == 3 and t.shape[2] == 4
        self.textures.append(t)
        self.texture_masks.append(bool(aperture_mask))
        return len(self.textures) - 1

    # ---------------------------------------------------------------- descriptor
    def desc(self):
        ms = (abi.MeshDesc * max(1, len(self.meshes)))()
        for i, (v, t, n, tg, uv) in enumerate(self.meshes):
            ms[i].vertices, ms[i].triangles = _fptr(v), t.ctypes.data_as(abi.U32P)
            ms[i].normals, ms[i].tangents, ms[i].uvs = _fptr(n), _fptr(tg), _fptr(uv)
            ms[i].num_vertices, ms[i].num_triangles = len(v), len(t)
        obs = (abi.ObjectDesc * max(1, len(self.objects)))()
        for i, (m, kind, mat, x) in enumerate(self.objects):
            obs[i].mesh, obs[i].kind, obs[i].material = m, kind, mat
            obs[i].xfm[:] = x
        mats = (abi.MaterialDesc * max(1, len(self.materials)))()
        for i, (b, l, mi, me) in enumerate(self.materials):
            mats[i].bxdf_node, mats[i].light, mats[i].medium_interior, mats[i].medium_exterior = b, l, mi, me
        nodes = (abi.NodeDesc * max(1, len(self.nodes)))(*self.nodes)
        lights = (abi.LightDesc * max(1, len(self.lights)))(*self.lights)
        media = (abi.MediumDesc * max(1, len(self.media)))()
        for i, (sa, ss, g) in enumerate(self.media):
            media[i].sigma_a[:] = sa
            media[i].sigma_s[:] = ss
            media[i].g = g
        texs = (abi.TextureDesc * max(1, len(self.textures)))()
        for i, t in enumerate(self.textures):
            texs[i].rgba, texs[i].height, texs[i].width = _fptr(t), t.shape[0], t.shape[1]
            texs[i].aperture_mask = int(self.texture_masks[i])
        d = abi.SceneDesc(ms, len(self.meshes), obs, len(self.objects), mats, len(self.materials),
                          nodes, len(self.nodes), lights, len(self.lights), media, len(self.media),
                          int(self.has_volumes), int(self.light_strategy), texs, len(self.textures))
        self._keep.extend([ms, obs, mats, nodes, lights, media, texs])
        return d

    @property
    def num_triangles(self):
        return sum(len(m[1]) for m in self.meshes)


class Link:
    """A link to output socket `socket` of node `node`."""

    def __init__(self, node, socket=0):
        self.node, self.socket = node, socket


def out(node, socket=0):
    return Link(node, socket)
