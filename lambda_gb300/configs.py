"""Seeded synthetic scenes for the benchmark workloads (no external assets exist for them).

  cornell(256, 256)      Cornell box: 5 wall quads (10 tris), icosphere subdiv 3 (1280 tris, r 0.3,
                         GGX roughness 0.2), 0.25 x 0.25 quad light with a 6500 K blackbody;
                         256^2, 16 spp, depth 8.
  terrain(1920, 1080)    1024^2-vertex heightfield displaced by 6-octave gradient noise
                         (2,093,058 tris), 10,000 emissive triangles (blackbody 2000-10000 K,
                         log-uniform intensity 0.1-100) sampled through the light tree, procedural
                         sky environment, GGX albedo/roughness from a noise node graph;
                         1080p, 64 spp, depth 6.
  volume(1280, 720)      homogeneous medium box (sigma_a 0.05, sigma_s 0.5, HG g 0.3), 16 point +
                         4 spot lights (30 degree cones), 1000 instances of a ~100k-tri displaced
                         sphere (random rotation, scale 0.5-2), half dielectric IOR 1.5, half
                         Mix(Oren-Nayar sigma 20 deg, GGX) at 0.5; 720p, 128 spp, depth 12.
"""
import math

import numpy as np

from . import abi
from .scene import Camera, SceneBuilder, out


# ------------------------------------------------------------------ procedural helpers
def gradient_noise_2d(x, y, seed, period=256):
    """Gradient noise on the integer lattice with a seeded permutation (quintic fade)."""
    rng = np.random.RandomState(seed)
    perm = rng.permutation(period)
    perm = np.concatenate([perm, perm]).astype(np.int64)
    ang = rng.uniform(0, 2 * np.pi, period)
    gx, gy = np.cos(ang), np.sin(ang)
    xi = np.floor(x).astype(np.int64)
    yi = np.floor(y).astype(np.int64)
    xf, yf = x - xi, y - yi

    def grad(ix, iy, dx, dy):
        h = perm[(perm[ix % period] + iy % period) % (2 * period)] % period
        return gx[h] * dx + gy[h] * dy

    def fade(t):
        return t * t * t * (t * (t * 6 - 15) + 10)

    n00 = grad(xi, yi, xf, yf)
    n10 = grad(xi + 1, yi, xf - 1, yf)
    n01 = grad(xi, yi + 1, xf, yf - 1)
    n11 = grad(xi + 1, yi + 1, xf - 1, yf - 1)
    u, v = fade(xf), fade(yf)
    return (n00 * (1 - u) + n10 * u) * (1 - v) + (n01 * (1 - u) + n11 * u) * v


def fbm(x, y, octaves, seed):
    tot = np.zeros_like(x)
    amp, freq = 1.0, 1.0
    for o in range(octaves):
        tot += amp * gradient_noise_2d(x * freq, y * freq, seed + o)
        amp *= 0.5
        freq *= 2.0
    return tot


def quad(p0, p1, p2, p3):
    """Two triangles (p0,p1,p2), (p0,p2,p3)."""
    return np.array([p0, p1, p2, p3], np.float32), np.array([[0, 1, 2], [0, 2, 3]], np.uint32)


def icosphere(subdiv, radius=1.0, center=(0, 0, 0)):
    t = (1.0 + 5 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
             (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache, nf = {}, []

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    v = np.array(verts) * radius + np.asarray(center, np.float64)
    return v.astype(np.float32), np.array(faces, np.uint32)


def latlong_sphere(nlat, nlon, radius=1.0, displace=None):
    """UV sphere with smooth normals, tangents and uvs; optional radial displacement f(dirs)."""
    th = np.linspace(0, np.pi, nlat + 1)
    ph = np.linspace(0, 2 * np.pi, nlon + 1)
    T, P = np.meshgrid(th, ph, indexing="ij")
    d = np.stack([np.sin(T) * np.cos(P), np.cos(T), np.sin(T) * np.sin(P)], -1)
    r = radius * (1.0 + (displace(d) if displace is not None else 0.0))
    v = d * r[..., None] if np.ndim(r) else d * r
    tang = np.stack([-np.sin(P), np.zeros_like(P), np.cos(P)], -1)
    uv = np.stack([P / (2 * np.pi), T / np.pi], -1)
    idx = np.arange((nlat + 1) * (nlon + 1)).reshape(nlat + 1, nlon + 1)
    a, b = idx[:-1, :-1], idx[:-1, 1:]
    c, e = idx[1:, 1:], idx[1:, :-1]
    tris = np.concatenate([np.stack([a, c, b], -1)[1:], np.stack([a, e, c], -1)[:-1]], 0).reshape(-1, 3)
    v = v.reshape(-1, 3)
    # smooth normals from geometry
    n = np.zeros_like(v)
    fn = np.cross(v[tris[:, 1]] - v[tris[:, 0]], v[tris[:, 2]] - v[tris[:, 0]])
    for k in range(3):
        np.add.at(n, tris[:, k], fn)
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-12)
    tg = tang.reshape(-1, 3)
    tg = tg - n * np.sum(tg * n, 1, keepdims=True)
    tg /= np.maximum(np.linalg.norm(tg, axis=1, keepdims=True), 1e-12)
    tg4 = np.concatenate([tg, np.ones((len(tg), 1))], 1)
    return (v.astype(np.float32), tris.astype(np.uint32), n.astype(np.float32), tg4.astype(np.float32),
            uv.reshape(-1, 2).astype(np.float32))


def rotation_matrix(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def affine(m3, t):
    """Column-major 3x3 + translation, the affine3<Real>::xfm layout."""
    m3 = np.asarray(m3, np.float64)
    return list(m3.T.reshape(-1)) + list(map(float, t))


def blackbody_emission(sb, temperature):
    t = sb.node("SCALAR", [temperature])
    return out(sb.node("BLACKBODY", [3], {0: out(t)}))


# ------------------------------------------------------------------ config: Cornell box
def cornell(width=256, height=256, spp=16, max_depth=8, subdiv=3, light_intensity=40.0):
    sb = SceneBuilder()
    white = sb.node("BXDF_LAMBERTIAN", inputs={0: (0.73, 0.73, 0.73, 1)})
    red = sb.node("BXDF_LAMBERTIAN", inputs={0: (0.65, 0.05, 0.05, 1)})
    green = sb.node("BXDF_LAMBERTIAN", inputs={0: (0.05, 0.65, 0.05, 1)})
    black = sb.node("BXDF_LAMBERTIAN", inputs={0: (0.0, 0.0, 0.0, 1)})
    ggx = sb.node("BXDF_MICROFACET_R", [abi.DIST_TROWBRIDGE_REITZ, 1.5],
                  {0: (0.9, 0.9, 0.9, 1), 1: 0.2})
    m_white, m_red, m_green = sb.material(white), sb.material(red), sb.material(green)
    m_ggx = sb.material(ggx)
    walls = [  # floor, ceiling, back, left (red), right (green); normals point into the box
        ((-1, -1, -1), (-1, -1, 1), (1, -1, 1), (1, -1, -1), m_white),
        ((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1), m_white),
        ((-1, -1, 1), (-1, 1, 1), (1, 1, 1), (1, -1, 1), m_white),
        ((-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1), m_red),
        ((1, -1, -1), (1, -1, 1), (1, 1, 1), (1, 1, -1), m_green),
    ]
    for p0, p1, p2, p3, m in walls:
        v, t = quad(p0, p1, p2, p3)
        sb.obj(sb.mesh(v, t), m)
    sv, st = icosphere(subdiv, 0.3, (0.2, -0.7, 0.2))
    sb.obj(sb.mesh(sv, st), m_ggx)
    h = 0.125
    lv, lt = quad((-h, 0.999, -h), (h, 0.999, -h), (h, 0.999, h), (-h, 0.999, h))
    emis = blackbody_emission(sb, 6500.0)
    m_light = sb.material(black, light=len(sb.lights))
    lobj = sb.obj(sb.mesh(lv, lt), m_light)
    sb.light_mesh(lobj, emis, light_intensity)
    cam = Camera((0, 0, -3.4), (0, 0, 0), fov=0.75)
    opts = abi.render_opts(width, height, spp, max_depth)
    return sb, cam, opts


# ------------------------------------------------------------------ parity scene: every graph node
def node_zoo(width=48, height=48, spp=4, max_depth=6, light_strategy=abi.LIGHT_STRATEGY_POWER):
    """Closed box whose materials route through every shader-graph node kind the GPU compiles
    (value noise, checker, vector maths with all four operators, dot, cross, magnitude, separate
    XYZ / RGBA, merge XYZ / RGBA, surface information, constant spectrum, sqrt and power), a
    Beckmann microfacet sphere with noise-driven roughness, a specular mirror sphere, an Oren-Nayar
    wall, lit by a quad emitter, a point light and a spotlight through the power-CDF light sampler
    (light_strategy) -- a parity scene for the branches the benchmark scenes leave out."""
    sb = SceneBuilder()
    sb.light_strategy = light_strategy
    # floor albedo: r = value noise * 0.7, g = checker (scaled by sqrt), b = |normal x (0,0,1)| and
    # the surface normal through vector maths; every output feeds the albedo so nothing is folded away
    vnoise = sb.node("VALUE_NOISE", [6.0])
    chk = sb.node("CHECKER", [8.0])
    nrm = sb.node("SURFACE_INFO")
    k07, k2, k3, k05 = (sb.node("SCALAR", [v]) for v in (0.7, 2.0, 3.0, 0.5))
    r = sb.node("MATHS", inputs={0: out(vnoise), 1: out(k07)}, op=abi.MATHS_MULTIPLY)
    sq = sb.node("MATHS", inputs={0: out(chk), 1: 0.0}, op=abi.MATHS_SQRT)
    g = sb.node("MATHS", inputs={0: out(sq), 1: out(k05)}, op=abi.MATHS_MULTIPLY)
    axis = sb.node("VECTOR3", [0.0, 0.0, 1.0])
    cr = sb.node("CROSS_PRODUCT", inputs={0: out(nrm), 1: out(axis)})
    mag = sb.node("VECTOR_MAGNITUDE", inputs={0: out(cr)})
    vsum = sb.node("VECTOR_MATHS", inputs={0: out(nrm), 1: out(axis)}, op=abi.MATHS_ADD)
    vdif = sb.node("VECTOR_MATHS", inputs={0: out(vsum), 1: (0.25, 0.5, 0.25, 0)}, op=abi.MATHS_SUBTRACT)
    vmul = sb.node("VECTOR_MATHS", inputs={0: out(vdif), 1: (0.5, 0.5, 0.5, 0)}, op=abi.MATHS_MULTIPLY)
    vdiv = sb.node("VECTOR_MATHS", inputs={0: out(vmul), 1: (2.0, 4.0, 8.0, 1)}, op=abi.MATHS_DIVIDE)
    sep = sb.node("SEPARATE_XYZ", inputs={0: out(vdiv)})
    dot = sb.node("DOT_PRODUCT", inputs={0: out(nrm), 1: out(vdiv)})
    b0 = sb.node("MATHS", inputs={0: out(mag), 1: out(sep, 1)}, op=abi.MATHS_ADD)
    b1 = sb.node("MATHS", inputs={0: out(b0), 1: out(dot)}, op=abi.MATHS_SUBTRACT)
    bpow = sb.node("MATHS", inputs={0: out(b1), 1: out(k2)}, op=abi.MATHS_POWER)
    b = sb.node("MATHS", inputs={0: out(bpow), 1: out(k3)}, op=abi.MATHS_DIVIDE)
    rgba = sb.node("MERGE_RGBA", inputs={0: out(r), 1: out(g), 2: out(b), 3: 1.0})
    chan = sb.node("SEPARATE_RGBA", inputs={0: out(rgba)})
    xyz = sb.node("MERGE_XYZ", inputs={0: out(chan, 0), 1: out(chan, 1), 2: out(chan, 2)})
    floor = sb.node("BXDF_LAMBERTIAN", inputs={0: out(xyz)})
    # Beckmann sphere, roughness 0.1 + 0.4 * value noise; mirror sphere; Oren-Nayar back wall with
    # a constant-spectrum albedo
    rn = sb.node("VALUE_NOISE", [3.0])
    rs = sb.node("MATHS", inputs={0: out(rn), 1: 0.4}, op=abi.MATHS_MULTIPLY)
    rough = sb.node("MATHS", inputs={0: out(rs), 1: 0.1}, op=abi.MATHS_ADD)
    beck = sb.node("BXDF_MICROFACET_R", [abi.DIST_BECKMANN, 1.5], {0: (0.9, 0.7, 0.5, 1), 1: out(rough)})
    mirror = sb.node("BXDF_SPECULAR_R", [1.5], {0: (0.95, 0.95, 0.95, 1)})
    spec = sb.node("SPECTRUM", [0.6, 0.5, 0.4])
    onw = sb.node("BXDF_OREN_NAYAR_R", inputs={0: out(spec), 1: math.radians(30.0)})
    white = sb.node("BXDF_LAMBERTIAN", inputs={0: (0.73, 0.73, 0.73, 1)})
    black = sb.node("BXDF_LAMBERTIAN", inputs={0: (0.0, 0.0, 0.0, 1)})
    m_floor, m_beck, m_mirror, m_on, m_white = (sb.material(x) for x in (floor, beck, mirror, onw, white))
    uv = [(0, 0), (0, 4), (4, 4), (4, 0)]
    walls = [((-1, -1, -1), (-1, -1, 1), (1, -1, 1), (1, -1, -1), m_floor),
             ((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1), m_white),
             ((-1, -1, 1), (-1, 1, 1), (1, 1, 1), (1, -1, 1), m_on),
             ((-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1), m_white),
             ((1, -1, -1), (1, -1, 1), (1, 1, 1), (1, 1, -1), m_white)]
    for p0, p1, p2, p3, m in walls:
        v, t = quad(p0, p1, p2, p3)
        sb.obj(sb.mesh(v, t, uvs=uv), m)
    for centre, m in (((-0.4, -0.65, 0.2), m_beck), ((0.45, -0.7, -0.1), m_mirror)):
        sv, st, sn, stg, suv = latlong_sphere(16, 24, 0.3)
        sb.obj(sb.mesh(sv + np.asarray(centre, np.float32), st, sn, stg, suv), m)
    h = 0.15
    lv, lt = quad((-h, 0.999, -h), (h, 0.999, -h), (h, 0.999, h), (-h, 0.999, h))
    m_light = sb.material(black, light=len(sb.lights))
    lobj = sb.obj(sb.mesh(lv, lt), m_light)
    sb.light_mesh(lobj, blackbody_emission(sb, 5000.0), 30.0)
    warm = out(sb.node("RGB", [1.0, 0.8, 0.6]))
    sb.light_point((0.6, 0.5, -0.5), warm, 1.5)
    sb.light_spot((-0.5, 0.9, 0.3), (0.3, -1.0, 0.1), math.radians(35.0), math.radians(25.0), warm, 4.0)
    cam = Camera((0, 0, -3.4), (0, -0.2, 0), fov=0.75)
    opts = abi.render_opts(width, height, spp, max_depth)
    return sb, cam, opts


# ------------------------------------------------------------------ config: inverse rendering
def inverse_cameras(n=8, radius=3.0, spread=0.6):
    """n pinhole cameras on an arc of the ring of the given radius around the box centre, facing
    the open side of the box (a full ring would see the outside of the walls)."""
    cams = []
    for k in range(n):
        a = -spread + 2 * spread * k / max(1, n - 1)
        cams.append(Camera((radius * np.sin(a), 0.15 * np.cos(3 * a), -radius * np.cos(a)), (0, 0, 0), fov=0.8))
    return cams


def cornell_inverse(width=512, height=512, spp=4, max_depth=8, albedo=None, roughness=0.3, sigma_a=0.1,
                    sigma_s=0.8, tex_res=64, seed=5):
    """Cornell box whose back wall albedo is a tex_res^2 image texture, whose sphere is GGX with a
    scalar roughness, and which holds a homogeneous-medium cube of side 0.4 (null surface).  The
    unknowns of the inverse-rendering workload are that texture, the roughness and the cube's
    sigma_a / sigma_s.  albedo: (tex_res, tex_res, 3) array, default seeded uniform [0.1, 0.9]."""
    rng = np.random.RandomState(seed)
    if albedo is None:
        albedo = rng.uniform(0.1, 0.9, (tex_res, tex_res, 3)).astype(np.float32)
    sb = SceneBuilder()
    sb.has_volumes = True
    tex = sb.texture(albedo)
    img = sb.node("IMAGE_TEXTURE", [tex])
    back = sb.node("BXDF_LAMBERTIAN", inputs={0: out(img, 0)})
    white = sb.node("BXDF_LAMBERTIAN", inputs={0: (0.73, 0.73, 0.73, 1)})
    red = sb.node("BXDF_LAMBERTIAN", inputs={0: (0.65, 0.05, 0.05, 1)})
    green = sb.node("BXDF_LAMBERTIAN", inputs={0: (0.05, 0.65, 0.05, 1)})
    black = sb.node("BXDF_LAMBERTIAN", inputs={0: (0.0, 0.0, 0.0, 1)})
    ggx = sb.node("BXDF_MICROFACET_R", [abi.DIST_TROWBRIDGE_REITZ, 1.5], {0: (0.9, 0.9, 0.9, 1), 1: float(roughness)})
    m_back, m_white, m_red, m_green, m_ggx = (sb.material(b) for b in (back, white, red, green, ggx))
    walls = [((-1, -1, -1), (-1, -1, 1), (1, -1, 1), (1, -1, -1), m_white),
             ((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1), m_white),
             ((-1, -1, 1), (-1, 1, 1), (1, 1, 1), (1, -1, 1), m_back),
             ((-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1), m_red),
             ((1, -1, -1), (1, -1, 1), (1, 1, 1), (1, 1, -1), m_green)]
    for p0, p1, p2, p3, m in walls:
        v, t = quad(p0, p1, p2, p3)
        sb.obj(sb.mesh(v, t, uvs=[(0, 0), (0, 1), (1, 1), (1, 0)]), m)
    sv, st = icosphere(3, 0.3, (0.35, -0.7, 0.25))
    sb.obj(sb.mesh(sv, st), m_ggx)
    med = sb.medium(float(sigma_a), float(sigma_s), 0.0)
    m_box = sb.material(-1, medium_interior=med)
    c, hs = np.array([-0.4, -0.6, -0.1]), 0.2
    for p0, p1, p2, p3 in box_faces(c, hs):
        v, t = quad(p0, p1, p2, p3)
        sb.obj(sb.mesh(v, t), m_box)
    h = 0.125
    lv, lt = quad((-h, 0.999, -h), (h, 0.999, -h), (h, 0.999, h), (-h, 0.999, h))
    emis = blackbody_emission(sb, 6500.0)
    m_light = sb.material(black, light=len(sb.lights))
    lobj = sb.obj(sb.mesh(lv, lt), m_light)
    sb.light_mesh(lobj, emis, 40.0)
    opts = abi.render_opts(width, height, spp, max_depth)
    return sb, inverse_cameras(), opts


def box_faces(c, hs):
    """Six outward-facing quads of an axis-aligned cube (centre c, half side hs)."""
    x0, y0, z0 = c - hs
    x1, y1, z1 = c + hs
    return [((x0, y0, z0), (x1, y0, z0), (x1, y0, z1), (x0, y0, z1)),
            ((x0, y1, z0), (x0, y1, z1), (x1, y1, z1), (x1, y1, z0)),
            ((x0, y0, z0), (x0, y1, z0), (x1, y1, z0), (x1, y0, z0)),
            ((x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)),
            ((x0, y0, z0), (x0, y0, z1), (x0, y1, z1), (x0, y1, z0)),
            ((x1, y0, z0), (x1, y1, z0), (x1, y1, z1), (x1, y0, z1))]


# ------------------------------------------------------------------ config: many-light terrain
def sky_texture(w=512, h=256):
    v = (np.arange(h) + 0.5) / h
    theta = v * np.pi                          # 0 = up (+y)
    up = np.cos(theta)
    zen = np.array([0.25, 0.45, 0.95])
    hor = np.array([0.85, 0.9, 1.0])
    gnd = np.array([0.12, 0.1, 0.08])
    t = np.clip(up, 0, 1)[:, None]
    col = np.where(up[:, None] >= 0, hor * (1 - t) + zen * t, gnd * np.ones_like(t))
    tex = np.repeat(col[:, None, :], w, axis=1)
    return tex.astype(np.float32)


def terrain(width=1920, height=1080, spp=64, max_depth=6, grid=1024, n_emitters=10000, size=100.0,
            seed=1):
    sb = SceneBuilder()
    lin = np.linspace(-size / 2, size / 2, grid)
    X, Z = np.meshgrid(lin, lin, indexing="ij")
    Hh = fbm(X / 12.0, Z / 12.0, 6, seed) * 6.0
    verts = np.stack([X, Hh, Z], -1).reshape(-1, 3)
    # smooth normals from central differences; tangent along +x
    dx = size / (grid - 1)
    gxh = np.gradient(Hh, dx, axis=0)
    gzh = np.gradient(Hh, dx, axis=1)
    n = np.stack([-gxh, np.ones_like(Hh), -gzh], -1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    tg = np.stack([np.ones_like(Hh), gxh, np.zeros_like(Hh)], -1)
    tg -= n * np.sum(tg * n, -1, keepdims=True)
    tg /= np.linalg.norm(tg, axis=-1, keepdims=True)
    tg4 = np.concatenate([tg, np.ones(Hh.shape + (1,))], -1)
    uv = np.stack([(X + size / 2) / size, (Z + size / 2) / size], -1)
    idx = np.arange(grid * grid).reshape(grid, grid)
    a, b, c, d = idx[:-1, :-1], idx[1:, :-1], idx[1:, 1:], idx[:-1, 1:]
    # winding so that the geometric normal points up (+y)
    tris = np.concatenate([np.stack([a, d, c], -1).reshape(-1, 3), np.stack([a, c, b], -1).reshape(-1, 3)], 0)
    # shader graph: albedo / roughness from 2D gradient noise (Perlin), Voronoi and octave noise
    perlin = sb.node("PERLIN_NOISE", [1.0])
    octave = sb.node("OCTAVE_NOISE", [6.0, 3], {0: out(perlin)})
    vor = sb.node("VORONOI", [24.0])
    c06, c05, c055, c005, c01, c1 = (sb.node("SCALAR", [v]) for v in (0.6, 0.5, 0.55, 0.05, 0.1, 1.0))
    r_ch = sb.node("MATHS", inputs={0: out(octave), 1: out(c06)}, op=abi.MATHS_MULTIPLY)
    g_ch = sb.node("MATHS", inputs={0: out(vor), 1: out(c05)}, op=abi.MATHS_MULTIPLY)
    alb = sb.node("MERGE_RGBA", inputs={0: out(r_ch), 1: out(g_ch), 2: out(c01), 3: out(c1)})
    rough_n = sb.node("MATHS", inputs={0: out(vor), 1: out(c055)}, op=abi.MATHS_MULTIPLY)
    rough = sb.node("MATHS", inputs={0: out(rough_n), 1: out(c005)}, op=abi.MATHS_ADD)
    ggx = sb.node("BXDF_MICROFACET_R", [abi.DIST_TROWBRIDGE_REITZ, 1.5],
                  {0: out(alb), 1: out(rough)})
    m_ground = sb.material(ggx)
    sb.obj(sb.mesh(verts, tris, n.reshape(-1, 3), tg4.reshape(-1, 4), uv.reshape(-1, 2)), m_ground)
    # emitters: uniform over the terrain surface (area-weighted triangle choice)
    rng = np.random.RandomState(seed + 1)
    V = verts.astype(np.float64)
    e1 = V[tris[:, 1]] - V[tris[:, 0]]
    e2 = V[tris[:, 2]] - V[tris[:, 0]]
    fn = np.cross(e1, e2)
    area = 0.5 * np.linalg.norm(fn, axis=1)
    cdf = np.cumsum(area)
    pick = np.searchsorted(cdf, rng.uniform(0, cdf[-1], n_emitters))
    r1, r2 = rng.uniform(size=n_emitters), rng.uniform(size=n_emitters)
    s = np.sqrt(r1)
    P = V[tris[pick, 0]] * (1 - s)[:, None] + V[tris[pick, 1]] * (s * (1 - r2))[:, None] + V[tris[pick, 2]] * (s * r2)[:, None]
    N = fn[pick] / np.linalg.norm(fn[pick], axis=1, keepdims=True)
    temps = rng.uniform(2000, 10000, n_emitters)
    inten = np.exp(rng.uniform(np.log(0.1), np.log(100.0), n_emitters))
    black = sb.node("BXDF_LAMBERTIAN", inputs={0: (0, 0, 0, 1)})
    ang = rng.uniform(0, 2 * np.pi, n_emitters)
    for i in range(n_emitters):
        nrm = N[i]
        t0 = np.cross(nrm, [0.0, 0.0, 1.0])
        t0 /= np.linalg.norm(t0)
        t1 = np.cross(nrm, t0)
        sz = 0.35
        dirs = [math.cos(ang[i] + k * 2 * math.pi / 3) * t0 + math.sin(ang[i] + k * 2 * math.pi / 3) * t1 for k in range(3)]
        c0 = P[i] + nrm * 1e-3
        tv = np.array([c0 + sz * d for d in dirs])
        tri = np.array([[0, 1, 2]], np.uint32)
        if np.dot(np.cross(tv[1] - tv[0], tv[2] - tv[0]), nrm) < 0:
            tri = np.array([[0, 2, 1]], np.uint32)
        emis = blackbody_emission(sb, float(temps[i]))
        m = sb.material(black, light=len(sb.lights))
        o = sb.obj(sb.mesh(tv, tri), m)
        sb.light_mesh(o, emis, float(inten[i]))
    sb.light_env(sky_texture(), 1.0)
    cam = Camera((-30.0, 22.0, -38.0), (5.0, -2.0, 5.0), fov=1.1)
    opts = abi.render_opts(width, height, spp, max_depth)
    return sb, cam, opts


# ------------------------------------------------------------------ config: volume + instancing
def volume(width=1280, height=720, spp=128, max_depth=12, n_instances=1000, sphere_res=(224, 224), seed=4):
    sb = SceneBuilder()
    sb.has_volumes = True
    med = sb.medium(0.05, 0.5, 0.3)
    rng = np.random.RandomState(seed)

    def disp(d):
        return 0.08 * gradient_noise_2d(d[..., 0] * 4 + d[..., 2] * 3, d[..., 1] * 4 + 7.0, 11)
    sv, st, sn, stg, suv = latlong_sphere(sphere_res[0], sphere_res[1], 1.0, disp)
    proxy = sb.mesh(sv, st, sn, stg, suv)
    diel = sb.node("BXDF_FRESNEL", inputs={0: (1, 1, 1, 1), 1: 1.5})
    on = sb.node("BXDF_OREN_NAYAR_R", inputs={0: (0.7, 0.5, 0.3, 1), 1: math.radians(20.0)})
    gx = sb.node("BXDF_MICROFACET_R", [abi.DIST_TROWBRIDGE_REITZ, 1.5], {0: (0.8, 0.8, 0.8, 1), 1: 0.3})
    mix = sb.node("BXDF_MIX", inputs={0: out(on), 1: out(gx), 2: 0.5})
    m_diel, m_mix = sb.material(diel), sb.material(mix)
    for i in range(n_instances):
        R = rotation_matrix(rng) * rng.uniform(0.5, 2.0)
        t = rng.uniform([-28, -2, -28], [28, 14, 28])
        sb.obj(proxy, m_diel if i % 2 == 0 else m_mix, affine(R, t))
    floor = sb.node("BXDF_LAMBERTIAN", inputs={0: (0.5, 0.5, 0.5, 1)})
    fv, ft = quad((-40, -4, -40), (-40, -4, 40), (40, -4, 40), (40, -4, -40))
    sb.obj(sb.mesh(fv, ft), sb.material(floor))
    # medium box (null surface: media boundary only), 12 triangles
    lo, hi = np.array([-12.0, -3.9, -12.0]), np.array([12.0, 8.0, 12.0])
    bv = np.array([[lo[0], lo[1], lo[2]], [hi[0], lo[1], lo[2]], [hi[0], hi[1], lo[2]], [lo[0], hi[1], lo[2]],
                   [lo[0], lo[1], hi[2]], [hi[0], lo[1], hi[2]], [hi[0], hi[1], hi[2]], [lo[0], hi[1], hi[2]]])
    bt = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5], [0, 5, 4], [3, 6, 2], [3, 7, 6],
                   [0, 4, 7], [0, 7, 3], [1, 2, 6], [1, 6, 5]], np.uint32)   # outward normals
    sb.obj(sb.mesh(bv, bt), sb.material(-1, medium_interior=med))
    white = out(sb.node("RGB", [1.0, 0.95, 0.9]))
    for i in range(16):
        p = rng.uniform([-25, 2, -25], [25, 16, 25])
        sb.light_point(p, white, float(rng.uniform(50, 200)))
    for i in range(4):
        p = rng.uniform([-15, 18, -15], [15, 22, 15])
        sb.light_spot(p, (0, -1, 0), math.radians(30.0), math.radians(24.0), white, 400.0)
    cam = Camera((0.0, 10.0, -60.0), (0.0, 2.0, 0.0), fov=0.9)
    opts = abi.render_opts(width, height, spp, max_depth)
    return sb, cam, opts


CONFIGS = {"cornell": cornell, "terrain": terrain, "volume": volume}
