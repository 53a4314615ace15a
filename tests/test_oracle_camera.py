"""The oracle's cameras on the CPU: the masked aperture's restatement (MaskedAperture,
src/camera/Aperture.cpp:29-51) -- its points follow the mask -- and the ray of each camera type at
known film coordinates.  Pinhole, thin-lens (no aperture, circular, blade) and spherical rays are
also pinned against the reference's own camera code in test_oracle_golden.py."""
import ctypes as C

import numpy as np
import pytest

from lambda_gb300 import configs
from lambda_gb300.scene import Camera


def _lib():
    from oracle import oracle
    L = oracle.lib()
    L.oracle_camera_ray.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_void_p,
                                    C.c_void_p, C.c_void_p]
    return oracle, L


def _ray(L, handle, cam, w, h, u, v, ap_u):
    o, d = np.zeros(3, np.float32), np.zeros(3, np.float32)
    ap = np.ascontiguousarray(ap_u, np.float32)
    cd = cam.desc()
    L.oracle_camera_ray(handle, C.byref(cd), w, h, u, v, ap.ctypes.data, o.ctypes.data, d.ctypes.data)
    return o, d


def test_masked_aperture_follows_mask():
    oracle, L = _lib()
    sb, cam0, _ = configs.cornell(8, 8, 1)
    mask = np.zeros((16, 16, 4), np.float32)
    mask[:8, 8:, 0] = 1.0            # only rows 0-7, columns 8-15 open (|red| is the density)
    mask[:8, 8:, 0][2, 3] = -2.0     # negative red counts by magnitude
    t = sb.texture(mask, aperture_mask=True)
    o = oracle.Oracle(sb)
    size = 0.4
    cam = Camera(cam0.origin, cam0.origin + cam0.z, fov=cam0.fov, kind="thin_lens", focal_length=3.0,
                 aperture="masked", aperture_size=size, aperture_mask=t)
    rng = np.random.RandomState(3)
    pts = []
    for _ in range(400):
        org, _d = _ray(L, o._h, cam, 64, 64, 0.5, 0.5, rng.uniform(0, 1, 2))
        off = org - cam.origin
        pts.append([np.dot(off, cam.x), np.dot(off, cam.y)])
    pts = np.array(pts)
    # Piecewise2D sample (x, y) in [0, 1)^2 mapped to (x, y) * size - size / 2
    sx, sy = pts[:, 0] / size + 0.5, pts[:, 1] / size + 0.5
    assert np.all((sx >= 0.5 - 1e-5) & (sx <= 1 + 1e-5)), "column range of the open block"
    assert np.all((sy >= -1e-5) & (sy <= 0.5 + 1e-5)), "row range of the open block"
    # the texel with negative red is open too (density |red|)
    cell = (np.floor(sy * 16).astype(int) == 2) & (np.floor(sx * 16).astype(int) == 11)
    assert cell.sum() > 0
    o.close()


@pytest.mark.parametrize("kind", ["pinhole", "thin_lens", "spherical"])
def test_camera_rays_unit_and_centred(kind):
    oracle, L = _lib()
    cam = Camera((0.5, -0.2, -3.0), (0.0, 0.1, 0.0), fov=0.9, kind=kind, focal_length=2.0, aperture="circular",
                 aperture_size=0.0, offset_phi=0.0, offset_theta=0.0)
    o, d = _ray(L, None, cam, 64, 48, 0.5, 0.5, [0.3, 0.7])
    assert abs(np.linalg.norm(d) - 1) < 1e-5
    if kind == "spherical":
        # u = v = 1/2: phi = pi, theta = pi/2 -> -x axis of the camera frame
        np.testing.assert_allclose(d, -cam.x, atol=1e-5)
    else:
        # the centre of the film looks down z; a circular aperture of size 0 sits at -size/2 = 0
        np.testing.assert_allclose(d, cam.z, atol=1e-5)
        np.testing.assert_allclose(o, cam.origin, atol=1e-6)


def test_masked_aperture_needs_flagged_texture():
    oracle, L = _lib()
    sb, cam0, opts = configs.cornell(4, 4, 1)
    t = sb.texture(np.ones((4, 4, 4), np.float32))           # not flagged: no distribution
    o = oracle.Oracle(sb)
    cam = Camera(cam0.origin, cam0.origin + cam0.z, kind="thin_lens", aperture="masked", aperture_size=0.1,
                 aperture_mask=t)
    with pytest.raises(ValueError):
        o.render_paths(cam, opts, np.arange(4, dtype=np.uint64))
    o.close()


def test_camera_descriptor_fields():
    """scene.Camera fills lgpu_camera_desc: kind and aperture codes, lens values, spherical offsets,
    and an orthonormal frame with z towards the target."""
    from lambda_gb300 import abi
    c = Camera((1.0, 2.0, 3.0), (1.0, 2.0, 10.0), fov=0.7, kind="thin_lens", focal_length=2.5, aperture="blade",
               aperture_size=0.2, blades=5)
    d = c.desc()
    assert (d.type, d.aperture, d.blades) == (abi.CAMERA_THIN_LENS, abi.APERTURE_BLADE, 5)
    assert d.focal_length == pytest.approx(2.5) and d.aperture_size == pytest.approx(0.2) and d.fov == pytest.approx(0.7)
    x, y, z = (np.array(v) for v in (d.x_hat, d.y_hat, d.z_hat))
    np.testing.assert_allclose(z, [0, 0, 1], atol=1e-6)
    np.testing.assert_allclose([x @ y, y @ z, z @ x], 0, atol=1e-6)
    s = Camera((0, 0, 0), (0, 0, 1), kind="spherical", offset_phi=0.25, offset_theta=-0.5).desc()
    assert s.type == abi.CAMERA_SPHERICAL and s.offset_phi == pytest.approx(0.25) and s.offset_theta == pytest.approx(-0.5)
    assert Camera((0, 0, 0), (0, 0, 1)).desc().type == abi.CAMERA_PINHOLE


def test_texture_mask_flag_in_scene_descriptor():
    sb, _cam, _opts = configs.cornell(4, 4, 1)
    a = sb.texture(np.ones((2, 3, 4), np.float32))
    b = sb.texture(np.ones((5, 4, 3), np.float32), aperture_mask=True)
    d = sb.desc()
    assert d.num_textures == 2
    assert (d.textures[a].aperture_mask, d.textures[a].width, d.textures[a].height) == (0, 3, 2)
    assert (d.textures[b].aperture_mask, d.textures[b].width, d.textures[b].height) == (1, 4, 5)
