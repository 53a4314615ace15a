"""Thin-lens (no aperture, circular, blade, masked) and spherical cameras on the GPU against the
oracle, per path (same criterion as the pinhole parity tests: 1e-4 relative on >= 99 % of paths),
in the megakernel and the wavefront; batched views with mixed cameras; camera validation."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from tests.parity import path_agreement, sample_ids

pytestmark = pytest.mark.gpu

CAMS = {
    "thin_lens_none": dict(kind="thin_lens", focal_length=3.4, aperture="none"),
    "thin_lens_circular": dict(kind="thin_lens", focal_length=3.0, aperture="circular", aperture_size=0.15),
    "thin_lens_blade": dict(kind="thin_lens", focal_length=3.6, aperture="blade", aperture_size=0.2, blades=6),
    "thin_lens_masked": dict(kind="thin_lens", focal_length=3.2, aperture="masked", aperture_size=0.25),
    "spherical": dict(kind="spherical", offset_phi=0.3, offset_theta=-0.2),
}


def _scene(lg_configs):
    sb, cam0, opts = lg_configs.cornell(40, 40, 4)
    yy, xx = np.mgrid[0:16, 0:16]
    mask = np.zeros((16, 16, 4), np.float32)
    mask[..., 0] = ((xx - 7.5) ** 2 + (yy - 7.5) ** 2 < 36) * (1.0 + 0.1 * xx)   # a disc, brighter to the right
    t = sb.texture(mask, aperture_mask=True)
    return sb, cam0, opts, t


def _camera(cam0, name, t):
    from lambda_gb300.scene import Camera
    kw = dict(CAMS[name])
    if name == "spherical":   # inside the box: every direction meets a wall
        return Camera((0.0, 0.0, -0.5), (0.0, 0.0, 1.0), **kw)
    if kw.get("aperture") == "masked":
        kw["aperture_mask"] = t
    return Camera(cam0.origin, cam0.origin + cam0.z, fov=cam0.fov, **kw)


@pytest.mark.parametrize("mode", [1, 2], ids=["megakernel", "wavefront"])
@pytest.mark.parametrize("name", list(CAMS))
def test_camera_paths(gpu_lib, mode, name):
    from lambda_gb300 import configs
    sb, cam0, opts, t = _scene(configs)
    cam = _camera(cam0, name, t)
    opts.kernel_mode = mode
    ids = sample_ids(opts, opts.width * opts.height * opts.spp)
    r = gpu_lib.Renderer(sb)
    try:
        g = r.render_paths(cam, opts, ids)
    finally:
        r.close()
    o = Oracle(sb).render_paths(cam, opts, ids)
    frac, _ = path_agreement(g, o)
    assert np.isfinite(g).all()
    assert frac >= 0.999, "per-path agreement %.5f" % frac
    # random numbers drawn per path: the aperture's come before the integrator's
    assert np.mean(g[:, 3] == o[:, 3]) >= 0.999


def test_batched_views_mixed_cameras(gpu_lib):
    """A batch of a pinhole, a thin-lens and a spherical view renders the films each view renders alone."""
    import torch
    from lambda_gb300 import configs
    sb, cam0, opts, t = _scene(configs)
    cams = [cam0, _camera(cam0, "thin_lens_blade", t), _camera(cam0, "spherical", t)]
    opts.kernel_mode = 2
    r = gpu_lib.Renderer(sb)
    try:
        films = [torch.zeros((opts.height, opts.width, 4), dtype=torch.float32, device="cuda") for _ in cams]
        r.render_batch([(c, opts.width, opts.height, opts.spp, opts.max_bounces, opts.seed, f.data_ptr())
                        for c, f in zip(cams, films)], opts)
        torch.cuda.synchronize()
        for c, f in zip(cams, films):
            alone = torch.zeros_like(f)
            r.render_device(c, opts, alone.data_ptr())
            torch.cuda.synchronize()
            a, b = f.cpu().numpy(), alone.cpu().numpy()
            np.testing.assert_array_equal(a[..., 3], b[..., 3])
            np.testing.assert_allclose(a[..., :3], b[..., :3], rtol=1e-4, atol=1e-5)
    finally:
        r.close()


def test_camera_validation(gpu_lib):
    from lambda_gb300 import configs
    from lambda_gb300.scene import Camera
    sb, cam0, opts, t = _scene(configs)
    plain = sb.texture(np.ones((4, 4, 4), np.float32))            # no distribution built
    r = gpu_lib.Renderer(sb)
    try:
        bad = [Camera(cam0.origin, cam0.origin + cam0.z, kind="thin_lens", aperture="masked", aperture_mask=plain),
               Camera(cam0.origin, cam0.origin + cam0.z, kind="thin_lens", aperture="masked", aperture_mask=99),
               Camera(cam0.origin, cam0.origin + cam0.z, kind="thin_lens", aperture="blade", blades=0),
               Camera(cam0.origin, cam0.origin + cam0.z, kind="thin_lens", focal_length=float("nan"))]
        for c in bad:
            with pytest.raises(gpu_lib.LambdaGPUError):
                r.render_paths(c, opts, np.arange(8, dtype=np.uint64))

        class Odd(Camera):
            def desc(self):
                d = super().desc()
                d.type = 7
                return d
        with pytest.raises(gpu_lib.LambdaGPUError, match="camera type"):
            r.render_paths(Odd(cam0.origin, cam0.origin + cam0.z), opts, np.arange(8, dtype=np.uint64))
    finally:
        r.close()
