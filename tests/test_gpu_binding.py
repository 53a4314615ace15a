"""Rendering through the GPU module's Lambda-side binding (lambda_gb300/binding) on lambda::Scene
objects built by the reference's own classes (oracle/ref_li.cpp): lambda_gpu::GpuRenderer's
RenderDirective over the whole film, and the GpuTileRenderer that RenderMosaic calls per 16 x 16
tile, against the module rendering the original scene description directly.

The binding translates the scene, camera (frame and tan(fov / 2) recovered exactly), integrator and
bounce limits, so the films must be identical: same paths, same random numbers, same per-pixel
summation order (a film that starts empty takes each pixel's samples in sample order both ways)."""
import numpy as np
import pytest

from oracle import reference as R

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(R.binding_lib() is None, reason=str(R.binding_unavailable_reason()))]


def _cases():
    from lambda_gb300 import abi, configs
    return {
        "cornell_mis": lambda: configs.cornell(48, 40, 4),
        "node_zoo_tree": lambda: configs.node_zoo(light_strategy=abi.LIGHT_STRATEGY_TREE),
        "volume_instances": lambda: configs.volume(48, 32, 2, n_instances=20, sphere_res=(24, 24)),
        "cornell_inverse_textured": lambda: configs.cornell_inverse(40, 40, 4, tex_res=8),
    }


@pytest.mark.parametrize("mode", [0, 1], ids=["render_directive", "tile_renderer"])
@pytest.mark.parametrize("name", list(_cases()))
def test_binding_film_equals_direct_render(gpu_lib, name, mode):
    sb, cams, opts = _cases()[name]()
    cam = cams[0] if isinstance(cams, (list, tuple)) else cams
    direct = gpu_lib.Renderer(sb)
    try:
        want = direct.render(cam, opts)
    finally:
        direct.close()
    b = R.BindingScene(sb)
    try:
        got = b.render(cam, opts, mode=mode)
    finally:
        b.close()
    assert np.isfinite(got).all()
    assert np.array_equal(got[..., 3], want[..., 3]), "sample counts differ"
    diff = np.abs(got[..., :3] - want[..., :3])
    assert np.array_equal(got, want), "max |diff| %g at %s" % (diff.max(), np.unravel_index(diff.argmax(), diff.shape))


def test_binding_volumetric_path_integrator(gpu_lib):
    """VolumetricPathIntegrator selected through the directive's integrator object."""
    from lambda_gb300 import abi, configs
    sb, cam, opts = configs.volume(32, 32, 2, n_instances=10, sphere_res=(16, 16))
    opts.integrator = abi.INTEGRATOR_VOLPATH
    direct = gpu_lib.Renderer(sb)
    try:
        want = direct.render(cam, opts)
    finally:
        direct.close()
    b = R.BindingScene(sb)
    try:
        got = b.render(cam, opts, mode=0)
    finally:
        b.close()
    assert np.array_equal(got, want)
