"""GPU path vs CPU oracle on the same seeded inputs (per path, per ray, per image).

Criteria (the oracle reproduces the reference's own integrators path by path, see
tests/test_oracle_reference.py):
  * per-path radiance within 1e-4 relative and the same number of random numbers drawn on
    >= 99.9 % of paths (the device code is built without multiply-add contraction, so it rounds as
    the reference does; the rest differ where a math-library result differs in its last bit);
  * closest-hit primitive ids agree on >= 99.99 % of rays and t within 1e-5 relative;
  * images: per-pixel means agree within a 3-sigma band of the per-pixel sample variance.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from tests.parity import path_agreement, sample_ids

pytestmark = pytest.mark.gpu

MODES = pytest.mark.parametrize("mode", [1, 2, 3], ids=["megakernel", "wavefront", "wavefront_graph"])


def _render_both(lg, sb, cam, opts, n):
    ids = sample_ids(opts, n)
    r = lg.Renderer(sb)
    g = r.render_paths(cam, opts, ids)
    o = Oracle(sb).render_paths(cam, opts, ids)
    r.close()
    return g, o


@MODES
def test_cornell_rgb_paths(gpu_lib, mode):
    from lambda_gb300 import configs
    sb, cam, opts = configs.cornell(48, 48, 4)
    opts.kernel_mode = mode
    g, o = _render_both(gpu_lib, sb, cam, opts, 48 * 48 * 4)
    frac, ok = path_agreement(g, o)
    assert np.isfinite(g).all()
    assert frac >= 0.999, "per-path agreement %.5f" % frac


@MODES
def test_cornell_hero_paths(gpu_lib, mode):
    from lambda_gb300 import abi, configs
    sb, cam, opts = configs.cornell(32, 32, 4)
    opts.kernel_mode = mode
    opts.spectral_mode = abi.SPECTRAL_HERO4
    g, o = _render_both(gpu_lib, sb, cam, opts, 32 * 32 * 4)
    frac, _ = path_agreement(g, o)
    assert frac >= 0.999, "per-path agreement %.5f" % frac


@MODES
def test_terrain_small_paths(gpu_lib, mode):
    from lambda_gb300 import configs
    sb, cam, opts = configs.terrain(64, 36, 4, grid=96, n_emitters=300)
    opts.kernel_mode = mode
    g, o = _render_both(gpu_lib, sb, cam, opts, 64 * 36 * 4)
    frac, _ = path_agreement(g, o)
    assert frac >= 0.999, "per-path agreement %.5f" % frac


@MODES
def test_volume_small_paths(gpu_lib, mode):
    from lambda_gb300 import configs
    sb, cam, opts = configs.volume(48, 27, 4, max_depth=12, n_instances=40, sphere_res=(24, 24))
    opts.kernel_mode = mode
    g, o = _render_both(gpu_lib, sb, cam, opts, 48 * 27 * 4)
    frac, _ = path_agreement(g, o)
    assert frac >= 0.999, "per-path agreement %.5f" % frac


@MODES
def test_film_matches_paths(gpu_lib, mode):
    """lgpu_render's film equals the per-pixel sum of the per-path radiance."""
    from lambda_gb300 import configs
    sb, cam, opts = configs.cornell(32, 32, 32)
    opts.kernel_mode = mode
    r = gpu_lib.Renderer(sb)
    film = r.render(cam, opts)
    ids = np.arange(32 * 32 * 32, dtype=np.uint64)
    p = r.render_paths(cam, opts, ids).reshape(32, 32, 32, 4)
    r.close()
    np.testing.assert_allclose(film[..., 3], 32.0)
    np.testing.assert_allclose(film[..., :3], p[..., :3].sum(axis=2), rtol=1e-4, atol=1e-5)


def test_wavefront_equals_megakernel_terrain(gpu_lib):
    """The two execution schemes draw the same random numbers in the same order: same paths."""
    from lambda_gb300 import configs
    sb, cam, opts = configs.terrain(64, 36, 8, grid=96, n_emitters=300)
    ids = np.arange(64 * 36 * 8, dtype=np.uint64)
    r = gpu_lib.Renderer(sb)
    opts.kernel_mode = 1
    a = r.render_paths(cam, opts, ids)
    opts.kernel_mode = 2
    opts.pool_slots = 1000   # small pool: exercises path regeneration
    b = r.render_paths(cam, opts, ids)
    opts.kernel_mode = 3      # same kernels, device-driven, bounce loop as a CUDA graph
    c = r.render_paths(cam, opts, ids)
    r.close()
    np.testing.assert_array_equal(a[:, 3], b[:, 3])
    frac, _ = path_agreement(a, b, rel=1e-5)
    assert frac >= 0.999
    np.testing.assert_array_equal(b, c)


@MODES
def test_inverse_cornell_texture_medium_paths(gpu_lib, mode):
    """Image-textured back wall (bilinear at fract(uv)), GGX sphere and a medium cube."""
    from lambda_gb300 import configs
    sb, cams, opts = configs.cornell_inverse(40, 40, 4, tex_res=16)
    opts.kernel_mode = mode
    for cam in (cams[0], cams[4]):
        g, o = _render_both(gpu_lib, sb, cam, opts, 40 * 40 * 4)
        frac, _ = path_agreement(g, o)
        assert np.isfinite(g).all()
        assert frac >= 0.999, "per-path agreement %.5f" % frac


INTEGRATORS = pytest.mark.parametrize("integ", [0, 1, 2, 3, 4], ids=["path", "volpath", "direct", "normal", "depth"])


@INTEGRATORS
@pytest.mark.parametrize("scene", ["cornell", "volume", "terrain"])
def test_other_integrators_paths(gpu_lib, integ, scene):
    """PathIntegrator, VolumetricPathIntegrator, DirectLightingIntegrator and the normal / depth
    passes (megakernel) against the oracle's restatements, per path."""
    from lambda_gb300 import configs
    if scene == "cornell":
        sb, cam, opts = configs.cornell(32, 32, 4)
    elif scene == "volume":
        sb, cam, opts = configs.volume(32, 18, 4, max_depth=12, n_instances=40, sphere_res=(24, 24))
    else:
        sb, cam, opts = configs.terrain(32, 18, 4, grid=96, n_emitters=300)
    opts.integrator = integ
    g, o = _render_both(gpu_lib, sb, cam, opts, opts.width * opts.height * 4)
    frac, _ = path_agreement(g, o)
    assert np.isfinite(g).all()
    assert frac >= 0.999, "per-path agreement %.5f" % frac
