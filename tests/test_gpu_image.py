"""Converged-image parity: the GPU's film against the CPU oracle's film of the same frame.

Config 0 at full size (Cornell box, 256^2, 16 spp, depth 8; the oracle itself is pinned path by path
to the reference's integrator by tests/test_oracle_reference.py).  Every path of the frame is
rendered by both; the per-pixel means must agree within a 3-sigma band of the pixel's standard error
(sample spread over its 16 paths) on at least 99.7 % of pixels, and the two images' relMSE,
mean((I - R)^2 / (R^2 + 1e-2)), must stay below 1e-5 -- both renders draw the same counter-based
random numbers, so they differ only where a path's decision flips on a rounding difference.  The
GPU film from lgpu_render (the film entry point) must also equal the sum of its per-path values.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from tests.parity import pixel_band, rel_mse

pytestmark = pytest.mark.gpu


def test_cornell_full_image_matches_oracle(gpu_lib):
    from lambda_gb300 import configs
    sb, cam, opts = configs.cornell()   # 256 x 256, 16 spp, depth 8
    n = opts.width * opts.height * opts.spp
    ids = np.arange(n, dtype=np.uint64)
    r = gpu_lib.Renderer(sb)
    try:
        g = r.render_paths(cam, opts, ids)
        film = r.render(cam, opts)
    finally:
        r.close()
    o = Oracle(sb).render_paths(cam, opts, ids)
    inside, mg, mo = pixel_band(g, o, opts.spp)
    assert inside >= 0.997, "pixels inside the 3-sigma band: %.5f" % inside
    err = rel_mse(mg.reshape(opts.height, opts.width, 3), mo.reshape(opts.height, opts.width, 3))
    assert err < 1e-5, "relMSE GPU vs oracle %.3g" % err
    sums = g[:, :3].astype(np.float64).reshape(-1, opts.spp, 3).sum(1).reshape(opts.height, opts.width, 3)
    np.testing.assert_allclose(film[..., :3], sums, rtol=1e-4, atol=1e-5)
    assert np.all(film[..., 3] == opts.spp)
