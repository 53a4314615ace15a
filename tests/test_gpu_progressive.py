"""Progressive passes (lgpu_render_progressive) and the film resolve (lgpu_film_resolve): two passes
of 2 spp give the film of one 4-spp render (the same sample indices), and the resolved RGBA is the
per-pixel mean with alpha 1."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [1, 2], ids=["megakernel", "wavefront"])
def test_progressive_equals_single_render(gpu_lib, mode):
    torch = pytest.importorskip("torch")
    from lambda_gb300 import configs
    sb, cam, opts = configs.cornell(24, 20, 2)
    opts.kernel_mode = mode
    r = gpu_lib.Renderer(sb)
    try:
        film = torch.zeros((20, 24, 4), dtype=torch.float32, device="cuda")
        rgba = torch.zeros_like(film)
        r.render_progressive(cam, opts, 2, film.data_ptr(), rgba.data_ptr())
        opts.spp = 4
        ref = torch.zeros_like(film)
        r.render_device(cam, opts, ref.data_ptr())
        torch.cuda.synchronize()
        f, g, a = film.cpu().numpy(), ref.cpu().numpy(), rgba.cpu().numpy()
        assert np.all(f[..., 3] == 4)
        np.testing.assert_allclose(f, g, rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(a[..., :3], f[..., :3] / f[..., 3:4], rtol=1e-6, atol=1e-7)
        assert np.all(a[..., 3] == 1)
    finally:
        r.close()
