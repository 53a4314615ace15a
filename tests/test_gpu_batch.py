"""Batched views (lgpu_render_batch): every view's film must equal the film of the same view
rendered alone (same paths, same random numbers, same per-pixel summation order), whatever the pool
size and however the views share it.  The megakernel batch scheme sums with atomics, so it is
compared within 1e-4 relative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _views(Camera):
    return [(Camera((0, 0, -3.4), (0, 0, 0), fov=0.75), 32, 24, 4, 8, 1),
            (Camera((0.4, 0.2, -3.0), (0, 0, 0), fov=0.9), 16, 16, 1, 4, 2),
            (Camera((-0.5, -0.3, -3.2), (0, 0.1, 0), fov=0.7), 40, 40, 8, 6, 3),
            (Camera((0, 0.6, -2.5), (0, -0.2, 0), fov=1.0), 8, 64, 2, 12, 4),
            (Camera((0, 0, -3.4), (0, 0, 0), fov=0.75), 8, 8, 2, 0, 5)]   # depth 0: black, sample counts only


def _render_batch(torch, r, views, opts):
    films = [torch.zeros((h, w, 4), dtype=torch.float32, device="cuda") for (_, w, h, _, _, _) in views]
    r.render_batch([(c, w, h, spp, d, seed, f.data_ptr()) for (c, w, h, spp, d, seed), f in zip(views, films)], opts)
    torch.cuda.synchronize()
    return [f.cpu().numpy() for f in films]


def _render_alone(torch, r, views, opts):
    out = []
    for cam, w, h, spp, depth, seed in views:
        opts.width, opts.height, opts.spp, opts.max_bounces, opts.seed = w, h, spp, depth, seed
        f = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
        r.render_device(cam, opts, f.data_ptr())
        torch.cuda.synchronize()
        out.append(f.cpu().numpy())
    return out


@pytest.mark.parametrize("pool,mode", [(0, 2), (700, 2), (0, 3), (700, 3)],
                         ids=["host_loop", "host_loop_small_pool", "graph", "graph_small_pool"])
def test_batch_equals_single_views_cornell(gpu_lib, pool, mode):
    torch = pytest.importorskip("torch")
    from lambda_gb300 import abi, configs
    from lambda_gb300.scene import Camera
    sb, _, opts = configs.cornell(16, 16, 1)
    opts.pool_slots = pool
    opts.kernel_mode = mode
    views = _views(Camera)
    r = gpu_lib.Renderer(sb)
    try:
        batch = _render_batch(torch, r, views, opts)
        assert r.stats()["paths"] == sum(w * h * spp for (_, w, h, spp, _, _) in views)
        opts.kernel_mode = abi.KERNEL_WAVEFRONT
        alone = _render_alone(torch, r, views, opts)
        for (cam, w, h, spp, _, _), b, a in zip(views, batch, alone):
            assert np.all(b[..., 3] == spp)
            np.testing.assert_allclose(b, a, rtol=1e-6, atol=1e-7)
    finally:
        r.close()


def test_batch_megakernel_matches_wavefront_hero_volume(gpu_lib):
    torch = pytest.importorskip("torch")
    from lambda_gb300 import abi, configs
    from lambda_gb300.scene import Camera
    sb, _, opts = configs.volume(16, 16, 1, max_depth=12, n_instances=40, sphere_res=(24, 24))
    opts.spectral_mode = abi.SPECTRAL_HERO4
    views = [(Camera((0.0, 10.0, -60.0), (0.0, 2.0, 0.0), fov=0.9), 24, 16, 4, 12, 7),
             (Camera((20.0, 8.0, -50.0), (0.0, 2.0, 0.0), fov=0.8), 16, 16, 2, 6, 8)]
    r = gpu_lib.Renderer(sb)
    try:
        opts.kernel_mode = abi.KERNEL_WAVEFRONT
        wave = _render_batch(torch, r, views, opts)
        opts.kernel_mode = abi.KERNEL_MEGAKERNEL
        mega = _render_batch(torch, r, views, opts)
        for w_, m_ in zip(wave, mega):
            assert np.isfinite(w_).all()
            np.testing.assert_allclose(w_, m_, rtol=1e-4, atol=1e-5)
    finally:
        r.close()


def test_batch_rejects_bad_view(gpu_lib):
    torch = pytest.importorskip("torch")
    from lambda_gb300 import configs
    from lambda_gb300.scene import Camera
    sb, _, opts = configs.cornell(16, 16, 1)
    r = gpu_lib.Renderer(sb)
    try:
        f = torch.zeros((4, 4, 4), dtype=torch.float32, device="cuda")
        with pytest.raises(gpu_lib.LambdaGPUError, match="spp"):
            r.render_batch([(Camera((0, 0, -3.4), (0, 0, 0)), 4, 4, 0, 4, 1, f.data_ptr())], opts)
    finally:
        r.close()


def test_autotune_then_auto_mode(gpu_lib):
    """The autotuner times its candidates on a probe and AUTO renders then use the winner; the
    films still match the plain wavefront (exactly, or within the atomic-order tolerance when the
    megakernel wins)."""
    torch = pytest.importorskip("torch")
    from lambda_gb300 import abi, configs
    from lambda_gb300.scene import Camera
    sb, _, opts = configs.cornell(16, 16, 1)
    views = _views(Camera)[:3]
    r = gpu_lib.Renderer(sb)
    try:
        t = r.autotune([v + (0,) for v in views], opts, probe_spp=1)
        assert t["kernel_mode"] in (abi.KERNEL_MEGAKERNEL, abi.KERNEL_WAVEFRONT, abi.KERNEL_WAVEFRONT_GRAPH)
        assert t["tried"] >= 5 and t["mpaths_per_s"] > 0
        opts.kernel_mode = abi.KERNEL_AUTO
        auto = _render_batch(torch, r, views, opts)
        opts.kernel_mode = abi.KERNEL_WAVEFRONT
        opts.pool_slots, opts.block_size = 0, 0
        ref = _render_batch(torch, r, views, opts)
        for a, b in zip(auto, ref):
            np.testing.assert_allclose(a, b, rtol=1e-4, atol=1e-5)
    finally:
        r.close()
