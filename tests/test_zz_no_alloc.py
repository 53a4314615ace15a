"""lgpu_render_paths_noalloc (fixed scratch, caller-owned device buffers) against lgpu_render_paths.

Both run the wavefront kernels with the same counter-based random numbers, so every path must give
the same radiance (within 1e-5 relative) and draw the same number of random numbers.  Each case
calls the fixed-scratch entry point twice in a row on the same scratch, with more paths than the
pool holds, so the second call also checks that the first left nothing behind.
"""
import ctypes as C

import numpy as np
import pytest

from tests.parity import sample_ids

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-5, 1e-6


def _bind():
    from lambda_gb300 import abi, lib
    L = lib()
    vp = C.c_void_p
    L.lgpu_render_paths_noalloc.argtypes = [vp, C.POINTER(abi.CameraDesc), C.POINTER(abi.RenderOpts), vp,
                                            C.c_uint64, vp, vp]
    L.lgpu_render_paths_noalloc.restype = C.c_int
    return L


def _noalloc(torch, L, r, cam, opts, ids_dev, n):
    out = torch.full((n, 4), float("nan"), dtype=torch.float32, device="cuda")
    desc = cam.desc()
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.lgpu_render_paths_noalloc(r.handle, C.byref(desc), C.byref(opts), C.c_void_p(ids_dev.data_ptr()), n,
                                     C.c_void_p(out.data_ptr()), C.c_void_p(stream))
    assert rc == 0, L.lgpu_last_error(r.handle).decode()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _check(sb, cam, opts, n):
    torch = pytest.importorskip("torch")
    import lambda_gb300 as lg
    L = _bind()
    ids = sample_ids(opts, n)
    r = lg.Renderer(sb)
    try:
        ref = r.render_paths(cam, opts, ids)
        ids_dev = torch.from_numpy(ids.view(np.int64)).to("cuda")
        for _ in range(2):
            got = _noalloc(torch, L, r, cam, opts, ids_dev, len(ids))
            assert np.isfinite(got).all()
            np.testing.assert_allclose(got[:, :3], ref[:, :3], rtol=RTOL, atol=ATOL)
            np.testing.assert_array_equal(got[:, 3], ref[:, 3])
    finally:
        r.close()


def test_noalloc_cornell_rgb_whole_pool(gpu_lib):
    from lambda_gb300 import configs
    sb, cam, opts = configs.cornell(96, 96, 4)   # 36864 paths through the 16384-slot pool
    _check(sb, cam, opts, 96 * 96 * 4)


def test_noalloc_volume_hero_small_pool(gpu_lib):
    from lambda_gb300 import abi, configs
    sb, cam, opts = configs.volume(48, 27, 4, max_depth=12, n_instances=40, sphere_res=(24, 24))
    opts.spectral_mode = abi.SPECTRAL_HERO4
    opts.pool_slots = 1000
    _check(sb, cam, opts, 48 * 27 * 4)


def test_noalloc_paths_ending_in_spawn(gpu_lib):
    # max_bounces = 0: every path ends inside the spawn that starts it, so the pool empties after
    # each spawn and the call must start the next pool of ids itself (NaN marks unwritten paths)
    from lambda_gb300 import configs
    sb, cam, opts = configs.cornell(40, 40, 2)
    opts.max_bounces = 0
    opts.pool_slots = 700
    _check(sb, cam, opts, 40 * 40 * 2)


def test_noalloc_rejects_other_integrators(gpu_lib):
    torch = pytest.importorskip("torch")
    import lambda_gb300 as lg
    from lambda_gb300 import abi, configs
    L = _bind()
    sb, cam, opts = configs.cornell(16, 16, 1)
    opts.integrator = abi.INTEGRATOR_PATH
    r = lg.Renderer(sb)
    try:
        ids = torch.arange(16 * 16, dtype=torch.int64, device="cuda")
        out = torch.zeros((16 * 16, 4), dtype=torch.float32, device="cuda")
        desc = cam.desc()
        rc = L.lgpu_render_paths_noalloc(r.handle, C.byref(desc), C.byref(opts), C.c_void_p(ids.data_ptr()),
                                         16 * 16, C.c_void_p(out.data_ptr()), None)
        assert rc == abi.ERR_INVALID_ARG
        assert "GPU_MISVOLPATH" in L.lgpu_last_error(r.handle).decode()
    finally:
        r.close()


def test_noalloc_rejects_pool_beyond_scratch(gpu_lib):
    torch = pytest.importorskip("torch")
    import lambda_gb300 as lg
    from lambda_gb300 import abi, configs
    L = _bind()
    sb, cam, opts = configs.cornell(16, 16, 1)
    opts.pool_slots = 16384 + 1
    r = lg.Renderer(sb)
    try:
        ids = torch.arange(16 * 16, dtype=torch.int64, device="cuda")
        out = torch.zeros((16 * 16, 4), dtype=torch.float32, device="cuda")
        desc = cam.desc()
        rc = L.lgpu_render_paths_noalloc(r.handle, C.byref(desc), C.byref(opts), C.c_void_p(ids.data_ptr()),
                                         16 * 16, C.c_void_p(out.data_ptr()), None)
        assert rc == abi.ERR_INVALID_ARG
        assert "fixed scratch" in L.lgpu_last_error(r.handle).decode()
    finally:
        r.close()
