"""torch.autograd binding of the adjoint (lambda_gb300.autograd.render): its gradients equal a
direct lgpu_adjoint call, and the texture gradient matches a common-random-number central
difference of the forward without Russian roulette (albedo then moves no sampling decision).
eps = 1e-2: at 1e-3 the float32 film limits the difference to about 1e-3 relative on this small
frame; the remaining error (third-order terms of paths meeting one texel three times) is far
below the 3e-3 tolerance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W = H = 32
SPP = 256
CAM = 3


def _scene_fn(configs):
    def fn(albedo, roughness, sigma_a, sigma_s):
        return configs.cornell_inverse(W, H, SPP, tex_res=8, albedo=albedo, roughness=roughness, sigma_a=sigma_a,
                                       sigma_s=sigma_s)[0]
    return fn


def test_autograd_gradients(gpu_lib):
    torch = pytest.importorskip("torch")
    from lambda_gb300 import autograd, configs
    rng = np.random.RandomState(5)
    w = torch.from_numpy(rng.uniform(0, 1, (H, W, 3)).astype(np.float32)).cuda()
    a0 = rng.uniform(0.1, 0.9, (8, 8, 3)).astype(np.float32)
    sb, cams, opts = configs.cornell_inverse(W, H, SPP, tex_res=8, albedo=a0)
    opts.min_bounces = opts.max_bounces          # no Russian roulette
    cam, fn, params = cams[CAM], _scene_fn(configs), (0, 0, 4, 0)
    albedo = torch.tensor(a0, requires_grad=True)
    scalars = torch.tensor([0.3, 0.1, 0.8], requires_grad=True)
    img = autograd.render(fn, cam, opts, params, albedo, scalars)
    assert img.shape == (H, W, 3) and torch.isfinite(img).all()
    (img * w).sum().backward()
    ga, gs = albedo.grad.numpy().astype(np.float64), scalars.grad.numpy().astype(np.float64)

    # the same adjoint called directly
    r = gpu_lib.Renderer(fn(a0, 0.3, 0.1, 0.8))
    try:
        d = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
        d[..., :3] = w
        gt = torch.zeros((8, 8, 4), dtype=torch.float32, device="cuda")
        g3 = torch.zeros(3, dtype=torch.float32, device="cuda")
        r.adjoint(cam, opts, params, d.data_ptr(), gt.data_ptr(), g3.data_ptr())
        torch.cuda.synchronize()
    finally:
        r.close()
    # (gradients are accumulated with float atomics: equal up to summation order)
    np.testing.assert_allclose(ga, gt.cpu().numpy()[..., :3], rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(gs, g3.cpu().numpy(), rtol=1e-4, atol=1e-6)

    # CRN central difference of the forward along a random texture direction
    v = rng.uniform(-1, 1, (8, 8, 3)).astype(np.float32)
    eps = 1e-2

    def loss(a):
        with torch.no_grad():
            im = autograd.render(fn, cam, opts, params, torch.from_numpy(a), torch.tensor([0.3, 0.1, 0.8]))
            return float((im.double() * w.double()).sum())
    fd = (loss(a0 + eps * v) - loss(a0 - eps * v)) / (2 * eps)
    adj = float(np.sum(ga * v))
    assert abs(adj - fd) <= 3e-3 * abs(fd) + 1e-6, (adj, fd)
