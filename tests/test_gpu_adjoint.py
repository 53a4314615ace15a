"""Path-replay adjoint (lgpu_adjoint) against common-random-number central finite differences of the
forward render, on the inverse-rendering Cornell box (textured back wall, GGX sphere, medium cube).

Loss: L = sum over pixels of w . I with fixed random weights w, so dL/dI = w.  The finite
difference re-renders with the same seed at theta +- eps.

* Albedo texture: without Russian roulette the albedo moves no sampling decision, so the difference
  is the derivative of the same estimator and must match to 1e-3 (eps = 1e-3); the same
  difference of the reference renderer's own integrator must match to 1 %; with roulette the two
  agree within 3 % at 2048 spp (eps = 1e-2).
* GGX roughness moves the microfacet sample; the replay holds it fixed and adds the score of the
  sample's validity (the reference drops a vertex's light-sampled estimate when the reflected
  direction falls below the horizon, with a probability that changes with roughness).  Checked to
  5 % (measured 0.01 % at this seed; the difference itself varies by about 2 % across seeds).
* Medium sigma_a and sigma_s move the distance sample; the difference is noisier here (it moved by
  15 % across seeds at 2048 spp while the adjoint moved by 1 %), so these are checked to 15 %.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W = H = 64
SPP = 2048
SPP_EXACT = 512
EPS = 1e-2
EPS_EXACT = 1e-3
TOL = 0.03
TOL_SCALAR = {"roughness": 0.05, "sigma_a": 0.15, "sigma_s": 0.15}
CAM = 3


def _setup(torch, lg, configs, no_rr=False, spp=None, **kw):
    sb, cams, opts = configs.cornell_inverse(W, H, spp or SPP, tex_res=8, **kw)
    opts.kernel_mode = 1          # megakernel: the estimator the adjoint replays
    if no_rr:
        opts.min_bounces = opts.max_bounces   # no Russian roulette: albedo moves no sampling decision
    r = lg.Renderer(sb)
    return r, cams[CAM], opts


def _loss(torch, lg, configs, w, no_rr=False, spp=None, **kw):
    r, cam, opts = _setup(torch, lg, configs, no_rr, spp, **kw)
    opts.kernel_mode = 2          # same paths as the megakernel, film summed in a fixed order
    try:
        film = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
        r.render_device(cam, opts, film.data_ptr())
        torch.cuda.synchronize()
        f = film.double().cpu().numpy()
        img = f[..., :3] / f[..., 3:4]
        return float(np.sum(img * w))
    finally:
        r.close()


def _adjoint(torch, lg, configs, w, no_rr=False, spp=None, **kw):
    r, cam, opts = _setup(torch, lg, configs, no_rr, spp, **kw)
    try:
        dloss = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
        dloss[..., :3] = torch.from_numpy(w.astype(np.float32)).cuda()
        gtex = torch.zeros((8, 8, 4), dtype=torch.float32, device="cuda")
        gsc = torch.zeros(3, dtype=torch.float32, device="cuda")
        # material indices of cornell_inverse: 0 = textured back wall, 4 = GGX sphere; medium 0
        r.adjoint(cam, opts, (0, 0, 4, 0), dloss.data_ptr(), gtex.data_ptr(), gsc.data_ptr())
        torch.cuda.synchronize()
        return gtex.cpu().numpy()[..., :3].astype(np.float64), gsc.cpu().numpy().astype(np.float64)
    finally:
        r.close()


@pytest.fixture(scope="module")
def setup(gpu_lib):
    torch = pytest.importorskip("torch")
    from lambda_gb300 import configs
    rng = np.random.RandomState(11)
    w = rng.uniform(0.0, 1.0, (H, W, 3))
    albedo = rng.uniform(0.1, 0.9, (8, 8, 3)).astype(np.float32)
    base = dict(albedo=albedo, roughness=0.3, sigma_a=0.1, sigma_s=0.8)
    gtex, gsc = _adjoint(torch, gpu_lib, configs, w, **base)
    gtex_nr, _ = _adjoint(torch, gpu_lib, configs, w, no_rr=True, spp=SPP_EXACT, **base)
    return torch, configs, w, base, gtex, gsc, gtex_nr


def _fd(setup, lg, no_rr=False, spp=None, eps=EPS, **delta):
    torch, configs, w, base = setup[:4]
    plus, minus = dict(base), dict(base)
    for k, v in delta.items():
        plus[k] = base[k] + eps * v
        minus[k] = base[k] - eps * v
    return (_loss(torch, lg, configs, w, no_rr, spp, **plus) - _loss(torch, lg, configs, w, no_rr, spp, **minus)) / (2 * eps)


def test_adjoint_texture_direction_exact(setup, gpu_lib):
    gtex_nr = setup[6]
    v = np.random.RandomState(3).uniform(-1, 1, (8, 8, 3)).astype(np.float32)
    fd = _fd(setup, gpu_lib, no_rr=True, spp=SPP_EXACT, eps=EPS_EXACT, albedo=v)
    adj = float(np.sum(gtex_nr * v))
    assert np.isfinite(adj) and abs(adj - fd) <= 1e-3 * abs(fd) + 1e-6, (adj, fd)


def test_adjoint_texture_direction_vs_reference_fd(setup, gpu_lib):
    """The same direction derivative against central differences of the reference renderer's own
    MIS volumetric integrator (the oracle/_ref build of its sources, tile renderer, the same
    counter-based random numbers), no roulette, eps 1e-3: within 1 %."""
    from oracle import reference as R
    if not R.available():
        pytest.skip(R.unavailable_reason())
    torch, configs, w, base = setup[:4]
    gtex_nr = setup[6]
    v = np.random.RandomState(3).uniform(-1, 1, (8, 8, 3)).astype(np.float32)

    def loss(albedo):
        kw = dict(base)
        kw["albedo"] = albedo
        sb, cams, opts = configs.cornell_inverse(W, H, SPP_EXACT, tex_res=8, **kw)
        opts.min_bounces = opts.max_bounces
        ref = R.Reference(sb)
        try:
            film = ref.render(cams[CAM], opts).astype(np.float64)
        finally:
            ref.close()
        return float(np.sum(film[..., :3] / film[..., 3:4] * w))

    fd = (loss(base["albedo"] + EPS_EXACT * v) - loss(base["albedo"] - EPS_EXACT * v)) / (2 * EPS_EXACT)
    adj = float(np.sum(gtex_nr * v))
    assert np.isfinite(adj) and abs(adj - fd) <= 1e-2 * abs(fd), (adj, fd)


def test_adjoint_texture_direction(setup, gpu_lib):
    gtex = setup[4]
    v = np.random.RandomState(3).uniform(-1, 1, (8, 8, 3)).astype(np.float32)
    fd = _fd(setup, gpu_lib, albedo=v)
    adj = float(np.sum(gtex * v))
    assert np.isfinite(adj) and abs(adj - fd) <= TOL * abs(fd), (adj, fd)


@pytest.mark.parametrize("name,idx", [("roughness", 0), ("sigma_a", 1), ("sigma_s", 2)])
def test_adjoint_scalars(setup, gpu_lib, name, idx):
    gsc = setup[5]
    fd = _fd(setup, gpu_lib, **{name: 1.0})
    assert np.isfinite(gsc[idx]) and np.sign(gsc[idx]) == np.sign(fd), (name, gsc[idx], fd)
    assert abs(gsc[idx] - fd) <= TOL_SCALAR[name] * abs(fd), (name, gsc[idx], fd)


def test_adjoint_rejects_hero_mode(gpu_lib):
    torch = pytest.importorskip("torch")
    from lambda_gb300 import abi, configs
    r, cam, opts = _setup(torch, gpu_lib, configs)
    try:
        opts.spectral_mode = abi.SPECTRAL_HERO4
        buf = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
        with pytest.raises(gpu_lib.LambdaGPUError, match="RGB3"):
            r.adjoint(cam, opts, (0, 0, 4, 0), buf.data_ptr(), buf.data_ptr(), buf.data_ptr())
    finally:
        r.close()
