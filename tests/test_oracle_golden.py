"""The oracle's restatement against golden vectors computed by the reference renderer's own code
(tests/golden/ref_kat.npz, made by tests/golden/gen_golden.py from the reference's Fresnel,
Henyey-Greenstein, homogeneous-medium, spectrum, piecewise-distribution, camera, aperture, texture
and sampling code).

Tolerance: 2e-6 relative (1e-7 absolute) -- both sides are the same float arithmetic built with
-ffp-contract=off; the slack covers libm differences between hosts.  Indices are exact.
The one intended difference is the documented patch B3: the reference's PDFDistance is always 0
(integer division 1 / nSamples); the oracle returns the channel-averaged density."""
import ctypes as C
import pathlib
import re
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
GOLD = ROOT / "tests" / "golden" / "ref_kat.npz"
sys.path.insert(0, str(ROOT / "tests" / "golden"))
RT, AT = 2e-6, 1e-7


@pytest.fixture(scope="module")
def oracle_out():
    from oracle import oracle
    import gen_golden
    L = oracle.lib()
    return gen_golden.inputs(), gen_golden.evaluate(L, "oracle_kat_", gen_golden.inputs()), L


@pytest.fixture(scope="module")
def gold():
    g = np.load(GOLD)
    return {k[4:]: g[k] for k in g.files}


def close(a, b, rt=RT, at=AT):
    np.testing.assert_allclose(a, b, rtol=rt, atol=at, equal_nan=True)


def test_fresnel(oracle_out, gold):
    _, o, _ = oracle_out
    close(o["fr"], gold["fr"])
    close(o["fe"], gold["fe"])


def test_henyey_greenstein(oracle_out, gold):
    _, o, _ = oracle_out
    close(o["hg_p"], gold["hg_p"])
    close(o["hg_pdf"], gold["hg_pdf"])
    close(o["hg_wi"], gold["hg_wi"], at=1e-6)


def test_homogeneous_medium(oracle_out, gold):
    d, o, _ = oracle_out
    keep = [0, 1, 2, 3, 4, 5, 6, 7, 8, 10]
    close(o["med"][:, keep], gold["med"][:, keep])
    # B3: the reference's PDFDistance is identically 0; the oracle's is the channel mean of sigma_t * Tr
    assert np.all(gold["med"][:, 9] == 0)
    st = (d["med_sa"] + d["med_ss"]).astype(np.float64)
    expect = np.mean(st * np.exp(-st * np.minimum(d["med_tfar"][:, None], np.finfo(np.float32).max)), axis=1)
    close(o["med"][:, 9], expect, rt=1e-5, at=1e-30)


def test_spectrum_conversions(oracle_out, gold):
    _, o, _ = oracle_out
    close(o["fs3"], gold["fs3"], rt=1e-5)
    close(o["fs8"], gold["fs8"], rt=1e-5)
    close(o["xyz_rgb"], gold["xyz_rgb"])
    close(o["y"], gold["y"])


def test_piecewise(oracle_out, gold):
    _, o, _ = oracle_out
    for k in [k for k in gold if k.startswith("pw")]:
        close(o[k][:, [0, 1, 4, 5, 6]] if k.startswith("pw1") else o[k],
              gold[k][:, [0, 1, 4, 5, 6]] if k.startswith("pw1") else gold[k])
        if k.startswith("pw1"):
            np.testing.assert_array_equal(o[k][:, [2, 3]], gold[k][:, [2, 3]])


def test_cameras(oracle_out, gold):
    """Pinhole, thin lens (no aperture, circular, blade) and spherical rays: origin and direction."""
    d, o, _ = oracle_out
    assert gold["cam"].shape == (len(d["cam_kind"]), 6)
    close(o["cam"], gold["cam"], rt=2e-6, at=2e-6)
    # the thin lens with an aperture moves the origin off the camera position
    moved = (d["cam_kind"][:, 0] == 1) & (d["cam_kind"][:, 1] > 0) & (d["cam_lens"][:, 1] > 0.01)
    assert np.all(np.linalg.norm(gold["cam"][moved, :3] - d["cam_org"][moved], axis=1) > 1e-4)


def test_texture_bilinear_and_cosine_hemisphere(oracle_out, gold):
    """Image-texture fetch (GetPixelUVBilinear with its clamping) and cosine-hemisphere sampling."""
    _, o, _ = oracle_out
    for k in [k for k in gold if k.startswith("tex_")]:
        close(o[k], gold[k])
    close(o["cos_hemi"], gold["cos_hemi"])


def _smits_tables():
    """Wavelength knots and the 14 Smits basis curves (refl W C M Y R G B, illum W C M Y R G B)
    as compiled into the GPU module and the oracle."""
    text = (ROOT / "lambda_gb300" / "csrc" / "spectral_tables.h").read_text()

    def block(name):
        body = text.split("#define " + name + " \\")[1].split("\n\n")[0]
        return np.array([float(x.rstrip("f")) for x in re.findall(r"[-+]?\d[\d.eE+-]*f", body)], np.float32)
    lam = block("LGPU_SMITS_LAMBDA_DATA")
    basis = block("LGPU_SMITS_BASIS_DATA").reshape(14, 32)
    return lam, basis


def _bin_average(lam, vals, l0, l1, swapped_lerp):
    """AverageSpectrumSamples (core/Spectrum.cpp:70-96) in float32.  With swapped_lerp the segment
    interpolation is the reference's call Lerp(t, v_i, v_i+1) against Lerp(a, b, r) = a + (b - a) r."""
    f = np.float32
    if l1 <= lam[0]:
        return vals[0]
    if l0 >= lam[-1]:
        return vals[-1]
    s = f(0)
    if l0 < lam[0]:
        s += vals[0] * (lam[0] - l0)
    if l1 > lam[-1]:
        s += vals[-1] * (l1 - lam[-1])
    i = 0
    while l0 > lam[i + 1]:
        i += 1

    def interp(w, i):
        t = f((w - lam[i]) / (lam[i + 1] - lam[i]))
        return f(t + (vals[i] - t) * vals[i + 1]) if swapped_lerp else f(vals[i] + (vals[i + 1] - vals[i]) * t)
    while i + 1 < len(lam) and l1 >= lam[i]:
        a, b = max(l0, lam[i]), min(l1, lam[i + 1])
        s += f(0.5) * (interp(a, i) + interp(b, i)) * f(b - a)
        i += 1
    return f(s / f(l1 - l0))


def _smits_weights(rgb, illum):
    """SampledSpectrum::FromRGB (core/Spectrum.cpp:104-187): basis index -> weight, and the scale."""
    r, g, b = (float(x) for x in rgb)
    W, Cy, M, Y, R, G, B = range(7)
    if r <= g and r <= b:
        w = {W: r, Cy: (g - r) if g <= b else (b - r)}
        w.update({B: b - g} if g <= b else {G: g - b})
    elif g <= r and g <= b:
        w = {W: g, M: (r - g) if r <= b else (b - g)}
        w.update({B: b - r} if r <= b else {R: r - b})
    else:
        w = {W: b, Y: (r - b) if r <= g else (g - b)}
        w.update({G: g - r} if r <= g else {R: r - g})
    off = 7 if illum else 0
    return {k + off: v for k, v in w.items()}, (0.86445 if illum else 0.94)


def _init_edges():
    """Bin edges of SampledSpectrum::Init (core/Spectrum.h:246-252): Lerp is instantiated with the
    unsigned wavelength bounds, so every edge is truncated to a whole nanometre."""
    return [np.float32(int(np.float32(400) + np.float32(300) * (np.float32(i) * np.float32(1 / 32)))) for i in range(33)]


def _smits_bins(rgb, illum, lam, basis, swapped_lerp):
    edges = _init_edges()
    w, scale = _smits_weights(rgb, illum)
    out = np.zeros(32)
    for j, wt in w.items():
        out += wt * np.array([_bin_average(lam, basis[j], edges[i], edges[i + 1], swapped_lerp) for i in range(32)],
                             np.float64)
    return np.maximum(out * scale, 0)


def test_smits_golden_explained_by_reference_code(gold, oracle_out):
    """Step 1: the reference's 32 Smits bins are reproduced by restating FromRGB and its bin
    averaging -- including the argument order of its Lerp call, a defect of the reference (the
    interpolated value is t + (v_i - t) v_i+1).  It affects only the SampledSpectrum build."""
    d, _, _ = oracle_out
    lam, basis = _smits_tables()
    for illum in (0, 1):
        for i, rgb in enumerate(d["rgb"][:20]):
            np.testing.assert_allclose(_smits_bins(rgb, illum, lam, basis, True), gold["smits_bins"][illum, i],
                                       rtol=1e-5, atol=1e-6)


def test_smits_oracle_matches_patched_reference(oracle_out):
    """Step 2: the oracle's Smits upsampling at a wavelength (hero-wavelength mode), averaged over
    each bin, equals the same restatement with the Lerp defect patched."""
    d, _, L = oracle_out
    L.oracle_smits.argtypes = [C.c_void_p, C.c_int, C.c_float]
    L.oracle_smits.restype = C.c_float
    lam, basis = _smits_tables()
    edges = _init_edges()
    for illum in (0, 1):
        for rgb in d["rgb"][:20]:
            rgb = np.ascontiguousarray(rgb)
            bins = []
            for b in range(32):
                x = np.linspace(edges[b], edges[b + 1], 129)
                v = np.array([L.oracle_smits(C.c_void_p(rgb.ctypes.data), illum, float(t)) for t in x])
                bins.append(np.trapezoid(v, x) / (x[-1] - x[0]))
            np.testing.assert_allclose(bins, _smits_bins(rgb, illum, lam, basis, False), atol=2e-3, rtol=0)


def test_live_reference_library_matches_golden():
    """Where the reference tree is present, the golden file is what its code computes now."""
    from oracle import build_ref
    lib = build_ref.build()
    if lib is None:
        pytest.skip("reference tree not present")
    import gen_golden
    o = gen_golden.evaluate(C.CDLL(str(lib)), "ref_", gen_golden.inputs())
    g = np.load(GOLD)
    for k, v in o.items():
        close(v, g["out_" + k])
