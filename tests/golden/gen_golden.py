"""Generate tests/golden/ref_kat.npz: golden vectors computed by the reference renderer's own code.

Loads oracle/_ref/libref_kat.so (built by oracle/build_ref.py from the reference's Fresnel.cpp,
HenyeyGreenstein.cpp, HomogeneousMedium.cpp, Spectrum.cpp, SPD_Data.cpp, Piecewise.cpp, Camera.cpp,
Aperture.cpp and TextureEncoding.cpp, plus the header-only texture class and sampling routines) and
evaluates it on seeded inputs.  Needs the reference tree, so it runs where that exists:

    python tests/golden/gen_golden.py <reference_root>     (or LAMBDA_REFERENCE_ROOT)
"""
import ctypes as C
import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
OUT = pathlib.Path(__file__).resolve().parent / "ref_kat.npz"
F = np.float32


def _p(a):
    return C.c_void_p(a.ctypes.data)


def unit(rng, n):
    v = rng.normal(size=(n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(F)


def inputs(seed=7):
    """Seeded inputs for every known-answer function (shared with the test)."""
    rng = np.random.RandomState(seed)
    d = {}
    c = np.concatenate([rng.uniform(-1, 1, 200), [-1, -0.5, 0, 0.5, 1, 1e-4, -1e-4]]).astype(F)
    ei = rng.choice([1.0, 1.33, 1.5, 2.4], c.size).astype(F)
    et = rng.choice([1.0, 1.5, 2.4, 1e-5, 1.33], c.size).astype(F)
    d["fr_in"] = np.stack([c, ei, et], 1)
    d["fe_in"] = np.stack([rng.choice([1.5, 1.33, 2.0], 200), rng.uniform(-1, 1, 200),
                           rng.choice([1e-5, 1.0, 1.5], 200)], 1).astype(F)
    g = np.array([-0.7, -0.3, 0.0, 0.0005, 0.3, 0.9], F)
    d["hg_g"] = np.repeat(g, 40).astype(F)
    d["hg_wo"] = unit(rng, g.size * 40)
    d["hg_wi"] = unit(rng, g.size * 40)
    d["hg_u"] = rng.uniform(0, 1, (g.size * 40, 2)).astype(F)
    n = 120
    d["med_sa"] = rng.uniform(0.01, 1, (n, 3)).astype(F)
    d["med_ss"] = rng.uniform(0.01, 1, (n, 3)).astype(F)
    d["med_ray"] = np.concatenate([rng.uniform(-1, 1, (n, 3)), unit(rng, n)], 1).astype(F)
    d["med_tfar"] = rng.choice([0.5, 3.0, 40.0, np.inf], n).astype(F)
    d["med_u"] = rng.uniform(0, 0.999, (n, 2)).astype(F)
    d["med_lp"] = rng.uniform(-3, 3, (n, 3)).astype(F)
    d["med_teq"] = rng.uniform(0, 0.5, n).astype(F)
    d["fs_lam3"] = np.tile(np.array([400, 500, 600], F), (40, 1))
    d["fs_v3"] = rng.uniform(0, 2, (40, 3)).astype(F)
    lam8 = rng.uniform(380, 720, (20, 8)).astype(F)        # unsorted: exercises the sort path
    d["fs_lam8"] = lam8
    d["fs_v8"] = rng.uniform(0, 2, (20, 8)).astype(F)
    d["xyz"] = rng.uniform(0, 1.5, (60, 3)).astype(F)
    rgb = rng.uniform(0, 1, (60, 3)).astype(F)
    rgb[:6] = np.array([[1, 1, 1], [0.73, 0.65, 0.05], [0.05, 0.65, 0.73], [0.65, 0.05, 0.73],
                        [0.2, 0.2, 0.2], [0, 0, 0]], F)
    d["rgb"] = rgb
    d["pw1_f"] = [rng.uniform(0, 1, k).astype(F) * (rng.uniform(size=k) > 0.3) for k in (1, 5, 64, 64)]
    d["pw1_f"][3][:] = 0      # all-zero function: uniform fallback
    d["pw1_u"] = np.concatenate([rng.uniform(0, 1, 30), [0.0, 0.5, 0.9999999]]).astype(F)
    d["pw2_f"] = [rng.uniform(0, 1, (4, 8)).astype(F), rng.uniform(0, 1, (16, 16)).astype(F) ** 4]
    d["pw2_u"] = rng.uniform(0, 1, (30, 2)).astype(F)
    # cameras: (type, aperture) pairs, each with random axes, fov, film size and lens values
    kinds = [(0, 0), (1, 0), (1, 1), (1, 2), (2, 0)] * 12
    d["cam_kind"] = np.array(kinds, np.int32)
    n = len(kinds)
    z = unit(rng, n)
    x = np.cross(z, np.array([0, 1, 0], F))
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    d["cam_axes"] = np.stack([x, np.cross(x, z), z], 1).astype(F)            # (n, 3, 3): x, y, z
    d["cam_org"] = rng.uniform(-5, 5, (n, 3)).astype(F)
    d["cam_fov"] = rng.uniform(0.3, 1.6, n).astype(F)
    d["cam_wh"] = rng.choice([64, 256, 1920, 1080], (n, 2)).astype(np.int32)
    d["cam_lens"] = np.stack([rng.uniform(0.5, 8, n), rng.uniform(0, 0.3, n), rng.randint(3, 9, n),
                              rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)], 1).astype(F)  # focal, size, blades, offPhi, offTheta
    d["cam_uv"] = rng.uniform(0, 1, (n, 2)).astype(F)
    d["cam_ap_u"] = rng.uniform(0, 1, (n, 8)).astype(F)
    # image texture bilinear fetch: odd sizes, edge and out-of-range coordinates (clamped)
    d["tex"] = [rng.uniform(-0.5, 2, (h, w, 4)).astype(F) for h, w in ((1, 1), (3, 5), (8, 8), (17, 6))]
    uv = rng.uniform(-0.2, 1.2, (40, 2))
    uv[:6] = [[0, 0], [1, 1], [0.9999, 0.5], [0.5, 0], [1e-7, 1 - 1e-7], [0.25, 0.75]]
    d["tex_uv"] = uv.astype(F)
    d["cos_u"] = np.concatenate([rng.uniform(0, 1, (60, 2)), [[0, 0], [1, 0], [0.5, 1]]]).astype(F)
    return d


def evaluate(L, prefix, d):
    """Run every known-answer function of library L (symbol prefix 'ref_' or 'oracle_kat_')."""
    f = lambda name: getattr(L, prefix + name)
    for n_, at, rt in [("fr_dielectric", [C.c_float] * 3, C.c_float),
                       ("fresnel_dielectric_eval", [C.c_float] * 3, C.c_float),
                       ("hg_p", [C.c_float, C.c_void_p, C.c_void_p], C.c_float),
                       ("hg_sample", [C.c_float, C.c_void_p, C.c_float, C.c_float, C.c_void_p], C.c_float),
                       ("medium", [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_void_p,
                                   C.c_float, C.c_void_p], None),
                       ("rgb_from_sampled", [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p], None),
                       ("xyz_to_rgb", [C.c_void_p, C.c_void_p], None),
                       ("rgb_y", [C.c_void_p], C.c_float),
                       ("piecewise1d", [C.c_void_p, C.c_int, C.c_float, C.c_void_p], None),
                       ("piecewise2d", [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_void_p], None),
                       ("camera_ray", [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_int,
                                       C.c_int, C.c_float, C.c_int, C.c_float, C.c_int, C.c_float, C.c_float, C.c_float,
                                       C.c_float, C.c_void_p, C.c_void_p, C.c_void_p], None),
                       ("texture_bilinear", [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_void_p], None),
                       ("cos_hemisphere", [C.c_float, C.c_float, C.c_void_p], None)]:
        f(n_).argtypes, f(n_).restype = at, rt
    o = {}
    o["fr"] = np.array([f("fr_dielectric")(*r) for r in d["fr_in"]], F)
    o["fe"] = np.array([f("fresnel_dielectric_eval")(*r) for r in d["fe_in"]], F)
    o["hg_p"] = np.array([f("hg_p")(g, _p(a), _p(b)) for g, a, b in zip(d["hg_g"], d["hg_wo"], d["hg_wi"])], F)
    hs, hw = [], []
    for g, wo, u in zip(d["hg_g"], d["hg_wo"], d["hg_u"]):
        wi = np.zeros(3, F)
        hs.append(f("hg_sample")(g, _p(wo), u[0], u[1], _p(wi)))
        hw.append(wi)
    o["hg_pdf"], o["hg_wi"] = np.array(hs, F), np.array(hw, F)
    med = []
    for i in range(len(d["med_sa"])):
        out = np.zeros(11, F)
        f("medium")(_p(d["med_sa"][i]), _p(d["med_ss"][i]), _p(d["med_ray"][i]), d["med_tfar"][i], d["med_u"][i][0],
                    d["med_u"][i][1], _p(d["med_lp"][i]), d["med_teq"][i], _p(out))
        med.append(out)
    o["med"] = np.array(med, F)
    for k in ("3", "8"):
        res = []
        for lam, v in zip(d["fs_lam" + k], d["fs_v" + k]):
            rgb = np.zeros(3, F)
            f("rgb_from_sampled")(_p(np.ascontiguousarray(lam)), _p(np.ascontiguousarray(v)), lam.size, _p(rgb))
            res.append(rgb)
        o["fs" + k] = np.array(res, F)
    res = []
    for x in d["xyz"]:
        rgb = np.zeros(3, F)
        f("xyz_to_rgb")(_p(np.ascontiguousarray(x)), _p(rgb))
        res.append(rgb)
    o["xyz_rgb"] = np.array(res, F)
    o["y"] = np.array([f("rgb_y")(_p(np.ascontiguousarray(x))) for x in d["rgb"]], F)
    for j, fn in enumerate(d["pw1_f"]):
        res = []
        for u in d["pw1_u"]:
            out = np.zeros(7, F)
            f("piecewise1d")(_p(fn), fn.size, u, _p(out))
            res.append(out)
        o["pw1_%d" % j] = np.array(res, F)
    for j, fn in enumerate(d["pw2_f"]):
        res = []
        fc = np.ascontiguousarray(fn)
        for u in d["pw2_u"]:
            out = np.zeros(4, F)
            f("piecewise2d")(_p(fc), fn.shape[1], fn.shape[0], u[0], u[1], _p(out))
            res.append(out)
        o["pw2_%d" % j] = np.array(res, F)
    res = []
    for i, (t, a) in enumerate(d["cam_kind"]):
        ax = np.ascontiguousarray(d["cam_axes"][i])
        org, dd = np.zeros(3, F), np.zeros(3, F)
        fl, size, blades, ophi, oth = d["cam_lens"][i]
        f("camera_ray")(int(t), _p(np.ascontiguousarray(d["cam_org"][i])), _p(ax[0]), _p(ax[1]), _p(ax[2]),
                        float(d["cam_fov"][i]), int(d["cam_wh"][i][0]), int(d["cam_wh"][i][1]), float(fl), int(a),
                        float(size), int(blades), float(ophi), float(oth), float(d["cam_uv"][i][0]),
                        float(d["cam_uv"][i][1]), _p(np.ascontiguousarray(d["cam_ap_u"][i])), _p(org), _p(dd))
        res.append(np.concatenate([org, dd]))
    o["cam"] = np.array(res, F)
    for j, t in enumerate(d["tex"]):
        res = []
        tc = np.ascontiguousarray(t)
        for u, v in d["tex_uv"]:
            out = np.zeros(4, F)
            f("texture_bilinear")(_p(tc), t.shape[1], t.shape[0], float(u), float(v), _p(out))
            res.append(out)
        o["tex_%d" % j] = np.array(res, F)
    res = []
    for u in d["cos_u"]:
        out = np.zeros(3, F)
        f("cos_hemisphere")(float(u[0]), float(u[1]), _p(out))
        res.append(out)
    o["cos_hemi"] = np.array(res, F)
    return o


def main(ref_root=None):
    from oracle import build_ref
    lib = build_ref.build(ref_root, force=True)
    if lib is None:
        raise SystemExit("reference tree not found (pass it or set LAMBDA_REFERENCE_ROOT)")
    L = C.CDLL(str(lib))
    d = inputs()
    o = evaluate(L, "ref_", d)
    L.ref_sampled_from_rgb.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    bins = np.zeros((2, len(d["rgb"]), 32), F)
    for illum in (0, 1):
        for i, x in enumerate(d["rgb"]):
            L.ref_sampled_from_rgb(_p(np.ascontiguousarray(x)), illum, _p(bins[illum, i]))
    o["smits_bins"] = bins
    np.savez_compressed(OUT, **{"out_" + k: v for k, v in o.items()})
    print("wrote", OUT, sum(v.size for v in o.values()), "values")


if __name__ == "__main__":
    main(*sys.argv[1:2])
