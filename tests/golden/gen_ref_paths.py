"""Generate tests/golden/ref_paths.npz: per-path radiance computed by the REFERENCE renderer's own
integrators (lambda::MISVolumetricPathIntegrator::Li, PathIntegrator::Li, VolumetricPathIntegrator::Li
with their scene, light, BSDF, graph and medium code), built from a patched copy of the reference
sources by oracle/build_ref.py and driven by oracle/ref_li.cpp with the counter-based sampler.

Each case is a seeded scene of lambda_gb300.configs, a camera, render options and a seeded sample of
path ids; the fixture stores the ids and, per path, RGB radiance plus the number of random numbers
drawn.  The CPU oracle and the GPU module are checked against these values (tests/
test_oracle_reference.py, tests/test_gpu_reference.py).  The reference needs its source tree, so this
runs where that exists:

    python tests/golden/gen_ref_paths.py <reference_root>     (or LAMBDA_REFERENCE_ROOT)
"""
import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[2]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
OUT = pathlib.Path(__file__).resolve().parent / "ref_paths.npz"

# name: (scene recipe, path ids sampled); the full-size cases are the benchmark configurations
CASES = {
    "cornell_48": 2000, "terrain_small": 2000, "volume_small": 2000, "inverse_48": 2000,
    "zoo_power": 2000, "zoo_tree": 2000,
    "cornell_path": 1000, "volume_volpath": 1000, "terrain_path": 1000,
    "cornell_full": 1000, "terrain_full": 1000, "volume_full": 1000,
}
FULL = ("cornell_full", "terrain_full", "volume_full")


def case(name):
    """(scene builder, camera, render opts) of one fixture case."""
    from lambda_gb300 import abi, configs
    if name == "cornell_48":
        return configs.cornell(48, 48, 4)
    if name == "terrain_small":
        return configs.terrain(64, 36, 4, grid=96, n_emitters=300)
    if name == "volume_small":
        return configs.volume(48, 27, 4, max_depth=12, n_instances=40, sphere_res=(24, 24))
    if name == "inverse_48":
        sb, cams, opts = configs.cornell_inverse(48, 48, 4)
        return sb, cams[3], opts
    if name == "zoo_power":
        return configs.node_zoo(light_strategy=abi.LIGHT_STRATEGY_POWER)
    if name == "zoo_tree":
        return configs.node_zoo(light_strategy=abi.LIGHT_STRATEGY_TREE)
    if name == "cornell_path":
        sb, cam, opts = configs.cornell(32, 32, 4)
        opts.integrator = abi.INTEGRATOR_PATH
        return sb, cam, opts
    if name == "volume_volpath":
        sb, cam, opts = configs.volume(32, 18, 4, max_depth=8, n_instances=40, sphere_res=(24, 24))
        opts.integrator = abi.INTEGRATOR_VOLPATH
        return sb, cam, opts
    if name == "terrain_path":
        sb, cam, opts = configs.terrain(32, 18, 4, grid=64, n_emitters=100)
        opts.integrator = abi.INTEGRATOR_PATH
        return sb, cam, opts
    if name == "cornell_full":
        return configs.cornell()
    if name == "terrain_full":
        return configs.terrain()
    if name == "volume_full":
        return configs.volume()
    raise KeyError(name)


def ids_of(name, opts):
    from tests.parity import sample_ids
    return sample_ids(opts, CASES[name], seed=sum(map(ord, name)))


def load():
    """{case: (ids, per-path rgb + draws)} from the committed fixture."""
    d = np.load(OUT)
    return {k: (d["ids_" + k], d["out_" + k]) for k in CASES}


def main(ref_root=None):
    from oracle import build_ref
    from oracle.reference import Reference
    if build_ref.build_li(ref_root) is None:
        raise SystemExit("reference tree not found (pass it or set LAMBDA_REFERENCE_ROOT)")
    out = {}
    for name in CASES:
        sb, cam, opts = case(name)
        ids = ids_of(name, opts)
        ref = Reference(sb)
        out["ids_" + name] = ids
        out["out_" + name] = ref.render_paths(cam, opts, ids)
        ref.close()
        print(name, len(ids), out["out_" + name][:, :3].mean(0), flush=True)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main(*sys.argv[1:2])
