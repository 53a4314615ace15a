"""The 8-wide compressed BVH layout (a build with LGPU_BVH_WIDE=1, in lambda_gb300/_build_wide):
closest hits against the oracle and per-path agreement with the reference's own integrator, the
same checks the default binary-node build passes.  The library is chosen per process, so the checks
run in a child pytest with LGPU_LIB_PATH pointing at the variant."""
import os
import pathlib
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = pathlib.Path(__file__).resolve().parents[1]


def test_wide_bvh_layout(gpu_lib):
    from lambda_gb300.build_ext import build
    lib = build(out_dir=ROOT / "lambda_gb300" / "_build_wide", defines=["LGPU_BVH_WIDE=1"])
    env = dict(os.environ, LGPU_LIB_PATH=str(lib))
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider",
                        "tests/test_gpu_intersect.py", "tests/test_gpu_reference.py"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=3000)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert " passed" in r.stdout and " failed" not in r.stdout, r.stdout[-2000:]
