"""CPU oracle against the reference renderer's own integrators, path by path.

The fixture (tests/golden/ref_paths.npz, made by tests/golden/gen_ref_paths.py) holds radiance and the
number of random numbers drawn for seeded path ids of twelve scenes, computed by the reference's
MISVolumetricPathIntegrator / PathIntegrator / VolumetricPathIntegrator built from its own sources
(patched for the defects listed in oracle/build_ref.py) with the counter-based sampler.  The oracle
must reproduce every path: RGB within 1e-4 relative (1e-6 absolute floor) and the same number of
random numbers drawn, i.e. the same control flow.  Where the reference can be built here, the live
test also runs it on ids the fixture does not hold.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from tests.golden import gen_ref_paths as G
from tests.parity import path_agreement

SMALL = [c for c in G.CASES if c not in G.FULL]


def _check(name, ids, ref, got):
    frac, ok = path_agreement(got, ref)
    same = got[:, 3] == ref[:, 3]
    bad = np.where(~(ok & same))[0]
    assert bad.size == 0, "%s: %d of %d paths differ, first ids %s" % (name, bad.size, len(ids), ids[bad[:5]])


@pytest.mark.parametrize("name", list(G.CASES))
def test_oracle_reproduces_reference_paths(name):
    fixture = G.load()
    ids, ref = fixture[name]
    sb, cam, opts = G.case(name)
    got = Oracle(sb).render_paths(cam, opts, ids)
    _check(name, ids, ref, got)


@pytest.mark.parametrize("name", ["cornell_48", "volume_small", "zoo_power", "inverse_48"])
def test_oracle_matches_reference_live(name):
    from oracle import reference
    if not reference.available():
        pytest.skip(reference.unavailable_reason())
    from tests.parity import sample_ids
    sb, cam, opts = G.case(name)
    ids = sample_ids(opts, 3000, seed=12345)
    ref = reference.Reference(sb).render_paths(cam, opts, ids)
    got = Oracle(sb).render_paths(cam, opts, ids)
    _check(name, ids, ref, got)
