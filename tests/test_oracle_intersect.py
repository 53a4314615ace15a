"""The oracle's restatement of Embree's closest hit (binned-SAH BVH, two-sided Moller-Trumbore,
tnear = 0) against brute force over every triangle, on the Cornell box (no GPU).  Pins the
restated ray-query semantics that the GPU traversal is compared with."""
import numpy as np
import pytest


def _brute(tris, o, d):
    v0, v1, v2 = tris[:, 0], tris[:, 1], tris[:, 2]
    e1, e2 = v1 - v0, v2 - v0
    p = np.cross(d, e2)
    det = np.einsum("ij,ij->i", e1, p)
    ok = np.abs(det) > 1e-12
    inv = np.where(ok, 1.0 / np.where(ok, det, 1.0), 0.0)
    s = o - v0
    u = np.einsum("ij,ij->i", s, p) * inv
    q = np.cross(s, e1)
    v = (q @ d) * inv
    t = np.einsum("ij,ij->i", e2, q) * inv
    hit = ok & (u >= 0) & (v >= 0) & (u + v <= 1) & (t > 0)
    t = np.where(hit, t, np.inf)
    k = int(np.argmin(t))
    return (t[k], k) if np.isfinite(t[k]) else (np.inf, -1)


def test_oracle_closest_hit_matches_brute_force():
    from lambda_gb300 import configs
    from oracle.oracle import Oracle
    sb, cam, opts = configs.cornell(8, 8, 1)
    tris, owner = [], []
    for oi, (m, kind, mat, x) in enumerate(sb.objects):
        assert kind == 0
        v, t = sb.meshes[m][0].astype(np.float64), sb.meshes[m][1]
        tris.append(v[t])
        owner += [(oi, j) for j in range(len(t))]
    tris = np.concatenate(tris)
    orc = Oracle(sb)
    rng = np.random.RandomState(0)
    n, agree, ties, misses = 3000, 0, 0, 0
    for _ in range(n):
        o = rng.uniform(-0.95, 0.95, 3)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        t_ref, k = _brute(tris, o, d)
        hit, t, obj, prim = orc.intersect(o.astype(np.float32), d.astype(np.float32))
        if k < 0:
            assert not hit
            misses += 1
            continue
        assert hit
        assert abs(t - t_ref) <= 1e-5 * max(1.0, t_ref)
        if (obj, prim) == owner[k]:
            agree += 1
        else:   # a tie on a shared edge: the other triangle is at the same distance
            j = owner.index((obj, prim))
            t_other, _ = _brute(tris[j:j + 1], o, d)
            assert abs(t_other - t_ref) <= 1e-5 * max(1.0, t_ref)
            ties += 1
    assert agree + ties + misses == n and misses < n // 2
    assert ties <= n * 1e-3
