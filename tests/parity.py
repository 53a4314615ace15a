"""Shared helpers for the GPU-vs-oracle parity tests (test infrastructure)."""
import numpy as np


def path_agreement(a, b, rel=1e-4, floor=1e-6):
    """Fraction of paths whose RGB radiance agrees within `rel` relative error (abs floor)."""
    a = np.asarray(a, np.float64)[:, :3]
    b = np.asarray(b, np.float64)[:, :3]
    err = np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), floor)
    ok = np.all((err <= rel) | (np.abs(a - b) <= floor), axis=1)
    return ok.mean(), ok


def sample_ids(opts, n, seed=0):
    total = opts.width * opts.height * opts.spp
    rng = np.random.RandomState(seed)
    if n >= total:
        return np.arange(total, dtype=np.uint64)
    return np.sort(rng.choice(total, n, replace=False)).astype(np.uint64)


def rel_mse(img, ref, eps=1e-2):
    """mean((I - R)^2 / (R^2 + eps)) over pixels and RGB channels (images as (H, W, >=3) means)."""
    i = np.asarray(img, np.float64)[..., :3]
    r = np.asarray(ref, np.float64)[..., :3]
    return float(np.mean((i - r) ** 2 / (r * r + eps)))


def pixel_band(paths_a, paths_b, spp, k=3.0):
    """Per-pixel means of two renders of the same frame (per-path values in pixel-major order,
    spp consecutive samples per pixel) and the fraction of pixels whose means agree within k
    standard errors of the pixel mean (standard error from the per-pixel sample spread of both)."""
    a = np.asarray(paths_a, np.float64)[:, :3].reshape(-1, spp, 3)
    b = np.asarray(paths_b, np.float64)[:, :3].reshape(-1, spp, 3)
    ma, mb = a.mean(1), b.mean(1)
    se = np.sqrt((a.var(1, ddof=1) + b.var(1, ddof=1)) / spp)
    inside = np.abs(ma - mb) <= k * se + 1e-7
    return float(np.all(inside, axis=1).mean()), ma, mb
