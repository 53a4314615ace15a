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
