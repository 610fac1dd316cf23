"""Shared helpers for the test modules (scene builders, error metrics)."""
import numpy as np


def rel_err(a, b):
    """max |a - b| / max |b| over all entries (complex allowed)."""
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))


def random_scene(seed, n_src=7, n_snk=45, n_tris=60, box=1.0, src_z=-2.0, snk_r=4.0):
    """Small random scene: sources below, sinks on a sphere, triangles in a box."""
    rng = np.random.default_rng(seed)
    src = np.stack([rng.uniform(-0.5, 0.5, n_src), rng.uniform(-0.5, 0.5, n_src),
                    np.full(n_src, src_z)], 1).astype(np.float32)
    d = rng.normal(size=(n_snk, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    snk = (snk_r * d).astype(np.float32)
    snk_n = (-d).astype(np.float32)
    c = rng.uniform(-box, box, size=(n_tris, 3))
    v = (c[:, None, :] + rng.uniform(-0.3, 0.3, size=(n_tris, 3, 3))).reshape(-1, 3).astype(np.float32)
    f = np.arange(3 * n_tris, dtype=np.int32).reshape(-1, 3)
    E = (rng.normal(size=(n_src, 3)) + 1j * rng.normal(size=(n_src, 3))).astype(np.complex64)
    return src, snk, snk_n, v, f, E
