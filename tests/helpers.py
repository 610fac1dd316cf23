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


# Numba-engine fixtures (tests/golden/numba_engine.npz, written by make_golden.py from the reference's own
# numba engine): path-index cases (scene, max_scatter, line of sight) and per-path-product cases
# (index case, wavelength, magnetic sources, tolerance).  The reference forms path lengths and phases in
# float32, so at lambda = 0.05 m (k r ~ 250 rad on these ~2 m paths) its own output sits ~2.5e-5 from FP64,
# ten times closer at 0.5 m; the tolerances say so.
NUMBA_INDEX_CASES = [("a", 1, True), ("a", 2, True), ("a", 2, False), ("b", 3, True), ("b", 3, False),
                     ("t", 2, True)]
NUMBA_FIELD_CASES = [("a2los", 0.5, 0, 1e-5), ("a2los", 0.05, 0, 1e-4), ("a2los", 0.5, 3, 1e-5),
                     ("b3los", 0.5, 0, 1e-5)]
NUMBA_ALPHA = 0.02


def numba_golden():
    import os
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "numba_engine.npz"))


def numba_index_key(scene, max_scatter, los):
    return f"{scene}{max_scatter}{'los' if los else 'nolos'}"


def numba_golden_scene(d, scene):
    """(src, snk, scat, verts, faces, pos, nrm, w) of a fixture scene; pos / nrm / w cover
    [sources, sinks, scatter points] with +z source normals, as the fixtures were made."""
    g = lambda k: d[f"{scene}_{k}"]  # noqa: E731
    src, snk, scat = g("src"), g("snk"), g("scat")
    pos = np.concatenate([src, snk, scat])
    nrm = np.concatenate([np.tile([[0, 0, 1.0]], (src.shape[0], 1)), g("snk_n"), g("scat_n")]).astype(np.float32)
    return src, snk, scat, g("verts"), g("faces"), pos, nrm, g("w")


def numba_golden_magnetic(n_points, magnetic):
    """Magnetic flags and impedances of the fixture points (the first `magnetic` sources magnetic)."""
    mag = np.zeros(n_points, bool)
    mag[:magnetic] = True
    imp = np.full(n_points, np.sqrt(np.float32(1.25663706212e-6).astype(np.float64)
                                    / np.float32(8.8541878176e-12).astype(np.float64)), np.float32)
    return mag, imp


# visiblespace fixture cases: (label, vertex_area key or value, az_range, elev_range); shell radius 4 m
NUMBA_VS_SHELL = 4.0


def numba_vs_cases(d):
    return [("ones", np.array([0.0]), None, None), ("one_area", np.array([0.7]), None, None),
            ("areas", d["vs_area"], np.linspace(-180.0, 180.0, 13), np.linspace(-90.0, 90.0, 7))]


# calculate_scattering(cuda=False) fixture cases: (scene, scattering, los, elements, project_vectors); aperture
# normals +z and areas 0.5, desired E axis +x, lambda = 0.5 m, beta = 2 pi / lambda
NUMBA_MODEL_CASES = [("m", 0, True, False, False), ("m", 0, True, False, True), ("m", 1, True, False, False),
                     ("m", 1, False, False, False), ("m", 1, True, True, False), ("d", 2, True, False, False)]


def numba_model_key(scene, scattering, los, elements, project):
    return f"model_{scene}_{scattering}{int(los)}{int(elements)}{int(project)}"


# CUDA-engine model fixtures (tests/golden/cuda_model.npz): calculate_scattering(cuda=True) cases as keyword
# arguments, on scene "s" (5 sources, 50 sinks, 20 scatter points, 90 triangles), areas 0.5, E axis +x,
# lambda = 0.04 m; far fields on 9 azimuths x 5 elevations with farfield_distance 5.
CUDA_MODEL_LAMBDA = 0.04
CUDA_MODEL_CASES = [("s0", {}), ("s0_elements", dict(elements=True)), ("s0_project", dict(project_vectors=True)),
                    ("s1", dict(scattering=1)), ("s1_elements", dict(scattering=1, elements=True)),
                    ("s1_chunks2", dict(scattering=1, elements=True, chunks=2))]
CUDA_FARFIELD_CASES = [("ff0", {}), ("ff1", dict(scattering=1))]


def cuda_model_golden():
    import os
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cuda_model.npz"))


# time-domain model fixture cases on scene "t": (label, keyword arguments); areas 0.25, E axis +x, lambda 0.05 m,
# 20 GHz sampling, 400 samples, the excitation of the TimeDomainv3 fixture
NUMBA_TD_CASES = [("s0", dict(scattering=0, project_vectors=False)), ("s1", dict(scattering=1, project_vectors=False)),
                  ("s1_project", dict(scattering=1)),
                  ("s1_elements", dict(scattering=1, elements=True, project_vectors=False))]

