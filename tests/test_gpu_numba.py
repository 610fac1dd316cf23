"""GPU parity of the numba-engine entry points against the oracle's restatement.

workchunkingv2's path index must equal the oracle's row for row (visibility
is bit-exact); EMGPUFreqDomain and calculate_scattering(cuda=False) must be
within 1e-5 (max-normalised) of the oracle's FP64 per-path product."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

from helpers import (CUDA_FARFIELD_CASES, CUDA_MODEL_CASES, CUDA_MODEL_LAMBDA, NUMBA_ALPHA, NUMBA_FIELD_CASES,
                     NUMBA_INDEX_CASES, NUMBA_MODEL_CASES, NUMBA_VS_SHELL, cuda_model_golden,
                     numba_golden, numba_golden_scene, numba_index_key, numba_model_key, numba_vs_cases,
                     random_scene, rel_err)

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from lyceanem_gb300 import build
    build.build_native()


def _scene(seed=3, n_src=6, n_snk=40, n_tris=80, n_scat=25):
    src, snk, snk_n, v, f, E = random_scene(seed, n_src=n_src, n_snk=n_snk, n_tris=n_tris)
    rng = np.random.default_rng(seed + 10)
    scat = rng.uniform(-1, 1, (n_scat, 3)).astype(np.float32)
    scat_n = rng.normal(size=(n_scat, 3)).astype(np.float32)
    scat_n /= np.linalg.norm(scat_n, axis=1, keepdims=True)
    return src, snk, snk_n, v, f, E, scat, scat_n


def _no_device_errors():
    from lyceanem_gb300 import propagation as P
    assert P.device_errors() == (0, 0)


@pytest.mark.parametrize("max_scatter,los", [(1, True), (2, True), (2, False), (3, True), (3, False)])
def test_workchunkingv2_matches_oracle(max_scatter, los):
    from lyceanem_gb300 import raycasting as RC
    src, snk, snk_n, v, f, E, scat, scat_n = _scene()
    idx, rays = RC.workchunkingv2(src, snk, scat, (v, f), max_scatter, line_of_sight=los)
    masks = O.numba_masks(src, snk, scat, O.pack_triangles(v, f))
    oidx, orays = O.numba_path_index(src.shape[0], snk.shape[0], scat.shape[0], *masks, max_scatter,
                                     line_of_sight=los)
    assert idx.dtype == np.int32 and np.array_equal(idx, oidx)
    assert rays == orays
    # the triangle_t records of convertTriangles give the same index
    from lyceanem_gb300.geometry import Mesh
    recs = RC.convertTriangles(Mesh(v, [("triangle", f)]))
    idx2, _ = RC.workchunkingv2(src, snk, scat, recs, max_scatter, line_of_sight=los)
    assert np.array_equal(idx2, idx)
    _no_device_errors()


def _points(src, snk, snk_n, scat, scat_n, E, rng):
    from lyceanem_gb300.empropagation import scattering_point
    N, M, Pn = src.shape[0], snk.shape[0], scat.shape[0]
    pts = np.zeros(N + M + Pn, dtype=scattering_point)
    pos = np.concatenate([src, snk, scat])
    nrm = np.concatenate([np.tile([[0, 0, 1.0]], (N, 1)), snk_n, scat_n]).astype(np.float32)
    w = (rng.normal(size=(N + M + Pn, 3)) + 1j * rng.normal(size=(N + M + Pn, 3))).astype(np.complex64)
    w[:N] = E
    for k, c in enumerate("xyz"):
        pts[f"p{c}"] = pos[:, k]
        pts[f"n{c}"] = nrm[:, k]
        pts[f"e{c}"] = w[:, k]
    pts["Electric"] = True
    pts["permittivity"] = 8.8541878176e-12
    pts["permeability"] = 1.25663706212e-6
    return pts, pos, nrm, w


@pytest.mark.parametrize("max_scatter", [1, 2, 3])
def test_emgpufreqdomain_vs_oracle(max_scatter):
    from lyceanem_gb300 import raycasting as RC
    from lyceanem_gb300.empropagation import EMGPUFreqDomain
    src, snk, snk_n, v, f, E, scat, scat_n = _scene(seed=5)
    rng = np.random.default_rng(7)
    pts, pos, nrm, w = _points(src, snk, snk_n, scat, scat_n, E, rng)
    N, M = src.shape[0], snk.shape[0]
    idx, _ = RC.workchunkingv2(src, snk, scat, (v, f), max_scatter)
    beta = 2 * np.pi / 0.05
    S = EMGPUFreqDomain(N, M, idx, pts, 0.05, 0.02, beta)
    So = O.path_field(idx, pos, nrm, w, N, M, 0.02, beta)
    assert S.shape == (N, M, 3) and S.dtype == np.complex128
    assert rel_err(S, So) < FIELD_TOL
    # magnetic sources: the launched field is (w x d) / sqrt(mu / eps)
    pts["Electric"][: N // 2] = False
    mag = ~pts["Electric"]
    imp = np.sqrt(np.real(pts["permeability"]) / np.real(pts["permittivity"])).astype(np.float32)
    S = EMGPUFreqDomain(N, M, idx, pts, 0.05, 0.02, beta)
    So = O.path_field(idx, pos, nrm, w, N, M, 0.02, beta, magnetic=mag, impedance=imp)
    assert rel_err(S, So) < FIELD_TOL
    _no_device_errors()


def test_emgpufreqdomain_many_rows():
    """The per-path product on a path list of a few hundred thousand rows (32 sources, 400 sinks, 150 scatter
    points, one bounce) against the FP64 oracle's per-path sum."""
    from lyceanem_gb300 import raycasting as RC
    from lyceanem_gb300.empropagation import EMGPUFreqDomain
    src, snk, snk_n, v, f, E, scat, scat_n = _scene(seed=12, n_src=32, n_snk=400, n_tris=300, n_scat=150)
    rng = np.random.default_rng(13)
    pts, pos, nrm, w = _points(src, snk, snk_n, scat, scat_n, E, rng)
    N, M = src.shape[0], snk.shape[0]
    idx, _ = RC.workchunkingv2(src, snk, scat, (v, f), 2)
    assert idx.shape[0] > 100000
    beta = 2 * np.pi / 0.05
    S = EMGPUFreqDomain(N, M, idx, pts, 0.05, 0.02, beta)
    So = O.path_field(idx, pos, nrm, w, N, M, 0.02, beta)
    assert rel_err(S, So) < FIELD_TOL
    _no_device_errors()


def test_emgpufreqdomain_rejects_bad_rows():
    from lyceanem_gb300._native import LyemError
    from lyceanem_gb300.empropagation import EMGPUFreqDomain
    src, snk, snk_n, v, f, E, scat, scat_n = _scene(seed=6, n_scat=4)
    pts, _, _, _ = _points(src, snk, snk_n, scat, scat_n, E, np.random.default_rng(1))
    bad = np.array([[1, 10_000, 0]], np.int32)  # an index past the last point
    with pytest.raises(LyemError):
        EMGPUFreqDomain(src.shape[0], snk.shape[0], bad, pts, 0.05, 0.0, 100.0)


@pytest.mark.parametrize("scattering,los,elements", [(0, True, False), (1, True, False), (1, False, False),
                                                     (1, True, True), (2, True, False)])
def test_calculate_scattering_numba_branch(scattering, los, elements):
    from lyceanem_gb300.geometry import Mesh
    from lyceanem_gb300.models import frequency_domain as FD
    src, snk, snk_n, v, f, E, scat, scat_n = _scene(seed=8, n_src=5, n_snk=50, n_tris=90, n_scat=20)
    N, M, Pn = src.shape[0], snk.shape[0], scat.shape[0]
    solid = Mesh(v, [("triangle", f)])
    ap = Mesh(src, point_data={"Normals": np.tile([[0, 0, 1.0]], (N, 1)), "Area": np.full(N, 0.5)})
    sk = Mesh(snk, point_data={"Normals": snk_n})
    sc = Mesh(scat, point_data={"Normals": scat_n})
    beta = 2 * np.pi / 0.04
    axis = np.array([[1.0, 0.0, 0.0]])
    out = FD.calculate_scattering(ap, sk, solid, axis, scatter_points=sc, wavelength=0.04, scattering=scattering,
                                  elements=elements, los=los, beta=beta, cuda=False)
    got = np.stack(out, -1)
    # excitation of the numba branch: areas with scattering 0, the bare first row otherwise
    Esrc = np.tile(axis * (0.5 if scattering == 0 else 1.0), (N, 1)).astype(np.complex64)
    masks = O.numba_masks(src, snk, scat, O.pack_triangles(v, f))
    pos = np.concatenate([src, snk, scat])
    nrm = np.concatenate([np.tile([[0, 0, 1]], (N, 1)), snk_n, scat_n]).astype(np.float32)
    w = np.ones((N + M + Pn, 3), np.complex128)
    w[:N] = Esrc
    idx, _ = O.numba_path_index(N, M, Pn, *masks, scattering + 1, line_of_sight=los)
    net = O.path_field(idx, pos, nrm, w, N, M, 0.0, beta)
    ref = net if elements else net.sum(0)
    assert rel_err(got, ref) < FIELD_TOL
    if scattering <= 1 and not elements:
        fact = O.numba_sink_field(src, Esrc, snk, snk_n, scat, scat_n, 0.0, beta, masks, scattering, los=los)
        assert rel_err(got, fact) < FIELD_TOL
    _no_device_errors()


@pytest.mark.parametrize("scene,max_scatter,los", NUMBA_INDEX_CASES)
def test_workchunkingv2_reference_golden(scene, max_scatter, los):
    """workchunkingv2 against the reference's own numba engine (fixture executed from its source):
    the same rows in the same order, and the same ray count."""
    from lyceanem_gb300 import raycasting as RC
    d = numba_golden()
    src, snk, scat, v, f, _, _, _ = numba_golden_scene(d, scene)
    idx, rays = RC.workchunkingv2(src, snk, scat, (v, f), max_scatter, line_of_sight=los)
    key = numba_index_key(scene, max_scatter, los)
    assert np.array_equal(idx, d[f"index_{key}"])
    assert rays == int(d[f"rays_{key}"])
    _no_device_errors()


@pytest.mark.parametrize("key,lam,magnetic,tol", NUMBA_FIELD_CASES)
def test_emgpufreqdomain_reference_golden(key, lam, magnetic, tol):
    """EMGPUFreqDomain against the reference's own per-path product on the fixture's path list (within the
    reference's float32 phase rounding, see helpers)."""
    from lyceanem_gb300.empropagation import EMGPUFreqDomain, scattering_point
    d = numba_golden()
    src, snk, _, _, _, pos, nrm, w = numba_golden_scene(d, key[0])
    pts = np.zeros(pos.shape[0], dtype=scattering_point)
    for k, c in enumerate("xyz"):
        pts[f"p{c}"], pts[f"n{c}"], pts[f"e{c}"] = pos[:, k], nrm[:, k], w[:, k]
    pts["Electric"] = True
    pts["Electric"][:magnetic] = False
    pts["permittivity"] = 8.8541878176e-12
    pts["permeability"] = 1.25663706212e-6
    S = EMGPUFreqDomain(src.shape[0], snk.shape[0], d[f"index_{key}"], pts, lam, NUMBA_ALPHA, 2 * np.pi / lam)
    assert rel_err(S, d[f"field_{key}_{lam}_{magnetic}"]) < tol
    _no_device_errors()


def test_visiblespace_reference_golden():
    """visiblespace against the reference's own function (fixture executed from its source on the same
    elevation-major shell): visible pairs counted exactly, projected areas within 1e-5."""
    from lyceanem_gb300 import raycasting as RC
    from lyceanem_gb300.geometry import Mesh
    d = numba_golden()
    src, _, _, v, f, _, _, _ = numba_golden_scene(d, "a")
    for label, area, az, el in numba_vs_cases(d):
        kw = {} if az is None else dict(az_range=az, elev_range=el)
        area_in = np.array(area, copy=True)
        pat, shell = RC.visiblespace(Mesh(src), d["vs_normals"], (v, f), vertex_area=area_in,
                                     shell_range=NUMBA_VS_SHELL, **kw)
        ref = d[f"vs_{label}"]
        assert np.array_equal(np.asarray(shell.points), d[f"vs_{label}_shell"])
        assert pat.shape == ref.shape and pat.dtype == np.float32
        if label == "ones":
            assert np.array_equal(pat, ref)
        assert rel_err(pat, ref) < 1e-5, label
        assert np.array_equal(shell.point_data["Projected_Area"].reshape(-1), pat.reshape(-1))
        assert np.array_equal(np.isnan(area_in), np.isnan(np.asarray(area)))  # the caller's areas stay as given
    _no_device_errors()


@pytest.mark.parametrize("scene,scattering,los,elements,project", NUMBA_MODEL_CASES)
def test_calculate_scattering_numba_branch_reference_golden(scene, scattering, los, elements, project):
    """calculate_scattering(cuda=False) against the reference's own model function (fixture executed from its
    source under the numba stand-in) within 1e-5."""
    from lyceanem_gb300.geometry import Mesh
    from lyceanem_gb300.models import frequency_domain as FD
    d = numba_golden()
    src, snk, scat, v, f, _, _, _ = numba_golden_scene(d, scene)
    N = src.shape[0]
    ap = Mesh(src, point_data={"Normals": np.tile([[0, 0, 1.0]], (N, 1)), "Area": np.full(N, 0.5)})
    sk = Mesh(snk, point_data={"Normals": d[f"{scene}_snk_n"]})
    sc = Mesh(scat, point_data={"Normals": d[f"{scene}_scat_n"]})
    out = FD.calculate_scattering(ap, sk, Mesh(v, [("triangle", f)]), np.array([[1.0, 0.0, 0.0]]), scatter_points=sc,
                                  wavelength=0.5, scattering=scattering, elements=elements, los=los,
                                  project_vectors=project, beta=2 * np.pi / 0.5, cuda=False)
    assert rel_err(np.stack(out, -1), d[numba_model_key(scene, scattering, los, elements, project)]) < 1e-5
    _no_device_errors()


def _cuda_model_meshes(d):
    from lyceanem_gb300.geometry import Mesh
    g = lambda k: d[f"s_{k}"]  # noqa: E731
    n = g("src").shape[0]
    ap = Mesh(g("src"), point_data={"Normals": np.tile([[0, 0, 1.0]], (n, 1)), "Area": np.full(n, 0.5)})
    return (ap, Mesh(g("snk"), point_data={"Normals": g("snk_n")}),
            Mesh(g("scat"), point_data={"Normals": g("scat_n")}), Mesh(g("verts"), [("triangle", g("faces"))]))


@pytest.mark.parametrize("label,kw", CUDA_MODEL_CASES)
def test_calculate_scattering_cuda_reference_golden(label, kw):
    """calculate_scattering(cuda=True) against the reference's own model layer (calculate_scattering_cuda and
    Tile_acceleration_structure.calculate_scattering executed from its source on the oracle's per-pair
    networks) within 1e-5."""
    from lyceanem_gb300.models import frequency_domain as FD
    d = cuda_model_golden()
    ap, sk, sc, solid = _cuda_model_meshes(d)
    out = FD.calculate_scattering(ap, sk, solid, np.array([[1.0, 0.0, 0.0]]), scatter_points=sc,
                                  wavelength=CUDA_MODEL_LAMBDA, beta=2 * np.pi / CUDA_MODEL_LAMBDA, cuda=True, **kw)
    assert rel_err(np.stack(out, -1), d[f"cs_{label}"]) < 1e-5
    _no_device_errors()


@pytest.mark.parametrize("label,kw", CUDA_FARFIELD_CASES)
def test_calculate_farfield_reference_golden(label, kw):
    """calculate_farfield(cuda=True) against the reference's own function (the same unit-sphere sinks with
    outward normals that its positional farfield_distance produces) within 1e-5."""
    from lyceanem_gb300.models import frequency_domain as FD
    d = cuda_model_golden()
    ap, _, sc, solid = _cuda_model_meshes(d)
    et, ep = FD.calculate_farfield(ap, solid, np.array([[1.0, 0.0, 0.0]]), az_range=np.linspace(-180, 180, 9),
                                   el_range=np.linspace(-90, 90, 5), scatter_points=sc, wavelength=CUDA_MODEL_LAMBDA,
                                   farfield_distance=5.0, beta=2 * np.pi / CUDA_MODEL_LAMBDA, cuda=True, **kw)
    assert rel_err(et, d[f"{label}_theta"]) < 1e-5 and rel_err(ep, d[f"{label}_phi"]) < 1e-5
    _no_device_errors()

