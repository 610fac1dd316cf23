"""GPU parity of the time-domain products (TimeDomainv3 and the time-domain calculate_scattering)
against the oracle's FP64 restatement of timedomainkernal."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

from helpers import NUMBA_ALPHA, NUMBA_TD_CASES, numba_golden, numba_golden_scene, random_scene, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from lyceanem_gb300 import build
    build.build_native()


def _scene(seed=4, n_src=5, n_snk=30, n_tris=70, n_scat=15):
    src, snk, snk_n, v, f, E = random_scene(seed, n_src=n_src, n_snk=n_snk, n_tris=n_tris)
    rng = np.random.default_rng(seed + 3)
    scat = rng.uniform(-1, 1, (n_scat, 3)).astype(np.float32)
    scat_n = rng.normal(size=(n_scat, 3)).astype(np.float32)
    scat_n /= np.linalg.norm(scat_n, axis=1, keepdims=True)
    return src, snk, snk_n, v, f, E, scat, scat_n


@pytest.mark.parametrize("max_scatter", [1, 2, 3])
def test_path_times_vs_oracle(max_scatter):
    from lyceanem_gb300 import raycasting as RC
    from lyceanem_gb300.empropagation import path_times, time_map
    src, snk, snk_n, v, f, E, scat, scat_n = _scene()
    N, M = src.shape[0], snk.shape[0]
    idx, _ = RC.workchunkingv2(src, snk, scat, (v, f), max_scatter)
    pos = np.concatenate([src, snk, scat])
    nrm = np.concatenate([np.tile([[0, 0, 1.0]], (N, 1)), snk_n, scat_n]).astype(np.float32)
    rng = np.random.default_rng(2)
    w = (rng.uniform(0.5, 1.5, (pos.shape[0], 3)) + 1j * rng.uniform(0, 2e-9, (pos.shape[0], 3))).astype(np.complex64)
    amp, arr, pair = path_times(idx, pos, nrm, w, N, M, 0.01, 2 * np.pi / 0.05)
    oamp, oarr, opair = O.path_times(idx, pos, nrm, w, N, M, 0.01, 2 * np.pi / 0.05)
    assert np.array_equal(pair.cpu().numpy(), opair)
    assert rel_err(amp.cpu().numpy(), oamp) < 1e-5
    assert np.abs(arr.cpu().numpy() - oarr).max() < 1e-15  # seconds (path lengths to ~1e-7 m)
    exc = np.sin(np.linspace(0, 6 * np.pi, 40)) * np.hanning(40)
    tm, wake = time_map(amp, arr, pair, N, M, exc, 20e9, 400)
    otm, owake = O.time_map(amp.cpu().numpy(), arr.cpu().numpy(), pair.cpu().numpy(), N, M, exc, 20e9, 400)
    assert wake == owake
    assert np.abs(tm.cpu().numpy() - otm).max() <= 1e-12 * np.abs(otm).max()


def test_time_domain_calculate_scattering():
    from lyceanem_gb300.empropagation import TimeDomainv3, scattering_point
    from lyceanem_gb300.geometry import Mesh
    from lyceanem_gb300.models import time_domain as TD
    src, snk, snk_n, v, f, E, scat, scat_n = _scene(seed=9)
    N, M, Pn = src.shape[0], snk.shape[0], scat.shape[0]
    solid = Mesh(v, [("triangle", f)])
    ap = Mesh(src, point_data={"Normals": np.tile([[0, 0, 1.0]], (N, 1)), "Area": np.full(N, 0.25)})
    sk = Mesh(snk, point_data={"Normals": snk_n})
    sc = Mesh(scat, point_data={"Normals": scat_n})
    exc = np.cos(np.linspace(0, 8 * np.pi, 64)) * np.hanning(64)
    fs, S = 40e9, 600
    Ex, Ey, Ez, wake = TD.calculate_scattering(ap, sk, exc, solid, np.array([1.0, 0.0, 0.0]), scatter_points=sc,
                                               scattering=1, sampling_freq=fs, num_samples=S, los=True,
                                               project_vectors=False, beta=2 * np.pi / 0.03)
    # oracle: the same path rows, FP64 per-row product and accumulation, then the wake shift
    masks = O.numba_masks(src, snk, scat, O.pack_triangles(v, f))
    idx, _ = O.numba_path_index(N, M, Pn, *masks, 2, line_of_sight=True)
    pos = np.concatenate([src, snk, scat])
    nrm = np.concatenate([np.tile([[0, 0, 1]], (N, 1)), snk_n, scat_n]).astype(np.float32)
    w = np.ones((N + M + Pn, 3), np.complex64)
    w[:N] = np.array([0.25, 0, 0])
    oamp, oarr, opair = O.path_times(idx, pos, nrm, w, N, M, 0.0, 2 * np.pi / 0.03)
    otm, owake = O.time_map(oamp, oarr, opair, N, M, exc, fs, S)
    assert abs(wake[0] - owake) < 1e-15
    total = otm.sum(axis=(0, 1))
    k = int(np.digitize(owake, np.linspace(0, S / fs, S)))
    ref = np.zeros((S, 3))
    ref[k:] = total[:S - k]
    assert rel_err(np.stack([Ex, Ey, Ez], 1), ref) < 1e-5
    # TimeDomainv3 through scattering_point records gives the same map
    pts = np.zeros(N + M + Pn, dtype=scattering_point)
    for j, c in enumerate("xyz"):
        pts[f"p{c}"] = pos[:, j]
        pts[f"n{c}"] = nrm[:, j]
        pts[f"e{c}"] = w[:, j]
    pts["Electric"] = True
    tm, wk = TimeDomainv3(N, M, pts, idx, 0.25 * np.pi, 0.03, exc, fs, S, 0.0, 2 * np.pi / 0.03)
    assert tm.shape == (N, M, S, 3) and abs(wk - owake) < 1e-15
    assert rel_err(tm, otm) < 1e-5
    from lyceanem_gb300 import propagation as P
    assert P.device_errors() == (0, 0)


def test_timedomainv3_reference_golden():
    """TimeDomainv3 against the reference's own time kernel on a one-block path list (fixture executed from
    its source): wake time to the float32 path lengths it forms, time map within 1e-6."""
    from lyceanem_gb300.empropagation import TimeDomainv3, scattering_point
    d = numba_golden()
    src, snk, _, _, _, pos, nrm, _ = numba_golden_scene(d, "t")
    w = d["time_w"]
    pts = np.zeros(pos.shape[0], dtype=scattering_point)
    for k, c in enumerate("xyz"):
        pts[f"p{c}"], pts[f"n{c}"], pts[f"e{c}"] = pos[:, k], nrm[:, k], w[:, k]
    pts["Electric"] = True
    pts["permittivity"] = 8.8541878176e-12
    pts["permeability"] = 1.25663706212e-6
    tm, wake = TimeDomainv3(src.shape[0], snk.shape[0], pts, d["index_t2los"], 0.25 * np.pi, 0.05,
                            d["time_excitation"], 20e9, 400, NUMBA_ALPHA, 2 * np.pi / 0.05)
    assert abs(wake - float(d["time_wake"])) < 1e-14
    assert rel_err(tm, d["time_map"]) < 1e-6
    # 120 samples: rows whose excitation would run past the map are cut at its end
    tm, wake = TimeDomainv3(src.shape[0], snk.shape[0], pts, d["index_t2los"], 0.25 * np.pi, 0.05,
                            d["time_excitation"], 20e9, 120, NUMBA_ALPHA, 2 * np.pi / 0.05)
    assert abs(wake - float(d["time_wake_short"])) < 1e-14
    assert rel_err(tm, d["time_map_short"]) < 1e-6
    from lyceanem_gb300 import propagation as P
    assert P.device_errors() == (0, 0)


@pytest.mark.parametrize("label,kw", NUMBA_TD_CASES)
def test_time_domain_model_reference_golden(label, kw):
    """models.time_domain.calculate_scattering against the reference's own model function (fixture executed
    from its source under the numba stand-in, one block of rows per time-kernel launch): wake time to the
    reference's float32 path lengths, time series within 1e-5."""
    from lyceanem_gb300.geometry import Mesh
    from lyceanem_gb300.models import time_domain as TD
    d = numba_golden()
    src, snk, scat, v, f, _, _, _ = numba_golden_scene(d, "t")
    n = src.shape[0]
    ap = Mesh(src, point_data={"Normals": np.tile([[0, 0, 1.0]], (n, 1)), "Area": np.full(n, 0.25)})
    sk = Mesh(snk, point_data={"Normals": d["t_snk_n"]})
    sc = Mesh(scat, point_data={"Normals": d["t_scat_n"]})
    out = TD.calculate_scattering(ap, sk, d["time_excitation"], Mesh(v, [("triangle", f)]), np.array([1.0, 0.0, 0.0]),
                                  scatter_points=sc, wavelength=0.05, sampling_freq=20e9, num_samples=400, los=True,
                                  beta=2 * np.pi / 0.05, **kw)
    got = np.stack(out[:3], -1)
    ref = d[f"td_{label}"]
    assert got.shape == ref.shape
    assert np.abs(np.asarray(out[3], np.float64).reshape(-1) - d[f"td_{label}_wake"].reshape(-1)).max() < 1e-14
    assert rel_err(got, ref) < 1e-5
    from lyceanem_gb300 import propagation as P
    assert P.device_errors() == (0, 0)

