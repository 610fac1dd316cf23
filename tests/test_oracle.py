"""CPU tests of the oracle itself: known answers, grid == brute force, and an
independent NumPy restatement of the field formula (lyceanem/src/em.cuh:18-120)."""
import numpy as np
import pytest

from oracle import oracle as O

from helpers import random_scene, rel_err


def _tri(v0, v1, v2):
    return O.pack_triangles(np.array([v0, v1, v2], np.float32), np.array([[0, 1, 2]], np.int32))[0]


def test_hit_known_answers():
    # triangle in the plane x = 0 with normal +x (e1 x e2 = (4, 0, 0))
    t = _tri([0, -1, -1], [0, 1, -1], [0, 0, 1])
    o = np.array([1, 0, 0], np.float32)
    d = np.array([-1, 0, 0], np.float32)
    assert O.hit_one(d, 2.0, o, t)                      # front face, crossing at t = 1
    assert not O.hit_one(-d, 2.0, -o, t)                # back face: culled (raycasting.cuh:31-34)
    assert O.hit_one(-d, 2.0, -o, t, cull=False)        # numba engine: no cull
    assert not O.hit_one(d, 0.5, o, t)                  # segment ends before the plane
    assert not O.hit_one(d, 1.0 + 1e-6, o, t)           # hit within 2*eps of the end point
    o2 = np.array([1, 0.9, 0.9], np.float32)
    assert not O.hit_one(d, 2.0, o2, t)                 # outside the triangle (U + V > 1)
    d_par = np.array([0, 1, 0], np.float32)
    assert not O.hit_one(d_par, 5.0, o, t)              # parallel: |A| < eps


def test_pack_triangles_matches_fp32_edges():
    rng = np.random.default_rng(3)
    v = rng.normal(size=(20, 3)).astype(np.float32)
    f = rng.integers(0, 20, size=(15, 3)).astype(np.int32)
    t = O.pack_triangles(v, f)
    assert np.array_equal(t[:, 0:3], v[f[:, 0]])
    assert np.array_equal(t[:, 4:7], v[f[:, 1]] - v[f[:, 0]])
    assert np.array_equal(t[:, 8:11], v[f[:, 2]] - v[f[:, 0]])


@pytest.mark.parametrize("seed", range(6))
def test_grid_mask_equals_brute(seed):
    src, snk, snk_n, v, f, E = random_scene(seed, n_src=9, n_snk=120, n_tris=150)
    tris = O.pack_triangles(v, f)
    brute = O.mask_brute(src, snk, tris)
    for cell in (0.11, 0.37, 2.5):
        g = O.Grid(tris, cell)
        assert np.array_equal(g.mask(src, snk), brute), cell
    assert 0 < brute.sum() < brute.size


def test_grid_axis_aligned_and_ground():
    # axis-aligned rays through a tessellated ground plane (rays along cell faces)
    from lyceanem_gb300 import scenes
    v, f = scenes.ground_plane(2.0, 10, -1.0)
    tris = O.pack_triangles(v, f)
    xs = np.linspace(-1.2, 1.2, 13)
    src = np.stack([xs, np.zeros_like(xs), np.full_like(xs, 0.5)], 1).astype(np.float32)
    snk = np.stack([xs, np.full_like(xs, 0.2), np.full_like(xs, -3.0)], 1).astype(np.float32)
    brute = O.mask_brute(src, snk, tris, self_to_self=True)
    for cell in (0.2, 0.1, 0.5):
        assert np.array_equal(O.Grid(tris, cell).mask(src, snk, self_to_self=True), brute)
    # straight down inside the plane's footprint is blocked, outside is not
    assert not brute[6, 6] and brute[0, 0]


def test_self_to_self_rule():
    src, snk, snk_n, v, f, E = random_scene(11, n_src=10, n_snk=10, n_tris=20, box=0.5)
    snk[:, 2] = 2.0 + np.abs(snk[:, 2])  # all sinks above a wall at z = 0 facing the sources
    wall = np.array([[-50, -50, 0], [50, 0, 0], [-50, 50, 0]], np.float32)  # e1 x e2 along -z
    v = np.concatenate([v, wall])
    f = np.concatenate([f, np.array([[v.shape[0] - 3, v.shape[0] - 1, v.shape[0] - 2]], np.int32)])
    tris = O.pack_triangles(v, f)
    a = O.mask_brute(src, snk, tris, self_to_self=False)
    b = O.mask_brute(src, snk, tris, self_to_self=True)
    off = ~np.eye(10, dtype=bool)
    assert np.array_equal(a[off], b[off])
    assert a[np.eye(10, dtype=bool)].all()     # untested diagonal pairs count as visible
    assert not b[np.eye(10, dtype=bool)].all()


def _numpy_em_wave(src, snk, snk_n, E, alpha, beta):
    """Independent vectorised restatement of ray_launch + em_wave (em.cuh:18-120) in FP64."""
    r = snk[None, :, :].astype(np.float64) - src[:, None, :].astype(np.float64)
    L = np.linalg.norm(r, axis=-1)
    d = r / L[..., None]
    Ed = np.einsum("nc,nmc->nm", E.astype(np.complex128), d)
    EL = E[:, None, :] - Ed[..., None] * d                    # (E.u)u + (E.v)v == E - (E.d)d
    G = np.exp(-(alpha + 1j * beta) * L) / L
    dG = (-alpha - 1.0 / L - 1j * beta) * G
    loss = -(1 / (2 * np.pi)) * dG * np.einsum("mc,nmc->nm", snk_n.astype(np.float64), d)
    return EL * loss[..., None]


def test_pair_field_matches_numpy_restatement():
    src, snk, snk_n, v, f, E = random_scene(5, n_src=6, n_snk=30)
    beta, alpha = 2 * np.pi / 0.0107, 0.01
    S = O.pair_field(src, E, snk, snk_n, None, alpha, beta)
    ref = _numpy_em_wave(src, snk, snk_n, E, alpha, beta)
    assert rel_err(S, ref) < 1e-12


def test_sink_field_is_masked_source_sum():
    src, snk, snk_n, v, f, E = random_scene(7, n_src=8, n_snk=40, n_tris=120)
    tris = O.pack_triangles(v, f)
    beta = 2 * np.pi / 0.03
    S, mask = O.scattering_network(src, E, snk, snk_n, tris, 0.0, beta)
    assert np.all(S[~mask] == 0)
    out = O.sink_field(src, E, snk, snk_n, 0.0, beta, tris12=tris)
    assert rel_err(out, S.sum(axis=0)) < 1e-12
    g = O.Grid(tris, 0.3)
    out_g, cnt = O.sink_field(src, E, snk, snk_n, 0.0, beta, grid=g, return_counters=True)
    assert rel_err(out_g, out) < 1e-12
    assert cnt["visible"] == int(mask.sum())


def test_onebounce_factorised_equals_reference_composition():
    """1^T (S0 + S1 @ S2) with S2 driven by e_p = 1^T S1 (frequency_domain.py:230-260, 847-849)."""
    src, snk, snk_n, v, f, E = random_scene(9, n_src=5, n_snk=25, n_tris=80)
    rng = np.random.default_rng(1)
    scat = rng.uniform(-1, 1, size=(12, 3)).astype(np.float32)
    scat_n = rng.normal(size=(12, 3))
    scat_n = (scat_n / np.linalg.norm(scat_n, axis=1, keepdims=True)).astype(np.float32)
    tris = O.pack_triangles(v, f)
    beta = 2 * np.pi / 0.05
    S0, _ = O.scattering_network(src, E, snk, snk_n, tris, 0.0, beta)
    S1, _ = O.scattering_network(src, E, scat, scat_n, tris, 0.0, beta)
    e_p = S1.sum(axis=0)
    S2, _ = O.scattering_network(scat, e_p, snk, snk_n, tris, 0.0, beta)
    total = S0.copy()
    for c in range(3):
        total[:, :, c] += S1[:, :, c] @ S2[:, :, c]
    ref = total.sum(axis=0)
    got, e_p2 = O.onebounce_sink_field(src, E, snk, snk_n, scat, scat_n, 0.0, beta, tris12=tris)
    assert rel_err(e_p2, e_p) < 1e-12
    assert rel_err(got, ref) < 1e-10


def _numba_scene(seed=3):
    from helpers import random_scene
    src, snk, snk_n, v, f, E = random_scene(seed, n_src=6, n_snk=40, n_tris=80)
    rng = np.random.default_rng(seed + 10)
    scat = rng.uniform(-1, 1, (25, 3)).astype(np.float32)
    scat_n = rng.normal(size=(25, 3)).astype(np.float32)
    scat_n /= np.linalg.norm(scat_n, axis=1, keepdims=True)
    return src, snk, snk_n, v, f, E, scat, scat_n


def test_numba_path_product_factorises():
    """The numba engine's per-path sum (freqdomainkernal over workchunkingv2's rows) equals the
    factored form the GPU composition uses (direct projected at the sinks, bounce driven by the
    projected scatter excitation), in FP64."""
    src, snk, snk_n, v, f, E, scat, scat_n = _numba_scene()
    masks = O.numba_masks(src, snk, scat, O.pack_triangles(v, f))
    N, M, Pn = src.shape[0], snk.shape[0], scat.shape[0]
    pos = np.concatenate([src, snk, scat])
    nrm = np.concatenate([np.tile([[0, 0, 1]], (N, 1)), snk_n, scat_n]).astype(np.float32)
    w = np.ones((N + M + Pn, 3), np.complex128)
    w[:N] = E
    for max_scatter, los in ((1, True), (2, True), (2, False)):
        idx, rays = O.numba_path_index(N, M, Pn, *masks, max_scatter, line_of_sight=los)
        net = O.path_field(idx, pos, nrm, w, N, M, 0.0, 60.0)
        ref = O.numba_sink_field(src, E, snk, snk_n, scat, scat_n, 0.0, 60.0, masks, max_scatter - 1, los=los)
        assert np.abs(net.sum(0) - ref).max() <= 1e-12 * np.abs(ref).max()
        assert rays == N * (M + Pn) if max_scatter == 1 else rays >= N * Pn
    # two bounces: rows of four columns; direct and one-bounce rows also take the last point's
    # normal in their projection (the index 0 read as Python's -1)
    idx, _ = O.numba_path_index(N, M, Pn, *masks, 3)
    assert idx.shape[1] == 4 and np.all(idx[:, 0] >= 1)
    full = idx[np.all(idx != 0, axis=1)]
    assert np.all(full[:, 1] != full[:, 2])
    net = O.path_field(idx, pos, nrm, w, N, M, 0.0, 60.0)
    assert np.all(np.isfinite(net))


def test_numba_ratio_decisions_exact():
    """The non-culling kernels decide the numba engine's U < 0, U > 1 and V < 0 (there F = 1.0 / A and
    U = F * u in FP64, lyceanem/raycasting/rayfunctions.py:55-100) by comparing the float32 numerator with
    the float32 determinant: u / A < 0 as a sign test, u / A > 1 as sign(A) * u > |A|.  Both agree with the
    FP64 evaluation on random and adversarial float32 pairs: u == A and its neighbours, both signs, zeros,
    tiny and huge magnitudes."""
    rng = np.random.default_rng(0)
    n = 200000
    A = (rng.choice([-1.0, 1.0], n) * 2.0 ** rng.uniform(-60, 60, n)).astype(np.float32)
    near = np.stack([A, np.nextafter(A, np.float32(np.inf)), np.nextafter(A, np.float32(-np.inf)), -A,
                     np.zeros_like(A), -np.zeros_like(A),
                     (A * rng.uniform(0.999999, 1.000001, n)).astype(np.float32),
                     (rng.choice([-1.0, 1.0], n) * 2.0 ** rng.uniform(-149, 127, n)).astype(np.float32)])
    for u in near:
        F = 1.0 / A.astype(np.float64)
        U = F * u.astype(np.float64)
        neg = np.where(A < 0, u > 0, u < 0)
        above = np.where(A < 0, -u, u) > np.abs(A)
        assert np.array_equal(neg, U < 0)
        assert np.array_equal(above, U > 1)
