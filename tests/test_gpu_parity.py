"""GPU parity: the CUDA path against the CPU oracle on the same seeded inputs.

Masks must be bit-exact; fields within 1e-5 relative (max-normalised) of the
FP64 oracle."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

from helpers import random_scene, rel_err

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from lyceanem_gb300 import build
    build.build_native()


def _P():
    from lyceanem_gb300 import propagation as P
    return P


def _no_device_errors():
    st, flags = _P().device_errors()
    assert st == 0 and flags == 0, f"device error word {flags:#x}"


def _pair_rel(S, So, src=None, snk=None, E=None, beta=None, alpha=0.0):
    """Per-pair vector error relative to the pair's unprojected amplitude
    |E_n| |alpha + 1/r + j beta| exp(-alpha r) / (2 pi r): the polarisation
    projection and n.d can make a pair's field arbitrarily small, while the FP32
    ray direction carries an absolute error of ~1e-7 of that amplitude.  Without
    geometry the scale falls back to the largest pair."""
    e = np.linalg.norm(S - So, axis=-1)
    if src is None:
        n = np.linalg.norm(So, axis=-1)
        return float((e / n.max()).max())
    r = np.linalg.norm(snk[None].astype(np.float64) - src[:, None].astype(np.float64), axis=-1)
    amp = np.linalg.norm(np.asarray(E, np.complex128), axis=-1)[:, None]
    scale = amp * np.abs(alpha + 1.0 / r + 1j * beta) * np.exp(-alpha * r) / (2 * np.pi * r)
    return float((e / np.maximum(scale, 1e-30)).max())


def test_direct_config_full_size():
    """8x8 array, 2,664 sinks, 1,024 triangles, brute force: mask, sink field and per-pair network."""
    from lyceanem_gb300 import scenes
    P = _P()
    s = scenes.direct_scene()
    beta = 2 * np.pi / s.wavelength
    tris = P.pack_triangles(torch.from_numpy(s.verts), torch.from_numpy(s.faces))
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    r = P.pair_stage(s.src, s.E, s.snk, s.snk_n, beta=beta, tris=tris, want_mask=True, want_pairs=True, counters=cnt)
    mask = r.mask().cpu().numpy()
    _no_device_errors()
    otris = O.pack_triangles(s.verts, s.faces)
    assert np.array_equal(tris.cpu().numpy(), otris)
    omask = O.mask_brute(s.src, s.snk, otris)
    assert np.array_equal(mask, omask), f"{(mask != omask).sum()} mismatching pairs"
    ofield = O.sink_field(s.src, s.E, s.snk, s.snk_n, 0.0, beta, mask=omask)
    assert rel_err(r.sink.cpu().numpy(), ofield) < FIELD_TOL
    opairs = O.pair_field(s.src, s.E, s.snk, s.snk_n, omask, 0.0, beta)
    pairs = r.pairs.cpu().numpy()
    assert np.all(pairs[~omask] == 0)
    assert _pair_rel(pairs, opairs, s.src, s.snk, s.E, beta) < FIELD_TOL
    assert int(cnt[0]) == int(omask.sum())
    assert 0 < omask.sum() < omask.size


@pytest.mark.parametrize("seed", range(4))
def test_grid_and_brute_masks_bit_exact(seed):
    P = _P()
    src, snk, snk_n, v, f, E = random_scene(seed, n_src=37, n_snk=300, n_tris=700, box=1.0)
    tris = P.pack_triangles(torch.from_numpy(v), torch.from_numpy(f))
    omask = O.mask_brute(src, snk, O.pack_triangles(v, f))
    rb = P.pair_stage(src, E, snk, snk_n, beta=100.0, tris=tris, want_mask=True)
    assert np.array_equal(rb.mask().cpu().numpy(), omask)
    for cell in (None, 0.07, 0.3, 1.9):
        g = P.UniformGrid(tris, cell=cell)
        rg = P.pair_stage(src, E, snk, snk_n, beta=100.0, grid=g, want_mask=True)
        assert np.array_equal(rg.mask().cpu().numpy(), omask), cell
        assert rel_err(rg.sink.cpu().numpy(), rb.sink.cpu().numpy()) < 1e-6
    _no_device_errors()


@pytest.mark.parametrize("eps", [1e-6, 0.0])
def test_grazing_rays_masks_bit_exact(eps):
    """Rays nearly in the planes of the triangles (determinant near zero, both windings, triangle sizes
    1e-3 to 0.3 m, plane tilts 1e-8 to 1e-1): culled masks of the grid walk and of the brute-force kernel
    bit-exact to the oracle."""
    P = _P()
    rng = np.random.default_rng(21)
    n_t = 600
    size = 10.0 ** rng.uniform(-3, -0.5, n_t)
    tilt = 10.0 ** rng.uniform(-8, -1, n_t) * rng.choice([-1.0, 1.0], n_t)
    centre = rng.uniform(-1, 1, (n_t, 3)) * np.array([2.0, 1.0, 0.05])
    verts = []
    for k in range(n_t):
        a = rng.uniform(-1, 1, (3, 2)) * size[k]
        pts = centre[k] + np.stack([a[:, 0], a[:, 1], tilt[k] * a[:, 0]], 1)
        verts.append(pts[::-1] if rng.random() < 0.5 else pts)
    v = np.concatenate(verts).astype(np.float32)
    f = np.arange(3 * n_t, dtype=np.int32).reshape(-1, 3)
    n_src, n_snk = 40, 256
    src = np.stack([np.full(n_src, -3.0), rng.uniform(-1, 1, n_src), rng.uniform(-0.05, 0.05, n_src)], 1)
    snk = np.stack([np.full(n_snk, 3.0), rng.uniform(-1, 1, n_snk), rng.uniform(-0.05, 0.05, n_snk)], 1)
    src, snk = src.astype(np.float32), snk.astype(np.float32)
    snk_n = np.tile(np.array([[-1.0, 0.0, 0.0]], np.float32), (n_snk, 1))
    E = np.tile(np.array([[1, 0, 0]], np.complex64), (n_src, 1))
    om = O.mask_brute(src, snk, O.pack_triangles(v, f), cull=True, eps=eps)
    assert 0 < om.sum() < om.size
    tris = P.pack_triangles(torch.from_numpy(v), torch.from_numpy(f))
    rb = P.pair_stage(src, E, snk, snk_n, beta=10.0, tris=tris, eps=eps, want_mask=True)
    assert np.array_equal(rb.mask().cpu().numpy(), om)
    for cell in (0.05, 0.5):
        g = P.UniformGrid(tris, cell=cell)
        r = P.pair_stage(src, E, snk, snk_n, beta=10.0, grid=g, eps=eps, want_mask=True)
        assert np.array_equal(r.mask().cpu().numpy(), om), cell
    _no_device_errors()


@pytest.mark.parametrize("scale,snk_r", [(1.0, 4.0), (1e3, 4e3), (1.0, 3e9), (3e-3, 12e-3)])
def test_masks_bit_exact_across_scales(scale, snk_r):
    """Scenes scaled by 1e3 and 3e-3, and sinks 3e9 m away (segment lengths beyond 2^30, where the culling
    test's reciprocal-free decisions give way to the reference's own sequence): culled masks of the brute-force
    kernel and of the grid walk bit-exact to the oracle."""
    P = _P()
    src, snk, snk_n, v, f, E = random_scene(41, n_src=24, n_snk=300, n_tris=500, box=1.0)
    src = (src.astype(np.float64) * scale).astype(np.float32)
    v = (v.astype(np.float64) * scale).astype(np.float32)
    snk = (snk_n.astype(np.float64) * -snk_r).astype(np.float32)
    om = O.mask_brute(src, snk, O.pack_triangles(v, f), cull=True, eps=1e-6)
    assert 0 < om.sum() < om.size
    tris = P.pack_triangles(torch.from_numpy(v), torch.from_numpy(f))
    rb = P.pair_stage(src, E, snk, snk_n, beta=1.0, tris=tris, want_mask=True)
    assert np.array_equal(rb.mask().cpu().numpy(), om)
    for cell in (None, 0.4 * scale):
        g = P.UniformGrid(tris, cell=cell)
        r = P.pair_stage(src, E, snk, snk_n, beta=1.0, grid=g, want_mask=True)
        assert np.array_equal(r.mask().cpu().numpy(), om), cell
    _no_device_errors()


@pytest.mark.parametrize("cull", [True, False])
def test_lattice_scene_masks_bit_exact(cull):
    """Axis-aligned geometry on a lattice: axis-aligned quads lying on cell faces, sources and sinks on cell
    planes, rays along the axes (zero direction components) and at 45 degrees; the grid walk (cell boxes,
    own-surface hint, direction order) against the oracle's brute force, both visibility rules."""
    P = _P()
    cell = 0.25
    quads = []
    for k in range(-3, 4):          # planes z = k * cell, x = k * cell (exactly on cell faces)
        for a in range(-2, 2):
            for b in range(-2, 2):
                u0, u1, v0, v1 = a * cell, (a + 1) * cell, b * cell, (b + 1) * cell
                if (a + b + k) % 2 == 0:
                    quads.append([[u0, v0, k * cell], [u1, v0, k * cell], [u1, v1, k * cell], [u0, v1, k * cell]])
                else:
                    quads.append([[k * cell, u0, v0], [k * cell, u1, v0], [k * cell, u1, v1], [k * cell, u0, v1]])
    q = np.array(quads, np.float32)
    v = q.reshape(-1, 3)
    f = np.concatenate([np.stack([4 * i + np.array([0, 1, 2]), 4 * i + np.array([0, 2, 3])]) for i in range(len(q))])
    f = f.astype(np.int32)
    g1 = np.arange(-4, 5) * cell
    src = np.array([[x, y, z] for x in g1[::2] for y in g1[::3] for z in (-1.0, 0.5 * cell, 1.0)], np.float32)
    snk = np.concatenate([
        np.array([[x, y, 2.0] for x in g1 for y in g1], np.float32),           # straight up from lattice points
        np.array([[2.0, y, z] for y in g1[::2] for z in g1[::2]], np.float32),  # along +x
        np.array([[x, x, -2.0] for x in g1], np.float32),                       # 45 degree diagonals
    ])
    snk_n = -snk / np.linalg.norm(snk, axis=1, keepdims=True)
    eps = 1e-6 if cull else 1e-7
    om = O.mask_brute(src, snk, O.pack_triangles(v, f), cull=cull, eps=eps)
    assert 0 < om.sum() < om.size
    tris = P.pack_triangles(torch.from_numpy(v), torch.from_numpy(f))
    E = np.tile(np.array([[1, 0, 0]], np.complex64), (src.shape[0], 1))
    for c in (cell, 2 * cell, None):
        g = P.UniformGrid(tris, cell=c)
        for order in (None, P.direction_order(snk, g.centre)):
            r = P.pair_stage(src, E, snk, snk_n, beta=20.0, grid=g, cull=cull, eps=eps, want_mask=True,
                             snk_order=order)
            assert np.array_equal(r.mask().cpu().numpy(), om), (c, order is None)
    _no_device_errors()


def test_grid_build_matches_cpu_binning():
    """Cell ranges of the device grid equal a NumPy restatement of the padded-box binning."""
    P = _P()
    src, snk, snk_n, v, f, E = random_scene(3, n_tris=500, box=2.0)
    tris = P.pack_triangles(torch.from_numpy(v), torch.from_numpy(f))
    g = P.UniformGrid(tris, cell=0.4)
    t = tris.cpu().numpy()
    vv = np.stack([t[:, 0:3], t[:, 0:3] + t[:, 4:7], t[:, 0:3] + t[:, 8:11]], 1)
    lo, hi = vv.min(1) - g.cell * 1e-3, vv.max(1) + g.cell * 1e-3
    org = np.array(g.origin, np.float32)
    i0 = np.clip(np.floor((lo - org) * np.float32(1 / g.cell)), 0, np.array(g.dims) - 1).astype(int)
    i1 = np.clip(np.floor((hi - org) * np.float32(1 / g.cell)), 0, np.array(g.dims) - 1).astype(int)
    cells = [[] for _ in range(g.n_cells)]
    for k in range(t.shape[0]):
        for z in range(i0[k, 2], i1[k, 2] + 1):
            for y in range(i0[k, 1], i1[k, 1] + 1):
                for x in range(i0[k, 0], i1[k, 0] + 1):
                    cells[(z * g.dims[1] + y) * g.dims[0] + x].append(k)
    start = g.cell_start.cpu().numpy()
    ct = g.cell_tris.cpu().numpy()
    assert start[-1] == g.n_refs == sum(len(c) for c in cells)
    # cell table: per cell child A (centroid below the split plane) then child B, each in triangle order, with the
    # box of its padded triangle boxes within the cell widened by 2 pads; the split plane is the candidate (k/8 of
    # the cell on one axis, k = 1..7) of least surface-area cost (clipped child boxes' areas times their counts)
    box = g.cell_box.cpu().numpy()
    refs = np.ascontiguousarray(box[:, [3, 7, 11, 15]]).view(np.int32)
    assert np.array_equal(refs[:, 0], start[:-1]) and np.array_equal(refs[:, 3], start[1:])
    assert np.array_equal(refs[:, 1], refs[:, 2])
    pad = np.float32(1e-3) * np.float32(g.cell)
    vlo, vhi = vv.min(1) - pad, vv.max(1) + pad
    cen = vv.astype(np.float64).mean(1)
    for c in range(g.n_cells):
        L = np.array(cells[c], dtype=int)
        if not len(L):
            continue
        ix = np.array([c % g.dims[0], (c // g.dims[0]) % g.dims[1], c // (g.dims[0] * g.dims[1])])
        c0 = org + ix * np.float32(g.cell)
        got = ct[start[c]:start[c + 1]]
        na = refs[c, 1] - refs[c, 0]
        assert sorted(map(tuple, got.tolist())) == sorted(map(tuple, t[L].tolist())), c
        if len(L) > 1:
            # the split is one of the candidates (no centroid within 1e-5 of its plane, where FP32 and FP64
            # centroids could disagree), and its cost is the least of all candidates' to FP32 rounding
            costs, match = [], []
            for a in range(3):
                for k in range(1, 8):
                    plane = org[a] + (ix[a] + 0.125 * k) * g.cell
                    in_a = cen[L, a] < plane
                    cost = 0.0
                    for sel in (in_a, ~in_a):
                        if not sel.any():
                            continue
                        lo = np.maximum(vlo[L[sel]].min(0), c0 - 2 * pad).astype(np.float64)
                        hi = np.minimum(vhi[L[sel]].max(0), c0 + np.float32(g.cell) + 2 * pad).astype(np.float64)
                        e = np.maximum(hi - lo, 0.0)
                        cost += (e[0] * e[1] + e[1] * e[2] + e[2] * e[0]) * sel.sum()
                    costs.append(cost)
                    clear = np.all(np.abs(cen[L, a] - plane) > 1e-5)
                    match.append(clear and np.array_equal(got[:na], t[L[in_a]]) and np.array_equal(got[na:], t[L[~in_a]]))
            if any(match):
                best = min(cst for cst, mt in zip(costs, match) if mt)
                assert best <= min(costs) * (1 + 1e-4) + 1e-12, c
            else:  # only where a centroid lies at a candidate plane may no candidate reproduce the split
                assert np.any([np.any(np.abs(cen[L, a] - (org[a] + (ix[a] + 0.125 * k) * g.cell)) <= 1e-5)
                               for a in range(3) for k in range(1, 8)]), c
        for child, rows in ((0, got[:na]), (1, got[na:])):
            lo_b, hi_b = box[c, 8 * child:8 * child + 3], box[c, 8 * child + 4:8 * child + 7]
            if not len(rows):
                assert np.all(np.isinf(lo_b)) and np.all(np.isinf(hi_b)), c
                continue
            rv = np.stack([rows[:, 0:3], rows[:, 0:3] + rows[:, 4:7], rows[:, 0:3] + rows[:, 8:11]], 1)
            lo = np.maximum(rv.min(1).min(0) - pad, c0 - 2 * pad)
            hi = np.minimum(rv.max(1).max(0) + pad, c0 + np.float32(g.cell) + 2 * pad)
            assert np.allclose(lo_b, lo, rtol=0, atol=1e-5) and np.allclose(hi_b, hi, rtol=0, atol=1e-5), c


def test_bounce_scene_reduced_vs_oracle():
    """Direct + one bounce (ground + clutter, scatter points) on a reduced bounce recipe."""
    from lyceanem_gb300 import scenes
    from lyceanem_gb300.models import acceleration_structures as A
    from lyceanem_gb300.models.frequency_domain import sink_field
    P = _P()
    s = scenes.bounce_scene(n_side=4, n_ground=30, n_clutter=1500, n_scatter=200, el_n=13, az_n=25)
    beta = 2 * np.pi / s.wavelength
    dev = A._DeviceScene(s.verts, s.faces, grid_cell=s.cell)
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    E = sink_field(type("S", (), {"device": dev})(), s.src, s.E, s.snk, s.snk_n, 0.0, beta, s.scat, s.scat_n,
                   scattering=1, counters=cnt).cpu().numpy()
    _no_device_errors()
    otris = O.pack_triangles(s.verts, s.faces)
    og = O.Grid(otris, s.cell)
    ref, e_p = O.onebounce_sink_field(s.src, s.E, s.snk, s.snk_n, s.scat, s.scat_n, 0.0, beta, grid=og)
    assert rel_err(E, ref) < FIELD_TOL
    # tracing the one bounce only from the scattering points some source sees: the same field, fewer tests
    seen = og.mask(s.src, s.scat).any(0)
    seen[:min(len(s.src), len(s.scat))] = True  # self_to_self=False: the pair n == p is untested, so visible
    assert 0 < seen.sum() < len(seen)
    cnt_l = torch.zeros(2, dtype=torch.int64, device="cuda")
    El = sink_field(type("S", (), {"device": dev})(), s.src, s.E, s.snk, s.snk_n, 0.0, beta, s.scat, s.scat_n,
                    scattering=1, counters=cnt_l, skip_unlit=True).cpu().numpy()
    assert rel_err(El, ref) < FIELD_TOL and rel_err(El, E) < 1e-6
    assert 0 < int(cnt_l[1]) < int(cnt[1])
    # stage masks are bit-exact against the oracle
    for a, an, b, bn in ((s.src, s.src_n, s.snk, s.snk_n), (s.src, s.src_n, s.scat, s.scat_n),
                         (s.scat, s.scat_n, s.snk, s.snk_n)):
        r = P.pair_stage(a, np.ones((a.shape[0], 3), np.complex64), b, bn, beta=beta, grid=dev.grid, want_mask=True)
        assert np.array_equal(r.mask().cpu().numpy(), og.mask(a, b))


def test_bounce_config_full_geometry_slice():
    """The 28 GHz one-bounce workload at full geometry (32x32 array, all 120,000 triangles, the 0.5 m
    grid) on a slice of its sinks (every 128th, 511) and scatter points (every 125th, 400), through the
    same kernels, processing orders and grid as the benchmarked step: per-stage masks bit-exact against
    the oracle, the sink field within FIELD_TOL of the FP64 oracle."""
    from lyceanem_gb300 import scenes
    P = _P()
    s = scenes.bounce_scene()
    beta = 2 * np.pi / s.wavelength
    snk, snk_n = s.snk[::128], s.snk_n[::128]
    scat, scat_n = s.scat[::125], s.scat_n[::125]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    tris = P.pack_triangles(t(s.verts), t(s.faces))
    grid = P.UniformGrid(tris, cell=s.cell)
    src, E, yk, ykn, pk, pkn = t(s.src), t(s.E), t(snk), t(snk_n), t(scat), t(scat_n)
    o_snk, o_scat = P.direction_order(yk, grid.centre), P.spatial_order(pk)
    r0 = P.pair_stage(src, E, yk, ykn, beta=beta, grid=grid, want_mask=True, snk_order=o_snk)
    r1 = P.pair_stage(src, E, pk, pkn, beta=beta, grid=grid, want_mask=True, snk_order=o_scat)
    field = r0.sink.clone()
    r2 = P.pair_stage(pk, r1.sink, yk, ykn, beta=beta, grid=grid, src_W=r1.sink, sink_out=field, accumulate=True,
                      want_mask=True, src_order=o_scat, snk_order=o_snk)
    _no_device_errors()
    og = O.Grid(O.pack_triangles(s.verts, s.faces), s.cell)
    m0, m1, m2 = og.mask(s.src, snk), og.mask(s.src, scat), og.mask(scat, snk)
    assert np.array_equal(r0.mask().cpu().numpy(), m0)
    assert np.array_equal(r1.mask().cpu().numpy(), m1)
    assert np.array_equal(r2.mask().cpu().numpy(), m2)
    assert 0 < m2.sum() < m2.size and 0 < m0.sum() < m0.size  # the slice sees both blocked and visible paths
    ep = O.sink_field(s.src, s.E, scat, scat_n, 0.0, beta, mask=m1)
    ref = O.sink_field(s.src, s.E, snk, snk_n, 0.0, beta, mask=m0)
    ref = ref + O.sink_field(scat, ep, snk, snk_n, 0.0, beta, srcW=ep, mask=m2)
    assert rel_err(r1.sink.cpu().numpy(), ep) < FIELD_TOL
    assert rel_err(field.cpu().numpy(), ref) < FIELD_TOL


@pytest.mark.parametrize("traversal", [36, 38, 1, 102, 104, 203])
def test_grid_schedules_bit_identical_full_geometry(traversal):
    """Every grid schedule (lockstep capped and uncapped; the transposed schedule; two phases split at 2, 4 and 3
    cells) gives the
    oracle's masks and the same sink field on the full 28 GHz geometry (slice of sinks and scatter points,
    the benchmarked processing orders), for the array-to-sink and scatter-to-sink stages, with and without
    the test counters."""
    from lyceanem_gb300 import scenes
    P = _P()
    s = scenes.bounce_scene()
    beta = 2 * np.pi / s.wavelength
    snk, snk_n = s.snk[::97], s.snk_n[::97]
    scat, scat_n = s.scat[::131], s.scat_n[::131]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    grid = P.UniformGrid(P.pack_triangles(t(s.verts), t(s.faces)), cell=s.cell)
    yk, ykn, pk = t(snk), t(snk_n), t(scat)
    o_snk, o_scat = P.direction_order(yk, grid.centre), P.spatial_order(pk)
    og = O.Grid(O.pack_triangles(s.verts, s.faces), s.cell)
    W = torch.ones((pk.shape[0], 3), dtype=torch.complex64, device="cuda")
    for a, b, bn, kw in ((s.src, snk, snk_n, dict(snk_order=o_snk)),
                         (scat, snk, snk_n, dict(src_order=o_scat, snk_order=o_snk, src_W=W))):
        E = np.ones((a.shape[0], 3), np.complex64)
        ref = P.pair_stage(a, E, b, bn, beta=beta, grid=grid, want_mask=True, traversal=36, **kw)
        r = P.pair_stage(a, E, b, bn, beta=beta, grid=grid, want_mask=True, traversal=traversal, **kw)
        assert np.array_equal(r.mask().cpu().numpy(), og.mask(a, b))
        if traversal == 38:  # 32 sources per block, summed across the warp: another summation order
            assert rel_err(r.sink.cpu().numpy(), ref.sink.cpu().numpy()) < 1e-6
        else:
            assert torch.equal(r.sink, ref.sink)
        # with counters (the default schedule then runs its counting variant): same results
        cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
        rc = P.pair_stage(a, E, b, bn, beta=beta, grid=grid, want_mask=True, traversal=traversal, counters=cnt, **kw)
        assert torch.equal(rc.mask_bits, r.mask_bits) and torch.equal(rc.sink, r.sink)
        assert int(cnt[0]) == int(r.mask().sum()) and int(cnt[1]) > 0
    _no_device_errors()


def test_em_dropin_functions():
    """The four lyceanem.em functions against the oracle network."""
    from lyceanem_gb300 import em
    src, snk, snk_n, v, f, E = random_scene(21, n_src=6, n_snk=70, n_tris=130)
    beta = float(np.float32(2 * np.pi / 0.03))  # the em interface takes beta as float32
    normal = np.concatenate([np.tile([[0, 0, 1]], (6, 1)), snk_n]).astype(np.float32)
    args = (E[:, 0].real, E[:, 0].imag, E[:, 1].real, E[:, 1].imag, E[:, 2].real, E[:, 2].imag, normal)
    out = em.calculate_scattering_brute_force(src, snk, f, v, 0.03, *args, 0.0, beta, False)
    S = out.view(np.complex64).reshape(6, 70, 3)
    So, mask = O.scattering_network(src, E, snk, snk_n, O.pack_triangles(v, f), 0.0, beta)
    assert np.array_equal(np.any(S != 0, axis=-1), mask & np.any(So != 0, axis=-1))
    assert _pair_rel(S, So, src, snk, E, beta) < FIELD_TOL
    # tile structure: bins over y-z, then the tiles entry point
    ymin, zmin, w, ny, nz = -1.4, -1.4, 0.35, 9, 9
    counts = em.bin_counts_to_numpy(v, f, ny, nz, ymin, w, zmin)
    assert counts.shape == (ny * nz,) and counts.sum() >= f.shape[0]
    binned = em.bin_triangles_to_numpy(v, f, ny, nz, ymin, w, zmin, counts, int(counts.sum()))
    assert binned.shape == (3 * counts.sum(),)
    assert set(map(tuple, binned.reshape(-1, 3))) == set(map(tuple, f))
    out2 = em.calculate_scattering_tiles(src, snk, v, 0.03, *args, -2, 2, ymin, 2, zmin, 2, w, counts, binned, ny, nz,
                                         int(counts.sum()), 0.0, beta, False)
    S2 = out2.view(np.complex64).reshape(6, 70, 3)
    assert _pair_rel(S2, So, src, snk, E, beta) < FIELD_TOL
    assert np.array_equal(S2 == 0, S == 0)
    with pytest.raises(RuntimeError, match="normal.shape"):
        em.calculate_scattering_brute_force(src, snk, f, v, 0.03, *args[:6], normal[:5], 0.0, beta, False)


def test_bins_cover_every_overlapped_cell():
    from lyceanem_gb300 import em
    src, snk, snk_n, v, f, E = random_scene(4, n_tris=90, box=1.0)
    ymin, zmin, w, ny, nz = -1.5, -1.5, 0.25, 12, 12
    counts = em.bin_counts_to_numpy(v, f, ny, nz, ymin, w, zmin)
    binned = em.bin_triangles_to_numpy(v, f, ny, nz, ymin, w, zmin, counts, int(counts.sum())).reshape(-1, 3)
    start = np.concatenate([[0], np.cumsum(counts)])
    tri = v[f]
    for k in range(f.shape[0]):
        lo = tri[k].min(0) - 1e-3 * w
        hi = tri[k].max(0) + 1e-3 * w
        iy = np.clip(np.floor((np.array([lo[1], hi[1]]) - ymin) / w), 0, ny - 1).astype(int)
        iz = np.clip(np.floor((np.array([lo[2], hi[2]]) - zmin) / w), 0, nz - 1).astype(int)
        for y in range(iy[0], iy[1] + 1):
            for z in range(iz[0], iz[1] + 1):
                c = y * nz + z
                assert any((binned[start[c]:start[c + 1]] == f[k]).all(1)), (k, y, z)


def test_numba_engine_visibility_mode():
    """cull=False, eps=1e-7: the numba engine's rule (rayfunctions.py:37-104)."""
    P = _P()
    src, snk, snk_n, v, f, E = random_scene(8, n_src=11, n_snk=200, n_tris=300)
    tris = P.pack_triangles(torch.from_numpy(v), torch.from_numpy(f))
    om = O.mask_brute(src, snk, O.pack_triangles(v, f), cull=False, eps=1e-7)
    r = P.pair_stage(src, E, snk, snk_n, beta=50.0, tris=tris, cull=False, eps=1e-7, want_mask=True)
    assert np.array_equal(r.mask().cpu().numpy(), om)
    g = P.UniformGrid(tris, cell=0.2)
    r2 = P.pair_stage(src, E, snk, snk_n, beta=50.0, grid=g, cull=False, eps=1e-7, want_mask=True)
    assert np.array_equal(r2.mask().cpu().numpy(), om)
    assert not np.array_equal(om, O.mask_brute(src, snk, O.pack_triangles(v, f)))


def test_self_to_self_flag():
    P = _P()
    src, snk, snk_n, v, f, E = random_scene(13, n_src=40, n_snk=40, n_tris=400, box=0.6)
    tris = P.pack_triangles(torch.from_numpy(v), torch.from_numpy(f))
    ot = O.pack_triangles(v, f)
    for sts in (False, True):
        om = O.mask_brute(src, snk, ot, self_to_self=sts)
        r = P.pair_stage(src, E, snk, snk_n, beta=30.0, tris=tris, self_to_self=sts, want_mask=True)
        assert np.array_equal(r.mask().cpu().numpy(), om)
        g = P.UniformGrid(tris)
        r = P.pair_stage(src, E, snk, snk_n, beta=30.0, grid=g, self_to_self=sts, want_mask=True)
        assert np.array_equal(r.mask().cpu().numpy(), om)


@pytest.mark.parametrize("n_src,n_snk,n_tris", [(1, 1, 0), (1, 33, 1), (33, 1, 129), (5, 129, 257), (70, 31, 128),
                                                (3, 200, 1000)])
def test_edge_sizes(n_src, n_snk, n_tris):
    P = _P()
    src, snk, snk_n, v, f, E = random_scene(n_src * 7 + n_snk, n_src=n_src, n_snk=n_snk, n_tris=max(n_tris, 1))
    v, f = v[:3 * n_tris], f[:n_tris]
    tris = P.pack_triangles(torch.from_numpy(v), torch.from_numpy(f))
    ot = O.pack_triangles(v, f)
    om = O.mask_brute(src, snk, ot)
    beta = 2 * np.pi / 0.02
    ref = O.sink_field(src, E, snk, snk_n, 0.0, beta, mask=om)
    r = P.pair_stage(src, E, snk, snk_n, beta=beta, tris=tris, want_mask=True, want_pairs=True)
    assert np.array_equal(r.mask().cpu().numpy(), om)
    assert rel_err(r.sink.cpu().numpy(), ref) < FIELD_TOL
    g = P.UniformGrid(tris)  # also with no triangles: a one-cell grid whose cell table is empty
    r = P.pair_stage(src, E, snk, snk_n, beta=beta, grid=g, want_mask=True)
    assert np.array_equal(r.mask().cpu().numpy(), om)
    # the transposed schedule (lanes over up to 32 sources, fewer in a ragged last chunk), with the per-pair output
    rt = P.pair_stage(src, E, snk, snk_n, beta=beta, grid=g, want_mask=True, want_pairs=True, traversal=38)
    assert np.array_equal(rt.mask().cpu().numpy(), om)
    assert rel_err(rt.sink.cpu().numpy(), ref) < FIELD_TOL
    rb = P.pair_stage(src, E, snk, snk_n, beta=beta, tris=tris, want_pairs=True)
    assert rel_err(rt.pairs.cpu().numpy(), rb.pairs.cpu().numpy()) < 1e-6
    _no_device_errors()


def test_stage_buffer_checks():
    """Caller buffers of the wrong type or length are refused before any launch (the kernels index them
    without bounds checks)."""
    P = _P()
    src, snk, snk_n, v, f, E = random_scene(3, n_src=6, n_snk=40, n_tris=50)
    tris = P.pack_triangles(torch.from_numpy(v), torch.from_numpy(f))
    cu = dict(device="cuda")
    bad = [dict(src_order=torch.arange(6, dtype=torch.int64, **cu)),     # int64 order
           dict(src_order=torch.arange(7, dtype=torch.int32, **cu)),     # more entries than rows
           dict(snk_order=torch.arange(39, dtype=torch.int32, **cu)),    # not a permutation's length
           dict(snk_visible=torch.zeros(39, dtype=torch.int32, **cu)),   # too short
           dict(src_visible=torch.zeros(6, dtype=torch.int32)),          # host tensor
           dict(counters=torch.zeros(2, dtype=torch.int32, **cu))]       # int32 counters
    for kw in bad:
        with pytest.raises(ValueError):
            P.pair_stage(src, E, snk, snk_n, beta=10.0, tris=tris, **kw)
    r = P.pair_stage(src, E, snk, snk_n, beta=10.0, tris=tris, snk_visible=torch.zeros(40, dtype=torch.int32, **cu))
    assert r.sink.shape == (40, 3)
    _no_device_errors()


def test_empty_inputs():
    P = _P()
    z = np.zeros((0, 3), np.float32)
    r = P.pair_stage(z, np.zeros((0, 3), np.complex64), np.ones((4, 3), np.float32), np.ones((4, 3), np.float32),
                     beta=1.0, tris=None)
    assert torch.all(r.sink == 0)


def test_brute_force_test_counter_without_hits():
    P = _P()
    src, snk, snk_n, v, f, E = random_scene(2, n_src=3, n_snk=50, n_tris=300)
    v = v + np.float32(100.0)  # move every triangle far away: nothing blocks
    tris = P.pack_triangles(torch.from_numpy(v), torch.from_numpy(f))
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    P.pair_stage(src, E, snk, snk_n, beta=1.0, tris=tris, counters=cnt, self_to_self=True)
    torch.cuda.synchronize()
    assert int(cnt[0]) == 150 and int(cnt[1]) == 150 * 300


def test_repeatable_bits():
    P = _P()
    src, snk, snk_n, v, f, E = random_scene(6, n_src=64, n_snk=500, n_tris=800)
    tris = P.pack_triangles(torch.from_numpy(v), torch.from_numpy(f))
    g = P.UniformGrid(tris)
    a = P.pair_stage(src, E, snk, snk_n, beta=300.0, grid=g).sink.clone()
    b = P.pair_stage(src, E, snk, snk_n, beta=300.0, grid=g).sink.clone()
    assert torch.equal(a, b)


def test_frequency_domain_api():
    """calculate_scattering (elements False/True) and calculate_farfield through the model API."""
    from lyceanem_gb300.geometry import Mesh
    from lyceanem_gb300.models import frequency_domain as FD
    src, snk, snk_n, v, f, E = random_scene(17, n_src=5, n_snk=60, n_tris=100)
    solid = Mesh(v, [("triangle", f)])
    ap = Mesh(src, point_data={"Normals": np.tile([[0, 0, 1.0]], (5, 1)), "Area": np.full(5, 0.5)})
    sk = Mesh(snk, point_data={"Normals": snk_n})
    beta = 2 * np.pi / 0.04
    axis = np.array([1.0, 0, 0])
    Ex, Ey, Ez = FD.calculate_scattering(ap, sk, solid, axis, wavelength=0.04, beta=beta, cuda=True)
    # the CUDA engine's em bindings take beta as float32
    Eo = O.sink_field(src, np.tile(axis * 0.5, (5, 1)), snk, snk_n, 0.0, float(np.float32(beta)),
                      tris12=O.pack_triangles(v, f))
    assert rel_err(np.stack([Ex, Ey, Ez], 1), Eo) < FIELD_TOL
    Sx, Sy, Sz = FD.calculate_scattering(ap, sk, solid, axis, wavelength=0.04, beta=beta, elements=True, cuda=True)
    assert Sx.shape == (5, 60)
    assert rel_err(np.stack([Sx, Sy, Sz], -1).sum(0), Eo) < FIELD_TOL
    et, ep = FD.calculate_farfield(ap, solid, axis, az_range=np.linspace(-180, 180, 9),
                                   el_range=np.linspace(-90, 90, 5), wavelength=0.04, farfield_distance=5.0, beta=beta,
                                   cuda=True)
    assert et.shape == (45,) and np.isfinite(et).all() and np.isfinite(ep).all()


def test_spatial_order_and_ordered_stages():
    """A spatial order is a permutation, and ordered stages give the same masks (and fields to rounding)."""
    P = _P()
    src, snk, snk_n, v, f, E = random_scene(31, n_src=150, n_snk=700, n_tris=600)
    tris = P.pack_triangles(torch.from_numpy(v), torch.from_numpy(f))
    o_src, o_snk = P.spatial_order(src), P.spatial_order(snk)
    assert sorted(o_snk.cpu().tolist()) == list(range(700))
    assert sorted(o_src.cpu().tolist()) == list(range(150))
    om = O.mask_brute(src, snk, O.pack_triangles(v, f))
    g = P.UniformGrid(tris, cell=0.25)
    for kw in (dict(tris=tris), dict(grid=g), dict(grid=g, traversal=38)):
        a = P.pair_stage(src, E, snk, snk_n, beta=80.0, want_mask=True, want_pairs=True, **kw)
        b = P.pair_stage(src, E, snk, snk_n, beta=80.0, want_mask=True, want_pairs=True, src_order=o_src,
                         snk_order=o_snk, **kw)
        assert np.array_equal(b.mask().cpu().numpy(), om)
        assert torch.equal(a.pairs, b.pairs)
        assert rel_err(b.sink.cpu().numpy(), a.sink.cpu().numpy()) < 1e-6
    _no_device_errors()


@pytest.mark.parametrize("mode", ["brute", "grid", "grid38"])
def test_source_subset_order(mode):
    """A src_order shorter than the source arrays traces only the listed rows: their mask rows, per-pair
    rows and visible counts are the full stage's, the other rows stay zero, and the field is the oracle's sum
    over the listed sources.  Rows 0 and 3 are listed, so the untested pairs (0, 0) and (3, 3) of
    self_to_self=False stay with their rows."""
    P = _P()
    src, snk, snk_n, v, f, E = random_scene(53, n_src=70, n_snk=90, n_tris=300)
    tris = P.pack_triangles(torch.from_numpy(v), torch.from_numpy(f))
    om = O.mask_brute(src, snk, O.pack_triangles(v, f))
    rng = np.random.default_rng(5)
    sub = np.unique(np.concatenate([rng.choice(70, size=37, replace=False), [0, 3]]))[::-1].copy()
    keep = np.zeros(70, bool)
    keep[sub] = True
    if mode == "brute":
        kw = dict(tris=tris)
    else:
        kw = dict(grid=P.UniformGrid(tris), traversal=38 if mode == "grid38" else 0)
    vis = torch.zeros(70, dtype=torch.int32, device="cuda")
    order = torch.from_numpy(sub.astype(np.int32)).cuda()
    r = P.pair_stage(src, E, snk, snk_n, beta=50.0, want_mask=True, want_pairs=True, src_visible=vis,
                     src_order=order, **kw)
    full = P.pair_stage(src, E, snk, snk_n, beta=50.0, want_mask=True, want_pairs=True, **kw)
    mk = r.mask().cpu().numpy()
    assert mk.shape == om.shape
    assert np.array_equal(mk[keep], om[keep]) and not mk[~keep].any()
    assert np.array_equal(vis.cpu().numpy(), np.where(keep, om.sum(1), 0))
    pr, pf = r.pairs.cpu().numpy(), full.pairs.cpu().numpy()
    assert np.all(pr[~keep] == 0) and np.array_equal(pr[keep], pf[keep])
    ref = O.sink_field(src, E, snk, snk_n, 0.0, 50.0, mask=om & keep[:, None])
    assert rel_err(r.sink.cpu().numpy(), ref) < FIELD_TOL
    _no_device_errors()


def test_direction_order():
    """Direction order: a permutation that sorts by (elevation band, azimuth tile, position in the tile)
    seen from the centre, and ordered stages keep masks and fields."""
    from lyceanem_gb300 import scenes
    P = _P()
    el = np.linspace(-90.0, 90.0, 37)
    az = np.linspace(-180.0, 180.0, 72, endpoint=False)
    snk, snk_n, _, _ = scenes.farfield_sinks(10.0, el, az)
    centre = [0.2, -0.1, 0.05]
    o = P.direction_order(snk, centre).cpu().numpy()
    assert sorted(o.tolist()) == list(range(snk.shape[0]))
    d = snk.astype(np.float64) - np.array(centre)
    tile = max(0.009, 4 * np.sqrt(2 * np.pi ** 2 / snk.shape[0]))
    na = int(np.ceil(2 * np.pi / tile)) + 2
    fe = (np.arctan2(d[:, 2], np.hypot(d[:, 0], d[:, 1])) + np.pi / 2) / tile + 0.125
    fa = (np.arctan2(d[:, 1], d[:, 0]) + np.pi) / tile + 0.125
    be, ba = np.floor(fe), np.floor(fa)
    key = ((be * na + ba).astype(np.int64) << 12) | (np.floor((fe - be) * 64).astype(np.int64) << 6) | \
        np.floor((fa - ba) * 64).astype(np.int64)
    # sorted by the key, up to float32-vs-float64 rounding of points on a quantisation boundary
    assert np.mean(np.diff(key[o]) < 0) < 0.01
    src, _, _, v, f, _ = random_scene(32, n_src=40, n_snk=10, n_tris=400)
    E = np.tile(np.array([[1, 0, 0]], np.complex64), (40, 1))
    tris = P.pack_triangles(torch.from_numpy(v), torch.from_numpy(f))
    g = P.UniformGrid(tris, cell=0.3)
    om = O.mask_brute(src, snk, O.pack_triangles(v, f))
    a = P.pair_stage(src, E, snk, snk_n, beta=80.0, grid=g, want_mask=True)
    b = P.pair_stage(src, E, snk, snk_n, beta=80.0, grid=g, want_mask=True,
                     snk_order=P.direction_order(snk, g.centre))
    assert np.array_equal(b.mask().cpu().numpy(), om)
    assert torch.equal(a.sink, b.sink)  # one writer per sink, same chunk order
    _no_device_errors()


SWEEP_TOL = 1e-4  # relative Frobenius error of a mixed-precision sweep against FP64 (the stated bar)


@pytest.mark.parametrize("mode,tol", [("fp32", 2e-6), ("bf16x3g", SWEEP_TOL), ("fp16x3g", SWEEP_TOL)])
def test_beam_sweep_modes_against_fp64(mode, tol):
    """Beam sweep of a formed network against a complex128 product of the same network."""
    from lyceanem_gb300 import beam_sweep as BS
    from lyceanem_gb300 import scenes
    P = _P()
    s = scenes.sweep_scene(n_side=12, n_clutter=300, n_ground=20, el_n=21, az_n=40, n_beams=37)
    beta = 2 * np.pi / s.wavelength
    tris = P.pack_triangles(torch.from_numpy(s.verts), torch.from_numpy(s.faces))
    g = P.UniformGrid(tris, cell=0.5)
    G = BS.form_network(s.src, s.pol, s.snk, s.snk_n, beta=beta, grid=g)
    W = torch.from_numpy(s.weights).cuda()
    sw = BS.BeamSweep(G, mode)
    E = sw.fields(sw.run(W)).cpu().numpy()
    ref = torch.einsum("nmc,kn->mkc", G.cpu().to(torch.complex128), W.cpu().to(torch.complex128)).numpy()
    err = np.linalg.norm(E - ref) / np.linalg.norm(ref)
    assert err < tol, err
    # the network itself against the oracle
    om = O.Grid(O.pack_triangles(s.verts, s.faces), 0.5).mask(s.src, s.snk, self_to_self=True)
    Go = O.pair_field(s.src, np.tile(s.pol, (s.src.shape[0], 1)), s.snk, s.snk_n, om, 0.0, beta)
    assert _pair_rel(G.cpu().numpy(), Go, s.src, s.snk, np.tile(s.pol, (s.src.shape[0], 1)), beta) < FIELD_TOL


def _sweep_vs_fp64(G, W, mode):
    from lyceanem_gb300 import beam_sweep as BS
    sw = BS.BeamSweep(G, mode)
    E = sw.fields(sw.run(W)).cpu().numpy()
    ref = torch.einsum("nmc,kn->mkc", G.cpu().to(torch.complex128), W.cpu().to(torch.complex128)).numpy()
    _no_device_errors()
    return float(np.linalg.norm(E - ref) / np.linalg.norm(ref)), E, ref


@pytest.mark.parametrize("multicast", [True, False])
@pytest.mark.parametrize("k_tile", [64, 32])
@pytest.mark.parametrize("n_src,n_snk,n_beams", [(13, 300, 5), (200, 129, 257), (64, 128, 256), (1, 1, 1),
                                                  (8, 5, 3), (40, 1100, 600)])
def test_beam_sweep_tensor_core_shapes(multicast, k_tile, n_src, n_snk, n_beams):
    """The tensor-core kernel on ragged sizes (sources not a multiple of 8 or of the k-tile, sinks and
    beams across tile edges, odd and even counts of sink tiles) and on exact tile multiples, both k-tiles,
    with and without the two-CTA multicast clusters, against a complex128 product; every output column and
    row inside the sizes is written."""
    from lyceanem_gb300 import beam_sweep as BS
    g = torch.Generator().manual_seed(n_src * 7 + n_beams)
    G = torch.randn((n_src, n_snk, 3), dtype=torch.complex64, generator=g).cuda()
    W = torch.exp(2j * np.pi * torch.rand((n_beams, n_src), generator=g)).to(torch.complex64).cuda()
    BS.set_k_tile(k_tile)
    BS.set_multicast(multicast)
    try:
        for mode in ("bf16x3g", "fp16x3g"):
            err, E, ref = _sweep_vs_fp64(G, W, mode)
            assert err < SWEEP_TOL, (mode, err)
            # no entry is left unwritten (a stale tile would show as a large per-entry error)
            assert np.abs(E - ref).max() < 1e-3 * np.abs(ref).max(), mode
    finally:
        BS.set_k_tile(32)
        BS.set_multicast(False)


@pytest.mark.parametrize("scale", [1e-8, 1e-4, 1e4])
def test_beam_sweep_fp16_scaling(scale):
    """FP16 halves of a network of very small or very large entries: the power-of-two scaling keeps the
    halves out of FP16's subnormal and overflow ranges, so the error stays at the O(1) network's."""
    g = torch.Generator().manual_seed(5)
    G = (torch.randn((96, 700, 3), dtype=torch.complex64, generator=g) * scale).cuda()
    W = (torch.exp(2j * np.pi * torch.rand((40, 96), generator=g)) * 0.01).to(torch.complex64).cuda()
    for mode in ("fp16x3g", "bf16x3g"):
        err, _, _ = _sweep_vs_fp64(G, W, mode)
        assert err < SWEEP_TOL, (mode, scale, err)


def test_beam_sweep_repeat_and_reuse():
    """Two runs of one prepared sweep give identical results (the kernel writes every output once, from
    a fixed accumulation order), and a second weight set reuses the operand."""
    from lyceanem_gb300 import beam_sweep as BS
    g = torch.Generator().manual_seed(9)
    G = torch.randn((40, 333, 3), dtype=torch.complex64, generator=g).cuda()
    W1 = torch.randn((70, 40), dtype=torch.complex64, generator=g).cuda()
    W2 = torch.randn((70, 40), dtype=torch.complex64, generator=g).cuda()
    sw = BS.BeamSweep(G, "bf16x3g")
    a = sw.run(W1).clone()
    b = sw.run(W1).clone()
    assert torch.equal(sw.fields(a), sw.fields(b))
    c = sw.fields(sw.run(W2)).cpu().numpy()
    ref = torch.einsum("nmc,kn->mkc", G.cpu().to(torch.complex128), W2.cpu().to(torch.complex128)).numpy()
    assert np.linalg.norm(c - ref) / np.linalg.norm(ref) < SWEEP_TOL
    _no_device_errors()


@pytest.mark.parametrize("case", ["direct", "random"])
def test_masks_bit_exact_to_reference_device_code(case):
    """Our brute-force and grid masks against the reference's own hit() run on a GPU
    (tests/golden/reference_pairs.npz, both builds), and our field against its FP32 field."""
    import os
    P = _P()
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_pairs.npz"))
    g = {x: d[f"{case}_{x}"] for x in ("src", "snk", "snk_n", "verts", "faces", "E", "alpha", "beta", "flag",
                                       "sample")}
    N, M = g["src"].shape[0], g["snk"].shape[0]
    tris = P.pack_triangles(torch.from_numpy(g["verts"]), torch.from_numpy(g["faces"]))
    kw = dict(beta=float(g["beta"]), alpha=float(g["alpha"]), self_to_self=bool(g["flag"]), want_mask=True,
              want_pairs=True)
    for r in (P.pair_stage(g["src"], g["E"], g["snk"], g["snk_n"], tris=tris, **kw),
              P.pair_stage(g["src"], g["E"], g["snk"], g["snk_n"], grid=P.UniformGrid(tris), **kw)):
        mask = r.mask().cpu().numpy()
        for variant in ("fma", "nofma"):
            ref = np.unpackbits(d[f"{case}_{variant}_vis"])[:N * M].reshape(N, M).astype(bool)
            assert np.array_equal(mask, ref), f"{int((mask != ref).sum())} pairs differ from the reference"
        got = r.pairs.cpu().numpy().reshape(-1, 3)[g["sample"]]
        ref_f = d[f"{case}_fma_field"].astype(np.float32).view(np.complex64).reshape(-1, 3)
        assert np.abs(got - ref_f).max() / np.abs(ref_f).max() < 1e-3


def test_scene_cache_reuses_device_grid():
    """Repeated model calls on the same solid reuse its device triangles and grid; the results are
    identical and a different solid builds a new scene."""
    from lyceanem_gb300.geometry import Mesh
    from lyceanem_gb300.models import acceleration_structures as A
    from lyceanem_gb300.models import frequency_domain as FD
    src, snk, snk_n, v, f, E = random_scene(31, n_src=4, n_snk=50, n_tris=90)
    ap = Mesh(src, point_data={"Normals": np.tile([[0, 0, 1.0]], (4, 1)), "Area": np.ones(4)})
    sk = Mesh(snk, point_data={"Normals": snk_n})
    axis = np.array([0.0, 1.0, 0.0])
    h0, m0 = A.cache_stats["hits"], A.cache_stats["misses"]
    first = FD.calculate_scattering(ap, sk, Mesh(v, [("triangle", f)]), axis, beta=150.0, cuda=True)
    again = FD.calculate_scattering(ap, sk, Mesh(v.copy(), [("triangle", f.copy())]), axis, beta=150.0, cuda=True)
    assert A.cache_stats["misses"] == m0 + 1 and A.cache_stats["hits"] == h0 + 1
    for x, y in zip(first, again):
        assert np.array_equal(x, y)
    v2 = v.copy()
    v2[0, 0] += 0.01
    FD.calculate_scattering(ap, sk, Mesh(v2, [("triangle", f)]), axis, beta=150.0, cuda=True)
    assert A.cache_stats["misses"] == m0 + 2
    _no_device_errors()
