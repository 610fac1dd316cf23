"""Golden vectors taken from the reference's own tests and code (tests/golden/make_golden.py)."""
import os

import numpy as np

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_convert_triangles_golden():
    """receive_horn.ply -> triangle records (lyceanem/tests/test_ray_functions.py:9-24)."""
    from lyceanem_gb300.geometry import read_ply, triangles_of
    d = np.load(os.path.join(GOLD, "convert_triangles.npz"))
    mesh = read_ply(d["ply"].tobytes())
    v, f = triangles_of(mesh)
    got = np.concatenate([v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]], axis=1)
    assert got.shape == d["triangles"].shape
    assert np.array_equal(got, d["triangles"])
    # the oracle's packing keeps v0 and forms the FP32 edges from the same vertices
    t = O.pack_triangles(v, f)
    assert np.array_equal(t[:, 0:3], d["triangles"][:, 0:3])
    assert np.array_equal(t[:, 4:7], d["triangles"][:, 3:6] - d["triangles"][:, 0:3])


def test_vector_mapping_golden():
    """Known answers of lyceanem/tests/test_empropagation.py:8-95."""
    from lyceanem_gb300.geometry import vector_mapping
    d = np.load(os.path.join(GOLD, "vector_mapping.npz"))
    for i in range(len(d["names"])):
        got = vector_mapping(d["desired"][i], d["normal"][i], d["rotation"][i])
        np.testing.assert_allclose(got, d["expected"][i], atol=1e-12, err_msg=str(d["names"][i]))


def test_tile_structure_geometry_golden():
    """Bounds / tile size / cell counts of Tile_acceleration_structure.__init__."""
    from lyceanem_gb300.models.acceleration_structures import tile_geometry
    d = np.load(os.path.join(GOLD, "tile_structure.npz"))
    keys = ["max_x", "min_x", "max_y", "min_y", "max_z", "min_z", "tile_size", "y_cells_count", "z_cells_count"]
    for pts, n_cells, vals in zip(d["points"], d["n_cells"], d["values"]):
        g = tile_geometry(pts, int(n_cells))
        got = np.array([g[k] for k in keys], np.float64)
        assert np.array_equal(got, vals), (got, vals)


class _Cloud:
    def __init__(self, points, normals, area=None):
        self.points = points
        self.point_data = {"Normals": normals}
        if area is not None:
            self.point_data["Area"] = area


def test_excitation_function_golden():
    """The seven known-answer cases of lyceanem/tests/test_base_classes.py:70-152 (one point at +x of a
    unit cube, normal +x, antenna pose rotated) and steered / area-weighted apertures, against the outputs
    of the reference's own excitation_function.  The stated answers are unit vectors; the reference
    function scales them to 1 W over the default area (|E| = sqrt(4 * 120 pi)), so they pin the direction."""
    from lyceanem_gb300.excitation import excitation_function
    d = np.load(os.path.join(GOLD, "excitation.npz"))
    for i in range(len(d["names"])):
        Rm = d["rotation"][i]
        pt = (Rm @ np.array([0.5, 0.0, 0.0])).reshape(1, 3)
        nrm = (Rm @ np.array([1.0, 0.0, 0.0])).reshape(1, 3)
        got = excitation_function(_Cloud(pt, nrm), d["desired"][i]).reshape(3)
        np.testing.assert_allclose(got, d["reference"][i], rtol=1e-6, atol=1e-5, err_msg=str(d["names"][i]))
        st = d["stated"][i]
        np.testing.assert_allclose(got / np.linalg.norm(got), st / np.linalg.norm(st), atol=1e-6)
        assert abs(np.linalg.norm(got) - np.sqrt(4 * 120 * np.pi)) < 1e-4
    kws = {"wavefront_area": dict(phase_shift="wavefront", wavelength=0.03, steering_vector=d["steer"],
                                  transmit_power=2.5),
           "coherence": dict(phase_shift="coherence", wavelength=0.03, steering_vector=d["target"]),
           "no_projection": dict(local_projection=False, wavelength=0.05, transmit_power=10.0)}
    for i, name in enumerate(d["extra_names"]):
        area = None if name == "coherence" else d["ap_area"]
        desired = d["extra_desired"][i].reshape(1, 3) if name == "no_projection" else d["extra_desired"][i]
        got = excitation_function(_Cloud(d["ap_points"], d["ap_normals"], area), desired, **kws[str(name)])
        np.testing.assert_allclose(got, d["extra_reference"][i], rtol=2e-6, atol=1e-4, err_msg=str(name))


def test_numba_engine_golden_oracle():
    """The oracle's numba-engine restatement against the reference's own numba engine (fixtures made by
    executing workchunkingv2, EMGPUFreqDomain and TimeDomainv3 from the reference's source,
    tests/golden/numba_sim.py): path index and ray count row for row, per-path products and the time map
    within the reference's own float32 rounding."""
    from helpers import (NUMBA_ALPHA, NUMBA_FIELD_CASES, NUMBA_INDEX_CASES, NUMBA_VS_SHELL, numba_golden,
                         numba_golden_magnetic, numba_golden_scene, numba_index_key, numba_vs_cases, rel_err)
    d = numba_golden()
    for scene, ms, los in NUMBA_INDEX_CASES:
        src, snk, scat, v, f, _, _, _ = numba_golden_scene(d, scene)
        masks = O.numba_masks(src, snk, scat, O.pack_triangles(v, f))
        idx, rays = O.numba_path_index(src.shape[0], snk.shape[0], scat.shape[0], *masks, ms, line_of_sight=los)
        key = numba_index_key(scene, ms, los)
        assert np.array_equal(idx, d[f"index_{key}"]), key
        assert rays == int(d[f"rays_{key}"]), key
    src, _, _, v, f, _, _, _ = numba_golden_scene(d, "a")
    for label, area, az, el in numba_vs_cases(d):
        shell = d[f"vs_{label}_shell"]
        mask = O.numba_masks(src, shell, np.zeros((0, 3), np.float32), O.pack_triangles(v, f))[0]
        pat = O.visible_patterns(src, d["vs_normals"], shell, mask, area)
        ref = d[f"vs_{label}"].reshape(-1)
        if label == "ones":
            assert np.array_equal(pat, ref)  # visible pairs in front of their source, counted
        assert rel_err(pat, ref) < 1e-5, label
    for key, lam, mag, tol in NUMBA_FIELD_CASES:
        src, snk, _, _, _, pos, nrm, w = numba_golden_scene(d, key[0])
        m, imp = numba_golden_magnetic(pos.shape[0], mag)
        S = O.path_field(d[f"index_{key}"], pos, nrm, w, src.shape[0], snk.shape[0], NUMBA_ALPHA, 2 * np.pi / lam,
                         magnetic=m if mag else None, impedance=imp if mag else None)
        assert rel_err(S, d[f"field_{key}_{lam}_{mag}"]) < tol, (key, lam, mag)
    src, snk, _, _, _, pos, nrm, _ = numba_golden_scene(d, "t")
    amp, arr, pair = O.path_times(d["index_t2los"], pos, nrm, d["time_w"], src.shape[0], snk.shape[0], NUMBA_ALPHA,
                                  2 * np.pi / 0.05)
    tm, wake = O.time_map(amp, arr, pair, src.shape[0], snk.shape[0], d["time_excitation"], 20e9, 400)
    assert abs(wake - float(d["time_wake"])) < 1e-14  # seconds: float32 path lengths in the reference
    assert rel_err(tm, d["time_map"]) < 1e-6
    tm, wake = O.time_map(amp, arr, pair, src.shape[0], snk.shape[0], d["time_excitation"], 20e9, 120)
    assert abs(wake - float(d["time_wake_short"])) < 1e-14
    assert rel_err(tm, d["time_map_short"]) < 1e-6



def test_numba_stand_in_typing():
    """The stand-in that ran the reference's numba engine for the fixtures reproduces numba's typing of
    constants: a float literal or global promotes float32 to FP64 (F = 1.0 / A), float32 x float32 stays
    float32, and a kernel's threads run block by block through cuda.syncthreads()."""
    import sys
    sys.path.insert(0, GOLD)
    try:
        import numba_sim
    finally:
        sys.path.remove(GOLD)
    ns = {"EPS": np.float64(1e-7)}
    src = ("def f(a, b):\n"
           "    F = 1.0 / a\n"
           "    p = a * b\n"
           "    rejected = -EPS < a < EPS\n"
           "    return F, p, rejected, 2 * EPS\n")
    exec(src, ns)
    import inspect
    import linecache
    linecache.cache["<numba_sim_test>"] = (len(src), None, src.splitlines(True), "<numba_sim_test>")
    ns["f"].__code__ = ns["f"].__code__.replace(co_filename="<numba_sim_test>")
    assert inspect.getsource(ns["f"]).startswith("def f")
    g = numba_sim._numba_typed(ns["f"])
    F, p, rejected, two_eps = g(np.float32(3.0), np.float32(0.1))
    assert type(F) is np.float64 and F == 1.0 / 3.0
    assert type(p) is np.float32 and p == np.float32(3.0) * np.float32(0.1)
    assert not rejected and type(two_eps) is np.float64
    # barrier: every thread of a block writes before any reads
    src2 = ("def k(buf, out):\n"
            "    i = cuda.grid(1)\n"
            "    buf[i] = i\n"
            "    cuda.syncthreads()\n"
            "    out[i] = buf[(i + 1) % 4 + 4 * (i // 4)]\n")
    ns2 = {"cuda": numba_sim._make_cuda()}
    exec(src2, ns2)
    linecache.cache["<numba_sim_test2>"] = (len(src2), None, src2.splitlines(True), "<numba_sim_test2>")
    ns2["k"].__code__ = ns2["k"].__code__.replace(co_filename="<numba_sim_test2>")
    kern = numba_sim._Kernel(ns2["k"])
    buf, out = np.zeros(8, np.int64), np.zeros(8, np.int64)
    kern[2, 4](buf, out)
    assert kern.lockstep and out.tolist() == [1, 2, 3, 0, 5, 6, 7, 4]


def test_numba_model_golden_oracle():
    """The oracle's composition of the numba branch of calculate_scattering (visibility rule, path index,
    per-path product, source sum) against the reference's own calculate_scattering(cuda=False) run under the
    numba stand-in, for the cases without vector projection."""
    from helpers import NUMBA_MODEL_CASES, numba_golden, numba_golden_scene, numba_model_key, rel_err
    d = numba_golden()
    beta = 2 * np.pi / 0.5
    for scene, scattering, los, elements, project in NUMBA_MODEL_CASES:
        if project:
            continue
        src, snk, scat, v, f, pos, nrm, _ = numba_golden_scene(d, scene)
        N, M, Pn = src.shape[0], snk.shape[0], scat.shape[0]
        Esrc = np.tile([[0.5 if scattering == 0 else 1.0, 0.0, 0.0]], (N, 1)).astype(np.complex64)
        masks = O.numba_masks(src, snk, scat, O.pack_triangles(v, f))
        idx, _ = O.numba_path_index(N, M, Pn, *masks, scattering + 1, line_of_sight=los)
        w = np.ones((N + M + Pn, 3), np.complex128)
        w[:N] = Esrc
        net = O.path_field(idx, pos, nrm, w, N, M, 0.0, beta)
        ref = d[numba_model_key(scene, scattering, los, elements, project)]
        assert rel_err(net if elements else net.sum(0), ref) < 1e-5, (scene, scattering, los, elements)


def test_cuda_model_golden_oracle():
    """The oracle's composition of the CUDA engine's model layer (source sum, one bounce with the scatter
    points excited by the summed source->scatter field, per-element networks, far-field projection) against
    the reference's own model functions run on the oracle's per-pair networks."""
    from helpers import CUDA_MODEL_LAMBDA, cuda_model_golden, rel_err
    from lyceanem_gb300.geometry import spherical_field
    d = cuda_model_golden()
    g = lambda k: d[f"s_{k}"]  # noqa: E731
    src, snk, snk_n, scat, scat_n = g("src"), g("snk"), g("snk_n"), g("scat"), g("scat_n")
    tris = O.pack_triangles(g("verts"), g("faces"))
    beta = float(np.float32(2 * np.pi / CUDA_MODEL_LAMBDA))  # the compiled em module takes beta as float32
    E = np.tile([[0.5, 0.0, 0.0]], (src.shape[0], 1))
    S0, _ = O.scattering_network(src, E, snk, snk_n, tris, 0.0, beta)
    assert rel_err(S0.sum(0), d["cs_s0"]) < 1e-6
    assert rel_err(S0, d["cs_s0_elements"]) < 1e-6
    field, _ = O.onebounce_sink_field(src, E, snk, snk_n, scat, scat_n, 0.0, beta, tris12=tris)
    assert rel_err(field, d["cs_s1"]) < 1e-6
    sh = spherical_field(np.linspace(-180, 180, 9), np.linspace(-90, 90, 5), 5.0)  # unit sphere, outward
    for label, bounce in (("ff0", False), ("ff1", True)):
        pn = np.asarray(sh.point_data["Normals"])
        F = (O.onebounce_sink_field(src, E, sh.points, pn, scat, scat_n, 0.0, beta, tris12=tris)[0] if bounce
             else O.scattering_network(src, E, sh.points, pn, tris, 0.0, beta)[0].sum(0))
        et, ep = O.farfield_theta_phi(F, sh.point_data["theta_(Radians)"], sh.point_data["phi_(Radians)"])
        assert rel_err(et, d[f"{label}_theta"]) < 1e-6 and rel_err(ep, d[f"{label}_phi"]) < 1e-6, label

