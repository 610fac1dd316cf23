"""Generates the golden fixtures of tests/golden from the reference (run in a
container where the reference tree is mounted; the fixtures are committed).

Fixtures:
  convert_triangles.npz   receive_horn.ply (raw bytes) and the reference's
                          triangle_type_array_ref.npy (lyceanem/tests/test_ray_functions.py:9-24)
  vector_mapping.npz      the six vector_mapping known-answer cases of
                          lyceanem/tests/test_empropagation.py:8-95, evaluated from the
                          test file's own assignments
  tile_structure.npz      bounds, tile size and cell counts computed by the
                          reference's Tile_acceleration_structure.__init__
                          (lyceanem/models/acceleration_structures.py:55-71), imported
                          with a recording stand-in for its compiled `em` module
  excitation.npz          the seven excitation_function known-answer cases of
                          lyceanem/tests/test_base_classes.py:70-152 (desired vector, pose
                          rotation, stated answer) and, for them and for steered and
                          area-weighted apertures, the outputs of the reference's own
                          excitation_function (lyceanem/electromagnetics/emfunctions.py:9-82)
                          and helpers, executed from their source text (the modules
                          themselves import numba and pyvista, absent here)
  numba_engine.npz        outputs of the reference's numba engine on small seeded scenes,
                          executed under numba_sim (a stand-in for numba and cupy that runs the
                          engine's kernels as Python with numba's typing of constants; see
                          numba_sim.py for what it reproduces and what it cannot):
                          workchunkingv2's path index and ray count
                          (lyceanem/raycasting/rayfunctions.py:2681-2955) for one, two and three
                          interactions, with and without line of sight; visiblespace (:316-427) on
                          an elevation-major shell standing in for pyvista's; EMGPUFreqDomain
                          (lyceanem/electromagnetics/empropagation.py:2197-2410) on those paths at
                          two wavelengths and with magnetic sources; TimeDomainv3 (:2910-3170) on a
                          one-block path list, with 400 and with 120 samples; and the model-level
                          calculate_scattering(cuda=False) (lyceanem/models/frequency_domain.py:
                          267-718) for direct, one- and two-bounce paths; the time-domain model
                          (lyceanem/models/time_domain.py) on a one-block scene.
  cuda_model.npz          the reference's CUDA-engine model layer (calculate_scattering(cuda=True),
                          calculate_scattering_cuda, Tile_acceleration_structure.calculate_scattering,
                          calculate_farfield; lyceanem/models/frequency_domain.py:94-264, 719-926,
                          lyceanem/models/acceleration_structures.py:72-115) executed from its source
                          with its compiled `em` module replaced by the oracle's per-pair network.
The numba_engine and cuda_model fixtures install stand-in modules, so each runs in its own process
(--only NAME); the others run together.
Usage: python tests/golden/make_golden.py [reference_root] [--only NAME]
"""
import ast
import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 and not sys.argv[1].startswith("--") else "/root/reference"
PKG = os.path.join(REF, "lyceanem")


def convert_triangles():
    ply = open(os.path.join(PKG, "tests", "data", "receive_horn.ply"), "rb").read()
    ref = np.load(os.path.join(PKG, "tests", "data", "triangle_type_array_ref.npy"))
    names = ["v0x", "v0y", "v0z", "v1x", "v1y", "v1z", "v2x", "v2y", "v2z"]
    tri = np.stack([ref[n] for n in names], axis=1).astype(np.float32)
    np.savez(os.path.join(HERE, "convert_triangles.npz"), ply=np.frombuffer(ply, np.uint8), triangles=tri)


def vector_mapping_cases():
    from scipy.spatial.transform import Rotation as R
    src = open(os.path.join(PKG, "tests", "test_empropagation.py")).read()
    tree = ast.parse(src)
    rows = []
    for fn in tree.body:
        if not (isinstance(fn, ast.FunctionDef) and fn.name.startswith("test_vector_mapping")):
            continue
        ns = {"np": np, "R": R}
        for st in fn.body:
            if isinstance(st, ast.Assign):
                exec(compile(ast.Module(body=[st], type_ignores=[]), "<case>", "exec"), ns)
        rows.append((fn.name, ns["rotation_matrix"], ns["normal_vector"], ns["desired_E_vector"],
                     ns["final_E_vector"]))
    np.savez(os.path.join(HERE, "vector_mapping.npz"), names=np.array([r[0] for r in rows]),
             rotation=np.stack([r[1] for r in rows]), normal=np.stack([r[2] for r in rows]),
             desired=np.stack([r[3] for r in rows]), expected=np.stack([r[4] for r in rows]))


class _Cells:
    def __init__(self, data):
        self.data = data
        self.type = "triangle"


class _MeshStub:
    def __init__(self, points, faces):
        self.points = points
        self.cells = [_Cells(faces)]
        self.point_data = {}


def tile_structure():
    calls = []
    em = types.ModuleType("lyceanem.em")

    def bin_counts_to_numpy(*a):
        calls.append(("counts", a[2:]))
        return np.ones(a[2] * a[3], np.int32)

    def bin_triangles_to_numpy(*a):
        return np.zeros(3 * int(a[8]), np.int32)

    em.bin_counts_to_numpy = bin_counts_to_numpy
    em.bin_triangles_to_numpy = bin_triangles_to_numpy
    em.calculate_scattering_brute_force = None
    em.calculate_scattering_tiles = None
    pkg = types.ModuleType("lyceanem")
    pkg.__path__ = []
    sys.modules["lyceanem"] = pkg
    sys.modules["lyceanem.em"] = em
    spec = importlib.util.spec_from_file_location("ref_accel", os.path.join(PKG, "models", "acceleration_structures.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    rng = np.random.default_rng(123)
    meshes = []
    for k in range(6):
        pts = (rng.normal(size=(30, 3)) * rng.uniform(0.1, 5, size=3) + rng.normal(size=3) * 3).astype(np.float32)
        if k == 5:
            pts[:, 2] = -1.0  # a flat mesh (zero extent in z, nonzero margin)
        faces = rng.integers(0, 30, size=(20, 3)).astype(np.int32)
        meshes.append((pts, faces, int(rng.integers(1, 6))))
    out_pts, out_faces, out_n, out_vals = [], [], [], []
    for pts, faces, n_cells in meshes:
        t = mod.Tile_acceleration_structure(_MeshStub(pts, faces), n_cells)
        out_pts.append(pts)
        out_faces.append(faces)
        out_n.append(n_cells)
        out_vals.append([t.max_x, t.min_x, t.max_y, t.min_y, t.max_z, t.min_z, t.tile_size, t.y_cells_count,
                         t.z_cells_count])
    np.savez(os.path.join(HERE, "tile_structure.npz"), points=np.stack(out_pts), faces=np.stack(out_faces),
             n_cells=np.array(out_n), values=np.array(out_vals, np.float64))


def _functions(path, names, strip_decorators=True):
    """Source of the named top-level functions of a reference file, decorators (numba's njit) and
    function-local imports removed, as one module to exec."""
    class _NoImports(ast.NodeTransformer):
        def visit_Import(self, node):
            return ast.Pass()

        visit_ImportFrom = visit_Import

    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", SyntaxWarning)  # escape sequences in the reference's docstrings
        tree = ast.parse(open(path).read())
    out = []
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and node.name in names:
            if strip_decorators:
                node.decorator_list = []
            out.append(_NoImports().visit(node))
    return ast.fix_missing_locations(ast.Module(body=out, type_ignores=[]))


class _PointCloud:
    def __init__(self, points, normals, area=None):
        self.points = points
        self.point_data = {"Normals": normals}
        if area is not None:
            self.point_data["Area"] = area


def excitation_cases():
    import scipy.constants
    from scipy.spatial import distance
    from scipy.spatial.transform import Rotation as R
    ns = {"np": np, "scipy": scipy, "distance": distance, "__name__": "reference_functions"}
    for rel, names in ((("electromagnetics", "empropagation.py"), {"vector_mapping", "calculate_conformalVectors"}),
                       (("electromagnetics", "beamforming.py"), {"WavefrontWeights", "ArbitaryCoherenceWeights"}),
                       (("utility", "math_functions.py"), {"discrete_transmit_power"}),
                       (("electromagnetics", "emfunctions.py"), {"excitation_function"})):
        exec(compile(_functions(os.path.join(PKG, *rel), names), rel[-1], "exec"), ns)
    ref_excitation = ns["excitation_function"]
    # the known-answer cases: one point at +x of a unit cube with normal +x, antenna pose rotated
    src = open(os.path.join(PKG, "tests", "test_base_classes.py")).read()
    tree = ast.parse(src)
    names, desired, rot, stated, outputs = [], [], [], [], []

    class _Antenna:
        def __init__(self):
            self.pose = np.eye(4)

    for fn in tree.body:
        if not (isinstance(fn, ast.FunctionDef) and fn.name.startswith("test_excitation_function")):
            continue
        case = {"np": np, "R": R, "standard_antenna": _Antenna()}
        for st in fn.body:
            if isinstance(st, ast.Assign):
                exec(compile(ast.Module(body=[st], type_ignores=[]), "<case>", "exec"), case)
        pose = case["standard_antenna"].pose
        pt = (pose @ np.array([0.5, 0.0, 0.0, 1.0]))[:3].reshape(1, 3)
        nrm = (pose @ np.array([1.0, 0.0, 0.0, 0.0]))[:3].reshape(1, 3)
        names.append(fn.name)
        desired.append(case["desired_E_vector"])
        rot.append(pose[:3, :3])
        stated.append(case["final_vector"].reshape(3))
        outputs.append(np.asarray(ref_excitation(_PointCloud(pt, nrm), case["desired_E_vector"])).reshape(3))
    # steered and area-weighted apertures through the same function
    rng = np.random.default_rng(31)
    ap_pts = np.stack(np.meshgrid(np.arange(4) * 0.015, np.arange(4) * 0.015, [0.0]), -1).reshape(-1, 3)
    ap_n = np.tile(np.array([[0.0, 0.0, 1.0]]), (16, 1))
    area = rng.uniform(0.5, 2.0, 16) * 1e-4
    steer = np.array([[0.3, -0.2, 0.93]])
    target = np.array([[0.4, 0.1, 2.0]])
    extra = []
    for label, kw, cloud in (
            ("wavefront_area", dict(phase_shift="wavefront", wavelength=0.03, steering_vector=steer,
                                    transmit_power=2.5), _PointCloud(ap_pts, ap_n, area)),
            ("coherence", dict(phase_shift="coherence", wavelength=0.03, steering_vector=target),
             _PointCloud(ap_pts, ap_n)),
            ("no_projection", dict(local_projection=False, wavelength=0.05, transmit_power=10.0),
             _PointCloud(ap_pts, ap_n, area))):
        d = np.array([[1.0, 0.5j, 0.0]], dtype=np.complex64) if label == "no_projection" else \
            np.array([0.0, 1.0, 0.0], dtype=np.complex64)
        extra.append((label, d.reshape(-1)[:3], kw, np.asarray(ref_excitation(cloud, d, **kw))))
    np.savez(os.path.join(HERE, "excitation.npz"), names=np.array(names), desired=np.stack(desired),
             rotation=np.stack(rot), stated=np.stack(stated), reference=np.stack(outputs),
             ap_points=ap_pts, ap_normals=ap_n, ap_area=area, steer=steer, target=target,
             extra_names=np.array([e[0] for e in extra]), extra_desired=np.stack([e[1] for e in extra]),
             extra_reference=np.stack([e[3] for e in extra]))


def _numba_scene(seed, n_src, n_snk, n_tris, n_scat):
    """Seeded scene of the numba-engine fixtures: sources below, sinks on a sphere, triangles and
    scatter points in a box (the recipe of tests/helpers.py random_scene, restated so the
    fixtures do not depend on it)."""
    rng = np.random.default_rng(seed)
    src = np.stack([rng.uniform(-0.5, 0.5, n_src), rng.uniform(-0.5, 0.5, n_src), np.full(n_src, -2.0)],
                   1).astype(np.float32)
    d = rng.normal(size=(n_snk, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    snk, snk_n = (4.0 * d).astype(np.float32), (-d).astype(np.float32)
    c = rng.uniform(-1.0, 1.0, size=(n_tris, 3))
    verts = (c[:, None, :] + rng.uniform(-0.3, 0.3, size=(n_tris, 3, 3))).reshape(-1, 3).astype(np.float32)
    faces = np.arange(3 * n_tris, dtype=np.int32).reshape(-1, 3)
    scat = rng.uniform(-1, 1, (n_scat, 3)).astype(np.float32)
    scat_n = rng.normal(size=(n_scat, 3)).astype(np.float32)
    scat_n /= np.linalg.norm(scat_n, axis=1, keepdims=True)
    w = (rng.normal(size=(n_src + n_snk + n_scat, 3)) + 1j * rng.normal(size=(n_src + n_snk + n_scat, 3)))
    return dict(src=src, snk=snk, snk_n=snk_n, verts=verts, faces=faces, scat=scat, scat_n=scat_n,
                w=w.astype(np.complex64))


def numba_engine():
    sys.path.insert(0, HERE)
    import numba_sim
    numba_sim.install()
    sys.path.insert(0, REF)
    import lyceanem.base_types as BT
    import lyceanem.electromagnetics.empropagation as EM
    import lyceanem.raycasting.rayfunctions as RF
    numba_sim.freeze_float_globals(RF)
    numba_sim.freeze_float_globals(EM)

    def environment(sc):
        v, f = sc["verts"], sc["faces"]
        env = np.empty(f.shape[0], dtype=BT.triangle_t)
        for k, c in enumerate("xyz"):
            for j in range(3):
                env[f"v{j}{c}"] = v[f[:, j], k]
        return env

    def points(sc, w, magnetic=0):
        n_src = sc["src"].shape[0]
        pos = np.concatenate([sc["src"], sc["snk"], sc["scat"]])
        nrm = np.concatenate([np.tile([[0, 0, 1.0]], (n_src, 1)), sc["snk_n"], sc["scat_n"]]).astype(np.float32)
        pts = np.zeros(pos.shape[0], dtype=BT.scattering_t.dtype)
        for k, c in enumerate("xyz"):
            pts[f"p{c}"], pts[f"n{c}"], pts[f"e{c}"] = pos[:, k], nrm[:, k], w[:, k]
        pts["Electric"] = True
        pts["Electric"][:magnetic] = False
        pts["permittivity"] = 8.8541878176e-12
        pts["permeability"] = 1.25663706212e-6
        return pts

    out = {}
    scenes = {"a": _numba_scene(13, 6, 40, 80, 25), "b": _numba_scene(11, 4, 20, 40, 12),
              "t": _numba_scene(4, 2, 16, 40, 5)}
    for name, sc in scenes.items():
        for k, val in sc.items():
            out[f"{name}_{k}"] = val
    # path index: (scene, max_scatter, line of sight)
    cases = [("a", 1, True), ("a", 2, True), ("a", 2, False), ("b", 3, True), ("b", 3, False), ("t", 2, True)]
    index = {}
    for name, ms, los in cases:
        sc = scenes[name]
        idx, rays = RF.workchunkingv2(sc["src"], sc["snk"], sc["scat"], environment(sc), ms, line_of_sight=los)
        key = f"{name}{ms}{'los' if los else 'nolos'}"
        out[f"index_{key}"], out[f"rays_{key}"] = idx, np.int64(rays)
        index[key] = idx
        print("  workchunkingv2", key, idx.shape, rays)
    # visiblespace (rayfunctions.py:316-427) on scene a's sources with seeded normals and a 4 m shell; the
    # shell comes from an elevation-major sphere standing in for targets.spherical_field (pyvista is absent)
    def sphere(az_range, elev_range, outward_normals=False, field_radius=1.0):
        E, A = np.meshgrid(np.deg2rad(elev_range), np.deg2rad(az_range), indexing="ij")
        d = np.stack([np.cos(E) * np.cos(A), np.cos(E) * np.sin(A), np.sin(E)], -1).reshape(-1, 3)
        return types.SimpleNamespace(points=(field_radius * d).astype(np.float32),
                                     point_data={"Normals": (d if outward_normals else -d).astype(np.float32)})
    RF.TG.spherical_field = sphere
    sc = scenes["a"]
    rng = np.random.default_rng(21)
    vs_nrm = rng.normal(size=sc["src"].shape).astype(np.float32)
    vs_nrm /= np.linalg.norm(vs_nrm, axis=1, keepdims=True)
    vs_area = rng.uniform(0.5, 1.5, sc["src"].shape[0])
    vs_area[2] = np.nan
    out["vs_normals"], out["vs_area"] = vs_nrm, vs_area
    for label, area, az, el in (("ones", np.array([0.0]), None, None), ("one_area", np.array([0.7]), None, None),
                                ("areas", vs_area, np.linspace(-180.0, 180.0, 13), np.linspace(-90.0, 90.0, 7))):
        kw = {} if az is None else dict(az_range=az, elev_range=el)
        pat, shell = RF.visiblespace(types.SimpleNamespace(points=sc["src"]), vs_nrm, environment(sc),
                                     vertex_area=np.array(area, copy=True), shell_range=4.0, **kw)
        out[f"vs_{label}"] = np.asarray(pat)
        out[f"vs_{label}_shell"] = np.asarray(shell.points)
        print("  visiblespace", label, np.asarray(pat).shape, float(np.nansum(pat)))
    # the model-level numba branch: calculate_scattering(cuda=False) (lyceanem/models/frequency_domain.py:267-718)
    # on meshio-like meshes; its module imports acceleration_structures, whose compiled `em` it never calls here
    em = types.ModuleType("lyceanem.em")
    for name in ("bin_counts_to_numpy", "bin_triangles_to_numpy", "calculate_scattering_brute_force",
                 "calculate_scattering_tiles"):
        setattr(em, name, None)
    sys.modules["lyceanem.em"] = em
    import meshio
    import lyceanem.models.frequency_domain as FD
    for name, sc in (("m", _numba_scene(8, 5, 50, 90, 20)), ("d", _numba_scene(9, 3, 20, 40, 8))):
        for k, val in sc.items():
            out[f"{name}_{k}"] = val
        n_src = sc["src"].shape[0]
        solid = meshio.Mesh(sc["verts"], [("triangle", sc["faces"])])
        sk = meshio.Mesh(sc["snk"], [], point_data={"Normals": sc["snk_n"]})
        sp = meshio.Mesh(sc["scat"], [], point_data={"Normals": sc["scat_n"]})
        cases = [(2, True, False, False)] if name == "d" else \
            [(0, True, False, False), (0, True, False, True), (1, True, False, False), (1, False, False, False),
             (1, True, True, False)]
        for scattering, los, elements, project in cases:
            ap = meshio.Mesh(sc["src"], [], point_data={"Normals": np.tile([[0, 0, 1.0]], (n_src, 1)),
                                                       "Area": np.full(n_src, 0.5)})
            res = FD.calculate_scattering(ap, sk, solid, np.array([[1.0, 0.0, 0.0]]), scatter_points=sp,
                                          wavelength=0.5, scattering=scattering, elements=elements, los=los,
                                          project_vectors=project, beta=2 * np.pi / 0.5, cuda=False)
            key = f"model_{name}_{scattering}{int(los)}{int(elements)}{int(project)}"
            out[key] = np.stack(res, -1)
            print("  calculate_scattering(cuda=False)", key, out[key].shape)
    # the time-domain model (lyceanem/models/time_domain.py:14-...) on scene t (its path lists stay within one
    # thread block of the time kernel, whose wake time is synchronised only within a block)
    import lyceanem.models.time_domain as TDM
    sc = scenes["t"]
    n_src = sc["src"].shape[0]
    exc = np.sin(np.linspace(0, 6 * np.pi, 40)) * np.hanning(40)
    solid = meshio.Mesh(sc["verts"], [("triangle", sc["faces"])])
    for label, kw in (("s0", dict(scattering=0, project_vectors=False)), ("s1", dict(scattering=1, project_vectors=False)),
                      ("s1_project", dict(scattering=1)), ("s1_elements", dict(scattering=1, elements=True,
                                                                                project_vectors=False))):
        ap = meshio.Mesh(sc["src"], [], point_data={"Normals": np.tile([[0, 0, 1.0]], (n_src, 1)),
                                                   "Area": np.full(n_src, 0.25)})
        sk = meshio.Mesh(sc["snk"], [], point_data={"Normals": sc["snk_n"]})
        sp = meshio.Mesh(sc["scat"], [], point_data={"Normals": sc["scat_n"]})
        try:
            res = TDM.calculate_scattering(ap, sk, exc, solid, np.array([1.0, 0.0, 0.0]), scatter_points=sp,
                                           wavelength=0.05, sampling_freq=20e9, num_samples=400, los=True,
                                           beta=2 * np.pi / 0.05, **kw)
        except TypeError as e:  # a reference call path that raises is recorded as such
            print("  time_domain.calculate_scattering", label, "raises TypeError:", e)
            out[f"td_{label}_raises"] = np.array(str(e))
            continue
        out[f"td_{label}"] = np.stack(res[:3], -1)
        out[f"td_{label}_wake"] = np.asarray(res[3], np.float64)
        print("  time_domain.calculate_scattering", label, out[f"td_{label}"].shape, np.asarray(res[3]))
    # per-path products: (case, wavelength, magnetic sources)
    alpha = 0.02
    for key, lam, mag in (("a2los", 0.5, 0), ("a2los", 0.05, 0), ("a2los", 0.5, 3), ("b3los", 0.5, 0)):
        sc = scenes[key[0]]
        S = EM.EMGPUFreqDomain(sc["src"].shape[0], sc["snk"].shape[0], index[key], points(sc, sc["w"], mag),
                               lam, alpha, 2 * np.pi / lam)
        out[f"field_{key}_{lam}_{mag}"] = S
        print("  EMGPUFreqDomain", key, lam, mag, S.shape)
    # time domain on one block of rows (the reference's wake time is block-synchronised only)
    sc = scenes["t"]
    idx = index["t2los"]
    assert idx.shape[0] <= 256, idx.shape
    rng = np.random.default_rng(2)
    n_pts = sc["w"].shape[0]
    wt = (rng.uniform(0.5, 1.5, (n_pts, 3)) + 1j * rng.uniform(0, 2e-9, (n_pts, 3))).astype(np.complex64)
    exc = np.sin(np.linspace(0, 6 * np.pi, 40)) * np.hanning(40)
    tm, wake = EM.TimeDomainv3(sc["src"].shape[0], sc["snk"].shape[0], points(sc, wt), idx, 0.25 * np.pi, 0.05, exc,
                               20e9, 400, alpha, 2 * np.pi / 0.05)
    out.update(time_w=wt, time_excitation=exc, time_map=tm, time_wake=np.float64(wake))
    print("  TimeDomainv3", tm.shape, wake)
    # a short map: the kernel cuts rows whose excitation would run past its end
    tm, wake = EM.TimeDomainv3(sc["src"].shape[0], sc["snk"].shape[0], points(sc, wt), idx, 0.25 * np.pi, 0.05, exc,
                               20e9, 120, alpha, 2 * np.pi / 0.05)
    out.update(time_map_short=tm, time_wake_short=np.float64(wake))
    print("  TimeDomainv3 short", tm.shape, wake)
    np.savez_compressed(os.path.join(HERE, "numba_engine.npz"), **out)


def cuda_model():
    """The reference's CUDA-engine model layer (calculate_scattering(cuda=True), calculate_scattering_cuda,
    Tile_acceleration_structure.calculate_scattering, calculate_farfield) run from its source, with its
    compiled `em` module replaced by the oracle: the per-pair networks are the oracle's (pinned to the
    reference's device code by reference_pairs.npz), everything composed around them is the reference's."""
    sys.path.insert(0, HERE)
    import numba_sim
    numba_sim.install()
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle import oracle as O
    em = types.ModuleType("lyceanem.em")

    def bin_counts_to_numpy(vertices, tri_index, ny, nz, ymin, cell, zmin):
        counts = np.zeros(int(ny) * int(nz), np.int32)
        counts[0] = np.asarray(tri_index).shape[0]  # one bin: the oracle's networks do not use the bins
        return counts

    def bin_triangles_to_numpy(vertices, tri_index, ny, nz, ymin, cell, zmin, counts, total):
        return np.ascontiguousarray(np.asarray(tri_index, np.int32).ravel())

    def calculate_scattering_tiles(source, end, vertices, wavelength, exr, exi, eyr, eyi, ezr, ezi, normal, xmin,
                                   xmax, ymin, ymax, zmin, zmax, tile, counts, binned, ny, nz, n_binned, alpha,
                                   beta, self_to_self):
        src, snk = np.asarray(source, np.float32), np.asarray(end, np.float32)
        tris = O.pack_triangles(np.asarray(vertices, np.float32), np.asarray(binned, np.int32).reshape(-1, 3))
        E = np.stack([np.asarray(exr) + 1j * np.asarray(exi), np.asarray(eyr) + 1j * np.asarray(eyi),
                      np.asarray(ezr) + 1j * np.asarray(ezi)], 1)
        S, _ = O.scattering_network(src, E, snk, np.asarray(normal, np.float32)[src.shape[0]:], tris,
                                    float(np.float32(alpha)), float(np.float32(beta)), self_to_self=bool(self_to_self))
        return S.astype(np.complex64).view(np.float32).ravel()

    em.bin_counts_to_numpy, em.bin_triangles_to_numpy = bin_counts_to_numpy, bin_triangles_to_numpy
    em.calculate_scattering_tiles = calculate_scattering_tiles
    em.calculate_scattering_brute_force = None
    sys.modules["lyceanem.em"] = em
    sys.path.insert(0, REF)
    import meshio
    import lyceanem.geometry.geometryfunctions as GF
    import lyceanem.geometry.targets as TL
    import lyceanem.models.frequency_domain as FD

    def sphere(az_range, elev_range, outward_normals=False, field_radius=1.0):
        # elevation-major sphere standing in for pyvista's; theta / phi from the reference's theta_phi_r
        E, A = np.meshgrid(np.deg2rad(elev_range), np.deg2rad(az_range), indexing="ij")
        d = np.stack([np.cos(E) * np.cos(A), np.cos(E) * np.sin(A), np.sin(E)], -1).reshape(-1, 3)
        m = meshio.Mesh((field_radius * d).astype(np.float32), [],
                        point_data={"Normals": (d if outward_normals else -d).astype(np.float32)})
        return GF.theta_phi_r(m)
    TL.spherical_field = sphere

    sc = _numba_scene(17, 5, 50, 90, 20)
    out = {f"s_{k}": v for k, v in sc.items()}
    n_src = sc["src"].shape[0]
    lam = 0.04

    def meshes():
        ap = meshio.Mesh(sc["src"], [], point_data={"Normals": np.tile([[0, 0, 1.0]], (n_src, 1)),
                                                   "Area": np.full(n_src, 0.5)})
        sk = meshio.Mesh(sc["snk"], [], point_data={"Normals": sc["snk_n"]})
        sp = meshio.Mesh(sc["scat"], [], point_data={"Normals": sc["scat_n"]})
        return ap, sk, sp, meshio.Mesh(sc["verts"], [("triangle", sc["faces"])])

    axis = np.array([[1.0, 0.0, 0.0]])
    for label, kw in (("s0", {}), ("s0_elements", dict(elements=True)), ("s0_project", dict(project_vectors=True)),
                      ("s1", dict(scattering=1)), ("s1_elements", dict(scattering=1, elements=True)),
                      ("s1_chunks2", dict(scattering=1, elements=True, chunks=2))):
        ap, sk, sp, solid = meshes()
        res = FD.calculate_scattering(ap, sk, solid, axis, scatter_points=sp, wavelength=lam, beta=2 * np.pi / lam,
                                      cuda=True, **kw)
        out[f"cs_{label}"] = np.stack(res, -1)
        print("  calculate_scattering(cuda=True)", label, out[f"cs_{label}"].shape)
    for label, kw in (("ff0", {}), ("ff1", dict(scattering=1))):
        ap, _, sp, solid = meshes()
        et, ep = FD.calculate_farfield(ap, solid, axis, az_range=np.linspace(-180, 180, 9),
                                       el_range=np.linspace(-90, 90, 5), scatter_points=sp, wavelength=lam,
                                       farfield_distance=5.0, beta=2 * np.pi / lam, cuda=True, **kw)
        out[f"{label}_theta"], out[f"{label}_phi"] = np.asarray(et), np.asarray(ep)
        print("  calculate_farfield(cuda=True)", label, np.asarray(et).shape)
    np.savez_compressed(os.path.join(HERE, "cuda_model.npz"), **out)


if __name__ == "__main__":
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    plain = (convert_triangles, vector_mapping_cases, tile_structure, excitation_cases)
    with_stand_ins = (numba_engine, cuda_model)  # each installs stand-in modules: one per process
    for fn in plain + with_stand_ins:
        if (only is None and fn in plain) or (only is not None and fn.__name__ == only):
            fn()
    print("golden fixtures written to", HERE)
