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
Usage: python tests/golden/make_golden.py [reference_root]
"""
import ast
import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
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


if __name__ == "__main__":
    convert_triangles()
    vector_mapping_cases()
    tile_structure()
    excitation_cases()
    print("golden fixtures written to", HERE)
