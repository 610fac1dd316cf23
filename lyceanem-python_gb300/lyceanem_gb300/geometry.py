"""Minimal mesh / point-cloud containers with the attribute shape of meshio.Mesh.

The reference passes meshio.Mesh objects around (lyceanem/models/acceleration_structures.py:55-72,
lyceanem/models/frequency_domain.py:195-264): `.points`, `.cells[i].type`,
`.cells[i].data`, `.point_data[...]`.  Any object with those attributes is
accepted by this package; these classes are provided because meshio is not a
dependency.
"""
import numpy as np


class CellBlock:
    def __init__(self, type, data):
        self.type = type
        self.data = np.asarray(data)


class Mesh:
    def __init__(self, points, cells=None, point_data=None, cell_data=None):
        self.points = np.asarray(points)
        self.cells = []
        for c in cells or []:
            if isinstance(c, CellBlock):
                self.cells.append(c)
            else:
                self.cells.append(CellBlock(c[0], c[1]))
        self.point_data = dict(point_data or {})
        self.cell_data = dict(cell_data or {})


def triangles_of(mesh):
    """(vertices float32 [V,3], faces int32 [T,3]) of a mesh-like object or list of them."""
    if isinstance(mesh, (list, tuple)):
        vs, fs, off = [], [], 0
        for m in mesh:
            v, f = triangles_of(m)
            vs.append(v)
            fs.append(f + off)
            off += v.shape[0]
        if not vs:
            return np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32)
        return np.concatenate(vs), np.concatenate(fs)
    if hasattr(mesh, "solids"):  # structures-like container
        return triangles_of(list(mesh.solids))
    pts = np.asarray(mesh.points, dtype=np.float32).reshape(-1, 3)
    faces = np.zeros((0, 3), np.int32)
    for c in getattr(mesh, "cells", []):
        if getattr(c, "type", "triangle") == "triangle":
            faces = np.asarray(c.data, dtype=np.int32).reshape(-1, 3)
    return np.ascontiguousarray(pts), np.ascontiguousarray(faces)


def spherical_field(az_range, elev_range, outward_normals=False, field_radius=1.0):
    """Far-field sink points on a sphere (elevation-major: every azimuth of the
    first elevation, then the next), with normals and theta/phi.

    Mirrors lyceanem/geometry/targets.py:448-497: inward normals unless
    outward_normals; point_data holds "Normals", "Radial_Distance_(m)",
    "theta_(Radians)" and "phi_(Radians)", formed from the stored points as
    theta_phi_r does (lyceanem/geometry/geometryfunctions.py:447-470: arccos of
    z / r and arctan2(y, x)).  Point order is this package's own."""
    az = np.deg2rad(np.asarray(az_range, dtype=np.float64))
    el = np.deg2rad(np.asarray(elev_range, dtype=np.float64))
    E, A = np.meshgrid(el, az, indexing="ij")
    E, A = E.ravel(), A.ravel()
    d = np.stack([np.cos(E) * np.cos(A), np.cos(E) * np.sin(A), np.sin(E)], axis=1)
    pts = (field_radius * d).astype(np.float32)
    nrm = d if outward_normals else -d
    r = np.linalg.norm(pts - np.zeros((1, 3)), axis=1)
    return Mesh(points=pts, point_data={
        "Normals": nrm.astype(np.float32), "Radial_Distance_(m)": r, "theta_(Radians)": np.arccos(pts[:, 2] / r),
        "phi_(Radians)": np.arctan2(pts[:, 1], pts[:, 0])})


_PLY_TYPES = {"char": "i1", "int8": "i1", "uchar": "u1", "uint8": "u1", "short": "i2", "int16": "i2",
              "ushort": "u2", "uint16": "u2", "int": "i4", "int32": "i4", "uint": "u4", "uint32": "u4",
              "float": "f4", "float32": "f4", "double": "f8", "float64": "f8"}


def read_ply(source):
    """Triangle mesh from a PLY file (ascii or binary, path or bytes) as a Mesh.

    Vertices keep their stored precision; faces must be triangles."""
    data = source if isinstance(source, (bytes, bytearray)) else open(source, "rb").read()
    end = data.index(b"end_header") + len(b"end_header")
    end = data.index(b"\n", end) + 1
    header = data[:end].decode("ascii").splitlines()
    fmt, elements = None, []
    for line in header:
        tok = line.split()
        if not tok:
            continue
        if tok[0] == "format":
            fmt = tok[1]
        elif tok[0] == "element":
            elements.append([tok[1], int(tok[2]), []])
        elif tok[0] == "property":
            elements[-1][2].append(tok[1:])
    body = data[end:]
    out = {}
    if fmt == "ascii":
        words = body.split()
        pos = 0
        for name, count, props in elements:
            rows = []
            for _ in range(count):
                row = []
                for p in props:
                    if p[0] == "list":
                        k = int(words[pos]); pos += 1
                        row.append([float(w) for w in words[pos:pos + k]]); pos += k
                    else:
                        row.append(float(words[pos])); pos += 1
                rows.append(row)
            out[name] = (props, rows)
    else:
        endian = "<" if fmt == "binary_little_endian" else ">"
        pos = 0
        for name, count, props in elements:
            if all(p[0] != "list" for p in props):
                dt = np.dtype([(p[1], endian + _PLY_TYPES[p[0]]) for p in props])
                arr = np.frombuffer(body, dtype=dt, count=count, offset=pos)
                pos += dt.itemsize * count
                out[name] = (props, [[arr[p[1]][i] for p in props] for i in range(count)])
            else:
                rows = []
                for _ in range(count):
                    row = []
                    for p in props:
                        if p[0] == "list":
                            ct = np.dtype(endian + _PLY_TYPES[p[1]])
                            it = np.dtype(endian + _PLY_TYPES[p[2]])
                            k = int(np.frombuffer(body, dtype=ct, count=1, offset=pos)[0]); pos += ct.itemsize
                            row.append(np.frombuffer(body, dtype=it, count=k, offset=pos).tolist())
                            pos += it.itemsize * k
                        else:
                            t = np.dtype(endian + _PLY_TYPES[p[0]])
                            row.append(np.frombuffer(body, dtype=t, count=1, offset=pos)[0]); pos += t.itemsize
                    rows.append(row)
                out[name] = (props, rows)
    vprops, vrows = out["vertex"]
    names = [p[-1] for p in vprops]
    xyz = [names.index(c) for c in ("x", "y", "z")]
    vdtype = np.float64 if any(p[0] in ("double", "float64") for p in vprops if p[-1] in "xyz") else np.float32
    pts = np.array([[r[i] for i in xyz] for r in vrows], dtype=vdtype)
    faces = np.zeros((0, 3), np.int32)
    if "face" in out:
        fprops, frows = out["face"]
        li = [i for i, p in enumerate(fprops) if p[0] == "list"][0]
        faces = np.array([r[li] for r in frows], dtype=np.int32).reshape(-1, 3)
    return Mesh(points=pts, cells=[("triangle", faces)])


def read_stl(source):
    """STL file (binary or ASCII, path or bytes) -> Mesh with unique points, one triangle cell block
    and the facet normals as cell_data["Normals"] (the scenes meshio reads for the reference)."""
    if isinstance(source, (bytes, bytearray)):
        raw = bytes(source)
    else:
        with open(source, "rb") as fh:
            raw = fh.read()
    binary = len(raw) >= 84 and len(raw) == 84 + 50 * int(np.frombuffer(raw[80:84], "<u4")[0])
    if binary:
        n = int(np.frombuffer(raw[80:84], "<u4")[0])
        rec = np.frombuffer(raw[84:84 + 50 * n], dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)),
                                                                  ("attr", "<u2")]))
        normals = rec["n"].astype(np.float32)
        tri = rec["v"].astype(np.float32)
    else:
        words = raw.decode("ascii", errors="replace").split()
        normals, verts = [], []
        i = 0
        while i < len(words):
            w = words[i].lower()
            if w == "normal":
                normals.append([float(x) for x in words[i + 1:i + 4]])
                i += 4
            elif w == "vertex":
                verts.append([float(x) for x in words[i + 1:i + 4]])
                i += 4
            else:
                i += 1
        tri = np.asarray(verts, np.float32).reshape(-1, 3, 3)
        normals = np.asarray(normals, np.float32).reshape(-1, 3)
    pts, inv = np.unique(tri.reshape(-1, 3), axis=0, return_inverse=True)
    faces = inv.reshape(-1, 3).astype(np.int32)
    return Mesh(pts.astype(np.float32), [("triangle", faces)], cell_data={"Normals": [normals]})


def mesh_conversion(conversion_object):
    """Triangle records (triangle_t layout) of a mesh, a list of meshes, or a structures-like object
    (lyceanem/geometry/geometryfunctions.py:473-510); anything else gives no triangles."""
    from .raycasting import convertTriangles, triangle_t
    if conversion_object is None:
        return np.empty(0, dtype=triangle_t)
    if hasattr(conversion_object, "triangles_base_raycaster"):
        return np.asarray(conversion_object.triangles_base_raycaster())
    if hasattr(conversion_object, "export_all_structures"):
        return mesh_conversion(list(conversion_object.export_all_structures()))
    if isinstance(conversion_object, (list, tuple)):
        parts = [mesh_conversion(item) for item in conversion_object]
        return np.concatenate(parts) if parts else np.empty(0, dtype=triangle_t)
    if hasattr(conversion_object, "points") and hasattr(conversion_object, "cells"):
        return convertTriangles(conversion_object)
    return np.empty(0, dtype=triangle_t)


def face_normals(vertices, faces):
    v = np.asarray(vertices, dtype=np.float64)
    f = np.asarray(faces)
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    ln[ln == 0] = 1.0
    return n / ln


def vector_mapping(local_E_vector, point_normal, rotation_matrix):
    """Local (u, v, n) E-vector of a face to global axes.

    Same construction as lyceanem/electromagnetics/empropagation.py:3693-3765:
    n = normal @ R; u = (z x n)/|z x n| unless n is along z, then (x x n)/|x x n|;
    v = (n x u)/|u x n|; result = local @ [u; v; n]."""
    dtype = np.asarray(local_E_vector).dtype
    n = np.matmul(np.asarray(point_normal).astype(dtype), rotation_matrix)
    if not np.iscomplexobj(np.zeros(0, dtype)):
        n = np.real(n)  # the axes of a real E-vector are real (the reference's store drops the zero imaginary part)
    axes = np.eye(3)
    uvn = np.zeros((3, 3), dtype=dtype)
    uvn[2, :] = n
    if abs(np.linalg.norm(np.cross(axes[:, 2], n))) == 0:
        c = np.cross(axes[0, :], n)
    else:
        c = np.cross(axes[2, :], n)
    uvn[0, :] = c / np.linalg.norm(c)
    uvn[1, :] = np.cross(n, uvn[0, :]) / np.linalg.norm(np.cross(uvn[0, :], n))
    return np.matmul(local_E_vector, uvn)


def calculate_conformal_vectors(desired_E_vector, source_normals, antenna_axes=np.eye(3)):
    """Per-source E-vectors conformal to the source normals
    (lyceanem/electromagnetics/empropagation.py:3807-3849)."""
    normals = np.asarray(source_normals)
    desired = np.asarray(desired_E_vector)
    out = np.zeros((normals.shape[0], 3), dtype=np.complex64)
    R = np.asarray(antenna_axes).astype(np.complex64)
    per_point = desired.ndim == 2 and desired.shape[0] == normals.shape[0]
    for i in range(normals.shape[0]):
        out[i, :] = vector_mapping(desired[i, :] if per_point else desired.ravel(), normals[i, :], R)
    return out
