"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No dataset is involved; every scene is generated from numpy's default_rng
with a recorded seed.

  direct_scene     plain direct path, 8x8 array at 10 GHz, 2,664 far-field sinks
                   at 10 m, 1,024 small obstruction triangles (brute force)
  bounce_scene     direct + one bounce at 28 GHz: 32x32 array, 20x20 m ground
                   (80,000 triangles) + 40,000 clutter triangles, 50,000 scatter
                   points, 65,341 sinks at 100 m, 0.5 m grid cells
  adjoint_scene    the bounce recipe with a 16x16 array, 10,000 scatter points,
                   32,761 front-hemisphere sinks
  sweep_scene      64x64 array at 28 GHz, ground + 20,000 clutter triangles,
                   65,341 sinks, K steering vectors over the front hemisphere
  batched_scenes   uneven scenes for the persistent batched launch
Every generator takes scale arguments so tests can run reduced sizes.
"""
import numpy as np

C0 = 299792458.0


class Scene:
    """Host (numpy) description of one propagation problem."""

    def __init__(self, **kw):
        self.__dict__.update(kw)

    def __repr__(self):
        keys = ", ".join(f"{k}={getattr(self, k).shape if hasattr(getattr(self, k), 'shape') else getattr(self, k)}"
                         for k in sorted(self.__dict__))
        return f"Scene({keys})"


def planar_array(nx, ny, wavelength, z=0.0):
    """nx x ny half-wavelength array centred on the origin in the plane z, normals +z."""
    p = wavelength / 2.0
    xs = (np.arange(nx) - (nx - 1) / 2.0) * p
    ys = (np.arange(ny) - (ny - 1) / 2.0) * p
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), np.full(X.size, z)], axis=1).astype(np.float32)
    nrm = np.tile(np.array([[0.0, 0.0, 1.0]], np.float32), (pts.shape[0], 1))
    return pts, nrm


def farfield_sinks(radius, el_deg, az_deg):
    """Elevation-major sphere grid with inward normals."""
    el = np.deg2rad(np.asarray(el_deg, np.float64))
    az = np.deg2rad(np.asarray(az_deg, np.float64))
    E, A = np.meshgrid(el, az, indexing="ij")
    d = np.stack([np.cos(E) * np.cos(A), np.cos(E) * np.sin(A), np.sin(E)], axis=-1).reshape(-1, 3)
    return (radius * d).astype(np.float32), (-d).astype(np.float32), (np.pi / 2 - E).ravel(), A.ravel()


def front_hemisphere_sinks(radius, n_az, n_el):
    """Sinks on the hemisphere z >= 0 (boresight +z): az, el in [-90, 90] deg."""
    az = np.deg2rad(np.linspace(-90.0, 90.0, n_az))
    el = np.deg2rad(np.linspace(-90.0, 90.0, n_el))
    E, A = np.meshgrid(el, az, indexing="ij")
    d = np.stack([np.sin(A) * np.cos(E), np.sin(E), np.cos(A) * np.cos(E)], axis=-1).reshape(-1, 3)
    return (radius * d).astype(np.float32), (-d).astype(np.float32)


def fibonacci_sinks(radius, n):
    i = np.arange(n) + 0.5
    z = 1.0 - 2.0 * i / n
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = np.pi * (3.0 - np.sqrt(5.0)) * i
    d = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    return (radius * d).astype(np.float32), (-d).astype(np.float32)


def random_triangles(rng, n, lo, hi, half_offset):
    """n triangles with centroid-box uniform positions and vertex offsets U[-h, h]^3."""
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    c = lo + (hi - lo) * rng.random((n, 3))
    v = c[:, None, :] + rng.uniform(-half_offset, half_offset, size=(n, 3, 3))
    verts = v.reshape(-1, 3).astype(np.float32)
    faces = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    return verts, faces


def ground_plane(size, n, z):
    """size x size square at height z as n x n quads, two triangles each, normals +z."""
    xs = np.linspace(-size / 2.0, size / 2.0, n + 1)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    verts = np.stack([X.ravel(), Y.ravel(), np.full(X.size, z)], axis=1).astype(np.float32)
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a = (i * (n + 1) + j).ravel()
    b = ((i + 1) * (n + 1) + j).ravel()
    c = ((i + 1) * (n + 1) + j + 1).ravel()
    d = (i * (n + 1) + j + 1).ravel()
    faces = np.concatenate([np.stack([a, b, c], 1), np.stack([a, c, d], 1)]).astype(np.int32)
    return verts, faces


def merge(*meshes):
    vs, fs, off = [], [], 0
    for v, f in meshes:
        vs.append(v)
        fs.append(f + off)
        off += v.shape[0]
    return np.concatenate(vs).astype(np.float32), np.concatenate(fs).astype(np.int32)


def scatter_points(rng, verts, faces, n, offset=1e-3):
    """n distinct triangle centroids with face normals, lifted `offset` along the normal."""
    n = min(n, faces.shape[0])
    pick = np.sort(rng.choice(faces.shape[0], size=n, replace=False))
    v = verts.astype(np.float64)
    f = faces[pick]
    cen = (v[f[:, 0]] + v[f[:, 1]] + v[f[:, 2]]) / 3.0
    nrm = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
    return (cen + offset * nrm).astype(np.float32), nrm.astype(np.float32)


def direct_scene(seed=0, n_side=8, freq=10e9, el_step=5.0, az_step=5.0, radius=10.0, n_tris=1024):
    """8x8 isotropic array at 10 GHz, sinks on a 5 deg sphere at 10 m, 1,024 obstruction triangles."""
    rng = np.random.default_rng(seed)
    lam = 0.029979 if freq == 10e9 else C0 / freq
    src, src_n = planar_array(n_side, n_side, lam)
    el = np.arange(-90.0, 90.0 + 1e-9, el_step)
    az = np.arange(-180.0, 180.0 - 1e-9, az_step)
    snk, snk_n, theta, phi = farfield_sinks(radius, el, az)
    verts, faces = random_triangles(rng, n_tris, (-1, -1, 0.5), (1, 1, 1.5), 0.05)
    E = np.tile(np.array([[1, 0, 0]], np.complex64), (src.shape[0], 1))
    return Scene(name="direct", seed=seed, wavelength=lam, src=src, src_n=src_n, E=E, snk=snk, snk_n=snk_n,
                 theta=theta, phi=phi, verts=verts, faces=faces, scat=np.zeros((0, 3), np.float32),
                 scat_n=np.zeros((0, 3), np.float32), cell=None)


def bounce_scene(seed=1, n_side=32, freq=28e9, n_ground=200, ground_size=20.0, n_clutter=40000, n_scatter=50000,
                 el_n=181, az_n=361, radius=100.0, cell=0.5):
    """Direct + one-bounce scene at 28 GHz (ground plane + clutter, scatter points, 1 deg sphere)."""
    rng = np.random.default_rng(seed)
    lam = C0 / freq
    src, src_n = planar_array(n_side, n_side, lam)
    g = ground_plane(ground_size, n_ground, -1.0)
    h = ground_size / 2.0
    cl = random_triangles(rng, n_clutter, (-h, -h, 0.0), (h, h, 5.0), 0.25)
    verts, faces = merge(g, cl)
    scat, scat_n = scatter_points(rng, verts, faces, n_scatter)
    el = np.linspace(-90.0, 90.0, el_n)
    az = np.linspace(-180.0, 180.0, az_n)
    snk, snk_n, theta, phi = farfield_sinks(radius, el, az)
    E = np.tile(np.array([[1, 0, 0]], np.complex64), (src.shape[0], 1))
    return Scene(name="bounce", seed=seed, wavelength=lam, src=src, src_n=src_n, E=E, snk=snk, snk_n=snk_n,
                 theta=theta, phi=phi, verts=verts, faces=faces, scat=scat, scat_n=scat_n, cell=cell)


def adjoint_scene(seed=2, n_side=16, n_scatter=10000, n_az=181, n_el=181, **kw):
    """Differentiation scene: bounce recipe, 16x16 array, 10,000 scatter points, front-hemisphere sinks."""
    s = bounce_scene(seed=seed, n_side=n_side, n_scatter=n_scatter, el_n=2, az_n=2, **kw)
    s.snk, s.snk_n = front_hemisphere_sinks(100.0, n_az, n_el)
    rng = np.random.default_rng(seed + 1000)
    s.target_excitation = np.exp(1j * rng.uniform(0, 2 * np.pi, s.src.shape[0])).astype(np.complex64)
    s.name = "adjoint"
    return s


def steering_weights(src, directions, wavelength):
    """Unit-amplitude progressive-phase weights [K, N] steering toward unit directions [K,3].

    Same phases as WavefrontWeights (lyceanem/electromagnetics/beamforming.py:81-120)
    in its far-point limit: w_n = exp(j k (max_n(s.p_n) - s.p_n))."""
    k = 2 * np.pi / wavelength
    proj = directions.astype(np.float64) @ src.astype(np.float64).T
    ph = k * (proj.max(axis=1, keepdims=True) - proj)
    return np.exp(1j * ph).astype(np.complex64)


def sweep_scene(seed=3, n_side=64, freq=28e9, n_clutter=20000, with_ground=True, el_n=181, az_n=361, radius=100.0,
                n_beams=2048, n_ground=200, cell=0.5):
    """Beam sweep scene: 64x64 array, ground + 20,000 clutter triangles, 1 deg sphere, K steering vectors."""
    rng = np.random.default_rng(seed)
    lam = C0 / freq
    src, src_n = planar_array(n_side, n_side, lam)
    parts = []
    if with_ground:
        parts.append(ground_plane(20.0, n_ground, -1.0))
    parts.append(random_triangles(rng, n_clutter, (-10, -10, 0.0), (10, 10, 5.0), 0.25))
    verts, faces = merge(*parts)
    el = np.linspace(-90.0, 90.0, el_n)
    az = np.linspace(-180.0, 180.0, az_n)
    snk, snk_n, theta, phi = farfield_sinks(radius, el, az)
    z = rng.random(n_beams)
    ph = rng.uniform(0, 2 * np.pi, n_beams)
    r = np.sqrt(1 - z * z)
    dirs = np.stack([r * np.cos(ph), r * np.sin(ph), z], axis=1)
    W = steering_weights(src, dirs, lam)
    pol = np.array([1, 0, 0], np.complex64)
    return Scene(name="sweep", seed=seed, wavelength=lam, src=src, src_n=src_n, pol=pol, snk=snk, snk_n=snk_n,
                 theta=theta, phi=phi, verts=verts, faces=faces, weights=W, directions=dirs, cell=cell)


def batched_scenes(seed=4, n_scenes=64, elem_range=(16, 16384), tri_range=(1000, 500000), n_sinks=10000,
                   n_freqs=64, f_range=(24e9, 30e9), scatter_frac=0.1, max_scatter=10000):
    """Uneven scenes: log-uniform element and triangle counts, Fibonacci sinks at 50 m, linear frequency list."""
    rng = np.random.default_rng(seed)
    freqs = np.linspace(f_range[0], f_range[1], n_freqs)
    lam_c = C0 / np.mean(f_range)
    snk, snk_n = fibonacci_sinks(50.0, n_sinks)
    scenes = []
    for i in range(n_scenes):
        ne = int(np.exp(rng.uniform(np.log(elem_range[0]), np.log(elem_range[1]))))
        side = max(1, int(round(np.sqrt(ne))))
        nt = int(np.exp(rng.uniform(np.log(tri_range[0]), np.log(tri_range[1]))))
        src, src_n = planar_array(side, side, lam_c)
        n_ground = max(1, int(np.sqrt(nt * 2.0 / 3.0 / 2.0)))
        g = ground_plane(20.0, n_ground, -1.0)
        n_cl = max(0, nt - g[1].shape[0])
        cl = random_triangles(rng, n_cl, (-10, -10, 0.0), (10, 10, 5.0), 0.25)
        verts, faces = merge(g, cl)
        n_sc = int(min(max_scatter, max(1, scatter_frac * faces.shape[0])))
        scat, scat_n = scatter_points(rng, verts, faces, n_sc)
        scenes.append(Scene(name=f"batched{i}", src=src, src_n=src_n, verts=verts, faces=faces, scat=scat,
                            scat_n=scat_n))
    return scenes, snk, snk_n, freqs
