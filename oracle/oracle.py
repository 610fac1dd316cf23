"""NumPy front end of the CPU oracle (test infrastructure only).

This module is the oracle the CUDA path is compared with: tests, the smoke
check and the CPU-baseline leg of bench.py use it.  It is never imported by the product
package.  Visibility is the bit-faithful FP32 restatement in lyem_oracle.c;
fields are FP64.

Reference behaviour restated here (paths within LyceanEM-Python):
  - pair visibility + field per (source, sink): lyceanem/src/raycasting_brute_force.cuh:68-88,
    lyceanem/src/raycasting.cuh:19-95, lyceanem/src/em.cuh:18-120
  - the self_to_self flag: the C++ parameter `not_self_to_self` receives Python's
    self_to_self; when it is False the pair whose source index equals its sink
    index is not tested (lyceanem/src/raycasting_brute_force.cuh:27,
    lyceanem/models/acceleration_structures.py:99)
  - one-bounce composition: lyceanem/models/frequency_domain.py:195-264
  - source sum to sink fields: lyceanem/models/frequency_domain.py:847-849
  - far-field E_theta/E_phi: lyceanem/models/frequency_domain.py:179-190
  - visiblespace's projected-area sum per shell point: lyceanem/raycasting/rayfunctions.py:316-427
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_int = ctypes.c_int
_f32 = ctypes.c_float
_f64 = ctypes.c_double

EPSILON = np.float32(0.000001)  # lyceanem/src/math_utility.cuh:9


def _opt(arr):
    return None if arr is None else arr.ctypes.data_as(ctypes.c_void_p)


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        L.orc_pack_triangles.argtypes = [_f32p, _i64, _i32p, _i64, _f32p]
        L.orc_mask_brute.argtypes = [_f32p, _i64, _f32p, _i64, _f32p, _i64, _int, _int, _f32, _u8p, _int]
        L.orc_grid_build.argtypes = [_f32p, _i64, _f64, _f64]
        L.orc_grid_build.restype = _vp
        L.orc_grid_free.argtypes = [_vp]
        L.orc_grid_info.argtypes = [_vp, _f64p, _i32p, _i64p]
        L.orc_mask_grid.argtypes = [_vp, _f32p, _i64, _f32p, _i64, _int, _int, _f32, _u8p, _int]
        L.orc_pair_field.argtypes = [_f32p, _f64p, _i64, _f32p, _f32p, _i64, _vp, _f64, _f64, _f64p, _int]
        L.orc_sink_field.argtypes = [_f32p, _f64p, _vp, _i64, _f32p, _f32p, _i64, _vp, _vp, _vp, _i64,
                                     _int, _int, _f32, _f64, _f64, _f64p, _i64p, _int]
        L.orc_rays.argtypes = [_f32p, _i64, _f32p, _i64, _f32p]
        L.orc_hit_one.argtypes = [_f32p, _f32, _f32p, _f32p, _int, _f32]
        L.orc_hit_one.restype = _int
        L.orc_max_threads.restype = _int
        _lib = L
    return _lib


def _f3(a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, 3))
    return a


def _c6(E, n):
    """Complex (n,3) excitation -> float64 (n,6) interleaved (re, im)."""
    E = np.asarray(E)
    if E.ndim == 1:
        E = np.broadcast_to(E.reshape(1, 3), (n, 3))
    E = np.ascontiguousarray(E.astype(np.complex128).reshape(n, 3))
    return E.view(np.float64).reshape(n, 6).copy()


def max_threads():
    return int(lib().orc_max_threads())


def pack_triangles(verts, idx):
    """Mesh (V,3) + (T,3) -> (T,12) float32: v0, 0, e1, 0, e2, 0 per triangle."""
    v = _f3(verts)
    i = np.ascontiguousarray(np.asarray(idx, dtype=np.int32).reshape(-1, 3))
    out = np.zeros((i.shape[0], 12), dtype=np.float32)
    lib().orc_pack_triangles(v, v.shape[0], i, i.shape[0], out)
    return out


def rays(src, snk):
    s, e = _f3(src), _f3(snk)
    out = np.zeros((s.shape[0] * e.shape[0], 4), dtype=np.float32)
    lib().orc_rays(s, s.shape[0], e, e.shape[0], out)
    return out.reshape(s.shape[0], e.shape[0], 4)


def hit_one(d, length, origin, tri12, cull=True, eps=EPSILON):
    return bool(lib().orc_hit_one(np.ascontiguousarray(d, np.float32), np.float32(length),
                                  np.ascontiguousarray(origin, np.float32),
                                  np.ascontiguousarray(tri12, np.float32), int(cull), np.float32(eps)))


def mask_brute(src, snk, tris12, self_to_self=False, cull=True, eps=EPSILON, nthreads=0):
    """Bool (N,M): True where source n sees sink m (brute force over all triangles)."""
    s, e = _f3(src), _f3(snk)
    t = np.ascontiguousarray(tris12, dtype=np.float32).reshape(-1, 12)
    out = np.zeros((s.shape[0], e.shape[0]), dtype=np.uint8)
    lib().orc_mask_brute(s, s.shape[0], e, e.shape[0], t, t.shape[0], int(not self_to_self),
                         int(cull), np.float32(eps), out, nthreads)
    return out.astype(bool)


class Grid:
    """CPU uniform grid over packed triangles (any-hit, FP64 walk, padded boxes)."""

    def __init__(self, tris12, cell, pad=None):
        self.tris = np.ascontiguousarray(tris12, dtype=np.float32).reshape(-1, 12)
        pad = 1e-3 * cell if pad is None else pad
        self.h = lib().orc_grid_build(self.tris, self.tris.shape[0], float(cell), float(pad))
        oc = np.zeros(4, np.float64)
        dims = np.zeros(3, np.int32)
        nref = np.zeros(1, np.int64)
        lib().orc_grid_info(self.h, oc, dims, nref)
        self.origin, self.cell, self.dims, self.n_refs = oc[:3], oc[3], dims, int(nref[0])

    def mask(self, src, snk, self_to_self=False, cull=True, eps=EPSILON, nthreads=0):
        s, e = _f3(src), _f3(snk)
        out = np.zeros((s.shape[0], e.shape[0]), dtype=np.uint8)
        lib().orc_mask_grid(self.h, s, s.shape[0], e, e.shape[0], int(not self_to_self), int(cull),
                            np.float32(eps), out, nthreads)
        return out.astype(bool)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_grid_free(self.h)
            self.h = None


def pair_field(src, srcE, snk, snk_nrm, mask, alpha, beta, nthreads=0):
    """FP64 scattering network S[n, m, :] (complex128 (N,M,3)), zero where masked."""
    s, e, nr = _f3(src), _f3(snk), _f3(snk_nrm)
    N, M = s.shape[0], e.shape[0]
    E6 = _c6(srcE, N)
    mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8).reshape(N, M)
    out = np.zeros((N, M, 6), dtype=np.float64)
    lib().orc_pair_field(s, E6, N, e, nr, M, _opt(mk), float(alpha), float(beta), out, nthreads)
    return out.view(np.complex128).reshape(N, M, 3)


def sink_field(src, srcE, snk, snk_nrm, alpha, beta, mask=None, grid=None, tris12=None,
               srcW=None, self_to_self=False, cull=True, eps=EPSILON, nthreads=0,
               return_counters=False):
    """FP64 sink field out[m, c] = sum_n w[n, c] S[n, m, c] (complex128 (M,3)).

    Visibility comes from `mask` (bool (N,M)) if given, else it is traced here
    with `grid` (a Grid) or brute force over `tris12`."""
    s, e, nr = _f3(src), _f3(snk), _f3(snk_nrm)
    N, M = s.shape[0], e.shape[0]
    E6 = _c6(srcE, N)
    W6 = None if srcW is None else _c6(srcW, N)
    mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8).reshape(N, M)
    t = None
    T = 0
    if mask is None and grid is None:
        t = np.ascontiguousarray(tris12, dtype=np.float32).reshape(-1, 12)
        T = t.shape[0]
    out = np.zeros((M, 6), dtype=np.float64)
    cnt = np.zeros(2, np.int64)
    lib().orc_sink_field(s, E6, _opt(W6), N, e, nr, M, _opt(mk), grid.h if grid is not None else None,
                         _opt(t), T, int(not self_to_self), int(cull), np.float32(eps), float(alpha),
                         float(beta), out, cnt, nthreads)
    res = out.view(np.complex128).reshape(M, 3)
    if return_counters:
        return res, {"visible": int(cnt[0]), "tests": int(cnt[1])}
    return res


def scattering_network(src, srcE, snk, snk_nrm, tris12, alpha, beta, self_to_self=False,
                       grid=None, nthreads=0):
    """The reference's per-pair network (em.calculate_scattering_*): complex128 (N,M,3)."""
    if grid is not None:
        mask = grid.mask(src, snk, self_to_self=self_to_self, nthreads=nthreads)
    else:
        mask = mask_brute(src, snk, tris12, self_to_self=self_to_self, nthreads=nthreads)
    return pair_field(src, srcE, snk, snk_nrm, mask, alpha, beta, nthreads=nthreads), mask


def onebounce_sink_field(src, srcE, snk, snk_nrm, scat, scat_nrm, alpha, beta, grid=None,
                         tris12=None, los=True, nthreads=0):
    """Sink field of calculate_scattering_cuda(scatter_depth=1) summed over sources.

    total = S0 + S1 @ S2 per component with S2 driven by e_p = 1^T S1
    (frequency_domain.py:230-260), summed over sources (:847-849):
      E[m, c] = sum_n S0[n,m,c] + sum_p e_p[c] * S2[p,m,c].
    Returns (E (M,3) complex128, e_p (P,3) complex128)."""
    kw = dict(grid=grid, tris12=tris12, nthreads=nthreads)
    N = _f3(src).shape[0]
    M = _f3(snk).shape[0]
    direct = sink_field(src, srcE, snk, snk_nrm, alpha, beta, **kw) if los else np.zeros((M, 3), np.complex128)
    e_p = sink_field(src, srcE, scat, scat_nrm, alpha, beta, **kw)
    # the scatter points' excitation is stored as complex64 by the reference
    # (point_data assignment of a complex64 dot product); keep FP64 here.
    bounce = sink_field(scat, e_p, snk, snk_nrm, alpha, beta, srcW=e_p, **kw)
    del N
    return direct + bounce, e_p


def farfield_theta_phi(E, theta, phi):
    """E_theta / E_phi from cartesian E (frequency_domain.py:179-190)."""
    Ex, Ey, Ez = E[:, 0], E[:, 1], E[:, 2]
    et = Ex * np.cos(phi) * np.cos(theta) + Ey * np.sin(phi) * np.cos(theta) - Ez * np.sin(theta)
    ep = -Ex * np.sin(phi) + Ey * np.cos(phi)
    return et, ep


# ---------------------------------------------------------------- numba engine
# Restatement of the numba engine's path list and per-path product (test
# infrastructure), following its source and checked against the engine's own
# outputs on small scenes (tests/golden/numba_engine.npz, made by running the
# engine under a stand-in for numba and cupy):
#   path index   workchunkingv2 / create_model_index / rayHits1Dv2
#                (lyceanem/raycasting/rayfunctions.py:2624-2955, 1845-1878)
#   path product freqdomainkernal / sourcelaunchtransformGPU / lossy_propagation
#                (lyceanem/electromagnetics/empropagation.py:1083-1265, 179-258, 769-801)
#   visibility   hit without back-face culling, EPSILON 1e-7 (rayfunctions.py:19, 37-104),
#                every pair tested (create_model_index drops only index-equal end points).

NUMBA_EPSILON = np.float32(1e-7)


def numba_masks(src, snk, scat, tris12):
    """Visibility of the numba engine's three ray sets: (sources->sinks, sources->scatter,
    scatter->sinks, scatter->scatter), bool arrays."""
    kw = dict(self_to_self=True, cull=False, eps=NUMBA_EPSILON)
    P = _f3(scat).shape[0]
    m0 = mask_brute(src, snk, tris12, **kw)
    m1 = mask_brute(src, scat, tris12, **kw) if P else np.zeros((_f3(src).shape[0], 0), bool)
    m2 = mask_brute(scat, snk, tris12, **kw) if P else np.zeros((0, _f3(snk).shape[0]), bool)
    m3 = mask_brute(scat, scat, tris12, **kw) if P else np.zeros((0, 0), bool)
    return m0, m1, m2, m3


def visible_patterns(src, src_normals, shell, mask, vertex_area):
    """Per shell point, the summed projected area of the sources that see it: visiblespace's sum
    (lyceanem/raycasting/rayfunctions.py:316-427) from the numba-rule mask [sources, shell points].
    A visible pair adds area_n |cos angle| (angle between the float32 ray direction and the source
    normal, in FP64 here), nothing past pi / 2; a single zero area counts each visible pair as 1 and
    NaN areas count as 0.  Returns float64 [shell points]."""
    src, shell = _f3(src).astype(np.float64), _f3(shell).astype(np.float64)
    nrm = _f3(src_normals).astype(np.float64)
    area = np.nan_to_num(np.asarray(vertex_area, np.float64).reshape(-1), nan=0.0)
    n, m = np.nonzero(mask)
    d = shell[m] - src[n]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    u = nrm[n] / np.linalg.norm(nrm[n], axis=1, keepdims=True)
    c = np.clip(np.sum(d * u, axis=1), -1.0, 1.0)
    if area.size == 1:
        part = np.ones_like(c) if area[0] == 0 else area[0] * np.abs(c)
    else:
        part = area[n] * np.abs(c)
    part[c < 0] = 0.0
    return np.bincount(m, weights=part, minlength=shell.shape[0])


def numba_path_index(N, M, P, m0, m1, m2, m3, max_scatter, line_of_sight=True):
    """full_index and RAYS_CAST of workchunkingv2 (unchunked ordering for max_scatter 1 and 2;
    the source-chunked ordering of max_scatter 3).  Indices are 1-based into
    [sources, sinks, scatter points]."""
    snk0, sc0 = N + 1, N + M + 1
    if max_scatter == 1:
        n, m = np.nonzero(m0)
        return np.stack([n + 1, m + snk0], 1).astype(np.int32), N * (M + P)
    if max_scatter == 2:
        rows = []
        if line_of_sight:
            n, m = np.nonzero(m0)
            rows.append(np.stack([n + 1, m + snk0, np.zeros_like(n)], 1))
        n1, p1 = np.nonzero(m1)
        k, m = np.nonzero(m2[p1])
        rows.append(np.stack([n1[k] + 1, p1[k] + sc0, m + snk0], 1))
        rays = N * ((M if line_of_sight else 0) + P) + n1.size * M
        return np.concatenate(rows, 0).astype(np.int32).reshape(-1, 3), rays
    if max_scatter != 3:
        raise ValueError("max_scatter must be 1, 2 or 3")
    ray_estimate = N * (M + P) + N * (P * M * max_scatter)
    chunknum = max(2, min(N, int(np.ceil(ray_estimate / 2e8))))
    bounds = np.linspace(0, N, chunknum, dtype=np.int32)
    out = []
    rays = 0
    for c in range(bounds.size - 1):
        s0, s1 = int(bounds[c]), int(bounds[c + 1])
        rows = []
        if line_of_sight:
            n, m = np.nonzero(m0[s0:s1])
            rows.append(np.stack([n + s0 + 1, m + snk0, np.zeros_like(n), np.zeros_like(n)], 1))
        n1, p1 = np.nonzero(m1[s0:s1])
        n1 = n1 + s0
        # second wave: each (n, p) to every sink, then every scatter point q != p
        k, m = np.nonzero(m2[p1])
        rows.append(np.stack([n1[k] + 1, p1[k] + sc0, m + snk0, np.zeros_like(k)], 1))
        vis_q = m3[p1].copy()
        vis_q[np.arange(p1.size), p1] = False
        k2, q = np.nonzero(vis_q)
        # third wave: each (n, p, q) to every sink
        k3, m3_ = np.nonzero(m2[q])
        rows.append(np.stack([n1[k2][k3] + 1, p1[k2][k3] + sc0, q[k3] + sc0, m3_ + snk0], 1))
        out.append(np.concatenate(rows, 0))
        first = (s1 - s0) * ((M if line_of_sight else 0) + P)
        rays = first + n1.size * (M + P - 1) + k2.size * M  # the reference keeps the last chunk's count
    return np.concatenate(out, 0).astype(np.int32).reshape(-1, 4), rays


def _proj(f, x):
    """f - (f . x^) x^ for complex f (..., 3) and real x (..., 3)."""
    u = x / np.linalg.norm(x, axis=-1, keepdims=True)
    return f - np.sum(f * u, axis=-1, keepdims=True) * u


def _seg_loss(a, b, nb, alpha, beta):
    d = b - a
    r = np.linalg.norm(d, axis=-1)
    dn = d / r[:, None]
    G = np.exp(-(alpha + 1j * beta) * r) / r
    dG = (-(alpha + 1j * beta) - 1.0 / r) * G
    return -(1.0 / (2 * np.pi)) * dG * np.sum(dn * nb, axis=-1), dn


def path_field(full_index, pos, nrm, w, n_src, n_snk, alpha, beta, magnetic=None, impedance=None):
    """FP64 per-path product of freqdomainkernal summed per (source, sink): complex128 (N, M, 3).
    A zero index read as a point is the last point (Python's -1), as in the reference."""
    idx = np.asarray(full_index, dtype=np.int64)
    pos = np.asarray(pos, np.float32).astype(np.float64)
    nrm = np.asarray(nrm, np.float32).astype(np.float64)
    w = np.asarray(w).astype(np.complex128)
    npt = pos.shape[0]
    pt = np.where(idx > 0, idx - 1, npt - 1)
    R, K = idx.shape
    a0, a1 = pt[:, 0], pt[:, 1]
    f = w[a0].copy()
    if magnetic is not None and np.any(magnetic[a0]):
        sel = np.asarray(magnetic, bool)[a0]
        d = pos[a1] - pos[a0]
        d /= np.linalg.norm(d, axis=-1, keepdims=True)
        f[sel] = np.cross(w[a0][sel], d[sel]) / np.asarray(impedance, np.float64)[a0][sel][:, None]
    loss = np.ones(R, np.complex128)
    for i in range(K - 1):
        ai = pt[:, i]
        if i > 0:
            f = _proj(f, nrm[ai])
        has = idx[:, i + 1] != 0
        if np.any(has):
            b = pt[has, i + 1]
            L, dn = _seg_loss(pos[ai[has]], pos[b], nrm[b], alpha, beta)
            f[has] = _proj(f[has], dn) * w[b]
            loss[has] *= L
    f *= loss[:, None]
    last = np.zeros(R, np.int64)
    for i in range(K):
        last = np.where(idx[:, i] != 0, idx[:, i], last)
    out = np.zeros((n_src, n_snk, 3), np.complex128)
    np.add.at(out, (idx[:, 0] - 1, last - n_src - 1), f)
    return out


def numba_sink_field(src, srcE, snk, snk_nrm, scat, scat_nrm, alpha, beta, masks, scattering, los=True):
    """FP64 sink field of the numba engine for scattering 0 or 1 in factored form:
      scattering 0:  sum_n S0[n, m]
      scattering 1:  P(n_m) sum_n S0[n, m] (if los) + sum_p vis2 S2(p, m; P(n_p) e_p),  e_p = sum_n S1[n, p]
    (S the em_wave pair field, P the tangential projection), which equals the sum of
    path_field over workchunkingv2's rows."""
    m0, m1, m2, _ = masks
    kw = dict(self_to_self=True, cull=False, eps=NUMBA_EPSILON)
    M = _f3(snk).shape[0]
    out = np.zeros((M, 3), np.complex128)
    if scattering == 0 or los:
        out = sink_field(src, srcE, snk, snk_nrm, alpha, beta, mask=m0, **kw)
    if scattering >= 1:
        out = _proj(out, _f3(snk_nrm).astype(np.float64))
        if _f3(scat).shape[0]:
            e_p = sink_field(src, srcE, scat, scat_nrm, alpha, beta, mask=m1, **kw)
            u_p = _proj(e_p, _f3(scat_nrm).astype(np.float64))
            out = out + sink_field(scat, u_p, snk, snk_nrm, alpha, beta, mask=m2, **kw)
    return out


def path_times(full_index, pos, nrm, w, n_src, n_snk, alpha, beta, magnetic=None, impedance=None):
    """FP64 per-row part of timedomainkernal (lyceanem/electromagnetics/empropagation.py:1346-1560):
    real magnitude vector (R,3), arrival time (R,) and (source, sink) (R,2).  The path length adds,
    for i >= 1, the distance to the point of index row[i+1] even when it is 0 (the last point)."""
    idx = np.asarray(full_index, dtype=np.int64)
    pos = np.asarray(pos, np.float32).astype(np.float64)
    nrm = np.asarray(nrm, np.float32).astype(np.float64)
    w = np.asarray(w).astype(np.complex128)
    npt = pos.shape[0]
    pt = np.where(idx > 0, idx - 1, npt - 1)
    R, K = idx.shape
    a0, a1 = pt[:, 0], pt[:, 1]
    f = w[a0].real.copy()
    delay = w[a0, 0].imag.copy()
    if magnetic is not None and np.any(np.asarray(magnetic)[a0]):
        sel = np.asarray(magnetic, bool)[a0]
        d = pos[a1] - pos[a0]
        d /= np.linalg.norm(d, axis=-1, keepdims=True)
        f[sel] = np.cross(w[a0].real[sel], d[sel]) / np.asarray(impedance, np.float64)[a0][sel][:, None]
    mag = np.ones(R)
    length = np.zeros(R)
    for i in range(K - 1):
        ai, bi = pt[:, i], pt[:, i + 1]
        if i > 0:
            f = _proj(f, nrm[ai])
        length += np.linalg.norm(pos[bi] - pos[ai], axis=-1)
        has = idx[:, i + 1] != 0
        if np.any(has):
            L, dn = _seg_loss(pos[ai[has]], pos[bi[has]], nrm[bi[has]], alpha, beta)
            f[has] = _proj(f[has], dn) * w[bi[has]].real
            delay[has] += w[bi[has], 0].imag
            mag[has] *= np.abs(L)
    last = np.zeros(R, np.int64)
    for i in range(K):
        last = np.where(idx[:, i] != 0, idx[:, i], last)
    pair = np.stack([idx[:, 0] - 1, last - n_src - 1], 1)
    return f * mag[:, None], length / 299792458.0 + delay, pair


def time_map(amp, arrival, pair, n_src, n_snk, excitation, sampling_freq, num_samples, map_bytes_limit=1e9):
    """Each row's excitation times its magnitudes, placed at floor((arrival - wake) / (1 / fs))
    and cut at num_samples (the accumulation of timedomainkernal); returns (map, reported wake).
    Wake times follow TimeDomainv3 (lyceanem/electromagnetics/empropagation.py:2955-3170), taken
    before any row is placed: one wake, min(1 s, arrivals), when the float64 map fits map_bytes_limit;
    else source chunks (np.linspace bounds) whose wake array starts at ones, chunk n updating
    element 0 of a copy of it (chunk 0 from 1 s, later chunks from chunk 0's result) and storing it
    as its own; chunks whose wakes differ by a sample or more are shifted by round((wake_n - min) /
    step) samples (the alignment the reference intends; its slice for the minimum chunk is empty and
    raises); the reported wake is chunk 0's."""
    S = int(num_samples)
    step = 1.0 / sampling_freq
    exc = np.asarray(excitation, np.float64).ravel()
    out = np.zeros((n_src, n_snk, S, 3))
    arrival = np.asarray(arrival, np.float64)
    src_row = np.asarray(pair)[:, 0]
    nbytes = float(n_src) * n_snk * S * 3 * 8
    if np.ceil(nbytes / map_bytes_limit) > 1:
        bounds = np.linspace(0, n_src, int(np.ceil(nbytes / map_bytes_limit)) + 1).astype(np.int32)
        wake_times = np.ones(len(bounds) - 1)
        t0 = np.zeros(len(arrival), np.int64)
        for n in range(len(bounds) - 1):
            rows = (src_row >= bounds[n]) & (src_row < bounds[n + 1])
            d = wake_times.copy()
            if rows.any():
                d[0] = min(d[0], float(arrival[rows].min()))
            t0[rows] = np.floor_divide(arrival[rows] - d[0], step).astype(np.int64)
            wake_times[n] = d[0]
        if np.max((wake_times - np.min(wake_times)) / step) >= 1.0:
            adj = np.round((wake_times - np.min(wake_times)) / step).astype(np.int64)
            for n in range(len(bounds) - 1):
                t0[(src_row >= bounds[n]) & (src_row < bounds[n + 1])] += adj[n]
        wake = float(wake_times[0])
    else:
        wake = min(1.0, float(np.min(arrival)))
        t0 = np.floor_divide(arrival - wake, step).astype(np.int64)
    for r in range(len(t0)):
        k = min(exc.size, S - t0[r])
        if k > 0:
            out[pair[r, 0], pair[r, 1], t0[r]:t0[r] + k] += exc[:k, None] * amp[r][None]
    return out, wake


def edge_pairs(src, snk, pairs, tris12, cull=True, eps=EPSILON, rel=1e-5):
    """For each (n, m) of `pairs` (int (K,2)): True when the segment src[n] -> snk[m] is an epsilon-edge
    case, i.e. some triangle's Moller-Trumbore test, evaluated in FP64, lies within `rel` of one of the
    decision thresholds of hit() (lyceanem/src/raycasting.cuh:19-68: determinant against eps, U in
    [0, 1], V >= 0, U + V <= 1, t inside (2 eps, len - 2 eps)) while every other threshold is met to within
    the same margin, so that FP32 rounding could decide the pair either way.  Slacks are relative: the
    determinant's to max(|A|, eps), U, V and U + V as they are, t's to the segment length."""
    t = np.asarray(tris12, dtype=np.float64).reshape(-1, 12)
    v0, e1, e2 = t[:, 0:3], t[:, 4:7], t[:, 8:11]
    src = np.asarray(src, dtype=np.float32).reshape(-1, 3)
    snk = np.asarray(snk, dtype=np.float32).reshape(-1, 3)
    out = np.zeros(len(pairs), dtype=bool)
    for i, (n, m) in enumerate(np.asarray(pairs, dtype=np.int64).reshape(-1, 2)):
        o = src[n].astype(np.float64)
        r = snk[m].astype(np.float64) - o
        length = np.sqrt(r @ r)
        d = r / length
        p = np.cross(d, e2)
        A = np.einsum("ij,ij->i", e1, p)
        with np.errstate(divide="ignore", invalid="ignore"):
            tv = o - v0
            U = np.einsum("ij,ij->i", tv, p) / A
            q = np.cross(tv, e1)
            V = (q @ d) / A
            T = np.einsum("ij,ij->i", e2, q) / A
            det = ((A if cull else np.abs(A)) - eps) / np.maximum(np.abs(A), eps)
            slack = np.stack([det, U, 1.0 - U, V, 1.0 - U - V, (T - 2 * eps) / length,
                              (length - 2 * eps - T) / length], 1)
        slack = np.nan_to_num(slack, nan=-np.inf)
        near = (np.abs(slack) < rel).any(1) & (slack > -rel).all(1)
        out[i] = bool(near.any())
    return out

