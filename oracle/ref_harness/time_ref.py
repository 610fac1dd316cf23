"""Times the reference's own brute-force kernels on a GPU (test infrastructure only).

Loads oracle/_ref/ref_harness.cubin (built by build_ref.py from the reference's
sources with its release flags), finds the reference's set_values and
raycast_brute_force kernels by name, and runs them on the 8x8-array direct
scene (64 sources, 2,664 sinks, 1,024 triangles) with the launch shape of
raycast_wrapper_brute_force (<<<32, 512>>>, lyceanem/src/raycasting_brute_force.cuh:152-170),
inputs already on the device.  The same scene through this repository's
brute-force pair stage is timed beside it, and the two visibility results are
compared.  Prints one JSON line.

Usage on a GPU machine:  python oracle/ref_harness/time_ref.py [reps]
"""
import ctypes
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(HERE), "_ref")
ROOT = os.path.dirname(os.path.dirname(HERE))


class _Float2(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float)]


class _Int2(ctypes.Structure):
    _fields_ = [("x", ctypes.c_int), ("y", ctypes.c_int)]


def _functions(cu, mod):
    """Name -> CUfunction of every kernel in the module."""
    n = ctypes.c_uint()
    assert cu.cuModuleGetFunctionCount(ctypes.byref(n), mod) == 0
    fns = (ctypes.c_void_p * n.value)()
    assert cu.cuModuleEnumerateFunctions(fns, n, mod) == 0
    out = {}
    for f in fns:
        name = ctypes.c_char_p()
        assert cu.cuFuncGetName(ctypes.byref(name), ctypes.c_void_p(f)) == 0
        out[name.value.decode()] = ctypes.c_void_p(f)
    return out


def _launch(cu, fn, grid, block, args, stream):
    params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
    st = cu.cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, 0, stream, params, None)
    assert st == 0, f"cuLaunchKernel {st}"


def main(reps=20):
    import torch
    sys.path.insert(0, os.path.join(ROOT, "lyceanem-python_gb300"))
    from lyceanem_gb300 import propagation as P
    from lyceanem_gb300 import scenes
    torch.zeros(1, device="cuda")
    cu = ctypes.CDLL("libcuda.so.1")
    ctx = ctypes.c_void_p()
    assert cu.cuDevicePrimaryCtxRetain(ctypes.byref(ctx), 0) == 0
    assert cu.cuCtxSetCurrent(ctx) == 0
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    mod = ctypes.c_void_p()
    image = open(os.path.join(REF, "ref_harness.cubin"), "rb").read()
    assert cu.cuModuleLoadData(ctypes.byref(mod), ctypes.c_char_p(image)) == 0
    fns = _functions(cu, mod)
    set_values = next(f for k, f in fns.items() if "set_values" in k)
    brute = next(f for k, f in fns.items() if "raycast_brute_force" in k)

    s = scenes.direct_scene(seed=0)
    N, M, T = s.src.shape[0], s.snk.shape[0], s.faces.shape[0]
    assert T % 32 == 0  # the reference kernel reads triangles in groups of 32
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    pts = np.zeros((N + M, 10), np.float32)  # PointData: complex_float3 E, float3 normal, padding (40 B)
    pts[:N, 0:6] = s.E.astype(np.complex64).view(np.float32).reshape(N, 6)
    pts[:N, 6:9] = np.tile(np.array([[0, 0, 1]], np.float32), (N, 1))
    pts[N:, 6:9] = s.snk_n
    beta = np.float32(2 * np.pi / s.wavelength)
    b = dict(src=t(s.src), snk=t(s.snk), ray=torch.zeros((N * M, 4), device="cuda"), verts=t(s.verts),
             faces=t(s.faces.astype(np.int32)), idx=torch.zeros((N * M, 2), dtype=torch.int32, device="cuda"),
             pts=t(pts), net=torch.zeros((N * M, 6), device="cuda"))
    p = lambda k: ctypes.c_void_p(b[k].data_ptr())  # noqa: E731
    flag = 0  # not_self_to_self as the reference's default call passes it (self_to_self=False)
    sv_args = [p("idx"), ctypes.c_int(N * M), _Int2(-1, -1), ctypes.c_int(M), ctypes.c_int(N)]
    bf_args = [p("src"), p("snk"), p("ray"), ctypes.c_int(N), ctypes.c_int(M), ctypes.c_int(flag), p("verts"),
               p("faces"), ctypes.c_int(T), ctypes.c_int(N * M), p("idx"), p("pts"), ctypes.c_float(float(s.wavelength)),
               p("net"), _Float2(0.0, float(beta))]

    def ref_step():
        _launch(cu, set_values, 32, 512, sv_args, stream)
        _launch(cu, brute, 32, 512, bf_args, stream)

    tris = P.pack_triangles(t(s.verts), t(s.faces))
    E = t(s.E.astype(np.complex64))
    snk, snk_n, src = t(s.snk), t(s.snk_n), t(s.src)

    sink_out = torch.empty((M, 3), dtype=torch.complex64, device="cuda")
    ws = torch.empty(P.lib.lyem_pair_stage_workspace(N, M, T, 0, 0), dtype=torch.uint8, device="cuda")

    def ours(**kw):  # outputs and scratch allocated once, as the reference's timed kernels have theirs
        return P.pair_stage(src, E, snk, snk_n, beta=float(beta), tris=tris, sink_out=sink_out, workspace=ws, **kw)

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            fn()
        e.record()
        torch.cuda.synchronize()
        return a.elapsed_time(e) / reps

    ref_ms = timed(ref_step)
    ref_vis = (b["idx"][:, 0] != -1).cpu().numpy().reshape(N, M)
    our_ms = timed(ours)
    our_net_ms = timed(lambda: ours(want_pairs=True))
    our_vis = ours(want_mask=True).mask().cpu().numpy().astype(bool)
    pairs = N * M
    print(json.dumps({"workload": f"direct scene: {N} sources, {M} sinks, {T} triangles, brute force",
                      "reference_ms": ref_ms, "reference_launch": "set_values + raycast_brute_force, <<<32, 512>>> each",
                      "ours_ms": our_ms, "ours": "lyem_pair_stage brute force (TMA-staged tiles), field summed over sources",
                      "ours_with_network_ms": our_net_ms, "speedup": ref_ms / our_ms,
                      "speedup_with_network": ref_ms / our_net_ms, "reference_paths_per_s": pairs / (ref_ms / 1e3),
                      "ours_paths_per_s": pairs / (our_ms / 1e3),
                      "visibility_mismatches": int((ref_vis != our_vis).sum()), "pairs": pairs,
                      "reference_visible": int(ref_vis.sum()), "ours_visible": int(our_vis.sum())}))
    cu.cuModuleUnload(mod)


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 20)
