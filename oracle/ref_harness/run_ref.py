"""Runs the reference's device functions (oracle/_ref/*.cubin, built by build_ref.py) on seeded
inputs and writes golden vectors (test infrastructure only).

Usage on a GPU machine:  python oracle/ref_harness/run_ref.py OUT.npz
The output holds, per case, the inputs, the reference's visibility (bit-packed)
and its FP32 field on a seeded sample of pairs, for the default build and the
--fmad=false build.  tests/golden/reference_pairs.npz is this file.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(HERE), "_ref")
ROOT = os.path.dirname(os.path.dirname(HERE))


def _cases():
    sys.path.insert(0, os.path.join(ROOT, "lyceanem-python_gb300"))
    from lyceanem_gb300 import scenes
    s = scenes.direct_scene(seed=0)
    src_n = np.tile(np.array([[0, 0, 1]], np.float32), (s.src.shape[0], 1))
    yield dict(name="direct", src=s.src, snk=s.snk, src_n=src_n, snk_n=s.snk_n, verts=s.verts, faces=s.faces,
               E=s.E.astype(np.complex64), alpha=0.0, beta=np.float32(2 * np.pi / s.wavelength), flag=0)
    rng = np.random.default_rng(2024)
    n, m, t = 40, 500, 300
    src = np.stack([rng.uniform(-0.5, 0.5, n), rng.uniform(-0.5, 0.5, n), np.full(n, -2.0)], 1).astype(np.float32)
    d = rng.normal(size=(m, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    c = rng.uniform(-1.2, 1.2, size=(t, 3))
    v = (c[:, None, :] + rng.uniform(-0.4, 0.4, size=(t, 3, 3))).reshape(-1, 3).astype(np.float32)
    E = (rng.normal(size=(n, 3)) + 1j * rng.normal(size=(n, 3))).astype(np.complex64)
    yield dict(name="random", src=src, snk=(4.0 * d).astype(np.float32),
               src_n=np.tile(np.array([[0, 0, 1]], np.float32), (n, 1)), snk_n=(-d).astype(np.float32), verts=v,
               faces=np.arange(3 * t, dtype=np.int32).reshape(t, 3), E=E, alpha=0.05,
               beta=np.float32(2 * np.pi / 0.05), flag=1)


class _Float2(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float)]


def _run(lib, fn, case, stream):
    import torch
    N, M = case["src"].shape[0], case["snk"].shape[0]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    pts = np.zeros((N + M, 10), np.float32)  # PointData: complex_float3 E (24 B), float3 normal, pad -> 40 B
    pts[:N, 0:6] = case["E"].view(np.float32).reshape(N, 6)
    pts[:N, 6:9] = case["src_n"]
    pts[N:, 6:9] = case["snk_n"]
    bufs = dict(src=t(case["src"]), snk=t(case["snk"]), ray=torch.zeros((N * M, 4), device="cuda"),
                verts=t(case["verts"]), faces=t(case["faces"].astype(np.int32)), pts=t(pts),
                vis=torch.zeros(N * M, dtype=torch.uint8, device="cuda"),
                field=torch.zeros((N * M, 6), device="cuda"))
    P = lambda k: ctypes.c_void_p(bufs[k].data_ptr())  # noqa: E731
    args = [P("src"), P("snk"), P("ray"), ctypes.c_int(N), ctypes.c_int(M), ctypes.c_int(case["flag"]), P("verts"),
            P("faces"), ctypes.c_int(case["faces"].shape[0]), P("pts"), ctypes.c_float(1.0),
            _Float2(float(case["alpha"]), float(case["beta"])), P("vis"), P("field")]
    params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
    blocks = min(4096, (N * M + 255) // 256)
    st = lib.cuLaunchKernel(fn, blocks, 1, 1, 256, 1, 1, 0, stream, params, None)
    assert st == 0, f"cuLaunchKernel {st}"
    torch.cuda.synchronize()
    return bufs["vis"].cpu().numpy().reshape(N, M), bufs["field"].cpu().numpy().reshape(N, M, 6)


def main(out_path):
    import torch
    torch.cuda.init()
    torch.zeros(1, device="cuda")
    lib = ctypes.CDLL("libcuda.so.1")
    ctx = ctypes.c_void_p()
    assert lib.cuDevicePrimaryCtxRetain(ctypes.byref(ctx), 0) == 0
    assert lib.cuCtxSetCurrent(ctx) == 0
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = {}
    for variant, fname in (("fma", "ref_harness.cubin"), ("nofma", "ref_harness_nofma.cubin")):
        image = open(os.path.join(REF, fname), "rb").read()
        mod = ctypes.c_void_p()
        assert lib.cuModuleLoadData(ctypes.byref(mod), ctypes.c_char_p(image)) == 0
        fn = ctypes.c_void_p()
        assert lib.cuModuleGetFunction(ctypes.byref(fn), mod, b"ref_pairs") == 0
        for case in _cases():
            vis, field = _run(lib, fn, case, stream)
            k = case["name"]
            if variant == "fma":
                for key in ("src", "snk", "src_n", "snk_n", "verts", "faces", "E"):
                    out[f"{k}_{key}"] = case[key]
                out[f"{k}_alpha"] = np.float64(case["alpha"])
                out[f"{k}_beta"] = np.float32(case["beta"])
                out[f"{k}_flag"] = np.int32(case["flag"])
                rng = np.random.default_rng(99)
                out[f"{k}_sample"] = rng.choice(vis.size, size=min(4096, vis.size), replace=False)
            sample = out[f"{k}_sample"]
            out[f"{k}_{variant}_vis"] = np.packbits(vis.astype(bool).ravel())
            out[f"{k}_{variant}_field"] = field.reshape(-1, 6)[sample]
        lib.cuModuleUnload(mod)
    np.savez_compressed(out_path, **out)
    print("wrote", out_path, {k: v.shape for k, v in out.items() if hasattr(v, "shape")})


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "reference_pairs.npz")
