#!/usr/bin/env python
"""Benchmark of the raycasting + frequency-domain propagation path on one GB300.

Workload (default): the direct + one-bounce scene at 28 GHz -- 32x32
half-wave array, 20x20 m ground plane (80,000 triangles) + 40,000 clutter
triangles, 50,000 scatter points on triangle centroids, 65,341 far-field sinks
(1 deg grid at 100 m), uniform grid with 0.5 m cells.  One step = triangle
packing + grid build + direct stage + source->scatter stage + scatter->sink
stage (visibility, field, sink sum) with the inputs resident in HBM.

Metric: paths evaluated per second, paths = N*M direct pairs + N*P*M
source-scatter-sink triples (every path gets mask + field); the visible-path
count and rate are reported beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the same path (the reference has
no CPU implementation; its only engines run on the GPU) on the host cores, on a
bounded sample of the same workload, extrapolated stage by stage.

Side legs of the default run, each reported in its own object of the JSON line
(skipped with --no-<leg>): full-geometry parity against the oracle, the
direct-path workload (brute force) with its roofline and parity, the
mixed-precision beam sweep, the adjoint, the batched many-scene launch, the
model layer's field with and without the opt-in skip of unlit scattering
points (--no-unlit), the end-to-end call through the reference-shaped API, and
the CPU baseline.  The headline step traces every scatter->sink ray.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "lyceanem-python_gb300"))
sys.path.insert(0, ROOT)

METRIC = "visible paths/s (mask+field) on 1 GB300; mixed-prec vs FP32 sweep at ≤1e-4 rel err"
OPS_PER_TEST = 30  # FP32-pipe operations of one Moller-Trumbore test (lyceanem/src/raycasting.cuh:23-59)
L2_FLUSH_BYTES = 256 << 20
# sample strides of the CPU legs and of the parity leg: every k-th sink and scatter point, all sources
# (the direct workload is small enough to run whole)
CPU_STRIDES = (16, 11)
CPU_STRIDES_DIRECT = (1, 2)
PARITY_STRIDE = 16
# DRAM traffic (read + write bytes per launch) of the dominant kernels, from one-pass ncu captures of
# committed builds; each entry names its capture command and the commit it was measured on
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "dram_traffic.json")


def measured_peak(key):
    """A peak of MEASURED_PEAKS.json (TFLOP/s or GB/s) and where it came from; the profiling recipe's
    fallback when the file is absent."""
    fallback = {"bf16_tflops": 1900.0, "hbm_gbs": 6800.0}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)[key]), f"measured ({key} of MEASURED_PEAKS.json)"
    except (OSError, ValueError, KeyError):
        return fallback[key], "fallback (no measured peak file)"


def traffic_record(workload):
    """The recorded DRAM traffic of the dominant kernel of `workload` (dict with bytes, kernel, command,
    commit) or None."""
    try:
        with open(TRAFFIC_FILE) as f:
            return json.load(f).get(workload)
    except (OSError, ValueError):
        return None


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["bounce", "direct", "bounce_small"], default="bounce",
                    help="bounce_small: the bounce scene with 2,000 scatter points and a 4 deg sink grid "
                         "(profiling case)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-sweep", action="store_true", help="skip the mixed-precision beam-sweep measurement")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint (differentiation) measurement")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched 64-scene x 64-frequency measurement")
    ap.add_argument("--batched-scenes", type=int, default=64,
                    help="scenes of the batched measurement (the first S of the 64-scene recipe; profiling cases)")
    ap.add_argument("--batched-config", default="",
                    help="fg,chunk,blocks_per_sm for the batched launch instead of the autotuner (profiling cases)")
    ap.add_argument("--batched-cell-scale", type=float, default=0.0,
                    help="grid cell scale k of the batched scenes instead of the autotuner (profiling cases)")
    ap.add_argument("--no-parity", action="store_true", help="skip the full-geometry parity check against the oracle")
    ap.add_argument("--no-unlit", action="store_true",
                    help="skip the side leg timing the one-bounce field traced only from lit scattering points")
    ap.add_argument("--no-direct", action="store_true",
                    help="skip the direct-path (8x8 array, brute force) leg of the bounce workload's run")
    ap.add_argument("--sweep-case", choices=["full", "small"], default="full",
                    help="small: the beam-sweep scene on a 4 deg sink grid (4,186 sinks; profiling case)")
    ap.add_argument("--src-chunk", type=int, default=0,
                    help="sources per thread block of the pair stages (0 = automatic)")
    ap.add_argument("--traversal", type=int, default=0,
                    help="grid schedule of the pair stages (0 = automatic; see lyem_pair_stage in include/lyem.h)")
    ap.add_argument("--array-traversal", type=int, default=-1,
                    help="grid schedule of the two stages that start at the array elements (-1 = the model layer's "
                         "choice, propagation.source_schedule, unless --traversal is given)")
    return ap.parse_args()


def array_schedule(args, src, grid):
    """Grid schedule of the stages that start at the array elements: --array-traversal, else --traversal when
    given, else the model layer's choice (the transposed schedule for a compact source set)."""
    from lyceanem_gb300 import propagation as P
    if args.array_traversal >= 0:
        return args.array_traversal
    if args.traversal != 0:
        return args.traversal
    return P.source_schedule(src, grid)


def workload_scene(name):
    from lyceanem_gb300 import scenes
    if name == "direct":
        return scenes.direct_scene()
    if name == "bounce_small":
        return scenes.bounce_scene(n_scatter=2000, el_n=46, az_n=91)
    return scenes.bounce_scene()


def describe(s, name):
    N, M, P, T = s.src.shape[0], s.snk.shape[0], s.scat.shape[0], s.faces.shape[0]
    paths = N * M + N * P * M
    if name == "direct":
        wl = "direct path, 10 GHz, 8x8 array, 2,664 sinks at 10 m, 1,024 obstruction triangles, brute force"
    elif name == "bounce_small":
        wl = ("profiling case: bounce scene with 2,000 scatter points and 4,186 sinks (4 deg grid at 100 m), "
              "0.5 m grid")
    else:
        wl = ("direct + one bounce, 28 GHz, 32x32 array, 80,000 ground + 40,000 clutter triangles, "
              "50,000 scatter points, 65,341 sinks at 100 m, 0.5 m grid")
    cfg = {"workload": wl, "n_sources": N, "n_scatter": P, "n_sinks": M, "n_triangles": T, "paths_per_step": paths,
           "grid_cell_m": s.cell, "l2": "flushed by a 256 MiB device write before every timed step"}
    if P:
        cfg["path_count"] = ("N*M direct pairs + N*P*M source-scatter-sink triples, the triples counted "
                             "algebraically: the fused composition traces N*M + N*P + P*M rays and never forms a "
                             "triple (rays_per_s and visible_paths_per_s are reported beside the value)")
    return cfg, paths


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")
        self.gpu_index = gpu_index

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu_index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        mhz = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(mhz) if mhz else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------ ours
def max_over_ranks(value, device):
    """The largest of `value` over the ranks of the process group (the slowest replica sets the
    whole job's time); `value` itself without a group or with one rank."""
    import torch
    dist = torch.distributed
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_step, world, steps, total_ms):
    """Units per second of the whole job: every rank processes units_per_step each step (weak scaling)."""
    return units_per_step * world * steps / (total_ms / 1e3)


def run_ours(args, rank, world):
    import numpy as np
    import torch

    from lyceanem_gb300 import propagation as P

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    s = workload_scene(args.workload)
    cfg, paths = describe(s, args.workload)
    beta = 2 * np.pi / s.wavelength
    t = lambda a, dt=None: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    src, E, snk, snk_n = t(s.src), t(s.E), t(s.snk), t(s.snk_n)
    scat, scat_n = t(s.scat), t(s.scat_n)
    verts, faces = t(s.verts), t(s.faces)
    N, M, Pn = src.shape[0], snk.shape[0], scat.shape[0]
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    cnt_s2 = torch.zeros(2, dtype=torch.int64, device=dev)
    cnt_all = torch.zeros(2, dtype=torch.int64, device=dev)
    vis_scat_in = torch.zeros(Pn, dtype=torch.int32, device=dev)
    vis_scat_out = torch.zeros(Pn, dtype=torch.int32, device=dev)
    vis_direct = torch.zeros(M, dtype=torch.int32, device=dev)
    ev = {}

    def step(mark=False, count=False):
        # count: the test counters (one untimed step after the timed ones; the timed steps run the kernels
        # without per-test counting, as a caller passing no counters does); otherwise the visible-pair counts
        c_all, c_s2 = (cnt_all, cnt_s2) if count else (None, None)
        v_dir, v_in, v_out = (None, None, None) if count else (vis_direct, vis_scat_in, vis_scat_out)
        tris = P.pack_triangles(verts, faces)
        if args.workload == "direct":
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            out = P.pair_stage(src, E, snk, snk_n, beta=beta, tris=tris, counters=c_all, snk_visible=v_dir)
            b.record()
            if mark:
                ev.setdefault("s2_list", []).append((a, b))
            return out.sink
        grid = P.UniformGrid(tris, cell=s.cell)
        o_scat = P.spatial_order(scat)  # scatter points are traced in Morton order
        o_snk = P.direction_order(snk, grid.centre)  # sinks in direction order from the scene
        ta = array_schedule(args, s.src, grid)
        out = P.pair_stage(src, E, snk, snk_n, beta=beta, grid=grid, counters=c_all, snk_visible=v_dir,
                           snk_order=o_snk, traversal=ta, src_chunk=args.src_chunk).sink
        e_p = P.pair_stage(src, E, scat, scat_n, beta=beta, grid=grid, counters=c_all,
                           snk_visible=v_in, snk_order=o_scat, traversal=ta,
                           src_chunk=args.src_chunk).sink
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        P.pair_stage(scat, e_p, snk, snk_n, beta=beta, grid=grid, src_W=e_p, sink_out=out, accumulate=True,
                     counters=c_s2, src_visible=v_out, src_order=o_scat, snk_order=o_snk,
                     traversal=args.traversal, src_chunk=args.src_chunk)
        b.record()
        if mark:
            ev.setdefault("s2_list", []).append((a, b))
        return out

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # visible-pair counts describe one step: zero them after warm-up, divide by K afterwards; the test
    # counters are filled by one counting step after the timed loop
    for c in (cnt_s2, cnt_all, vis_scat_in, vis_scat_out, vis_direct):
        c.zero_()
    fma_rate = P.fp32_fma_rate()
    clocks = ClockSampler(dev.index)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    launches0 = P.kernel_launches()
    step_ms = []
    for _ in range(args.steps):
        flush.fill_(1)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        step(mark=True)
        b.record()
        step_ms.append((a, b))
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    launches = P.kernel_launches() - launches0
    clk = clocks.stop()
    step(count=True)  # untimed: ray-triangle tests of one step (deterministic)
    torch.cuda.synchronize()
    total_ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in step_ms), dev)
    K = args.steps
    ms_per_step = total_ms / K
    value = whole_job_rate(paths, world, K, total_ms)
    st, flags = P.device_errors()
    if st != 0 or flags != 0:
        raise RuntimeError(f"device error word {flags:#x}")
    vis_direct_total = int(vis_direct.sum().item()) // K
    if args.workload != "direct":
        vin = vis_scat_in.double() / K
        vout = vis_scat_out.double() / K
        visible_paths = vis_direct_total + float((vin * vout).sum().item())
    else:
        visible_paths = vis_direct_total
    rays = N * M + (N * Pn + Pn * M if args.workload != "direct" else 0)
    res = {"metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": K, "warmup": args.warmup,
           "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 (visibility bit-specified FP32; field FP32 with FP64 phase)", "data": "synthetic",
           "config": dict(cfg, parallelism="replicas" if world > 1 else "single GPU"),
           "visible_paths_per_step": visible_paths, "visible_paths_per_s": visible_paths * world * K / (total_ms / 1e3),
           "rays_per_s": rays * world * K / (total_ms / 1e3), "gpu_launches": launches}
    # roofline of the dominant kernel (scatter->sink grid stage; direct stage for the direct workload)
    T = int(faces.shape[0])
    if args.workload != "direct":
        s2_ms = sum(a.elapsed_time(b) for a, b in ev["s2_list"]) / K
        tests = int(cnt_s2[1].item())
        brute_tests = float(Pn) * M * T
        kernel = "grid_stage_kernel (scatter->sink stage incl. its partial-sum reduction)"
    else:
        s2_ms = sum(a.elapsed_time(b) for a, b in ev["s2_list"]) / K
        tests = int(cnt_all[1].item())
        brute_tests = float(N) * M * T
        kernel = "brute_stage_kernel (the pair stage: brute-force launch and its partial-sum reduction)"
    achieved = tests * OPS_PER_TEST / (s2_ms / 1e3) / 1e12
    peak = fma_rate / 1e12
    tr = traffic_record(args.workload)
    res["roofline"] = {"bound": "fp32", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                       "frac": achieved / peak,
                       "traffic": tr["bytes"] if tr else None,
                       "traffic_source": ({k: tr[k] for k in ("kernel", "command", "commit") if k in tr}
                                          if tr else "no capture recorded"),
                       "peak_source": "measured FP32 FMA lane-op rate (lyem_fp32_fma_probe, same run; FMA = 1 op)",
                       "tests_per_launch": tests, "ops_per_test": OPS_PER_TEST, "launch_ms": s2_ms,
                       "share_of_step": s2_ms / ms_per_step,
                       # the same launch counted in brute-force tests (every ray against every triangle)
                       "effective_tests_per_s": brute_tests / (s2_ms / 1e3),
                       "effective_frac": brute_tests * OPS_PER_TEST / (s2_ms / 1e3) / 1e12 / peak}
    if clk:
        res["clocks"] = clk
    if rank == 0 and world == 1 and not args.no_parity:
        res["parity"] = run_parity(args, s)
    if rank == 0 and world == 1 and not args.no_sweep:
        res["sweep"] = run_sweep(args)
    if rank == 0 and world == 1 and not args.no_adjoint:
        res["adjoint"] = run_adjoint(args)
    if rank == 0 and world == 1 and not args.no_batched:
        res["batched"] = run_batched(args)
    if rank == 0 and world == 1 and not args.no_direct and args.workload == "bounce":
        res["direct"] = run_direct(args, rank, world)
    if rank == 0 and world == 1 and not args.no_unlit and args.workload == "bounce":
        res["skip_unlit"] = run_unlit(args, s)
    if rank == 0 and world == 1 and not args.no_e2e:
        res["e2e"] = run_e2e(args, s, paths)
    if rank == 0 and world == 1 and not args.no_cpu:
        res["cpu_baseline"] = cpu_baseline(args, s, paths)
    return res


def run_direct(args, rank, world, steps=50, warmup=5):
    """The direct-path workload (8x8 array at 10 GHz, 2,664 sinks at 10 m, 1,024 obstruction triangles, brute
    force) timed the same way as the main workload (L2 flushed before every step, CUDA events), with its
    roofline and its full-size parity against the oracle; a reported side leg of the default run."""
    a = argparse.Namespace(**vars(args))
    a.workload, a.steps, a.warmup = "direct", steps, warmup
    a.no_e2e = a.no_cpu = a.no_sweep = a.no_adjoint = a.no_batched = a.no_direct = True
    a.no_parity = False
    sub = run_ours(a, rank, world)
    r = sub["roofline"]
    return {"workload": sub["config"]["workload"], "steps": steps, "warmup": warmup,
            "ms_per_step": sub["ms_per_step"], "value": sub["value"], "unit": sub["unit"],
            "roofline": {k: r[k] for k in ("bound", "kernel", "achieved", "peak", "unit", "frac", "tests_per_launch",
                                            "ops_per_test", "traffic")},
            "parity": {k: sub["parity"][k] for k in ("sample", "pairs", "mask_mismatches", "edge_pairs",
                                                     "field_rel_err", "ok")}}


def run_unlit(args, s, reps=3):
    """Side leg: the model layer's fused field (models.frequency_domain.sink_field, device-resident scene and
    grid) with and without skip_unlit, which traces the one bounce only from the scattering points that some
    source sees.  Each call is timed with CUDA events after an L2 flush; the fields are compared."""
    import numpy as np
    import torch

    from lyceanem_gb300 import propagation as P
    from lyceanem_gb300.models import acceleration_structures as AS
    from lyceanem_gb300.models.frequency_domain import sink_field
    beta = 2 * np.pi / s.wavelength
    dev = AS._DeviceScene(s.verts, s.faces, grid_cell=s.cell)
    st = type("S", (), {"device": dev})()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    out, ms, tests = {}, {}, {}
    for skip in (False, True):
        cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
        out[skip] = sink_field(st, s.src, s.E, s.snk, s.snk_n, 0.0, beta, s.scat, s.scat_n, scattering=1,
                               counters=cnt, skip_unlit=skip)
        tests[skip] = int(cnt[1].item())
        times = []
        for _ in range(reps):
            flush.fill_(1)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            sink_field(st, s.src, s.E, s.snk, s.snk_n, 0.0, beta, s.scat, s.scat_n, scattering=1, skip_unlit=skip)
            b.record()
            torch.cuda.synchronize()
            times.append(a.elapsed_time(b))
        ms[skip] = min(times)
    seen = torch.zeros(s.scat.shape[0], dtype=torch.int32, device="cuda")
    P.pair_stage(s.src, s.E, s.scat, s.scat_n, beta=beta, grid=dev.grid, snk_visible=seen)
    st_, flags = P.device_errors()
    if st_ != 0 or flags != 0:
        raise RuntimeError(f"device error word {flags:#x}")
    d = (out[True] - out[False]).abs().max().item() / out[False].abs().max().item()
    return {"api": "models.frequency_domain.sink_field(scattering=1), scene and grid resident, inputs uploaded "
                   "per call; best of %d calls, L2 flushed before each" % reps,
            "ms_full": ms[False], "ms_skip_unlit": ms[True], "speedup": ms[False] / ms[True],
            "lit_scatter_points": int((seen > 0).sum().item()), "scatter_points": int(s.scat.shape[0]),
            "tests_full": tests[False], "tests_skip_unlit": tests[True], "field_rel_diff": d}


def run_e2e(args, s, paths):
    """Same metric through the reference-shaped host API: numpy in, numpy out, copies inside the timed region."""
    import numpy as np
    import torch

    from lyceanem_gb300.geometry import Mesh
    from lyceanem_gb300.models import acceleration_structures as AS
    from lyceanem_gb300.models import frequency_domain as FD
    beta = 2 * np.pi / s.wavelength
    solid = Mesh(s.verts, [("triangle", s.faces)])
    ap = Mesh(s.src, point_data={"Normals": s.src_n, "Area": np.ones(s.src.shape[0], np.float32)})
    sk = Mesh(s.snk, point_data={"Normals": s.snk_n})
    sc = Mesh(s.scat, point_data={"Normals": s.scat_n}) if s.scat.shape[0] else None
    scattering = 0 if args.workload == "direct" else 1
    axis = np.array([1.0, 0.0, 0.0])

    def call():
        AS.clear_cache()  # every call uploads the mesh and builds its grid, as a first call on a scene does
        return FD.calculate_scattering(ap, sk, solid, axis, scatter_points=sc, wavelength=s.wavelength,
                                       scattering=scattering, beta=beta, cuda=True, grid_cell=s.cell)

    call()
    torch.cuda.synchronize()
    K = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(K):
        Ex, Ey, Ez = call()
    dt = (time.perf_counter() - t0) / K
    V, T = s.verts.shape[0], s.faces.shape[0]
    h2d = (3 * (V * 12 + T * 12) + s.src.nbytes + s.src.shape[0] * 24 + s.snk.nbytes + s.snk_n.nbytes
           + s.scat.nbytes + s.scat_n.nbytes)
    # the reference-shaped tile structure built in the call reads its y-z bins back to the host
    tile = next(iter(AS._CACHE.values()))
    d2h = Ex.nbytes + Ey.nbytes + Ez.nbytes + tile.bin_counts.nbytes + tile.binned_triangles.nbytes
    return {"value": paths / dt, "unit": "paths/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "seconds_per_step": dt,
            "api": "lyceanem_gb300.models.frequency_domain.calculate_scattering (host numpy in/out; the scene "
                   "cache is cleared before every call, so each call uploads the mesh and builds the grid)"}


# ------------------------------------------------------------------ sweep
def run_sweep(args, n_check=256, reps=5):
    """Mixed-precision beam sweep: 64x64 array at 28 GHz, ground + 20,000 clutter triangles, 65,341 sinks,
    K = 2,048 steering vectors.  Times the three component GEMMs per mode on the formed network and measures
    each mode's error against an FP64 product on a seeded sample of sinks (oracle network, all beams)."""
    import numpy as np
    import torch

    from lyceanem_gb300 import beam_sweep as BS
    from lyceanem_gb300 import propagation as P
    from lyceanem_gb300 import scenes
    from oracle import oracle as O
    s = scenes.sweep_scene(el_n=46, az_n=91) if args.sweep_case == "small" else scenes.sweep_scene()
    beta = 2 * np.pi / s.wavelength
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    tris = P.pack_triangles(t(s.verts), t(s.faces))
    grid = P.UniformGrid(tris, cell=s.cell)
    N, M, K = s.src.shape[0], s.snk.shape[0], s.weights.shape[0]
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    G = BS.form_network(t(s.src), s.pol, t(s.snk), t(s.snk_n), beta=beta, grid=grid)
    b.record()
    torch.cuda.synchronize()
    form_ms = a.elapsed_time(b)
    W = t(s.weights)
    rng = np.random.default_rng(7)
    pick = np.sort(rng.choice(M, size=n_check, replace=False))
    flops = 8.0 * M * N * K * 3
    res = {"n_elements": N, "n_sinks": M, "n_beams": K, "network_form_ms": form_ms,
           "algorithmic_flops": flops}
    # tensor work the kernel issues: 3 components x 3 real products x 3 split products of 2 flops per
    # MAC over whole tiles (128 sinks x 256 beams x 64 sources)
    rnd = lambda a, b: -(-a // b) * b  # noqa: E731
    issued = 3 * 9 * 2.0 * rnd(M, 128) * rnd(K, 256) * rnd(N, 64)
    peak, peak_src = measured_peak("bf16_tflops")
    res["tensor_issued_flops"] = issued
    outs = {}
    for name, mode, k_tile, mc in (("fp32", "fp32", 32, False), ("bf16x3g", "bf16x3g", 32, False),
                                   ("fp16x3g", "fp16x3g", 32, False), ("bf16x3g_k64", "bf16x3g", 64, False),
                                   ("bf16x3g_multicast", "bf16x3g", 32, True)):
        BS.set_k_tile(k_tile)
        BS.set_multicast(mc)
        sw = BS.BeamSweep(G, mode)
        torch.cuda.synchronize()
        px, py = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        px.record()
        sw.refresh(G)  # the network's operand again: transpose, split, scales (once per network)
        py.record()
        out = sw.run(W)
        torch.cuda.synchronize()
        ev = []
        for _ in range(reps):
            x, y = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            x.record()
            sw.run(W, out=out)
            y.record()
            ev.append((x, y))
        torch.cuda.synchronize()
        ms = min(x.elapsed_time(y) for x, y in ev)
        outs[name] = sw.fields(out)[torch.from_numpy(pick).cuda()].cpu().numpy()
        res[name] = {"ms": ms, "tflops_algorithmic": flops / (ms * 1e-3) / 1e12,
                     "prepare_network_ms": px.elapsed_time(py)}
        if mode != "fp32":
            res[name]["k_tile"] = k_tile
            res[name]["multicast_clusters"] = mc
            res[name]["tensor_tflops_issued"] = issued / (ms * 1e-3) / 1e12
            res[name]["tensor_frac"] = issued / (ms * 1e-3) / 1e12 / peak
        del sw, out
        torch.cuda.empty_cache()
    BS.set_k_tile(32)
    BS.set_multicast(False)
    st, flags = P.device_errors()
    res["device_errors"] = [int(st), int(flags)]
    res["roofline"] = {"bound": "tensor", "kernel": "sweep_tc_kernel (bf16x3g, k-tile 32, single-CTA)",
                       "achieved": res["bf16x3g"]["tensor_tflops_issued"], "peak": peak, "unit": "TFLOP/s",
                       "frac": res["bf16x3g"]["tensor_frac"], "peak_source": peak_src,
                       "note": "achieved = issued tensor flops (whole tiles, 9 real products per complex product) / "
                               "time of one run (weight split + the three component products)"}
    del G
    # FP64 reference on the sampled sinks: oracle visibility + FP64 network, FP64 product
    og = O.Grid(O.pack_triangles(s.verts, s.faces), s.cell)
    snk, snk_n = s.snk[pick], s.snk_n[pick]
    mask = og.mask(s.src, snk, self_to_self=True)  # the network tests every pair (sink indices are sampled)
    G64 = O.pair_field(s.src, np.tile(s.pol, (N, 1)), snk, snk_n, mask, 0.0, beta)
    E64 = np.einsum("nmc,kn->mkc", G64, s.weights.astype(np.complex128), optimize=True)
    for mode, E in outs.items():
        res[mode]["rel_err_fp64"] = float(np.linalg.norm(E - E64) / np.linalg.norm(E64))
    res["speedup_bf16x3g_vs_fp32"] = res["fp32"]["ms"] / res["bf16x3g"]["ms"]
    res["speedup_fp16x3g_vs_fp32"] = res["fp32"]["ms"] / res["fp16x3g"]["ms"]
    res["error_sample"] = f"{n_check} seeded sinks x {K} beams x 3 components, relative Frobenius norm"
    return res


# ------------------------------------------------------------------ batched
BATCH_TUNE_CANDIDATES = [(2, 64, 8), (2, 64, 6), (1, 64, 8), (4, 64, 8)]
# grid cell edge per scene = k * (box volume / triangles)^(1/3); the autotuner picks k
BATCH_TUNE_CELL_SCALES = [1.0, 1.25, 1.5]


def run_batched(args, reps=2):
    """Batched uneven workload: 64 scenes (square half-wave arrays of 16-16,384 elements and 1e3-5e5
    triangles, both log-uniform, ground + clutter recipe scaled to the count, scatter points on 10% of the
    triangles up to 10,000), 10,000 Fibonacci sinks at 50 m, 64 frequencies 24-30 GHz, direct + one bounce.
    One persistent launch per step, replayed from a captured CUDA graph; configuration and grid cell
    scale picked by the autotuner on a cost-stratified quarter of the scenes.  Checked against the per-scene pair-stage path
    (three scenes, first/middle/last frequency) and against the FP64 oracle on the smallest scene."""
    import numpy as np
    import torch

    from lyceanem_gb300 import batched as B
    from lyceanem_gb300 import propagation as P
    from lyceanem_gb300 import scenes as SC
    from oracle import oracle as O
    scenes, snk, snk_n, freqs = SC.batched_scenes(n_scenes=args.batched_scenes)
    t0 = time.time()
    fixed = args.batched_config and args.batched_cell_scale > 0
    bs = B.BatchedScattering(scenes, snk, snk_n, freqs, cell_scale=args.batched_cell_scale if fixed else 1.0)
    torch.cuda.synchronize()
    setup_s = time.time() - t0
    t0 = time.time()
    if fixed:
        bs.configure(tuple(int(v) for v in args.batched_config.split(",")))
        tune = {}
    else:
        proxy = B.BatchedScattering([scenes[i] for i in B.stratified_subset(scenes, snk.shape[0])], snk, snk_n,
                                    freqs, cell_scale=1.0)
        cands = [tuple(int(v) for v in args.batched_config.split(","))] if args.batched_config else \
            BATCH_TUNE_CANDIDATES
        scales = [args.batched_cell_scale] if args.batched_cell_scale > 0 else BATCH_TUNE_CELL_SCALES
        tune = bs.autotune(candidates=cands, proxy=proxy, use_cache=False, cell_scales=scales)
        del proxy
        torch.cuda.empty_cache()
    tune_s = time.time() - t0
    bs.capture()
    bs.run()
    torch.cuda.synchronize()
    ev = []
    for _ in range(reps):
        x, y = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        x.record()
        bs.run()
        y.record()
        ev.append((x, y))
    torch.cuda.synchronize()
    times = [x.elapsed_time(y) for x, y in ev]
    st, flags = P.device_errors()
    cnt = bs.counters.cpu().numpy()
    ms = statistics.mean(times)
    paths = bs.paths()
    res = {"workload": "64 uneven scenes x 64 frequencies (24-30 GHz), direct + one bounce, 10,000 sinks at 50 m",
           "n_scenes": bs.n_scenes, "n_freq": bs.n_freq, "n_sinks": bs.n_snk,
           "elements_total": int(sum(d.src.shape[0] for d in bs.data)),
           "triangles_total": int(sum(d.n_tris for d in bs.data)),
           "scatter_total": int(sum(d.scat.shape[0] for d in bs.data)),
           "config": {"freq_group": bs.config[0], "src_chunk": bs.config[1], "blocks_per_sm": bs.config[2],
                      "blocks": bs.blocks, "cell_scale": bs.cell_scale,
                      "grid_cell_m": {"min": min(bs.grid_cells()), "median": statistics.median(bs.grid_cells()),
                                      "max": max(bs.grid_cells())}},
           "autotune_ms": {str(list(k)): v for k, v in tune.items()}, "autotune_s": tune_s, "setup_s": setup_s,
           "items": bs.items(), "ms_per_launch": ms, "ms_runs": times,
           "paths_per_launch": paths, "paths_per_s": paths / (ms / 1e3),
           "visibility_pairs_per_launch": bs.pairs(),
           "visible_pairs": [int(v) for v in cnt[:, :3].sum(0)],
           "ray_triangle_tests": int(cnt[:, 3].sum()), "tests_per_s": float(cnt[:, 3].sum() / (ms / 1e3)),
           "graph": "1 persistent kernel + 2 memsets per replay", "kernels_per_step": 1,
           "device_errors": [int(st), int(flags)]}
    # per-scene pair stages at the same frequency (FP64 phase path)
    worst = 0.0
    field = bs.field
    for si in (0, len(scenes) // 2, len(scenes) - 1):
        d, sc = bs.data[si], scenes[si]
        scat, scat_n = torch.from_numpy(sc.scat).cuda(), torch.from_numpy(sc.scat_n).cuda()
        E = np.array([1, 0, 0], np.complex64)
        for f in (0, bs.n_freq // 2, bs.n_freq - 1):
            kw = dict(grid=d.grid, alpha=0.0, beta=float(bs.betas[f]), self_to_self=False)
            out = P.pair_stage(sc.src, E, snk, snk_n, **kw).sink
            ep = P.pair_stage(sc.src, E, scat, scat_n, **kw).sink
            P.pair_stage(scat, ep, snk, snk_n, src_W=ep, sink_out=out, accumulate=True, **kw)
            ref = out.cpu().numpy()
            worst = max(worst, float(np.abs(field[si, f].cpu().numpy() - ref).max() / np.abs(ref).max()))
    res["rel_err_vs_pair_stages"] = worst
    res["fp64_check_large"] = batched_fp64_check(bs, scenes, snk, snk_n, freqs)
    # FP64 oracle (brute-force visibility on the host) on the scene with the fewest ray-triangle tests,
    # first and last frequency; skipped when even that scene is too large for a bounded CPU check
    costs = [(d.src.shape[0] * (bs.n_snk + d.scat.shape[0]) + d.scat.shape[0] * bs.n_snk) * d.n_tris for d in bs.data]
    si = int(np.argmin(costs))
    if costs[si] > 5e10:
        res["rel_err_fp64_oracle"] = None
        res["oracle_scene"] = "skipped: smallest scene needs more than 5e10 host ray-triangle tests"
        return res
    sc = scenes[si]
    t12 = O.pack_triangles(sc.verts, sc.faces)
    m0, m1, m2 = O.mask_brute(sc.src, snk, t12), O.mask_brute(sc.src, sc.scat, t12), O.mask_brute(sc.scat, snk, t12)
    E = np.tile(np.array([[1, 0, 0]], np.complex64), (sc.src.shape[0], 1))
    worst = 0.0
    for f in (0, bs.n_freq - 1):
        b_ = float(bs.betas[f])
        e = O.sink_field(sc.src, E, snk, snk_n, 0.0, b_, mask=m0)
        ep = O.sink_field(sc.src, E, sc.scat, sc.scat_n, 0.0, b_, mask=m1)
        e = e + O.sink_field(sc.scat, ep, snk, snk_n, 0.0, b_, srcW=ep, mask=m2)
        worst = max(worst, float(np.abs(field[si, f].cpu().numpy() - e).max() / np.abs(e).max()))
    res["rel_err_fp64_oracle"] = worst
    res["oracle_scene"] = {"index": si, "elements": int(sc.src.shape[0]), "scatter": int(sc.scat.shape[0]),
                           "triangles": int(sc.faces.shape[0])}
    return res


def batched_fp64_check(bs, scenes, snk, snk_n, freqs, n_snk=500, n_scat=600, freq_idx=None):
    """The batched kernel against the FP64 oracle on the scenes with the most triangles and with the most
    elements, each on a sample of its scatter points and of the sinks (every k-th), all sources, the full
    mesh, with the launch configuration and grid rule of `bs`; relative error per checked frequency (the
    first, a middle and the last, where the kernel's per-group phase rotation has run longest)."""
    import numpy as np

    from lyceanem_gb300 import batched as B
    from oracle import oracle as O
    if freq_idx is None:
        freq_idx = sorted({0, len(freqs) // 2 + 1, len(freqs) - 1})
    picks = sorted({int(np.argmax([sc.faces.shape[0] for sc in scenes])),
                    int(np.argmax([sc.src.shape[0] for sc in scenes]))})
    ks = max(1, snk.shape[0] // n_snk)
    ys, yn = snk[::ks], snk_n[::ks]
    out = []
    for si in picks:
        sc = scenes[si]
        kp = max(1, sc.scat.shape[0] // n_scat)
        scat, scat_n = sc.scat[::kp], sc.scat_n[::kp]
        sub = dict(src=sc.src, verts=sc.verts, faces=sc.faces, scat=scat, scat_n=scat_n)
        cb = B.BatchedScattering([sub], ys, yn, freqs, cell_scale=bs.cell_scale or 1.0, config=bs.config)
        field = cb.run().cpu().numpy()[0]
        og = O.Grid(O.pack_triangles(sc.verts, sc.faces), 0.5)
        m0, m1, m2 = og.mask(sc.src, ys), og.mask(sc.src, scat), og.mask(scat, ys)
        E = np.tile(np.array([[1, 0, 0]], np.complex64), (sc.src.shape[0], 1))
        errs = []
        for f in freq_idx:
            b_ = float(cb.betas[f])
            e = O.sink_field(sc.src, E, ys, yn, 0.0, b_, mask=m0)
            ep = O.sink_field(sc.src, E, scat, scat_n, 0.0, b_, mask=m1)
            e = e + O.sink_field(scat, ep, ys, yn, 0.0, b_, srcW=ep, mask=m2)
            errs.append(float(np.abs(field[f] - e).max() / np.abs(e).max()))
        pts = np.concatenate([sc.src, scat]).astype(np.float64)
        rmax = float(np.sqrt(((ys.astype(np.float64)[None] - pts[:, None]) ** 2).sum(-1)).max())
        out.append({"scene": si, "elements": int(sc.src.shape[0]), "triangles": int(sc.faces.shape[0]),
                    "scatter_sampled": int(scat.shape[0]), "sinks_sampled": int(ys.shape[0]),
                    "freq_index": [int(f) for f in freq_idx], "rel_err_per_freq": errs,
                    "max_kr_rad": float(cb.betas.max()) * rmax,
                    "visible_pairs": [int(m0.sum()), int(m1.sum()), int(m2.sum())]})
        del cb
    return {"metric": "max |E - E_fp64| / max |E_fp64| per frequency over the sampled sinks and components",
            "scenes": out, "max_rel_err": max(e for o in out for e in o["rel_err_per_freq"])}


# ------------------------------------------------------------------ adjoint
def _model_fp64(a, x, y, pol, y_n, scat, scat_n, m0, m1, m2, beta, chunk=256):
    """FP64 torch restatement of the forward sink field (em_wave composed as the reference's one bounce),
    visibility from the given masks, chunked over scatter points; runs on the GPU in float64."""
    import numpy as np
    import torch
    kappa = 1j * beta
    front = -1.0 / (2 * np.pi)

    def G(s, e, t, t_n, mask):
        rv = t[None, :, :] - s[:, None, :]
        r = torch.sqrt((rv * rv).sum(-1))
        d = rv / r[..., None]
        F = front * (-(kappa / r + 1.0 / r ** 2)) * torch.exp(-kappa * r)
        sd = (t_n[None, :, :] * d).sum(-1)
        q = e[:, None, :] - (e[:, None, :] * d).sum(-1, keepdim=True) * d
        return mask[..., None] * (F * sd)[..., None] * q

    E_src = a[:, None] * pol
    E = G(x, E_src, y, y_n, m0).sum(0)
    w = G(x, E_src, scat, scat_n, m1).sum(0)
    for p0 in range(0, scat.shape[0], chunk):
        p1 = min(p0 + chunk, scat.shape[0])
        E = E + (w[p0:p1, None, :] * G(scat[p0:p1], w[p0:p1], y, y_n, m2[p0:p1])).sum(0)
    return E


def run_adjoint(args, reps=3):
    """Differentiation scene: 16x16 array, 10,000 scatter points, 32,761 front-hemisphere sinks; loss
    sum |E - E_target|^2 with E_target the field of a seeded random-phase excitation.  Times forward and
    backward and checks gradient components against FP64 central differences (step 1e-4 wavelengths for
    positions) of an FP64 restatement of the forward model with the same masks."""
    import numpy as np
    import torch

    from lyceanem_gb300 import adjoint as A
    from lyceanem_gb300 import propagation as P
    from lyceanem_gb300 import scenes
    s = scenes.adjoint_scene()
    beta = 2 * np.pi / s.wavelength
    dev = torch.device("cuda")
    t = lambda z: torch.from_numpy(np.ascontiguousarray(z)).to(dev)  # noqa: E731
    tris = P.pack_triangles(t(s.verts), t(s.faces))
    grid = P.UniformGrid(tris, cell=s.cell)
    x0, y0, pol = t(s.src), t(s.snk), t(s.E)
    sn, sc, scn = t(s.snk_n), t(s.scat), t(s.scat_n)
    kw = dict(beta=beta, grid=grid)
    with torch.no_grad():
        target = A.sink_field(t(s.target_excitation), x0, y0, pol, sn, sc, scn, **kw).clone()
    N, M, Pn = x0.shape[0], y0.shape[0], sc.shape[0]
    fw, bw = [], []
    for _ in range(reps + 1):
        a = torch.ones(N, dtype=torch.complex64, device=dev, requires_grad=True)
        x = x0.clone().requires_grad_(True)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record()
        E = A.sink_field(a, x, y0, pol, sn, sc, scn, **kw)
        loss = ((E - target).abs() ** 2).sum()
        e1.record()
        loss.backward()
        e2.record()
        torch.cuda.synchronize()
        fw.append(e0.elapsed_time(e1))
        bw.append(e1.elapsed_time(e2))
    ga, gx = a.grad.detach(), x.grad.detach()
    # masks of the forward's three stages (deterministic), then FP64 central differences
    m0 = P.pair_stage(x0, pol, y0, sn, want_mask=True, **kw).mask().double()
    m1 = P.pair_stage(x0, pol, sc, scn, want_mask=True, **kw).mask().double()
    m2 = P.pair_stage(sc, pol[:1].expand(Pn, 3), y0, sn, want_mask=True, **kw).mask().double()
    d64 = lambda z: z.detach().to(torch.float64)  # noqa: E731
    c64 = lambda z: z.detach().to(torch.complex128)  # noqa: E731
    args64 = (d64(y0), c64(pol), d64(sn), d64(sc), d64(scn), m0, m1, m2, beta)

    def L(a_, x_):
        with torch.no_grad():
            E_ = _model_fp64(a_, x_, args64[0], args64[1], *args64[2:])
            return float(((E_ - c64(target)).abs() ** 2).sum())

    a64, x64 = torch.ones(N, dtype=torch.complex128, device=dev), d64(x0)
    h = 1e-4 * s.wavelength
    rng = np.random.default_rng(11)
    errs = []
    for n in rng.choice(N, size=2, replace=False):
        for part in (1.0, 1j):
            da = torch.zeros_like(a64)
            da[n] = part * 1e-4
            fd = (L(a64 + da, x64) - L(a64 - da, x64)) / 2e-4
            got = ga[n].real if part == 1.0 else ga[n].imag
            errs.append(abs(float(got) - fd) / float(ga.abs().max()))
    for n, k in zip(rng.choice(N, size=2, replace=False), (0, 2)):
        dx = torch.zeros_like(x64)
        dx[n, k] = h
        fd = (L(a64, x64 + dx) - L(a64, x64 - dx)) / (2 * h)
        errs.append(abs(float(gx[n, k]) - fd) / float(gx.abs().max()))
    return {"n_elements": N, "n_scatter": Pn, "n_sinks": M, "forward_ms": min(fw[1:]), "backward_ms": min(bw[1:]),
            "fd_components": len(errs), "fd_max_rel_err": max(errs),
            "fd_check": "FP64 central differences of an FP64 restatement of the forward with the forward's masks; "
                        "error = |grad - fd| / max|grad| over 4 excitation and 2 position components"}


# ------------------------------------------------------------------ parity
def run_parity(args, s):
    """Parity of the benchmarked workload at full geometry: the step's stages (same kernels, orders and
    grid) run on every PARITY_STRIDE-th sink and scatter point with all sources and the full mesh (the
    direct workload runs whole); each stage's mask is compared bit for bit with the oracle's, mismatching
    pairs are classified as epsilon-edge cases by an FP64 re-test, and the sink field of the sample is
    compared with the FP64 oracle's field on the oracle's masks.  Reference behaviour:
    lyceanem/src/raycasting.cuh:19-95, lyceanem/src/em.cuh:18-120, composed as
    lyceanem/models/frequency_domain.py:195-264, 847-849."""
    import numpy as np
    import torch

    from lyceanem_gb300 import propagation as P
    from oracle import oracle as O
    dev = torch.device("cuda")
    beta = 2 * np.pi / s.wavelength
    k = 1 if args.workload == "direct" else PARITY_STRIDE
    snk, snk_n = s.snk[::k], s.snk_n[::k]
    scat, scat_n = s.scat[::k], s.scat_n[::k]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    tris = P.pack_triangles(t(s.verts), t(s.faces))
    t12 = O.pack_triangles(s.verts, s.faces)
    if args.workload == "direct":
        grid = og = None
        kw = dict(beta=beta, tris=tris)
    else:
        grid = P.UniformGrid(tris, cell=s.cell)
        og = O.Grid(t12, s.cell)
        kw = dict(beta=beta, grid=grid)
    src, E = t(s.src), t(s.E)
    yk, ykn = t(snk), t(snk_n)
    o_snk = P.direction_order(yk, grid.centre) if grid is not None else None
    ta = array_schedule(args, s.src, grid)
    r0 = P.pair_stage(src, E, yk, ykn, want_mask=True, snk_order=o_snk, traversal=ta, **kw)
    field = r0.sink.clone()
    stages = [("direct", s.src, snk, r0)]
    if scat.shape[0]:
        pk, pkn = t(scat), t(scat_n)
        o_scat = P.spatial_order(pk)
        r1 = P.pair_stage(src, E, pk, pkn, want_mask=True, snk_order=o_scat, traversal=ta, **kw)
        e_p = r1.sink
        r2 = P.pair_stage(pk, e_p, yk, ykn, src_W=e_p, sink_out=field, accumulate=True, want_mask=True,
                          src_order=o_scat, snk_order=o_snk, traversal=args.traversal, **kw)
        stages += [("source_scatter", s.src, scat, r1), ("scatter_sink", scat, snk, r2)]
    gpu_masks = {name: r.mask().cpu().numpy() for name, _, _, r in stages}
    field = field.cpu().numpy()
    st, flags = P.device_errors()
    res = {"sample": (f"every {k}th sink ({snk.shape[0]}) and scatter point ({scat.shape[0]}), all "
                      f"{s.src.shape[0]} sources, all {s.faces.shape[0]} triangles"
                      + (f", the bench's {s.cell} m grid" if grid is not None else ", brute force")),
           "stages": {}, "device_errors": [int(st), int(flags)]}
    om = {}
    mism = edge = pairs_total = 0
    for name, a, b, _ in stages:
        m = (og.mask(a, b) if og is not None else O.mask_brute(a, b, t12)).astype(bool)
        om[name] = m
        bad = np.argwhere(gpu_masks[name] != m)
        checked = bad[:200]
        n_edge = int(O.edge_pairs(a, b, checked, t12).sum()) if len(checked) else 0
        res["stages"][name] = {"pairs": int(m.size), "visible": int(m.sum()), "mask_mismatches": int(len(bad)),
                               "edge_pairs": n_edge, "mismatches_classified": int(len(checked))}
        mism += len(bad)
        edge += n_edge
        pairs_total += m.size
    E64 = O.sink_field(s.src, s.E, snk, snk_n, 0.0, beta, mask=om["direct"])
    if scat.shape[0]:
        ep64 = O.sink_field(s.src, s.E, scat, scat_n, 0.0, beta, mask=om["source_scatter"])
        E64 = E64 + O.sink_field(scat, ep64, snk, snk_n, 0.0, beta, srcW=ep64, mask=om["scatter_sink"])
    err = float(np.abs(field - E64).max() / np.abs(E64).max())
    res.update({"pairs": int(pairs_total), "mask_mismatches": int(mism), "edge_pairs": int(edge),
                "field_rel_err": err, "field_tol": 1e-5,
                "field_metric": "max |E_gpu - E_fp64| / max |E_fp64| over the sample's sinks and components",
                "ok": bool(mism == edge and err <= 1e-5 and st == 0 and flags == 0)})
    return res


# ------------------------------------------------------------------ CPU
def cpu_sample(s, stride_snk, stride_scat, nthreads):
    """Times the oracle on every stride-th sink / scatter point; returns per-stage seconds."""
    import numpy as np

    from oracle import oracle as O
    beta = 2 * np.pi / s.wavelength
    snk, snk_n = s.snk[::stride_snk], s.snk_n[::stride_snk]
    scat, scat_n = s.scat[::stride_scat], s.scat_n[::stride_scat]
    t0 = time.perf_counter()
    tris = O.pack_triangles(s.verts, s.faces)
    grid = O.Grid(tris, s.cell) if s.cell else None
    kw = dict(grid=grid, tris12=None if grid else tris, nthreads=nthreads)
    t_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.sink_field(s.src, s.E, snk, snk_n, 0.0, beta, **kw)
    t_direct = time.perf_counter() - t0
    t_s1 = t_s2 = 0.0
    if scat.shape[0]:
        t0 = time.perf_counter()
        e_p = O.sink_field(s.src, s.E, scat, scat_n, 0.0, beta, **kw)
        t_s1 = time.perf_counter() - t0
        t0 = time.perf_counter()
        O.sink_field(scat, e_p, snk, snk_n, 0.0, beta, srcW=e_p, **kw)
        t_s2 = time.perf_counter() - t0
    return dict(build=t_build, direct=t_direct, s1=t_s1, s2=t_s2, n_snk=snk.shape[0], n_scat=scat.shape[0])


def cpu_extrapolate(s, paths, nthreads, stride):
    """Times the oracle on every stride-th sink and scatter point (all sources, full mesh and grid) and
    extrapolates stage by stage to the full workload.  Returns (paths/s of the full step, record)."""
    M, P = s.snk.shape[0], s.scat.shape[0]
    r = cpu_sample(s, stride, stride, nthreads)
    f_direct = M / r["n_snk"]
    f_s1 = P / r["n_scat"] if r["n_scat"] else 0.0
    f_s2 = (P * M) / (r["n_scat"] * r["n_snk"]) if r["n_scat"] else 0.0
    full = r["build"] + r["direct"] * f_direct + r["s1"] * f_s1 + r["s2"] * f_s2
    sample_s = r["build"] + r["direct"] + r["s1"] + r["s2"]
    N = s.src.shape[0]
    rec = {"stride": stride, "n_sinks": r["n_snk"], "n_scatter": r["n_scat"], "sample_s": sample_s,
           "stage_s": {k: r[k] for k in ("build", "direct", "s1", "s2")},
           "extrapolation": {"direct": f_direct, "source_scatter": f_s1, "scatter_sink": f_s2},
           "extrapolated_full_step_s": full, "paths_per_s": paths / full,
           "rays_per_s": {"direct": N * r["n_snk"] / r["direct"] if r["direct"] else None,
                          "source_scatter": N * r["n_scat"] / r["s1"] if r["s1"] else None,
                          "scatter_sink": r["n_scat"] * r["n_snk"] / r["s2"] if r["s2"] else None}}
    return paths / full, rec


def cpu_describe(s, rec):
    return (f"oracle (FP32 bit-faithful visibility on a CPU uniform grid, FP64 field) on every {rec['stride']}th "
            f"sink ({rec['n_sinks']}) and scatter point ({rec['n_scatter']}) with all {s.src.shape[0]} sources, "
            f"the full mesh and grid; {rec['sample_s']:.2f} s measured, extrapolated stage by stage "
            f"(direct x M/M', source->scatter x P/P', scatter->sink x PM/(P'M')) to "
            f"{rec['extrapolated_full_step_s']:.1f} s for the full step")


def cpu_strides(args):
    return CPU_STRIDES_DIRECT if args.workload == "direct" else CPU_STRIDES


def cpu_baseline(args, s, paths):
    """The oracle port on all host cores, on two sample sizes of the same workload (CPU_STRIDES); the
    value is the larger sample's extrapolated rate, the other is reported beside it."""
    from oracle import oracle as O
    n = O.max_threads()
    recs = [cpu_extrapolate(s, paths, n, k)[1] for k in cpu_strides(args)]
    main = max(recs, key=lambda r: r["sample_s"])
    rates = [r["paths_per_s"] for r in recs]
    return {"value": main["paths_per_s"], "unit": "paths/s", "cores": n, "kind": "port",
            "sample": cpu_describe(s, main), "samples": recs,
            "stride_spread": max(rates) / min(rates) - 1.0}


def run_reference(args, rank, world):
    """CPU restatement of the path on the host cores (the reference has no CPU engine).  Each step is one
    bounded sample (every CPU_STRIDES[0]-th sink and scatter point, all sources, the full mesh and grid),
    timed and extrapolated stage by stage; ms_per_step is the measured sample time.  After the timed
    steps the second sample size is measured once and reported beside the first."""
    from oracle import oracle as O
    s = workload_scene(args.workload)
    cfg, paths = describe(s, args.workload)
    n = O.max_threads()
    strides = cpu_strides(args)
    stride = strides[0]
    for _ in range(args.warmup):
        cpu_extrapolate(s, paths, n, stride)
    recs = [cpu_extrapolate(s, paths, n, stride)[1] for _ in range(max(1, args.steps))]
    other = cpu_extrapolate(s, paths, n, strides[1])[1]
    value = len(recs) / sum(1.0 / r["paths_per_s"] for r in recs)
    ms = 1e3 * sum(r["sample_s"] for r in recs) / len(recs)
    full_ms = 1e3 * sum(r["extrapolated_full_step_s"] for r in recs) / len(recs)
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 visibility / f64 field (CPU)", "data": "synthetic",
            "config": cfg, "extrapolated_full_step_ms": full_ms,
            "step": "one sample of the workload per step (ms_per_step is its measured time); value = full-step "
                    "paths / the sample's stage-by-stage extrapolated full-step time",
            "cpu_baseline": {"value": value, "unit": "paths/s", "cores": n, "kind": "port",
                             "sample": cpu_describe(s, recs[-1]), "samples": [recs[-1], other],
                             "stride_spread": max(value, other["paths_per_s"]) /
                             min(value, other["paths_per_s"]) - 1.0},
            "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args, rank, world)), flush=True)
        return 0
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    res = run_ours(args, rank, world)
    if rank == 0:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
